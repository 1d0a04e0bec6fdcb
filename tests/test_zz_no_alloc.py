"""ih_mean_dev_noalloc against ih_mean_dev, through the C ABI.

The no-allocation variant exists for callers that cannot call cudaMalloc
where they need the reduction (a program that hands all device memory to its
own arena, a loop that must not allocate, code without an ih_context).  It
keeps its partial sums in a fixed array inside the library, shared by all
calls.  This file is collected last so that a run stopping at its first
failure has already run every other test.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _lib(gpu_mod):
    L = gpu_mod.load()
    L.ih_mean_dev_noalloc.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    L.ih_mean_dev_noalloc.restype = C.c_int
    L.ih_mean_dev_noalloc_max_n.restype = C.c_size_t
    L.ih_mean_dev.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    return L


def test_noalloc_mean_matches_allocating_entry_point(gpu_mod):
    torch = pytest.importorskip("torch")
    L = _lib(gpu_mod)
    ctx = gpu_mod.Context(n=(16, 16, 16))
    out_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_na = torch.zeros(1, dtype=torch.float64, device="cuda")
    # two calls in a row; the second reuses the scratch the first one filled
    # (it has more blocks than the first, then fewer in a third call)
    for n, shift in [(3_000_017, 0.5), (9_437_185, -2.0), (70_001, 7.0)]:
        x = torch.randn(n, dtype=torch.float64, device="cuda") + shift
        torch.cuda.synchronize()
        assert L.ih_mean_dev(ctx.h, C.c_void_p(x.data_ptr()), n, C.c_void_p(out_ref.data_ptr())) == 0
        st = L.ih_mean_dev_noalloc(C.c_void_p(x.data_ptr()), n, C.c_void_p(out_na.data_ptr()), None)
        assert st == 0
        torch.cuda.synchronize()
        ref, got = out_ref.item(), out_na.item()
        assert abs(got - ref) <= 1e-13 * abs(ref), (n, got, ref)
        assert abs(got - x.mean().item()) <= 1e-12 * abs(ref)


def test_noalloc_mean_edge_sizes(gpu_mod):
    # one element, exactly one block's chunk (65536), and one past it (2 blocks)
    torch = pytest.importorskip("torch")
    L = _lib(gpu_mod)
    ctx = gpu_mod.Context(n=(16, 16, 16))
    out_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_na = torch.zeros(1, dtype=torch.float64, device="cuda")
    for n in (1, 65536, 65537, 1, 65537):
        x = torch.randn(n, dtype=torch.float64, device="cuda") + 3.0
        torch.cuda.synchronize()
        assert L.ih_mean_dev(ctx.h, C.c_void_p(x.data_ptr()), n, C.c_void_p(out_ref.data_ptr())) == 0
        assert L.ih_mean_dev_noalloc(C.c_void_p(x.data_ptr()), n, C.c_void_p(out_na.data_ptr()),
                                     None) == 0
        torch.cuda.synchronize()
        ref, got = out_ref.item(), out_na.item()
        assert abs(got - ref) <= 1e-13 * abs(ref), (n, got, ref)


def test_noalloc_mean_on_user_stream(gpu_mod):
    # the call runs on the caller's stream and returns without waiting
    torch = pytest.importorskip("torch")
    L = _lib(gpu_mod)
    s = torch.cuda.Stream()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(s):
        x = torch.randn(2_000_003, dtype=torch.float64, device="cuda") - 1.5
        y = torch.randn(131_073, dtype=torch.float64, device="cuda") + 4.0
        for i, v in enumerate((x, y)):
            assert L.ih_mean_dev_noalloc(C.c_void_p(v.data_ptr()), v.numel(),
                                         C.c_void_p(out.data_ptr() + 8 * i),
                                         C.c_void_p(s.cuda_stream)) == 0
    s.synchronize()
    for i, v in enumerate((x, y)):
        ref = v.mean().item()
        assert abs(out[i].item() - ref) <= 1e-12 * abs(ref), (i, out[i].item(), ref)


def test_noalloc_mean_rejects_oversize(gpu_mod):
    torch = pytest.importorskip("torch")
    L = _lib(gpu_mod)
    limit = L.ih_mean_dev_noalloc_max_n()
    assert limit == 2 ** 28
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # the size check happens before any launch, so no buffer of that size is needed
    assert L.ih_mean_dev_noalloc(C.c_void_p(x.data_ptr()), limit + 1, C.c_void_p(out.data_ptr()),
                                 None) == 7  # IH_ERR_TOO_LARGE
    assert L.ih_status_string(7).startswith(b"input larger")
