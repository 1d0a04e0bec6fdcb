"""CPU tests of the C-ABI boundary: the library builds, loads and exports every
function include/*.h declares; host-only entry points behave (no GPU calls);
without a GPU the product path fails loudly."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ih_[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_header(gpu_mod):
    names = declared(ROOT / "include" / "instaheat_gpu.h")
    assert len(names) > 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(gpu_mod.lib_path())],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (\w+)$", out, flags=re.M))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = gpu_mod.load()
    for n in names:
        getattr(L, n)


def test_host_only_entry_points(gpu_mod):
    assert gpu_mod.sizes(64, 64, 64) == (262144, 64 * 64 * 33, 2 * 64 * 64 * 33,
                                         4 * 262144 + 8 * 64 * 64 * 33 + 1)
    c, a, b, bhh, er = gpu_mod.tableau()
    assert abs(b.sum() - 1.0) < 1e-14
    assert np.allclose(a.sum(axis=1), c, atol=1e-14)
    L = gpu_mod.load()
    assert L.ih_status_string(5) == b"step size underflow"


def test_gpu_tableau_equals_oracle_tableau(gpu_mod, oracle_mod):
    for x, y in zip(gpu_mod.tableau(), oracle_mod.tableau()):
        assert np.array_equal(x, y)


def test_invalid_grid_is_rejected_before_any_device_call(gpu_mod):
    import ctypes as C
    L = gpu_mod.load()
    h = C.c_void_p()
    # a prime factor other than 2 and 3, odd, out of order, too small, too large
    bad = [(20, 20, 20), (28, 28, 14), (27, 27, 27), (16, 32, 16), (16, 16, 4), (1024, 64, 64)]
    for n in bad:
        p = gpu_mod.Params(n[0], n[1], n[2], 20.0, 20.0, 20.0, 1.0, 1, 1, 8, 0, 0)
        assert L.ih_create(C.byref(p), C.byref(h)) == 1  # IH_ERR_ARG


def test_no_gpu_fails_loudly(gpu_mod):
    """Without a usable GPU the product path raises (no CPU fallback): context
    creation reports the CUDA error instead of computing anything."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu_mod.IHError, match="CUDA"):
        gpu_mod.Context(n=(16, 16, 16))
