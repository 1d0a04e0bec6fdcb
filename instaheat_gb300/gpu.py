"""ctypes binding of libinstaheat_gpu.so (include/instaheat_gpu.h).

This is the Python mirror of the reference's hot-path interface: a ``Context``
owns one grid on one GPU and exposes ``mk_rhs`` (src/toolbox.c:75-88),
``fft``/``ifft`` (toolbox.c:806-827), the DOPRI853 stepper (src/dopri853.c)
and RK4 (src/rk4.c), with the reference's flat state layout on the host side.

There is no CPU fallback: if the CUDA library is missing, loading fails with
an error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

PREC_F64 = 0
PREC_MIXED = 1
FFT_STOCKHAM, FFT_TWOSTEP, FFT_TWOSTEP_HALF, FFT_PIPELINED, FFT_THREESTEP = 0, 1, 2, 3, 4
FFT_TWOSTEP_HALF_OCC = 5

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "allocation failed",
          4: "call out of order", 5: "step size underflow", 6: "non-finite value"}

_dp = C.POINTER(C.c_double)


class Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("mass", C.c_double), ("enable_gw", C.c_int), ("enable_filter", C.c_int),
                ("bins", C.c_int), ("precision", C.c_int), ("device", C.c_int)]


class DopriCfg(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("beta", C.c_double),
                ("safe", C.c_double), ("minscale", C.c_double), ("maxscale", C.c_double),
                ("max_dt_hubble_fraction", C.c_double), ("dt_min", C.c_double),
                ("max_steps", C.c_double)]


class Output(C.Structure):
    _fields_ = [("phi_ps", _dp), ("psi_ps", _dp), ("rho_ps", _dp), ("gw", _dp),
                ("cstr", C.c_double * 4), ("smry", (C.c_double * 4) * 6)]


class StepInfo(C.Structure):
    _fields_ = [("t", C.c_double), ("dt_did", C.c_double), ("dt_next", C.c_double),
                ("err", C.c_double), ("tries", C.c_int), ("status", C.c_int)]


class IHError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it in tree if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise OSError(f"{path} is missing; run instaheat_gb300.build.build()")
        _build.build()
    L = C.CDLL(str(path))
    vp = C.c_void_p
    L.ih_status_string.restype = C.c_char_p
    L.ih_status_string.argtypes = [C.c_int]
    L.ih_sizes.argtypes = [C.c_int] * 3 + [C.POINTER(C.c_size_t)] * 4
    L.ih_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.ih_destroy.argtypes = [vp]
    L.ih_destroy.restype = None
    L.ih_last_error.restype = C.c_char_p
    L.ih_last_error.argtypes = [vp]
    L.ih_device_bytes.restype = C.c_size_t
    L.ih_device_bytes.argtypes = [vp]
    L.ih_set_state.argtypes = [vp, _dp, C.c_double]
    L.ih_get_state.argtypes = [vp, _dp]
    L.ih_get_dstate.argtypes = [vp, _dp]
    L.ih_set_dstate.argtypes = [vp, _dp]
    L.ih_mean_dev.argtypes = [vp, C.c_void_p, C.c_size_t, C.c_void_p]
    L.ih_time.restype = C.c_double
    L.ih_time.argtypes = [vp]
    L.ih_mk_rhs_host.argtypes = [vp, C.c_double, _dp, _dp, C.c_int, C.c_int]
    L.ih_mk_rhs_dev.argtypes = [vp, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    L.ih_get_means.argtypes = [vp, _dp, _dp]
    L.ih_get_field.argtypes = [vp, C.c_int, _dp]
    L.ih_get_output.argtypes = [vp, C.POINTER(Output)]
    L.ih_calls_rhs.restype = C.c_ulonglong
    L.ih_calls_rhs.argtypes = [vp]
    L.ih_fft_host.argtypes = [vp, _dp, _dp]
    L.ih_ifft_host.argtypes = [vp, _dp, _dp]
    L.ih_ic_fluctuations.argtypes = [vp, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double]
    L.ih_initial_psi.argtypes = [vp]
    L.ih_dopri853_init.argtypes = [vp, C.POINTER(DopriCfg), C.c_double, C.c_double]
    L.ih_dopri853_step.argtypes = [vp, C.c_double, C.c_int, C.POINTER(StepInfo)]
    L.ih_dopri853_run.argtypes = [vp, C.c_double, C.c_long, _dp, C.c_long, C.POINTER(C.c_long)]
    L.ih_dopri853_counters.argtypes = [vp, _dp, C.POINTER(C.c_long), C.POINTER(C.c_long),
                                       C.POINTER(C.c_long)]
    L.ih_dopri853_tableau.argtypes = [_dp] * 5
    L.ih_rk4_step.argtypes = [vp, C.c_double, C.c_int]
    L.ih_sync.argtypes = [vp]
    L.ih_profile_enable.argtypes = [vp, C.c_int]
    L.ih_profile_read.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_long)]
    L.ih_kernel_launches.restype = C.c_ulonglong
    L.ih_kernel_launches.argtypes = [vp]
    L.ih_profile_kernel.argtypes = [vp, C.c_int, _dp, C.POINTER(C.c_long), _dp]
    L.ih_profile_kernel_name.restype = C.c_char_p
    L.ih_profile_kernel_name.argtypes = [C.c_int]
    L.ih_profile_kernel_count.restype = C.c_int
    L.ih_timer_start.argtypes = [vp]
    L.ih_timer_stop.argtypes = [vp, _dp]
    L.ih_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    L.ih_host_free.argtypes = [C.c_void_p]
    L.ih_dopri853_set_noise_floor.argtypes = [vp, C.c_double]
    L.ih_dopri853_diag_enable.argtypes = [vp, C.c_int]
    L.ih_prepare_output.argtypes = [vp]
    _fp = C.POINTER(C.c_float)
    L.ih_mlp_create.argtypes = [C.c_int, C.c_uint, C.POINTER(vp)]
    L.ih_mlp_destroy.argtypes = [vp]
    L.ih_mlp_destroy.restype = None
    L.ih_mlp_last_error.restype = C.c_char_p
    L.ih_mlp_last_error.argtypes = [vp]
    L.ih_mlp_set_params.argtypes = [vp, _fp]
    L.ih_mlp_get_params.argtypes = [vp, _fp]
    L.ih_mlp_get_bf16_params.argtypes = [vp, _fp]
    L.ih_mlp_set_norm.argtypes = [vp, _fp, _fp, C.c_float, C.c_float]
    L.ih_mlp_forward.argtypes = [vp, _fp, C.c_int, _fp]
    L.ih_mlp_gradients.argtypes = [vp, _fp, _fp, C.c_int, _fp, _fp]
    L.ih_mlp_train.argtypes = [vp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint, _fp]
    L.ih_step_features.argtypes = [vp, _fp]
    L.ih_dopri853_set_proposer.argtypes = [vp, vp]
    L.ih_dopri853_error_breakdown.argtypes = [vp, _dp]
    L.ih_dopri853_init_ex.argtypes = [vp, C.POINTER(DopriCfg), C.c_double, C.c_double, C.c_int]
    L.ih_mean_host.argtypes = [vp, _dp, C.c_size_t, _dp]
    L.ih_variance_host.argtypes = [vp, C.c_double, _dp, C.c_size_t, _dp]
    L.ih_get_step_start_state.argtypes = [vp, _dp]
    L.ih_autotune.argtypes = [vp]
    L.ih_autotune_report.restype = C.c_char_p
    L.ih_autotune_report.argtypes = [vp]
    L.ih_fft_set_engine.argtypes = [vp, C.c_int, C.c_int]
    L.ih_fft_get_engine.argtypes = [vp, C.c_int]
    L.ih_graphs_enable.argtypes = [vp, C.c_int]
    L.ih_rhs_roundtrip.argtypes = [vp, C.c_int]
    L.ih_stage_fusion.argtypes = [vp, C.c_int]
    L.ih_velocity_form.argtypes = [vp, C.c_int]
    L.ih_dopri853_dense.argtypes = [vp, C.c_double, C.c_int, _dp]
    L.ih_dopri853_dense_tableau.argtypes = [_dp, _dp]
    L.ih_ensemble_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
    L.ih_ensemble_destroy.argtypes = [vp]
    L.ih_ensemble_destroy.restype = None
    L.ih_ensemble_last_error.restype = C.c_char_p
    L.ih_ensemble_last_error.argtypes = [vp]
    L.ih_ensemble_size.argtypes = [vp]
    L.ih_ensemble_member.restype = vp
    L.ih_ensemble_member.argtypes = [vp, C.c_int]
    L.ih_ensemble_autotune.argtypes = [vp]
    L.ih_ensemble_dopri_init.argtypes = [vp, C.POINTER(DopriCfg), C.c_double, C.c_double]
    L.ih_ensemble_run.argtypes = [vp, C.c_double, C.c_long, C.POINTER(C.c_long),
                                  C.POINTER(C.c_long)]
    L.ih_fp64_fma_peak.argtypes = [C.c_int, C.c_int, C.c_int, _dp]
    L.ih_gw_plane_probe.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp]
    _lib = L
    return L


def gw_plane_probe(form, mz=129, reps=20, device=0) -> float:
    """Milliseconds per launch of the tensor sources' plane transforms alone
    (ih_gw_plane_probe; form 1 one cluster per plane, 2 persistent, 3 persistent
    with the TT projection)."""
    v = C.c_double()
    st = load().ih_gw_plane_probe(device, form, mz, reps, C.byref(v))
    if st != 0:
        raise IHError(st, "ih_gw_plane_probe")
    return v.value


def fp64_fma_peak(device=0, iters=8192, reps=5) -> float:
    """Measured FP64 FMA throughput of the GPU in TFLOP/s (ih_fp64_fma_peak)."""
    v = C.c_double()
    st = load().ih_fp64_fma_peak(device, iters, reps, C.byref(v))
    if st != 0:
        raise IHError(st, "ih_fp64_fma_peak")
    return v.value


MLP_INPUTS = 12
MLP_NPARAMS = 5057


def _fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MLP:
    """The learned step-size proposer (ih_mlp): 12 -> 64 -> 64 -> 1, GELU,
    BF16 weights with FP32 accumulation, trained on the GPU."""

    def __init__(self, device=0, seed=0):
        self.L_ = load()
        h = C.c_void_p()
        st = self.L_.ih_mlp_create(device, seed, C.byref(h))
        if st:
            raise IHError(st, "ih_mlp_create")
        self.h = h
        self.norm = None

    def close(self):
        if getattr(self, "h", None):
            self.L_.ih_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st:
            raise IHError(st, f"{what}: {self.L_.ih_mlp_last_error(self.h).decode()}")

    @property
    def params(self):
        p = np.zeros(MLP_NPARAMS, dtype=np.float32)
        self._ck(self.L_.ih_mlp_get_params(self.h, _fptr(p)), "ih_mlp_get_params")
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == MLP_NPARAMS
        self._ck(self.L_.ih_mlp_set_params(self.h, _fptr(p)), "ih_mlp_set_params")

    def bf16_params(self):
        p = np.zeros(MLP_NPARAMS, dtype=np.float32)
        self._ck(self.L_.ih_mlp_get_bf16_params(self.h, _fptr(p)), "ih_mlp_get_bf16_params")
        return p

    def set_norm(self, in_mean, in_std, out_mean, out_std):
        m = np.ascontiguousarray(in_mean, dtype=np.float32)
        s = np.ascontiguousarray(in_std, dtype=np.float32)
        self._ck(self.L_.ih_mlp_set_norm(self.h, _fptr(m), _fptr(s), float(out_mean), float(out_std)),
                 "ih_mlp_set_norm")
        self.norm = (m.copy(), s.copy(), float(out_mean), float(out_std))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_INPUTS)
        y = np.zeros(len(X), dtype=np.float32)
        self._ck(self.L_.ih_mlp_forward(self.h, _fptr(X), len(X), _fptr(y)), "ih_mlp_forward")
        return y

    def gradients(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_INPUTS)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.zeros(MLP_NPARAMS, dtype=np.float32)
        loss = C.c_float()
        self._ck(self.L_.ih_mlp_gradients(self.h, _fptr(X), _fptr(Y), len(X), _fptr(g), C.byref(loss)),
                 "ih_mlp_gradients")
        return g, loss.value

    def train(self, X, Y, iters=2000, batch=128, lr=3e-3, seed=1):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_INPUTS)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        hist = np.zeros(iters, dtype=np.float32)
        self._ck(self.L_.ih_mlp_train(self.h, _fptr(X), _fptr(Y), len(X), iters, batch, lr, seed,
                                      _fptr(hist)), "ih_mlp_train")
        return hist


class PinnedArray:
    """A float64 numpy view on pinned (page-locked) host memory."""

    def __init__(self, n):
        self.L = load()
        p = C.c_void_p()
        st = self.L.ih_host_alloc(8 * n, C.byref(p))
        if st:
            raise IHError(st, "ih_host_alloc")
        self.p = p
        self.a = np.ctypeslib.as_array(C.cast(p, _dp), shape=(n,))

    def free(self):
        if self.p:
            self.L.ih_host_free(self.p)
            self.p = None


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def sizes(nx, ny, nz):
    v = [C.c_size_t() for _ in range(4)]
    st = load().ih_sizes(nx, ny, nz, *[C.byref(x) for x in v])
    if st:
        raise IHError(st, "ih_sizes")
    return tuple(int(x.value) for x in v)


def tableau():
    c = np.zeros(12); a = np.zeros((12, 12)); b = np.zeros(12); bhh = np.zeros(3); er = np.zeros(12)
    load().ih_dopri853_tableau(_ptr(c), _ptr(a), _ptr(b), _ptr(bhh), _ptr(er))
    return c, a, b, bhh, er


def dense_tableau():
    """(ad[3][16], d[4][16]): the inputs of DOPRI853 stages 14..16 and the
    dense-output weights d4..d7 over stages 1..16."""
    ad = np.zeros((3, 16)); d = np.zeros((4, 16))
    load().ih_dopri853_dense_tableau(_ptr(ad), _ptr(d))
    return ad, d


def dopri_cfg(rtol=1e-10, atol=1e-10, beta=0.0, safe=0.9, minscale=0.333, maxscale=3.0,
              max_dt_hubble_fraction=1e-2, dt_min=1e-9, max_steps=1e15) -> DopriCfg:
    """DOPRI853 controller; defaults are src/parameters.sh:56-62."""
    return DopriCfg(rtol, atol, beta, safe, minscale, maxscale, max_dt_hubble_fraction,
                    dt_min, max_steps)


class Context:
    """One grid on one GPU (wraps ih_context)."""

    def __init__(self, n=(32, 32, 32), L=(20.0, 20.0, 20.0), mass=1.0, gw=True,
                 filter=True, bins=None, precision=PREC_F64, device=0, autotune=False):
        self.L_ = load()
        nx, ny, nz = n
        self.n = (nx, ny, nz)
        self.box = tuple(float(x) for x in L)
        self.bins = int(bins if bins is not None else nx // 2)
        self.precision = precision
        self.p = Params(nx, ny, nz, self.box[0], self.box[1], self.box[2], mass, int(gw),
                        int(filter), self.bins, precision, device)
        h = C.c_void_p()
        st = self.L_.ih_create(C.byref(self.p), C.byref(h))
        if st:
            raise IHError(st, "ih_create")
        self.h = h
        self.N, self.M, self.Next, self.Ntot = sizes(nx, ny, nz)
        if autotune:
            self.autotune(wisdom=True)

    # --- FFT engines ---
    def autotune(self, wisdom=False):
        """Time the FFT engine variants on the device and keep the fastest.

        With wisdom=True the choice is kept in a small JSON file (like FFTW's
        wisdom; path $IH_FFT_WISDOM, default _lib/fft_wisdom.json) keyed by
        grid and precision, and an existing entry is reused instead of timing
        again -- so that a later run of the same program, e.g. under a
        profiler whose serialised launches would time the engines
        differently, uses the same engines."""
        import json
        import os
        path = Path(os.environ.get("IH_FFT_WISDOM", str(_build.OUT / "fft_wisdom.json")))
        key = "%dx%dx%d:%d" % (self.n + (self.precision,))
        if wisdom and path.exists():
            try:
                known = json.loads(path.read_text()).get(key)
            except ValueError:
                known = None
            if known and len(known.get("engines", ())) == len(self.engines()):
                for p, e in enumerate(known["engines"]):
                    self.set_engine(p, e)
                self._wisdom_report = "from wisdom: " + known["report"]
                return self._wisdom_report
        self._ck(self.L_.ih_autotune(self.h), "ih_autotune")
        report = self.L_.ih_autotune_report(self.h).decode()
        self._wisdom_report = None
        if wisdom:
            try:
                data = json.loads(path.read_text()) if path.exists() else {}
            except ValueError:
                data = {}
            data[key] = {"engines": list(self.engines()), "report": report}
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(data))
        return report

    @property
    def autotune_report(self):
        if getattr(self, "_wisdom_report", None):
            return self._wisdom_report
        return self.L_.ih_autotune_report(self.h).decode()

    def set_engine(self, pass_, engine):
        self._ck(self.L_.ih_fft_set_engine(self.h, pass_, engine), "ih_fft_set_engine")

    def graphs(self, on=True):
        """Replay DOPRI853 tries and post-step RHS evaluations as CUDA graphs."""
        self._ck(self.L_.ih_graphs_enable(self.h, int(on)), "ih_graphs_enable")

    def roundtrip(self, on=True):
        """Derivatives of phi in RHS evaluations without the filter and output
        flags from x and y round trips on its z spectrum (on, the default) or
        from the full 3-D spectrum (off)."""
        self._ck(self.L_.ih_rhs_roundtrip(self.h, int(on)), "ih_rhs_roundtrip")

    def stage_fusion(self, on=True):
        """DOPRI853 stage inputs formed by the previous stage's RHS kernels
        (on) or by separate combination passes (off, the default); the results
        are identical to the bit."""
        self._ck(self.L_.ih_stage_fusion(self.h, int(on)), "ih_stage_fusion")

    def velocity_form(self, on=True):
        """Mixed form: DOPRI853 combinations from the velocity halves of the
        stage vectors (on, the default) or the reference's formulation (off).
        No effect in FP64."""
        self._ck(self.L_.ih_velocity_form(self.h, int(on)), "ih_velocity_form")

    def engines(self):
        """Engines of the x, y, fused x passes, the x, y round trips, the form
        of the last tensor x pass (0 separate, 1 fused), of the fused z pass
        (1 wide rows where they apply, 0 a warp per row), the kz slab width
        of the tensor sources' y/x passes (0 whole arrays) and the plane-major
        tensor sources (0 rows, 1 one cluster per plane, 2 persistent clusters)."""
        return tuple(int(self.L_.ih_fft_get_engine(self.h, p)) for p in range(9))

    @classmethod
    def _member(cls, handle, p: Params):
        """A view of an ensemble member (the ensemble owns the context)."""
        self = cls.__new__(cls)
        self.L_ = load()
        self.n = (p.nx, p.ny, p.nz)
        self.box = (p.lx, p.ly, p.lz)
        self.bins = p.bins
        self.precision = p.precision
        self.p = p
        self.h = C.c_void_p(handle)
        self._borrowed = True
        self.N, self.M, self.Next, self.Ntot = sizes(p.nx, p.ny, p.nz)
        return self

    # --- lifecycle ---
    def close(self):
        if getattr(self, "h", None):
            if not getattr(self, "_borrowed", False):
                self.L_.ih_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st:
            raise IHError(st, f"{what}: {self.L_.ih_last_error(self.h).decode()}")

    @property
    def device_bytes(self):
        return int(self.L_.ih_device_bytes(self.h))

    @property
    def t(self):
        return float(self.L_.ih_time(self.h))

    @property
    def calls_rhs(self):
        return int(self.L_.ih_calls_rhs(self.h))

    @property
    def kernel_launches(self):
        return int(self.L_.ih_kernel_launches(self.h))

    # --- state ---
    def set_state(self, f, t=0.0):
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.size == self.Ntot
        self._ck(self.L_.ih_set_state(self.h, _ptr(f), t), "ih_set_state")

    def get_state(self):
        f = np.zeros(self.Ntot)
        self._ck(self.L_.ih_get_state(self.h, _ptr(f)), "ih_get_state")
        return f

    def step_start_state(self):
        """The state at the start of the last step, after its filter."""
        f = np.zeros(self.Ntot)
        self._ck(self.L_.ih_get_step_start_state(self.h, _ptr(f)), "ih_get_step_start_state")
        return f

    def mean_host(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros(1)
        self._ck(self.L_.ih_mean_host(self.h, _ptr(a), a.size, _ptr(out)), "ih_mean_host")
        return float(out[0])

    def variance_host(self, mean, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.zeros(1)
        self._ck(self.L_.ih_variance_host(self.h, float(mean), _ptr(a), a.size, _ptr(out)),
                 "ih_variance_host")
        return float(out[0])

    def get_dstate(self, out=None):
        f = np.zeros(self.Ntot) if out is None else out
        self._ck(self.L_.ih_get_dstate(self.h, _ptr(f)), "ih_get_dstate")
        return f

    def set_dstate(self, df):
        df = np.ascontiguousarray(df, dtype=np.float64)
        assert df.size == self.Ntot
        self._ck(self.L_.ih_set_dstate(self.h, _ptr(df)), "ih_set_dstate")

    def get_state_into(self, out):
        self._ck(self.L_.ih_get_state(self.h, _ptr(out)), "ih_get_state")
        return out

    # --- RHS ---
    def mk_rhs(self, f, t=0.0, filter=0, output=0):
        """mk_rhs on host arrays; returns (result, f_after_filter)."""
        f = np.array(f, dtype=np.float64, copy=True)
        res = np.zeros(self.Ntot)
        self._ck(self.L_.ih_mk_rhs_host(self.h, t, _ptr(f), _ptr(res), int(filter), int(output)),
                 "ih_mk_rhs_host")
        return res, f

    def means(self):
        r, p = C.c_double(), C.c_double()
        self._ck(self.L_.ih_get_means(self.h, C.byref(r), C.byref(p)), "ih_get_means")
        return r.value, p.value

    def field(self, which):
        names = {"rho": 0, "pressure": 1, "lap": 2}
        out = np.zeros(self.N)
        self._ck(self.L_.ih_get_field(self.h, names[which], _ptr(out)), "ih_get_field")
        return out

    def prepare_output(self):
        """Diagnostics of the device state (prepare_and_save_timeslice)."""
        self._ck(self.L_.ih_prepare_output(self.h), "ih_prepare_output")
        return self.output()

    def output(self):
        b = self.bins
        arrs = {k: np.zeros(b) for k in ("phi_ps", "psi_ps", "rho_ps", "gw")}
        o = Output(_ptr(arrs["phi_ps"]), _ptr(arrs["psi_ps"]), _ptr(arrs["rho_ps"]), _ptr(arrs["gw"]))
        self._ck(self.L_.ih_get_output(self.h, C.byref(o)), "ih_get_output")
        arrs["cstr"] = np.array(o.cstr[:])
        arrs["smry"] = np.array([list(r) for r in o.smry])
        return arrs

    # --- transforms ---
    def fft(self, real):
        nx, ny, nz = self.n
        real = np.ascontiguousarray(real, dtype=np.float64).reshape(-1)
        out = np.zeros(2 * self.M)
        self._ck(self.L_.ih_fft_host(self.h, _ptr(real), _ptr(out)), "ih_fft_host")
        return out.view(np.complex128).reshape(nx, ny, nz // 2 + 1)

    def ifft(self, spec):
        nx, ny, nz = self.n
        spec = np.ascontiguousarray(spec, dtype=np.complex128).reshape(-1).view(np.float64)
        out = np.zeros(self.N)
        self._ck(self.L_.ih_ifft_host(self.h, _ptr(spec), _ptr(out)), "ih_ifft_host")
        return out.reshape(nx, ny, nz)

    # --- initial conditions ---
    def ic(self, seed, phi0=1.0, dphi0=None, a0=1.0, amp=1.0e-3, kcut=None, psi=True):
        if dphi0 is None:
            V = 0.5 * self.p.mass ** 2 * phi0 ** 2
            dphi0 = -self.p.mass ** 2 * phi0 / (3.0 * np.sqrt(V / 3.0))
        if kcut is None:
            kcut = (self.n[0] // 2) * 2.0 * np.pi / self.box[0]
        self._ck(self.L_.ih_ic_fluctuations(self.h, int(seed), phi0, dphi0, a0, amp, kcut),
                 "ih_ic_fluctuations")
        if psi:
            self._ck(self.L_.ih_initial_psi(self.h), "ih_initial_psi")

    def initial_psi(self):
        self._ck(self.L_.ih_initial_psi(self.h), "ih_initial_psi")

    # --- steppers ---
    def dopri_init(self, cfg: DopriCfg, t0=0.0, dt0=1e-3, output=False):
        self._ck(self.L_.ih_dopri853_init_ex(self.h, C.byref(cfg), t0, dt0, int(output)),
                 "ih_dopri853_init_ex")

    def dopri_step(self, dt_try, output=False):
        info = StepInfo()
        st = self.L_.ih_dopri853_step(self.h, dt_try, int(output), C.byref(info))
        self._ck(st, "ih_dopri853_step")
        return info

    def dopri_dense(self, t_out, output=False):
        """The DOP853 continuous extension of the last accepted step at t_out
        (in [t - dt_did, t]); with output=True the interpolated state passes
        through the output RHS (filtered, diagnostics for get_output).
        Returns the interpolated state (reference layout)."""
        f = np.zeros(self.Ntot)
        self._ck(self.L_.ih_dopri853_dense(self.h, t_out, int(output), _ptr(f)),
                 "ih_dopri853_dense")
        return f

    def dopri_run(self, tf, max_steps=10 ** 9, log_cap=0):
        log = np.zeros(4 * max(1, log_cap))
        n = C.c_long()
        st = self.L_.ih_dopri853_run(self.h, tf, max_steps, _ptr(log), log_cap, C.byref(n))
        self._ck(st, "ih_dopri853_run")
        return n.value, log[: 4 * min(n.value, log_cap)].reshape(-1, 4)

    def dopri_counters(self):
        dtn = C.c_double()
        ok, bad, tries = C.c_long(), C.c_long(), C.c_long()
        self._ck(self.L_.ih_dopri853_counters(self.h, C.byref(dtn), C.byref(ok), C.byref(bad),
                                              C.byref(tries)), "ih_dopri853_counters")
        return dict(dt_next=dtn.value, n_ok=ok.value, n_bad=bad.value, tries=tries.value)

    def rk4_step(self, dt, output=False):
        self._ck(self.L_.ih_rk4_step(self.h, dt, int(output)), "ih_rk4_step")

    # --- timing ---
    def sync(self):
        self._ck(self.L_.ih_sync(self.h), "ih_sync")

    def profile(self, on=True):
        self._ck(self.L_.ih_profile_enable(self.h, int(on)), "ih_profile_enable")

    def error_breakdown(self, enable=None):
        """Per-segment error sums of the last try (enable=True/False toggles)."""
        if enable is not None:
            self._ck(self.L_.ih_dopri853_diag_enable(self.h, int(enable)), "ih_dopri853_diag_enable")
            return None
        out = np.zeros(12)
        self._ck(self.L_.ih_dopri853_error_breakdown(self.h, _ptr(out)), "ih_dopri853_error_breakdown")
        names = ["phi", "dphi", "psi", "dpsi", "h", "dh"]
        return {n: (out[2 * i], out[2 * i + 1]) for i, n in enumerate(names)}

    def step_features(self):
        f = np.zeros(MLP_INPUTS, dtype=np.float32)
        self._ck(self.L_.ih_step_features(self.h, _fptr(f)), "ih_step_features")
        return f

    def set_proposer(self, mlp):
        self._proposer = mlp  # keep it alive while the context uses it
        self._ck(self.L_.ih_dopri853_set_proposer(self.h, mlp.h if mlp is not None else None),
                 "ih_dopri853_set_proposer")

    def set_noise_floor(self, eta):
        self._ck(self.L_.ih_dopri853_set_noise_floor(self.h, eta), "ih_dopri853_set_noise_floor")

    def timer_start(self):
        self._ck(self.L_.ih_timer_start(self.h), "ih_timer_start")

    def timer_stop(self):
        ms = C.c_double()
        self._ck(self.L_.ih_timer_stop(self.h, C.byref(ms)), "ih_timer_stop")
        return ms.value

    def profile_kernels(self):
        """{kernel name: (ms, launches, algorithmic bytes)} since profile(True)."""
        out = {}
        for k in range(self.L_.ih_profile_kernel_count()):
            ms, n, b = C.c_double(), C.c_long(), C.c_double()
            self._ck(self.L_.ih_profile_kernel(self.h, k, C.byref(ms), C.byref(n), C.byref(b)),
                     "ih_profile_kernel")
            out[self.L_.ih_profile_kernel_name(k).decode()] = (ms.value, n.value, b.value)
        return out

    def profile_read(self, cls):
        ms, n = C.c_double(), C.c_long()
        self._ck(self.L_.ih_profile_read(self.h, cls, C.byref(ms), C.byref(n)), "ih_profile_read")
        return ms.value, n.value


class Ensemble:
    """Member grids stepped together (wraps ih_ensemble).  members: list of
    dicts with the Context keywords n, L, and optionally mass, gw, filter,
    bins, precision."""

    def __init__(self, members, device=0):
        self.L_ = load()
        ps = []
        for m in members:
            nx, ny, nz = m["n"]
            L = tuple(float(x) for x in m.get("L", (20.0, 20.0, 20.0)))
            ps.append(Params(nx, ny, nz, L[0], L[1], L[2], m.get("mass", 1.0), int(m.get("gw", True)),
                             int(m.get("filter", True)), int(m.get("bins", nx // 2)),
                             m.get("precision", PREC_MIXED), device))
        arr = (Params * len(ps))(*ps)
        h = C.c_void_p()
        st = self.L_.ih_ensemble_create(arr, len(ps), C.byref(h))
        if st:
            raise IHError(st, "ih_ensemble_create")
        self.h = h
        self.members = [Context._member(self.L_.ih_ensemble_member(h, i), ps[i]) for i in range(len(ps))]

    def _ck(self, st, what):
        if st:
            raise IHError(st, f"{what}: {self.L_.ih_ensemble_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.L_.ih_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.members)

    def autotune(self):
        self._ck(self.L_.ih_ensemble_autotune(self.h), "ih_ensemble_autotune")

    def dopri_init(self, cfg, t0=0.0, dt0=1e-3):
        self._ck(self.L_.ih_ensemble_dopri_init(self.h, C.byref(cfg), t0, dt0),
                 "ih_ensemble_dopri_init")

    def run(self, tf, max_rounds=10 ** 9):
        """Advance every member to tf; returns (rounds, accepted steps)."""
        rounds, steps = C.c_long(), C.c_long()
        self._ck(self.L_.ih_ensemble_run(self.h, tf, max_rounds, C.byref(rounds), C.byref(steps)),
                 "ih_ensemble_run")
        return int(rounds.value), int(steps.value)
