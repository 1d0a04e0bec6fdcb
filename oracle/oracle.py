"""ctypes front end of the CPU oracle (oracle/ih_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by ``__graft_entry__.smoke()`` as the
checker and by ``bench.py``'s CPU-baseline leg.  The product library never
imports this module.

The oracle restates nikikilbertus/InstaHeat's hot path (src/toolbox.c,
src/dopri853.c, src/rk4.c, src/setup.c) in C99 + OpenMP; see ih_oracle.h for
the parity pin.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libih_oracle.so"
SOURCES = [HERE / "ih_oracle.c", HERE / "ih_oracle_fft.c"]

_dp = C.POINTER(C.c_double)


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc -fopenmp into oracle/_build/."""
    BUILD.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + [HERE / "ih_oracle.h", HERE / "ih_oracle_internal.h"])
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-std=c99", "-O2", "-fopenmp", "-fPIC", "-shared", "-Wall",
           "-o", str(tmp)] + [str(s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("mass", C.c_double), ("gw", C.c_int), ("filter", C.c_int),
                ("bins", C.c_int), ("threads", C.c_int)]


class Output(C.Structure):
    _fields_ = [("phi_ps", _dp), ("psi_ps", _dp), ("rho_ps", _dp), ("gw", _dp),
                ("cstr", C.c_double * 4), ("smry", (C.c_double * 4) * 6)]


class DopriCfg(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("beta", C.c_double),
                ("safe", C.c_double), ("minscale", C.c_double), ("maxscale", C.c_double),
                ("max_dt_hubble_fraction", C.c_double), ("dt_min", C.c_double),
                ("max_steps", C.c_double)]


class DopriState(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("dt_next", C.c_double),
                ("dt_did", C.c_double), ("err_old", C.c_double), ("reject", C.c_int),
                ("n_stp", C.c_long), ("n_ok", C.c_long), ("n_bad", C.c_long),
                ("last_err", C.c_double), ("tries", C.c_long)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        L.iho_create.restype = C.c_void_p
        L.iho_create.argtypes = [C.POINTER(Params)]
        L.iho_destroy.argtypes = [C.c_void_p]
        L.iho_sizes.argtypes = [C.c_int] * 3 + [C.POINTER(C.c_size_t)] * 4
        L.iho_kgrid.argtypes = [C.c_void_p] + [_dp] * 8
        L.iho_filter_mask.argtypes = [C.c_void_p, _dp]
        L.iho_fft.argtypes = [C.c_void_p, _dp, _dp]
        L.iho_ifft.argtypes = [C.c_void_p, _dp, _dp]
        L.iho_mk_rhs.argtypes = [C.c_void_p, C.c_double, _dp, _dp, C.c_int, C.c_int,
                                 C.POINTER(Output)]
        for n in ("iho_rho_mean", "iho_pressure_mean"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [C.c_void_p]
        for n in ("iho_rho", "iho_pressure", "iho_lap", "iho_grad2"):
            getattr(L, n).restype = _dp
            getattr(L, n).argtypes = [C.c_void_p]
        L.iho_calls_rhs.restype = C.c_ulong
        L.iho_calls_rhs.argtypes = [C.c_void_p]
        L.iho_initial_psi.argtypes = [C.c_void_p, _dp, C.c_double]
        L.iho_mean.restype = C.c_double
        L.iho_mean.argtypes = [_dp, C.c_size_t]
        L.iho_variance.restype = C.c_double
        L.iho_variance.argtypes = [C.c_double, _dp, C.c_size_t]
        L.iho_dopri853_tableau.argtypes = [_dp] * 5
        L.iho_dopri853_dense_tableau.argtypes = [_dp] * 2
        L.iho_dopri853_step_dense.restype = C.c_int
        L.iho_dopri853_step_dense.argtypes = [C.c_void_p, C.POINTER(DopriCfg), C.POINTER(DopriState),
                                              _dp, _dp, C.c_double, C.c_int, _dp, _dp]
        L.iho_dopri853_init.argtypes = [C.c_void_p, C.POINTER(DopriCfg), C.POINTER(DopriState),
                                        _dp, _dp, C.c_double, C.c_double]
        L.iho_dopri853_step.restype = C.c_int
        L.iho_dopri853_step.argtypes = [C.c_void_p, C.POINTER(DopriCfg), C.POINTER(DopriState),
                                        _dp, _dp, C.c_double, C.POINTER(Output)]
        L.iho_dopri853_run.restype = C.c_long
        L.iho_dopri853_run.argtypes = [C.c_void_p, C.POINTER(DopriCfg), C.POINTER(DopriState),
                                       _dp, _dp, C.c_double, C.c_long, _dp, C.c_long]
        L.iho_rk4_step.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
        L.iho_ic_fluctuations.argtypes = [C.c_void_p, _dp, C.c_ulonglong, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double]
        _lib = L
    return _lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def sizes(nx, ny, nz):
    v = [C.c_size_t() for _ in range(4)]
    lib().iho_sizes(nx, ny, nz, *[C.byref(x) for x in v])
    return tuple(int(x.value) for x in v)


def tableau():
    c = np.zeros(12); a = np.zeros((12, 12)); b = np.zeros(12); bhh = np.zeros(3); er = np.zeros(12)
    lib().iho_dopri853_tableau(ptr(c), ptr(a), ptr(b), ptr(bhh), ptr(er))
    return c, a, b, bhh, er


def dense_tableau():
    """(ad[3][16], d[4][16]): the inputs of DOPRI853 stages 14..16 and the
    dense-output weights d4..d7, over stages 1..16 (dopri853_constants.c:23-25,
    98-173)."""
    ad = np.zeros((3, 16)); d = np.zeros((4, 16))
    lib().iho_dopri853_dense_tableau(ptr(ad), ptr(d))
    return ad, d


class DiagOutput:
    """Holds the diagnostic buffers the output flag fills."""

    def __init__(self, bins: int):
        self.phi_ps = np.zeros(bins); self.psi_ps = np.zeros(bins)
        self.rho_ps = np.zeros(bins); self.gw = np.zeros(bins)
        self.s = Output(ptr(self.phi_ps), ptr(self.psi_ps), ptr(self.rho_ps), ptr(self.gw))

    @property
    def cstr(self):
        return np.array(self.s.cstr[:])

    @property
    def smry(self):
        return np.array([list(r) for r in self.s.smry])


class Oracle:
    """One oracle context (grid, k vectors, temporaries, DOPRI work vectors)."""

    def __init__(self, n=(16, 16, 16), L=(20.0, 20.0, 20.0), mass=1.0, gw=True,
                 filter=True, bins=None, threads=0):
        nx, ny, nz = n
        self.n = (nx, ny, nz)
        self.L = tuple(L)
        self.bins = int(bins if bins is not None else nx // 2)
        self.p = Params(nx, ny, nz, L[0], L[1], L[2], mass, int(gw), int(filter), self.bins, threads)
        self.ctx = lib().iho_create(C.byref(self.p))
        if not self.ctx:
            raise ValueError("unsupported grid for the oracle")
        self.N, self.M, self.Next, self.Ntot = sizes(nx, ny, nz)

    def close(self):
        if self.ctx:
            lib().iho_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- grids ---
    def kgrid(self):
        arrs = [np.zeros(self.M) for _ in range(7)]
        kmax = C.c_double()
        lib().iho_kgrid(self.ctx, *[ptr(a) for a in arrs], C.cast(C.byref(kmax), _dp))
        return dict(zip(["x", "y", "z", "xf", "yf", "zf", "sq"], arrs)), kmax.value

    def filter_mask(self):
        m = np.zeros(self.M)
        lib().iho_filter_mask(self.ctx, ptr(m))
        return m

    # --- transforms (complex returned as complex128 [nx,ny,nz/2+1]) ---
    def fft(self, real):
        real = np.ascontiguousarray(real, dtype=np.float64).reshape(-1)
        out = np.zeros(2 * self.M)
        lib().iho_fft(self.ctx, ptr(real), ptr(out))
        nx, ny, nz = self.n
        return out.view(np.complex128).reshape(nx, ny, nz // 2 + 1)

    def ifft(self, spec):
        nx, ny, nz = self.n
        spec = np.ascontiguousarray(spec, dtype=np.complex128).reshape(-1).view(np.float64)
        out = np.zeros(self.N)
        lib().iho_ifft(self.ctx, ptr(spec), ptr(out))
        return out.reshape(nx, ny, nz)

    # --- RHS ---
    def rhs(self, f, t=0.0, filter=0, output=0, diag: DiagOutput | None = None):
        """mk_rhs on a copy of f; returns (result, f_after) (f_after is the
        possibly filtered state)."""
        f = np.array(f, dtype=np.float64, copy=True)
        res = np.zeros(self.Ntot)
        lib().iho_mk_rhs(self.ctx, t, ptr(f), ptr(res), int(filter), int(output),
                         C.byref(diag.s) if diag is not None else None)
        return res, f

    @property
    def rho_mean(self):
        return lib().iho_rho_mean(self.ctx)

    @property
    def pressure_mean(self):
        return lib().iho_pressure_mean(self.ctx)

    def field_array(self, name):
        p = getattr(lib(), "iho_" + name)(self.ctx)
        return np.ctypeslib.as_array(p, shape=(self.N,)).copy()

    @property
    def calls_rhs(self):
        return int(lib().iho_calls_rhs(self.ctx))

    def initial_psi(self, f, t=0.0):
        lib().iho_initial_psi(self.ctx, ptr(f), t)
        return f

    def ic(self, seed, phi0=1.0, dphi0=None, a0=1.0, amp=1.0e-3, kcut=None, psi=True):
        """Seeded fluctuation initial state, psi from the constraints."""
        if dphi0 is None:
            dphi0 = slow_roll_dphi0(phi0, self.p.mass)
        if kcut is None:
            kcut = (self.n[0] // 2) * 2.0 * np.pi / self.L[0]
        f = np.zeros(self.Ntot)
        lib().iho_ic_fluctuations(self.ctx, ptr(f), int(seed), phi0, dphi0, a0, amp, kcut)
        if psi:
            self.initial_psi(f)
        return f

    # --- steppers ---
    def dopri_init(self, field, cfg: DopriCfg, t0=0.0, dt0=1e-3):
        st = DopriState()
        dfield = np.zeros(self.Ntot)
        lib().iho_dopri853_init(self.ctx, C.byref(cfg), C.byref(st), ptr(field), ptr(dfield), t0, dt0)
        return st, dfield

    def dopri_step(self, field, dfield, cfg, st, dt_try, diag: DiagOutput | None = None):
        return lib().iho_dopri853_step(self.ctx, C.byref(cfg), C.byref(st), ptr(field), ptr(dfield),
                                       dt_try, C.byref(diag.s) if diag is not None else None)

    def dopri_step_dense(self, field, dfield, cfg, st, dt_try, theta):
        """One DOPRI853 step, then the continuous extension of the accepted
        step at the fractions theta of it: returns (status, array [len, Ntot])."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).ravel())
        out = np.zeros((len(th), self.Ntot))
        rc = lib().iho_dopri853_step_dense(self.ctx, C.byref(cfg), C.byref(st), ptr(field),
                                           ptr(dfield), dt_try, len(th), ptr(th), ptr(out))
        return rc, out

    def dopri_run(self, field, dfield, cfg, st, tf, max_steps, log_cap=0):
        log = np.zeros(4 * max(log_cap, 1))
        n = lib().iho_dopri853_run(self.ctx, C.byref(cfg), C.byref(st), ptr(field), ptr(dfield),
                                   tf, max_steps, ptr(log), log_cap)
        return n, log[: 4 * min(n, log_cap)].reshape(-1, 4)

    def rk4_step(self, field, t, dt):
        lib().iho_rk4_step(self.ctx, ptr(field), t, dt)


def slow_roll_dphi0(phi0, mass=1.0):
    """dphi0 = -V'/(3H), H = sqrt(V/3), V = m^2 phi^2/2."""
    V = 0.5 * mass * mass * phi0 * phi0
    H = np.sqrt(V / 3.0)
    return -mass * mass * phi0 / (3.0 * H)


def default_cfg(rtol=1e-10, atol=1e-10, max_dt_hubble_fraction=1e-2):
    """DOPRI853 controller defaults of src/parameters.sh:56-62."""
    return DopriCfg(rtol, atol, 0.0, 0.9, 0.333, 3.0, max_dt_hubble_fraction, 1e-9, 1e15)
