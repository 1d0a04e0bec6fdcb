"""The second oracle: nikikilbertus/InstaHeat's own C sources, compiled
unmodified and driven from Python.

TEST INFRASTRUCTURE ONLY: used by tests/, by the golden-fixture script under
tests/golden/ and by ``bench.py``'s reference arm.  The product library never
imports this module.

Recipe.  The reference needs FFTW3, HDF5 (h5cc) and GSL, none of which is
installed; its compile-time parameters come from ``parameters.sh`` through
its ``configure`` script, which turns ``src/main_template.h`` into
``main.h``.  Here:

* ``stage(root)`` copies the reference's path sources -- src/toolbox.c,
  setup.c, io.c, rk4.c, dopri853.c, dopri853_constants.c, main.c and their
  headers, main_template.h -- unmodified into ``oracle/_ref/src``
  (git-ignored, never committed).  The GPU host has no reference checkout;
  the staged copy travels with the working tree so that the same recipe
  builds there for its own CPU.
* ``build(params)`` renders ``main.h`` from the staged main_template.h with
  configure's substitution rules (src/configure:1-32) and compiles each source
  with the reference's flags (src/Makefile:3: -std=c99 -O3 -fopenmp) against
  the shims in ``oracle/ref_shim/`` (an FFTW3 subset over the oracle's FP64
  transforms, an HDF5 recorder, GSL's MT19937) into
  ``oracle/_ref/cfg_<hash>/libihref.so``.  main.c is compiled with main
  renamed to ``ihref_main``; ``oracle/ref_harness.c`` adds entry points and
  includes src/dopri853.c for its static step functions.
* ``run(build_dir, job, ...)`` runs one job in a child process (the reference
  calls exit() on errors): it writes the initial state as the reference's
  ``.dat`` format (io.c:801-820), calls ``allocate_and_init_all`` and then
  ``mk_rhs`` / DOPRI853 steps / ``run_rk4`` / the whole ``main``, and returns
  the arrays it read back, plus the recorded output file.

The shims change nothing the reference computes except the FFT algorithm
(the oracle's Stockham transforms instead of FFTW's codelets: both are exact
DFTs, different in rounding only) and the GSL quadrature behind Bunch-Davies
initial data, which is not provided (the BASELINE initial data enter through
``IC_FROM_DAT_FILE_*``).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import shutil
import struct
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_ref"
STAGE = OUT / "src"
SHIM = HERE / "ref_shim"

REF_FILES = ["toolbox.c", "setup.c", "io.c", "rk4.c", "dopri853.c", "dopri853_constants.c",
             "main.c", "toolbox.h", "setup.h", "io.h", "rk4.h", "dopri853.h", "gsl_stepper.h",
             "main_template.h", "parameters.sh"]
# compiled as their own translation units (dopri853.c comes in through the harness)
REF_UNITS = ["toolbox.c", "setup.c", "io.c", "rk4.c", "dopri853_constants.c", "main.c"]
OWN_UNITS = [HERE / "ref_harness.c", SHIM / "ih_ref_shim.c", HERE / "ih_oracle_fft.c"]
CFLAGS = ["-std=c99", "-O3", "-fopenmp", "-fPIC", "-D_DEFAULT_SOURCE", "-w"]

# Every parameters.sh key (src/parameters.sh) with the values of the
# workloads here: L = 20/m box, m = 1, DOPRI853 at rtol = atol = 1e-10, GW
# and filter on, every output on, initial data from a .dat file with psi
# solved by the reference (IC_FROM_DAT_FILE_WITHOUT_PSI).
DEFAULTS = {
    "DATAPATH": "out.h5rec", "INITIAL_DATAPATH": "initial.dat",
    "INITIAL_CONDITIONS": "IC_FROM_DAT_FILE_WITHOUT_PSI", "MASS": "1.0", "A_INITIAL": "1.0",
    "FINAL_TIME": "1.0", "GRIDPOINTS_X": "16", "GRIDPOINTS_Y": "16", "GRIDPOINTS_Z": "16",
    "SPATIAL_LOWER_BOUND_X": "-10.0", "SPATIAL_UPPER_BOUND_X": "10.0",
    "SPATIAL_LOWER_BOUND_Y": "-10.0", "SPATIAL_UPPER_BOUND_Y": "10.0",
    "SPATIAL_LOWER_BOUND_Z": "-10.0", "SPATIAL_UPPER_BOUND_Z": "10.0",
    "FFTW_DEFAULT_FLAG": "FFTW_ESTIMATE", "VERSION_CONTROL": "VERSION_CONTROL_NONE",
    "GSL_OUTPUT_NUMBER": "1000", "ENABLE_FFT_FILTER": "1", "ENABLE_GW": "1",
    "WRITE_OUT_BUFFER_NUMBER": "5", "POWER_SPECTRUM_BINS": "8", "TIME_STEP_SKIPS": "1",
    "STRIDE_X": "1", "STRIDE_Y": "1", "STRIDE_Z": "1", "INFLATON_MASS": "1.0e-3",
    "MASS_KARSTEN": "1.0e-2", "RELATIVE_TOLERANCE": "1.0e-10", "ABSOLUTE_TOLERANCE": "1.0e-10",
    "MAX_DT_HUBBLE_FRACTION": "1.0e-2", "THREAD_NUMBER": "0", "FFTW_THREAD_NUMBER": "0",
    "BUNCH_DAVIES_CUTOFF": "64", "ENABLE_FOLLOWUP": "1", "ENABLE_STIFFNESSCHECK": "0",
    "INTEGRATION_METHOD": "DOPRI853", "INITIAL_TIME": "0.0", "DELTA_T": "1.0e-3",
    "MINIMAL_DELTA_T": "1.0e-9", "MAX_STEPS": "1e15", "SMALLEST_SCALING": "0.333",
    "LARGEST_SCALING": "3.0", "BETA": "0.0", "SAFE": "0.9", "SEED": "93", "COUPLING": "1.0",
    "LAMBDA": "1.876e-4", "ENABLE_TIMING": "0", "MAX_RUNTIME": "172500",
    "OUTPUT_PHI": "1", "OUTPUT_DPHI": "1", "OUTPUT_PSI": "1", "OUTPUT_DPSI": "1", "OUTPUT_RHO": "1",
    "OUTPUT_PHI_PS": "1", "OUTPUT_PSI_PS": "1", "OUTPUT_RHO_PS": "1",
    "OUTPUT_PHI_SMRY": "1", "OUTPUT_DPHI_SMRY": "1", "OUTPUT_PSI_SMRY": "1",
    "OUTPUT_DPSI_SMRY": "1", "OUTPUT_RHO_SMRY": "1", "OUTPUT_PRESSURE_SMRY": "1",
    "OUTPUT_H1_SMRY": "0", "OUTPUT_H2_SMRY": "0", "OUTPUT_CONSTRAINTS": "1",
}


class Unavailable(RuntimeError):
    """The reference's sources are neither staged nor given."""


def stage(reference_root=None) -> Path:
    """Copy the reference's path sources into oracle/_ref/src (unchanged).
    ``reference_root`` is the reference checkout (its src/ holds the files);
    without it the existing staged copy is used."""
    if reference_root is not None:
        src = Path(reference_root) / "src"
        if not (src / "toolbox.c").exists():
            raise Unavailable(f"no reference sources under {src}")
        STAGE.mkdir(parents=True, exist_ok=True)
        for name in REF_FILES:
            dst = STAGE / name
            if not dst.exists() or dst.read_bytes() != (src / name).read_bytes():
                shutil.copyfile(src / name, dst)
    if not all((STAGE / n).exists() for n in REF_FILES):
        raise Unavailable("the reference's sources are not staged under oracle/_ref/src")
    return STAGE


def available() -> bool:
    return all((STAGE / n).exists() for n in REF_FILES)


def _switch(name: str) -> bool:
    return name.startswith("ENABLE") or name.startswith("OUTPUT")


def render_main_h(template: str, params: dict) -> str:
    """configure's rules (src/configure:1-32): __NAME__ -> value; for
    ENABLE_* / OUTPUT_* keys __NAME__ -> NAME when the value is 1, else
    NOT_NAME."""
    out = template
    for name, value in params.items():
        value = str(value)
        if _switch(name):
            out = out.replace(f"__{name}__", name if value.strip() == "1" else f"NOT_{name}")
        else:
            out = out.replace(f"__{name}__", value)
    return out


def config(**overrides) -> dict:
    p = dict(DEFAULTS)
    for k, v in overrides.items():
        if k not in DEFAULTS:
            raise KeyError(f"unknown parameters.sh key {k}")
        p[k] = str(v)
    return p


def _digest(params: dict) -> str:
    h = hashlib.sha1(json.dumps(sorted(params.items())).encode())
    for f in [STAGE / n for n in REF_FILES] + OWN_UNITS + sorted(SHIM.rglob("*.[ch]")) + [
            HERE / "ih_oracle_internal.h", HERE / "ih_oracle.h"]:
        h.update(f.read_bytes())
    h.update(" ".join(CFLAGS).encode())
    return h.hexdigest()[:16]


def prepare(params: dict | None = None) -> Path:
    """The directory of one parameter set with its main.h (rendered from the
    staged main_template.h) and params.json."""
    stage()
    params = config() if params is None else params
    d = OUT / f"cfg_{_digest(params)}"
    d.mkdir(parents=True, exist_ok=True)
    if not (d / "main.h").exists():
        (d / "main.h").write_text(render_main_h((STAGE / "main_template.h").read_text(), params))
        (d / "params.json").write_text(json.dumps(params, indent=1))
    return d


def build(params: dict | None = None, cc: str | None = None) -> Path:
    """Compile the reference for one parameter set; returns its directory
    (holding main.h and libihref.so).  Cached by the parameters and sources."""
    d = prepare(params)
    lib = d / "libihref.so"
    if lib.exists():
        return d
    cc = cc or shutil.which("gcc") or "cc"
    inc = ["-I", str(d), "-I", str(SHIM), "-I", str(STAGE), "-I", str(HERE)]

    def compile_one(src: Path):
        obj = d / (src.stem + ".o")
        extra = ["-Dmain=ihref_main"] if src.name == "main.c" else []
        cmd = [cc, *CFLAGS, *extra, *inc, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{r.stderr}")
        return obj

    units = [STAGE / u for u in REF_UNITS] + OWN_UNITS
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = lib.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [cc, "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference link failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, lib)
    return d


def build_dropin(params: dict, gpu_lib, dropin_src, include_dir, cc: str | None = None) -> Path:
    """The reference program relinked with the drop-in layer: the reference's
    own main.c, setup.c and io.c (unchanged, against the same main.h and
    shims) plus ``dropin_src`` (ih_dropin.c, which defines the symbols of
    toolbox.c, dopri853.c, dopri853_constants.c and rk4.c) linked with
    ``gpu_lib`` (libinstaheat_gpu.so).  Returns the executable; it reads
    INITIAL_DATAPATH and writes DATAPATH (the recorder format) in its working
    directory, like the reference's ``run``."""
    d = prepare(params)   # the reference's own toolbox/stepper files are not needed
    gpu_lib, dropin_src = Path(gpu_lib), Path(dropin_src)
    h = hashlib.sha1(dropin_src.read_bytes() + str(gpu_lib).encode() +
                     (Path(include_dir) / "instaheat_dropin.h").read_bytes() +
                     (Path(include_dir) / "instaheat_gpu.h").read_bytes()).hexdigest()[:12]
    exe = d / f"run_dropin_{h}"
    if exe.exists():
        return exe
    cc = cc or shutil.which("gcc") or "cc"
    inc = ["-I", str(d), "-I", str(SHIM), "-I", str(STAGE), "-I", str(HERE)]
    objs = []
    for src, extra in [(STAGE / "main.c", []), (STAGE / "setup.c", []), (STAGE / "io.c", []),
                       (SHIM / "ih_ref_shim.c", []), (HERE / "ih_oracle_fft.c", []),
                       (dropin_src, ["-I", str(include_dir)])]:
        obj = d / f"dropin_{src.stem}.o"
        cmd = [cc, *CFLAGS, *inc, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"drop-in build failed:\n{' '.join(cmd)}\n{r.stderr}")
        objs.append(obj)
    tmp = exe.with_name(exe.name + f".tmp{os.getpid()}")
    cmd = [cc, "-fopenmp", "-o", str(tmp), *map(str, objs), "-L", str(gpu_lib.parent),
           "-l" + gpu_lib.stem[3:], f"-Wl,-rpath,{gpu_lib.parent}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"drop-in link failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, exe)
    return exe


def run_program(exe, state: np.ndarray, build_dir, workdir=None, timeout=None):
    """Run a reference-layout program (the relinked drop-in) on ``state`` in
    a scratch directory; returns (CompletedProcess, recorded datasets or
    None)."""
    params = json.loads((Path(build_dir) / "params.json").read_text())
    n = tuple(int(params[f"GRIDPOINTS_{a}"]) for a in "XYZ")
    own = workdir is None
    work = Path(tempfile.mkdtemp(prefix="ihdrop_")) if own else Path(workdir)
    work.mkdir(parents=True, exist_ok=True)
    try:
        write_dat(work / params["INITIAL_DATAPATH"], state, n[0] * n[1] * n[2], n)
        r = subprocess.run([str(exe)], cwd=work, capture_output=True, text=True, timeout=timeout)
        rec = work / params["DATAPATH"]
        return r, (read_h5rec(rec) if rec.exists() else None)
    finally:
        if own:
            shutil.rmtree(work, ignore_errors=True)


# ---------------------------------------------------------------- files

def write_dat(path, field: np.ndarray, N: int, n: tuple):
    """The reference's .dat initial data (io.c:801-820): one line per grid
    point in memory order, "i j k phi dphi psi dpsi", printed with %.17g so
    that fscanf("%lf") reads back the same doubles."""
    nx, ny, nz = n
    idx = np.indices((nx, ny, nz)).reshape(3, -1).T
    cols = np.column_stack([field[0:N], field[N:2 * N], field[2 * N:3 * N], field[3 * N:4 * N]])
    with open(path, "w") as fh:
        for (i, j, k), row in zip(idx, cols):
            fh.write(f"{i} {j} {k} {row[0]:.17g} {row[1]:.17g} {row[2]:.17g} {row[3]:.17g}\n")


def write_h5rec(path, datasets: dict):
    """A file in the HDF5 recorder's format (rank-1 double datasets), e.g.
    {"followup": state, "time": [t]} for the reference's IC_FROM_H5_FILE
    restart (io.c:754-788)."""
    with open(path, "wb") as fh:
        fh.write(b"IHH5REC1")
        for name, v in datasets.items():
            a = np.ascontiguousarray(np.asarray(v, dtype="<f8").reshape(-1))
            nb = name.encode()
            fh.write(struct.pack("<I", len(nb)) + nb + struct.pack("<II", 0, 1))
            fh.write(struct.pack("<QQ", a.size, a.nbytes))
            fh.write(a.tobytes())


def read_h5rec(path) -> dict:
    """The HDF5 recorder's file (ref_shim/ih_ref_shim.c): name -> array
    (rank-2 datasets as (rows, dim), rank-1 as (n,)) or bytes (strings)."""
    data = Path(path).read_bytes()
    if data[:8] != b"IHH5REC1":
        raise ValueError("not an HDF5 recorder file")
    pos, out = 8, {}
    while pos < len(data):
        (ln,) = struct.unpack_from("<I", data, pos)
        pos += 4
        name = data[pos:pos + ln].decode()
        pos += ln
        cls, rank = struct.unpack_from("<II", data, pos)
        pos += 8
        dims = struct.unpack_from(f"<{rank}Q", data, pos)
        pos += 8 * rank
        (nb,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        raw = data[pos:pos + nb]
        pos += nb
        out[name] = raw if cls == 1 else np.frombuffer(raw, dtype="<f8").reshape(dims).copy()
    return out


# ---------------------------------------------------------------- jobs

class _Output(C.Structure):
    # struct output (main_template.h:200-206); hsize_t is unsigned long long
    _fields_ = [("dim", C.c_size_t), ("id", C.c_ulonglong), ("buf", C.POINTER(C.c_double)),
                ("tmp", C.POINTER(C.c_double))]


class _Flags(C.Structure):
    _fields_ = [("filter", C.c_uint8), ("output", C.c_uint8)]


OUTPUTS = ["phi_ps", "psi_ps", "rho_ps", "gw", "cstr", "phi_smry", "dphi_smry", "psi_smry",
           "dpsi_smry", "rho_smry", "p_smry"]


def _child(build_dir: Path, work: Path):
    """Runs inside the child process, cwd = work."""
    job = json.loads((work / "job.json").read_text())
    inp = dict(np.load(work / "in.npz"))
    L = C.CDLL(str(build_dir / "libihref.so"))
    for name in ("ihref_lap", "ihref_tmp_f"):
        getattr(L, name).restype = C.POINTER(C.c_double)
    L.ihref_time.restype = C.c_double
    L.mk_rhs.argtypes = [C.c_double, C.c_void_p, C.c_void_p]
    L.ihref_set_time.argtypes = [C.c_double] * 3
    sz = (C.c_size_t * 6)()
    L.ihref_sizes(sz)
    params = json.loads((build_dir / "params.json").read_text())
    n = tuple(int(params[f"GRIDPOINTS_{a}"]) for a in "XYZ")
    N = n[0] * n[1] * n[2]
    if job.get("ic") == "h5":
        write_h5rec(work / params["INITIAL_DATAPATH"],
                    {"followup": inp["state"], "time": [float(job.get("t0", 0.0))]})
    else:
        write_dat(work / params["INITIAL_DATAPATH"], inp["state"], N, n)
    res = {}
    kind = job["kind"]
    if kind == "main":
        argv = (C.c_char_p * 2)(b"ihref", None)
        L.ihref_main.argtypes = [C.c_int, C.c_void_p]
        L.ihref_main(1, argv)
        np.savez(work / "out.npz", **res)
        return
    L.ihref_init()
    L.ihref_sizes(sz)
    Ntot = int(sz[3])

    def arr(sym, n_=None):
        p = C.c_void_p.in_dll(L, sym).value
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), (n_ or Ntot,))

    field, dfield = arr("field"), arr("dfield")
    res["init_field"] = field.copy()
    res["init_dfield"] = dfield.copy()
    if job.get("set_state", job.get("ic") != "h5"):
        field[:] = inp["state"]
    flags = _Flags.in_dll(L, "evo_flags")
    if kind == "rhs":
        flags.filter, flags.output = int(job["filter"]), int(job["output"])
        L.mk_rhs(float(job.get("t", 0.0)), C.c_void_p(field.ctypes.data), C.c_void_p(dfield.ctypes.data))
        flags.filter = flags.output = 0
        res["field"] = field.copy()
        res["dfield"] = dfield.copy()
        res["rho_mean"] = np.array(C.c_double.in_dll(L, "rho_mean").value)
        res["pressure_mean"] = np.array(C.c_double.in_dll(L, "pressure_mean").value)
        res["rho"] = arr("rho", N).copy()
        res["pressure"] = arr("pressure", N).copy()
        res["lap"] = np.ctypeslib.as_array(L.ihref_lap(), (N,)).copy()
        if job["output"]:
            for o in OUTPUTS:
                s = _Output.in_dll(L, o)
                res["out_" + o] = np.ctypeslib.as_array(s.tmp, (int(s.dim),)).copy()
    elif kind == "dopri":
        L.ihref_set_time(float(job["t0"]), float(job["tf"]), float(job["dt0"]))
        L.ihref_dopri_begin.restype = None
        L.ihref_dopri_step.argtypes = [C.c_double, C.POINTER(C.c_double)]
        L.ihref_dopri_step.restype = C.c_int
        L.ihref_dopri_begin()
        res["begin_field"] = field.copy()
        res["begin_dfield"] = dfield.copy()
        info = (C.c_double * 5)()
        dt = float(job["dt0"])
        rows = []
        for _ in range(int(job["steps"])):
            st = L.ihref_dopri_step(dt, info)
            rows.append([st] + list(info))
            if st:
                break
            dt = info[2]
        res["steps"] = np.array(rows)
        res["field"] = field.copy()
        res["dfield"] = dfield.copy()
        res["rho_mean"] = np.array(C.c_double.in_dll(L, "rho_mean").value)
        L.ihref_dopri_end()
    elif kind == "rk4":
        L.ihref_set_time(float(job["t0"]), float(job["tf"]), float(job["dt"]))
        L.run_rk4()
        res["field"] = field.copy()
        res["t"] = np.array(L.ihref_time())
    elif kind == "bench":
        # run_dopri853's prologue from the state the reference read, steps
        # to settle_t untimed, then `steps` perform_step calls timed one by
        # one (wall clock around each call; the reference is single-process
        # OpenMP code)
        import time as _time
        L.ihref_set_time(L.ihref_time(), 1.0e30, float(job["dt0"]))
        L.ihref_dopri_begin.restype = None
        L.ihref_dopri_step.argtypes = [C.c_double, C.POINTER(C.c_double)]
        L.ihref_dopri_step.restype = C.c_int
        calls = C.c_size_t.in_dll(L, "mon")  # monitor.calls_rhs, its first member
        L.ihref_dopri_begin()
        info = (C.c_double * 5)()
        dt = float(job["dt0"])
        settle = 0
        while L.ihref_time() < float(job.get("settle_t", -1.0)):
            if L.ihref_dopri_step(dt, info):
                raise RuntimeError("step-size underflow while settling")
            dt = info[2]
            settle += 1
        rows = []
        for _ in range(int(job["steps"])):
            c0 = calls.value
            t0 = _time.perf_counter()
            st = L.ihref_dopri_step(dt, info)
            sec = _time.perf_counter() - t0
            # each try is 11 RHS (try_step), the accepted step adds one
            rows.append([info[0], info[1], sec, (calls.value - c0 - 1) / 11.0, st])
            if st:
                break
            dt = info[2]
        res["rows"] = np.array(rows)
        res["settle_steps"] = np.array(settle)
        res["dt_next"] = np.array(dt)
        L.ihref_dopri_end()
    elif kind == "init":
        pass
    else:
        raise ValueError(kind)
    L.ihref_free()
    np.savez(work / "out.npz", **res)


def run(build_dir, kind: str, state: np.ndarray, workdir=None, timeout=None, **job) -> dict:
    """Run one job of the reference in a child process.  ``state`` is the
    Ntot-double initial state in the reference layout (its phi, dphi, psi,
    dpsi go into the .dat file; with set_state (default) the whole array
    replaces ``field`` after initialisation).  Returns the arrays the job
    read back; with a recorder file, its datasets under ``"h5"``.  With
    ic="h5" (builds with INITIAL_CONDITIONS = IC_FROM_H5_FILE) the state and
    the time t0 reach the reference as a follow-up file instead (binary, fast
    at any size), read by its own h5_read_followup."""
    build_dir = Path(build_dir)
    own = workdir is None
    work = Path(tempfile.mkdtemp(prefix="ihref_")) if own else Path(workdir)
    work.mkdir(parents=True, exist_ok=True)
    try:
        job["kind"] = kind
        (work / "job.json").write_text(json.dumps(job))
        np.savez(work / "in.npz", state=np.ascontiguousarray(state, dtype=np.float64))
        env = dict(os.environ)
        env["PYTHONPATH"] = str(ROOT) + os.pathsep + env.get("PYTHONPATH", "")
        r = subprocess.run([sys.executable, "-m", "oracle.ref", str(build_dir), str(work)],
                           cwd=work, env=env, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference job {kind} failed ({r.returncode}):\n"
                               f"{r.stdout[-2000:]}\n{r.stderr[-4000:]}")
        out = dict(np.load(work / "out.npz"))
        out["stdout"] = r.stdout
        rec = work / json.loads((build_dir / "params.json").read_text())["DATAPATH"]
        if rec.exists():
            out["h5"] = read_h5rec(rec)
        return out
    finally:
        if own:
            shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    _child(Path(sys.argv[1]), Path(sys.argv[2]))
