#!/usr/bin/env python3
"""Benchmark: m*t advanced per wall-second at 256^3 on one GB300.

A step is one accepted DOPRI853 step (perform_step of src/dopri853.c:271-311:
every rejected try, the 12 RHS evaluations of each try, and the filtered
post-step RHS) of the 256^3 workload: box L = 20/m, V = m^2 phi^2 / 2, m = 1,
seeded fluctuation initial data (phi0 = 1, slow-roll dphi0, amplitude 1e-3,
psi from the constraints), GW on, filter on, DOPRI853 rtol = atol = 1e-8.
The timed steps start after the step-size ramp (t >= 0.1) and W warm-up steps.

  value  -- m*t/s of the mixed FP32/FP64 form with the learned step-size
            proposer, state resident in HBM, timed with CUDA events on the
            context stream (inputs > L2: the state is 1.1 GB, each stage
            reads >= 2 of them).
  e2e    -- the same through the public C ABI with host buffers: every step
            uploads the state from pinned host memory, steps, and downloads
            the new state.
  f64    -- the plain FP64 form on the same workload (the ratio the metric
            names), with its step against both of its bounds: algorithmic
            bytes vs the HBM copy peak, flops vs the FP64 FMA rate measured on
            this GPU (ih_fp64_fma_peak).
  roofline -- the kernel with the largest share of device time in the timed
            region: algorithmic bytes per launch / mean launch time (CUDA
            events around each launch), against the measured HBM copy peak.
  accuracy_vs_f64 -- FP64, mixed + controller and mixed + proposer from the
            same data to --accuracy-t (default 10/m): GW spectrum and
            constraint residuals against FP64, steps, tries, wall time.
  cpu_baseline -- the reference's own code (oracle/_ref: its src/*.c
            compiled unmodified against the FFTW/HDF5/GSL shims) on this
            host's cores, started from the GPU arm's state at the start of its
            timed window and at its step size (handed over through the
            reference's follow-up restart, outside every timed region); the
            C oracle where the reference's sources are not staged.

--impl reference times that CPU path alone: the reference settles from the
same initial data to t >= 0.1 with its own controller, then its steps are
timed one by one.  Under torchrun each rank runs an independent realization
(replicas only; no collective on the data path).

Profiling and study legs (the commands under profiles/ use them):
  --case-rhs K / --case-steps K [--grid n --prec mixed|f64 --engine E
      --autotune]   K RHS evaluations or DOPRI853 steps of the seeded
      workload (the program ncu captures)
  --dt-study ETAS   12 DOPRI853 steps of FP64 and of the mixed form per
      rounding-floor factor eta: step size reached, per-segment error sums
  --gw-accuracy T [--etas ...]   GW spectrum at T of FP64 (and a 100x
      tighter FP64 run), the mixed form per eta, and the mixed form
      replaying the FP64 steps
  --long-run CHECKPOINTS [--forms f64,mixed_pi,mixed_learned --seed s
      --box L --phi0 p --model file]   the forms from the same data through
      each checkpoint time: spectra, constraints, steps, tries, wall time
  --config-run 1|2   configuration 1 (32^3 RK4, t in [0, 50]) or 2 (64^3
      DOPRI853 at 1e-10, t in [0, 200]) through the reference program on the
      CPU cores and the relinked drop-in program on the GPU: wall times and
      every recorded dataset compared
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("m·t advanced per wall-s at 256³: mixed+learned vs plain FP64 on one "
          "GB300, same error")
UNIT = "m*t/s"
N_GRID = 256
L_BOX = 20.0
RTOL = ATOL = 1e-8
AMP = 1e-3


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max/sum over ranks (gloo, scalars only) when WORLD_SIZE > 1."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def reduce(self, x, op):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region; the raw
    samples go to $IH_CLOCKS_DIR/clocks_rank<i>.csv (default: the system's
    temporary directory)."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = (Path(os.environ.get("IH_CLOCKS_DIR", tempfile.gettempdir())) /
                     f"clocks_rank{gpu_index}.csv")

    def start(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.f = open(self.path, "w")
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


ENGINE_NAMES = {0: "stockham", 1: "two-step", 2: "two-step-half", 3: "pipelined", 4: "three-step",
                5: "two-step-half-occ"}


def make_context(gpu, precision, device):
    # the FFT engines are autotuned on the device when the context is made
    ctx = gpu.Context(n=(N_GRID,) * 3, L=(L_BOX,) * 3, precision=precision, device=device,
                      autotune=True)
    return ctx


def init_workload(ctx, gpu, seed):
    ctx.ic(seed=seed, amp=AMP)
    cfg = gpu.dopri_cfg(RTOL, ATOL)
    ctx.dopri_init(cfg, 0.0, 1e-3)
    return cfg


def run_steps(ctx, dt, k):
    mt = 0.0
    for _ in range(k):
        info = ctx.dopri_step(dt)
        dt = info.dt_next
        mt += info.dt_did
    return dt, mt


def bench_form(gpu, precision, device, seed, steps, warmup, profile=False, clocks=None, dist=None,
               proposer=None, t_settle=0.1, keep_start=False):
    ctx = make_context(gpu, precision, device)
    init_workload(ctx, gpu, seed)
    if proposer is not None:
        ctx.set_proposer(proposer)
    # settle: advance past the step-size ramp from dt0 (untimed), then warm up
    dt = 1e-3
    while ctx.t < t_settle:
        dt = ctx.dopri_step(dt).dt_next
    dt, _ = run_steps(ctx, dt, warmup)
    ctx.sync()
    start = None
    if keep_start:
        # the state (reference layout, FP64) and step size at the start of
        # the timed window, for the CPU baseline; copied before timing
        start = {"state": ctx.get_state(), "t": ctx.t, "dt": dt}
    if dist:
        dist.barrier()
    if clocks:
        clocks.start()
    launches0 = ctx.kernel_launches
    ctx.timer_start()
    dt, mt = run_steps(ctx, dt, steps)
    ms = ctx.timer_stop()
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop() if clocks else None
    kern = None
    if profile:
        # per-kernel CUDA-event timing over further steps (kernel by kernel:
        # the timed steps above replay each DOPRI853 try as one CUDA graph)
        ctx.profile(True)
        dt, _ = run_steps(ctx, dt, steps)
        kern = ctx.profile_kernels()
        ctx.profile(False)
    res = {"ms": ms, "mt": mt, "dt_next": dt, "launches": launches, "kernels": kern, "clocks": clk,
           "start": start,
           "t": ctx.t, "device_bytes": ctx.device_bytes,
           "fft_engines": dict(zip(("x", "y", "deriv4_x", "roundtrip_x", "roundtrip_y"),
                                   (ENGINE_NAMES[e] for e in ctx.engines()[:5])))
                          | {"tensor_x": ("fused" if ctx.engines()[5] else "separate"),
                             "z_fused": ("warp rows", "wide rows",
                                         "wide rows, next row prefetched")[ctx.engines()[6]],
                             "gw_yx_slab": ctx.engines()[7],
                             "gw_planes": ("persistent planes", "planes", "rows")[
                                 2 - ctx.engines()[8]]},
           "fft_autotune": ctx.autotune_report}
    return ctx, res


def step_roofline(ms_per_step, peak, peak_src, elem=4):
    n = N_GRID
    N = n ** 3
    Next = 2 * n * n * (n // 2 + 1)
    Ntot = 4 * N + 4 * Next + 1
    b_step = (12 * 15 * (N + Next) + 72 * Ntot) * elem
    achieved = b_step / (ms_per_step / 1e3) / 1e9
    return {"bytes_per_step": b_step, "achieved": achieved, "peak": peak, "peak_source": peak_src,
            "unit": "GB/s", "frac": achieved / peak,
            "floor_ms_per_step": b_step / (peak * 1e9) * 1e3}


# FP64 FMA rate of a GB300 (nominal), used only if the measurement fails
FP64_NOMINAL_TFLOPS = 1.25


def fp64_peak(gpu, device):
    try:
        return gpu.fp64_fma_peak(device), "measured"
    except Exception:
        return FP64_NOMINAL_TFLOPS, "nominal"


def f64_roofline(ms_per_step, peak, peak_src, fp64=FP64_NOMINAL_TFLOPS, fp64_src="nominal"):
    """Both bounds of the plain FP64 form: its algorithmic bytes (the
    per-step formula at 8 bytes per value) against the HBM copy peak, and its
    flops -- 12 RHS x 11 transforms x 2.5 N log2 N plus about 160 Ntot in the
    stage combinations -- against the FP64 FMA rate (measured by
    ih_fp64_fma_peak on this GPU)."""
    n = N_GRID
    N = n ** 3
    Next = 2 * n * n * (n // 2 + 1)
    Ntot = 4 * N + 4 * Next + 1
    flops = 12 * 11 * 2.5 * N * np.log2(N) + 160 * Ntot
    tflops = flops / (ms_per_step / 1e3) / 1e12
    hbm = step_roofline(ms_per_step, peak, peak_src, elem=8)
    alu = {"flops_per_step": flops, "achieved": tflops, "peak": fp64, "peak_source": fp64_src,
           "unit": "TFLOP/s", "frac": tflops / fp64,
           "floor_ms_per_step": flops / (fp64 * 1e12) * 1e3}
    return {"bound": "fp64" if alu["frac"] >= hbm["frac"] else "hbm", "hbm": hbm, "fp64": alu}


def bench_e2e(gpu, ctx, steps):
    """Public-API loop with host buffers: upload, step, download per step."""
    Ntot = ctx.Ntot
    field, dfield = gpu.PinnedArray(Ntot), gpu.PinnedArray(Ntot)
    ctx.get_state_into(field.a)
    ctx.get_dstate(out=dfield.a)
    t = ctx.t
    dt = ctx.dopri_counters()["dt_next"]
    ctx.sync()
    t0 = time.perf_counter()
    mt = 0.0
    for _ in range(steps):
        ctx.set_state(field.a, t)           # H2D from pinned memory: field and dfield
        ctx.set_dstate(dfield.a)
        info = ctx.dopri_step(dt)
        dt = info.dt_next
        mt += info.dt_did
        t = info.t
        ctx.get_state_into(field.a)         # D2H of the step's result
        ctx.get_dstate(out=dfield.a)
    wall = time.perf_counter() - t0
    field.free()
    dfield.free()
    return {"value": mt / wall, "unit": UNIT, "h2d_bytes_per_step": 16 * Ntot,
            "d2h_bytes_per_step": 16 * Ntot, "ms_per_step": 1e3 * wall / steps}


def accuracy_check(device, seed, t_end):
    """FP64, mixed + controller alone, and mixed + learned proposer from the
    same initial data to t_end (the last step lands on t_end): GW spectrum and
    constraint residuals of the final states against the FP64 run, and each
    run's wall time (an equal-span speed ratio)."""
    from instaheat_gb300 import learned_dt
    r = learned_dt.evaluate(N_GRID, seed, t_end, device=device)
    ml = r["mixed_learned"]
    return {"t_end": t_end, "runs": {k: r[k] for k in ("f64", "mixed_pi", "mixed_learned")},
            "gw_max_rel_diff": ml["gw_max_rel_vs_f64"],
            "speedup_equal_span": r["f64"]["wall_s"] / ml["wall_s"],
            "within_1pct": bool(ml["gw_max_rel_vs_f64"] < 0.01)}


def reference_params():
    """parameters.sh values of the bench workload for the reference's own
    code: 256^3, L = 20/m, DOPRI853 rtol = atol = 1e-8, GW and filter on,
    the state handed over as a follow-up file (IC_FROM_H5_FILE), no output
    slices inside the timed steps (TIME_STEP_SKIPS beyond the run)."""
    from oracle import ref
    h = L_BOX / 2
    return ref.config(GRIDPOINTS_X=N_GRID, GRIDPOINTS_Y=N_GRID, GRIDPOINTS_Z=N_GRID,
                      SPATIAL_LOWER_BOUND_X=-h, SPATIAL_UPPER_BOUND_X=h,
                      SPATIAL_LOWER_BOUND_Y=-h, SPATIAL_UPPER_BOUND_Y=h,
                      SPATIAL_LOWER_BOUND_Z=-h, SPATIAL_UPPER_BOUND_Z=h,
                      POWER_SPECTRUM_BINS=N_GRID // 2, RELATIVE_TOLERANCE=RTOL,
                      ABSOLUTE_TOLERANCE=ATOL, INITIAL_CONDITIONS="IC_FROM_H5_FILE",
                      INITIAL_DATAPATH="initial.h5rec", TIME_STEP_SKIPS=1000000000,
                      ENABLE_FOLLOWUP=0, OUTPUT_PHI=0, OUTPUT_DPHI=0, OUTPUT_PSI=0, OUTPUT_DPSI=0,
                      OUTPUT_RHO=0)


def cpu_steps(state, t, dt, steps, settle_t=-1.0):
    """DOPRI853 steps of the 256^3 workload on this host's CPU cores from
    `state` at time t with first step size dt: the reference's own code when
    its sources are staged (kind "reference"), else the C oracle ("port").
    Steps until t >= settle_t are untimed; each of the `steps` timed steps is
    timed alone.  Returns per-step rows (t, dt_did, seconds, tries)."""
    cores = os.cpu_count()
    from oracle import ref
    if ref.available():
        r = ref.run(ref.build(reference_params()), "bench", state, ic="h5", t0=t, dt0=dt,
                    settle_t=settle_t, steps=steps, timeout=3600)
        rows = r["rows"][:, :4]
        kind, what = "reference", ("the reference's src/*.c (DOPRI853 perform_step) compiled "
                                   "unmodified against the FFTW/HDF5/GSL shims (FFTW API over "
                                   "the project's FP64 Stockham transforms)")
    else:
        from oracle import oracle as orc
        o = orc.Oracle(n=(N_GRID,) * 3, L=(L_BOX,) * 3, threads=cores)
        f = np.array(state, dtype=np.float64)
        cfg = orc.default_cfg(RTOL, ATOL, 1e-2)
        st, df = o.dopri_init(f, cfg, t, dt)
        while st.t < settle_t:
            o.dopri_step(f, df, cfg, st, dt)
            dt = st.dt_next
        out = []
        for _ in range(steps):
            tries0 = st.tries
            t0 = time.perf_counter()
            o.dopri_step(f, df, cfg, st, dt)
            out.append([st.t, st.dt_did, time.perf_counter() - t0, st.tries - tries0])
            dt = st.dt_next
        o.close()
        rows = np.array(out)
        kind, what = "port", "the C99+OpenMP oracle's DOPRI853 step"
    sec = rows[:, 2].sum()
    return {"value": rows[:, 1].sum() / sec, "unit": UNIT, "cores": cores, "kind": kind,
            "ms_per_step": 1e3 * sec / len(rows), "dt_per_step": rows[:, 1].tolist(),
            "tries_per_step": rows[:, 3].tolist(), "t_start": float(rows[0, 0] - rows[0, 1]),
            "what": what, "rows": rows}


def cpu_baseline(start, steps=2):
    """The CPU baseline leg: `steps` steps from the GPU arm's timed-window
    start (state, t, dt)."""
    r = cpu_steps(start["state"], start["t"], start["dt"], steps)
    r["sample"] = (f"{len(r['rows'])} DOPRI853 steps of the 256^3 workload from the GPU arm's "
                   f"state at t={start['t']:.4g} and its step size {start['dt']:.4g} "
                   f"({r['what']}), {r['cores']} threads, "
                   f"{r['ms_per_step'] / 1e3:.2f} s per step")
    r["gpu_dt"] = start["dt"]
    return {k: r[k] for k in ("value", "unit", "cores", "kind", "sample", "ms_per_step",
                              "dt_per_step", "tries_per_step", "t_start", "gpu_dt")}


def reference_arm(args, dist):
    """--impl reference: the CPU path alone on the same workload, rank 0."""
    if dist.rank != 0:
        return
    from oracle import oracle as orc
    o = orc.Oracle(n=(N_GRID,) * 3, L=(L_BOX,) * 3)
    f = o.ic(seed=0, amp=AMP)
    o.close()
    k = max(1, min(args.steps, 4))
    r = cpu_steps(f, 0.0, 1e-3, k, settle_t=0.1)
    line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": len(r["rows"]), "warmup": 0,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "256^3 DOPRI853 rtol=atol=1e-8, L=20/m, phi^2, GW+filter",
                       "grid": N_GRID, "settle_t": 0.1, "t_start": r["t_start"],
                       "dt_per_step": r["dt_per_step"], "tries_per_step": r["tries_per_step"]},
            "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"],
                             "kind": r["kind"],
                             "sample": (f"{len(r['rows'])} DOPRI853 steps after the reference's "
                                        f"own controller settled from dt0=1e-3 to t>=0.1, each "
                                        f"timed alone ({r['what']}), {r['cores']} threads")},
            "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ study legs

def plane_probe(gpu, forms, reps):
    """The tensor sources' plane pass (ih_fft_set_engine pass 8 forms) alone
    on six 256 x 256 x 129 complex FP32 spectra (405 MB): ms per launch and
    the rate of its algorithmic bytes (forms 1, 2: the six spectra read and
    written; form 3: read, and the two projected spectra written)."""
    M = 256 * 256 * 129
    for form in forms:
        ms = gpu.gw_plane_probe(form, 129, max(1, reps))
        nbytes = (12 if form < 3 else 8) * M * 8
        print(json.dumps({"form": form, "ms": ms, "bytes": nbytes,
                          "GBs": nbytes / (ms * 1e-3) / 1e9}), flush=True)


def case_workload(gpu, args):
    """K RHS evaluations or DOPRI853 steps of the seeded workload (the
    program the ncu captures under profiles/ run)."""
    prec = gpu.PREC_MIXED if args.prec == "mixed" else gpu.PREC_F64
    ctx = gpu.Context(n=(args.grid,) * 3, precision=prec)
    if args.engine is not None:  # pin the x/y (and, where it exists, fused x) FFT engine
        for p in range(3):
            if not (p == 2 and args.engine in (gpu.FFT_THREESTEP, gpu.FFT_TWOSTEP_HALF_OCC)):
                ctx.set_engine(p, args.engine)
    elif args.autotune:
        print(ctx.autotune(wisdom=True), flush=True)
    ctx.ic(seed=0, amp=AMP)
    cfg = gpu.dopri_cfg(args.rtol, args.rtol)
    ctx.dopri_init(cfg, 0.0, 1e-3)   # one filtered RHS
    for _ in range(args.case_rhs):
        ctx.dopri_init(cfg, 0.0, 1e-3)
    dt = 1e-3
    for _ in range(args.case_steps):
        dt = ctx.dopri_step(dt).dt_next
    ctx.sync()
    print(f"done: n={args.grid} prec={args.prec} rhs={ctx.calls_rhs} "
          f"launches={ctx.kernel_launches}", flush=True)
    ctx.close()


def dt_study(gpu, n, etas, rtol, steps=12):
    """12 DOPRI853 steps of FP64 and of the mixed form per rounding-floor
    factor eta: the step size reached and the per-segment error sums."""
    runs = [(gpu.PREC_F64, 0.0)] + [(gpu.PREC_MIXED, e) for e in etas]
    for prec, eta in runs:
        ctx = gpu.Context(n=(n,) * 3, precision=prec)
        ctx.ic(seed=0, amp=AMP)
        ctx.set_noise_floor(eta)
        ctx.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
        ctx.error_breakdown(True)
        dt = 1e-3
        for _ in range(steps):
            info = ctx.dopri_step(dt)
            dt = info.dt_next
        bd = ctx.error_breakdown()
        print(json.dumps({"n": n, "prec": "f64" if prec == gpu.PREC_F64 else "mixed", "eta": eta,
                          "dt_next": dt, "t": info.t, "err": info.err,
                          "segments_e5": {k: v[0] for k, v in bd.items()}}), flush=True)
        ctx.close()


def gw_accuracy(gpu, n, t_end, etas, rtol):
    """GW spectrum and constraints at t_end of the FP64 form (rtol and a
    100x tighter run), of the mixed form per eta, and of the mixed form
    replaying the FP64 run's accepted steps."""
    def run(prec, eta, tol):
        ctx = gpu.Context(n=(n,) * 3, precision=prec)
        ctx.ic(seed=0, amp=AMP)
        ctx.set_noise_floor(eta)
        ctx.dopri_init(gpu.dopri_cfg(tol, tol), 0.0, 1e-3)
        steps, _ = ctx.dopri_run(t_end)
        d = ctx.prepare_output()
        ctx.close()
        return steps, d

    ref_steps, refd = run(gpu.PREC_F64, 0.0, rtol / 100)
    gref = refd["gw"]
    sig = gref > 1e-3 * gref.max()
    print(json.dumps({"case": "f64_ref", "rtol": rtol / 100, "steps": ref_steps,
                      "gw": [float(x) for x in gref], "cstr": [float(x) for x in refd["cstr"]]}),
          flush=True)
    c64 = gpu.Context(n=(n,) * 3, precision=gpu.PREC_F64)
    c64.ic(seed=0, amp=AMP)
    c64.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
    steps64, log = c64.dopri_run(t_end, log_cap=100000)
    d64 = c64.prepare_output()
    c64.close()
    cm = gpu.Context(n=(n,) * 3, precision=gpu.PREC_MIXED)
    cm.ic(seed=0, amp=AMP)
    cm.set_noise_floor(1e30)  # every try is accepted: the step sizes are imposed
    cm.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
    for row in log:
        cm.dopri_step(row[1])
    dm = cm.prepare_output()
    cm.close()
    g64 = d64["gw"]
    rel = np.abs(dm["gw"] - g64) / np.where(g64 > 0, g64, 1.0)
    sig64 = g64 > 1e-3 * g64.max()
    print(json.dumps({"case": "mixed_replay_vs_f64", "rtol": rtol, "steps": int(steps64),
                      "gw_max_rel_sig": float(rel[sig64].max()), "gw_rel": [float(x) for x in rel],
                      "cstr": [float(x) for x in dm["cstr"]],
                      "cstr_f64": [float(x) for x in d64["cstr"]]}), flush=True)
    for prec, eta in [(gpu.PREC_F64, 0.0)] + [(gpu.PREC_MIXED, e) for e in etas]:
        steps, d = run(prec, eta, rtol)
        rel = np.abs(d["gw"] - gref) / np.where(gref > 0, gref, 1.0)
        print(json.dumps({"case": "f64" if prec == gpu.PREC_F64 else "mixed", "eta": eta,
                          "rtol": rtol, "steps": steps, "gw_max_rel_sig": float(rel[sig].max()),
                          "gw_rel": [float(x) for x in rel],
                          "cstr": [float(x) for x in d["cstr"]]}), flush=True)


def _rel_sig(x, ref, floor=1e-3):
    """max relative difference over the bins holding at least `floor` of the
    reference spectrum's maximum."""
    sig = ref > floor * ref.max()
    return float((np.abs(x - ref)[sig] / ref[sig]).max()) if sig.any() else 0.0


def long_run(gpu, n, checkpoints, forms, seed, rtol, device=0, L=L_BOX, phi0=1.0, model=None):
    """The forms from the same seeded data through each checkpoint time
    (each run's last step lands on the checkpoint, as the reference's run
    loop lands on tf, dopri853.c:120-123; the output slice there filters the
    state as prepare_and_save_timeslice does): per checkpoint the field and
    GW spectra, constraint residuals, accepted steps, tries and wall time.
    Prints one JSON line per form and checkpoint, then one comparison line
    per checkpoint against the FP64 run (or, without it, the first form)."""
    from instaheat_gb300 import learned_dt
    res = {}
    for form in forms:
        prec = gpu.PREC_F64 if form == "f64" else gpu.PREC_MIXED
        ctx = gpu.Context(n=(n,) * 3, L=(L,) * 3, precision=prec, device=device, autotune=True)
        ctx.ic(seed=seed, amp=AMP, phi0=phi0)
        ctx.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
        if form == "mixed_learned":
            mlp, _ = learned_dt.load(model or learned_dt.DEFAULT_MODEL, device=device)
            ctx.set_proposer(mlp)
        wall, steps_all = 0.0, 0
        res[form] = []
        for tc in checkpoints:
            ctx.sync()
            t0 = time.perf_counter()
            steps, _ = ctx.dopri_run(tc)
            ctx.sync()
            wall += time.perf_counter() - t0
            steps_all += steps
            cnt = ctx.dopri_counters()
            d = ctx.prepare_output()
            row = {"form": form, "n": n, "seed": seed, "L": L, "phi0": phi0, "t": ctx.t,
                   "steps": steps_all, "tries": cnt["tries"], "rejected": cnt["tries"] - steps_all,
                   "wall_s": wall, "mt_per_s": ctx.t / wall, "dt_next": cnt["dt_next"],
                   "gw": d["gw"].tolist(), "phi_ps": d["phi_ps"].tolist(),
                   "psi_ps": d["psi_ps"].tolist(), "rho_ps": d["rho_ps"].tolist(),
                   "cstr": d["cstr"].tolist(), "smry": d["smry"].tolist()}
            res[form].append(row)
            print(json.dumps(row), flush=True)
        ctx.close()
    base = "f64" if "f64" in res else forms[0]
    for i, tc in enumerate(checkpoints):
        b = res[base][i]
        cmp = {"compare_at": tc, "base": base, "n": n, "seed": seed}
        for form in forms:
            r = res[form][i]
            cmp[form] = {k: _rel_sig(np.array(r[k]), np.array(b[k]))
                         for k in ("gw", "phi_ps", "psi_ps", "rho_ps")}
            cmp[form].update(cstr_ratio=(np.array(r["cstr"]) / np.array(b["cstr"])).tolist(),
                             steps=r["steps"], tries=r["tries"], wall_s=r["wall_s"],
                             mt_per_s=r["mt_per_s"],
                             speedup_vs_base=b["wall_s"] / r["wall_s"])
        print(json.dumps(cmp), flush=True)
    return res


def config_params(which):
    """parameters.sh values of the reference's configurations 1 and 2:
    1 -- 32^3, RK4 at dt = 0.005 over t in [0, 50], a slice every 200 steps
         (every dt = 1);
    2 -- 64^3, DOPRI853 at rtol = atol = 1e-10 over t in [0, 200], GW
         spectrum with N/2 = 32 shells, a slice every 10 steps, timing on.
    Both: L = 20/m, phi^2 potential (m = 1), the seeded fluctuation data
    (amplitude 1e-3) from a .dat file, psi solved by the program."""
    from oracle import ref
    common = dict(SPATIAL_LOWER_BOUND_X=-10.0, SPATIAL_UPPER_BOUND_X=10.0,
                  SPATIAL_LOWER_BOUND_Y=-10.0, SPATIAL_UPPER_BOUND_Y=10.0,
                  SPATIAL_LOWER_BOUND_Z=-10.0, SPATIAL_UPPER_BOUND_Z=10.0,
                  OUTPUT_PHI=0, OUTPUT_DPHI=0, OUTPUT_PSI=0, OUTPUT_DPSI=0, OUTPUT_RHO=0,
                  MAX_RUNTIME=172500)
    if which == 1:
        return ref.config(GRIDPOINTS_X=32, GRIDPOINTS_Y=32, GRIDPOINTS_Z=32,
                          POWER_SPECTRUM_BINS=16, INTEGRATION_METHOD="RK4", DELTA_T=0.005,
                          FINAL_TIME=50.0, TIME_STEP_SKIPS=200, ENABLE_FOLLOWUP=0,
                          ENABLE_TIMING=0, **common)
    return ref.config(GRIDPOINTS_X=64, GRIDPOINTS_Y=64, GRIDPOINTS_Z=64, POWER_SPECTRUM_BINS=32,
                      INTEGRATION_METHOD="DOPRI853", RELATIVE_TOLERANCE=1e-10,
                      ABSOLUTE_TOLERANCE=1e-10, DELTA_T=1e-3, FINAL_TIME=200.0,
                      TIME_STEP_SKIPS=10, ENABLE_FOLLOWUP=1, ENABLE_TIMING=1, **common)


def config_run(which, seed=0):
    """Configuration 1 or 2 through the reference program (its own main(),
    this host's CPU cores) and through the same program relinked with the
    drop-in layer (the reference's main.c/setup.c/io.c + ih_dropin.o +
    libinstaheat_gpu.so, one GPU), from the same .dat data: wall times and
    the recorded datasets compared slice by slice (JSON line)."""
    from instaheat_gb300 import build as libbuild
    from instaheat_gb300 import dropin
    from oracle import oracle as orc
    from oracle import ref
    params = config_params(which)
    n = int(params["GRIDPOINTS_X"])
    o = orc.Oracle(n=(n,) * 3, L=(L_BOX,) * 3, bins=int(params["POWER_SPECTRUM_BINS"]))
    f0 = o.ic(seed=seed, amp=AMP, psi=False)
    o.close()
    exe = ref.build_dropin(params, libbuild.build(), dropin.HERE / "ih_dropin.c",
                           dropin.ROOT / "include")
    t0 = time.perf_counter()
    r, got = ref.run_program(exe, f0, exe.parent, timeout=7200)
    wall_gpu = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    t0 = time.perf_counter()
    want = ref.run(ref.build(params), "main", f0, timeout=14400)["h5"]
    wall_ref = time.perf_counter() - t0
    span = float(params["FINAL_TIME"]) - float(params["INITIAL_TIME"])
    out = {"config": which, "grid": n, "method": params["INTEGRATION_METHOD"], "span": span,
           "cores": os.cpu_count(), "seed": seed,
           "reference": {"runtime_total_s": float(want["runtime_total"][0]), "wall_s": wall_ref,
                         "mt_per_s": span / float(want["runtime_total"][0]),
                         "calls_rhs": float(want["calls_rhs"][0])},
           "dropin_gpu": {"runtime_total_s": float(got["runtime_total"][0]), "wall_s": wall_gpu,
                          "mt_per_s": span / float(got["runtime_total"][0]),
                          "calls_rhs": float(got["calls_rhs"][0])}}
    for k in ("runtime_stepper",):
        if k in want and k in got:
            for side, d in (("reference", want), ("dropin_gpu", got)):
                v = float(d[k][0])
                out[side][k + "_s"] = v
                if v > 0:
                    out[side]["mt_per_s_stepper"] = span / v
    for k in ("steps_total", "steps_ok", "steps_bad"):
        if k in want:
            out[k] = {"reference": float(want[k][0]), "dropin_gpu": float(got[k][0])}
    cmp = {}
    for k, w in want.items():
        if not isinstance(w, np.ndarray) or k.startswith("runtime") or k == "calls_rhs":
            continue
        g = got.get(k)
        if g is None or g.shape != w.shape:
            cmp[k] = {"shape": [list(np.shape(g)) if g is not None else None, list(w.shape)]}
            continue
        sc = np.abs(w).max()
        if w.ndim == 2 and w.shape[0] > 1:
            per = np.abs(g - w).max(axis=1) / np.maximum(np.abs(w).max(axis=1), 1e-300)
            cmp[k] = {"max_rel": float(per.max()), "first_rel": float(per[0]),
                      "last_rel": float(per[-1]), "slices": int(w.shape[0])}
        else:
            cmp[k] = {"max_rel": float(np.abs(g - w).max() / sc) if sc > 0 else 0.0}
    out["datasets"] = cmp
    if "time" in want:
        out["slice_times_equal"] = bool(got["time"].shape == want["time"].shape and
                                        np.allclose(got["time"], want["time"], rtol=1e-9))
    print(json.dumps(out), flush=True)
    return out


# ------------------------------------------------------------------ main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--accuracy-t", type=float, default=10.0,
                    help="span of the mixed-vs-FP64 accuracy check (0 disables)")
    # profiling and study legs
    ap.add_argument("--case-rhs", type=int, default=0)
    ap.add_argument("--case-steps", type=int, default=0)
    ap.add_argument("--grid", type=int, default=N_GRID)
    ap.add_argument("--prec", choices=["mixed", "f64"], default="mixed")
    ap.add_argument("--engine", type=int, default=None)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--rtol", type=float, default=RTOL)
    ap.add_argument("--dt-study", default=None)
    ap.add_argument("--gw-accuracy", type=float, default=0.0)
    ap.add_argument("--etas", default="0,64,256")
    ap.add_argument("--long-run", default=None, help="comma-separated checkpoint times")
    ap.add_argument("--forms", default="f64,mixed_pi,mixed_learned")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--box", type=float, default=L_BOX)
    ap.add_argument("--phi0", type=float, default=1.0)
    ap.add_argument("--model", default=None, help="proposer model file (default: the committed one)")
    ap.add_argument("--plane-probe", default=None,
                    help="comma-separated forms of the tensor sources' plane pass, timed alone")
    ap.add_argument("--config-run", type=int, default=0, choices=[0, 1, 2],
                    help="configuration 1 or 2 through the reference program and the relinked one")
    args = ap.parse_args()
    dist = Dist()
    if args.impl == "reference":
        reference_arm(args, dist)
        dist.close()
        return
    from instaheat_gb300 import build, gpu
    build.build()
    if args.case_rhs or args.case_steps:
        return case_workload(gpu, args)
    if args.plane_probe:
        return plane_probe(gpu, [int(x) for x in args.plane_probe.split(",")], args.steps)
    if args.dt_study is not None:
        return dt_study(gpu, args.grid, [float(x) for x in args.dt_study.split(",")], args.rtol)
    if args.gw_accuracy > 0:
        return gw_accuracy(gpu, args.grid, args.gw_accuracy,
                           [float(x) for x in args.etas.split(",")], args.rtol)
    if args.config_run:
        config_run(args.config_run, args.seed)
        return
    if args.long_run:
        long_run(gpu, args.grid, [float(x) for x in args.long_run.split(",")],
                 args.forms.split(","), args.seed, args.rtol, L=args.box, phi0=args.phi0,
                 model=args.model)
        return
    steps, warmup = args.steps, max(args.warmup, 3)
    device = dist.local if dist.ws > 1 else 0
    seed = dist.rank
    clocks = Clocks(device)
    from instaheat_gb300 import learned_dt
    proposer, _ = learned_dt.load(device=device)  # the committed trained model
    want_cpu = dist.rank == 0 and not args.no_cpu_baseline
    ctx, mixed = bench_form(gpu, gpu.PREC_MIXED, device, seed, steps, warmup, profile=True,
                            clocks=clocks, dist=dist, proposer=proposer, keep_start=want_cpu)
    e2e = bench_e2e(gpu, ctx, max(2, min(steps, 5)))
    ctx.close()
    f64 = None
    if not args.no_f64:
        c64, f64 = bench_form(gpu, gpu.PREC_F64, device, seed, max(2, min(steps, 3)), 3,
                              profile=True)
        c64.close()
    # whole-job figures (max time over ranks, sum of m*t)
    ms = dist.reduce(mixed["ms"], "max")
    mt_all = dist.reduce(mixed["mt"], "sum")
    value = mt_all / (ms / 1e3)
    e2e_val = dist.reduce(e2e["value"], "sum")
    peak, peak_src = load_peaks()
    fp64, fp64_src = fp64_peak(gpu, device)
    kern = mixed["kernels"]
    dom = max(kern.items(), key=lambda kv: kv[1][0])
    dname, (dms, dn, dbytes) = dom
    total_ms = sum(v[0] for v in kern.values())
    achieved = (dbytes / dn) / (dms / dn / 1e3) / 1e9 if dn else 0.0
    traffic = None
    tfile = ROOT / "profiles" / "traffic_256.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get(dname)
    acc = None
    if args.accuracy_t > 0 and not args.no_f64:
        acc = accuracy_check(device, seed, args.accuracy_t)
    cpu = cpu_baseline(mixed["start"]) if want_cpu else None
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": steps,
            "warmup": warmup, "ms_per_step": ms / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic: seeded fluctuation initial data (amp 1e-3), psi from the constraints",
            "config": {"workload": "256^3 box L=20/m, V=m^2 phi^2/2, DOPRI853 rtol=atol=1e-8, GW on, "
                                   "filter on; mixed FP32 fields/FFTs + FP64 k=0 parts, a, H, "
                                   "reductions and error norm; learned step-size proposer "
                                   "(DOPRI853 accepts/rejects every try)",
                       "grid": N_GRID, "rtol": RTOL, "atol": ATOL, "learned_dt": True,
                       "settle_t": 0.1,
                       "l2": "inputs larger than L2 (state 1.1 GB)",
                       "dt_next": mixed["dt_next"], "t_reached": mixed["t"],
                       "device_GB": mixed["device_bytes"] / 1e9,
                       "fft_engines": mixed["fft_engines"],
                       "fft_autotune": mixed["fft_autotune"]},
            "gpu_launches": mixed["launches"],
            "e2e": {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")}
                   | {"value": e2e_val},
            "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak,
                         "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "launches": dn,
                         "algorithmic_bytes_per_launch": dbytes / dn if dn else None,
                         "share_of_device_time": dms / total_ms if total_ms else None},
            "kernels_ms_per_step": {k: v[0] / steps for k, v in kern.items() if v[1]},
            # the whole step against compulsory traffic: 12 RHS x 11 transforms
            # (input read + output written once each) + the result write, and
            # 72 state-vector passes of the stepper, B_step = [12*15*(N + Next)
            # + 72*Ntot]*sizeof(float), over the device time of a step
            "step_roofline": step_roofline(ms / steps, peak, peak_src),
            "cpu_baseline": cpu,
            "clocks": mixed["clocks"],
        }
        if f64:
            f64v = f64["mt"] / (f64["ms"] / 1e3)
            ms64 = f64["ms"] / max(1, min(steps, 3))
            n64 = max(1, min(steps, 3))
            line["f64"] = {"value": f64v, "unit": UNIT, "ms_per_step": ms64,
                           "dt_next": f64["dt_next"],
                           "roofline": f64_roofline(ms64, peak, peak_src, fp64, fp64_src),
                           "kernels_ms_per_step": {k: v[0] / n64 for k, v in f64["kernels"].items()
                                                   if v[1]}}
            line["speedup_vs_f64"] = value / f64v
        if acc:
            line["accuracy_vs_f64"] = acc
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
