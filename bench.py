#!/usr/bin/env python3
"""Benchmark: m*t advanced per wall-second at 256^3 on one GB300.

A step is one accepted DOPRI853 step (perform_step of src/dopri853.c:271-311:
every rejected try, the 12 RHS evaluations of each try, and the filtered
post-step RHS) of the 256^3 workload: box L = 20/m, V = m^2 phi^2 / 2, m = 1,
seeded fluctuation initial data (phi0 = 1, slow-roll dphi0, amplitude 1e-3,
psi from the constraints), GW on, filter on, DOPRI853 rtol = atol = 1e-8.

  value  -- m*t/s of the mixed FP32/FP64 form, state resident in HBM, timed
            with CUDA events on the context stream (inputs > L2: the state is
            1.1 GB, each stage reads >= 2 of them).
  e2e    -- the same through the public C ABI with host buffers: every step
            uploads the state from pinned host memory, steps, and downloads
            the new state.
  f64    -- the plain FP64 form on the same workload (the ratio the metric
            names), with its step against both of its bounds: algorithmic
            bytes vs the HBM copy peak, flops vs the FP64 pipe.
  roofline -- the kernel with the largest share of device time in the timed
            region: algorithmic bytes per launch / mean launch time (CUDA
            events around each launch), against the measured HBM copy peak.
  cpu_baseline -- the CPU oracle (C99 + OpenMP restatement of the reference)
            on this host's cores, one DOPRI853 step of the same workload.

--impl reference times that CPU path alone (the reference itself does not
build here: FFTW3, HDF5 and GSL are absent).  Under torchrun each rank runs an
independent realization (replicas only; no collective on the data path).
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
               proposer=None, t_settle=0.1):
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
           "t": ctx.t, "device_bytes": ctx.device_bytes,
           "fft_engines": dict(zip(("x", "y", "deriv4_x", "roundtrip_x", "roundtrip_y"),
                                   (ENGINE_NAMES[e] for e in ctx.engines()[:5])))
                          | {"tensor_x": ("fused" if ctx.engines()[5] else "separate"),
                             "z_fused": ("wide rows" if ctx.engines()[6] else "warp rows"),
                             "gw_yx_slab": ctx.engines()[7]},
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


# FP64 FMA rate of a GB300 (nominal; the pipe the FP64 form's FFTs run on)
FP64_NOMINAL_TFLOPS = 1.25


def f64_roofline(ms_per_step, peak, peak_src):
    """Both bounds of the plain FP64 form: its algorithmic bytes (the
    per-step formula at 8 bytes per value) against the HBM copy peak, and its
    flops -- 12 RHS x 11 transforms x 2.5 N log2 N plus about 160 Ntot in the
    stage combinations -- against the FP64 pipe."""
    n = N_GRID
    N = n ** 3
    Next = 2 * n * n * (n // 2 + 1)
    Ntot = 4 * N + 4 * Next + 1
    flops = 12 * 11 * 2.5 * N * np.log2(N) + 160 * Ntot
    tflops = flops / (ms_per_step / 1e3) / 1e12
    hbm = step_roofline(ms_per_step, peak, peak_src, elem=8)
    alu = {"flops_per_step": flops, "achieved": tflops, "peak": FP64_NOMINAL_TFLOPS,
           "peak_source": "nominal", "unit": "TFLOP/s", "frac": tflops / FP64_NOMINAL_TFLOPS,
           "floor_ms_per_step": flops / (FP64_NOMINAL_TFLOPS * 1e12) * 1e3}
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


def cpu_baseline_sample(threads=None):
    """One DOPRI853 step of the 256^3 workload with the CPU oracle."""
    from oracle import oracle as orc
    threads = threads or os.cpu_count()
    o = orc.Oracle(n=(N_GRID,) * 3, L=(L_BOX,) * 3, threads=threads)
    f = o.ic(seed=0, amp=AMP)
    cfg = orc.default_cfg(RTOL, ATOL, 1e-2)
    st, df = o.dopri_init(f, cfg, 0.0, 1e-3)
    o.dopri_step(f, df, cfg, st, 1e-3)   # first step from the workload's dt0
    dt = st.dt_next
    t0 = time.perf_counter()
    o.dopri_step(f, df, cfg, st, dt)
    wall = time.perf_counter() - t0
    res = {"value": st.dt_did / wall, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"one DOPRI853 step of the 256^3 workload (dt={st.dt_did:.4g}, "
                     f"{st.tries} tries incl. the first step) with the C99+OpenMP oracle, "
                     f"{wall:.1f} s", "seconds": wall}
    o.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--accuracy-t", type=float, default=0.5,
                    help="span of the mixed-vs-FP64 accuracy check (0 disables)")
    args = ap.parse_args()
    steps, warmup = args.steps, max(args.warmup, 3) if args.impl == "ours" else args.warmup
    dist = Dist()
    if args.impl == "reference":
        if dist.rank == 0:
            res = cpu_baseline_sample()
            line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT,
                    "n_gpus": args.gpus, "steps": 1, "warmup": 1,
                    "ms_per_step": 1e3 * res["seconds"], "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                    "config": {"workload": "256^3 DOPRI853 rtol=atol=1e-8, L=20/m, phi^2, GW+filter",
                               "grid": N_GRID},
                    "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
                    "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}}
            print(json.dumps(line), flush=True)
        dist.close()
        return

    from instaheat_gb300 import build, gpu
    build.build()
    device = dist.local if dist.ws > 1 else 0
    seed = dist.rank
    clocks = Clocks(device)
    from instaheat_gb300 import learned_dt
    proposer, _ = learned_dt.load(device=device)  # the committed trained model
    ctx, mixed = bench_form(gpu, gpu.PREC_MIXED, device, seed, steps, warmup, profile=True,
                            clocks=clocks, dist=dist, proposer=proposer)
    e2e = bench_e2e(gpu, ctx, max(2, min(steps, 5)))
    ctx.close()
    f64 = None
    if not args.no_f64:
        c64, f64 = bench_form(gpu, gpu.PREC_F64, device, seed, max(2, min(steps, 3)), 3)
        c64.close()
    # whole-job figures (max time over ranks, sum of m*t)
    ms = dist.reduce(mixed["ms"], "max")
    mt_all = dist.reduce(mixed["mt"], "sum")
    value = mt_all / (ms / 1e3)
    e2e_val = dist.reduce(e2e["value"], "sum")
    peak, peak_src = load_peaks()
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
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample()
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
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
            line["f64"] = {"value": f64v, "unit": UNIT, "ms_per_step": ms64,
                           "dt_next": f64["dt_next"],
                           "roofline": f64_roofline(ms64, peak, peak_src)}
            line["speedup_vs_f64"] = value / f64v
        if acc:
            line["accuracy_vs_f64"] = acc
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
