"""Run a fixed number of RHS evaluations (or DOPRI853 steps) of the seeded
workload on one GPU -- the command the ncu captures under profiles/ use.

    python -m instaheat_gb300.profile_case --n 256 --prec mixed --rhs 3
    python -m instaheat_gb300.profile_case --n 256 --prec mixed --steps 2
    python -m instaheat_gb300.profile_case --n 256 --prec mixed --rhs 2 --autotune
    python -m instaheat_gb300.profile_case --n 256 --dt-study 0,32,256,2048

--dt-study runs 12 DOPRI853 steps of the FP64 form and of the mixed form
for each listed rounding-floor factor eta and prints, per run, the step size
reached and the per-segment error sums of the last try (JSON lines).
"""
from __future__ import annotations

import argparse
import json

from . import gpu


def dt_study(n, etas, rtol, steps=12):
    runs = [(gpu.PREC_F64, 0.0)] + [(gpu.PREC_MIXED, e) for e in etas]
    for prec, eta in runs:
        ctx = gpu.Context(n=(n,) * 3, precision=prec)
        ctx.ic(seed=0, amp=1e-3)
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


def gw_accuracy(n, t_end, etas, rtol):
    """GW spectrum and constraints at t_end of the FP64 form (rtol and a
    100x tighter reference) and of the mixed form for each eta."""
    import numpy as np

    def run(prec, eta, tol):
        ctx = gpu.Context(n=(n,) * 3, precision=prec)
        ctx.ic(seed=0, amp=1e-3)
        ctx.set_noise_floor(eta)
        ctx.dopri_init(gpu.dopri_cfg(tol, tol), 0.0, 1e-3)
        steps, _ = ctx.dopri_run(t_end)
        d = ctx.prepare_output()
        ctx.close()
        return steps, d

    ref_steps, ref = run(gpu.PREC_F64, 0.0, rtol / 100)
    gref = ref["gw"]
    sig = gref > 1e-3 * gref.max()
    print(json.dumps({"case": "f64_ref", "rtol": rtol / 100, "steps": ref_steps,
                      "gw": [float(x) for x in gref], "cstr": [float(x) for x in ref["cstr"]]}),
          flush=True)
    # replay: the mixed form retraces the FP64 run's accepted steps exactly
    # (same step sizes, hence the same number of filter applications)
    c64 = gpu.Context(n=(n,) * 3, precision=gpu.PREC_F64)
    c64.ic(seed=0, amp=1e-3)
    c64.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
    steps64, log = c64.dopri_run(t_end, log_cap=100000)
    d64 = c64.prepare_output()
    c64.close()
    cm = gpu.Context(n=(n,) * 3, precision=gpu.PREC_MIXED)
    cm.ic(seed=0, amp=1e-3)
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
        print(json.dumps({"case": "f64" if prec == gpu.PREC_F64 else "mixed", "eta": eta, "rtol": rtol,
                          "steps": steps, "gw_max_rel_sig": float(rel[sig].max()),
                          "gw_rel": [float(x) for x in rel], "cstr": [float(x) for x in d["cstr"]]}),
              flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--prec", choices=["mixed", "f64"], default="mixed")
    ap.add_argument("--rhs", type=int, default=0, help="RHS evaluations on the device state")
    ap.add_argument("--steps", type=int, default=0, help="DOPRI853 steps")
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--dt-study", default=None, help="comma-separated eta values")
    ap.add_argument("--gw-accuracy", type=float, default=0.0, help="t_end of the GW accuracy study")
    ap.add_argument("--etas", default="0,64,256", help="eta values of the GW accuracy study")
    ap.add_argument("--engine", type=int, default=None,
                    help="FFT engine of the x/y passes (0 Stockham .. 4 three-step)")
    ap.add_argument("--autotune", action="store_true",
                    help="the autotuner's engines, kept in and reused from the FFT wisdom file")
    args = ap.parse_args(argv)
    if args.gw_accuracy > 0:
        gw_accuracy(args.n, args.gw_accuracy, [float(x) for x in args.etas.split(",")], args.rtol)
        return
    if args.dt_study is not None:
        dt_study(args.n, [float(x) for x in args.dt_study.split(",")], args.rtol)
        return
    prec = gpu.PREC_MIXED if args.prec == "mixed" else gpu.PREC_F64
    ctx = gpu.Context(n=(args.n,) * 3, precision=prec)
    if args.engine is not None:  # pin the x/y (and, where it exists, fused x) FFT engine
        for p in range(3):
            if not (p == 2 and args.engine in (gpu.FFT_THREESTEP, gpu.FFT_TWOSTEP_HALF_OCC)):
                ctx.set_engine(p, args.engine)
    elif args.autotune:
        print(ctx.autotune(wisdom=True), flush=True)
    ctx.ic(seed=0, amp=1e-3)
    ctx.dopri_init(gpu.dopri_cfg(args.rtol, args.rtol), 0.0, 1e-3)   # one filtered RHS
    for _ in range(args.rhs):
        ctx.dopri_init(gpu.dopri_cfg(args.rtol, args.rtol), 0.0, 1e-3)
    dt = 1e-3
    for _ in range(args.steps):
        dt = ctx.dopri_step(dt).dt_next
    ctx.sync()
    print(f"done: n={args.n} prec={args.prec} rhs={ctx.calls_rhs} launches={ctx.kernel_launches}")
    ctx.close()


if __name__ == "__main__":
    main()
