"""Run a fixed number of RHS evaluations (or DOPRI853 steps) of the seeded
workload on one GPU -- the command the ncu captures under profiles/ use.

    python -m instaheat_gb300.profile_case --n 256 --prec mixed --rhs 3
    python -m instaheat_gb300.profile_case --n 256 --prec mixed --steps 2
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


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--prec", choices=["mixed", "f64"], default="mixed")
    ap.add_argument("--rhs", type=int, default=0, help="RHS evaluations on the device state")
    ap.add_argument("--steps", type=int, default=0, help="DOPRI853 steps")
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--dt-study", default=None, help="comma-separated eta values")
    args = ap.parse_args(argv)
    if args.dt_study is not None:
        dt_study(args.n, [float(x) for x in args.dt_study.split(",")], args.rtol)
        return
    prec = gpu.PREC_MIXED if args.prec == "mixed" else gpu.PREC_F64
    ctx = gpu.Context(n=(args.n,) * 3, precision=prec)
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
