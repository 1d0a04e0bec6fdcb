"""Ensemble benchmark: many seeded realizations of mixed grid sizes stepped
together (ih_ensemble_run) against the same realizations stepped one context
at a time.

Workload (seeded synthetic data): members of the listed sizes, box length L
drawn uniformly in [10, 40]/m and phi0 uniformly in [0.8, 1.2] from
numpy's default_rng(seed of the member), fluctuation amplitude 1e-3, psi from
the constraints, DOPRI853 rtol = atol = 1e-8, GW and filter on, the mixed
FP32/FP64 form, from t = 0 to --t-end.  Reports accepted steps per second and
m*t per second summed over members, for both ways, and the ensemble-mean GW
spectrum of each grid size.

    python -m instaheat_gb300.ensemble_bench --sizes 32:24,64:24,128:16 --t-end 0.2
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import gpu


def members_of(spec: str):
    out = []
    seed = 0
    for part in spec.split(","):
        n, cnt = (int(x) for x in part.split(":"))
        for _ in range(cnt):
            rng = np.random.default_rng(seed)
            L = float(rng.uniform(10.0, 40.0))
            phi0 = float(rng.uniform(0.8, 1.2))
            out.append(dict(n=(n, n, n), L=(L, L, L), precision=gpu.PREC_MIXED, seed=seed, phi0=phi0))
            seed += 1
    return out


def _prepare(ctx, m):
    ctx.ic(seed=m["seed"], phi0=m["phi0"], amp=1e-3)


def run(spec, t_end, rtol=1e-8, device=0):
    members = members_of(spec)
    cfg = gpu.dopri_cfg(rtol, rtol)
    ens = gpu.Ensemble([{k: m[k] for k in ("n", "L", "precision")} for m in members], device=device)
    ens.autotune()
    for ctx, m in zip(ens.members, members):
        _prepare(ctx, m)
    ens.dopri_init(cfg, 0.0, 1e-3)
    for ctx in ens.members:
        ctx.sync()
    t0 = time.perf_counter()
    rounds, steps = ens.run(t_end)
    wall_e = time.perf_counter() - t0
    gw = {}
    for ctx, m in zip(ens.members, members):
        gw.setdefault(m["n"][0], []).append(ctx.prepare_output()["gw"])
    ens.close()
    # the same members one context at a time (same engines: autotuned per size)
    engines = {}
    wall_s, steps_s = 0.0, 0
    for m in members:
        ctx = gpu.Context(n=m["n"], L=m["L"], precision=m["precision"], device=device)
        key = m["n"][0]
        if key not in engines:
            ctx.autotune()
            engines[key] = ctx.engines()
        else:
            for p, e in enumerate(engines[key]):
                ctx.set_engine(p, e)
        _prepare(ctx, m)
        ctx.dopri_init(cfg, 0.0, 1e-3)
        ctx.sync()
        t0 = time.perf_counter()
        n, _ = ctx.dopri_run(t_end)
        ctx.sync()
        wall_s += time.perf_counter() - t0
        steps_s += n
        ctx.close()
    mt = t_end * len(members)
    return {"members": len(members), "sizes": spec, "t_end": t_end, "rtol": rtol,
            "ensemble": {"wall_s": wall_e, "rounds": rounds, "steps": steps, "steps_per_s": steps / wall_e,
                         "mt_per_s": mt / wall_e},
            "one_at_a_time": {"wall_s": wall_s, "steps": steps_s, "steps_per_s": steps_s / wall_s,
                              "mt_per_s": mt / wall_s},
            "speedup": wall_s / wall_e,
            "gw_mean": {str(k): [float(x) for x in np.mean(v, axis=0)] for k, v in gw.items()}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="32:24,64:24,128:16", help="grid:count,...")
    ap.add_argument("--t-end", type=float, default=0.2)
    ap.add_argument("--rtol", type=float, default=1e-8)
    args = ap.parse_args(argv)
    print(json.dumps(run(args.sizes, args.t_end, args.rtol)), flush=True)


if __name__ == "__main__":
    main()
