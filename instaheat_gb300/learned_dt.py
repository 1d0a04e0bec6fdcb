"""The learned step-size proposer: step logs, GPU training, model files.

Why it exists: the mixed-precision form's DOPRI853 error estimate is mostly
below FP32 resolution at rtol = atol = 1e-8 (the embedded error of a step is
far smaller than the FP32 rounding of the stage sums it is formed from, and
the noise floor that keeps round-off from rejecting steps removes it), so its
controller alone does not reproduce the FP64 form's step sequence, and the
reference's per-step spectral filter makes the solution depend on that
sequence (the filter is applied once per accepted step, so the number of
steps sets how strongly the highest modes are damped).  The proposer is
trained to propose the FP64 form's next step size from what the mixed form
itself observes; DOPRI853 still accepts or rejects every try and the
reference controller handles rejections.

Step logs: for each run, the FP64 form runs with its own controller and logs
its accepted steps (t, dt, err, tries); the mixed form then replays exactly
those steps and records, after every step, its feature vector
(ih_step_features: last four log dt, last four log error norms, log a, H,
log rms delta phi, log rms delta psi).  Training pairs: features after step
n -> log dt_{n+1} of FP64.

    python -m instaheat_gb300.learned_dt --n 128,256 --seeds 1,2,3 --t-end 1.0 \\
        --out instaheat_gb300/data/dt_mlp.json [--save-data logs.npz]
    python -m instaheat_gb300.learned_dt --from-data logs.npz --out model.json

Runs are given as grids x seeds (box 20/m, phi0 = 1) or, with --runs, as
grid:seed:box:phi0 entries (box L in units of 1/m, phi0 the homogeneous
field).

Replayed FP64 trajectories only show the network states on that trajectory,
where "keep the last step" is nearly right; once its own proposals move the
mixed form off it, nothing in the data says how to come back.  --dagger R
adds R rounds of data from the mixed form running on the current proposer:
before each of its steps the state is handed to an FP64 context, which takes
the same step from it with the reference controller; the pair is (the mixed
form's features after its step, log of the FP64 controller's next step).
After each round the network is retrained on all pairs.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import gpu

DEFAULT_MODEL = Path(__file__).resolve().parent / "data" / "dt_mlp.json"
FORMAT = "instaheat_gb300 dt proposer v1"


def step_log(n, seed, t_end, rtol=1e-8, device=0, amp=1e-3, L=20.0, phi0=1.0):
    """(X, Y, info, log64) for one realization: mixed-form features replaying
    FP64, targets log dt of the FP64 run's next step, and the FP64 step log."""
    c64 = gpu.Context(n=(n,) * 3, L=(L,) * 3, precision=gpu.PREC_F64, device=device)
    c64.ic(seed=seed, amp=amp, phi0=phi0)
    c64.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
    t0 = time.perf_counter()
    steps, log = c64.dopri_run(t_end, log_cap=1_000_000)
    w64 = time.perf_counter() - t0
    c64.close()
    dts = log[:, 1]
    cm = gpu.Context(n=(n,) * 3, L=(L,) * 3, precision=gpu.PREC_MIXED, device=device)
    cm.ic(seed=seed, amp=amp, phi0=phi0)
    cm.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
    X, Y = [], []
    replayed = 0
    for k in range(len(dts) - 1):
        info = cm.dopri_step(dts[k])
        if info.tries != 1 or info.dt_did != dts[k]:
            break  # the mixed form rejected a FP64 step: the replay ends here
        replayed += 1
        if k + 1 < len(dts) - 1:  # the last FP64 step is truncated to land on t_end
            X.append(cm.step_features())
            Y.append(np.log(dts[k + 1]))
    cm.close()
    return (np.array(X, dtype=np.float32).reshape(-1, gpu.MLP_INPUTS), np.array(Y, dtype=np.float32),
            {"n": n, "seed": seed, "L": L, "phi0": phi0, "t_end": t_end, "steps_f64": int(steps),
             "replayed": replayed, "wall_f64_s": w64}, log)


def dagger_log(n, seed, t_end, mlp, rtol=1e-8, device=0, amp=1e-3, L=20.0, phi0=1.0,
               every=1, max_steps=5000):
    """(X, Y, info) from the mixed form running on the proposer `mlp`: for
    each of its steps (every `every`-th), the FP64 controller's next step
    after the same step from the same state, paired with the mixed form's
    features after its step.  At most max_steps mixed steps."""
    cfg = gpu.dopri_cfg(rtol, rtol)
    cm = gpu.Context(n=(n,) * 3, L=(L,) * 3, precision=gpu.PREC_MIXED, device=device)
    cm.ic(seed=seed, amp=amp, phi0=phi0)
    cm.dopri_init(cfg, 0.0, 1e-3)
    cm.set_proposer(mlp)
    c64 = gpu.Context(n=(n,) * 3, L=(L,) * 3, precision=gpu.PREC_F64, device=device)
    X, Y = [], []
    t, dt, k = 0.0, 1e-3, 0
    t0 = time.perf_counter()
    while t < t_end and k < max_steps:
        last = t + dt * 1.0001 > t_end  # the step landing on t_end: no pair
        if last:
            dt = t_end - t
        take = (k % every == 0) and not last
        if take:
            c64.set_state(cm.get_state(), t)
            c64.dopri_init(cfg, t, dt)
            dt64 = c64.dopri_step(dt).dt_next
        info = cm.dopri_step(dt)
        if take and info.tries == 1 and dt64 > 0:
            X.append(cm.step_features())
            Y.append(np.log(dt64))
        t, dt, k = info.t, info.dt_next, k + 1
    cm.close()
    c64.close()
    return (np.array(X, dtype=np.float32).reshape(-1, gpu.MLP_INPUTS), np.array(Y, dtype=np.float32),
            {"n": n, "seed": seed, "L": L, "phi0": phi0, "t_end": t_end, "t_reached": t,
             "mixed_steps": k, "pairs": len(X), "wall_s": time.perf_counter() - t0})


def pairs_from_data(z):
    """Training pairs of a saved step-log file: (X, Y) as saved when the file
    holds log dt targets, else rebuilt from the FP64 step logs (rows k of a
    run pair with log dt_{k+1}, the run's landing step excluded)."""
    target = str(z["target"]) if "target" in z.files else ""
    if target == "log_dt":
        return z["X"], z["Y"]
    X, Y, off = [], [], 0
    for i, r in enumerate(z["rows"]):
        dts = z[f"log{i}"][:, 1]
        for k in range(int(r)):
            if k + 1 < len(dts) - 1:
                X.append(z["X"][off + k])
                Y.append(np.log(dts[k + 1]))
        off += int(r)
    return np.array(X, dtype=np.float32), np.array(Y, dtype=np.float32)


def fit(X, Y, device=0, iters=3000, lr=3e-3, seed=1):
    mean = X.mean(axis=0)
    std = np.maximum(X.std(axis=0), 1e-3)
    om, osd = float(Y.mean()), float(max(Y.std(), 1e-3))
    mlp = gpu.MLP(device=device, seed=seed)
    mlp.set_norm(mean, std, om, osd)
    hist = mlp.train(X, Y, iters=iters, batch=128, lr=lr, seed=seed)
    return mlp, hist


def save(mlp, path, meta=None):
    m, s, om, osd = mlp.norm
    d = {"format": FORMAT, "params": [float(x) for x in mlp.params],
         "in_mean": [float(x) for x in m], "in_std": [float(x) for x in s],
         "out_mean": om, "out_std": osd, "meta": meta or {}}
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    Path(path).write_text(json.dumps(d))


def load(path=DEFAULT_MODEL, device=0):
    d = json.loads(Path(path).read_text())
    if d.get("format") != FORMAT:
        raise ValueError(f"{path}: a model of format {d.get('format')!r}; this library reads "
                         f"{FORMAT!r}")
    mlp = gpu.MLP(device=device)
    mlp.params = np.array(d["params"], dtype=np.float32)
    mlp.set_norm(np.array(d["in_mean"]), np.array(d["in_std"]), d["out_mean"], d["out_std"])
    return mlp, d.get("meta", {})


# the largest grid the FP64 form runs (its FFT tiles)
F64_MAX_N = 512


def evaluate(n, seed, t_end, model=DEFAULT_MODEL, rtol=1e-8, device=0, amp=1e-3):
    """FP64 with its controller, mixed with the controller alone, and mixed
    with the proposer, all to t_end from the same data: accepted steps, tries,
    wall time, and the GW spectrum / constraints against the FP64 run.  Above
    F64_MAX_N there is no FP64 run: the proposer is compared with the mixed
    form under the controller alone (key gw_max_rel_vs_ref, ref "mixed_pi")."""
    runs = {}
    mlp, _ = load(model, device)
    plan = [("f64", gpu.PREC_F64, None), ("mixed_pi", gpu.PREC_MIXED, None),
            ("mixed_learned", gpu.PREC_MIXED, mlp)]
    ref = "f64"
    if n > F64_MAX_N:
        plan = plan[1:]
        ref = "mixed_pi"
    for name, prec, prop in plan:
        ctx = gpu.Context(n=(n,) * 3, precision=prec, device=device)
        ctx.ic(seed=seed, amp=amp)
        ctx.dopri_init(gpu.dopri_cfg(rtol, rtol), 0.0, 1e-3)
        if prop is not None:
            ctx.set_proposer(prop)
        ctx.sync()
        t0 = time.perf_counter()
        steps, _ = ctx.dopri_run(t_end)
        ctx.sync()
        wall = time.perf_counter() - t0
        d = ctx.prepare_output()
        runs[name] = {"steps": int(steps), "tries": int(ctx.dopri_counters()["tries"]), "wall_s": wall,
                      "gw": d["gw"], "cstr": d["cstr"]}
        ctx.close()
    g64 = runs[ref]["gw"]
    sig = g64 > 1e-3 * g64.max()
    out = {"n": n, "seed": seed, "t_end": t_end, "ref": ref}
    key = "gw_max_rel_vs_f64" if ref == "f64" else "gw_max_rel_vs_ref"
    for k, r in runs.items():
        rel = np.abs(r["gw"] - g64)[sig] / g64[sig]
        out[k] = {"steps": r["steps"], "tries": r["tries"], "wall_s": r["wall_s"],
                  "mt_per_s": t_end / r["wall_s"], key: float(rel.max()),
                  "cstr": [float(x) for x in r["cstr"]]}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--evaluate", action="store_true", help="evaluate the saved model")
    ap.add_argument("--eval-n", type=int, default=256)
    ap.add_argument("--eval-seed", type=int, default=0)
    ap.add_argument("--eval-t", type=float, default=0.5)
    ap.add_argument("--n", default="128,256")
    ap.add_argument("--seeds", default="1,2,3")
    ap.add_argument("--runs", default=None,
                    help="grid:seed:box:phi0 entries (comma-separated); overrides --n/--seeds")
    ap.add_argument("--t-end", type=float, default=1.0)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=str(DEFAULT_MODEL))
    ap.add_argument("--save-data", default=None, help="write the step logs and pairs (.npz)")
    ap.add_argument("--from-data", default=None, help="train on saved step logs (.npz)")
    ap.add_argument("--dagger", type=int, default=0, help="rounds on the proposer's own states")
    ap.add_argument("--dagger-every", type=int, default=1)
    ap.add_argument("--dagger-max-steps", type=int, default=3000)
    ap.add_argument("--dagger-t-end", type=float, default=None,
                    help="end time of the rounds' runs (default: that of the replays)")
    ap.add_argument("--dagger-repeat", type=int, default=1,
                    help="weight of the rounds' pairs (each enters the training set this often)")
    args = ap.parse_args(argv)
    if args.evaluate:
        print(json.dumps(evaluate(args.eval_n, args.eval_seed, args.eval_t, args.out)), flush=True)
        return
    runs = None
    if args.runs:
        runs = [(int(a), int(b), float(c), float(d))
                for a, b, c, d in (r.split(":") for r in args.runs.split(","))]
    if args.from_data:
        z = np.load(args.from_data)
        X, Y = pairs_from_data(z)
        infos = json.loads(str(z["infos"]))
        if runs is None:  # the replayed runs of the file (not its earlier rounds)
            runs = [(i["n"], i["seed"], i["L"], i["phi0"]) for i in infos if "round" not in i]
    else:
        Xs, Ys, infos, logs = [], [], [], []
        if runs is None:
            runs = [(int(n), int(sd), 20.0, 1.0) for n in args.n.split(",")
                    for sd in args.seeds.split(",")]
        for n, sd, L, phi0 in runs:
            X, Y, info, log = step_log(n, sd, args.t_end, L=L, phi0=phi0)
            print(json.dumps(info), flush=True)
            Xs.append(X)
            Ys.append(Y)
            infos.append(info)
            logs.append(log)
        X = np.concatenate(Xs)
        Y = np.concatenate(Ys)
        if args.save_data:
            np.savez(args.save_data, X=X, Y=Y, infos=json.dumps(infos), target="log_dt",
                     rows=np.array([len(x) for x in Xs]), **{f"log{i}": lg for i, lg in enumerate(logs)})
    mlp, hist = fit(X, Y, iters=args.iters, lr=args.lr)
    t_end = infos[0]["t_end"] if infos else args.t_end
    t_round = args.dagger_t_end if args.dagger_t_end is not None else t_end
    prior = len({i["round"] for i in infos if "round" in i})  # rounds already in --from-data
    for rnd in range(args.dagger):
        for n, sd, L, phi0 in runs:
            Xd, Yd, info = dagger_log(n, sd, t_round, mlp, L=L, phi0=phi0, every=args.dagger_every,
                                      max_steps=args.dagger_max_steps)
            info["round"] = prior + rnd
            info["repeat"] = args.dagger_repeat
            print(json.dumps(info), flush=True)
            infos.append(info)
            X = np.concatenate([X] + [Xd] * args.dagger_repeat)
            Y = np.concatenate([Y] + [Yd] * args.dagger_repeat)
        mlp.close()
        mlp, hist = fit(X, Y, iters=args.iters, lr=args.lr)
        if rnd + 1 < args.dagger:  # the model of each intermediate round, for comparison
            save(mlp, args.out.replace(".json", f"_round{rnd}.json"),
                 {"rows": int(len(X)), "dagger_rounds": rnd + 1})
        if args.save_data:
            np.savez(args.save_data.replace(".npz", f"_dagger{rnd}.npz"), X=X, Y=Y,
                     infos=json.dumps(infos), target="log_dt")
    pred = mlp.forward(X)
    rms = float(np.sqrt(np.mean((pred - Y) ** 2)))
    meta = {"rows": int(len(X)), "runs": infos, "t_end": t_end,
            "dagger_rounds": prior + args.dagger,
            "iters": args.iters, "lr": args.lr, "final_loss": float(hist[-50:].mean()),
            "rms_log_dt_error": rms}
    save(mlp, args.out, meta)
    print(json.dumps({"saved": args.out, "rows": len(X), "loss_first": float(hist[:50].mean()),
                      "loss_last": float(hist[-50:].mean()), "rms_log_dt_error": rms}), flush=True)


if __name__ == "__main__":
    main()
