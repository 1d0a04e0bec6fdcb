"""CPU tests: the numpy MLP oracle's gradient agrees with central finite
differences of its own loss (pins the checker of the GPU backward kernel),
and the committed proposer model is consistent with the network."""
import numpy as np

from oracle import mlp_numpy as mn


def test_numpy_mlp_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(size=mn.NP) * 0.2
    X = rng.normal(size=(50, 12))
    Y = rng.normal(size=50)
    norm = (rng.normal(size=12), 0.5 + rng.random(12), 0.3, 1.7)
    g, _ = mn.gradients(p, X, Y, norm)
    idx = np.concatenate([rng.choice(mn.NP, 40, replace=False), [mn.NP - 1, mn.OFF_B1, mn.OFF_W3]])
    eps = 1e-6
    fd = []
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = mn.gradients(q, X, Y, norm)[1]
        q[i] -= 2 * eps
        lm = mn.gradients(q, X, Y, norm)[1]
        fd.append((lp - lm) / (2 * eps))
    assert np.max(np.abs(np.array(fd) - g[idx])) <= 1e-6 * np.abs(g[idx]).max()


def test_committed_proposer_model_is_consistent():
    """instaheat_gb300/data/dt_mlp.json (the model the bench loads): parameter
    count of the 12-64-64-1 network, finite values, positive input scales,
    the training record, and a plausible step size for the mean input."""
    import json
    from pathlib import Path
    d = json.loads((Path(__file__).resolve().parent.parent / "instaheat_gb300" / "data" /
                    "dt_mlp.json").read_text())
    p = np.array(d["params"])
    assert p.size == mn.NP == 5057 and np.all(np.isfinite(p))
    mean, std = np.array(d["in_mean"]), np.array(d["in_std"])
    assert mean.size == std.size == mn.NI and np.all(std > 0)
    meta = d["meta"]
    assert meta["rows"] > 0 and meta["rms_log_dt_error"] < 0.1
    assert {r["n"] for r in meta["runs"]} == {128, 256}
    y, _ = mn.forward(p, mean[None, :], (mean, std, d["out_mean"], d["out_std"]))
    assert np.isfinite(y).all() and 1e-4 < np.exp(y[0]) < 1.0


def test_training_pairs_from_saved_step_logs(tmp_path):
    """learned_dt.pairs_from_data: a step-log file that holds log dt targets
    is used as saved; one holding other targets is rebuilt from its FP64 step
    logs (features after replayed step k pair with log dt_{k+1}; the landing
    step of each run, shortened to hit t_end, gives no target)."""
    import json
    from instaheat_gb300 import learned_dt
    rng = np.random.default_rng(0)
    logs = [np.column_stack([np.arange(6.0), 0.01 * (1.0 + np.arange(6.0)), np.full(6, 0.4),
                             np.ones(6)]),
            np.column_stack([np.arange(4.0), 0.02 * (1.0 + np.arange(4.0)), np.full(4, 0.4),
                             np.ones(4)])]
    rows = np.array([5, 3])  # replayed steps per run (all but the landing step)
    X = rng.normal(size=(rows.sum(), 12)).astype(np.float32)
    p = tmp_path / "logs.npz"
    np.savez(p, X=X, Y=np.zeros(rows.sum(), np.float32), infos=json.dumps([{}, {}]), rows=rows,
             log0=logs[0], log1=logs[1])
    Xp, Yp = learned_dt.pairs_from_data(np.load(p))
    # run 0: k = 0..3 pair with dt_1..dt_4 (k = 4 would need the landing step);
    # run 1: k = 0, 1 with dt_1, dt_2
    want_x = np.concatenate([X[0:4], X[5:7]])
    want_y = np.log(np.concatenate([logs[0][1:5, 1], logs[1][1:3, 1]]))
    np.testing.assert_array_equal(Xp, want_x)
    np.testing.assert_allclose(Yp, want_y, rtol=1e-6)
    q = tmp_path / "pairs.npz"
    np.savez(q, X=X, Y=np.arange(rows.sum(), dtype=np.float32), target="log_dt")
    Xq, Yq = learned_dt.pairs_from_data(np.load(q))
    np.testing.assert_array_equal(Xq, X)
    np.testing.assert_array_equal(Yq, np.arange(rows.sum(), dtype=np.float32))
