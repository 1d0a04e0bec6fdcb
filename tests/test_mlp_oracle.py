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
