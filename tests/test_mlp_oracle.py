"""CPU test: the numpy MLP oracle's gradient agrees with central finite
differences of its own loss (pins the checker of the GPU backward kernel)."""
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
