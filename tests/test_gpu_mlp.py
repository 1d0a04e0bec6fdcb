"""GPU tests of the learned step-size proposer's kernels (ih_mlp.cu) against the
numpy oracle (oracle/mlp_numpy.py), and of what the trained proposer gains."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODEL = Path(__file__).resolve().parent.parent / "instaheat_gb300" / "data" / "dt_mlp.json"


def _net(gpu_mod, seed=3):
    rng = np.random.default_rng(seed)
    mlp = gpu_mod.MLP(seed=seed)
    mean = rng.normal(size=12).astype(np.float32)
    std = (0.5 + rng.random(12)).astype(np.float32)
    mlp.set_norm(mean, std, -4.0, 0.7)
    X = (mean + std * rng.normal(size=(300, 12))).astype(np.float32)
    Y = (-4.0 + 0.7 * rng.normal(size=300)).astype(np.float32)
    return mlp, X, Y


def test_mlp_forward_matches_numpy(gpu_mod):
    from oracle import mlp_numpy as mn
    mlp, X, _ = _net(gpu_mod)
    y = mlp.forward(X)
    ref, _ = mn.forward(mlp.bf16_params(), X, mlp.norm)
    assert np.abs(y - ref).max() <= 1e-4 * np.abs(ref).max()


def test_mlp_gradients_match_numpy(gpu_mod):
    """Backward kernel vs the float64 numpy gradient on the same BF16 weights:
    relative L2 error of the whole gradient within 1e-4 (FP32 accumulation)."""
    from oracle import mlp_numpy as mn
    mlp, X, Y = _net(gpu_mod)
    g, loss = mlp.gradients(X, Y)
    gr, lr = mn.gradients(mlp.bf16_params(), X, Y, mlp.norm)
    assert abs(loss - lr) <= 1e-4 * lr
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)
    # every block of the gradient is non-trivial and matches
    for a, b in [(0, 768), (768, 832), (832, 4928), (4928, 4992), (4992, 5056), (5056, 5057)]:
        assert np.linalg.norm(g[a:b] - gr[a:b]) <= 1e-3 * max(np.linalg.norm(gr[a:b]), 1e-12)


def test_mlp_training_fits_a_smooth_target(gpu_mod):
    rng = np.random.default_rng(0)
    X = rng.normal(size=(2000, 12)).astype(np.float32)
    Y = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * X[:, 5]).astype(np.float32)
    mlp = gpu_mod.MLP(seed=1)
    mlp.set_norm(X.mean(0), X.std(0), float(Y.mean()), float(Y.std()))
    hist = mlp.train(X, Y, iters=1500, batch=128, lr=3e-3)
    assert hist[-100:].mean() < 0.05 * hist[:20].mean()
    pred = mlp.forward(X)
    assert np.sqrt(np.mean((pred - Y) ** 2)) < 0.2 * Y.std()


@pytest.mark.skipif(not MODEL.exists(), reason="trained proposer not present")
def test_learned_proposer_gain_over_controller_alone(gpu_mod):
    """At 128^3 (held-out seed 0, t in [0, 0.5]) the mixed form with the
    trained proposer follows the FP64 step policy: its GW spectrum is within
    1% of the FP64 run and no further from it than the mixed form with the
    controller alone (to 0.1%), and its step count is within 10% of FP64's
    or no further from it than the controller's; DOPRI853 still
    accepts/rejects every try."""
    from instaheat_gb300 import learned_dt
    r = learned_dt.evaluate(128, 0, 0.5, MODEL)
    assert r["mixed_learned"]["gw_max_rel_vs_f64"] < 0.01, r
    assert r["mixed_learned"]["gw_max_rel_vs_f64"] <= r["mixed_pi"]["gw_max_rel_vs_f64"] + 1e-3, r
    n64 = r["f64"]["steps"]
    assert abs(r["mixed_learned"]["steps"] - n64) <= max(abs(r["mixed_pi"]["steps"] - n64),
                                                         0.1 * n64), r


def test_proposal_replaces_the_controller_step(gpu_mod):
    """After each accepted step the proposal (the network's log dt) replaces
    the controller's next step, clamped to [minscale, maxscale] x dt and to
    the Hubble cap: a network that always proposes 2e-3 (zero weights, output
    mean log 2e-3) makes every step after the first 2e-3, below the cap of
    about 1.9e-2; DOPRI853 still accepts each try on its own error estimate."""
    mlp = gpu_mod.MLP(seed=1)
    mlp.params = np.zeros_like(mlp.params)
    mlp.set_norm(np.zeros(12, np.float32), np.ones(12, np.float32), float(np.log(2e-3)), 1.0)
    ctx = gpu_mod.Context(n=(32, 32, 32), precision=gpu_mod.PREC_MIXED)
    ctx.ic(seed=0, amp=1e-3)
    ctx.dopri_init(gpu_mod.dopri_cfg(1e-8, 1e-8), 0.0, 1e-3)
    ctx.set_proposer(mlp)
    _, log = ctx.dopri_run(0.03, log_cap=1000)
    ctx.close()
    dts, tries = log[:, 1], log[:, 3]
    assert log.shape[0] >= 10 and np.all(tries == 1), log
    assert dts[0] == 1e-3
    # FP32 network output: exp(log 2e-3) to 1e-6 relative; the last step lands on t = 0.03
    np.testing.assert_allclose(dts[1:-1], 2e-3, rtol=1e-6)
