"""GPU tests of ensembles: member grids of different sizes, boxes and
precisions stepped together (ih_ensemble_run) follow exactly the step
sequences and states of the same runs done one context at a time."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MEMBERS = [
    dict(n=(16, 16, 16), L=(20.0, 20.0, 20.0), precision=1),
    dict(n=(32, 32, 32), L=(15.0, 15.0, 15.0), precision=1),
    dict(n=(32, 16, 16), L=(30.0, 15.0, 15.0), precision=0),
    dict(n=(16, 16, 16), L=(25.0, 25.0, 25.0), precision=0),
]
PHI0 = [1.0, 0.9, 1.1, 1.2]


def _setup(ctx, i, gpu_mod):
    ctx.ic(seed=100 + i, phi0=PHI0[i], amp=1e-3)


def test_ensemble_matches_single_runs(gpu_mod):
    tf = 0.08
    cfg = gpu_mod.dopri_cfg(1e-9, 1e-9)
    ens = gpu_mod.Ensemble(MEMBERS)
    for i, m in enumerate(ens.members):
        _setup(m, i, gpu_mod)
    ens.dopri_init(cfg, 0.0, 2e-3)
    rounds, steps = ens.run(tf)
    assert rounds >= max(1, steps // len(MEMBERS))
    total = 0
    for i, m in enumerate(MEMBERS):
        ctx = gpu_mod.Context(n=m["n"], L=m["L"], precision=m["precision"])
        _setup(ctx, i, gpu_mod)
        ctx.dopri_init(cfg, 0.0, 2e-3)
        n, _ = ctx.dopri_run(tf)
        total += n
        mem = ens.members[i]
        assert abs(mem.t - tf) < 1e-14 and abs(ctx.t - tf) < 1e-14
        c1, c2 = mem.dopri_counters(), ctx.dopri_counters()
        assert c1["dt_next"] == c2["dt_next"] and c1["tries"] == c2["tries"], (i, c1, c2)
        assert np.array_equal(mem.get_state(), ctx.get_state()), i
        ctx.close()
    assert steps == total
    ens.close()


def test_ensemble_autotune_shares_engines(gpu_mod):
    ens = gpu_mod.Ensemble(MEMBERS[:2] + [dict(MEMBERS[0])])
    ens.autotune()
    assert ens.members[0].engines() == ens.members[2].engines()
    ens.close()


def test_ensemble_with_radix3_members(gpu_mod):
    """Members of 24^3, 48^3 and 96^3 (the radix-3 sizes of the mixed-size
    ensembles) stepped together follow the single runs exactly."""
    members = [dict(n=(24, 24, 24), L=(20.0, 20.0, 20.0), precision=1),
               dict(n=(48, 48, 48), L=(30.0, 30.0, 30.0), precision=1),
               dict(n=(96, 96, 96), L=(40.0, 40.0, 40.0), precision=1),
               dict(n=(32, 32, 32), L=(10.0, 10.0, 10.0), precision=0)]
    tf = 0.05
    cfg = gpu_mod.dopri_cfg(1e-8, 1e-8)
    ens = gpu_mod.Ensemble(members)
    for i, m in enumerate(ens.members):
        m.ic(seed=200 + i, phi0=1.0 + 0.05 * i, amp=1e-3)
    ens.dopri_init(cfg, 0.0, 2e-3)
    ens.run(tf)
    for i, m in enumerate(members):
        ctx = gpu_mod.Context(n=m["n"], L=m["L"], precision=m["precision"])
        ctx.ic(seed=200 + i, phi0=1.0 + 0.05 * i, amp=1e-3)
        ctx.dopri_init(cfg, 0.0, 2e-3)
        ctx.dopri_run(tf)
        assert np.array_equal(ens.members[i].get_state(), ctx.get_state()), i
        ctx.close()
    ens.close()
