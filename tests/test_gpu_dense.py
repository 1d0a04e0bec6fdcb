"""GPU: DOPRI853 dense output (ih_dopri853_dense) against the oracle's
continuous extension of the same step (oracle/ih_oracle.c dense_output).

Tolerances: FP64 interpolated state within 1e-10 of each segment's largest
magnitude (three more RHS evaluations and two combinations on top of the
step's 1e-11); the mixed form within 1e-4 of each field segment's
fluctuation scale (as its DOPRI853 steps); diagnostics as the FP64 RHS
parity test."""
import numpy as np
import pytest

from test_gpu_parity import make_state, seg_rel_err

pytestmark = pytest.mark.gpu

THETAS = [0.0, 0.3, 0.75, 1.0]


def _step_both(gpu_mod, oracle_mod, n, precision, seed, dt, velocity_form=True):
    ctx = gpu_mod.Context(n=n, precision=precision)
    ctx.velocity_form(velocity_form)
    o = oracle_mod.Oracle(n=n)
    f = make_state(o, seed=seed)
    cfg_o = oracle_mod.default_cfg(1e-9, 1e-9, 1e-2)
    cfg_g = gpu_mod.dopri_cfg(1e-9, 1e-9, max_dt_hubble_fraction=1e-2)
    ctx.set_state(f)
    ctx.dopri_init(cfg_g, 0.0, dt)
    fo = f.copy()
    st, dfo = o.dopri_init(fo, cfg_o, 0.0, dt)
    t0 = ctx.t
    info = ctx.dopri_step(dt)
    rc, dense = o.dopri_step_dense(fo, dfo, cfg_o, st, dt, THETAS)
    assert rc == 0 and info.tries == 1 and st.dt_did == dt and info.dt_did == dt
    return ctx, o, fo, dense, t0, info.dt_did


def test_dense_f64_matches_oracle(gpu_mod, oracle_mod):
    n = (32, 32, 32)
    ctx, o, fo, dense, t0, h = _step_both(gpu_mod, oracle_mod, n, gpu_mod.PREC_F64, 6, 5e-2)
    state = ctx.get_state()
    for q, th in enumerate(THETAS):
        got = ctx.dopri_dense(t0 + th * h)
        errs = seg_rel_err(got, dense[q], o.N, o.Next)
        assert max(errs.values()) < 1e-10, (th, errs)
    # the context's own state is untouched; theta = 1 is the step's end state
    assert np.array_equal(ctx.get_state(), state)
    errs = seg_rel_err(ctx.dopri_dense(t0 + h), state, o.N, o.Next)
    assert max(errs.values()) < 1e-13, errs


@pytest.mark.parametrize("velocity_form", [True, False])
def test_dense_mixed_tracks_f64_oracle(gpu_mod, oracle_mod, velocity_form):
    """Mixed form: the interpolant of a velocity-form step (stages 6..12
    restored from their velocity halves) or of a reference-form step."""
    n = (32, 32, 32)
    ctx, o, fo, dense, t0, h = _step_both(gpu_mod, oracle_mod, n, gpu_mod.PREC_MIXED, 7, 5e-2,
                                          velocity_form)
    N = o.N
    for q, th in enumerate(THETAS):
        got = ctx.dopri_dense(t0 + th * h)
        ref = dense[q]
        for s in range(4):
            r, g = ref[s * N:(s + 1) * N], got[s * N:(s + 1) * N]
            scale = max(np.abs(r - r.mean()).max(), 1e-30)
            assert np.abs(g - r).max() <= 1e-4 * scale + 1e-9 * abs(r.mean()), (th, s)
        assert abs(got[-1] / ref[-1] - 1) < 1e-9


def test_dense_output_diagnostics(gpu_mod, oracle_mod):
    """want_output: the interpolated state passes through the output RHS
    (filtered; spectra, constraints and summaries as for a saved slice)."""
    n = (32, 32, 32)
    ctx, o, fo, dense, t0, h = _step_both(gpu_mod, oracle_mod, n, gpu_mod.PREC_F64, 8, 5e-2)
    th = THETAS[2]
    got = ctx.dopri_dense(t0 + th * h, output=True)
    d = oracle_mod.DiagOutput(o.bins)
    _, f_ref = o.rhs(dense[2], t=t0 + th * h, filter=1, output=1, diag=d)
    errs = seg_rel_err(got, f_ref, o.N, o.Next)
    assert max(errs.values()) < 1e-10, errs
    g = ctx.output()
    for k in ("phi_ps", "psi_ps", "rho_ps", "gw"):
        ref = getattr(d, k)
        assert np.abs(g[k] - ref).max() <= 1e-9 * np.abs(ref).max(), k
    atol = np.array([1e-26, 1e-14, 1e-26, 1e-14])
    assert np.all(np.abs(g["cstr"] - d.cstr) <= 1e-6 * np.abs(d.cstr) + atol), (g["cstr"], d.cstr)
    np.testing.assert_allclose(g["smry"], d.smry, rtol=1e-8, atol=1e-14)


def test_dense_output_errors(gpu_mod, oracle_mod):
    n = (16, 16, 16)
    ctx = gpu_mod.Context(n=n, precision=gpu_mod.PREC_F64)
    o = oracle_mod.Oracle(n=n)
    ctx.set_state(make_state(o, seed=9))
    ctx.dopri_init(gpu_mod.dopri_cfg(1e-9, 1e-9), 0.0, 1e-2)
    with pytest.raises(gpu_mod.IHError):  # no step yet
        ctx.dopri_dense(0.0)
    info = ctx.dopri_step(1e-2)
    t1 = ctx.t
    ctx.dopri_dense(t1 - 0.5 * info.dt_did)
    with pytest.raises(gpu_mod.IHError):  # outside the step
        ctx.dopri_dense(t1 + 0.5 * info.dt_did)
    with pytest.raises(gpu_mod.IHError):
        ctx.dopri_dense(t1 - 1.5 * info.dt_did)
    ctx.set_state(ctx.get_state(), t1)
    with pytest.raises(gpu_mod.IHError):  # a state upload ends the step's dense output
        ctx.dopri_dense(t1)
