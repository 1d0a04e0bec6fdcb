"""CPU tests: pin the oracle against the known answers the reference defines.

The reference ships no golden vectors (it has no test-suite); its validation
material defines these known answers, each checked here:
  * evaluation/testLaplacian.m: spectral gradient and Laplacian of
    sin x sin y sin z on [-pi, pi)^3, N = 64;
  * helpers/flrw_homogeneous.py: the homogeneous FLRW background (imported from
    the reference to make tests/golden/flrw_homogeneous.json);
  * evaluation/mkPowerSpectrum.m:27-33: the shell-binning rule;
  * the DOPRI853 tableau's order conditions;
and the C oracle is cross-checked against the independent numpy restatement.
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_fft_matches_pocketfft(oracle_mod):
    for n in [(8, 8, 8), (16, 16, 8), (32, 16, 16), (24, 12, 6)]:
        o = oracle_mod.Oracle(n=n)
        x = np.random.default_rng(1).standard_normal(n)
        X = o.fft(x)
        ref = np.fft.rfftn(x)
        assert np.abs(X - ref).max() <= 1e-13 * np.abs(ref).max()
        y = o.ifft(ref)
        assert np.abs(y - np.fft.irfftn(ref, s=n, axes=(0, 1, 2)) * x.size).max() <= 1e-12 * x.size


def test_laplacian_known_answer(oracle_mod):
    """evaluation/testLaplacian.m: f = sin x sin y sin z on [-pi, pi)^3."""
    n = 64
    o = oracle_mod.Oracle(n=(n, n, n), L=(2 * np.pi,) * 3, gw=False, filter=False)
    x = -np.pi + 2 * np.pi * np.arange(n) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    f = np.zeros(o.Ntot)
    phi = np.sin(X) * np.sin(Y) * np.sin(Z)
    f[: o.N] = phi.ravel()
    f[-1] = 1.0
    o.rhs(f)
    lap = o.field_array("lap").reshape(n, n, n)
    grad2 = o.field_array("grad2").reshape(n, n, n)
    g_exact = (np.cos(X) ** 2 * np.sin(Y) ** 2 * np.sin(Z) ** 2 + np.sin(X) ** 2 * np.cos(Y) ** 2 *
               np.sin(Z) ** 2 + np.sin(X) ** 2 * np.sin(Y) ** 2 * np.cos(Z) ** 2)
    assert np.abs(lap + 3 * phi).max() < 1e-12
    assert np.abs(grad2 - g_exact).max() < 1e-12


def test_c_oracle_matches_numpy_oracle(oracle_mod):
    from oracle.rhs_numpy import NumpyRHS
    n, L = (16, 16, 8), (20.0, 18.0, 14.0)
    o = oracle_mod.Oracle(n=n, L=L)
    nr = NumpyRHS(n, L)
    f = o.ic(seed=3, amp=1e-2)
    rng = np.random.default_rng(1)
    f[4 * o.N:-1] = 1e-4 * rng.standard_normal(4 * o.Next)
    for filt, out in [(0, 0), (1, 0), (1, 1)]:
        d = oracle_mod.DiagOutput(o.bins)
        r1, f1 = o.rhs(f, filter=filt, output=out, diag=d)
        r2, f2, dg = nr.rhs(f, filter=filt, output=out)
        assert np.abs(r1 - r2).max() <= 1e-13 * np.abs(r2).max()
        assert np.abs(f1 - f2).max() <= 1e-13
        if out:
            for k in ("phi_ps", "psi_ps", "rho_ps", "gw"):
                got = getattr(d, k)
                assert np.abs(got - dg[k]).max() <= 1e-12 * np.abs(dg[k]).max()
            # constraint residuals are cancellation-dominated: compare at 1e-6
            np.testing.assert_allclose(d.cstr, dg["cstr"], rtol=1e-6)
            # summaries (toolbox.c:676-690): mean, variance (N - 1), min, max of
            # phi, dphi, psi, dpsi of the (filtered) input state, rho and p
            N = o.N
            arrs = [f2[i * N:(i + 1) * N] for i in range(4)] + [dg["rho"], dg["p"]]
            ref = np.array([[x.mean(), x.var(ddof=1), x.min(), x.max()] for x in arrs])
            # means of zero-mean fields are rounding: a floor of 1e-12 of the
            # field's magnitude per row
            for row, x in zip(range(6), arrs):
                np.testing.assert_allclose(d.smry[row], ref[row], rtol=1e-10,
                                           atol=1e-12 * np.abs(x).max(), err_msg=str(row))


def test_binning_rule(oracle_mod):
    """mkPowerSpectrum.m:27-33: idx = fix(bins * k/kmax - 1e-14); one mode per test."""
    n = 16
    o = oracle_mod.Oracle(n=(n, n, n), L=(10.0,) * 3)
    g, kmax = o.kgrid()
    bins = o.bins
    for (i, j, k) in [(1, 0, 0), (0, 3, 2), (8, 8, 8), (5, 11, 4)]:
        spec = np.zeros((n, n, n // 2 + 1), dtype=complex)
        spec[i, j, k] = 1.0
        if k == 0 or k == n // 2:  # keep the real-space field real
            spec[(-i) % n, (-j) % n, k] = 1.0
        phi = o.ifft(spec) / o.N
        f = np.zeros(o.Ntot)
        f[: o.N] = phi.ravel()
        f[-1] = 1.0
        d = oracle_mod.DiagOutput(bins)
        o.rhs(f, filter=1, output=1, diag=d)
        kk = np.sqrt(g["sq"].reshape(spec.shape)[i, j, k])
        idx = int(np.trunc(bins * kk / kmax - 1e-14))
        nz = np.nonzero(d.phi_ps > 1e-12 * d.phi_ps.max())[0]
        assert list(nz) == [idx]


def test_dopri853_order_conditions(oracle_mod):
    c, a, b, bhh, er = oracle_mod.tableau()
    assert np.allclose(a.sum(axis=1), c, atol=1e-14)  # row sums = nodes
    # quadrature conditions sum b_i c_i^(q-1) = 1/q up to order 8
    for q in range(1, 9):
        assert abs(np.dot(b, c ** (q - 1)) - 1.0 / q) < 1e-13
    assert abs(np.sum(er)) < 1e-13          # the 3rd-order error weights sum to 0
    assert abs(b.sum() - bhh.sum()) < 1e-13  # the 5th-order error weights sum to 0
    # a few tree conditions: sum b_i a_ij c_j = 1/6, sum b_i c_i a_ij c_j = 1/8
    assert abs(b @ (a @ c) - 1.0 / 6.0) < 1e-13
    assert abs((b * c) @ (a @ c) - 1.0 / 8.0) < 1e-13
    assert abs(b @ (a @ (c ** 2)) - 1.0 / 12.0) < 1e-13


def test_flrw_background_golden(oracle_mod):
    """Homogeneous fields: the oracle's DOPRI853 matches the reference's own
    FLRW helper (helpers/flrw_homogeneous.py, scipy dopri5 rtol 1e-8)."""
    g = json.loads((GOLDEN / "flrw_homogeneous.json").read_text())
    for case in g["cases"]:
        o = oracle_mod.Oracle(n=(8, 8, 8))
        f = np.zeros(o.Ntot)
        f[: o.N] = case["phi0"]
        f[o.N:2 * o.N] = case["dphi0"]
        f[-1] = 1.0
        cfg = oracle_mod.default_cfg(1e-10, 1e-10, max_dt_hubble_fraction=0.0)
        st, df = o.dopri_init(f, cfg, 0.0, 1e-3)
        for k, t in enumerate(case["t"][1:], start=1):
            o.dopri_run(f, df, cfg, st, t, 100000)
            assert abs(st.t - t) < 1e-12
            assert abs(f[0] - case["phi"][k]) < 5e-8
            assert abs(f[o.N] - case["phi_dot"][k]) < 5e-8
            assert abs(f[-1] / case["a"][k] - 1) < 5e-8


def test_psi_solve_satisfies_momentum_constraint(oracle_mod):
    o = oracle_mod.Oracle(n=(16, 16, 16))
    f = o.ic(seed=7, amp=1e-3)
    d = oracle_mod.DiagOutput(o.bins)
    o.rhs(f, filter=1, output=1, diag=d)
    # momentum constraint residual (mean square) far below the field variance
    assert d.cstr[2] < 1e-12
    assert np.isfinite(d.cstr).all()


def test_ic_is_real_and_seeded(oracle_mod):
    o = oracle_mod.Oracle(n=(16, 16, 8))
    f1 = o.ic(seed=11, psi=False)
    f2 = o.ic(seed=11, psi=False)
    f3 = o.ic(seed=12, psi=False)
    assert np.array_equal(f1, f2)
    assert not np.array_equal(f1, f3)
    phi = f1[: o.N] - 1.0
    # Hermitian construction: forward transform round-trips
    spec = o.fft(phi)
    assert np.abs(o.ifft(spec) / o.N - phi.reshape(16, 16, 8)).max() < 1e-15
    assert abs(phi.mean()) < 1e-15


def test_rk4_step_reduces_to_background(oracle_mod):
    o = oracle_mod.Oracle(n=(8, 8, 8))
    f = np.zeros(o.Ntot)
    f[: o.N] = 1.0
    f[o.N:2 * o.N] = oracle_mod.slow_roll_dphi0(1.0)
    f[-1] = 1.0
    g = json.loads((GOLDEN / "flrw_homogeneous.json").read_text())["cases"][0]
    t = 0.0
    dt = 0.005
    while t < 0.5 - 1e-12:
        o.rk4_step(f, t, dt)
        t += dt
    assert abs(f[0] - g["phi"][1]) < 1e-8
    assert abs(f[-1] - g["a"][1]) < 1e-8


def test_c_oracle_rk4_step_matches_numpy(oracle_mod):
    """rk4.c:108-161 (filter on the first stage only): the oracle's RK4 step
    against the same step on the numpy restatement of the RHS, to 1e-12 of
    each state segment's largest magnitude."""
    from oracle.rhs_numpy import NumpyRHS
    n, L = (16, 16, 8), (20.0, 18.0, 14.0)
    o = oracle_mod.Oracle(n=n, L=L)
    nr = NumpyRHS(n, L)
    f = o.ic(seed=6, amp=1e-3)
    f[4 * o.N:-1] = 1e-6 * np.random.default_rng(6).standard_normal(4 * o.Next)
    dt = 0.01
    k1, y, _ = nr.rhs(f, filter=1)
    k2 = nr.rhs(y + dt * k1 / 2.0)[0]
    k3 = nr.rhs(y + dt * k2 / 2.0)[0]
    k4 = nr.rhs(y + dt * k3)[0]
    ref = y + dt * (k1 + 2.0 * k2 + 2.0 * k3 + k4) / 6.0
    got = f.copy()
    o.rk4_step(got, 0.0, dt)
    N, Next = o.N, o.Next
    edges = [0, N, 2 * N, 3 * N, 4 * N] + [4 * N + i * Next for i in range(1, 5)]
    for lo, hi in zip(edges[:-1], edges[1:]):
        assert np.abs(got[lo:hi] - ref[lo:hi]).max() <= 1e-12 * np.abs(ref[lo:hi]).max(), lo
    assert abs(got[-1] / ref[-1] - 1.0) < 1e-14


def test_c_oracle_psi_solve_matches_numpy(oracle_mod):
    """mk_initial_psi (setup.c:825-903) restated on the numpy RHS: with psi
    and dpsi zeroed, psi_k = (-<dphi> ddphi_k + <ddphi'> dphi_k) /
    (-<dphi>^2 + 2 k^2 / a^2) (k = 0 mode zero), dpsi = <dphi>/2 dphi - H psi;
    against the oracle to 1e-11 of each segment's largest magnitude."""
    from oracle.rhs_numpy import NumpyRHS
    n, L = (16, 16, 8), (20.0, 18.0, 14.0)
    o = oracle_mod.Oracle(n=n, L=L)
    nr = NumpyRHS(n, L)
    f = o.ic(seed=7, amp=1e-3, psi=False)
    N = o.N
    g = f.copy()
    g[2 * N:4 * N] = 0.0
    res, _, dg = nr.rhs(g)
    a2 = g[-1] ** 2
    H = np.sqrt(dg["rho_mean"] / 3.0)
    phim, dphim, ddphim = g[:N].mean(), g[N:2 * N].mean(), res[N:2 * N].mean()
    D = nr.fft(g[N:2 * N] - dphim)
    F = nr.fft(g[:N] - phim)
    P = (-dphim * D + ddphim * F) / (-dphim ** 2 + 2.0 * nr.g["sq"] / a2)
    P.flat[0] = 0.0
    psi = np.fft.irfftn(P, s=n, axes=(0, 1, 2)).ravel()
    dpsi = 0.5 * dphim * (g[:N] - phim) - H * psi
    o.initial_psi(f)
    assert np.abs(f[2 * N:3 * N] - psi).max() <= 1e-11 * np.abs(psi).max()
    assert np.abs(f[3 * N:4 * N] - dpsi).max() <= 1e-11 * np.abs(dpsi).max()
