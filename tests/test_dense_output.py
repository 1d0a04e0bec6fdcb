"""CPU: the DOP853 continuous extension (dense output; coefficients
dopri853_constants.c:23-25, 98-173, declared but unused by the reference's
stepper) -- its coefficients, the expanded form the GPU library evaluates,
and the oracle's dense output on an InstaHeat step.

Nested form (Hairer, Norsett & Wanner):
  y(th) = r1 + th (r2 + s (r3 + th (r4 + s (r5 + th (r6 + s (r7 + th r8)))))),
  s = 1 - th, r1 = y, r2 = y_new - y, r3 = h k1 - r2, r4 = r2 - h k13 - r3,
  r(5+i) = h sum_j d(4+i)j k_j.
Expanded form: y(th) = (1 - u) y + u y_new + h sum_j W_j k_j with
  u = th^2 (3 - 2 th),  W_j = th^2 s^2 d4j + th^3 s^2 d5j + th^3 s^3 d6j
  + th^4 s^3 d7j, plus th s^2 on k1 and - th^2 s on k13.
"""
import numpy as np


def dense_weights(th, d):
    """(u, W[16]) of the expanded form."""
    s = 1.0 - th
    g = np.array([th**2 * s**2, th**3 * s**2, th**3 * s**3, th**4 * s**3])
    W = g @ d
    W[0] += th * s * s
    W[12] -= th * th * s
    return th * th * (3.0 - 2.0 * th), W


def _dop853_step(f, y0, h, tab, dtab):
    c, a, b, bhh, er = tab
    ad, d = dtab
    k = [f(y0)]
    for s_ in range(1, 12):
        k.append(f(y0 + h * sum(a[s_, j] * k[j] for j in range(s_))))
    ynew = y0 + h * sum(b[j] * k[j] for j in range(12))
    k.append(f(ynew))  # stage 13
    for r in range(3):
        k.append(f(y0 + h * sum(ad[r, j] * k[j] for j in range(13 + r))))
    return ynew, k


def test_stage_rows_sum_to_nodes(oracle_mod):
    ad, d = oracle_mod.dense_tableau()
    assert np.allclose(ad.sum(axis=1), [0.1, 0.2, 7.0 / 9.0], atol=1e-14, rtol=0)
    assert np.all(ad[:, 1:5] == 0.0) and np.all(d[:, 1:5] == 0.0)
    for r in range(3):
        assert np.all(ad[r, 13 + r:] == 0.0)


def test_expanded_form_equals_nested_form(oracle_mod):
    ad, d = oracle_mod.dense_tableau()
    rng = np.random.default_rng(5)
    y, ynew = rng.standard_normal(7), rng.standard_normal(7)
    k = rng.standard_normal((16, 7))
    h = 0.3
    for th in (0.0, 0.2, 0.5, 0.9, 1.0):
        s = 1.0 - th
        r = [y, ynew - y]
        r.append(h * k[0] - r[1])
        r.append(r[1] - h * k[12] - r[2])
        r += [h * (d[i] @ k) for i in range(4)]
        nested = r[0] + th * (r[1] + s * (r[2] + th * (r[3] + s * (r[4] + th * (r[5] + s * (
            r[6] + th * r[7]))))))
        u, W = dense_weights(th, d)
        expanded = (1 - u) * y + u * ynew + h * (W @ k)
        assert np.abs(expanded - nested).max() <= 1e-13 * np.abs(nested).max()


def test_continuous_extension_order(oracle_mod):
    """y' = A y (a damped rotation and a decay): the interpolant's error at
    interior points falls as h^8 (order 7 continuous extension)."""
    tab = oracle_mod.tableau()
    dtab = oracle_mod.dense_tableau()
    A = np.array([[-0.3, 2.0, 0.0], [-2.0, -0.3, 0.0], [0.0, 0.0, -1.5]])
    w, V = np.linalg.eig(A)
    Vi = np.linalg.inv(V)

    def exact(y0, t):
        return (V @ (np.exp(w * t) * (Vi @ y0))).real

    y0 = np.array([1.0, 0.5, -0.7])
    for th in (0.37, 0.81):
        errs = []
        for h in (0.4, 0.2):
            ynew, k = _dop853_step(lambda y: A @ y, y0, h, tab, dtab)
            u, W = dense_weights(th, dtab[1])
            yd = (1 - u) * y0 + u * ynew + h * sum(W[j] * k[j] for j in range(16))
            errs.append(np.abs(yd - exact(y0, th * h)).max())
        assert np.log2(errs[0] / errs[1]) > 6.5, errs


def test_oracle_dense_output_on_a_step(oracle_mod):
    """The oracle's dense output on a 16^3 InstaHeat step (filter off, so the
    end state is the step's own): theta = 0 is the start state, theta = 1
    the end state, and theta = 1/2 agrees with a step landed there."""
    o = oracle_mod.Oracle(n=(16, 16, 16), filter=False)
    f0 = o.ic(seed=3, amp=1e-3)
    cfg = oracle_mod.default_cfg(1e-9, 1e-9, 1e-2)
    f = f0.copy()
    st, df = o.dopri_init(f, cfg, 0.0, 5e-2)
    df0 = df.copy()
    rc, dense = o.dopri_step_dense(f, df, cfg, st, 5e-2, [0.0, 0.5, 1.0])
    assert rc == 0
    h = st.dt_did
    assert np.array_equal(dense[0], f0)
    assert np.abs(dense[2] - f).max() <= 1e-14 * np.abs(f).max()
    g = f0.copy()
    st2, dg = o.dopri_init(g, cfg, 0.0, 0.5 * h)
    assert np.allclose(dg, df0, rtol=1e-12, atol=1e-14)  # OpenMP sums: same to rounding
    assert o.dopri_step(g, dg, cfg, st2, 0.5 * h) == 0
    assert st2.dt_did == 0.5 * h
    N = o.N
    for s in range(4):
        seg = slice(s * N, (s + 1) * N)
        scale = max(np.abs(g[seg] - g[seg].mean()).max(), 1e-30)
        assert np.abs(dense[1][seg] - g[seg]).max() <= 1e-6 * scale + 1e-12 * abs(g[seg].mean()), s
    assert abs(dense[1][-1] / g[-1] - 1.0) < 1e-12


def test_gpu_dense_tableau_equals_oracle(gpu_mod, oracle_mod):
    """The library's dense-output coefficients (no GPU needed to read them)."""
    for x, y in zip(gpu_mod.dense_tableau(), oracle_mod.dense_tableau()):
        assert np.array_equal(x, y)


def test_oracle_dense_matches_a_numpy_dop853_step(oracle_mod):
    """The oracle's DOPRI853 step and dense output against an independent
    numpy DOP853 step on the numpy restatement of the RHS
    (oracle/rhs_numpy.py, pocketfft): the error norm of the accepted try to
    1e-6 relative, and the post-step RHS filtering field_new, stages 14-16 and
    the nested interpolant to 1e-11 of each state segment's largest
    magnitude."""
    from oracle.rhs_numpy import NumpyRHS
    n, L = (16, 16, 8), (20.0, 18.0, 14.0)
    o = oracle_mod.Oracle(n=n, L=L)
    nr = NumpyRHS(n, L)
    f = o.ic(seed=4, amp=1e-3)
    f[4 * o.N:-1] = 1e-6 * np.random.default_rng(4).standard_normal(4 * o.Next)
    cfg = oracle_mod.default_cfg(1e-9, 1e-9, 1e-2)
    st, df = o.dopri_init(f, cfg, 0.0, 0.1)   # filters f in place, df = f(f)
    y0, k1 = f.copy(), df.copy()
    thetas = [0.25, 0.6, 1.0]
    # a long step, so that the error estimate stands well above FP64 rounding
    rc, dense = o.dopri_step_dense(f, df, cfg, st, 0.1, thetas)
    assert rc == 0
    h = st.dt_did  # the accepted try's size (the last try's stages)
    c, a, b, bhh, er = oracle_mod.tableau()
    ad, d = oracle_mod.dense_tableau()
    k = [k1]
    for s_ in range(1, 12):
        k.append(nr.rhs(y0 + h * sum(a[s_, j] * k[j] for j in range(s_)))[0])
    ynew = y0 + h * sum(b[j] * k[j] for j in range(12))
    # the error norm of the accepted try (dopri853.c:438-486), a cancellation
    # of the stages, which the C and numpy code round differently
    kb = sum(b[j] * k[j] for j in range(12))
    yerr = kb - bhh[0] * k[0] - bhh[1] * k[8] - bhh[2] * k[11]
    yerr2 = sum(er[j] * k[j] for j in range(12))
    sk = cfg.atol + cfg.rtol * np.maximum(np.abs(y0), np.abs(ynew))
    e2, e3 = np.sum((yerr / sk) ** 2), np.sum((yerr2 / sk) ** 2)
    err = h * e3 * np.sqrt(1.0 / (o.Ntot * (e3 + 0.01 * e2)))
    assert st.last_err > 1e-4 and abs(err / st.last_err - 1.0) < 1e-6, (err, st.last_err)
    k13, ynew_f, _ = nr.rhs(ynew, filter=1)
    k.append(k13)
    for r in range(3):
        k.append(nr.rhs(y0 + h * sum(ad[r, j] * k[j] for j in range(13 + r)))[0])
    K = np.array(k)
    for q, th in enumerate(thetas):
        s = 1.0 - th
        r1, r2 = y0, ynew_f - y0
        r3 = h * k1 - r2
        r4 = r2 - h * k13 - r3
        r5, r6, r7, r8 = (h * (d[i] @ K) for i in range(4))
        ref = r1 + th * (r2 + s * (r3 + th * (r4 + s * (r5 + th * (r6 + s * (r7 + th * r8))))))
        N, Next = o.N, o.Next
        edges = [0, N, 2 * N, 3 * N, 4 * N] + [4 * N + i * Next for i in range(1, 5)]
        for lo, hi in zip(edges[:-1], edges[1:]):  # each segment on its own scale
            seg = slice(lo, hi)
            assert np.abs(dense[q][seg] - ref[seg]).max() <= 1e-11 * np.abs(ref[seg]).max(), (th, lo)
        assert abs(dense[q][-1] / ref[-1] - 1.0) < 1e-13
