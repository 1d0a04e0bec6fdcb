"""CPU: the velocity form of the DOPRI853 combinations (the mixed form's
default) equals the reference's combinations (dopri853.c:340-486) whenever the
position half of every stage vector is the velocity half of its stage input,
as the RHS makes it (phi' = dphi, psi' = dpsi, h' = dh; toolbox.c:282-299,
311-346).

Stage vectors k_j = (Y_j^v, f_j) with arbitrary accelerations f_j; the
reference forms Y_s = y + dt sum_l a_sl k_l, field_new = y + dt sum_j b_j k_j
and the error sums with e5 = b - bhh (stages 1, 9, 12) and e3 = er.  The
velocity form reads only the velocity halves:
  Y_s^p  = y^p + dt (sum_l a_sl) y^v + dt^2 sum_l (A^2)_sl k_l^v,
  new^p  = y^p + dt (sum b) y^v + dt^2 sum_l (b^T A)_l k_l^v,
  err^p  = (sum e) y^v + dt sum_l (e^T A)_l k_l^v.
"""
import numpy as np


def _weights(oracle_mod):
    c, a, b, bhh, er = oracle_mod.tableau()
    e5 = b.copy()
    e5[0] -= bhh[0]
    e5[8] -= bhh[1]
    e5[11] -= bhh[2]
    return a, b, e5, er


def _reference_stages(a, yp, yv, f, dt):
    """Stage vectors in the reference's order: k_1 from y, k_s from Y_s."""
    kp, kv = [yv.copy()], [f[0]]
    for s in range(1, 12):
        Yv = yv + dt * sum(a[s, l] * kv[l] for l in range(s))
        kp.append(Yv)
        kv.append(f[s])
    return kp, kv


def test_stage_inputs_match_reference(oracle_mod):
    a, _, _, _ = _weights(oracle_mod)
    rng = np.random.default_rng(3)
    n, dt = 257, 0.37
    yp, yv = rng.standard_normal(n), rng.standard_normal(n)
    f = rng.standard_normal((12, n))
    kp, kv = _reference_stages(a, yp, yv, f, dt)
    a2 = a @ a
    for s in range(1, 12):
        ref_p = yp + dt * sum(a[s, l] * kp[l] for l in range(s))
        vel_p = yp + dt * a[s, :s].sum() * yv + dt * dt * sum(a2[s, l] * kv[l] for l in range(s))
        assert np.abs(vel_p - ref_p).max() <= 1e-13 * np.abs(ref_p).max(), s


def test_final_and_errors_match_reference(oracle_mod):
    a, b, e5, e3 = _weights(oracle_mod)
    rng = np.random.default_rng(4)
    n, dt = 129, 0.23
    yp, yv = rng.standard_normal(n), rng.standard_normal(n)
    f = rng.standard_normal((12, n))
    kp, kv = _reference_stages(a, yp, yv, f, dt)
    for w, with_y in ((b, True), (e5, False), (e3, False)):
        ref = sum(w[j] * kp[j] for j in range(12))
        wa = w @ a
        vel = w.sum() * yv + dt * sum(wa[l] * kv[l] for l in range(12))
        if with_y:
            ref, vel = yp + dt * ref, yp + dt * vel
        assert np.abs(vel - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1e-3)


def test_products_skip_nothing_the_reference_reads(oracle_mod):
    """The term lists of the velocity form: (A^2)_sl vanishes for l >= s - 1
    (strictly lower triangular A), so stage s + 1 reads stages 1..s only."""
    a, b, e5, e3 = _weights(oracle_mod)
    a2 = a @ a
    assert np.all(np.triu(a) == 0.0)
    assert np.all(np.abs(np.triu(a2, -1)) == 0.0)
    for w in (b, e5, e3):
        assert abs((w @ a)[11]) == 0.0
