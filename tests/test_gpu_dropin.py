"""GPU tests of the C99 drop-in layer: the standalone host (stand-in for the
reference's main.c / setup.c / io.c) runs run_dopri853 / run_rk4 through the
reference-facing symbols, and its output container is compared with the same
run of the CPU oracle, slice by slice.

Tolerances: FP64 throughout; times and a within 1e-12 relative, spectra,
summaries and fields within 1e-9 of their largest magnitude (several steps of
1e-11-per-RHS parity), constraint residuals within 1e-6 relative plus a
roundoff floor (they are cancellations)."""
from pathlib import Path

import numpy as np
import pytest

from instaheat_gb300 import dropin

PARAMS = Path(__file__).resolve().parent / "dropin"
pytestmark = pytest.mark.gpu


def _initial_state(o, seed=11):
    """phi, dphi from the seeded generator; psi, dpsi zero (the host solves
    them from the constraints); a = 1."""
    return o.ic(seed=seed, amp=1e-3, psi=False)


def _diag_slice(o, d):
    return {"phi_power_spectrum": d.phi_ps.copy(), "psi_power_spectrum": d.psi_ps.copy(),
            "rho_power_spectrum": d.rho_ps.copy(), "gravitational_wave_spectrum": d.gw.copy(),
            "constraints": d.cstr, "phi_summary": d.smry[0], "dphi_summary": d.smry[1],
            "psi_summary": d.smry[2], "dpsi_summary": d.smry[3], "rho_summary": d.smry[4],
            "pressure_summary": d.smry[5]}


def _record(out, o, f, t, d, rho):
    s = _diag_slice(o, d)
    s["time"] = np.array([t])
    s["a"] = np.array([f[-1]])
    n = o.n
    s["phi"] = f[: o.N].reshape(n)[::2, ::2, ::2].ravel()
    s["rho"] = rho.reshape(n)[::2, ::2, ::2].ravel()
    for k, v in s.items():
        out.setdefault(k, []).append(np.asarray(v, dtype=np.float64))


def _expected_dopri(oracle_mod, p):
    """run_dopri853 + save() + wrap-up (dopri853.c:112-233, io.c:494-616)
    restated over the oracle."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = _initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    skip = int(p["TIME_STEP_SKIPS"])
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    _record(out, o, f_filt, 0.0, d, o.field_array("rho"))
    st, df = o.dopri_init(f, cfg, 0.0, dt)
    t, n_stp, n_ok, n_bad = 0.0, 0, 0, 0
    while True:
        if t + dt * 1.0001 > tf:
            dt = tf - t
        want = (n_stp + 1) % skip == 0
        d = oracle_mod.DiagOutput(o.bins)
        assert o.dopri_step(f, df, cfg, st, dt, d if want else None) == 0
        if st.dt_did == dt:
            n_ok += 1
        else:
            n_bad += 1
        t = st.t
        if want:
            _record(out, o, f, t, d, o.field_array("rho"))
        if t >= tf:
            break
        dt = st.dt_next
        n_stp += 1
    # the wrap-up adds a last slice only while the output buffer is partly
    # filled (dopri853.c:209-212: index != 0)
    saves = len(out["time"])
    if saves % int(p["WRITE_OUT_BUFFER_NUMBER"]) != 0 and out["time"][-1][0] < t:
        d = oracle_mod.DiagOutput(o.bins)
        _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
        _record(out, o, f, t, d, o.field_array("rho"))
    steps = {"steps_total": n_stp, "steps_ok": n_ok, "steps_bad": n_bad}
    return {k: np.array(v) for k, v in out.items()}, steps, f


def _expected_rk4(oracle_mod, p):
    """run_rk4 (rk4.c:27-132) restated over the oracle."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = _initial_state(o)
    o.initial_psi(f)
    skip = int(p["TIME_STEP_SKIPS"])
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    out, t, nt = {}, 0.0, 0
    while t < tf:
        if t + dt * 1.0001 > tf:
            dt = tf - t
        if nt % skip == 0:
            d = oracle_mod.DiagOutput(o.bins)
            _, f_filt = o.rhs(f, t=t, filter=1, output=1, diag=d)
            _record(out, o, f_filt, t, d, o.field_array("rho"))
        o.rk4_step(f, t, dt)
        t += dt
        nt += 1
    d = oracle_mod.DiagOutput(o.bins)
    _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
    _record(out, o, f, t, d, o.field_array("rho"))
    return {k: np.array(v) for k, v in out.items()}, f


def _run_host(tmp_path, name, oracle_mod):
    import subprocess
    p = dropin.read_parameters(PARAMS / name)
    exe = dropin.build_host(p, tmp_path / "host")
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    _initial_state(o).tofile(tmp_path / "init.bin")
    r = subprocess.run([str(exe), str(tmp_path / "init.bin"), str(tmp_path / "out.ihc"),
                        str(tmp_path / "final.bin")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return p, dropin.read_container(tmp_path / "out.ihc"), np.fromfile(tmp_path / "final.bin")


def _compare_series(got, exp):
    for k, e in exp.items():
        g = got[k]
        assert g.shape == e.shape, (k, g.shape, e.shape)
        if k in ("time", "a"):
            np.testing.assert_allclose(g, e, rtol=1e-12, err_msg=k)
        elif k == "constraints":
            atol = np.array([1e-26, 1e-14, 1e-26, 1e-14])
            assert np.all(np.abs(g - e) <= 1e-6 * np.abs(e) + atol), k
        else:
            assert np.abs(g - e).max() <= 1e-9 * np.abs(e).max() + 1e-300, k


def test_run_dopri853_through_the_dropin(tmp_path, oracle_mod):
    p, got, final = _run_host(tmp_path, "parameters_dopri853.sh", oracle_mod)
    exp, steps, f_exp = _expected_dopri(oracle_mod, p)
    _compare_series(got, exp)
    for k, v in steps.items():
        assert got[k][0] == v, k
    # followup: the final state; calls_rhs counted
    scale = np.abs(f_exp[: 4 * 16 ** 3]).max()
    assert np.abs(final - f_exp).max() <= 1e-9 * scale
    assert np.abs(got["followup"] - f_exp).max() <= 1e-9 * scale
    assert got["calls_rhs"][0] > 12 * steps["steps_total"]
    assert got["gridpoints_internal"].tolist() == [16.0, 16.0, 16.0]


def test_run_rk4_through_the_dropin(tmp_path, oracle_mod):
    p, got, final = _run_host(tmp_path, "parameters_rk4.sh", oracle_mod)
    exp, f_exp = _expected_rk4(oracle_mod, p)
    _compare_series(got, exp)
    assert np.abs(final - f_exp).max() <= 1e-9 * np.abs(f_exp[: 4 * 16 ** 3]).max()


def _expected_landing(oracle_mod, p):
    """run_dopri853 with output landing (IH_OUTPUT_INTERVAL) restated over the
    oracle: steps shortened to end on multiples of the interval, slices there."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = _initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    interval = float(p["IH_OUTPUT_INTERVAL"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    _record(out, o, f_filt, 0.0, d, o.field_array("rho"))
    st, df = o.dopri_init(f, cfg, 0.0, dt)
    t, n_out = 0.0, 1
    t_next = n_out * interval
    while True:
        if t + dt * 1.0001 > tf:
            dt = tf - t
        want = False
        if t_next < tf and t + dt * 1.0001 > t_next:
            dt = t_next - t
            want = True
        d = oracle_mod.DiagOutput(o.bins)
        assert o.dopri_step(f, df, cfg, st, dt, d if want else None) == 0
        t = st.t
        if want and abs(t - t_next) <= 1e-12 * max(1.0, abs(t_next)):
            _record(out, o, f, t, d, o.field_array("rho"))
            n_out += 1
            t_next = n_out * interval
        if t >= tf:
            break
        dt = st.dt_next
    saves = len(out["time"])
    if saves % int(p["WRITE_OUT_BUFFER_NUMBER"]) != 0 and out["time"][-1][0] < t:
        d = oracle_mod.DiagOutput(o.bins)
        _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
        _record(out, o, f, t, d, o.field_array("rho"))
    return {k: np.array(v) for k, v in out.items()}


def test_run_dopri853_output_landing(tmp_path, oracle_mod):
    p, got, _ = _run_host(tmp_path, "parameters_landing.sh", oracle_mod)
    exp = _expected_landing(oracle_mod, p)
    times = got["time"][:, 0]
    # slices at 0, 0.02 and 0.04 (landed); the third fills the buffer of three,
    # so the wrap-up adds no slice at 0.05 (dopri853.c:209-212)
    np.testing.assert_allclose(times, [0.0, 0.02, 0.04], atol=1e-14)
    _compare_series(got, exp)


def _expected_dense(oracle_mod, p):
    """run_dopri853 with dense output (IH_OUTPUT_INTERVAL + IH_DENSE_OUTPUT)
    restated over the oracle: the controller's steps; a step that contains
    output times is redone from its start with the oracle's continuous
    extension at those times, whose states pass through the output RHS."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = _initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    interval = float(p["IH_OUTPUT_INTERVAL"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    _record(out, o, f_filt, 0.0, d, o.field_array("rho"))
    st, df = o.dopri_init(f, cfg, 0.0, dt)
    t, n_out = 0.0, 1
    t_next = n_out * interval
    dense_steps = 0
    while True:
        if t + dt * 1.0001 > tf:
            dt = tf - t
        f0, df0, st0, t0 = f.copy(), df.copy(), type(st).from_buffer_copy(st), t
        assert o.dopri_step(f, df, cfg, st, dt) == 0
        t = st.t
        times = []
        while t_next < tf and t_next <= t:
            times.append(t_next)
            n_out += 1
            t_next = n_out * interval
        if times:
            h = st.dt_did
            f[:], df[:] = f0, df0
            st = type(st).from_buffer_copy(st0)
            rc, dense = o.dopri_step_dense(f, df, cfg, st, dt, [(x - t0) / h for x in times])
            assert rc == 0 and st.dt_did == h
            dense_steps += 1
            for x, fd in zip(times, dense):
                d = oracle_mod.DiagOutput(o.bins)
                _, fd = o.rhs(fd, t=x, filter=1, output=1, diag=d)
                _record(out, o, fd, x, d, o.field_array("rho"))
        if t >= tf:
            break
        dt = st.dt_next
    saves = len(out["time"])
    if saves % int(p["WRITE_OUT_BUFFER_NUMBER"]) != 0 and out["time"][-1][0] < t:
        d = oracle_mod.DiagOutput(o.bins)
        _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
        _record(out, o, f, t, d, o.field_array("rho"))
    assert dense_steps >= 1
    return {k: np.array(v) for k, v in out.items()}


def test_run_dopri853_dense_output(tmp_path, oracle_mod):
    p, got, _ = _run_host(tmp_path, "parameters_dense.sh", oracle_mod)
    exp = _expected_dense(oracle_mod, p)
    times = got["time"][:, 0]
    # slices at 0, 0.02 and 0.04 from the continuous extension (the steps are
    # not shortened); the buffer of three is full, so the wrap-up adds none
    np.testing.assert_allclose(times, [0.0, 0.02, 0.04], atol=1e-14)
    _compare_series(got, exp)
