"""run_dopri853 / run_rk4 with save() and the wrap-up, restated over the C
oracle, for comparing whole drop-in runs slice by slice.

The loops follow dopri853.c:112-233, rk4.c:27-132 and io.c:494-616: output
every TIME_STEP_SKIPS steps (or landed / interpolated slices with the
drop-in's IH_OUTPUT_INTERVAL / IH_DENSE_OUTPUT keys), buffers of
WRITE_OUT_BUFFER_NUMBER slices, the wrap-up slice only while the buffer is
partly filled.  tests/test_ref_oracle.py checks the plain loops against the
reference's own main() run.
"""
import numpy as np

# the time-series datasets record() fills (io.h:14-36 names)
SERIES = ["phi_power_spectrum", "psi_power_spectrum", "rho_power_spectrum",
          "gravitational_wave_spectrum", "constraints", "phi_summary", "dphi_summary",
          "psi_summary", "dpsi_summary", "rho_summary", "pressure_summary", "time", "a", "phi",
          "rho"]


def initial_state(o, seed=11):
    """phi, dphi from the seeded generator; psi, dpsi zero (the host solves
    them from the constraints); a = 1."""
    return o.ic(seed=seed, amp=1e-3, psi=False)


def diag_slice(o, d):
    return {"phi_power_spectrum": d.phi_ps.copy(), "psi_power_spectrum": d.psi_ps.copy(),
            "rho_power_spectrum": d.rho_ps.copy(), "gravitational_wave_spectrum": d.gw.copy(),
            "constraints": d.cstr, "phi_summary": d.smry[0], "dphi_summary": d.smry[1],
            "psi_summary": d.smry[2], "dpsi_summary": d.smry[3], "rho_summary": d.smry[4],
            "pressure_summary": d.smry[5]}


def record(out, o, f, t, d, rho):
    s = diag_slice(o, d)
    s["time"] = np.array([t])
    s["a"] = np.array([f[-1]])
    n = o.n
    s["phi"] = f[: o.N].reshape(n)[::2, ::2, ::2].ravel()
    s["rho"] = rho.reshape(n)[::2, ::2, ::2].ravel()
    for k, v in s.items():
        out.setdefault(k, []).append(np.asarray(v, dtype=np.float64))


def expected_dopri(oracle_mod, p):
    """run_dopri853 + save() + wrap-up (dopri853.c:112-233, io.c:494-616)
    restated over the oracle."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    skip = int(p["TIME_STEP_SKIPS"])
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    record(out, o, f_filt, 0.0, d, o.field_array("rho"))
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
            record(out, o, f, t, d, o.field_array("rho"))
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
        record(out, o, f, t, d, o.field_array("rho"))
    steps = {"steps_total": n_stp, "steps_ok": n_ok, "steps_bad": n_bad}
    return {k: np.array(v) for k, v in out.items()}, steps, f


def expected_rk4(oracle_mod, p):
    """run_rk4 (rk4.c:27-132) restated over the oracle."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = initial_state(o)
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
            record(out, o, f_filt, t, d, o.field_array("rho"))
        o.rk4_step(f, t, dt)
        t += dt
        nt += 1
    d = oracle_mod.DiagOutput(o.bins)
    _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
    record(out, o, f, t, d, o.field_array("rho"))
    return {k: np.array(v) for k, v in out.items()}, f


def expected_landing(oracle_mod, p):
    """run_dopri853 with output landing (IH_OUTPUT_INTERVAL) restated over the
    oracle: steps shortened to end on multiples of the interval, slices there."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    interval = float(p["IH_OUTPUT_INTERVAL"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    record(out, o, f_filt, 0.0, d, o.field_array("rho"))
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
            record(out, o, f, t, d, o.field_array("rho"))
            n_out += 1
            t_next = n_out * interval
        if t >= tf:
            break
        dt = st.dt_next
    saves = len(out["time"])
    if saves % int(p["WRITE_OUT_BUFFER_NUMBER"]) != 0 and out["time"][-1][0] < t:
        d = oracle_mod.DiagOutput(o.bins)
        _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
        record(out, o, f, t, d, o.field_array("rho"))
    return {k: np.array(v) for k, v in out.items()}


def expected_dense(oracle_mod, p):
    """run_dopri853 with dense output (IH_OUTPUT_INTERVAL + IH_DENSE_OUTPUT)
    restated over the oracle: the controller's steps; a step that contains
    output times is redone from its start with the oracle's continuous
    extension at those times, whose states pass through the output RHS."""
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = initial_state(o)
    o.initial_psi(f)
    cfg = oracle_mod.default_cfg(float(p["RELATIVE_TOLERANCE"]), float(p["ABSOLUTE_TOLERANCE"]),
                                 float(p["MAX_DT_HUBBLE_FRACTION"]))
    tf, dt = float(p["FINAL_TIME"]), float(p["DELTA_T"])
    interval = float(p["IH_OUTPUT_INTERVAL"])
    out = {}
    d = oracle_mod.DiagOutput(o.bins)
    _, f_filt = o.rhs(f, filter=1, output=1, diag=d)
    record(out, o, f_filt, 0.0, d, o.field_array("rho"))
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
                record(out, o, fd, x, d, o.field_array("rho"))
        if t >= tf:
            break
        dt = st.dt_next
    saves = len(out["time"])
    if saves % int(p["WRITE_OUT_BUFFER_NUMBER"]) != 0 and out["time"][-1][0] < t:
        d = oracle_mod.DiagOutput(o.bins)
        _, f = o.rhs(f, t=t, filter=1, output=1, diag=d)
        record(out, o, f, t, d, o.field_array("rho"))
    assert dense_steps >= 1
    return {k: np.array(v) for k, v in out.items()}
