"""Cases run through the reference's own code (oracle/_ref) and the helpers
the tests use to compare with it.

Each case names a grid, box and parameters.sh values, a seeded state and a
job: one ``mk_rhs`` (toolbox.c:75-88) with given filter/output flags, the
psi constraint solve inside ``allocate_and_init_all`` (setup.c:825-903),
three DOPRI853 ``perform_step`` calls after ``run_dopri853``'s prologue
(dopri853.c:112-311), or ``run_rk4`` over four steps (rk4.c:27-132).

``reference(name)`` runs the case through oracle/_ref when the reference's
sources are staged (oracle/ref.py); otherwise it returns the committed
fixture ``tests/golden/ref_cases.npz`` (cases marked golden), made by
``tests/golden/make_ref_golden.py`` from the same runs.  Neither reads the
reference checkout itself.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_cases.npz"

SEGS = ["phi", "dphi", "psi", "dpsi", "h1", "h2", "dh1", "dh2"]

RK4_DT = 0.005
RK4_STEPS = 4
DOPRI_DT0 = 1e-3
DOPRI_STEPS = 3

CASES = {
    # non-cubic grid and box (Nx >= Ny >= Nz, setup.c:219-222): the golden set
    "rhs_16x16x8_fo": dict(n=(16, 16, 8), L=(20.0, 18.0, 14.0), bins=8, job="rhs", filter=1,
                           output=1, seed=3, amp=1e-2, hamp=1e-4, golden=True),
    "rhs_16x16x8": dict(n=(16, 16, 8), L=(20.0, 18.0, 14.0), bins=8, job="rhs", filter=0,
                        output=0, seed=4, amp=1e-2, hamp=1e-4, golden=True),
    "psi_16x16x8": dict(n=(16, 16, 8), L=(20.0, 18.0, 14.0), bins=8, job="psi", seed=5,
                        amp=1e-2, golden=True),
    "dopri_16x16x8": dict(n=(16, 16, 8), L=(20.0, 18.0, 14.0), bins=8, job="dopri", seed=6,
                          amp=1e-3, hamp=1e-6, golden=True),
    "rk4_16x16x8": dict(n=(16, 16, 8), L=(20.0, 18.0, 14.0), bins=8, job="rk4", seed=7,
                        amp=1e-3, hamp=1e-6, golden=True),
    # live-only cases (need the staged reference sources)
    "rhs_16_fo": dict(n=(16, 16, 16), L=(20.0,) * 3, bins=8, job="rhs", filter=1, output=1,
                      seed=3, amp=1e-2, hamp=1e-4),
    "rhs_32_fo": dict(n=(32, 32, 32), L=(20.0,) * 3, bins=16, job="rhs", filter=1, output=1,
                      seed=8, amp=1e-2, hamp=1e-4),
    "rhs_32_f": dict(n=(32, 32, 32), L=(20.0,) * 3, bins=16, job="rhs", filter=1, output=0,
                     seed=9, amp=1e-2, hamp=1e-4),
    "rhs_32x16x16_fo": dict(n=(32, 16, 16), L=(20.0, 15.0, 12.0), bins=16, job="rhs", filter=1,
                            output=1, seed=10, amp=1e-2, hamp=1e-4),
    "psi_32": dict(n=(32, 32, 32), L=(20.0,) * 3, bins=16, job="psi", seed=11, amp=1e-3),
    "dopri_16": dict(n=(16, 16, 16), L=(20.0,) * 3, bins=8, job="dopri", seed=2, amp=1e-3,
                     hamp=1e-6),
    "dopri_32": dict(n=(32, 32, 32), L=(20.0,) * 3, bins=16, job="dopri", seed=12, amp=1e-3,
                     hamp=1e-6),
    "rk4_32": dict(n=(32, 32, 32), L=(20.0,) * 3, bins=16, job="rk4", seed=13, amp=1e-3,
                   hamp=1e-6),
}

# what each job's result keeps (and the fixture stores)
KEEP = {
    "rhs": ["dfield", "field", "rho_mean", "pressure_mean", "out_phi_ps", "out_psi_ps",
            "out_rho_ps", "out_gw", "out_cstr", "out_phi_smry", "out_dphi_smry", "out_psi_smry",
            "out_dpsi_smry", "out_rho_smry", "out_p_smry"],
    "psi": ["psi"],
    "dopri": ["field", "dfield", "steps"],
    "rk4": ["field", "t"],
}


def params(case: dict, **extra) -> dict:
    from oracle import ref
    nx, ny, nz = case["n"]
    lx, ly, lz = case["L"]
    p = dict(GRIDPOINTS_X=nx, GRIDPOINTS_Y=ny, GRIDPOINTS_Z=nz,
             SPATIAL_LOWER_BOUND_X=-lx / 2, SPATIAL_UPPER_BOUND_X=lx / 2,
             SPATIAL_LOWER_BOUND_Y=-ly / 2, SPATIAL_UPPER_BOUND_Y=ly / 2,
             SPATIAL_LOWER_BOUND_Z=-lz / 2, SPATIAL_UPPER_BOUND_Z=lz / 2,
             POWER_SPECTRUM_BINS=case["bins"])
    if case["job"] == "rk4":
        p["INTEGRATION_METHOD"] = "RK4"
        p["ENABLE_FOLLOWUP"] = 0
    p.update(extra)
    return ref.config(**{k: repr(v) if isinstance(v, float) else v for k, v in p.items()})


def state(case: dict, oracle_mod) -> np.ndarray:
    """The case's initial state (reference layout, Ntot doubles): the seeded
    fluctuation data with psi solved (zero psi for the psi job), tensor
    modes filled with seeded Gaussians of size hamp."""
    o = oracle_mod.Oracle(n=case["n"], L=case["L"], bins=case["bins"])
    f = o.ic(seed=case["seed"], amp=case["amp"], psi=case["job"] != "psi")
    if case.get("hamp"):
        rng = np.random.default_rng(case["seed"])
        f[4 * o.N:-1] = case["hamp"] * rng.standard_normal(4 * o.Next)
    o.close()
    return f


def rk4_dts(t0=0.0, dt=RK4_DT, steps=RK4_STEPS):
    """The step sizes of run_rk4's loop (rk4.c:55-61, 103-105) over
    [t0, t0 + steps*dt]: the last step is shortened to land on tf."""
    tf = t0 + steps * dt
    t, out = t0, []
    while t < tf:
        if t + dt * 1.0001 > tf:
            dt = tf - t
        out.append(dt)
        t += dt
    return out, t


def run_reference(name: str) -> dict:
    """Run one case through oracle/_ref (the staged reference sources)."""
    from oracle import oracle as oracle_mod
    from oracle import ref
    case = CASES[name]
    d = ref.build(params(case))
    f = state(case, oracle_mod)
    job = case["job"]
    if job == "rhs":
        r = ref.run(d, "rhs", f, filter=case["filter"], output=case["output"])
    elif job == "psi":
        r = ref.run(d, "init", f, set_state=False)
        N = int(np.prod(case["n"]))
        r["psi"] = r["init_field"][2 * N:4 * N]
    elif job == "dopri":
        r = ref.run(d, "dopri", f, t0=0.0, tf=1.0e3, dt0=DOPRI_DT0, steps=DOPRI_STEPS)
    elif job == "rk4":
        r = ref.run(d, "rk4", f, t0=0.0, tf=RK4_DT * RK4_STEPS, dt=RK4_DT)
    else:
        raise ValueError(job)
    keep = [k for k in KEEP[job] if not (k == "field" and job == "rhs" and not case["filter"])]
    return {k: np.asarray(r[k]) for k in keep if k in r}


def reference(name: str) -> dict:
    from oracle import ref
    if ref.available():
        return run_reference(name)
    if not CASES[name].get("golden"):
        import pytest
        pytest.skip("the reference's sources are not staged (oracle/_ref/src)")
    z = np.load(GOLDEN)
    pre = name + "/"
    return {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}


def seg_bounds(N, Next):
    b = [0, N, 2 * N, 3 * N, 4 * N, 4 * N + Next, 4 * N + 2 * Next, 4 * N + 3 * Next,
         4 * N + 4 * Next]
    return [(b[i], b[i + 1]) for i in range(8)]


def seg_rel_err(x, ref, N, Next):
    """max |x - ref| / max |ref| per state segment (and a)."""
    out = {}
    for name, (a, b) in zip(SEGS, seg_bounds(N, Next)):
        sc = np.abs(ref[a:b]).max()
        out[name] = np.abs(x[a:b] - ref[a:b]).max() / sc if sc > 0 else np.abs(x[a:b]).max()
    out["a"] = abs(x[-1] - ref[-1]) / abs(ref[-1])
    return out


def dopri_rows(st_list):
    return np.array(st_list, dtype=np.float64)


def oracle_result(name: str, oracle_mod) -> dict:
    """The same case through the C oracle (oracle/ih_oracle.c)."""
    case = CASES[name]
    o = oracle_mod.Oracle(n=case["n"], L=case["L"], bins=case["bins"])
    f = state(case, oracle_mod)
    N = o.N
    job = case["job"]
    out = {}
    if job == "rhs":
        d = oracle_mod.DiagOutput(o.bins)
        r, ff = o.rhs(f, filter=case["filter"], output=case["output"], diag=d)
        out.update(dfield=r, field=ff, rho_mean=o.rho_mean, pressure_mean=o.pressure_mean)
        if case["output"]:
            out.update(out_phi_ps=d.phi_ps, out_psi_ps=d.psi_ps, out_rho_ps=d.rho_ps,
                       out_gw=d.gw, out_cstr=d.cstr)
            for i, k in enumerate(["phi", "dphi", "psi", "dpsi", "rho", "p"]):
                out[f"out_{k}_smry"] = d.smry[i]
    elif job == "psi":
        o.initial_psi(f)
        out["psi"] = f[2 * N:4 * N].copy()
    elif job == "dopri":
        cfg = oracle_mod.default_cfg(1e-10, 1e-10, 1e-2)
        st, df = o.dopri_init(f, cfg, 0.0, DOPRI_DT0)
        dt, rows = DOPRI_DT0, []
        for _ in range(DOPRI_STEPS):
            rc = o.dopri_step(f, df, cfg, st, dt)
            rows.append([rc, st.t, st.dt_did, st.dt_next, st.err_old, st.reject])
            dt = st.dt_next
        out.update(field=f, dfield=df, steps=dopri_rows(rows))
    elif job == "rk4":
        dts, t_end = rk4_dts()
        t = 0.0
        for dt in dts:
            o.rk4_step(f, t, dt)
            t += dt
        # run_rk4 ends with prepare_and_save_timeslice (rk4.c:110): the
        # final state passes through the filtered output RHS
        _, f = o.rhs(f, t=t, filter=1, output=1)
        out.update(field=f, t=np.array(t))
    o.close()
    return out


def compare(name: str, got: dict, ref: dict, rtol: float, field_atol: float,
            step_rtol: float, dstep_rtol: float) -> None:
    """Assert agreement per state segment (rtol of each segment's largest
    magnitude for one RHS; step_rtol / dstep_rtol for the state / derivative
    after several steps, where rounding differences compound and the psi
    acceleration is a cancellation) and of the diagnostics.  Constraint
    residuals are cancellations: 1e-6 relative plus a round-off floor."""
    case = CASES[name]
    n = case["n"]
    N = n[0] * n[1] * n[2]
    Next = n[0] * n[1] * (n[2] + 2)
    for k, r in ref.items():
        g = np.asarray(got[k])
        r = np.asarray(r)
        assert g.shape == r.shape, (name, k, g.shape, r.shape)
        stepper = case["job"] in ("dopri", "rk4")
        if k == "dfield" or (k == "field" and stepper):
            tol = (dstep_rtol if k == "dfield" else step_rtol) if stepper else rtol
            errs = seg_rel_err(g, r, N, Next)
            assert max(errs.values()) <= tol, (name, k, errs)
        elif k == "field":
            assert np.abs(g - r).max() <= field_atol, (name, k, np.abs(g - r).max())
        elif k == "psi":
            for a, b in ((0, N), (N, 2 * N)):
                assert np.abs(g[a:b] - r[a:b]).max() <= rtol * np.abs(r[a:b]).max(), (name, k)
        elif k == "steps":
            # status, t, dt_did, dt_next equal to rounding; err_old is a
            # cancellation of the stage vectors (error weights sum to 0)
            assert np.all(g[:, 0] == r[:, 0]), (name, g, r)
            np.testing.assert_allclose(g[:, 1:4], r[:, 1:4], rtol=1e-12, err_msg=name)
            np.testing.assert_allclose(g[:, 4], r[:, 4], rtol=1e-2, err_msg=name)
            assert np.all(g[:, 5] == r[:, 5]), (name, g, r)
        elif k == "out_cstr":
            atol = np.array([1e-26, 1e-14, 1e-26, 1e-14])
            assert np.all(np.abs(g - r) <= 1e-6 * np.abs(r) + atol), (name, g, r)
        elif k.endswith("_smry"):
            np.testing.assert_allclose(g, r, rtol=1e-9, atol=1e-14, err_msg=f"{name} {k}")
        elif k.startswith("out_"):
            assert np.abs(g - r).max() <= 1e-10 * np.abs(r).max(), (name, k)
        else:  # rho_mean, pressure_mean, t
            np.testing.assert_allclose(g, r, rtol=1e-12, atol=1e-15, err_msg=f"{name} {k}")
