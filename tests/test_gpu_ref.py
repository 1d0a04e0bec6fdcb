"""GPU tests: the plain FP64 CUDA path, through the C ABI, against the
reference's own code (oracle/_ref: nikikilbertus/InstaHeat's src/*.c compiled
unmodified against the project's FFTW/HDF5/GSL shims), case by case
(tests/ref_cases.py).  Where the reference's sources are not staged on the
GPU host, the golden cases come from the committed fixture
tests/golden/ref_cases.npz, made from the same runs.

Tolerances: one RHS within 1e-11 of each state segment's largest magnitude
(the filtered state within 1e-13 absolute); after three DOPRI853 or four RK4
steps the state within 1e-11 and its derivative within 1e-10; accepted step
sizes to 1e-12 relative; diagnostics as in the oracle parity tests.
"""
import numpy as np
import pytest

import ref_cases

pytestmark = pytest.mark.gpu


def gpu_result(name, gpu_mod, oracle_mod):
    case = ref_cases.CASES[name]
    ctx = gpu_mod.Context(n=case["n"], L=case["L"], bins=case["bins"], precision=gpu_mod.PREC_F64)
    f = ref_cases.state(case, oracle_mod)
    N = ctx.N
    job = case["job"]
    out = {}
    if job == "rhs":
        r, ff = ctx.mk_rhs(f, filter=case["filter"], output=case["output"])
        rm, pm = ctx.means()
        out.update(dfield=r, field=ff, rho_mean=rm, pressure_mean=pm)
        if case["output"]:
            g = ctx.output()
            out.update(out_phi_ps=g["phi_ps"], out_psi_ps=g["psi_ps"], out_rho_ps=g["rho_ps"],
                       out_gw=g["gw"], out_cstr=g["cstr"])
            for i, k in enumerate(["phi", "dphi", "psi", "dpsi", "rho", "p"]):
                out[f"out_{k}_smry"] = g["smry"][i]
    elif job == "psi":
        ctx.set_state(f)
        ctx.initial_psi()
        out["psi"] = ctx.get_state()[2 * N:4 * N]
    elif job == "dopri":
        ctx.set_state(f)
        ctx.dopri_init(gpu_mod.dopri_cfg(1e-10, 1e-10, max_dt_hubble_fraction=1e-2), 0.0,
                       ref_cases.DOPRI_DT0)
        dt, rows = ref_cases.DOPRI_DT0, []
        for _ in range(ref_cases.DOPRI_STEPS):
            info = ctx.dopri_step(dt)
            # the reference keeps max(err, 1e-4) of the accepted try
            # (dopri853.c:505-540) and clears its reject flag
            rows.append([info.status, info.t, info.dt_did, info.dt_next, max(info.err, 1e-4), 0])
            dt = info.dt_next
        out.update(field=ctx.get_state(), dfield=ctx.get_dstate(), steps=np.array(rows))
    elif job == "rk4":
        ctx.set_state(f)
        dts, t_end = ref_cases.rk4_dts()
        for dt in dts:
            ctx.rk4_step(dt)
        ctx.prepare_output()  # run_rk4's closing prepare_and_save_timeslice
        out.update(field=ctx.get_state(), t=np.array(ctx.t))
    ctx.close()
    return out


@pytest.mark.parametrize("name", sorted(ref_cases.CASES))
def test_f64_gpu_matches_reference(gpu_mod, oracle_mod, name):
    want = ref_cases.reference(name)
    got = gpu_result(name, gpu_mod, oracle_mod)
    ref_cases.compare(name, got, want, rtol=1e-11, field_atol=1e-13, step_rtol=1e-11,
                      dstep_rtol=1e-10)
