"""GPU tests of the failure paths, each provoked from the host (no fault, trap
or hang on the GPU): a non-finite value in the state, a step-size underflow,
the run limits MAX_STEPS and MAX_RUNTIME, and the controller's noise-floor
and error-breakdown controls.

The reference handles these in its run loop (dopri853.c:118-158): it prints a
message and ends the run (underflow, step and wall-clock limits) and still
wraps up (final slice, followup snapshot, step counters).  The relinked
program (the reference's own main.c/setup.c/io.c with the drop-in layer) is
compared with the reference program itself on each of those paths.
"""
from pathlib import Path

import numpy as np
import pytest

import dropin_expected as X
from instaheat_gb300 import dropin

pytestmark = pytest.mark.gpu

PARAMS = Path(__file__).resolve().parent / "dropin"
IH_ERR_UNDERFLOW, IH_ERR_NAN = 5, 6


def _state(o, seed=3):
    f = o.ic(seed=seed, amp=1e-3)
    rng = np.random.default_rng(seed)
    f[4 * o.N:-1] = 1e-6 * rng.standard_normal(4 * o.Next)
    return f


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_nonfinite_state_reports_nan_and_context_recovers(gpu_mod, oracle_mod, prec):
    """A NaN written into a host state: the DOPRI853 step returns IH_ERR_NAN
    (the reference's CHECK_FOR_NAN, toolbox.c:829-862, as a status raised from
    the reductions the kernels already do); a clean state afterwards steps
    normally in the same context."""
    n = (16, 16, 16)
    p = gpu_mod.PREC_F64 if prec == "f64" else gpu_mod.PREC_MIXED
    ctx = gpu_mod.Context(n=n, precision=p)
    o = oracle_mod.Oracle(n=n)
    f = _state(o)
    bad = f.copy()
    bad[123] = np.nan
    cfg = gpu_mod.dopri_cfg(1e-8, 1e-8)
    ctx.set_state(bad)
    with pytest.raises(gpu_mod.IHError) as ei:
        ctx.dopri_init(cfg, 0.0, 1e-3)
        ctx.dopri_step(1e-3)
    assert ei.value.status == IH_ERR_NAN
    assert "non-finite" in str(ei.value)
    ctx.set_state(f)
    ctx.dopri_init(cfg, 0.0, 1e-3)
    info = ctx.dopri_step(1e-3)
    assert info.status == 0 and info.dt_did == 1e-3
    assert np.isfinite(ctx.get_state()).all()
    ctx.close()


def test_dt_min_underflow_ends_the_run(gpu_mod, oracle_mod):
    """A proposed step at or below MINIMAL_DELTA_T ends the run loop with
    IH_ERR_UNDERFLOW after the accepted step (dopri853.c:150-153)."""
    n = (16, 16, 16)
    ctx = gpu_mod.Context(n=n, precision=gpu_mod.PREC_F64)
    o = oracle_mod.Oracle(n=n)
    ctx.set_state(_state(o))
    ctx.dopri_init(gpu_mod.dopri_cfg(1e-10, 1e-10, dt_min=1.0), 0.0, 1e-3)
    with pytest.raises(gpu_mod.IHError) as ei:
        ctx.dopri_run(10.0)
    assert ei.value.status == IH_ERR_UNDERFLOW
    assert abs(ctx.t - 1e-3) < 1e-15  # the one accepted step stands
    ctx.close()


def test_error_breakdown_sums_to_the_error_norm(gpu_mod, oracle_mod):
    """The per-segment error sums of the last try reproduce its error norm
    through error()'s formula (dopri853.c:469-486):
    err = dt S_er / sqrt(Ntot (S_er + 0.01 S_bhh)), the pairs' second (er) and
    first (b - bhh) members summed over segments."""
    n = (16, 16, 16)
    ctx = gpu_mod.Context(n=n, precision=gpu_mod.PREC_F64)
    o = oracle_mod.Oracle(n=n)
    ctx.set_state(_state(o))
    ctx.dopri_init(gpu_mod.dopri_cfg(1e-10, 1e-10), 0.0, 1e-3)
    ctx.error_breakdown(True)
    dt = 1e-3
    for _ in range(3):
        info = ctx.dopri_step(dt)
        bd = ctx.error_breakdown()
        s_bhh = sum(v[0] for v in bd.values())
        s_er = sum(v[1] for v in bd.values())
        err = info.dt_did * s_er / np.sqrt(o.Ntot * (s_er + 0.01 * s_bhh))
        # the scale factor's element is not in the breakdown: it is the
        # remainder (about 1e-5 of the norm here)
        assert abs(err - info.err) <= 1e-4 * info.err, (err, info.err, bd)
        assert err <= info.err * (1 + 1e-12)
        assert all(v[0] >= 0 and v[1] >= 0 for v in bd.values())
        dt = info.dt_next
    ctx.error_breakdown(False)
    with pytest.raises(gpu_mod.IHError):
        ctx.error_breakdown()
    ctx.close()


def test_noise_floor_setter(gpu_mod, oracle_mod):
    """The mixed form's rounding floor (ih_dopri853_set_noise_floor): a larger
    eta removes more of each error element, so the same try's error norm does
    not grow with eta; the FP64 form ignores it; negative eta is refused."""
    n = (32, 32, 32)
    o = oracle_mod.Oracle(n=n)
    f = _state(o, seed=8)
    errs = {}
    for eta in (0.0, 256.0, 4096.0):
        ctx = gpu_mod.Context(n=n, precision=gpu_mod.PREC_MIXED)
        ctx.set_noise_floor(eta)
        ctx.set_state(f)
        ctx.dopri_init(gpu_mod.dopri_cfg(1e-8, 1e-8), 0.0, 1e-2)
        errs[eta] = ctx.dopri_step(1e-2).err
        ctx.close()
    assert errs[256.0] <= errs[0.0] and errs[4096.0] <= errs[256.0], errs
    assert errs[4096.0] < errs[0.0], errs
    e64 = []
    for eta in (0.0, 4096.0):
        ctx = gpu_mod.Context(n=n, precision=gpu_mod.PREC_F64)
        ctx.set_noise_floor(eta)
        ctx.set_state(f)
        ctx.dopri_init(gpu_mod.dopri_cfg(1e-8, 1e-8), 0.0, 1e-2)
        e64.append(ctx.dopri_step(1e-2).err)
        with pytest.raises(gpu_mod.IHError):
            ctx.set_noise_floor(-1.0)
        ctx.close()
    assert e64[0] == e64[1]


@pytest.mark.parametrize("case,keys,message", [
    ("underflow", {"MINIMAL_DELTA_T": "1.0"}, "Stepsize underflow"),
    ("max_steps", {"MAX_STEPS": "2"}, "Reached maximal number of steps."),
    ("max_runtime", {"MAX_RUNTIME": "0"}, "Reached specified maximal runtime."),
])
def test_run_limits_match_the_reference(oracle_mod, case, keys, message):
    """The relinked program and the reference program on the same .dat data
    end the run on the same step with the same message, and write the same
    slices, counters and followup snapshot."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the reference's sources are not staged (oracle/_ref/src)")
    from instaheat_gb300 import build as libbuild
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    p.update(keys)
    sel = {k: v for k, v in p.items()
           if k in ref.DEFAULTS and k not in ("DATAPATH", "INITIAL_DATAPATH")}
    params = ref.config(**sel)
    exe = ref.build_dropin(params, libbuild.build(), dropin.HERE / "ih_dropin.c",
                           dropin.ROOT / "include")
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f0 = X.initial_state(o)
    r, got = ref.run_program(exe, f0, exe.parent, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    want_run = ref.run(ref.build(params), "main", f0)
    want = want_run["h5"]
    assert message in r.stdout + r.stderr
    assert message in want_run["stdout"]
    for k in ("steps_total", "steps_ok", "steps_bad"):
        assert got[k].tolist() == want[k].tolist(), (k, got[k], want[k])
    for k in X.SERIES:
        if k in want:
            g, w = got[k], want[k]
            assert g.shape == w.shape, (k, g.shape, w.shape)
            if k in ("time", "a"):
                np.testing.assert_allclose(g, w, rtol=1e-12, err_msg=k)
            elif k == "constraints":
                atol = np.array([1e-26, 1e-14, 1e-26, 1e-14])
                assert np.all(np.abs(g - w) <= 1e-6 * np.abs(w) + atol), k
            else:
                assert np.abs(g - w).max() <= 1e-9 * np.abs(w).max() + 1e-300, k
    sc = np.abs(want["followup"][:4 * o.N]).max()
    assert np.abs(got["followup"] - want["followup"]).max() <= 1e-9 * sc


def test_dropin_host_with_nonfinite_state_exits_with_the_error(tmp_path, oracle_mod):
    """Through the drop-in layer a non-finite state ends the program the way
    the reference ends on a failure: a message on stderr, exit(EXIT_FAILURE)."""
    import subprocess
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    exe = dropin.build_host(p, tmp_path / "host")
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f = X.initial_state(o)
    f[7] = np.inf
    f.tofile(tmp_path / "init.bin")
    r = subprocess.run([str(exe), str(tmp_path / "init.bin"), str(tmp_path / "out.ihc")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode != 0
    assert "non-finite" in r.stderr or "NaN" in r.stderr, (r.stdout[-1000:], r.stderr[-1000:])
