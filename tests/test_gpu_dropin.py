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

import dropin_expected as X
from instaheat_gb300 import dropin

PARAMS = Path(__file__).resolve().parent / "dropin"
pytestmark = pytest.mark.gpu


def _run_host(tmp_path, name, oracle_mod):
    import subprocess
    p = dropin.read_parameters(PARAMS / name)
    exe = dropin.build_host(p, tmp_path / "host")
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    X.initial_state(o).tofile(tmp_path / "init.bin")
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
    exp, steps, f_exp = X.expected_dopri(oracle_mod, p)
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
    exp, f_exp = X.expected_rk4(oracle_mod, p)
    _compare_series(got, exp)
    assert np.abs(final - f_exp).max() <= 1e-9 * np.abs(f_exp[: 4 * 16 ** 3]).max()


def test_run_dopri853_output_landing(tmp_path, oracle_mod):
    p, got, _ = _run_host(tmp_path, "parameters_landing.sh", oracle_mod)
    exp = X.expected_landing(oracle_mod, p)
    times = got["time"][:, 0]
    # slices at 0, 0.02 and 0.04 (landed); the third fills the buffer of three,
    # so the wrap-up adds no slice at 0.05 (dopri853.c:209-212)
    np.testing.assert_allclose(times, [0.0, 0.02, 0.04], atol=1e-14)
    _compare_series(got, exp)


def test_run_dopri853_dense_output(tmp_path, oracle_mod):
    p, got, _ = _run_host(tmp_path, "parameters_dense.sh", oracle_mod)
    exp = X.expected_dense(oracle_mod, p)
    times = got["time"][:, 0]
    # slices at 0, 0.02 and 0.04 from the continuous extension (the steps are
    # not shortened); the buffer of three is full, so the wrap-up adds none
    np.testing.assert_allclose(times, [0.0, 0.02, 0.04], atol=1e-14)
    _compare_series(got, exp)


@pytest.mark.parametrize("name", ["parameters_dopri853.sh", "parameters_rk4.sh"])
def test_reference_program_relinked_with_the_dropin(oracle_mod, name):
    """The reference's own main.c, setup.c and io.c, unchanged, relinked with
    ih_dropin.o + libinstaheat_gpu.so (oracle/ref.py build_dropin), against
    the reference program itself (oracle/_ref, CPU) on the same .dat initial
    data: every recorded dataset slice by slice, the step counters and the
    followup snapshot."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the reference's sources are not staged (oracle/_ref/src)")
    from instaheat_gb300 import build as libbuild
    p = dropin.read_parameters(PARAMS / name)
    keys = {k: v for k, v in p.items()
            if k in ref.DEFAULTS and k not in ("DATAPATH", "INITIAL_DATAPATH")}
    params = ref.config(**keys)
    exe = ref.build_dropin(params, libbuild.build(), dropin.HERE / "ih_dropin.c",
                           dropin.ROOT / "include")
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    f0 = X.initial_state(o)
    r, got = ref.run_program(exe, f0, exe.parent, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    want = ref.run(ref.build(params), "main", f0)["h5"]
    series = [k for k, v in want.items()
              if isinstance(v, np.ndarray) and k in X.SERIES]
    assert series, sorted(want)
    _compare_series({k: got[k] for k in series}, {k: want[k] for k in series})
    for k in ("steps_total", "steps_ok", "steps_bad", "gridpoints_internal", "tolerances",
              "strides_space", "mass", "filter", "gravitational_waves"):
        if k in want:
            assert got[k].tolist() == want[k].tolist(), k
    if "followup" in want:
        sc = np.abs(want["followup"][:4 * o.N]).max()
        assert np.abs(got["followup"] - want["followup"]).max() <= 1e-9 * sc
    assert got["method"] == want["method"] == b"hyperbolic"
