"""CPU tests: pin the oracle to the reference's own code.

oracle/ref.py compiles nikikilbertus/InstaHeat's src/toolbox.c, setup.c,
io.c, rk4.c, dopri853.c, dopri853_constants.c and main.c unmodified against
project shims (FFTW3 API over the oracle's FP64 transforms, an HDF5
recorder, GSL's MT19937).  Each case of tests/ref_cases.py runs through it
and through the C oracle on the same seeded state; they agree to 1e-13 of
each state segment (the FFTs are the same code; the rest differs only in the
order of floating-point reductions).  Where the reference's sources are not
staged (oracle/_ref/src), the golden cases come from the committed fixture.
After three DOPRI853 or four RK4 steps the states agree to 1e-12 and the
derivatives to 1e-11 (the psi acceleration is a cancellation).
"""
import numpy as np
import pytest

import ref_cases
from oracle import ref

needs_ref = pytest.mark.skipif(not ref.available(),
                               reason="the reference's sources are not staged (oracle/_ref/src)")


@pytest.mark.parametrize("name", sorted(ref_cases.CASES))
def test_oracle_matches_reference(oracle_mod, name):
    want = ref_cases.reference(name)
    got = ref_cases.oracle_result(name, oracle_mod)
    ref_cases.compare(name, got, want, rtol=1e-13, field_atol=1e-14, step_rtol=1e-12,
                      dstep_rtol=1e-11)


@needs_ref
def test_golden_fixture_is_the_reference_output():
    """The committed fixture holds what the reference computes now (to
    1e-12 of each array's largest magnitude: OpenMP reductions may sum in
    another order on another host or thread count)."""
    z = np.load(ref_cases.GOLDEN)
    for name, case in ref_cases.CASES.items():
        if not case.get("golden"):
            continue
        live = ref_cases.run_reference(name)
        assert sorted(live) == sorted(k.split("/", 1)[1] for k in z.files if k.startswith(name + "/"))
        for k, v in live.items():
            g = z[f"{name}/{k}"]
            assert g.shape == v.shape, (name, k)
            assert np.abs(g - v).max() <= 1e-12 * np.abs(v).max(), (name, k)


@needs_ref
def test_mt19937_known_answers():
    """The GSL shim's generator: MT19937 seeded with 5489 (the generator's
    reference seed) gives 3499211612 first and 4123659995 as its 10000th
    output; gsl_rng_uniform divides by 2^32."""
    import ctypes as C
    L = C.CDLL(str(ref.build() / "libihref.so"))
    L.gsl_rng_alloc.restype = C.c_void_p
    L.gsl_rng_alloc.argtypes = [C.c_void_p]
    L.gsl_rng_set.argtypes = [C.c_void_p, C.c_ulong]
    L.gsl_rng_get.restype = C.c_ulong
    L.gsl_rng_get.argtypes = [C.c_void_p]
    L.gsl_rng_uniform.restype = C.c_double
    L.gsl_rng_uniform.argtypes = [C.c_void_p]
    L.gsl_rng_free.argtypes = [C.c_void_p]
    r = L.gsl_rng_alloc(C.c_void_p.in_dll(L, "gsl_rng_mt19937").value)
    L.gsl_rng_set(r, 5489)
    vals = [L.gsl_rng_get(r) for _ in range(10000)]
    assert vals[0] == 3499211612 and vals[-1] == 4123659995
    L.gsl_rng_set(r, 5489)
    assert L.gsl_rng_uniform(r) == 3499211612 / 2.0 ** 32
    L.gsl_rng_free(r)


@needs_ref
def test_reference_rk4_lands_on_final_time():
    out = ref_cases.run_reference("rk4_16x16x8")
    dts, t_end = ref_cases.rk4_dts()
    assert float(out["t"]) == t_end


def _ref_params(path):
    from instaheat_gb300 import dropin
    p = dropin.read_parameters(path)
    keys = {k: v for k, v in p.items()
            if k in ref.DEFAULTS and k not in ("DATAPATH", "INITIAL_DATAPATH")}
    return p, ref.config(**keys)


@needs_ref
@pytest.mark.parametrize("name", ["parameters_dopri853.sh", "parameters_rk4.sh"])
def test_reference_main_run_matches_loop_restatement(oracle_mod, name):
    """The whole reference program (main.c:73-113: set-up from a .dat file
    with the psi solve, run_dopri853 or run_rk4 with save() every
    TIME_STEP_SKIPS steps, wrap-up, HDF5 output through the recorder) against
    the loop restatement over the oracle that the GPU drop-in tests use."""
    import dropin_expected as X
    from pathlib import Path
    p, params = _ref_params(Path(__file__).resolve().parent / "dropin" / name)
    n = (int(p["GRIDPOINTS_X"]),) * 3
    o = oracle_mod.Oracle(n=n, bins=int(p["POWER_SPECTRUM_BINS"]))
    r = ref.run(ref.build(params), "main", X.initial_state(o))
    h5 = r["h5"]
    if "dopri" in name:
        exp, steps, f_exp = X.expected_dopri(oracle_mod, p)
        for k, v in steps.items():
            assert h5[k].tolist() == [v], k
        assert np.abs(h5["followup"] - f_exp).max() <= 1e-12 * np.abs(f_exp[:4 * o.N]).max()
    else:
        exp, f_exp = X.expected_rk4(oracle_mod, p)
    for k, e in exp.items():
        g = h5[k].reshape(e.shape)
        if k in ("time", "a"):
            np.testing.assert_allclose(g, e, rtol=1e-14, err_msg=k)
        elif k == "constraints":
            atol = np.array([1e-26, 1e-14, 1e-26, 1e-14])
            assert np.all(np.abs(g - e) <= 1e-8 * np.abs(e) + atol), k
        else:
            assert np.abs(g - e).max() <= 1e-11 * np.abs(e).max() + 1e-300, k
    # the parameter datasets io.c:125-265 writes
    assert h5["gridpoints_internal"].tolist() == [float(x) for x in n]
    assert h5["tolerances"].tolist() == [float(p["RELATIVE_TOLERANCE"]),
                                         float(p["ABSOLUTE_TOLERANCE"])]
    assert h5["method"] == b"hyperbolic"
    assert h5["calls_rhs"][0] > 0
