"""CPU tests of the C99 drop-in layer: parameters.sh -> header, the host
build (-std=c99 -Wall -Wextra -Werror), the exported reference symbols, and
source compatibility with a main.h generated from the reference's own
template (when the reference tree is present)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from instaheat_gb300 import dropin
from oracle import ref

HERE = Path(__file__).resolve().parent
PARAMS = HERE / "dropin"
# the reference's sources as oracle/ref.py stages them (unchanged copies)
REF_SRC = ref.STAGE

# the symbols toolbox.h:15-35, dopri853.h:51 and rk4.h:14 declare
REFERENCE_SYMBOLS = ["mk_rhs", "prepare_and_save_timeslice", "mk_gradient_squared_and_laplacian",
                     "mk_rho_and_p", "fft", "ifft", "mean", "variance", "run_dopri853", "run_rk4",
                     "evo_flags"]


def test_read_parameters_like_configure():
    p = dropin.read_parameters('A="1.0" # comment\n\n# full line\nENABLE_GW="1"\nB=2\n')
    assert p == {"A": "1.0", "ENABLE_GW": "1", "B": "2"}
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    assert p["INTEGRATION_METHOD"] == "DOPRI853" and p["GRIDPOINTS_X"] == "16"


def test_header_text():
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    h = dropin.header_text(p)
    assert "#define GRIDPOINTS_X (16)" in h
    assert "#define ENABLE_GW\n" in h
    assert "/* OUTPUT_PSI off */" in h
    assert '#define DATAPATH ("unused")' in h
    assert "FFTW_DEFAULT_FLAG" not in h
    del p["MASS"]
    with pytest.raises(ValueError, match="MASS"):
        dropin.header_text(p)


def test_render_template_substitution():
    t = "#define MASS (__MASS__)\n#define __ENABLE_GW__\n#define __OUTPUT_PHI__\n"
    r = dropin.render_template(t, {"MASS": "4.0", "ENABLE_GW": "1", "OUTPUT_PHI": "0"})
    assert r == "#define MASS (4.0)\n#define ENABLE_GW\n#define NOT_OUTPUT_PHI\n"


@pytest.mark.parametrize("name", ["parameters_dopri853.sh", "parameters_rk4.sh",
                                  "parameters_landing.sh", "parameters_dense.sh"])
def test_host_builds_warning_free(tmp_path, name):
    exe = dropin.build_host(PARAMS / name, tmp_path / "host")
    assert exe.exists()


def test_dropin_object_exports_reference_symbols(tmp_path):
    dropin.write_header(dropin.read_parameters(PARAMS / "parameters_dopri853.sh"),
                        tmp_path / "ih_parameters.h")
    obj = tmp_path / "ih_dropin.o"
    cc = shutil.which("gcc") or shutil.which("cc")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-c", "-I", str(tmp_path),
                    "-I", str(dropin.HERE / "host"), "-I", str(dropin.ROOT / "include"),
                    str(dropin.HERE / "ih_dropin.c"), "-o", str(obj)], check=True)
    nm = subprocess.run(["nm", "-g", "--defined-only", str(obj)], capture_output=True, text=True,
                        check=True).stdout.split()
    for s in REFERENCE_SYMBOLS:
        assert s in nm, s


@pytest.mark.skipif(not ref.available(), reason="the reference's sources are not staged")
def test_dropin_compiles_against_reference_generated_headers(tmp_path):
    """ih_dropin.c against the main.h the reference's configure would make from
    its own parameters.sh (with FFTW/HDF5 type stubs): syntax-only."""
    params = dropin.read_parameters(REF_SRC / "parameters.sh")
    # the reference's default file is 1D and RK4-free; the drop-in needs the
    # DOPRI853 keys, which it has
    (tmp_path / "main.h").write_text(
        dropin.render_template((REF_SRC / "main_template.h").read_text(), params))
    shutil.copy(REF_SRC / "io.h", tmp_path / "io.h")
    cc = shutil.which("gcc") or shutil.which("cc")
    r = subprocess.run([cc, "-std=gnu99", "-fsyntax-only", "-I", str(tmp_path),
                        "-I", str(PARAMS / "stubs"), "-I", str(dropin.ROOT / "include"),
                        str(dropin.HERE / "ih_dropin.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_host_without_gpu_exits_with_the_error(tmp_path):
    """Without a GPU the drop-in does what the reference does on a failure:
    a message on stderr and exit(EXIT_FAILURE) -- no CPU fallback."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    exe = dropin.build_host(PARAMS / "parameters_dopri853.sh", tmp_path / "host")
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    n = int(p["GRIDPOINTS_X"])
    N, Next = n ** 3, 2 * n * n * (n // 2 + 1)
    f = np.zeros(4 * N + 4 * Next + 1)
    f[:N] = 1.0
    f[-1] = 1.0
    f.tofile(tmp_path / "init.bin")
    r = subprocess.run([str(exe), str(tmp_path / "init.bin"), str(tmp_path / "out.ihc")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "CUDA" in r.stderr or "CUDA" in r.stdout, (r.stdout, r.stderr)


def _relinked(name="parameters_dopri853.sh"):
    from instaheat_gb300 import build as libbuild
    p = dropin.read_parameters(PARAMS / name)
    keys = {k: v for k, v in p.items()
            if k in ref.DEFAULTS and k not in ("DATAPATH", "INITIAL_DATAPATH")}
    params = ref.config(**keys)
    exe = ref.build_dropin(params, libbuild.build(), dropin.HERE / "ih_dropin.c",
                           dropin.ROOT / "include")
    return p, params, exe


@pytest.mark.skipif(not ref.available(), reason="the reference's sources are not staged")
def test_reference_program_relinks_with_the_dropin():
    """The reference's own main.c, setup.c and io.c, unchanged, link against
    ih_dropin.o + libinstaheat_gpu.so in place of toolbox.o, dopri853.o,
    dopri853_constants.o and rk4.o: main comes from the reference, the
    toolbox/stepper symbols from the drop-in, nothing is left undefined."""
    _, _, exe = _relinked()
    syms = subprocess.run(["nm", str(exe)], capture_output=True, text=True, check=True).stdout
    defined = {ln.split()[-1] for ln in syms.splitlines() if len(ln.split()) == 3}
    for s in REFERENCE_SYMBOLS + ["main", "allocate_and_init_all", "h5_create_empty_by_path",
                                  "save"]:
        assert s in defined, s
    assert "ihref_main" not in defined and "perform_step" not in defined


@pytest.mark.skipif(not ref.available(), reason="the reference's sources are not staged")
def test_relinked_program_without_gpu_exits_with_the_error(oracle_mod):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p, params, exe = _relinked()
    o = oracle_mod.Oracle(n=(int(p["GRIDPOINTS_X"]),) * 3, bins=int(p["POWER_SPECTRUM_BINS"]))
    r, _ = ref.run_program(exe, o.ic(seed=11, amp=1e-3, psi=False), exe.parent, timeout=120)
    assert r.returncode != 0
    assert "Read initial data from file." in r.stdout  # the reference's set-up ran
    assert "CUDA" in r.stderr, r.stderr


@pytest.mark.skipif(not ref.available(), reason="the reference's sources are not staged")
@pytest.mark.parametrize("method", ["DOPRI853", "RK4"])
def test_relinked_program_builds_with_timing(method):
    """ENABLE_TIMING=1 (the runtime datasets of main.c:131-168) with the
    reference's own main.h: the drop-in compiles and links for either
    integration method (the reference's own rk4.c does not compile with it,
    rk4.c:120-124; the relinked program does not contain it)."""
    from instaheat_gb300 import build as libbuild
    p = dropin.read_parameters(PARAMS / "parameters_dopri853.sh")
    keys = {k: v for k, v in p.items()
            if k in ref.DEFAULTS and k not in ("DATAPATH", "INITIAL_DATAPATH")}
    keys.update(ENABLE_TIMING="1", INTEGRATION_METHOD=method)
    exe = ref.build_dropin(ref.config(**keys), libbuild.build(), dropin.HERE / "ih_dropin.c",
                           dropin.ROOT / "include")
    assert exe.exists()
