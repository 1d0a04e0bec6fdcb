"""The C99 drop-in layer: parameters.sh -> header, host build, output reader.

InstaHeat fixes its parameters at compile time: a ``parameters.sh`` file of
``NAME="value"`` lines is turned into preprocessor definitions (its
``configure`` script substitutes them into ``main_template.h``; ENABLE_* and
OUTPUT_* switches become defined / undefined macros).  ``write_header`` does
the same for the standalone host: it emits ``ih_parameters.h`` with one
``#define`` per key, the same macro names and meanings, plus two optional
keys of this project, IH_PRECISION (IH_PREC_F64 | IH_PREC_MIXED) and
IH_DEVICE.

``build_host`` compiles ``ih_dropin.c`` (the reference-facing symbols) and
the standalone host ``host/ih_host.c`` against such a header and links them
with libinstaheat_gpu.so; ``read_container`` reads the host's output file.
"""
from __future__ import annotations

import re
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
ROOT = PKG.parent

# keys the drop-in layer and the standalone host read
REQUIRED = [
    "GRIDPOINTS_X", "GRIDPOINTS_Y", "GRIDPOINTS_Z",
    "SPATIAL_LOWER_BOUND_X", "SPATIAL_UPPER_BOUND_X", "SPATIAL_LOWER_BOUND_Y",
    "SPATIAL_UPPER_BOUND_Y", "SPATIAL_LOWER_BOUND_Z", "SPATIAL_UPPER_BOUND_Z",
    "INITIAL_TIME", "FINAL_TIME", "DELTA_T", "MINIMAL_DELTA_T", "MAX_STEPS", "MASS",
    "SMALLEST_SCALING", "LARGEST_SCALING", "BETA", "SAFE", "RELATIVE_TOLERANCE",
    "ABSOLUTE_TOLERANCE", "MAX_DT_HUBBLE_FRACTION", "WRITE_OUT_BUFFER_NUMBER",
    "POWER_SPECTRUM_BINS", "TIME_STEP_SKIPS", "STRIDE_X", "STRIDE_Y", "STRIDE_Z", "MAX_RUNTIME",
    "INTEGRATION_METHOD", "INITIAL_CONDITIONS",
]
# string-valued keys (quoted in the header)
STRINGS = {"DATAPATH", "INITIAL_DATAPATH"}
# keys that only configure FFTW, version control or the GSL stepper
IGNORED = {"FFTW_DEFAULT_FLAG", "VERSION_CONTROL", "GSL_OUTPUT_NUMBER", "THREAD_NUMBER",
           "FFTW_THREAD_NUMBER"}


def read_parameters(src) -> dict:
    """NAME -> value from a parameters.sh file (path) or its text: comments
    after '#' and blank lines dropped, quotes removed, as configure does."""
    text = Path(src).read_text() if isinstance(src, (str, Path)) and Path(src).exists() else str(src)
    out = {}
    for line in text.splitlines():
        line = re.sub(r"\s*#.*", "", line).strip()
        if not line:
            continue
        if "=" not in line:
            raise ValueError(f"not a NAME=value line: {line!r}")
        name, value = line.split("=", 1)
        out[name.strip()] = value.strip().strip('"')
    return out


def _switch(name: str) -> bool:
    return name.startswith("ENABLE") or name.startswith("OUTPUT")


def header_text(params: dict, origin: str = "parameters") -> str:
    missing = [k for k in REQUIRED if k not in params]
    if missing:
        raise ValueError(f"parameters missing: {', '.join(missing)}")
    lines = [f"/* ih_parameters.h -- generated by instaheat_gb300.dropin from {origin} */",
             "#ifndef IH_PARAMETERS_H", "#define IH_PARAMETERS_H"]
    for name, value in params.items():
        if name in IGNORED:
            continue
        if _switch(name):
            lines.append(f"#define {name}" if value.strip() == "1" else f"/* {name} off */")
        elif name in STRINGS:
            lines.append(f'#define {name} ("{value}")')
        else:
            lines.append(f"#define {name} ({value})")
    lines.append("#endif")
    return "\n".join(lines) + "\n"


def render_template(template: str, params: dict) -> str:
    """The substitution InstaHeat's configure script applies to its
    main_template.h: __NAME__ -> value, and for ENABLE_* / OUTPUT_* switches
    __NAME__ -> NAME (value 1) or NOT_NAME (so `#define __NAME__` defines the
    switch or an unused macro)."""
    out = template
    for name, value in params.items():
        if _switch(name):
            out = out.replace(f"__{name}__", name if value.strip() == "1" else f"NOT_{name}")
        else:
            out = out.replace(f"__{name}__", value)
    return out


def write_header(params: dict, path, origin: str = "parameters") -> Path:
    path = Path(path)
    path.write_text(header_text(params, origin))
    return path


def build_host(params, out_dir, cc: str | None = None) -> Path:
    """Compile the standalone host + drop-in layer for one parameter set and
    return the executable.  Requires libinstaheat_gpu.so (build.build())."""
    from .. import build as libbuild
    lib = libbuild.build()
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    if not isinstance(params, dict):
        params = read_parameters(params)
    write_header(params, out_dir / "ih_parameters.h")
    exe = out_dir / "instaheat_host"
    cc = cc or shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found")
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-D_POSIX_C_SOURCE=200809L",
           "-I", str(out_dir), "-I", str(HERE / "host"), "-I", str(ROOT / "include"),
           str(HERE / "ih_dropin.c"), str(HERE / "host" / "ih_host.c"),
           "-L", str(lib.parent), "-linstaheat_gpu", f"-Wl,-rpath,{lib.parent}", "-lm",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe


def read_container(path) -> dict:
    """name -> array: parameter datasets as 1D arrays, time series as
    (slices, dim) arrays concatenated over their chunks."""
    data = Path(path).read_bytes()
    if data[:8] != b"IHCONT01":
        raise ValueError("not an instaheat output container")
    pos, series, params = 8, {}, {}
    while pos < len(data):
        (ln,) = struct.unpack_from("<I", data, pos)
        pos += 4
        name = data[pos:pos + ln].decode()
        pos += ln
        kind, rows, dim = struct.unpack_from("<IQQ", data, pos)
        pos += 20
        vals = np.frombuffer(data, dtype="<f8", count=rows * dim, offset=pos).reshape(rows, dim)
        pos += 8 * rows * dim
        if kind == 0:
            params[name] = vals[0].copy()
        else:
            series.setdefault(name, []).append(vals.copy())
    out = dict(params)
    out.update({k: np.concatenate(v, axis=0) for k, v in series.items()})
    return out
