"""Build libinstaheat_gpu.so (sm_103a) and the C99 drop-in host layer in tree.

nvcc compiles each CUDA translation unit in parallel for
``-gencode arch=compute_103a,code=sm_103a`` and links one shared library into
``instaheat_gb300/_lib/``.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libinstaheat_gpu.so"
CU_SOURCES = ["ih_api.cu", "ih_fft.cu", "ih_zwide.cu", "ih_rhs.cu", "ih_stepper.cu", "ih_mlp.cu",
              "ih_noalloc.cu", "ih_peak.cu", "ih_gwplane.cu"]
HEADERS = ["ih_internal.cuh", "ih_fftcore.cuh", "ih_tensor.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libinstaheat_gpu.so")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    OUT.mkdir(exist_ok=True)
    include = ROOT / "include" / "instaheat_gpu.h"
    deps_common = [CSRC / h for h in HEADERS] + [include]
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
             "-I", str(ROOT / "include")] + ARCH + list(extra_flags)
    nv = nvcc()

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = OUT / (Path(src).stem + ".o")
        if force or _stale(o, [s] + deps_common):
            cmd = [nv] + flags + ["-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        objs = list(ex.map(compile_one, CU_SOURCES))
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [nv, "-shared"] + ARCH + ["-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
