"""Build libastro_cuda.so in-tree for sm_103a with nvcc.

The CUDA translation units are compiled in parallel and linked into
astro_gb300/lib/libastro_cuda.so. Run as ``python -m astro_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libastro_cuda.so"
OBJ_DIR = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
SOURCES = ["sort.cu", "sort_noalloc.cu", "build.cu", "traverse.cu", "traverse_group.cu", "splat.cu",
           "context.cu", "tune.cu", "ic.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def extra_flags() -> list:
    """Additional nvcc flags from ASTRO_NVCC_FLAGS (space-separated), for
    builds with other compile-time tuning constants."""
    return os.environ.get("ASTRO_NVCC_FLAGS", "").split()


def _compile(src: str, verbose_ptxas: bool) -> Path:
    obj = OBJ_DIR / (src + ".o")
    s = CSRC / src
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-c", str(s), "-o", str(obj)]
    else:
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags(), "-c", str(s), "-o", str(obj)]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    """Compile every translation unit and link the shared library."""
    OBJ_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    deps = sorted(CSRC.glob("*")) + [PKG.parent / "include" / "astro_cuda.h"]
    newest = max(p.stat().st_mtime for p in deps)
    if LIB.exists() and not force and not extra_flags() and LIB.stat().st_mtime >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_oracle() -> Path:
    """Compile the CPU restatement used by tests and the CPU baseline."""
    oracle = PKG.parent / "oracle"
    res = subprocess.run(["make", "-C", str(oracle)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return oracle / "liboracle_astro.so"


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
