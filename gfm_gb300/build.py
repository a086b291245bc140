"""Build the native library in-tree: gfm_gb300/libgfm_gb300.so.

All CUDA translation units are compiled for sm_103a only (GB300), in parallel,
with nvcc; host C++ (case construction) with the same driver.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgfm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["asm.cu", "adi.cu", "adi_plane.cu", "bc.cu", "solver.cu", "noalloc.cu", "lp.cu", "lp_tc.cu", "lpsolve.cu", "rad.cu", "wall.cu", "gas.cu", "minor.cu"]
# per-file flags: the radiation transfer rounds every product and sum as the
# reference does (angle ties and energy splits must break the same way)
FILE_FLAGS = {"rad.cu": ["--fmad=false"], "gas.cu": ["--fmad=false"]}
CXX_SOURCES = ["case_build.cpp", "case_files.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gfm_gb300")
    return exe


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _needs(obj: pathlib.Path, src: pathlib.Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gfm_gb300.h"]
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in CUDA_SOURCES:
        src, obj = CSRC / s, BUILD / (s + ".o")
        if force or _needs(obj, src):
            extra = os.environ.get("GFM_NVCC_EXTRA", "").split()
            jobs.append([cc, "-std=c++17", *ARCH, "-O3", "-lineinfo", *FILE_FLAGS.get(s, []), *extra,
                         "-Xcompiler", "-fPIC", "-c", str(src), "-o", str(obj)])
    for s in CXX_SOURCES:
        src, obj = CSRC / s, BUILD / (s + ".o")
        if force or _needs(obj, src):
            jobs.append([cc, "-std=c++17", "-O2", "-x", "c++", "-Xcompiler", "-fPIC",
                         "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    objs = [str(BUILD / (s + ".o")) for s in CUDA_SOURCES + CXX_SOURCES]
    if force or jobs or not LIB.exists():
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
