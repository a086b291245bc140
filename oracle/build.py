"""Build the CPU oracle (test infrastructure): oracle/libgfm_oracle.so.

Compiled with -ffp-contract=off so that x86 and Arm hosts produce identical
FP64 results (no fused multiply-add contraction).
"""
from __future__ import annotations

import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "libgfm_oracle.so"


def build(check_bounds: bool = False) -> pathlib.Path:
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler for the oracle")
    out = HERE / ("libgfm_oracle_checked.so" if check_bounds else "libgfm_oracle.so")
    src = HERE / "gfm_oracle.cpp"
    if out.exists() and out.stat().st_mtime > max(src.stat().st_mtime, (HERE / "gfm_oracle.h").stat().st_mtime):
        return out
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(out), str(src)]
    if check_bounds:
        cmd.insert(1, "-DGFO_CHECK")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return out


if __name__ == "__main__":
    print(build(check_bounds="--check" in sys.argv))
