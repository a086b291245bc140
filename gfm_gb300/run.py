"""Run the solver on a named case: `python -m gfm_gb300.run --case large
--prec mixed --iters 1 --warmup 3`.

Builds the case (a synthetic furnace, or TC21 case 0041 from the case files
in tests/golden), starts it (INITSV), runs `warmup` outer iterations and then
`iters` more, and prints one JSON line with the device time per iteration,
the line solver's share and the last iteration's residuals.  It is the
workload the kernel profiles in profiles/ were taken on.

`--minor N` then runs INITSVM (from the major species) and N MSFLOW
iterations of the minor species, and one emission update on the band model
(RAD_GAS and SOOTA), and adds their times.
"""
from __future__ import annotations

import argparse
import json
import pathlib
import shutil
import tempfile

from . import Case, GpuSolver, abi, configs

CASES = {"tiny": configs.tiny_furnace, "small": configs.small_furnace, "medium": configs.medium_furnace,
         "large": configs.large_furnace, "xl": configs.xl_furnace}


def build_case(name: str) -> Case:
    if name == "tc21":
        gold = pathlib.Path(__file__).resolve().parent.parent / "tests" / "golden" / "case0041"
        with tempfile.TemporaryDirectory() as d:
            for n in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat", "relaxfactorc.txt"):
                shutil.copyfile(gold / n, pathlib.Path(d) / n)
            return Case.from_files(d, "0041")
    return Case(CASES[name]())


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=sorted(CASES) + ["tc21"], default="large")
    ap.add_argument("--prec", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--adi", choices=["redblack", "march"], default="redblack")
    ap.add_argument("--iters", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--minor", type=int, default=0, help="MSFLOW iterations and a band-model emission update after")
    a = ap.parse_args(argv)
    case = build_case(a.case)
    if a.minor:
        case.c.params.gas_model = 1
    s = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK if a.adi == "redblack" else abi.GFM_ADI_MARCH,
                  precision=abi.GFM_PREC_MIXED if a.prec == "mixed" else abi.GFM_PREC_FP64)
    s.start()
    if a.warmup:
        s.gflow(a.warmup)
    s.reset_kernel_times()
    st, nd = s.gflow(a.iters)
    kt = s.kernel_times()
    prof = s.iteration_profile()
    out = {"case": a.case, "cells": case.ncells, "prec": a.prec, "adi": a.adi, "iterations": nd,
           "ms_per_iteration": kt["gflow_ms"] / max(nd, 1), "line_solver_ms_per_iteration": kt["adi_ms"] / max(nd, 1),
           "kernels_per_iteration": prof["kernels_per_iter"], "res_mass": st["res_mass"]}
    if a.minor:
        import time
        s.initsvm(restart=False)
        t0 = time.perf_counter()
        ms = s.msflow(a.minor)
        # MSFLOW stops early once every residual is below BMCON
        out["msflow_iterations"] = ms["iterations"]
        out["msflow_ms_per_iteration"] = 1e3 * (time.perf_counter() - t0) / max(ms["iterations"], 1)
        out["msflow_resid"] = ms["resid_ms"]
        t0 = time.perf_counter()
        s.rad_emission()
        out["band_model_emission_ms"] = 1e3 * (time.perf_counter() - t0)
    s.close()
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
