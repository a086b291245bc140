"""Benchmark: steady SIMPLER outer iterations of the GFM combustion-space
solver on the 192x96x64 synthetic furnace (1,179,648 cells).

A step is one outer iteration (GFLOW: momentum, pressure, pressure correction,
seven scalar equations, properties, boundary values) over the whole furnace.
`value` is cells x iterations per second with the state resident in HBM (CUDA
events on the solver's stream around the timed iterations); `e2e` is the same
metric through the public C ABI with host buffers: upload of the state from
pinned host memory, one gfm_gpu_gflow call per step returning its statistics,
and the download of the fields at the end, all inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--prec mixed|fp64] [--adi redblack|march]

Multi-GPU runs are independent replicas (the iteration does not shard): every
rank solves its own furnace, `value` sums the replicas over the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-iters/s, steady SIMPLER outer iteration, 192x96x64 furnace"
UNIT = "cell-iter/s"
WORKLOAD = "furnace_192x96x64: GFLOW steady SIMPLER outer iteration, 1,179,648 cells"
BYTES_PER_CELL_VISIT = 10   # 8 coefficients + read x + write x per plane visit (algorithmic)
# whole iteration: sum over the equations of (reads + 8 coefficient writes) of
# the assembly, 20 per sweep (2 x-passes x (8 coefficients + read x + write
# x)) over the 41 sweeps, 15 for the property update (words per cell)
ITER_BYTES_PER_CELL = 182 + 20 * 41 + 15


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, local):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        # the raw samples; GFM_BENCH_OUT names the folder (default bench_out/)
        self.path = pathlib.Path(os.environ.get("GFM_BENCH_OUT", str(ROOT / "bench_out"))) / f"clocks_bench_{gpu}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit()) if rows else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def load_traffic(prec: str):
    """DRAM traffic of one colour visit of the line solver (one plane-visit
    launch) from the committed ncu summary of the same workload."""
    p = ROOT / "profiles" / f"ncu_adi_{prec}_192x96x64.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


def cpu_baseline_oracle(steps: int = 1, adi_mode=None):
    """The CPU oracle (FP64 restatement of the reference, 1 core) on the same
    case, in the reference's plane order unless `adi_mode` says otherwise;
    returns its rate, its time and its fields after `steps` iterations."""
    from gfm_gb300 import Case, configs
    from oracle.pyoracle import Oracle
    case = Case(configs.large_furnace())
    o = Oracle(case, adi_mode=adi_mode)
    o.initsv()
    t0 = time.perf_counter()
    o.gflow(steps)
    dt = time.perf_counter() - t0
    fields = o.download()
    o.close()
    return case.ncells * steps / dt, dt, fields


FIELD_ERRORS = (("u", "ug", 0), ("v", "ug", 1), ("w", "ug", 2), ("p", "p", None), ("T", "t", None),
                ("k", "gf", 3), ("eps", "gf", 4))


def field_errors(case, got, ref) -> dict:
    """Max and L2 error of each reported field relative to the reference's max
    and L2 norm, over the open positions (IBCELL <= 0)."""
    import numpy as np
    open_ = case.ibcell() <= 0
    out = {}
    for name, key, comp in FIELD_ERRORS:
        a = got.arrays[key] if comp is None else got.arrays[key][comp]
        b = ref.arrays[key] if comp is None else ref.arrays[key][comp]
        a, b = a[open_], b[open_]
        d = np.abs(a - b)
        out[name] = {"max": float(d.max() / max(np.abs(b).max(), 1e-300)),
                     "l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}
    return out


def time_to_residual(case, adi, prec, thresh: float, max_iter: int, lp=None, fields_out: list | None = None) -> dict:
    """Iterations and device time from the fresh start until res_mass < thresh,
    with the solver's own convergence test (BGCON = thresh); with `lp`, every
    p' solve starts from the learned guess.  The fields where the run stopped
    are appended to `fields_out` when given."""
    from gfm_gb300 import GpuSolver
    s = GpuSolver(case, adi_mode=adi, precision=prec, bgcon=thresh)
    s.start()
    if lp is not None:
        s.set_lp(lp)
    s.reset_kernel_times()
    st, nd = s.gflow(max_iter)
    ms = s.kernel_times()["gflow_ms"]
    if fields_out is not None:
        fields_out.append(s.download())
    s.close()
    out = {"threshold": thresh, "reached": bool(st["converged"]), "iterations": nd, "seconds": ms / 1e3,
           "ms_per_iteration": ms / max(nd, 1), "res_mass_last": st["res_mass"], "pcorr_resid_last": st["pcorr_resid"]}
    if lp is not None:
        out["lp_used_last"] = st["lp_used"]
        out["lp_ratio_last"] = st["lp_ratio"]
    return out


TTR_THRESHOLD = 1.0e-3
TTR_SEEDS = (20261203, 11, 12, 13)
TTR_REASON = ("res_mass <= 1e-5 is not reached by the method on these cases: the mass residual plateaus near 1e-3 "
              "with the exit factor oscillating, as the reference's own logs plateau (convg0041c.plt ends at "
              "1.3e-4); the time to the plateau threshold 1e-3 is reported")
TTR_NOTE = ("the iteration is chaotic at the plateau: a run can settle instead with the exit factor held at its "
            "0.8 bound and res_mass near 1.4e-3, whatever the arithmetic (seen in FP64 and in both forms of the "
            "mixed line solver); so the time is taken on four seeded furnaces (inlet-velocity jitter and initial "
            "noise from the seed) and the median over the runs that reached the threshold is reported with the "
            "count")


CEILING_SWEEPS = 20
CEILING_NOTE = ("not the case's schedule: the pressure (ntimesg 4) and p' (ntimesg 5) line-solver sweeps are raised "
                "from 6 and 5 to 20, which leaves the p' equation nearly solved each outer iteration; the outer "
                "iterations this run needs are the floor that a learned or otherwise better p' start could reach")


CONVERGED_FIELD_NOTE = ("with the pressure solves converged the iteration is no longer chaotic: the mixed and FP64 "
                        "runs of a seed stop at the same iteration, and field_error_vs_fp64 compares their fields "
                        "there (at res_mass 1e-3, not a converged state: the residual still oscillates as it "
                        "decays)")


def _median(v):
    v = sorted(v)
    return None if not v else (v[len(v) // 2] if len(v) % 2 else 0.5 * (v[len(v) // 2 - 1] + v[len(v) // 2]))


def time_to_residual_leg(case, adi, args) -> tuple:
    """Time from the fresh start to res_mass < 1e-3 for the plain FP64 path,
    the mixed path and the mixed path with the learned p' guess (trained here
    on seeded variants of the 48x24x16 furnace), on four seeded 192x96x64
    furnaces; each run carries the error of every reported field where it
    stopped against the plain FP64 path's run of the same seed (the FP64
    oracle's arithmetic, checked against it at 1e-9 per iteration).  The
    converged-pressure runs (pressure and p' sweeps raised to CEILING_SWEEPS)
    do the same for both precisions."""
    from gfm_gb300 import Case, abi, configs
    thr = args.ttr or TTR_THRESHOLD
    lp = None
    learned = None
    if not args.no_learned:
        from gfm_gb300.lp import train_default
        t0 = time.perf_counter()
        log = []
        lp = train_default((case.mp // 2 - 2, case.np // 2 - 2, case.lp // 2 - 2), log=log, steps=args.lp_steps)
        learned = {"threshold": thr, "train_seconds": time.perf_counter() - t0, "training": log, "runs": []}
    runs = {"fp64": [], "mixed": []}
    for seed in TTR_SEEDS:
        c = Case(configs.large_furnace(seed=seed))
        f64, fmix = [], []
        r64 = time_to_residual(c, adi, abi.GFM_PREC_FP64, thr, args.ttr_max, fields_out=f64)
        rmx = time_to_residual(c, adi, abi.GFM_PREC_MIXED, thr, args.ttr_max, fields_out=fmix)
        rmx["field_error_vs_fp64"] = field_errors(c, fmix[0], f64[0])
        for r in (r64, rmx):
            r["seed"] = seed
        runs["fp64"].append(r64)
        runs["mixed"].append(rmx)
        if lp is not None:
            flp = []
            rlp = time_to_residual(c, adi, abi.GFM_PREC_MIXED, thr, args.ttr_max, lp=lp, fields_out=flp)
            rlp["field_error_vs_fp64"] = field_errors(c, flp[0], f64[0])
            rlp["seed"] = seed
            learned["runs"].append(rlp)
    if lp is not None:
        lp.close()

    def summary(rs):
        ok = [r for r in rs if r["reached"]]
        return {"reached": f"{len(ok)} of {len(rs)}", "median_seconds": _median([r["seconds"] for r in ok]),
                "median_iterations": _median([r["iterations"] for r in ok])}

    ttr = {"threshold": thr, "why_not_1e-5": TTR_REASON, "seeds": list(TTR_SEEDS), "note": TTR_NOTE,
           "max_iterations": args.ttr_max, "fp64": summary(runs["fp64"]), "mixed": summary(runs["mixed"]),
           "runs": runs}
    if not args.no_ceiling:
        # Pressure and p' line-solver sweeps raised from the case's 6 and 5
        # to CEILING_SWEEPS: the outer iterations an (almost) exact pressure
        # solve leaves, the most any better p' start can save.
        v = list(configs.REFERENCE_SWEEPS)
        v[3] = v[4] = CEILING_SWEEPS
        cr, cr64 = [], []
        for seed in TTR_SEEDS:
            c = Case(configs.large_furnace(seed=seed, ntimesg=tuple(v)))
            f64, fmix = [], []
            r64 = time_to_residual(c, adi, abi.GFM_PREC_FP64, thr, args.ttr_max, fields_out=f64)
            r = time_to_residual(c, adi, abi.GFM_PREC_MIXED, thr, args.ttr_max, fields_out=fmix)
            if r["iterations"] == r64["iterations"]:
                r["field_error_vs_fp64"] = field_errors(c, fmix[0], f64[0])
            r["seed"] = r64["seed"] = seed
            cr.append(r)
            cr64.append(r64)
        cp = {"sweeps_p": CEILING_SWEEPS, "sweeps_pprime": CEILING_SWEEPS, "note": CEILING_NOTE,
              "field_note": CONVERGED_FIELD_NOTE, "mixed": summary(cr), "fp64": summary(cr64),
              "runs": cr, "runs_fp64": cr64}
        if cp["fp64"]["median_seconds"] and cp["mixed"]["median_seconds"]:
            cp["mixed_vs_fp64_speedup"] = cp["fp64"]["median_seconds"] / cp["mixed"]["median_seconds"]
        ttr["converged_pressure"] = cp
    if ttr["fp64"]["median_seconds"] and ttr["mixed"]["median_seconds"]:
        ttr["mixed_vs_fp64_speedup"] = ttr["fp64"]["median_seconds"] / ttr["mixed"]["median_seconds"]
    if learned is not None:
        learned["learned"] = summary(learned["runs"])
        learned["plain_mixed"] = ttr["mixed"]
        lm = learned["learned"]["median_seconds"]
        if lm:
            if ttr["mixed"]["median_seconds"]:
                learned["speedup_vs_plain_mixed"] = ttr["mixed"]["median_seconds"] / lm
            if ttr["fp64"]["median_seconds"]:
                learned["speedup_vs_fp64"] = ttr["fp64"]["median_seconds"] / lm
    return ttr, learned


def batched_leg(args, steps: int) -> dict:
    """The batched workload (64 seeded furnace variants) with every
    iteration queued on all variants' streams before any is waited for
    (gfm_gpu_gflow_batch), aggregate cells x iterations per second, next to
    the same variants one after another."""
    import torch
    from gfm_gb300 import Case, GpuSolver, abi, configs
    from gfm_gb300.solver import gflow_batch
    prec = abi.GFM_PREC_MIXED if args.prec == "mixed" else abi.GFM_PREC_FP64
    adi = abi.GFM_ADI_REDBLACK if args.adi == "redblack" else abi.GFM_ADI_MARCH
    ss = []
    for cfg in configs.batch_variants(args.batch):
        s = GpuSolver(Case(cfg), adi_mode=adi, precision=prec)
        s.start()
        ss.append(s)
    cells = sum(s.case.ncells for s in ss)
    gflow_batch(ss, 3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, nd = gflow_batch(ss, steps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    batched = sum(s.case.ncells * n for s, n in zip(ss, nd)) / (t1 - t0)
    t2 = time.perf_counter()
    nd_seq = [s.gflow(steps)[1] for s in ss]
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    seq = sum(s.case.ncells * n for s, n in zip(ss, nd_seq)) / (t3 - t2)
    launches = int(sum(s.iteration_profile()["kernels_per_iter"] for s in ss) * steps)
    for s in ss:
        s.close()
    return {"metric": f"cell-iters/s, {len(ss)} batched furnace variants", "value": batched, "unit": UNIT,
            "steps": steps, "ms_per_step": 1e3 * (t1 - t0) / steps,
            "workload": f"{len(ss)} seeded furnace variants, {cells} cells in total",
            "timing": "host wall clock around the batched call, device synchronised, after 3 warm-up iterations",
            "sequential": {"value": seq, "ms_per_step": 1e3 * (t3 - t2) / steps,
                           "note": "the same variants, one gfm_gpu_gflow call after another"},
            "gpu_launches": launches}


def _replica_worker(args):
    steps, warmup = args
    from gfm_gb300 import configs
    from oracle.pyoracle import Oracle, OracleCase
    # the oracle's own start-up: this process loads no part of the product
    case = OracleCase(configs.large_furnace())
    o = Oracle(case)
    o.initsv()
    if warmup:
        o.gflow(warmup)
    t0 = time.perf_counter()
    o.gflow(steps)
    return time.perf_counter() - t0, case.ncells


def run_reference(args):
    """Reference arm: the CPU oracle (FP64, the reference's serial algorithm)
    on the machine's host cores, one independent furnace per core."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import multiprocessing as mp
    ncpu = os.cpu_count() or 1
    mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    cores = max(1, min(ncpu, int(mem // (6 * 2 ** 30))))
    # the same K timed outer iterations as the GPU arm, after one untimed
    # one (an iteration of this furnace takes 16-22 s on one host core)
    steps = max(1, args.steps)
    warm = max(0, min(args.warmup, 1))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_replica_worker, [(steps, warm)] * cores)
    wall = time.perf_counter() - t0
    worst = max(r[0] for r in res)
    ncells = res[0][1]
    value = cores * ncells * steps / worst
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": 1e3 * worst / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": ncells, "replicas": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} independent replicas x {steps} outer iteration(s) of the FP64 oracle "
                                   f"(C++ restatement of the Fortran GFLOW, its own start-up of the furnace; no "
                                   f"part of the product loaded) after {warm} untimed, wall {wall:.1f}s"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pinned_fields(case):
    """Fresh-start fields in pinned host memory when torch+CUDA are present."""
    f = case.initial_fields()
    try:
        import torch
        if torch.cuda.is_available():
            for k, v in list(f.arrays.items()):
                # the numpy view keeps the pinned tensor alive
                a = torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
                a[...] = v
                f.arrays[k] = a
            f._pinned = True
    except Exception:
        f._pinned = False
    return f


def run_ours(args):
    rank, world, local = dist_env()
    dist = init_dist(world, local)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    from gfm_gb300 import Case, GpuSolver, abi, configs
    prec = abi.GFM_PREC_MIXED if args.prec == "mixed" else abi.GFM_PREC_FP64
    adi = abi.GFM_ADI_REDBLACK if args.adi == "redblack" else abi.GFM_ADI_MARCH
    if world > 1:
        import torch
        torch.cuda.set_device(local)
    case = Case({"large": configs.large_furnace, "medium": configs.medium_furnace, "xl": configs.xl_furnace}[args.case]())
    solver = GpuSolver(case, adi_mode=adi, precision=prec)
    solver.start()
    solver.gflow(max(args.warmup, 0))
    prof = solver.iteration_profile()
    solver.reset_kernel_times()
    barrier(dist)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        st, nd = solver.gflow(args.steps)
        t1 = time.perf_counter()
    barrier(dist)
    kt = solver.kernel_times()
    dev_s = kt["gflow_ms"] / 1e3
    dev_s = max_over_ranks(dist, dev_s)
    ncells = case.ncells
    value = world * ncells * nd / dev_s
    w = 4 if args.prec == "mixed" else 8
    # dominant kernel: the line solver (ADLBL3 plane updates)
    adi_launches = prof["adi_kernels_per_iter"] * nd
    adi_ms = kt["adi_ms"]
    achieved = (prof["adi_cell_visits_per_iter"] * nd * BYTES_PER_CELL_VISIT * w / 1e9) / (adi_ms / 1e3) if adi_ms > 0 else None
    peak, peak_kind = measured_peaks()
    traffic = load_traffic(args.prec)

    # e2e through the public API with host buffers (pinned when available)
    fields = pinned_fields(case)
    solver2 = GpuSolver(case, adi_mode=adi, precision=prec)
    solver2.upload(fields)
    solver2.initsv()
    solver2.gflow(max(args.warmup, 0))
    state = solver2.download()
    host_state = pinned_fields(case)            # the step's inputs, in pinned host memory
    for k, v in state.arrays.items():
        host_state.arrays[k][...] = v
    for a in ("itr_gas", "do_rad_qe_only_cnt", "i1st_rad_qe_done", "factor", "fadj", "gfin0", "q_h_in"):
        setattr(host_state, a, getattr(state, a))
    out = pinned_fields(case)
    import ctypes as C
    barrier(dist)
    e0 = time.perf_counter()
    solver2.upload(host_state)
    for _ in range(args.steps):
        solver2.gflow(1)
    f = out.to_c()
    solver2._check(solver2.lib.gfm_gpu_download(solver2.h, C.byref(f)))
    e1 = time.perf_counter()
    barrier(dist)
    e2e_s = max_over_ranks(dist, e1 - e0)
    n = case.mp * case.np * case.lp
    nfield = 9 + 3 + 8
    state_bytes = 8 * (nfield * n + 2 * (case.mp // 2) * (case.np // 2) * (case.lp // 2))
    stats_bytes = C.sizeof(abi.GfmIterStats) + 8 * 200
    h2d = state_bytes / args.steps + 16
    d2h = state_bytes / args.steps + stats_bytes
    e2e_value = world * ncells * args.steps / e2e_s
    solver2.close()

    plain = None
    if args.prec == "mixed" and not args.no_plain:
        s64 = GpuSolver(case, adi_mode=adi, precision=abi.GFM_PREC_FP64)
        s64.start()
        s64.gflow(max(args.warmup, 0))
        s64.reset_kernel_times()
        _, n64 = s64.gflow(args.steps)
        t64 = s64.kernel_times()["gflow_ms"] / 1e3
        v64 = ncells * n64 / t64
        plain = {"value": v64, "ms_per_step": 1e3 * t64 / n64, "dtype": "fp64",
                 "roofline_iteration": {
                     "bound": "hbm (whole iteration); the FP64 pipe binds first on GB300",
                     "achieved": v64 * ITER_BYTES_PER_CELL * 8 / 1e9,
                     "peak": measured_peaks()[0], "unit": "GB/s",
                     "frac": v64 * ITER_BYTES_PER_CELL * 8 / 1e9 / measured_peaks()[0],
                     "algorithmic_bytes": f"{ITER_BYTES_PER_CELL} x 8 B per cell per iteration"}}
        s64.close()

    cpu = None
    ferr = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, dt, fo = cpu_baseline_oracle(1)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"1 outer iteration of the FP64 oracle (C++ restatement of GFLOW) on the same "
                             f"192x96x64 furnace after INITSV, {dt:.1f}s on one host core"}
            # the GPU path from the same start, one iteration: error of every
            # reported field against the FP64 oracle run in the same plane
            # order, for the benchmarked order and the reference's march
            ferr = {"after_iterations": 1,
                    "reference": "FP64 oracle in the same plane order (the red-black oracle visits the planes "
                                 "colour by colour with the reference's ADLZ)"}
            orders = [(args.adi, adi)] + ([("march", abi.GFM_ADI_MARCH)] if args.adi != "march" else [])
            for name, mode in orders:
                ref_f = fo if mode == abi.GFM_ADI_MARCH else cpu_baseline_oracle(1, adi_mode=mode)[2]
                s1 = GpuSolver(case, adi_mode=mode, precision=prec)
                s1.start()
                s1.gflow(1)
                ferr[name] = field_errors(case, s1.download(), ref_f)
                s1.close()
        except Exception as e:   # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}

    ttr = None
    learned = None
    if rank == 0 and not args.no_ttr:
        ttr, learned = time_to_residual_leg(case, adi, args)

    rad = None
    if rank == 0 and not args.no_rad:
        try:
            rad = rad_transfer_leg(not args.no_cpu_baseline)
        except Exception as e:   # reported, never required
            rad = {"failed": str(e)}

    tc21 = None
    if rank == 0 and not args.no_tc21:
        try:
            tc21 = tc21_leg(not args.no_cpu_baseline)
        except Exception as e:   # reported, never required
            tc21 = {"failed": str(e)}

    wall = None
    if rank == 0 and not args.no_wall:
        try:
            wall = wall_exchange_leg(not args.no_cpu_baseline)
        except Exception as e:   # reported, never required
            wall = {"failed": str(e)}

    minor = None
    if rank == 0 and not args.no_minor:
        try:
            minor = minor_species_leg(args, not args.no_cpu_baseline)
        except Exception as e:   # reported, never required
            minor = {"failed": str(e)}

    batched = None
    if rank == 0 and not args.no_batched:
        try:
            batched = batched_leg(args, steps=min(args.steps, 5))
        except Exception as e:   # reported, never required
            batched = {"failed": str(e)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / nd, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32" if args.prec == "mixed" else "fp64", "data": "synthetic",
            "config": {"workload": WORKLOAD if args.case == "large" else (
                           f"{case.cfg.name}: GFLOW steady SIMPLER outer iteration, {ncells:,} cells, "
                           + ("10 gray bands; the combustion space of the large coupled configuration, no melt coupling"
                              if args.case == "xl" else "kernel-capture case, not the benchmark workload")),
                       "cells": ncells, "precision": args.prec, "adi_order": args.adi,
                       "l2": "inputs larger than L2 (device state ~%.1f GB)" % (state_bytes * (0.5 if w == 4 else 1) * 3 / 1e9),
                       "parallelism": f"replicas x{world}", "res_mass_last": st["res_mass"]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "pinned": bool(getattr(fields, "_pinned", False)),
                    "path": "gfm_gpu_upload + K x gfm_gpu_gflow(1) + gfm_gpu_download",
                    "transfers": "one upload of the whole state before the K steps and one download after them, "
                                 "inside the timed region; the bytes per step are that state's size divided by K, "
                                 "plus each step's statistics read back"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None,
                         "traffic": traffic.get("dram_bytes_per_colour_visit") if traffic else None,
                         "traffic_unit": "DRAM bytes per colour visit (one launch) of the 192x96x64 P equation, ncu",
                         "traffic_algorithmic": traffic.get("algorithmic_bytes_per_colour_visit") if traffic else None,
                         "peak_kind": peak_kind, "kernel": "ADLBL3 line solver (plane updates)",
                         "algorithmic_bytes": f"{BYTES_PER_CELL_VISIT} x {w} B per cell per plane visit",
                         "adi_launches": adi_launches, "adi_ms": adi_ms},
            "roofline_iteration": {"bound": "hbm", "achieved": value / world * ITER_BYTES_PER_CELL * w / 1e9,
                                   "peak": peak, "unit": "GB/s",
                                   "frac": value / world * ITER_BYTES_PER_CELL * w / 1e9 / peak,
                                   "algorithmic_bytes": f"{ITER_BYTES_PER_CELL} x {w} B per cell per iteration"},
            "cpu_baseline": cpu,
            "field_error": ferr,
            "batched": batched,
            "time_to_residual": ttr,
            "learned_p_prime": learned,
            "rad_transfer": rad,
            "tc21_case0041": tc21,
            "wall_exchange": wall,
            "minor_species": minor,
            "clocks": clk.summary(),
            "gpu_launches": int(prof["kernels_per_iter"] * nd),
            "plain_fp64": plain,
            "wall_s": t1 - t0,
        }
        print(json.dumps(line), flush=True)
    solver.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def tc21_leg(with_cpu: bool, iters: int = 200) -> dict:
    """The reference's own TC21 case 0041 (40x48x36 doubled grid, 4,407 open
    cells), read from its case files (tests/golden/case0041): seconds per
    outer iteration on the GPU in the reference's plane order (FP64) and in the
    fast form (mixed precision, red-black), device time over `iters`
    iterations after 20 warm-up iterations, and in FP64 with the red-black
    order, next to the FP64 oracle on one host core.  A grid this small is
    bound by launch latency, not HBM."""
    import pathlib
    import shutil
    import tempfile
    from gfm_gb300 import Case, GpuSolver, abi
    gold = pathlib.Path(__file__).resolve().parent / "tests" / "golden" / "case0041"
    with tempfile.TemporaryDirectory() as d:
        for n in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat", "relaxfactorc.txt"):
            shutil.copyfile(gold / n, pathlib.Path(d) / n)
        case = Case.from_files(d, "0041")
    out = {"workload": f"TC21 case 0041 from its case files, {case.ncells:,} open cells, fresh start",
           "timing": f"device time of {iters} iterations after 20 warm-up iterations"}
    for name, adi, prec in (("fp64_march", abi.GFM_ADI_MARCH, abi.GFM_PREC_FP64),
                            ("fp64_redblack", abi.GFM_ADI_REDBLACK, abi.GFM_PREC_FP64),
                            ("mixed_redblack", abi.GFM_ADI_REDBLACK, abi.GFM_PREC_MIXED)):
        g = GpuSolver(case, adi_mode=adi, precision=prec)
        g.start()
        g.gflow(20)
        g.reset_kernel_times()
        st, nd = g.gflow(iters)
        ms = g.kernel_times()["gflow_ms"] / nd
        out[name] = {"ms_per_iteration": ms, "res_mass_last": st["res_mass"], "iterations": nd}
        g.close()
    # the volume radiation transfer on this geometry (ports, flue, stepped
    # crown), gray kappa 0.5 1/m in its 10 bands, state after 3 FP64 iterations
    with tempfile.TemporaryDirectory() as d:
        for n in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat", "relaxfactorc.txt"):
            shutil.copyfile(gold / n, pathlib.Path(d) / n)
        rcase = Case.from_files(d, "0041", kappa=[0.5] * 16)
    from oracle.pyoracle import Oracle
    o = Oracle(rcase)
    o.initsv()
    o.gflow(3)
    state = o.download()
    g = GpuSolver(rcase, precision=abi.GFM_PREC_FP64)
    g.upload(state)
    g.rad_transfer()
    ts = []
    for _ in range(3):
        g.upload(state)
        t0 = time.perf_counter()
        tot = g.rad_transfer()
        ts.append(time.perf_counter() - t0)
    g.close()
    out["rad_transfer"] = {"emitters": tot["n_emitters"], "bands": rcase.grid.nwl, "seconds": sorted(ts)[1],
                           "timing": "host wall clock around the synchronous call (median of 3)"}
    if with_cpu:
        t0 = time.perf_counter()
        o.rad_transfer()
        out["rad_transfer"]["cpu_oracle_seconds"] = time.perf_counter() - t0
        out["rad_transfer"]["vs_cpu_oracle"] = out["rad_transfer"]["cpu_oracle_seconds"] / out["rad_transfer"]["seconds"]
    o.close()
    if with_cpu:
        o = Oracle(case)
        o.initsv()
        o.gflow(20)
        t0 = time.perf_counter()
        o.gflow(20)
        out["cpu_oracle_ms_per_iteration"] = (time.perf_counter() - t0) / 20 * 1e3
        o.close()
        for name in ("fp64_march", "fp64_redblack", "mixed_redblack"):
            out[name]["vs_cpu_oracle"] = out["cpu_oracle_ms_per_iteration"] / out[name]["ms_per_iteration"]
    return out


def rad_transfer_leg(with_cpu: bool) -> dict:
    """Volume radiation transfer (RAD0 + the QRNF emitter loop with QREF and
    QRTX/QRTY/QRTZ, Qrn.f90:58-229) of the 48x24x16 furnace from the state
    after 30 FP64 iterations: the whole call timed on the host around the
    synchronous gfm_gpu_rad_transfer, next to the FP64 oracle on one host core
    from the same state, and the largest per-cell difference of QA and QE."""
    import numpy as np
    from gfm_gb300 import Case, GpuSolver, abi, configs
    case = Case(configs.small_furnace())
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    g.start()
    g.gflow(30)
    state = g.download()
    g.rad_transfer()   # first call: buffers, kernel attributes
    times = []
    for _ in range(3):
        g.upload(state)
        t0 = time.perf_counter()
        tot = g.rad_transfer()
        times.append(time.perf_counter() - t0)
    fg = g.download()
    g.close()
    gpu_s = sorted(times)[len(times) // 2]
    out = {"workload": "volume radiation transfer, furnace_48x24x16 (18,432 cells), "
                       f"{case.grid.nwl} gray bands, state after 30 FP64 iterations",
           "emitters": tot["n_emitters"], "seconds": gpu_s, "seconds_all": times,
           "emitters_per_s": tot["n_emitters"] / gpu_s,
           "timing": "host wall clock around the synchronous call (median of 3)",
           "energy_balance": (tot["qe_sum_from_open"] - sum(tot[k] for k in (
               "qa_sum_to_open", "qa_sum_to_wall", "qa_sum_to_inlet", "qa_sum_to_exit", "qa_sum_to_melt")))
           / tot["qe_sum_from_open"],
           "totals": tot}
    if with_cpu:
        from oracle.pyoracle import Oracle
        o = Oracle(case, state)
        t0 = time.perf_counter()
        o.rad_transfer()
        cpu_s = time.perf_counter() - t0
        fo = o.download()
        o.close()
        qa_g, qa_o = fg.arrays["qa"], fo.arrays["qa"]
        sel = qa_o > 1e-9 * qa_o.max()
        qe_o = fo.arrays["qe"]
        hot = qe_o > 0
        out["cpu_baseline"] = {"seconds": cpu_s, "cores": 1, "kind": "port",
                               "sample": "the whole transfer of the same state, FP64 oracle on one host core"}
        out["speedup_vs_cpu"] = cpu_s / gpu_s
        out["max_rel_err"] = {"qa": float(np.max(np.abs(qa_g[sel] - qa_o[sel]) / qa_o[sel])),
                              "qe": float(np.max(np.abs(fg.arrays["qe"][hot] - qe_o[hot]) / qe_o[hot]))}
    return out


def _converged_case0041(d: pathlib.Path, **kw):
    """TC21 case 0041 read from its files with the end-of-run restarts of its
    reference run (rg0041c.d, rs0041c.d), and that run's minor species."""
    import lzma
    import shutil
    from gfm_gb300 import Case
    gold = pathlib.Path(__file__).resolve().parent / "tests" / "golden" / "case0041"
    for n in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat", "relaxfactorc.txt"):
        shutil.copyfile(gold / n, d / n)
    for k in ("rg", "rs"):
        (d / f"{k}0041c.d").write_bytes(lzma.decompress((gold / f"{k}0041c.d.xz").read_bytes()))
    case = Case.from_files(d, "0041", restart=True, gas_model=True, **kw)
    ref = json.loads((gold / "case0041_reference.json").read_text())["rad_detail_last"]
    return case, case.read_minor(d / "rs0041c.d"), ref


def minor_species_leg(args, with_cpu: bool) -> dict:
    """The band model and the minor species (gas.cu, minor.cu).  On TC21 case
    0041 from its reference run's end-of-run restarts (FP64): the volume
    transfer on the band model (RAD_GAS and SOOTA in RAD0) with its error
    against that run's own radiation record, and MSFLOW(300) after one gas
    iteration; next to the oracle on one host core (the transfer, and 30
    MSFLOW iterations scaled to 300).  On the 192x96x64 furnace (mixed, red-
    black, from INITSVM's new start after 3 iterations): one MSFLOW iteration
    and one emission update with the band model against the gray one."""
    import tempfile
    import numpy as np
    from gfm_gb300 import Case, GpuSolver, abi, configs
    from oracle.pyoracle import Oracle
    keys = (("tot_qe_h2o_co2", "qe_h2o_co2"), ("tot_qe_soot", "qe_soot"), ("qe_sum_from_open", "qe_from_media"),
            ("qa_sum_to_melt", "qa_melt"), ("qa_sum_to_wall", "qa_wall"), ("qa_sum_to_open", "qa_media"))
    out = {}
    with tempfile.TemporaryDirectory() as dd:
        case, minor, ref = _converged_case0041(pathlib.Path(dd))
        g = GpuSolver(case, precision=abi.GFM_PREC_FP64, adi_mode=abi.GFM_ADI_REDBLACK)
        g.start()
        g.minor_upload(minor)
        g.rad_transfer()   # first call: buffers, launch plan
        ts = []
        for _ in range(3):
            g.start()
            t0 = time.perf_counter()
            tot = g.rad_transfer()
            ts.append(time.perf_counter() - t0)
        err = max(abs(tot[a] / ref[b] - 1.0) for a, b in keys)
        g.start()
        g.gflow(1)
        g.initsvm(restart=True)
        t0 = time.perf_counter()
        st = g.msflow(300)
        t_ms = time.perf_counter() - t0
        g.close()
        out["tc21"] = {"workload": f"TC21 case 0041 ({case.ncells:,} open cells, 10 bands) from its reference run's "
                                   "end-of-run restarts, FP64, red-black order",
                       "transfer_seconds": sorted(ts)[1],
                       "transfer_max_rel_error_vs_reference_record": err,
                       "msflow_300_seconds": t_ms, "msflow_resid": st["resid_ms"],
                       "timing": "host wall clock around the synchronous calls (transfer: median of 3)"}
        if with_cpu:
            o = Oracle(case)
            o.initsv()
            o.minor_set(minor)
            t0 = time.perf_counter()
            o.rad_transfer()
            t_o = time.perf_counter() - t0
            o2 = Oracle(case)
            o2.initsv()
            o2.gflow(1)
            o2.minor_set(minor)
            o2.initsvm(restart=True)
            t0 = time.perf_counter()
            o2.msflow(30)
            t_o_ms = (time.perf_counter() - t0) * 10.0
            out["tc21"]["cpu_baseline"] = {"transfer_seconds": t_o, "msflow_300_seconds": t_o_ms, "cores": 1,
                                           "kind": "port", "sample": "the oracle's transfer; 30 MSFLOW iterations "
                                                                     "scaled to 300"}
            out["tc21"]["transfer_speedup"] = t_o / out["tc21"]["transfer_seconds"]
            out["tc21"]["msflow_speedup"] = t_o_ms / t_ms
            o.close()
            o2.close()
    # the 192x96x64 furnace
    prec = abi.GFM_PREC_MIXED if args.prec == "mixed" else abi.GFM_PREC_FP64
    case = Case(configs.large_furnace())
    case.c.params.gas_model = 1
    g = GpuSolver(case, precision=prec, adi_mode=abi.GFM_ADI_REDBLACK)
    g.start()
    g.gflow(3)
    g.initsvm(restart=False)
    g.msflow(3)
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = g.msflow(20)
    t_it = (time.perf_counter() - t0) / max(st["iterations"], 1)   # it may stop early, below BMCON
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        g.rad_emission()
        ts.append(time.perf_counter() - t0)
    t_band = sorted(ts)[1]
    g.close()
    case.c.params.gas_model = 0
    g = GpuSolver(case, precision=prec, adi_mode=abi.GFM_ADI_REDBLACK)
    g.start()
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        g.rad_emission()
        ts.append(time.perf_counter() - t0)
    t_gray = sorted(ts)[1]
    g.close()
    case.close()
    out["furnace_192x96x64"] = {"precision": args.prec, "msflow_ms_per_iteration": 1e3 * t_it,
                                "msflow_iterations": st["iterations"],
                                "emission_band_model_ms": 1e3 * t_band, "emission_gray_ms": 1e3 * t_gray,
                                "timing": "host wall clock around synchronous calls (MSFLOW: 20 iterations after 3; "
                                          "emission: median of 3)"}
    return out


def wall_exchange_leg(with_cpu: bool) -> dict:
    """The wall radiosity exchange (wall_q_amb and wallq after the volume
    transfer, Qwall.f90:990-1245) on TC21 case 0041 read from its files, gray
    kappa 0.5 1/m in its 10 bands, the wall sink on, from the state after 3
    FP64 iterations of the oracle: gfm_gpu_rad_transfer with the exchange set
    up, against the same call without it (the exchange's share is the
    difference of the medians), next to the oracle's Gauss-Seidel restatement
    on one host core, with the largest patch-temperature difference."""
    import numpy as np
    import shutil
    import tempfile
    from gfm_gb300 import Case, GpuSolver, abi
    from oracle.pyoracle import Oracle
    gold = pathlib.Path(__file__).resolve().parent / "tests" / "golden" / "case0041"
    with tempfile.TemporaryDirectory() as d:
        for n in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat", "relaxfactorc.txt"):
            shutil.copyfile(gold / n, pathlib.Path(d) / n)
        case = Case.from_files(d, "0041", kappa=[0.5] * 16, wall_sink=True)
    o = Oracle(case)
    o.initsv()
    o.gflow(3)
    state = o.download()

    def timed(with_wall: bool):
        g = GpuSolver(case, precision=abi.GFM_PREC_FP64)
        g.upload(state)
        g.rad_transfer()   # first call: buffers, kernel attributes
        setup = None
        if with_wall:
            t0 = time.perf_counter()
            g.wall_setup()
            setup = time.perf_counter() - t0
        ts, tot = [], None
        for _ in range(3):
            g.close()
            g = GpuSolver(case, precision=abi.GFM_PREC_FP64)
            g.upload(state)
            g.rad_transfer()
            if with_wall:
                g.wall_setup()
            g.upload(state)
            t0 = time.perf_counter()
            g.rad_transfer()
            ts.append(time.perf_counter() - t0)
            if with_wall:
                tot = g.wall_totals()
                bt = g.wall_array("b_t")
        g.close()
        return sorted(ts)[1], setup, (tot, bt) if with_wall else None

    t_rad, _, _ = timed(False)
    t_all, t_setup, (tot, bt) = timed(True)
    nb = tot["b_cnt"]
    out = {"workload": f"wall radiosity exchange, TC21 case 0041 ({nb:,} boundary patches, {case.ncells:,} open "
                       "cells), gray kappa 0.5 1/m in 10 bands, the wall sink on, state after 3 FP64 iterations",
           "patches": nb, "sweeps": tot["sweeps"], "outer_passes": tot["outer"],
           "seconds": t_all - t_rad, "seconds_with_volume_transfer": t_all, "setup_seconds": t_setup,
           "view_factor_bytes": nb * nb * 8,
           "timing": "host wall clock around the synchronous gfm_gpu_rad_transfer with the exchange set up, "
                     "less the same call without it (medians of 3)",
           "avg_wall_T": tot["avg_wall_T"], "q_melt": tot["q_melt"]}
    if with_cpu:
        o.wall_setup()
        t0 = time.perf_counter()
        o.rad_transfer()
        t_o = time.perf_counter() - t0
        o2 = Oracle(case, fields=state)
        t0 = time.perf_counter()
        o2.rad_transfer()
        t_o_rad = time.perf_counter() - t0
        o2.close()
        to = o.wall_totals()
        bt_o = o.patch_array("b_t")
        out["cpu_baseline"] = {"seconds": t_o - t_o_rad, "cores": 1, "kind": "port",
                               "sample": "the oracle's Gauss-Seidel exchange from the same state (its whole "
                                         "radiation call less its volume transfer alone)",
                               "sweeps": to["sweeps"], "avg_wall_T": to["avg_wall_T"], "q_melt": to["q_melt"]}
        out["max_rel_err_b_T"] = float(np.max(np.abs(bt - bt_o) / bt_o))
        out["vs_cpu_oracle"] = out["cpu_baseline"]["seconds"] / out["seconds"]
    o.close()
    return out


def run_batched(args):
    """The batched workload alone (`--batched`): its own JSON line."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    with ClockSampler(local) as clk:
        leg = batched_leg(args, args.steps)
    line = {"metric": leg["metric"], "value": leg["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": leg["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32" if args.prec == "mixed" else "fp64", "data": "synthetic",
            "config": {"workload": leg["workload"], "precision": args.prec, "adi_order": args.adi,
                       "timing": leg["timing"]},
            "sequential": leg["sequential"], "clocks": clk.summary(), "gpu_launches": leg["gpu_launches"]}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--prec", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--adi", choices=["redblack", "march"], default="redblack")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-rad", action="store_true", help="skip the volume radiation transfer leg")
    ap.add_argument("--no-tc21", action="store_true", help="skip the TC21 case 0041 leg")
    ap.add_argument("--no-wall", action="store_true", help="skip the wall radiosity exchange leg")
    ap.add_argument("--no-minor", action="store_true", help="skip the band model and minor species leg")
    ap.add_argument("--case", choices=["large", "medium", "xl"], default="large",
                    help="medium: the same furnace at 96x48x32, for kernel captures; xl: 384x160x96 with 10 bands "
                         "(neither is the benchmark workload)")
    ap.add_argument("--ttr", type=float, default=None,
                    help="threshold of the time-to-residual leg (default 1e-3, the plateau of the method)")
    ap.add_argument("--no-ttr", action="store_true", help="skip the time-to-residual and learned p' legs")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned p' leg")
    ap.add_argument("--no-ceiling", action="store_true",
                    help="skip the time-to-residual runs with converged pressure solves")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched furnace-variant leg")
    ap.add_argument("--ttr-max", type=int, default=1000)
    ap.add_argument("--batched", action="store_true",
                    help="run the batched furnace-variant workload instead of the 192x96x64 furnace")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lp-steps", type=int, default=1500, help="Adam steps per learning rate (two rates)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.batched:
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
