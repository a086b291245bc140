"""The replica path of bench.py under two ranks, on CPU with gloo: rank
discovery from the environment, the barrier, the max-over-ranks timing the
JSON line is built from, and the reference arm's rank-0-only rule.  The
solver itself is not run here (it needs a GPU); every rank solves its own
furnace and no collective touches the data path."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent

WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local = bench.dist_env()
import torch.distributed as dist
dist.init_process_group("gloo")
bench.barrier(dist)
t = bench.max_over_ranks(dist, 1.0 + rank)
s = bench.max_over_ranks(dist, 10.0 * (world - rank))
print(json.dumps({"rank": rank, "world": world, "local": local, "max_t": t, "max_s": s}))
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(code, world=2, extra_env=None):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code, str(ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_two_rank_barrier_and_max_over_ranks():
    pytest.importorskip("torch.distributed")
    outs = _run_ranks(WORKER)
    lines = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    for l in lines:
        assert l["world"] == 2 and l["local"] == l["rank"]
        assert l["max_t"] == 2.0 and l["max_s"] == 20.0


def test_reference_arm_other_ranks_exit_without_work():
    pytest.importorskip("torch.distributed")
    code = r"""
import sys
sys.path.insert(0, sys.argv[1])
import bench
class A: gpus = 2; steps = 1; warmup = 0
sys.exit(bench.run_reference(A()) if bench.dist_env()[0] != 0 else 0)
"""
    outs = _run_ranks(code)
    assert all(o.strip() == "" for o in outs)
