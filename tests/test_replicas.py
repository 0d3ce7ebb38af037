"""The multi-GPU form is replicas only (the path has no exchange step): each
rank runs the whole workload and rank 0 reports the aggregate over the
slowest rank.  These CPU tests cover the rank coordination of bench.py with
two gloo ranks, and the reference arm under torchrun, where rank 0 alone runs
and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    world, r, local = bench.dist_setup()
    bench.barrier(world)
    slowest = bench.max_over_ranks(world, 10.0 + 5.0 * r)  # ms per step of each rank
    out.put((r, world, local, slowest))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_coordination():
    """dist_setup joins two gloo ranks; max_over_ranks gives every rank the
    slowest rank's time (the timing rule of the replica bench)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_reference_arm_under_torchrun():
    """bench.py --impl reference with two ranks: rank 0 alone times the CPU
    path and prints one line; rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--workload", "c1", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--cpu-seconds", "0.2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
