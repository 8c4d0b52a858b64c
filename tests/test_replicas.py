"""Host logic of multi-GPU replica runs, on CPU: the instance split of a work
list (every item on exactly one rank, balanced cost, the same answer on every
rank) and the max/sum reductions, in two gloo processes."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from phrike_gb300.replicas import reduce_max, reduce_sum, shard


def test_shard_partitions_and_balances():
    costs = [float(n) ** 3 for n in (64, 512, 128, 256, 512, 64, 256, 128, 512, 64)]
    for world in (1, 2, 3, 4):
        parts = [shard(costs, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    with pytest.raises(ValueError):
        shard(costs, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = [1.0, 5.0, 2.0, 2.0, 3.0]
        mine = shard(costs, rank, world)
        out[rank] = (mine, reduce_max(1.5 + rank), reduce_sum(len(mine)))
    finally:
        dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res[0][0] + res[1][0]) == [0, 1, 2, 3, 4]
    assert res[0][1] == res[1][1] == 2.5          # max over ranks
    assert res[0][2] == res[1][2] == 5.0          # every item counted once


def test_reference_arm_under_torchrun_two_ranks():
    """bench.py --impl reference launched like the multi-GPU runs: rank 0
    times the reference path and prints one JSON line, rank 1 exits 0."""
    import json
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--size", "16", "--steps", "1", "--warmup", "1"]
    res = subprocess.run(cmd, cwd=repo, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
