"""Multi-rank host logic on CPU (gloo, world size 2).  Every rank extracts its
own volumes (independent units, weak scaling) and the job reports the
slowest rank's time with the units of all ranks; the reference arm runs on
rank 0 alone under torchrun."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _combine_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms, units = bench.combine_ranks(1.0 + rank, 10 * (rank + 1), dist, "cpu")
    out[rank] = (ms, units)
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_gloo():
    import torch.multiprocessing as mp
    mgr = mp.get_context("spawn").Manager()   # no fork of this multi-threaded process
    out = mgr.dict()
    mp.spawn(_combine_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    assert out[0] == out[1] == (2.0, 30.0)


def test_combine_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(3.5, 7, None, "cpu") == (3.5, 7)


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "sphere64",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cpu_model"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    for key in ("metric", "unit", "steps", "warmup", "ms_per_step", "higher_is_better", "config"):
        assert key in d


def _shard_exchange_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    from framework_gb300 import shard
    totals = shard.exchange_totals(10 + rank, 100 + 7 * rank, dist)
    out[rank] = (totals, shard.exclusive_offsets(totals, rank))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_exchange_gloo():
    """The one collective of a sharded extraction: every rank gets all ranks'
    totals in rank order, and its exclusive offsets from them."""
    import torch.multiprocessing as mp
    mgr = mp.get_context("spawn").Manager()   # no fork of this multi-threaded process
    out = mgr.dict()
    mp.spawn(_shard_exchange_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    assert out[0] == ([(10, 100), (11, 107)], (0, 0))
    assert out[1] == ([(10, 100), (11, 107)], (10, 100))


def test_shard_ranges_and_halo():
    sys.path.insert(0, ROOT)
    from framework_gb300 import shard
    for cz, world, align in [(1023, 8, 32), (1023, 3, 32), (100, 7, 32), (9, 9, 32), (5000, 4, 64), (260, 5, 32)]:
        r = shard.shard_ranges(cz, world, align)
        assert len(r) == world and r[0][0] == 0 and r[-1][1] == cz
        assert all(a < b for a, b in r) and all(r[i][1] == r[i + 1][0] for i in range(world - 1))
        if cz >= world * align:
            assert all(b % align == 0 for _, b in r[:-1])
    assert shard.point_planes(1024, 0, 100) == (0, 103)
    assert shard.point_planes(1024, 100, 1023) == (99, 1024)
    assert shard.point_planes(1024, 500, 520) == (499, 523)
    assert shard.exchange_totals(5, 6) == [(5, 6)]
    assert shard.exclusive_offsets([(1, 2), (3, 4), (5, 6)], 2) == (4, 6)
