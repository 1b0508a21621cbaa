"""The multi-rank logic of bench.py on CPU (gloo, world size 2): replicas
report the slowest rank's time and the sum of their work; the reference arm
runs on rank 0 only."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(1.5 + rank)          # rank 0: 1.5 s, rank 1: 2.5 s
    q.put((rank, slowest, bench.job_throughput(100.0, slowest, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2.5, 80.0), (1, 2.5, 80.0)]


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.job_throughput(10.0, 2.0, 1) == 5.0


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_roofline_traffic_is_read_from_the_committed_profile():
    """The DRAM traffic of the bench's dominant kernel comes from the ncu
    summary under profiles/ (indented key lines included)."""
    sys.path.insert(0, ROOT)
    import bench

    t = bench.profile_traffic("ch3_stream_f32_256")
    assert t is not None and 1e7 < t < 1e9
    assert bench.profile_traffic("no_such_kernel") is None
