"""The multi-replica path of bench.py on the CPU: two gloo ranks agree on the
slowest replica's time and the whole-job rate, and the reference arm under a
launcher runs on rank 0 only (other ranks exit at once, printing nothing)."""
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


def _rank(rank, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        ws, r, local = bench._dist()
        t = bench.max_over_ranks(1.5 * (rank + 1), dist, "cpu")
        dist.barrier()
        q.put((rank, ws, r, local, t, bench.whole_job_rate(100.0, ws, t)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_replica():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, ws, r, local, t, rate in got:
        assert (ws, r, local) == (2, rank, rank)
        assert t == 3.0                      # max of 1.5 and 3.0, on both ranks
        assert rate == pytest.approx(2 * 100.0 / 3.0)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5) == 2.5


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
