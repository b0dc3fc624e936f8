"""Replica timing across processes (gloo, world size 2, CPU): every rank gets
the slowest rank's time, the whole-job rate counts all ranks' work, and the
reference arm prints from rank 0 only."""

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    from rstsr_gb300 import replicas

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        replicas.barrier()
        secs = 0.5 if rank == 0 else 2.0  # rank 1 is the slow one
        rate, t = replicas.whole_job_rate(1000.0, secs)
        q.put((rank, replicas.world_size(), t, rate))
    finally:
        dist.destroy_process_group()


def test_max_time_and_whole_job_rate_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, world, t, rate in got:
        assert world == 2
        assert t == pytest.approx(2.0)
        assert rate == pytest.approx(2 * 1000.0 / 2.0)


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    from rstsr_gb300 import replicas

    assert replicas.world_size() == 1
    assert replicas.whole_job_rate(10.0, 0.5) == (20.0, 0.5)


def test_reference_arm_prints_from_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
