"""bench.py's multi-rank logic on the CPU (gloo, world size 2): the timing is the slowest rank's,
the value is the whole job's, and the reference arm's other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = bench.max_over_ranks(times[rank])
    out[rank] = (m, bench.whole_job_rate(1_000_000, m, world))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    times = [2.0, 3.5]  # ms per step on each rank
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        m, rate = out[r]
        assert m == 3.5
        assert rate == pytest.approx(2 * 1_000_000 / 3.5e-3)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(1.25) == 1.25
    assert bench.whole_job_rate(10, 2.0, 1) == pytest.approx(5000.0)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""
