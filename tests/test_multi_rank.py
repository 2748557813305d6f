"""The multi-GPU form of the benchmark is replicas only: every rank solves
its own systems, the step time is the slowest rank's (all-reduce MAX) and the
job's value counts every rank's systems; the reference arm runs on rank 0
alone.  Checked on the CPU with world_size 2 gloo ranks (127.0.0.1)."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from tests.conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    m = bench.max_over_ranks(torch, dist, values[rank], torch.device("cpu"))
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, m))


def test_max_over_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    values = [1.25, 3.5]
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, values, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 3.5, 1: 3.5}


def test_job_value_counts_every_rank():
    sys.path.insert(0, str(ROOT))
    import bench

    one = bench.job_value(1, 69632, 0.94)
    assert abs(bench.job_value(4, 69632, 0.94) - 4 * one) < 1e-6 * one
    # the slowest rank sets the step: same work, longer step, lower value
    assert bench.job_value(2, 69632, 1.0) < bench.job_value(2, 69632, 0.94)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
