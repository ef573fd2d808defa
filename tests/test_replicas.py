"""bench.py under torchrun runs one independent replica per GPU (the step has no exchange between GPUs): the job's
figure is every rank's agent-steps over the slowest rank's time, and the reference arm runs on rank 0 alone. The
cross-rank reduction is checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    # rank r: (r + 1) x 10 ms and (r + 1) x 1000 agent-steps
    t, a = bench.replica_totals(dist, "cpu", 10.0 * (rank + 1), 1000 * (rank + 1))
    out.put((rank, t, a))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for _, t, a in got:
        assert t == 20.0, "the slowest rank's time"
        assert a == 3000.0, "every rank's agent-steps"


def test_replica_totals_one_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(None, "cpu", 12.5, 700) == (12.5, 700.0)


def test_reference_arm_runs_on_rank_zero_only():
    """Ranks other than 0 exit at once without work (rank 0 alone times the CPU reference and prints its line)."""
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, gpus = 3, 3, 2
    assert bench.run_reference(Args(), 1, 2) == 0
