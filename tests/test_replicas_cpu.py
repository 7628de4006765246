"""The multi-GPU form is replicas (worlds are independent; a pass has no exchange step): each rank
runs the same workload and the job's time is the slowest rank's.  The rank logic of bench.py is
checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    class A:
        pass

    r, local, ws, pg = bench.dist_setup(A())
    assert (r, local, ws) == (rank, rank, world) and pg is dist
    assert dist.get_backend() == "gloo"
    slowest = bench.max_over_ranks(1.5 + rank, pg, "cpu")
    out[rank] = (slowest, bench.job_value(1000.0, ws, slowest))
    pg.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        assert out[0] == out[1] == (2.5, 2 * 1000.0 / 2.5)


def test_single_rank_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.0, None, "cpu") == 3.0
    assert bench.job_value(10.0, 1, 2.0) == 5.0
