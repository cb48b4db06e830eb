"""The N>1 host logic of bench.py (independent replicas: no data-path
collective, only the barrier and the max of the per-rank step times), run as
world_size-2 gloo process groups on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup()
    assert (r, w, local) == (rank, world, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank reports its own step time; the job's time is the slowest rank's
    t = bench.allreduce_max(10.0 + 5.0 * rank, w)
    # the reference arm does its work on rank 0 only: other ranks return at once
    if rank != 0:
        class A:
            pass
        bench.run_reference(A())
    bench.barrier(w)
    q.put((rank, t))
    dist.destroy_process_group()


def test_two_replicas_barrier_and_max_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert got == [(0, 15.0), (1, 15.0)]
