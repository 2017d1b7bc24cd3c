"""The multi-GPU form of the path is replicas only: every rank solves its
own problems with no data exchange, and the bench reduces the
barrier-bracketed step time to its maximum over the ranks.  That reduction,
and the reference arm's rank rule (rank 0 alone runs the CPU path), run
here as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, root, q):
    import sys
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 1.5 * rank, world, "cpu")
        dist.barrier()
        ref = bench.run_reference(None, rank, world) if rank != 0 else "rank 0"
        q.put((rank, ms, ref))
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_maximum_over_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, root, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    assert [g[1] for g in got] == [11.5, 11.5]
    # ranks other than 0 do no reference work and print nothing
    assert got[1][2] is None


def test_single_rank_time_is_unchanged():
    import bench
    assert bench.max_over_ranks(12.25, 1, "cpu") == 12.25
