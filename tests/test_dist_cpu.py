"""The multi-rank harness of bench.py (one process per GPU, replicas, no data-path collective)
on CPU: world_size 2 over gloo.  The timings of all ranks reduce by MAX, the units they
processed by SUM, and every rank picks its own device."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), LOCAL_RANK=str(rank))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        cpu = torch.device("cpu")
        mx = bench.dist_max([1.0 + rank, 10.0 - rank, 0.5 * rank], world, cpu)
        sm = bench.dist_sum([100.0 * (rank + 1), 1.0], world, cpu)
        torch.distributed.barrier()
        q.put((rank, mx, sm, bench.rank_device(rank, world)))
    finally:
        torch.distributed.destroy_process_group()


def test_replica_reductions_over_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(world):
        rank, mx, sm, dev = q.get(timeout=120)
        out[rank] = (mx, sm, dev)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        mx, sm, dev = out[rank]
        assert mx == [2.0, 10.0, 0.5]
        assert sm == [300.0, 2.0]
        assert dev == rank


def test_single_rank_is_the_identity():
    import bench
    assert bench.dist_max([3.0, 4.0], 1, None) == [3.0, 4.0]
    assert bench.dist_sum([5.0], 1, None) == [5.0]
    assert bench.rank_device(0, 1) == 0
