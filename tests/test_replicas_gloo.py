"""Replica partitioning and the max-over-ranks timing reduction, on two
gloo ranks on the CPU (the multi-GPU bench path is replicas only)."""
import os

import pytest
import torch.multiprocessing as mp

from fluidsurfacereconstructiongpu_gb300.replicas import frames_for_rank


def test_partition_covers_every_frame_once():
    sizes = [20000, 400000, 37000, 150000, 99999, 21000, 300000]
    parts = [frames_for_rank(sizes, 3, r) for r in range(3)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from fluidsurfacereconstructiongpu_gb300.replicas import frames_for_rank, max_over_ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [5, 3, 8, 1, 9, 2]
    mine = frames_for_rank(sizes, world, rank)
    t = max_over_ranks(1.0 + rank)  # rank 1 is the slow one
    q.put((rank, mine, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][2] == out[1][2] == 2.0
    assert sorted(out[0][1] + out[1][1]) == list(range(6))
