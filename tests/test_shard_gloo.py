"""Multi-rank logic on CPU with the gloo backend (world size 2): beam ownership is a disjoint
cover, and the cross-rank reductions the bench uses give the slowest rank's time and the
whole-job work."""
import os
import socket

import pytest

from transientx_gb300.shard import beams_for_rank, max_over_ranks, sum_over_ranks


def test_beams_cover_disjoint():
    for nb in (1, 2, 7, 64):
        for world in (1, 2, 3, 8):
            owned = [beams_for_rank(nb, r, world) for r in range(world)]
            flat = [b for o in owned for b in o]
            assert sorted(flat) == list(range(nb))
            assert max(map(len, owned)) - min(map(len, owned)) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = beams_for_rank(5, rank, world)
        t = 1.0 + rank          # rank 1 is slower
        slowest = max_over_ranks(t, dist)
        work = sum_over_ranks(100.0 * len(mine), dist)
        q.put((rank, mine, slowest, work))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == [0, 1, 2] and res[1][1] == [3, 4]
    assert all(r[2] == 2.0 for r in res)
    assert all(r[3] == 500.0 for r in res)
