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


def _lane_worker(rank, world, port, q):
    """One rank of the bench's many-beam job: its beam slice, its lane schedule, and the
    whole-job sums the bench reports (work summed, time the slowest rank's)."""
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from transientx_gb300 import synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        job = synth.beams64()
        mine = beams_for_rank(len(job.beams), rank, world)
        chans, steps = bench.lane_schedule(job, mine, 2, 40, 2)
        beams = sorted({it[2] for st in steps for it in st})
        blocks = sum(len(st) for st in steps)
        total = sum_over_ranks(float(blocks), dist)
        q.put((rank, mine, beams, chans, blocks, total))
    finally:
        dist.destroy_process_group()


def test_gloo_ranks_schedule_disjoint_beam_slices():
    """World size 2: each rank's lane schedule walks only beams of its own slice of the
    64-beam job (no beam searched twice across ranks, no data exchanged), and the whole-job
    block count is the sum over ranks."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_lane_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, mine0, b0, c0, n0, t0), (r1, mine1, b1, c1, n1, t1) = res
    assert set(mine0).isdisjoint(mine1) and sorted(mine0 + mine1) == list(range(64))
    assert set(b0) <= set(mine0) and set(b1) <= set(mine1)
    assert t0 == t1 == float(n0 + n1)
