"""The multi-rank path of bench.py (replicas only: every rank runs its own
replica batch, the only collectives are the max of the timed region and the
sums of the counters after it) on two CPU ranks over gloo."""

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench

    ws, r, local, dist = bench.dist_init()
    t_max = bench.reduce_max(dist, 1.0 + r)        # slowest rank's time
    props = bench.reduce_sum(dist, 1000.0 * (r + 1))  # proposals of all ranks
    bench.barrier(dist)
    # per-rank seeds differ (rank offset), so ranks run different chains
    seed0 = 20251203 * 1000 + 7919 * r
    out.put((r, ws, t_max, props, seed0))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[1] for x in res] == [2, 2]
    assert all(x[2] == 2.0 for x in res)      # max over ranks
    assert all(x[3] == 3000.0 for x in res)   # whole-job sum
    assert res[0][4] != res[1][4]
