"""Multi-rank plumbing of bench.py on CPU: two gloo ranks (world size 2).

The batched workload shards by system: every rank builds its own systems from
a rank-dependent seed, runs them with no data-path collective, and the job
reports the sum of collisions over the maximum time.  This checks the rank
set-up, the barrier, the max/sum reductions and that the shards are disjoint.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_init(world)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + r)
    n = bench.sum_over_ranks(dist, 10.0 * (r + 1))
    params = bench.batched_params(64, 7, r)
    out.put((r, w, t, n, params))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 2.0 for r in res)            # max over ranks
    assert all(r[3] == 30.0 for r in res)           # sum over ranks
    seeds0 = {p[2] for p in res[0][4]}
    seeds1 = {p[2] for p in res[1][4]}
    assert not seeds0 & seeds1                      # disjoint shards
