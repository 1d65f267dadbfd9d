"""The bench's N > 1 path on the CPU: two gloo ranks, replicas only.

Every rank builds its own index and answers its own query batches; the job's
rate is all ranks' queries over the slowest rank's time, and only rank 0
prints.  These tests run the rank logic of bench.py (process group set-up,
barriers, max over ranks, the reference arm's rank gate) in two processes with
the gloo backend and no GPU.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    dist, r, w, local = bench.init_dist(None)
    assert (r, w, local) == (rank, world, rank) and dist is not None
    bench.barrier(dist)
    # rank r took 1 + r seconds for 1,000 units: the job is 2,000 units over 2 s
    rate, t_max = bench.whole_job_rate(dist, w, 1000, 1.0 + r)
    m = bench.max_over_ranks(dist, [7.5, 3.0][r])
    # the reference arm runs on rank 0 alone; the other ranks return at once
    ref = bench.run_reference(None, dist, r, w, local) if r != 0 else "skipped"
    s, t, k = bench.make_queries(1000, 64, 5, seed=1000 + r)
    bench.barrier(dist)
    dist.destroy_process_group()
    out.put((rank, rate, t_max, m, ref, s.tolist(), t.tolist(), k.tolist()))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        rank, *rest = q.get(timeout=120)
        res[rank] = rest
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        rate, t_max, m, _, _, _, _ = res[r]
        assert t_max == pytest.approx(2.0)
        assert rate == pytest.approx(1000.0)
        assert m == pytest.approx(7.5)
    assert res[1][3] is None
    # each replica answers its own queries
    assert res[0][4] != res[1][4]
    for r in (0, 1):
        s, t, k = (np.asarray(x) for x in res[r][4:7])
        assert s.min() >= 0 and s.max() < 1000 and t.max() < 1000
        assert k.min() >= 1 and k.max() <= 5


def test_single_process_is_world_one(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, ROOT)
    import bench

    dist, r, w, local = bench.init_dist(None)
    assert dist is None and (r, w, local) == (0, 1, 0)
    assert bench.whole_job_rate(None, 1, 500, 0.5) == (1000.0, 0.5)
