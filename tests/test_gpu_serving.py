"""Serving loop: a persistent kernel answering (graph, s, t, k) requests over
several resident indexes while builds run.  Every answer must be the same
alone and in the mix, and equal the batched path's (itself pinned to the
oracle by test_gpu_parity)."""
import time

import numpy as np
import pytest

import gpu4hophl_code_gb300 as H
from gpu4hophl_code_gb300._native import HSDL_ERR_FULL, HSDL_ERR_TIMEOUT, HsdlError

pytestmark = pytest.mark.gpu

INT_MAX = 2147483647


def _graphs():
    return [H.HostGraph.chung_lu(6000, 8, 2.2, 600, 1, 100, seed=41),
            H.HostGraph.erdos_renyi(2000, 8000, 1, 100, seed=42),
            H.HostGraph.barabasi_albert(3000, 3, 1, 1000, seed=43)]


def _queries(rng, n, count, K):
    s = rng.integers(0, n, count).astype(np.int32)
    t = rng.integers(0, n, count).astype(np.int32)
    k = rng.integers(1, K + 1, count).astype(np.int32)
    return s, t, k


def test_alone_equals_mix_and_concurrent_build():
    K = 5
    hg = _graphs()
    devs = [H.Graph(g) for g in hg]
    idxs = [H.Index.build(d, K) for d in devs]
    srv = H.Server(idle_exit_s=0.2)
    gids = [srv.add_index(ix) for ix in idxs]
    rng = np.random.default_rng(3)
    qs = [_queries(rng, g.n, 20000, K) for g in hg]
    # alone: each graph's batch by itself
    alone = [srv.query(np.full(20000, gid, np.int32), *q) for gid, q in zip(gids, qs)]
    for ix, q, a in zip(idxs, qs, alone):
        assert np.array_equal(a, ix.query(*q))
    # mix: all graphs interleaved, while a new graph is being built
    extra = H.HostGraph.chung_lu(20000, 8, 2.2, 800, 1, 100, seed=44)
    extra_dev = H.Graph(extra)
    gid_new = srv.submit_build(extra_dev, K)
    order = rng.permutation(60000)
    g_all = np.concatenate([np.full(20000, gid, np.int32) for gid in gids])[order]
    s_all = np.concatenate([q[0] for q in qs])[order]
    t_all = np.concatenate([q[1] for q in qs])[order]
    k_all = np.concatenate([q[2] for q in qs])[order]
    mixed = srv.query(g_all, s_all, t_all, k_all)
    want = np.concatenate(alone)[order]
    assert np.array_equal(mixed, want)
    srv.wait_graph(gid_new, 300)
    assert srv.graph_state(gid_new)[0] == 2
    ref_new = H.Index.build(extra_dev, K)
    q_new = _queries(rng, extra.n, 20000, K)
    got_new = srv.query(np.full(20000, gid_new, np.int32), *q_new)
    assert np.array_equal(got_new, ref_new.query(*q_new))
    st = srv.stats()
    assert st["resident_graphs"] == 4 and st["bad_requests"] == 0 and st["builds_done"] == 1
    srv.close()


def test_loadgen_answers_and_latency():
    K = 5
    g = H.HostGraph.chung_lu(10000, 8, 2.2, 800, 1, 100, seed=51)
    dev = H.Graph(g)
    ix = H.Index.build(dev, K)
    srv = H.Server()
    gid = srv.add_index(ix)
    rng = np.random.default_rng(5)
    s, t, k = _queries(rng, g.n, 200000, K)
    r = srv.loadgen(np.full(len(s), gid, np.int32), s, t, k, offered_qps=2e6)
    assert r["completed"] == len(s)
    assert np.array_equal(r["answers"], ix.query(s, t, k))
    assert 0 < r["p50_us"] <= r["p99_us"] <= r["max_us"]
    r2 = srv.loadgen(np.full(len(s), gid, np.int32), s, t, k, offered_qps=0)  # saturation
    assert np.array_equal(r2["answers"], r["answers"])
    srv.close()


def test_idle_exit_relaunch_bad_ids_and_removal():
    K = 4
    g = H.HostGraph.erdos_renyi(1500, 6000, 1, 50, seed=61)
    dev = H.Graph(g)
    ix = H.Index.build(dev, K)
    srv = H.Server(idle_exit_s=0.05)
    gid = srv.add_index(ix)
    rng = np.random.default_rng(6)
    s, t, k = _queries(rng, g.n, 5000, K)
    a1 = srv.query(np.full(5000, gid, np.int32), s, t, k)
    time.sleep(0.3)  # the loop returns after 50 ms idle
    st = srv.stats()
    assert st["loop_running"] == 0  # its bounded idle wait ran out and it returned
    assert st["processed"] == st["submitted"] == 5000
    a2 = srv.query(np.full(5000, gid, np.int32), s, t, k)  # relaunched
    assert np.array_equal(a1, a2) and np.array_equal(a1, ix.query(s, t, k))
    bad = srv.query(np.array([gid + 7, -1], np.int32), s[:2], t[:2], k[:2])
    assert list(bad) == [INT_MAX, INT_MAX]
    assert srv.stats()["bad_requests"] == 2
    srv.remove_graph(gid)
    gone = srv.query(np.full(3, gid, np.int32), s[:3], t[:3], k[:3])
    assert list(gone) == [INT_MAX] * 3
    srv.close()


def test_build_admission_budget():
    g = H.HostGraph.chung_lu(50000, 8, 2.2, 1000, 1, 100, seed=71)
    dev = H.Graph(g)
    srv = H.Server(budget_bytes=1 << 20)  # 1 MiB: far below the estimate
    with pytest.raises(HsdlError) as e:
        srv.submit_build(dev, 5)
    assert e.value.code == HSDL_ERR_FULL and "budget" in str(e.value)
    srv.close()


def test_wait_that_runs_out_reports_timeout():
    """A bounded wait that runs out returns HSDL_ERR_TIMEOUT and leaves the
    server usable: waiting no time at all for a build that has just been
    queued."""
    g = H.HostGraph.chung_lu(200000, 8, 2.2, 2000, 1, 100, seed=71)
    dev = H.Graph(g)
    srv = H.Server(idle_exit_s=0.05)
    gid = srv.submit_build(dev, 5)
    with pytest.raises(HsdlError) as e:
        srv.wait_graph(gid, timeout_s=0.0)
    assert e.value.code == HSDL_ERR_TIMEOUT
    srv.wait_graph(gid, timeout_s=600.0)
    rng = np.random.default_rng(9)
    s, t, k = _queries(rng, g.n, 20000, 5)
    ref = H.Index.build(dev, 5)
    assert np.array_equal(srv.query(np.full(20000, gid, np.int32), s, t, k), ref.query(s, t, k))
    srv.close()


@pytest.mark.parametrize("lanes", [32, 16, 8])
def test_mixed_key_formats_in_one_warp(orc, lanes):
    """One index whose ranges fit the compact 4-byte query keys and one whose
    distances need the 8-byte keys, served together: with 16 or 8 lanes per
    request a warp answers requests of both formats in one step."""
    K = 5
    small = H.HostGraph.erdos_renyi(1500, 6000, 1, 100, seed=45)
    wide = H.HostGraph.erdos_renyi(1500, 6000, 1, 2_000_000, seed=46)
    devs = [H.Graph(small), H.Graph(wide)]
    idxs = [H.Index.build(d, K) for d in devs]
    assert idxs[0].info()["query_key_bytes"] == 4 and idxs[1].info()["query_key_bytes"] == 8
    srv = H.Server(idle_exit_s=0.2, lanes_per_query=lanes)
    gids = [srv.add_index(ix) for ix in idxs]
    rng = np.random.default_rng(9)
    g = rng.integers(0, 2, 30000).astype(np.int32)
    s = rng.integers(0, 1500, 30000).astype(np.int32)
    t = rng.integers(0, 1500, 30000).astype(np.int32)
    k = rng.integers(1, K + 1, 30000).astype(np.int32)
    got = srv.query(np.asarray(gids, np.int32)[g], s, t, k)
    for j, ix in enumerate(idxs):
        sel = g == j
        assert np.array_equal(got[sel], ix.query(s[sel], t[sel], k[sel]))
    srv.close()
    for ix, d in zip(idxs, devs):
        ix.close()
        d.close()


@pytest.mark.parametrize("ctas,ring_log2", [(1, 12), (3, 12), (0, 16)])
def test_pooled_chunks_few_blocks_and_ring_wraps(ctas, ring_log2):
    """The warps of a block pool their chunks of 8 tickets.  One block (the
    dispatcher's, 7 workers), three blocks (7 + 8 + 8 workers) and the default
    grid, with a ring the Poisson run wraps many times: every answer equals the
    batched path's, in a closed batch and under Poisson arrivals."""
    K = 5
    g = H.HostGraph.chung_lu(10000, 8, 2.2, 800, 1, 100, seed=71)
    dev = H.Graph(g)
    ix = H.Index.build(dev, K)
    srv = H.Server(ctas=ctas, ring_log2=ring_log2)
    gid = srv.add_index(ix)
    rng = np.random.default_rng(ctas + 7)
    s, t, k = _queries(rng, g.n, 50000, K)
    want = ix.query(s, t, k)
    m = min(len(s), (1 << ring_log2) - 64)  # a closed batch must fit the ring (answers are read after it)
    assert np.array_equal(srv.query(np.full(m, gid, np.int32), s[:m], t[:m], k[:m]), want[:m])
    r = srv.loadgen(np.full(len(s), gid, np.int32), s, t, k, offered_qps=2e6, seed=ctas + 1)
    assert r["completed"] == len(s) and np.array_equal(r["answers"], want)
    srv.close()
