"""Batched build: many graphs of uneven size and hop bound indexed together
as one rank-interleaved disjoint union must give every graph exactly the
labels of its own build (all four fields)."""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H

pytestmark = pytest.mark.gpu


def _batch(count, nmin, nmax, seed):
    rng = np.random.default_rng(seed)
    graphs, Ks = [], []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        if i % 2 == 0:
            g = H.HostGraph.erdos_renyi(n, 3 * n, 1, 1000, seed=seed * 1000 + i)
        else:
            g = H.HostGraph.barabasi_albert(n, 3, 1, 1000, seed=seed * 1000 + i)
        graphs.append(g)
        Ks.append(int(rng.integers(3, 7)))
    return graphs, Ks


def _single(g, K):
    dev = H.Graph(g)
    ix = H.Index.build(dev, K)
    out = ix.export()
    ix.close()
    dev.close()
    return out


def test_batched_equals_single_builds(orc):
    graphs, Ks = _batch(40, 200, 3000, 7)
    idxs = H.Index.build_batched(graphs, Ks)
    assert len(idxs) == len(graphs)
    for i, (g, K, ix) in enumerate(zip(graphs, Ks, idxs)):
        off, lab = ix.export()
        soff, slab = _single(g, K)
        assert np.array_equal(off, soff), i
        assert np.array_equal(lab, slab), i
        info = ix.info()
        assert info["n"] == g.n and info["K"] == K and info["cleaned"] == 1
    # two of them straight against the oracle
    for i in (0, 1):
        ref = orc.build(graphs[i], Ks[i], threads=1)
        off, lab = idxs[i].export()
        assert np.array_equal(off, ref.off) and np.array_equal(lab, ref.lab)
    # queries work on the per-graph indexes
    rng = np.random.default_rng(1)
    g, K, ix = graphs[3], Ks[3], idxs[3]
    s = rng.integers(0, g.n, 5000).astype(np.int32)
    t = rng.integers(0, g.n, 5000).astype(np.int32)
    k = rng.integers(1, K + 1, 5000).astype(np.int32)
    ref = orc.build(g, K, threads=1)
    assert np.array_equal(ix.query(s, t, k), orc.query(ref, s, t, k))


def test_batched_sub_batches_under_a_tight_budget():
    graphs, Ks = _batch(12, 300, 2000, 11)
    a = H.Index.build_batched(graphs, Ks)
    b = H.Index.build_batched(graphs, Ks, device_budget_bytes=64 << 20)  # forces several sub-batches
    for x, y in zip(a, b):
        ox, lx = x.export()
        oy, ly = y.export()
        assert np.array_equal(ox, oy) and np.array_equal(lx, ly)


def test_batched_autotune_and_small_waves():
    """The batched tuner returns valid shapes; a batch built with them, and
    with a small hub cap per wave, still gives every graph its own labels."""
    graphs, Ks = _batch(24, 200, 2000, 9)
    r = H.autotune_build_batched(graphs, Ks, sample_graphs=8)
    assert r["block_threads"] in (128, 256, 512) and r["prune_lanes"] in (0, 8, 16, 32)
    assert r["max_wave"] in (65536, 131072, 262144, 524288) and r["trials"] >= 10
    shapes = {k: r[k] for k in ("max_wave", "block_threads", "frontier_tile", "prune_lanes", "prune_pairs")}
    tuned = H.Index.build_batched(graphs, Ks, **shapes)
    small = H.Index.build_batched(graphs, Ks, max_wave=256, prune_lanes=8)
    for g, K, a, b in zip(graphs, Ks, tuned, small):
        want = _single(g, K)
        for ix in (a, b):
            off, lab = ix.export()
            assert np.array_equal(off, want[0]) and np.array_equal(lab, want[1])
