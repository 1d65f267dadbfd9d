"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's golden vectors.  Bit-exact on every integer field.

* uncleaned GPU labels == oracle generation with the same wave schedule
  (hub, parent, hop, distance - all four fields);
* cleaned GPU labels == oracle sequential run (all four fields) and the
  reference's labels (hub, hop, distance);
* query answers == reference answers == hop-bounded Bellman-Ford.
"""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H

pytestmark = pytest.mark.gpu

INT_MAX = 2147483647


def gpu_build(g, K, **opts):
    dev = H.Graph(g)
    idx = H.Index.build(dev, K, **opts)
    return dev, idx


def test_golden_cleaned_labels_and_queries(golden, orc):
    g, K = golden.g, golden.K
    dev, idx = gpu_build(g, K)
    off, lab = idx.export()
    ref = orc.build(g, K, threads=1)
    assert np.array_equal(off, ref.off)
    assert np.array_equal(lab, ref.lab)  # all four fields vs the oracle
    if golden.full:
        assert np.array_equal(lab[:, [0, 2, 3]], golden.d["labels"][:, [0, 2, 3]])
    got = idx.query(golden.d["q_s"], golden.d["q_t"], golden.d["q_k"])
    assert np.array_equal(got, golden.d["q_ans"])
    for src, hop, bf in zip(golden.d["bf_src"], golden.d["bf_hop"], golden.d["bf_dist"]):
        q = idx.query(np.full(g.n, src, np.int32), np.arange(g.n, dtype=np.int32), np.full(g.n, hop, np.int32))
        assert np.array_equal(q, bf)


@pytest.mark.parametrize("max_wave", [1, 4, 64, 0])
def test_uncleaned_generation_matches_wave_oracle(orc, max_wave):
    g = H.HostGraph.chung_lu(3000, 8, 2.2, 300, 1, 100, seed=21)
    K = 5
    dev, idx = gpu_build(g, K, clean=False, max_wave=max_wave)
    b = H.wave_bounds(g.n, max_wave=max_wave)
    off, lab = idx.export()
    ref = orc.build(g, K, threads=4, wave_bounds=b, clean=False)
    assert np.array_equal(off, ref.off)
    assert np.array_equal(lab, ref.lab)
    idx.clean()
    off2, lab2 = idx.export()
    canon = orc.build(g, K, threads=1)
    assert np.array_equal(off2, canon.off) and np.array_equal(lab2, canon.lab)


@pytest.mark.parametrize("block_threads,frontier_tile,prune_lanes,prune_pairs,prune_order,pool_key_bytes",
                         [(128, 0, 8, 1, 0, 0), (512, 4096, 16, 2, 1, 0), (256, 1024, 32, 1, 0, 8),
                          (256, 0, 0, 2, 0, 8), (256, 0, 8, 2, 1, 0), (256, 0, 0, 1, 1, 8), (256, 0, 16, 1, 0, 0),
                          (256, 0, 32, 1, 2, 0), (256, 0, 32, 1, 2, 8), (256, 0, 0, 1, 2, 0)])
def test_launch_shapes_do_not_change_labels(orc, block_threads, frontier_tile, prune_lanes, prune_pairs,
                                            prune_order, pool_key_bytes):
    """The uncleaned superset depends on the wave schedule only; threads per
    block, frontier tile, prune lanes, the order candidates are joined in and
    the width of the label pool's keys change the time, never a label."""
    g = H.HostGraph.chung_lu(3000, 8, 2.2, 300, 1, 100, seed=22)
    K = 5
    dev, idx = gpu_build(g, K, clean=False, max_wave=64, block_threads=block_threads,
                         frontier_tile=frontier_tile, prune_lanes=prune_lanes, prune_pairs=prune_pairs,
                         prune_order=prune_order, pool_key_bytes=pool_key_bytes)
    assert idx.info()["build_pool_key_bytes"] == (pool_key_bytes or 4)
    off, lab = idx.export()
    ref = orc.build(g, K, threads=4, wave_bounds=H.wave_bounds(g.n, max_wave=64), clean=False)
    assert np.array_equal(off, ref.off) and np.array_equal(lab, ref.lab)


def test_autotune_picks_valid_shapes():
    g = H.HostGraph.chung_lu(20000, 8, 2.2, 800, 1, 100, seed=24)
    dev = H.Graph(g)
    r = H.autotune_build(dev, 5, sample_hubs=4096)
    assert r["block_threads"] in (128, 256, 512) and r["prune_lanes"] in (0, 8, 16, 32)
    assert r["max_wave"] in (1024, 2048, 4096, 8192) and r["frontier_tile"] >= 0
    assert r["seconds"] > 0 and r["trials"] >= 10
    shapes = {k: r[k] for k in ("max_wave", "block_threads", "frontier_tile", "prune_lanes", "prune_pairs")}
    a = H.Index.build(dev, 5, **shapes).export()
    b = H.Index.build(dev, 5).export()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_memory_limited_build_splits_waves_and_grows_pool(orc):
    """Under a device budget far below what the waves want, waves whose
    candidate lists outgrow it run as halves and the label pool grows by
    chunks; the cleaned labels stay the canonical set."""
    g = H.HostGraph.chung_lu(8000, 8, 2.2, 600, 1, 100, seed=23)
    K = 5
    dev, idx = gpu_build(g, K, max_wave=2048, device_budget_bytes=8 << 20)
    info = idx.info()
    assert info["build_wave_splits"] > 0 and info["build_pool_chunks"] > 1
    assert info["build_peak_bytes"] > 0 and info["build_max_candidates"] > 0
    assert info["build_pool_entries"] >= info["labels_before_clean"] - g.n
    off, lab = idx.export()
    canon = orc.build(g, K, threads=8)
    assert np.array_equal(off, canon.off) and np.array_equal(lab, canon.lab)
    _, free_idx = gpu_build(g, K, max_wave=2048)
    assert free_idx.info()["build_wave_splits"] == 0


def test_gpu_clean_of_oracle_superset(orc):
    """hsdl_clean on an imported superset equals the oracle's clean of it."""
    g = H.HostGraph.erdos_renyi(800, 4000, 1, 50, seed=5)
    K = 5
    b = [0, 1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 800]
    sup = orc.build(g, K, threads=4, wave_bounds=b, clean=False)
    idx = H.Index.import_labels(g.n, K, sup.off, sup.lab)
    idx.clean()
    off, lab = idx.export()
    canon = orc.build(g, K, threads=1)
    assert np.array_equal(off, canon.off) and np.array_equal(lab, canon.lab)


@pytest.mark.parametrize("kind,K", [("er", 1), ("er", 3), ("ba", 6), ("cl", 4), ("unit", 5), ("er", 9)])
def test_graph_families_and_hop_bounds(orc, kind, K):
    if kind == "er":
        g = H.HostGraph.erdos_renyi(600, 2400, 1, 100, seed=K)
    elif kind == "ba":
        g = H.HostGraph.barabasi_albert(1500, 3, 1, 1000, seed=3)
    elif kind == "cl":
        g = H.HostGraph.chung_lu(5000, 10, 2.1, 500, 1, 100, seed=4)
    else:
        g = H.HostGraph.erdos_renyi(500, 1500, 1, 1, seed=6)  # unit weights: many ties
    dev, idx = gpu_build(g, K)
    off, lab = idx.export()
    ref = orc.build(g, K, threads=1)
    assert np.array_equal(off, ref.off) and np.array_equal(lab, ref.lab)
    rng = np.random.default_rng(K)
    s = rng.integers(0, g.n, 20000).astype(np.int32)
    t = rng.integers(0, g.n, 20000).astype(np.int32)
    k = rng.integers(-1, K + 2, 20000).astype(np.int32)
    assert np.array_equal(idx.query(s, t, k), orc.query(ref, s, t, k))


def test_edge_cases_small_and_disconnected(orc):
    # isolated vertices, two components, a path graph, n = 1
    a = np.array([0, 1, 2, 5, 6], np.int32)
    b = np.array([1, 2, 3, 6, 7], np.int32)
    w = np.array([3, 1, 4, 1, 5], np.int32)
    g = H.HostGraph.from_edges(10, a, b, w, rank_by_degree=True)
    dev, idx = gpu_build(g, 3)
    off, lab = idx.export()
    ref = orc.build(g, 3, threads=1)
    assert np.array_equal(off, ref.off) and np.array_equal(lab, ref.lab)
    s, t = np.meshgrid(np.arange(10, dtype=np.int32), np.arange(10, dtype=np.int32))
    s, t = s.ravel(), t.ravel()
    for k in (0, 1, 2, 3, 4):
        kk = np.full(len(s), k, np.int32)
        assert np.array_equal(idx.query(s, t, kk), orc.query(ref, s, t, kk))
    one = H.HostGraph.from_edges(1, [], [], [], rank_by_degree=False)
    d1, i1 = gpu_build(one, 2)
    o1, l1 = i1.export()
    assert list(o1) == [0, 1] and l1.tolist() == [[0, 0, 0, 0]]
    assert list(i1.query([0], [0], [1])) == [0]


def test_determinism_and_roundtrips(orc, tmp_path):
    g = H.HostGraph.chung_lu(4000, 10, 2.1, 400, 1, 100, seed=77)
    K = 5
    _, a = gpu_build(g, K)
    _, b = gpu_build(g, K)
    oa, la = a.export()
    ob, lb = b.export()
    assert np.array_equal(oa, ob) and np.array_equal(la, lb)
    c = H.Index.import_labels(g.n, K, oa, la)
    oc, lc = c.export()
    assert np.array_equal(oa, oc) and np.array_equal(la, lc)
    p = str(tmp_path / "labels.bin")
    a.save(p)
    d = H.Index.load(p, K)
    od, ld = d.export()
    assert np.array_equal(oa, od) and np.array_equal(la, ld)
    # file layout: size_t V, then per vertex size_t count + 16-byte records
    raw = open(p, "rb").read()
    assert int.from_bytes(raw[:8], "little") == g.n
    assert len(raw) == 8 + 8 * g.n + 16 * len(la)


def test_paths_are_valid_and_match_the_oracle(orc):
    g = H.HostGraph.erdos_renyi(400, 1600, 1, 100, seed=9)
    K = 5
    _, idx = gpu_build(g, K)
    ref = orc.build(g, K, threads=1)
    rng = np.random.default_rng(1)
    wmap = {}
    for v in range(g.n):
        for e in range(g.row_ptr[v], g.row_ptr[v + 1]):
            wmap[(v, int(g.col[e]))] = int(g.w[e])
    for _ in range(200):
        s, t, k = int(rng.integers(g.n)), int(rng.integers(g.n)), int(rng.integers(1, K + 1))
        p = idx.path(s, t, k)
        assert p == orc.path(ref, s, t, k)
        d = int(idx.query([s], [t], [k])[0])
        if s == t:
            assert p == []
        elif d == INT_MAX:
            assert p == []
        else:
            assert sum(wmap[(a, b)] for a, b in p) == d and len(p) <= k


def test_reference_shaped_api(orc):
    g = H.HostGraph.erdos_renyi(300, 1200, 1, 100, seed=2)
    ci = H.hop_constrained_case_info(upper_k=4, use_canonical_repair=True, thread_num=8)
    H.hop_constrained_two_hop_labels_generation(g, ci)
    ref = orc.build(g, 4, threads=1)
    assert ci.L.total() == len(ref.lab)
    assert ci.label_size_after_canonical_repair == len(ref.lab)
    assert ci.label_size_before_canonical_repair >= ci.label_size_after_canonical_repair
    for v in (0, 5, 299):
        assert np.array_equal(ci.L[v], ref.row(v))
    assert H.hop_constrained_extract_distance(ci.L, 3, 3, 2) == 0
    assert H.hop_constrained_extract_distance(ci.L, 3, 7, -1) == INT_MAX
    q = np.array([[1, 2, 3], [4, 5, 4], [7, 7, 0]], np.int32)
    ans, secs = H.gpu_query(ci.L, q, 4)
    assert np.array_equal(ans, orc.query(ref, q[:, 0], q[:, 1], q[:, 2]))


@pytest.mark.parametrize("tuning", [dict(block_threads=128), dict(block_threads=1024, prefetch_ahead=2),
                                    dict(block_threads=512, lanes_per_query=16), dict(block_threads=256,
                                                                                      lanes_per_query=8)])
def test_query_variants_agree(orc, tuning):
    """Every query kernel variant (block sizes, L2 prefetch of later rows,
    8/16/32 lanes per query) gives the same answers as the oracle."""
    g = H.HostGraph.chung_lu(6000, 8, 2.2, 600, 1, 100, seed=26)
    K = 5
    dev, idx = gpu_build(g, K)
    rng = np.random.default_rng(8)
    s = rng.integers(0, g.n, 50000).astype(np.int32)
    t = rng.integers(0, g.n, 50000).astype(np.int32)
    k = rng.integers(-1, K + 2, 50000).astype(np.int32)
    s[:100] = t[:100]
    base = idx.query(s, t, k)
    assert np.array_equal(base, orc.query(orc.build(g, K, threads=4), s, t, k, threads=4))
    idx.set_query_tuning(**tuning)
    assert np.array_equal(idx.query(s, t, k), base)
    assert idx.query_tuning()["block_threads"] == tuning["block_threads"]


def test_query_batch_rejects_vertices_outside_the_index():
    """hsdl_query_batch checks the vertex ids of a batch (on the device) and
    names the first query that is out of range."""
    g = H.HostGraph.erdos_renyi(500, 2000, 1, 50, seed=27)
    dev, idx = gpu_build(g, 4)
    s = np.arange(1000, dtype=np.int32) % g.n
    t = (np.arange(1000, dtype=np.int32) * 7) % g.n
    k = np.full(1000, 3, np.int32)
    ok = idx.query(s, t, k)
    assert ok.shape == (1000,)
    for bad_s, bad_t, at in ((g.n, 0, 417), (3, -1, 12), (-5, g.n + 9, 998)):
        s2, t2 = s.copy(), t.copy()
        s2[at], t2[at] = bad_s, bad_t
        with pytest.raises(H.HsdlError) as e:
            idx.query(s2, t2, k)
        assert f"at query {at}" in str(e.value)
    assert np.array_equal(idx.query(s, t, k), ok)  # the index is unaffected


@pytest.mark.parametrize("K,wmax", [(14, 19_000_000), (1, 250_000_000), (3, 80_000_000)])
def test_hop_bound_and_weight_limits(orc, K, wmax):
    """The largest hop bound (14) and weights near the 28-bit distance limit
    (K * max weight < 2^28): labels and answers still equal the oracle's."""
    g = H.HostGraph.erdos_renyi(400, 1600, max(1, wmax // 2), wmax, seed=K + 40)
    dev, idx = gpu_build(g, K)
    off, lab = idx.export()
    ref = orc.build(g, K, threads=1)
    assert np.array_equal(off, ref.off) and np.array_equal(lab, ref.lab)
    rng = np.random.default_rng(K)
    s = rng.integers(0, g.n, 20000).astype(np.int32)
    t = rng.integers(0, g.n, 20000).astype(np.int32)
    k = rng.integers(0, K + 2, 20000).astype(np.int32)
    got = idx.query(s, t, k)
    assert np.array_equal(got, orc.query(ref, s, t, k))
    assert lab[:, 3].max() < (1 << 28)  # each label's distance fits its 28-bit field
    assert got[(got != 2147483647)].max() >= wmax // 2  # the answers do carry the large weights


def test_build_rejects_weights_past_the_distance_limit():
    g = H.HostGraph.erdos_renyi(100, 300, 100_000_000, 100_000_000, seed=3)
    dev = H.Graph(g)
    with pytest.raises(H.HsdlError):
        H.Index.build(dev, 3)  # 3 * 1e8 >= 2^28


@pytest.mark.parametrize("wmax,key_bytes", [(100, 4), (3_000_000, 8)])
def test_query_key_formats_agree_with_the_oracle(orc, wmax, key_bytes):
    """Indexes whose ranges fit get the compact 4-byte query keys (hub:H |
    hop:P | distance:D); wide distances keep the 8-byte keys.  Both joins
    answer exactly as the oracle."""
    g = H.HostGraph.erdos_renyi(3000, 12000, 1, wmax, seed=61)
    K = 5
    dev, idx = gpu_build(g, K)
    info = idx.info()
    assert info["query_key_bytes"] == key_bytes
    if key_bytes == 4:
        assert info["query_key_hub_bits"] == 12
    # each join format's default launch shape
    tun = idx.query_tuning()
    assert (tun["block_threads"], tun["prefetch_ahead"]) == ((1024, 0) if key_bytes == 4 else (512, 0))
    ref = orc.build(g, K, threads=1)
    rng = np.random.default_rng(wmax)
    s = rng.integers(0, g.n, 200000).astype(np.int32)
    t = rng.integers(0, g.n, 200000).astype(np.int32)
    k = rng.integers(-1, K + 2, 200000).astype(np.int32)
    assert np.array_equal(idx.query(s, t, k), orc.query(ref, s, t, k))
    idx.close()
    dev.close()


def test_compact_keys_at_a_power_of_two_vertex_count(orc):
    """With n = 4,096 the compact key's hub field holds 0..n (13 bits), so the
    all-ones end-of-row key reads as a hub above vertex 4,095, whose self
    label ends its own row; queries on the last vertices answer as the
    oracle's."""
    g = H.HostGraph.erdos_renyi(4096, 16000, 1, 100, seed=67)
    K = 4
    dev, idx = gpu_build(g, K)
    info = idx.info()
    assert info["query_key_bytes"] == 4 and info["query_key_hub_bits"] == 13
    ref = orc.build(g, K, threads=1)
    rng = np.random.default_rng(67)
    m = 100000
    s = rng.integers(0, g.n, m).astype(np.int32)
    t = rng.integers(0, g.n, m).astype(np.int32)
    s[: m // 4] = g.n - 1 - rng.integers(0, 4, m // 4)
    t[m // 4: m // 2] = g.n - 1
    k = rng.integers(0, K + 1, m).astype(np.int32)
    assert np.array_equal(idx.query(s, t, k), orc.query(ref, s, t, k))
    idx.close()
    dev.close()
