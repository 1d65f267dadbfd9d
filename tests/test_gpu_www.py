"""GPU parity of the 2023WWW generation (hsdl_build_opts.generation = 1;
_2023WWW_thread_function, CPU_HopHL/include/HBPLL/
hop_constrained_two_hop_labels_generation.h:226-370): the CUDA path through
the C ABI against the oracle's restatement and the reference's golden
fixtures.  Bit-exact on (hub, hop, distance); parent_vertex is pinned by
validity, because the reference keeps the first of several equal-distance
predecessors in its processing order and the GPU the smallest id.

* uncleaned GPU labels == oracle 2023WWW generation with the same wave
  schedule, up to the reference's duplicate labels;
* cleaned GPU labels == the reference's cleaned 2023WWW labels == the HSDL
  canonical labels;
* the clean of an imported 2023WWW superset (hubs ranked below their vertex
  in the rows) == the canonical labels.
"""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H

pytestmark = pytest.mark.gpu


def rows_hhd(off, lab):
    """Distinct (vertex, hub, hop, distance) tuples, sorted."""
    v = np.repeat(np.arange(len(off) - 1), np.diff(off))
    return np.unique(np.column_stack([v, lab[:, 0], lab[:, 2], lab[:, 3]]), axis=0)


def check_parents(g, off, lab):
    """Every label (hub, p, h, d) of v with h > 0 names a neighbour p of v
    that holds the label (hub, h - 1, d - w(p, v)) in the same label set."""
    have = {tuple(x) for x in rows_hhd(off, lab).tolist()}
    vert = np.repeat(np.arange(g.n), np.diff(off))
    for v, (hub, p, h, d) in zip(vert, lab):
        if h == 0:
            assert hub == v and p == v and d == 0
            continue
        row = g.col[g.row_ptr[v]:g.row_ptr[v + 1]]
        j = np.searchsorted(row, p)
        assert j < len(row) and row[j] == p
        w = int(g.w[g.row_ptr[v] + j])
        assert (int(p), int(hub), int(h) - 1, int(d) - w) in have


@pytest.mark.parametrize("max_wave", [1, 4, 64, 0])
def test_www_uncleaned_matches_wave_oracle(orc, max_wave):
    g = H.HostGraph.chung_lu(2000, 8, 2.2, 200, 1, 100, seed=21)
    K = 5
    dev = H.Graph(g)
    idx = H.Index.build(dev, K, clean=False, max_wave=max_wave, generation=1)
    off, lab = idx.export()
    b = H.wave_bounds(g.n, max_wave=max_wave)
    ref = orc.build(g, K, threads=4, wave_bounds=b, clean=False, www=True)
    assert np.array_equal(rows_hhd(off, lab), rows_hhd(ref.off, ref.lab))
    assert len(lab) == len(rows_hhd(off, lab))  # no duplicates on the GPU
    check_parents(g, off, lab)
    hsdl = H.Index.build(dev, K, clean=False, max_wave=max_wave)
    if max_wave != 1:
        # no rank prune: more labels before the clean (with waves of one hub,
        # the run the reference makes, the distinct labels can be the same set)
        assert len(lab) > hsdl.info()["labels"]
    idx.clean()
    off2, lab2 = idx.export()
    canon = orc.build(g, K, threads=1)
    assert np.array_equal(off2, canon.off)
    assert np.array_equal(lab2[:, [0, 2, 3]], canon.lab[:, [0, 2, 3]])


def test_www_golden(golden_www):
    """Against the reference's own 2023WWW outputs: the sequential run (waves
    of one hub) before the clean, and the default build after it."""
    g, K, d = golden_www.g, golden_www.K, golden_www.d
    dev = H.Graph(g)
    seq = H.Index.build(dev, K, clean=False, first_wave=1, max_wave=1, generation=1)
    off, lab = seq.export()
    assert np.array_equal(rows_hhd(off, lab), rows_hhd(d["raw_off"], d["raw_labels"]))
    idx = H.Index.build(dev, K, generation=1)
    off, lab = idx.export()
    assert np.array_equal(off, d["off"])
    assert np.array_equal(lab[:, [0, 2, 3]], d["labels"][:, [0, 2, 3]])
    # the reference's own labels before its clean (repeats included), cleaned
    # by hsdl_clean: all four fields equal the reference's clean
    imp = H.Index.import_labels(g.n, K, d["raw_off"], d["raw_labels"])
    imp.clean()
    off, lab = imp.export()
    assert np.array_equal(off, d["off"]) and np.array_equal(lab, d["labels"])


def test_www_queries_and_paths(orc):
    g = H.HostGraph.erdos_renyi(400, 1600, 1, 100, seed=9)
    K = 5
    dev = H.Graph(g)
    www = H.Index.build(dev, K, generation=1)
    hsdl = H.Index.build(dev, K)
    rng = np.random.default_rng(3)
    s = rng.integers(0, g.n, 20000).astype(np.int32)
    t = rng.integers(0, g.n, 20000).astype(np.int32)
    k = rng.integers(-1, K + 2, 20000).astype(np.int32)
    assert np.array_equal(www.query(s, t, k), hsdl.query(s, t, k))
    wmap = {}
    for v in range(g.n):
        for e in range(g.row_ptr[v], g.row_ptr[v + 1]):
            wmap[(v, int(g.col[e]))] = int(g.w[e])
    for i in range(200):
        # paths within the index's hop bound: past K the labels need not
        # cover every walk, and a path may then beat the joined answer
        a, b, kk = int(s[i]), int(t[i]), int(np.clip(k[i], 1, K))
        p = www.path(a, b, kk)
        dist = int(www.query([a], [b], [kk])[0])
        if a == b or dist == 2147483647:
            assert p == []
        else:
            assert sum(wmap[e] for e in p) == dist and len(p) <= kk


def test_clean_of_imported_www_superset(orc):
    """hsdl_clean on an imported 2023WWW superset: no wave record, rows that
    hold hubs ranked below their vertex and repeated labels; only hubs ranked
    above a label's hub are witnesses, repeats are dropped, and the result is
    canonical."""
    g = H.HostGraph.erdos_renyi(800, 4000, 1, 50, seed=5)
    K = 5
    b = [0, 1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 800]
    sup = orc.build(g, K, threads=4, wave_bounds=b, clean=False, www=True)
    vert = np.repeat(np.arange(g.n), np.diff(sup.off))
    assert (sup.lab[:, 0] > vert).any()
    assert len(rows_hhd(sup.off, sup.lab)) < len(sup.lab)  # repeated labels, as the reference writes them
    idx = H.Index.import_labels(g.n, K, sup.off, sup.lab)
    idx.clean()
    off, lab = idx.export()
    canon = orc.build(g, K, threads=1)
    assert np.array_equal(off, canon.off)
    assert np.array_equal(lab[:, [0, 2, 3]], canon.lab[:, [0, 2, 3]])


def test_www_batched_and_case_info(orc):
    graphs = [H.HostGraph.erdos_renyi(300 + 50 * i, 1200 + 200 * i, 1, 100, seed=60 + i) for i in range(6)]
    Ks = [3, 4, 5, 6, 4, 5]
    idxs = H.Index.build_batched(graphs, Ks, generation=1)
    for g, K, ix in zip(graphs, Ks, idxs):
        off, lab = ix.export()
        canon = orc.build(g, K, threads=1)
        assert np.array_equal(off, canon.off)
        assert np.array_equal(lab[:, [0, 2, 3]], canon.lab[:, [0, 2, 3]])
    g = graphs[0]
    ci = H.hop_constrained_case_info(upper_k=4, use_2023WWW_generation=True)
    H.hop_constrained_two_hop_labels_generation(g, ci)
    canon = orc.build(g, 4, threads=1)
    assert ci.L.total() == len(canon.lab)
    assert ci.label_size_before_canonical_repair > ci.label_size_after_canonical_repair
    for v in (0, 7, g.n - 1):
        assert np.array_equal(ci.L[v][:, [0, 2, 3]], canon.row(v)[:, [0, 2, 3]])


@pytest.mark.parametrize("case", ["path_k1", "two_components", "single_vertex", "unit_ties_k6"])
def test_www_edge_cases(orc, case):
    if case == "path_k1":
        g, K = H.HostGraph.from_edges(6, [0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [3, 1, 4, 1, 5], rank_by_degree=True), 1
    elif case == "two_components":
        g, K = H.HostGraph.from_edges(10, [0, 1, 2, 5, 6], [1, 2, 3, 6, 7], [3, 1, 4, 1, 5], rank_by_degree=True), 3
    elif case == "single_vertex":
        g, K = H.HostGraph.from_edges(1, [], [], [], rank_by_degree=False), 2
    else:
        g, K = H.HostGraph.erdos_renyi(120, 360, 1, 1, seed=44), 6
    idx = H.Index.build(H.Graph(g), K, generation=1)
    off, lab = idx.export()
    canon = orc.build(g, K, threads=1)
    assert np.array_equal(off, canon.off)
    assert np.array_equal(lab[:, [0, 2, 3]], canon.lab[:, [0, 2, 3]])
