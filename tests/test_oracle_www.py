"""The 2023WWW generation (_2023WWW_thread_function,
CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:226-370,
selected by use_2023WWW_generation at :568-574): the oracle's restatement
against the reference's own outputs - the golden fixtures under
tests/golden/www/, and the compiled reference where it exists.  CPU only."""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H
from oracle.oracle import Reference


def test_oracle_www_matches_reference_golden(golden_www, orc):
    """Sequential run (one thread, rank order): the labels before the clean
    equal the reference's in all four fields, duplicates included (a vertex
    listed twice in Vh[h] is labelled twice, :276-336), and so do the cleaned
    labels."""
    g, K, d = golden_www.g, golden_www.K, golden_www.d
    raw = orc.build(g, K, threads=1, clean=False, www=True)
    assert np.array_equal(raw.off, d["raw_off"]) and np.array_equal(raw.lab, d["raw_labels"])
    cln = orc.build(g, K, threads=1, clean=True, www=True)
    assert np.array_equal(cln.off, d["off"]) and np.array_equal(cln.lab, d["labels"])


def test_www_and_hsdl_clean_to_the_same_labels(golden_www, orc):
    """The two searches differ before the clean (no rank prune: more labels)
    and agree on (hub, hop, distance) after."""
    g, K, d = golden_www.g, golden_www.K, golden_www.d
    hsdl = orc.build(g, K, threads=1)
    assert np.array_equal(hsdl.off, d["off"])
    assert np.array_equal(hsdl.lab[:, [0, 2, 3]], d["labels"][:, [0, 2, 3]])
    assert len(d["raw_labels"]) > len(d["labels"])


@pytest.mark.parametrize("schedule", ["ones", "doubling", "one_wave"])
def test_www_wave_mode_cleans_to_the_reference(golden_www, orc, schedule):
    """Wave mode (hubs of a wave see only earlier waves' labels, as on the GPU)
    gives a superset that the clean reduces to the reference's labels when
    every vertex is checked against the uncleaned rows of its hubs (clean mode
    1, the form the GPU clean follows).  The reference's in-place schedule
    (mode 0: rows of higher-ranked vertices already cleaned) is exact only on
    the sequential run: on a wave superset of this search it can keep labels
    whose only witness was dropped from the hub's row first."""
    g, K, d = golden_www.g, golden_www.K, golden_www.d
    if schedule == "ones":
        b = np.arange(g.n + 1, dtype=np.int32)
    elif schedule == "doubling":
        b = H.wave_bounds(g.n, first_wave=1, max_wave=64)
    else:
        b = np.array([0, g.n], np.int32)
    raw = orc.build(g, K, threads=3, wave_bounds=b, clean=False, www=True)
    if schedule == "ones":
        # waves of one hub are the sequential run, up to the duplicates
        want = np.unique(np.column_stack([np.repeat(np.arange(g.n), np.diff(d["raw_off"])), d["raw_labels"]]), axis=0)
        got = np.unique(np.column_stack([np.repeat(np.arange(g.n), np.diff(raw.off)), raw.lab]), axis=0)
        assert np.array_equal(got, want)
    cln = orc.clean(raw, K, threads=2, mode=1)
    assert np.array_equal(cln.off, d["off"])
    assert np.array_equal(cln.lab[:, [0, 2, 3]], d["labels"][:, [0, 2, 3]])
    if schedule == "ones":
        seq = orc.clean(raw, K, threads=1, mode=0)
        assert np.array_equal(seq.off, d["off"])


@pytest.mark.skipif(not Reference.available, reason="the reference checkout is not present")
def test_oracle_www_matches_compiled_reference(orc):
    """On graphs beyond the fixtures, against the reference compiled in place."""
    ref = Reference()
    for g, K in [(H.HostGraph.erdos_renyi(400, 1600, 1, 50, seed=41), 4),
                 (H.HostGraph.barabasi_albert(500, 3, 1, 1000, seed=42), 6),
                 (H.HostGraph.chung_lu(800, 6, 2.2, 100, 1, 100, seed=43), 5)]:
        r = ref.build(g, K, threads=1, clean=False, www=True)
        o = orc.build(g, K, threads=1, clean=False, www=True)
        assert np.array_equal(r.off, o.off) and np.array_equal(r.lab, o.lab)
        r = ref.build(g, K, threads=1, clean=True, www=True)
        o = orc.build(g, K, threads=1, clean=True, www=True)
        assert np.array_equal(r.off, o.off) and np.array_equal(r.lab, o.lab)


@pytest.mark.parametrize("case", ["path_k1", "two_components", "single_vertex", "unit_ties_k6", "star_k2"])
def test_www_edge_cases(orc, case):
    """Small and degenerate graphs: the 2023WWW search cleans to the HSDL
    labels, and (where the reference is compiled here) equals the reference
    before and after the clean."""
    if case == "path_k1":
        g, K = H.HostGraph.from_edges(6, [0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [3, 1, 4, 1, 5], rank_by_degree=True), 1
    elif case == "two_components":
        g, K = H.HostGraph.from_edges(10, [0, 1, 2, 5, 6], [1, 2, 3, 6, 7], [3, 1, 4, 1, 5], rank_by_degree=True), 3
    elif case == "single_vertex":
        g, K = H.HostGraph.from_edges(1, [], [], [], rank_by_degree=False), 2
    elif case == "unit_ties_k6":
        g, K = H.HostGraph.erdos_renyi(120, 360, 1, 1, seed=44), 6
    else:
        g, K = H.HostGraph.from_edges(9, [0] * 8, list(range(1, 9)), [2, 7, 1, 8, 2, 8, 1, 8]), 2
    hsdl = orc.build(g, K, threads=1)
    www = orc.build(g, K, threads=1, www=True)
    assert np.array_equal(www.off, hsdl.off)
    assert np.array_equal(www.lab[:, [0, 2, 3]], hsdl.lab[:, [0, 2, 3]])
    if Reference.available:
        ref = Reference()
        for clean in (False, True):
            r = ref.build(g, K, threads=1, clean=clean, www=True)
            o = orc.build(g, K, threads=1, clean=clean, www=True)
            assert np.array_equal(r.off, o.off) and np.array_equal(r.lab, o.lab)
