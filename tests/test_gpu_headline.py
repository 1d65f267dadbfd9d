"""Parity at the benchmark's configurations, through the C ABI on the GPU.

* The 1,000-vertex Erdos-Renyi configuration (m = 5,000, weights [1, 100],
  K = 5) at its full query count: 100,000 uniform (s, t, k), k in [1, 5], every
  answer compared with hop-bounded Bellman-Ford (the reference's
  graph_v_of_v_hop_constrained_shortest_distance,
  CPU_HopHL/include/graph_v_of_v/graph_v_of_v_hop_constrained_shortest_distance.h:7-38,
  restated in the oracle) - the check of
  hop_constrained_check_correctness (CPU_HopHL/include/HBPLL/test.h:60-134).
* The 1M-vertex Chung-Lu configuration (K = 5): the GPU's cleaned labels
  against the reference's own (sha256 of offsets and of the (hub, hop,
  distance) triples), its answers on 100,000 seeded queries and its
  Bellman-Ford distances on 20,000 sampled pairs
  (tests/golden/headline/chung_lu_1m_k5.npz, made by
  tests/golden/make_golden_1m.py from CPU_HopHL compiled in place).
"""
import os

import numpy as np
import pytest

import gpu4hophl_code_gb300 as H
from conftest import GOLDEN, GoldenCase

pytestmark = pytest.mark.gpu


def test_config1_100k_queries_against_bellman_ford(orc):
    case = GoldenCase(os.path.join(GOLDEN, "er_1000_5000_k5.npz"))
    g, K = case.g, case.K
    assert (g.n, g.num_edges, K) == (1000, 5000, 5)
    dev = H.Graph(g)
    idx = H.Index.build(dev, K)
    off, lab = idx.export()
    import bench

    assert bench.label_digests(off, lab)["hhd"] == str(case.d["hhd_digest"])
    rng = np.random.default_rng(0x48534C44 ^ 1)
    s = rng.integers(0, g.n, 100_000).astype(np.int32)
    t = rng.integers(0, g.n, 100_000).astype(np.int32)
    k = rng.integers(1, K + 1, 100_000).astype(np.int32)
    got = idx.query(s, t, k)
    # Bellman-Ford rows for every source and hop bound: dist[k - 1, s, t]
    dist = np.stack([np.stack([orc.bf(g, src, h) for src in range(g.n)]) for h in range(1, K + 1)])
    want = dist[k - 1, s, t]
    assert np.array_equal(got, want), int(np.count_nonzero(got != want))
    idx.close()
    dev.close()


def test_headline_1m_labels_and_answers_match_the_reference():
    import bench

    if not os.path.exists(bench.HEADLINE_FIXTURE):
        pytest.skip("headline fixture not generated")
    g = bench.make_graph(1_000_000)
    dev = H.Graph(g)
    idx = H.Index.build(dev, 5)
    off, lab = idx.export()
    par = bench.headline_parity(g, off, lab, idx.query)
    idx.close()
    dev.close()
    assert par is not None, "fixture made for another graph"
    assert par["labels"] == par["reference_labels"]
    assert par["labels_digest_match"], par
    assert par["reference_answer_mismatches"] == 0 and par["bf_mismatches"] == 0, par
