"""Device graph construction: degree ranking and CSR built on the GPU from an
edge list (hsdl_graph_create_from_edges) must equal the host path
(hsdl_host_graph_from_edges + hsdl_graph_create) bit for bit: the rank order,
the row offsets, and every row's (neighbour, weight) entries."""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H

pytestmark = pytest.mark.gpu


def _scrambled_edges(g, seed):
    """g's edges under a random relabelling, in random order and orientation."""
    rng = np.random.default_rng(seed)
    a, b, w = g.edges()
    perm = rng.permutation(g.n).astype(np.int32)
    a, b = perm[a], perm[b]
    order = rng.permutation(len(a))
    a, b, w = a[order], b[order], w[order]
    flip = rng.random(len(a)) < 0.5
    a2 = np.where(flip, b, a).astype(np.int32)
    b2 = np.where(flip, a, b).astype(np.int32)
    return a2, b2, w.astype(np.int32)


@pytest.mark.parametrize("kind", ["er", "cl", "ba"])
@pytest.mark.parametrize("rank", [True, False])
def test_device_ranking_and_csr_equal_host(kind, rank):
    g = {"er": lambda: H.HostGraph.erdos_renyi(3000, 12000, 1, 100, seed=31),
         "cl": lambda: H.HostGraph.chung_lu(20000, 8, 2.1, 2000, 1, 100, seed=32),
         "ba": lambda: H.HostGraph.barabasi_albert(5000, 3, 1, 1000, seed=33)}[kind]()
    a, b, w = _scrambled_edges(g, 7)
    host = H.HostGraph.from_edges(g.n, a, b, w, rank_by_degree=rank)
    dev = H.Graph.from_edges(g.n, a, b, w, rank_by_degree=rank)
    rp, col, wt = dev.csr()
    assert np.array_equal(rp, host.row_ptr)
    assert np.array_equal(col, host.col) and np.array_equal(wt, host.w)
    assert np.array_equal(dev.new_to_old, host.new_to_old)


def test_device_graph_builds_the_same_index():
    g = H.HostGraph.chung_lu(4000, 8, 2.2, 400, 1, 100, seed=34)
    a, b, w = _scrambled_edges(g, 8)
    host = H.HostGraph.from_edges(g.n, a, b, w)
    want = H.Index.build(H.Graph(host), 5).export()
    got = H.Index.build(H.Graph.from_edges(g.n, a, b, w), 5).export()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_device_graph_rejects_bad_edge_lists():
    a = np.array([0, 1, 2], np.int32)
    b = np.array([1, 2, 0], np.int32)
    w = np.array([3, 4, 5], np.int32)
    H.Graph.from_edges(3, a, b, w)  # a triangle is fine
    for aa, bb, ww in ((np.array([0, 1, 2]), np.array([1, 1, 0]), w),      # self loop
                       (np.array([0, 1, 2]), np.array([1, 3, 0]), w),      # id out of range
                       (np.array([0, 1, 2]), np.array([1, 2, 0]), np.array([3, 0, 5])),  # weight < 1
                       (np.array([0, 1, 1]), np.array([1, 2, 0]), w)):     # repeated edge
        with pytest.raises(H.HsdlError):
            H.Graph.from_edges(3, aa, bb, ww)
