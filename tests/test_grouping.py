"""Label-propagation grouping (generate_Group_CDLP,
Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20): the oracle's
deterministic restatement on the CPU, and the GPU kernels against it."""
import numpy as np
import pytest

import gpu4hophl_code_gb300 as H


def _graphs():
    return [H.HostGraph.chung_lu(8000, 8, 2.2, 800, 1, 100, seed=81),
            H.HostGraph.erdos_renyi(3000, 9000, 1, 100, seed=82),
            H.HostGraph.barabasi_albert(5000, 3, 1, 100, seed=83),
            H.HostGraph.from_edges(50, [0, 1, 2, 10], [1, 2, 3, 11], [1, 1, 1, 1]),
            # rows of several thousand neighbours: past the shared-memory table of the long-row kernel
            H.HostGraph.chung_lu(20000, 8, 2.1, 5000, 1, 100, seed=84)]


@pytest.mark.parametrize("gmax", [1, 7, 64, 1024])
def test_oracle_grouping_properties(orc, gmax):
    for g in _graphs():
        gov, ng, it = orc.lp_group(g, gmax, 50)
        sizes = np.bincount(gov, minlength=ng)
        assert sizes.sum() == g.n and len(sizes) == ng
        assert sizes.max() <= gmax and sizes.min() >= 1
        # groups come ordered by total degree, largest first
        deg = np.diff(g.row_ptr)
        tot = np.bincount(gov, weights=deg, minlength=ng)
        assert np.all(tot[:-1] >= tot[1:])
        again = orc.lp_group(g, gmax, 50)
        assert np.array_equal(again[0], gov)  # deterministic


def test_oracle_greedy_merge_leaves_no_mergeable_pair(orc):
    g = H.HostGraph.chung_lu(6000, 6, 2.3, 300, 1, 100, seed=84)
    gmax = 256
    gov, ng, _ = orc.lp_group(g, gmax, 30)
    sizes = np.sort(np.bincount(gov, minlength=ng))
    # the largest emitted groups are emitted only when nothing else fits, so
    # the two smallest groups cannot fit together
    assert ng == 1 or sizes[0] + sizes[1] > gmax


@pytest.mark.gpu
@pytest.mark.parametrize("gmax,iters", [(1024, 100), (64, 20), (5, 10), (1024, 1), (3000, 2)])
def test_gpu_grouping_matches_oracle(orc, gmax, iters):
    for g in _graphs():
        dev = H.Graph(g)
        gov, ng, it = H.group_lp(dev, gmax, iters)
        ref = orc.lp_group(g, gmax, iters)
        assert (ng, it) == (ref[1], ref[2])
        assert np.array_equal(gov, ref[0])


@pytest.mark.gpu
def test_reference_shaped_grouping(orc):
    g = H.HostGraph.chung_lu(5000, 8, 2.2, 500, 1, 100, seed=85)
    groups = []
    H.generate_Group_CDLP(g, groups, 1024)
    gov, ng, _ = orc.lp_group(g, 1024, 100)
    assert len(groups) == ng
    for i, grp in enumerate(groups):
        assert np.all(gov[np.asarray(grp)] == i)
