"""Label-propagation grouping (generate_Group_CDLP,
Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20): the oracle's
deterministic restatement on the CPU, and the GPU kernels against it.

The reference's propagation (CDLP_GPU) caps groups with racy atomics, so only
its second half - the group assembly (CDLP_group.cuh:39-100: bucketing by
label, greedy merge of small groups, ordering by total degree) - is
deterministic and can be pinned: the oracle's assembly is compared with the
reference's own code on fixed propagation labels, through a committed fixture
(tests/golden/lp/assembly.npz, made by tests/golden/make_golden.py) and, where
the reference is compiled here, live."""
import os

import numpy as np
import pytest

import gpu4hophl_code_gb300 as H
from conftest import GOLDEN

LP_FIXTURE = os.path.join(GOLDEN, "lp", "assembly.npz")


def _lp_cases():
    z = np.load(LP_FIXTURE)
    for gseed in (0, 1):
        g = H.HostGraph.chung_lu(3000, 8, 2.2, 300, 1, 100, seed=gseed)
        for gmax in (1, 5, 64, 1024):
            key = f"g{gseed}_m{gmax}"
            yield g, gmax, z[key + "_labels"], z[key + "_gov"]


def test_assembly_matches_the_reference_fixture(orc):
    n = 0
    for g, gmax, lab, want in _lp_cases():
        gov, ng = orc.lp_assemble(g, lab, gmax)
        assert ng == int(want.max()) + 1
        assert np.array_equal(gov, want), (gmax, ng)
        n += 1
    assert n == 8


def test_assembly_matches_the_reference_live(orc):
    from oracle.oracle import ReferenceLP

    if not ReferenceLP.available:
        pytest.skip("the reference's group assembly is not compiled here")
    R = ReferenceLP()
    rng = np.random.default_rng(3)
    for seed in range(4):
        g = H.HostGraph.barabasi_albert(2000, 3, 1, 100, seed=seed)
        for gmax in (2, 17, 300):
            # propagation labels: the oracle's own grouping at another cap,
            # and random groups
            lab = orc.lp_group(g, max(1, gmax // 2), 20)[0]
            for labels in (lab, rng.integers(0, g.n, g.n).astype(np.int32)):
                a = orc.lp_assemble(g, labels, gmax)
                b = R.assemble(g, labels, gmax)
                assert a[1] == b[1] and np.array_equal(a[0], b[0])


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
