"""hsdl_query_batch_static: the query entry point that allocates no device
memory (for callers that must not call cudaMalloc - e.g. next to a running
serving or build kernel, where cudaMalloc/cudaFree can synchronise the device,
or under another allocator's hard cap).  It stages queries and answers in a
fixed library-owned device array; this test calls it through the C ABI twice
in a row and compares with the allocating entry point hsdl_query_batch
(integer answers: exact).  Collected last so a stop-at-first-failure run has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_static_staging_matches_allocating_query(built):
    import gpu4hophl_code_gb300 as H
    from gpu4hophl_code_gb300 import _native

    fn = built.hsdl_query_batch_static
    g = H.HostGraph.chung_lu(20000, 8, 2.2, 500, 1, 100, seed=31)
    dev = H.Graph(g)
    idx = H.Index.build(dev, 5)
    rng = np.random.default_rng(5)
    # two calls in a row; the second is smaller so stale entries of the first
    # would show up if the staging array were read past nq
    for nq in (300_000, 123_457):
        s = rng.integers(0, g.n, nq).astype(np.int32)
        t = rng.integers(0, g.n, nq).astype(np.int32)
        k = rng.integers(-1, 7, nq).astype(np.int32)
        got = np.full(nq, -7, np.int32)
        rc = fn(idx.handle, nq, _p(s), _p(t), _p(k), _p(got))
        assert rc == 0, _native.last_error()
        want = idx.query(s, t, k)  # hsdl_query_batch (allocating)
        assert np.array_equal(got, want)
    # over the limit: rejected with a clear error, nothing touched
    big = (1 << 20) + 1
    one = np.zeros(1, np.int32)
    rc = fn(idx.handle, big, _p(one), _p(one), _p(one), _p(one))
    assert rc == _native.HSDL_ERR_INVALID
    assert "HSDL_STATIC_QUERY_MAX" in _native.last_error()
    idx.close()
    dev.close()
