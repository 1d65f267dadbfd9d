"""hsdl_query_batch_static: the query entry point that allocates no device
memory.  It is for callers that must not call cudaMalloc: a thread answering
queries next to a running serving loop or build (cudaMalloc/cudaFree can
synchronise the device and stall those kernels), or a process whose device
memory is owned by another allocator with a hard cap.  It stages queries and
answers in a fixed library-owned device array.

These tests call it through the C ABI: twice in a row against the allocating
entry point hsdl_query_batch (integer answers: exact), after a failure
injected on the host once work is queued (the lock must not be released while
that work can still touch the shared array), with ids outside the index, and
against the device's memory accounting (no allocation, transient or held).  Collected last so a
stop-at-first-failure run has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture(scope="module")
def index(built):
    import gpu4hophl_code_gb300 as H
    from gpu4hophl_code_gb300 import _native

    # set-up before anything else runs on the device
    assert built.hsdl_query_static_prepare() == 0, _native.last_error()
    g = H.HostGraph.chung_lu(20000, 8, 2.2, 500, 1, 100, seed=31)
    dev = H.Graph(g)
    idx = H.Index.build(dev, 5)
    yield g, idx
    idx.close()
    dev.close()


def _batch(rng, n, nq):
    s = rng.integers(0, n, nq).astype(np.int32)
    t = rng.integers(0, n, nq).astype(np.int32)
    k = rng.integers(-1, 7, nq).astype(np.int32)
    return s, t, k


def test_static_staging_matches_allocating_query(built, index):
    from gpu4hophl_code_gb300 import _native

    g, idx = index
    fn = built.hsdl_query_batch_static
    rng = np.random.default_rng(5)
    # two calls in a row; the second is smaller so stale entries of the first
    # would show up if the staging array were read past nq
    for nq in (300_000, 123_457):
        s, t, k = _batch(rng, g.n, nq)
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


def test_failure_after_queued_work_leaves_the_next_call_correct(built, index):
    from gpu4hophl_code_gb300 import _native

    g, idx = index
    fn = built.hsdl_query_batch_static
    rng = np.random.default_rng(6)
    s, t, k = _batch(rng, g.n, 1 << 20)
    out = np.zeros(len(s), np.int32)
    assert built.hsdl_debug_inject_failure(1, 1) == 0
    rc = fn(idx.handle, len(s), _p(s), _p(t), _p(k), _p(out))
    assert rc == _native.HSDL_ERR_CUDA and "injected failure" in _native.last_error()
    s2, t2, k2 = _batch(rng, g.n, 200_000)
    got = np.zeros(len(s2), np.int32)
    assert fn(idx.handle, len(s2), _p(s2), _p(t2), _p(k2), _p(got)) == 0, _native.last_error()
    assert np.array_equal(got, idx.query(s2, t2, k2))


def test_ids_outside_the_index_are_rejected(built, index):
    from gpu4hophl_code_gb300 import _native

    g, idx = index
    fn = built.hsdl_query_batch_static
    s = np.array([0, 1, g.n, 2], np.int32)
    t = np.array([1, 2, 3, -1], np.int32)
    k = np.full(4, 3, np.int32)
    out = np.zeros(4, np.int32)
    rc = fn(idx.handle, 4, _p(s), _p(t), _p(k), _p(out))
    assert rc == _native.HSDL_ERR_INVALID and "out of range at query 2" in _native.last_error()


def test_calls_allocate_no_device_memory(built, index):
    """Two calls leave the default memory pool's high-water mark (every
    stream-ordered allocation of the library draws from it) and the device's
    free memory exactly as they were; the allocating entry point moves the
    mark, which shows the check sees such allocations."""
    import torch

    from gpu4hophl_code_gb300 import _native

    g, idx = index
    fn = built.hsdl_query_batch_static
    rng = np.random.default_rng(7)
    s, t, k = _batch(rng, g.n, 400_000)
    got = np.zeros(len(s), np.int32)
    assert fn(idx.handle, len(s), _p(s), _p(t), _p(k), _p(got)) == 0, _native.last_error()  # warm
    torch.cuda.synchronize()
    hw = C.c_int64()
    assert built.hsdl_debug_pool_used_high(C.byref(hw), 1) == 0, _native.last_error()
    base = hw.value
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert fn(idx.handle, len(s), _p(s), _p(t), _p(k), _p(got)) == 0, _native.last_error()
    assert built.hsdl_debug_pool_used_high(C.byref(hw), 0) == 0
    assert hw.value == base
    assert torch.cuda.mem_get_info()[0] == free0
    want = idx.query(s, t, k)  # hsdl_query_batch: stages in a stream-ordered allocation
    assert np.array_equal(got, want)
    assert built.hsdl_debug_pool_used_high(C.byref(hw), 0) == 0
    assert hw.value >= base + 16 * len(s)
