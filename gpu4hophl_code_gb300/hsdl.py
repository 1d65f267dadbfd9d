"""Python host API over libhsdl.

Two layers:

* Object API - ``HostGraph`` (seeded generators, ranked CSR on the host),
  ``Graph`` (CSR resident in HBM) and ``Index`` (labels resident in HBM:
  build, clean, query, export/import, save/load, path extraction).

* Reference-shaped API - the names, arguments and result fields of the
  reference's CPU entry points, so code written against
  CPU_HopHL/include/HBPLL/*.h reads the same:
  ``hop_constrained_case_info``, ``hop_constrained_two_hop_labels_generation``,
  ``hop_constrained_clean_L``, ``hop_constrained_extract_distance``,
  ``hop_constrained_extract_shortest_path``, ``gpu_query``.

Every compute call goes through the CUDA library; nothing here computes labels
or distances on the CPU.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import check, lib

INT_MAX = 2147483647


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# host graphs
# ---------------------------------------------------------------------------
class HostGraph:
    """Undirected weighted graph as a rank-ordered CSR (vertex 0 = highest rank)."""

    def __init__(self, n: int, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray,
                 new_to_old: np.ndarray | None = None):
        self.n = int(n)
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.w = np.ascontiguousarray(w, dtype=np.int32)
        self.new_to_old = (np.arange(n, dtype=np.int32) if new_to_old is None
                           else np.ascontiguousarray(new_to_old, dtype=np.int32))

    @property
    def num_edges(self) -> int:
        return int(self.row_ptr[-1]) // 2

    @staticmethod
    def _take(handle: C.c_void_p) -> "HostGraph":
        L = lib()
        n = C.c_int32()
        m2 = C.c_int64()
        rp, col, w, nto = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        try:
            check(L.hsdl_host_graph_get(handle, C.byref(n), C.byref(m2), C.byref(rp), C.byref(col), C.byref(w),
                                        C.byref(nto)))
            nn, mm = n.value, m2.value

            def arr(p, cnt, ct, dt):
                if cnt == 0:
                    return np.zeros(0, dt)
                return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(cnt,)).astype(dt, copy=True)

            return HostGraph(nn, arr(rp, nn + 1, C.c_int64, np.int64), arr(col, mm, C.c_int32, np.int32),
                             arr(w, mm, C.c_int32, np.int32), arr(nto, nn, C.c_int32, np.int32))
        finally:
            L.hsdl_host_graph_free(handle)

    @classmethod
    def erdos_renyi(cls, n: int, m: int, wmin: int = 1, wmax: int = 100, seed: int = 1) -> "HostGraph":
        h = C.c_void_p()
        check(lib().hsdl_gen_erdos_renyi(n, m, wmin, wmax, seed, C.byref(h)))
        return cls._take(h)

    @classmethod
    def chung_lu(cls, n: int, avg_degree: float, exponent: float, max_degree: float, wmin: int = 1,
                 wmax: int = 100, seed: int = 1) -> "HostGraph":
        h = C.c_void_p()
        check(lib().hsdl_gen_chung_lu(n, avg_degree, exponent, max_degree, wmin, wmax, seed, C.byref(h)))
        return cls._take(h)

    @classmethod
    def barabasi_albert(cls, n: int, m0: int, wmin: int = 1, wmax: int = 1000, seed: int = 1) -> "HostGraph":
        h = C.c_void_p()
        check(lib().hsdl_gen_barabasi_albert(n, m0, wmin, wmax, seed, C.byref(h)))
        return cls._take(h)

    @classmethod
    def from_edges(cls, n: int, a, b, w, rank_by_degree: bool = True) -> "HostGraph":
        a = np.ascontiguousarray(a, np.int32)
        b = np.ascontiguousarray(b, np.int32)
        w = np.ascontiguousarray(w, np.int32)
        h = C.c_void_p()
        check(lib().hsdl_host_graph_from_edges(n, len(a), _ptr(a), _ptr(b), _ptr(w), int(rank_by_degree),
                                                C.byref(h)))
        return cls._take(h)

    @classmethod
    def read_text(cls, path: str, rank_by_degree: bool = True) -> "HostGraph":
        h = C.c_void_p()
        check(lib().hsdl_read_graph_text(path.encode(), int(rank_by_degree), C.byref(h)))
        return cls._take(h)

    def validate(self) -> None:
        check(lib().hsdl_validate_csr(self.n, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.w)))

    def edges(self):
        """(a, b, w) with a < b, one entry per undirected edge."""
        src = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.row_ptr))
        m = src < self.col
        return src[m], self.col[m], self.w[m]


# ---------------------------------------------------------------------------
# device objects
# ---------------------------------------------------------------------------
class Graph:
    """CSR graph resident in HBM."""

    def __init__(self, g: "HostGraph | None"):
        self._h = C.c_void_p()
        self.new_to_old = None
        if g is None:  # filled by from_edges
            self.n, self.host = 0, None
            return
        self.n = g.n
        self.host = g
        check(lib().hsdl_graph_create(g.n, _ptr(g.row_ptr), _ptr(g.col), _ptr(g.w), C.byref(self._h)))

    @classmethod
    def from_edges(cls, n: int, a, b, w, rank_by_degree: bool = True) -> "Graph":
        """Device graph from an undirected simple edge list, ranked and laid out
        as CSR on the GPU (hsdl_graph_create_from_edges); `new_to_old` holds
        each ranked vertex's original id."""
        a = np.ascontiguousarray(a, np.int32)
        b = np.ascontiguousarray(b, np.int32)
        w = np.ascontiguousarray(w, np.int32)
        g = cls(None)
        g.n = n
        g.new_to_old = np.zeros(n, np.int32)
        check(lib().hsdl_graph_create_from_edges(n, len(a), _ptr(a), _ptr(b), _ptr(w), int(rank_by_degree),
                                                 _ptr(g.new_to_old), C.byref(g._h)))
        return g

    def csr(self):
        """(row_ptr int64[n+1], col int32[2m], w int32[2m]) copied from the device."""
        n = C.c_int32()
        adj = C.c_int64()
        check(lib().hsdl_graph_get_csr(self._h, C.byref(n), C.byref(adj), None, None, None))
        rp = np.zeros(n.value + 1, np.int64)
        col = np.zeros(max(1, adj.value), np.int32)
        w = np.zeros(max(1, adj.value), np.int32)
        check(lib().hsdl_graph_get_csr(self._h, None, None, _ptr(rp), _ptr(col), _ptr(w)))
        return rp, col[: adj.value], w[: adj.value]

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            lib().hsdl_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def group_lp(graph: Graph, max_group: int = 1024, max_iterations: int = 100):
    """generate_Group_CDLP (Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20):
    returns (group_of_vertex int32[n], number of groups, iterations run)."""
    gov = np.zeros(graph.n, np.int32)
    ng = C.c_int32()
    it = C.c_int32()
    check(lib().hsdl_group_lp(graph.handle, max_group, max_iterations, _ptr(gov), C.byref(ng), C.byref(it)))
    return gov, ng.value, it.value


def generate_Group_CDLP(instance_graph, groups: list, MAX_GROUP_SIZE: int, max_iterations: int = 100) -> None:
    """Reference-shaped form: fills `groups` with one list of vertex ids per
    group, groups ordered by total degree (largest first)."""
    g = instance_graph if isinstance(instance_graph, Graph) else Graph(instance_graph)
    gov, ng, _ = group_lp(g, MAX_GROUP_SIZE, max_iterations)
    order = np.argsort(gov, kind="stable")
    bounds = np.searchsorted(gov[order], np.arange(ng + 1))
    groups.clear()
    groups.extend(order[bounds[i]:bounds[i + 1]].tolist() for i in range(ng))


def build_opts(clean: bool = True, first_wave: int = 1, max_wave: int = 0, block_threads: int = 0,
               frontier_tile: int = 0, prune_lanes: int = 0, prune_pairs: int = 0, generation: int = 0,
               prune_order: int = 0, pool_key_bytes: int = 0, device_budget_bytes: int = 0) -> N.hsdl_build_opts:
    """generation: 0 = the HSDL search, 1 = the 2023WWW search (the
    reference's use_2023WWW_generation); the cleaned labels are the same.
    prune_order: 0 = each hop's candidates grouped by vertex range before the
    pruning join, 1 = expansion order (no label changes)."""
    o = N.hsdl_build_opts()
    lib().hsdl_build_opts_default(C.byref(o))
    o.clean = int(clean)
    o.first_wave = first_wave
    o.max_wave = max_wave
    o.block_threads = block_threads
    o.frontier_tile = frontier_tile
    o.prune_lanes = prune_lanes
    o.prune_pairs = prune_pairs
    o.generation = generation
    o.prune_order = prune_order
    o.pool_key_bytes = pool_key_bytes
    o.device_budget_bytes = device_budget_bytes
    return o


_TUNABLES = ("max_wave", "block_threads", "frontier_tile", "prune_lanes", "prune_pairs")


def autotune_build(graph: "Graph", K: int, sample_hubs: int = 0, **opts) -> dict:
    """Fastest launch shapes for building this graph (hsdl_build_autotune):
    a dict of max_wave, block_threads, frontier_tile, prune_lanes to pass to
    Index.build, plus 'seconds' (the sample's time) and 'trials'."""
    o = build_opts(**opts)
    best = C.c_double()
    n_trials = C.c_int32()
    check(lib().hsdl_build_autotune(graph.handle, K, sample_hubs, C.byref(o), C.byref(best), C.byref(n_trials)))
    r = {f: getattr(o, f) for f in _TUNABLES}
    r.update(seconds=best.value, trials=n_trials.value)
    return r


def autotune_build_batched(graphs, Ks, sample_graphs: int = 0, **opts) -> dict:
    """Same for Index.build_batched (hsdl_build_batched_autotune)."""
    B = len(graphs)
    n = np.array([g.n for g in graphs], np.int32)
    K = np.array(Ks, np.int32)
    rps = (C.c_void_p * B)(*[g.row_ptr.ctypes.data for g in graphs])
    cols = (C.c_void_p * B)(*[g.col.ctypes.data for g in graphs])
    ws = (C.c_void_p * B)(*[g.w.ctypes.data for g in graphs])
    o = build_opts(**opts)
    best = C.c_double()
    n_trials = C.c_int32()
    check(lib().hsdl_build_batched_autotune(B, _ptr(n), C.cast(rps, C.c_void_p), C.cast(cols, C.c_void_p),
                                            C.cast(ws, C.c_void_p), _ptr(K), sample_graphs, C.byref(o),
                                            C.byref(best), C.byref(n_trials)))
    r = {f: getattr(o, f) for f in _TUNABLES}
    r.update(seconds=best.value, trials=n_trials.value)
    return r


def wave_bounds(n: int, **opts) -> np.ndarray:
    o = build_opts(**opts)
    cnt = C.c_int32()
    check(lib().hsdl_wave_bounds(n, C.byref(o), None, 0, C.byref(cnt)))
    b = np.zeros(cnt.value, np.int32)
    check(lib().hsdl_wave_bounds(n, C.byref(o), _ptr(b), len(b), C.byref(cnt)))
    return b


class Index:
    """Label index resident in HBM."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def build(cls, graph: Graph, K: int, **opts) -> "Index":
        o = build_opts(**opts)
        h = C.c_void_p()
        check(lib().hsdl_build(graph.handle, K, C.byref(o), C.byref(h)))
        return cls(h)

    @classmethod
    def build_batched(cls, graphs, Ks, **opts) -> list:
        """Indexes many host graphs together (hsdl_build_batched); one Index per graph."""
        B = len(graphs)
        n = np.array([g.n for g in graphs], np.int32)
        K = np.array(Ks, np.int32)
        rps = (C.c_void_p * B)(*[g.row_ptr.ctypes.data for g in graphs])
        cols = (C.c_void_p * B)(*[g.col.ctypes.data for g in graphs])
        ws = (C.c_void_p * B)(*[g.w.ctypes.data for g in graphs])
        outs = (C.c_void_p * B)()
        o = build_opts(**opts)
        check(lib().hsdl_build_batched(B, _ptr(n), C.cast(rps, C.c_void_p), C.cast(cols, C.c_void_p),
                                       C.cast(ws, C.c_void_p), _ptr(K), C.byref(o), C.cast(outs, C.c_void_p)))
        return [cls(C.c_void_p(outs[i])) for i in range(B)]

    @classmethod
    def import_labels(cls, n: int, K: int, offsets: np.ndarray, labels: np.ndarray) -> "Index":
        offsets = np.ascontiguousarray(offsets, np.int64)
        labels = np.ascontiguousarray(labels, np.int32).reshape(-1, 4)
        h = C.c_void_p()
        check(lib().hsdl_import(n, K, _ptr(offsets), _ptr(labels) if len(labels) else None, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str, K: int) -> "Index":
        h = C.c_void_p()
        check(lib().hsdl_load_labels(path.encode(), K, C.byref(h)))
        return cls(h)

    @property
    def handle(self):
        return self._h

    def clean(self) -> "Index":
        check(lib().hsdl_clean(self._h))
        return self

    def info(self) -> dict:
        i = N.hsdl_index_info()
        check(lib().hsdl_index_get_info(self._h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in N.hsdl_index_info._fields_}

    def export(self):
        """(offsets int64[n+1], labels int32[total, 4]) in the reference record
        layout (hub_vertex, parent_vertex, hop, distance)."""
        info = self.info()
        off = np.zeros(info["n"] + 1, np.int64)
        lab = np.zeros((max(1, info["labels"]), 4), np.int32)
        check(lib().hsdl_export(self._h, _ptr(off), _ptr(lab)))
        return off, lab[: info["labels"]]

    def query(self, s, t, k) -> np.ndarray:
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        out = np.zeros(len(s), np.int32)
        check(lib().hsdl_query_batch(self._h, len(s), _ptr(s), _ptr(t), _ptr(k), _ptr(out)))
        return out

    def query_device(self, nq: int, d_s: int, d_t: int, d_k: int, d_out: int, stream: int = 0) -> None:
        """Device pointers (e.g. torch tensor data_ptr()); asynchronous on `stream`."""
        check(lib().hsdl_query_batch_device(self._h, nq, C.c_void_p(d_s), C.c_void_p(d_t), C.c_void_p(d_k),
                                            C.c_void_p(d_out), C.c_void_p(stream) if stream else None))

    def loadgen(self, s, t, k, offered_qps: float, window_us: float = 0.0, seed: int = 1, answers=None,
                max_batch: int = 0) -> dict:
        """The plain path (hsdl_query_batch) under an open-loop Poisson stream
        of rate offered_qps, batched by arrival window (hsdl_query_loadgen).
        Pass pinned host arrays (e.g. torch pin_memory().numpy()) for a fair
        rate; `answers` (int32, len(s)) receives the answers."""
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        ans = np.zeros(len(s), np.int32) if answers is None else answers
        o = N.hsdl_query_loadgen_opts()
        o.struct_size = C.sizeof(N.hsdl_query_loadgen_opts)
        o.n = len(s)
        o.s, o.t, o.k, o.answers = s.ctypes.data, t.ctypes.data, k.ctypes.data, ans.ctypes.data
        o.offered_qps = offered_qps
        o.seed = seed
        o.window_us = window_us
        o.max_batch = max_batch
        r = N.hsdl_loadgen_result()
        check(lib().hsdl_query_loadgen(self._h, C.byref(o), C.byref(r)))
        res = {f: getattr(r, f) for f, _ in N.hsdl_loadgen_result._fields_}
        res["answers"] = ans
        return res

    def path(self, s: int, t: int, k: int, cap: int = 64):
        e = np.zeros((cap, 2), np.int32)
        cnt = C.c_int32()
        check(lib().hsdl_extract_path(self._h, s, t, k, _ptr(e), cap, C.byref(cnt)))
        return [tuple(x) for x in e[: cnt.value].tolist()]

    def set_query_tuning(self, block_threads: int = 512, prefetch_ahead: int = 0, lanes_per_query: int = 32) -> None:
        t = N.hsdl_query_tuning(C.sizeof(N.hsdl_query_tuning), block_threads, prefetch_ahead, lanes_per_query)
        check(lib().hsdl_set_query_tuning(self._h, C.byref(t)))

    def query_tuning(self) -> dict:
        t = N.hsdl_query_tuning()
        check(lib().hsdl_get_query_tuning(self._h, C.byref(t)))
        return {"block_threads": t.block_threads, "prefetch_ahead": t.prefetch_ahead,
                "lanes_per_query": t.lanes_per_query}

    def save(self, path: str) -> None:
        check(lib().hsdl_save_labels(self._h, path.encode()))

    def close(self) -> None:
        if self._h:
            lib().hsdl_index_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Reference-shaped API (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h
# and hop_constrained_two_hop_labels_generation.h)
# ---------------------------------------------------------------------------
class LabelLists:
    """Per-vertex label lists, as vector<vector<hop_constrained_two_hop_label>>:
    ``L[v]`` is an int32 array of rows (hub_vertex, parent_vertex, hop, distance)
    sorted by (hub, hop, distance).  Backed by a device index; rows are copied
    to the host on first access."""

    def __init__(self, index: Index):
        self.index = index
        self._off = None
        self._lab = None

    def _load(self):
        if self._off is None:
            self._off, self._lab = self.index.export()

    def __len__(self) -> int:
        return self.index.info()["n"]

    def __getitem__(self, v: int) -> np.ndarray:
        self._load()
        return self._lab[self._off[v]: self._off[v + 1]]

    def total(self) -> int:
        return self.index.info()["labels"]


@dataclass
class hop_constrained_case_info:
    """Mirror of hop_constrained_case_info (hop_constrained_two_hop_labels.h:54-142)."""
    thread_num: int = 1                 # accepted for signature parity; the GPU ignores it
    upper_k: int = 0
    use_rank_prune: bool = True
    use_2023WWW_generation: bool = False
    use_canonical_repair: bool = True
    time_initialization: float = 0.0
    time_generate_labels: float = 0.0
    time_sortL: float = 0.0
    time_canonical_repair: float = 0.0
    time_total: float = 0.0
    max_bit_size: int = int(1e12)
    max_run_time_seconds: float = 1e12
    L: LabelLists | None = None
    label_size_before_canonical_repair: float = 0.0
    label_size_after_canonical_repair: float = 0.0
    canonical_repair_remove_label_ratio: float = 0.0
    build_options: dict = field(default_factory=dict)

    def compute_label_bit_size(self) -> int:
        return 0 if self.L is None else self.L.total() * 16

    def clear_labels(self) -> None:
        if self.L is not None:
            self.L.index.close()
        self.L = None


def _as_host_graph(input_graph) -> HostGraph:
    if isinstance(input_graph, HostGraph):
        return input_graph
    if isinstance(input_graph, Graph):
        return input_graph.host
    raise TypeError("input_graph must be a HostGraph or Graph (ids = ranks)")


def hop_constrained_two_hop_labels_generation(input_graph, case_info: hop_constrained_case_info) -> None:
    """hop_constrained_two_hop_labels_generation (generation.h:513-632): builds
    labels of a graph whose ids are ranks, fills case_info.L and the timers."""
    if case_info.upper_k <= 0:
        raise ValueError("upper_k must be >= 1 (unbounded hops are not supported)")
    t0 = time.perf_counter()
    g = input_graph if isinstance(input_graph, Graph) else Graph(_as_host_graph(input_graph))
    t1 = time.perf_counter()
    opts = dict(case_info.build_options)
    if case_info.use_2023WWW_generation:
        opts["generation"] = 1  # _2023WWW_thread_function (generation.h:226-370, selected at :568-574)
    idx = Index.build(g, case_info.upper_k, clean=False, **opts)
    info = idx.info()
    case_info.time_initialization = t1 - t0
    case_info.time_generate_labels = info["time_generate_s"]
    case_info.time_sortL = info["time_sort_s"]
    case_info.L = LabelLists(idx)
    case_info.label_size_before_canonical_repair = info["labels"]
    case_info.label_size_after_canonical_repair = info["labels"]
    if case_info.use_canonical_repair:
        hop_constrained_clean_L(case_info, case_info.thread_num)
    case_info.time_total = (case_info.time_initialization + case_info.time_generate_labels +
                            case_info.time_sortL + case_info.time_canonical_repair)


def hop_constrained_clean_L(case_info: hop_constrained_case_info, thread_num: int = 1) -> None:
    """hop_constrained_clean_L (generation.h:422-511) on case_info.L."""
    idx = case_info.L.index
    before = idx.info()["labels"]
    idx.clean()
    info = idx.info()
    case_info.L = LabelLists(idx)
    case_info.time_canonical_repair = info["time_clean_s"]
    case_info.label_size_before_canonical_repair = before
    case_info.label_size_after_canonical_repair = info["labels"]
    case_info.canonical_repair_remove_label_ratio = (before - info["labels"]) / before if before else 0.0


def _index_of(L) -> Index:
    if isinstance(L, LabelLists):
        return L.index
    if isinstance(L, Index):
        return L
    raise TypeError("L must be LabelLists or Index")


def hop_constrained_extract_distance(L, source: int, terminal: int, hop_cst: int) -> int:
    """hop_constrained_extract_distance (two_hop_labels.h:144-222); INT_MAX if none."""
    return int(_index_of(L).query([source], [terminal], [hop_cst])[0])


def hop_constrained_extract_shortest_path(L, source: int, terminal: int, hop_cst: int):
    """hop_constrained_extract_shortest_path (two_hop_labels.h:224-319)."""
    return _index_of(L).path(source, terminal, hop_cst)


def gpu_query(L, queries, K: int | None = None):
    """gpu_query (Query_mdnd/src/gpu_query.cu:84): answers an (n, 3) array of
    (s, t, h) queries; returns (answers, seconds)."""
    q = np.ascontiguousarray(queries, np.int32).reshape(-1, 3)
    t0 = time.perf_counter()
    out = _index_of(L).query(q[:, 0], q[:, 1], q[:, 2])
    return out, time.perf_counter() - t0


# ---------------------------------------------------------------------------
# Serving loop
# ---------------------------------------------------------------------------
class Server:
    """Persistent device-resident serving loop over many resident indexes
    (hsdl_serve_* in include/hsdl.h)."""

    def __init__(self, ctas: int = 0, ring_log2: int = 22, max_indexes: int = 1024,
                 budget_bytes: int = 120 << 30, idle_exit_s: float = 0.5, lanes_per_query: int = 32):
        o = N.hsdl_serve_opts()
        lib().hsdl_serve_opts_default(C.byref(o))
        o.ctas = ctas
        o.ring_log2 = ring_log2
        o.max_indexes = max_indexes
        o.budget_bytes = budget_bytes
        o.idle_exit_s = idle_exit_s
        o.lanes_per_query = lanes_per_query
        self._h = C.c_void_p()
        check(lib().hsdl_serve_create(C.byref(o), C.byref(self._h)))
        self._keep = {}

    def add_index(self, index: Index) -> int:
        gid = C.c_int32()
        check(lib().hsdl_serve_add_index(self._h, index.handle, C.byref(gid)))
        self._keep[gid.value] = index
        return gid.value

    def submit_build(self, graph: Graph, K: int) -> int:
        gid = C.c_int32()
        check(lib().hsdl_serve_submit_build(self._h, graph.handle, K, C.byref(gid)))
        self._keep[gid.value] = graph
        return gid.value

    def graph_state(self, gid: int):
        st = C.c_int32()
        b = C.c_int64()
        check(lib().hsdl_serve_graph_state(self._h, gid, C.byref(st), C.byref(b)))
        return st.value, b.value

    def wait_graph(self, gid: int, timeout_s: float = 600.0) -> None:
        check(lib().hsdl_serve_wait_graph(self._h, gid, timeout_s))

    def remove_graph(self, gid: int) -> None:
        check(lib().hsdl_serve_remove_graph(self._h, gid))
        self._keep.pop(gid, None)

    def query(self, g, s, t, k, timeout_s: float = 60.0) -> np.ndarray:
        """Submits requests and waits for their answers."""
        g = np.ascontiguousarray(g, np.int32)
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        n = len(s)
        out = np.zeros(n, np.int32)
        first = C.c_int64()
        step = 1 << 20
        for lo in range(0, n, step):
            hi = min(n, lo + step)
            check(lib().hsdl_serve_submit(self._h, hi - lo, _ptr(g[lo:hi]), _ptr(s[lo:hi]), _ptr(t[lo:hi]),
                                          _ptr(k[lo:hi]), C.byref(first)))
            check(lib().hsdl_serve_wait(self._h, first.value, hi - lo, _ptr(out[lo:hi]), timeout_s))
        return out

    def loadgen(self, g, s, t, k, offered_qps: float = 0.0, seed: int = 1, want_answers: bool = True,
                consumers: int = 4) -> dict:
        g = np.ascontiguousarray(g, np.int32)
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        # written (not just allocated) before the run: first touches of fresh
        # pages inside the timed run would stall the consumer threads
        ans = np.full(len(s), -1, np.int32) if want_answers else None
        o = N.hsdl_loadgen_opts()
        o.struct_size = C.sizeof(N.hsdl_loadgen_opts)
        o.n = len(s)
        o.g, o.s, o.t, o.k = g.ctypes.data, s.ctypes.data, t.ctypes.data, k.ctypes.data
        o.answers = ans.ctypes.data if ans is not None else None
        o.offered_qps = offered_qps
        o.seed = seed
        o.consumers = consumers
        r = N.hsdl_loadgen_result()
        check(lib().hsdl_serve_loadgen(self._h, C.byref(o), C.byref(r)))
        res = {f: getattr(r, f) for f, _ in N.hsdl_loadgen_result._fields_}
        res["answers"] = ans
        return res

    def stats(self) -> dict:
        st = N.hsdl_serve_counters()
        check(lib().hsdl_serve_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in N.hsdl_serve_counters._fields_}

    def close(self) -> None:
        if self._h:
            lib().hsdl_serve_destroy(self._h)
            self._h = C.c_void_p()
        self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
