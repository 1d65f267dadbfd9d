"""ctypes wrapper of the HSDL oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker / timed CPU baseline.  The
product library never imports it.

* ``Oracle``    - liboracle.so, this project's CPU restatement of the
                  reference path (hsdl_oracle.cpp; every function cites the
                  reference file:line it follows).
* ``Reference`` - oracle/_ref/libhsdl_ref.so, the reference's own CPU_HopHL
                  headers compiled in place (only where a reference checkout
                  was available at build time).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libhsdl_ref.so")
REF_LP_LIB = os.path.join(HERE, "_ref", "libcdlp_ref.so")


def reference_dir() -> str:
    """The reference checkout the checkers read: $HSDL_REFERENCE_DIR, else the
    location oracle/Makefile names (it may not exist on this machine)."""
    d = os.environ.get("HSDL_REFERENCE_DIR") or os.environ.get("HSDL_REF_DIR")
    if d:
        return d
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref-dir"], capture_output=True, text=True)
    return r.stdout.strip()


def build(ref_dir: str | None = None) -> None:
    """Compiles liboracle.so, and _ref/libhsdl_ref.so when a reference
    checkout exists: `ref_dir`, else $HSDL_REFERENCE_DIR, else the location
    oracle/Makefile names."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    ref_dir = ref_dir or os.environ.get("HSDL_REFERENCE_DIR")
    subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"] + ([f"REF_DIR={ref_dir}"] if ref_dir else []),
                   check=True)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class CsrGraph:
    """A ranked CSR graph (n, row_ptr int64[n+1], col int32[2m], w int32[2m])."""

    def __init__(self, n: int, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray):
        self.n, self.row_ptr, self.col, self.w = int(n), row_ptr, col, w

    @property
    def num_edges(self) -> int:
        return int(self.row_ptr[-1]) // 2


class Labels:
    """CPU label set: offsets int64[n+1], labels int32[total, 4]
    (hub, parent, hop, distance)."""

    def __init__(self, off: np.ndarray, lab: np.ndarray, info: dict | None = None):
        self.off = off
        self.lab = lab
        self.info = info or {}

    @property
    def n(self):
        return len(self.off) - 1

    def row(self, v):
        return self.lab[self.off[v]: self.off[v + 1]]


class Oracle:
    def __init__(self, path: str = PORT_LIB):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        L.orc_build.restype = vp
        L.orc_build.argtypes = [i32, vp, vp, vp, i32, i32, vp, i32, i32, i32]
        L.orc_from_labels.restype = vp
        L.orc_from_labels.argtypes = [i32, i32, vp, vp]
        L.orc_clean.argtypes = [vp, i32, i32]
        L.orc_size.restype = C.c_longlong
        L.orc_size.argtypes = [vp]
        L.orc_info.argtypes = [vp, vp, vp]
        L.orc_export.argtypes = [vp, vp, vp]
        L.orc_query.argtypes = [vp, i64, vp, vp, vp, vp, i32]
        L.orc_path.restype = i32
        L.orc_path.argtypes = [vp, i32, i32, i32, vp, i32]
        L.orc_free.argtypes = [vp]
        L.orc_bf.argtypes = [i32, vp, vp, vp, i32, i32, vp]
        L.orc_lp_group.restype = i32
        L.orc_lp_group.argtypes = [i32, vp, vp, i32, i32, vp, vp]
        L.orc_lp_assemble.restype = i32
        L.orc_lp_assemble.argtypes = [i32, vp, vp, i32, vp]
        L.orc_set_time_cap.argtypes = [C.c_double]
        L.orc_gen_chung_lu.restype = vp
        L.orc_gen_chung_lu.argtypes = [i32, C.c_double, C.c_double, C.c_double, i32, i32, C.c_uint64, vp]
        L.orc_graph_copy.argtypes = [vp, vp, vp, vp]
        L.orc_graph_free.argtypes = [vp]
        self.L = L

    def chung_lu(self, n: int, avg_degree: float, exponent: float, max_degree: float, wmin: int, wmax: int,
                 seed: int) -> "CsrGraph":
        """The seeded Chung-Lu workload graph, ranked (the generator the
        product library uses, compiled into this library)."""
        m2 = np.zeros(1, np.int64)
        h = self.L.orc_gen_chung_lu(n, avg_degree, exponent, max_degree, wmin, wmax, seed, _p(m2))
        try:
            g = CsrGraph(n, np.zeros(n + 1, np.int64), np.zeros(int(m2[0]), np.int32), np.zeros(int(m2[0]), np.int32))
            self.L.orc_graph_copy(h, _p(g.row_ptr), _p(g.col), _p(g.w))
        finally:
            self.L.orc_graph_free(h)
        return g

    # -- handles -------------------------------------------------------------
    def _export(self, h) -> Labels:
        n = None
        tot = self.L.orc_size(h)
        info = np.zeros(6)
        work = np.zeros(3, np.int64)
        self.L.orc_info(h, _p(info), _p(work))
        # n is recovered from export
        off = np.zeros(self._n + 1, np.int64)
        lab = np.zeros((max(1, tot), 4), np.int32)
        self.L.orc_export(h, _p(off), _p(lab))
        return Labels(off, lab[:tot], {"t_gen": info[0], "t_sort": info[1], "t_clean": info[2],
                                       "before": int(info[3]), "after": int(info[4]),
                                       "hubs_searched": int(info[5]),
                                       "popped": int(work[0]), "relaxed": int(work[1]),
                                       "query_reads": int(work[2])})

    def build(self, g, K: int, threads: int = 1, wave_bounds=None, clean: bool = True,
              www: bool = False) -> Labels:
        """Generation (+ sortL, + clean).  wave_bounds: the GPU's wave schedule
        (hsdl_wave_bounds) to reproduce its uncleaned superset exactly.  www:
        the reference's 2023WWW generation (one thread, or wave mode)."""
        if www and wave_bounds is None and threads != 1:
            raise ValueError("the 2023WWW generation runs with one thread or in wave mode")
        b = None if wave_bounds is None else np.ascontiguousarray(wave_bounds, np.int32)
        self._n = g.n
        h = self.L.orc_build(g.n, _p(g.row_ptr), _p(g.col), _p(g.w), K, threads, _p(b),
                             0 if b is None else len(b), int(clean), int(www))
        try:
            return self._export(h)
        finally:
            self.L.orc_free(h)

    def set_time_cap(self, seconds: float) -> None:
        """Caps later builds' generation (reference schedule) at `seconds`
        (0 = none): hubs not started by then are not searched."""
        self.L.orc_set_time_cap(float(seconds))

    def clean(self, labels: Labels, K: int, threads: int = 1, mode: int = 0) -> Labels:
        """hop_constrained_clean_L on an arbitrary sorted label set."""
        self._n = labels.n
        lab = np.ascontiguousarray(labels.lab, np.int32)
        h = self.L.orc_from_labels(labels.n, K, _p(labels.off), _p(lab))
        try:
            self.L.orc_clean(h, threads, mode)
            return self._export(h)
        finally:
            self.L.orc_free(h)

    def index(self, labels: Labels) -> "OracleIndex":
        """Loads a label set once; queries and paths then run on it."""
        return OracleIndex(self, labels)

    def query(self, labels: Labels, s, t, k, threads: int = 1) -> np.ndarray:
        with self.index(labels) as ix:
            return ix.query(s, t, k, threads)

    def path(self, labels: Labels, s: int, t: int, k: int, cap: int = 64):
        with self.index(labels) as ix:
            return ix.path(s, t, k, cap)

    def bf(self, g, src: int, k: int) -> np.ndarray:
        out = np.zeros(g.n, np.int32)
        self.L.orc_bf(g.n, _p(g.row_ptr), _p(g.col), _p(g.w), src, k, _p(out))
        return out

    def lp_group(self, g, max_group: int, max_iterations: int = 100):
        """Deterministic capped label propagation + the reference's group
        assembly; returns (group_of_vertex, number of groups, iterations)."""
        gov = np.zeros(g.n, np.int32)
        it = np.zeros(1, np.int32)
        ng = self.L.orc_lp_group(g.n, _p(g.row_ptr), _p(g.col), max_group, max_iterations, _p(gov), _p(it))
        return gov, int(ng), int(it[0])

    def lp_assemble(self, g, labels, max_group: int):
        """The group assembly alone on given propagation labels (each in
        [0, n)); returns (group_of_vertex, number of groups)."""
        lab = np.ascontiguousarray(labels, np.int32)
        gov = np.zeros(g.n, np.int32)
        ng = self.L.orc_lp_assemble(g.n, _p(g.row_ptr), _p(lab), max_group, _p(gov))
        return gov, int(ng)


class Reference:
    """The reference's own CPU_HopHL (compiled from its headers in place)."""

    available = os.path.exists(REF_LIB)

    def __init__(self, path: str = REF_LIB):
        L = C.CDLL(path)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        L.ref_build.restype = C.c_int64
        L.ref_build.argtypes = [i32, vp, vp, vp, i32, i32, i32, i32]
        L.ref_times.argtypes = [vp]
        L.ref_export.argtypes = [vp, vp]
        L.ref_query.argtypes = [i64, vp, vp, vp, vp, i32]
        L.ref_bf.argtypes = [i32, i32, vp]
        L.ref_path.restype = i32
        L.ref_path.argtypes = [i32, i32, i32, vp, i32]
        self.L = L
        self.n = 0

    def build(self, g, K: int, threads: int = 1, clean: bool = True, www: bool = False) -> Labels:
        """www: the reference's 2023WWW generation instead of HSDL's."""
        tot = self.L.ref_build(g.n, _p(g.row_ptr), _p(g.col), _p(g.w), K, threads, int(clean), int(www))
        self.n = g.n
        off = np.zeros(g.n + 1, np.int64)
        lab = np.zeros((max(1, tot), 4), np.int32)
        self.L.ref_export(_p(off), _p(lab))
        t = np.zeros(4)
        self.L.ref_times(_p(t))
        return Labels(off, lab[:tot], {"t_init": t[0], "t_gen": t[1], "t_sort": t[2], "t_clean": t[3]})

    def query(self, s, t, k, threads: int = 1) -> np.ndarray:
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        out = np.zeros(len(s), np.int32)
        self.L.ref_query(len(s), _p(s), _p(t), _p(k), _p(out), threads)
        return out

    def bf(self, src: int, k: int) -> np.ndarray:
        out = np.zeros(self.n, np.int32)
        self.L.ref_bf(src, k, _p(out))
        return out

    def path(self, s: int, t: int, k: int, cap: int = 64):
        e = np.zeros((cap, 2), np.int32)
        c = self.L.ref_path(s, t, k, _p(e), cap)
        return [tuple(x) for x in e[:max(c, 0)].tolist()]


class ReferenceLP:
    """The reference's own LP group assembly (CDLP_group.cuh:39-100) compiled
    in place, fed given propagation labels (oracle/ref_lp_driver.cpp)."""

    available = os.path.exists(REF_LP_LIB)

    def __init__(self, path: str = REF_LP_LIB):
        L = C.CDLL(path)
        vp, i32 = C.c_void_p, C.c_int
        L.ref_lp_assemble.restype = i32
        L.ref_lp_assemble.argtypes = [i32, vp, vp, vp, i32, vp]
        self.L = L

    def assemble(self, g, labels, max_group: int):
        lab = np.ascontiguousarray(labels, np.int32)
        gov = np.zeros(g.n, np.int32)
        ng = self.L.ref_lp_assemble(g.n, _p(g.row_ptr), _p(g.col), _p(lab), max_group, _p(gov))
        return gov, int(ng)


class OracleIndex:
    """A label set loaded into the oracle (conversion paid once)."""

    def __init__(self, orc: Oracle, labels: Labels):
        self.L = orc.L
        lab = np.ascontiguousarray(labels.lab, np.int32)
        self.h = self.L.orc_from_labels(labels.n, 15, _p(labels.off), _p(lab))

    def query(self, s, t, k, threads: int = 1) -> np.ndarray:
        s = np.ascontiguousarray(s, np.int32)
        t = np.ascontiguousarray(t, np.int32)
        k = np.ascontiguousarray(k, np.int32)
        out = np.zeros(len(s), np.int32)
        self.L.orc_query(self.h, len(s), _p(s), _p(t), _p(k), _p(out), threads)
        return out

    def path(self, s: int, t: int, k: int, cap: int = 64):
        e = np.zeros((cap, 2), np.int32)
        c = self.L.orc_path(self.h, s, t, k, _p(e), cap)
        return [tuple(x) for x in e[:max(c, 0)].tolist()]

    def close(self):
        if self.h:
            self.L.orc_free(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
