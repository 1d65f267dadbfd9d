"""ctypes binding of libhsdl.so (declarations in include/hsdl.h).

The library is built in-tree by gpu4hophl_code_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhsdl.so")

HSDL_OK = 0
HSDL_ERR_INVALID = 1
HSDL_ERR_CUDA = 2
HSDL_ERR_NOMEM = 3
HSDL_ERR_TIMEOUT = 4
HSDL_ERR_STATE = 5
HSDL_ERR_FULL = 6
HSDL_ERR_IO = 7

_CODES = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "TIMEOUT", 5: "STATE", 6: "FULL", 7: "IO"}


class HsdlError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hsdl error {_CODES.get(code, code)}: {msg}")
        self.code = code


class hsdl_label(C.Structure):
    _fields_ = [("hub_vertex", C.c_int32), ("parent_vertex", C.c_int32), ("hop", C.c_int32),
                ("distance", C.c_int32)]


class hsdl_build_opts(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("clean", C.c_int32), ("first_wave", C.c_int32),
                ("max_wave", C.c_int32), ("block_threads", C.c_int32), ("frontier_tile", C.c_int32),
                ("prune_lanes", C.c_int32), ("prune_pairs", C.c_int32), ("generation", C.c_int32),
                ("prune_order", C.c_int32), ("pool_key_bytes", C.c_int32), ("reserved", C.c_int32),
                ("device_budget_bytes", C.c_int64)]


class hsdl_index_info(C.Structure):
    _fields_ = [("n", C.c_int32), ("K", C.c_int32), ("cleaned", C.c_int32), ("waves", C.c_int32),
                ("labels", C.c_int64), ("labels_before_clean", C.c_int64), ("labels_after_clean", C.c_int64),
                ("device_bytes", C.c_int64), ("time_generate_s", C.c_double), ("time_sort_s", C.c_double),
                ("time_clean_s", C.c_double), ("max_row", C.c_int64), ("work_relaxations", C.c_int64),
                ("work_join_reads", C.c_int64), ("work_labels_written", C.c_int64), ("work_clean_reads", C.c_int64),
                ("work_candidates", C.c_int64), ("work_join_visible", C.c_int64),
                ("build_peak_bytes", C.c_int64), ("build_pool_entries", C.c_int64),
                ("build_max_candidates", C.c_int64), ("build_wave_splits", C.c_int32), ("build_pool_chunks", C.c_int32),
                ("query_key_bytes", C.c_int32), ("query_key_hub_bits", C.c_int32),
                ("build_pool_key_bytes", C.c_int32), ("reserved", C.c_int32)]


class hsdl_serve_opts(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("ctas", C.c_int32), ("ring_log2", C.c_int32),
                ("max_indexes", C.c_int32), ("budget_bytes", C.c_int64), ("idle_exit_s", C.c_double),
                ("lanes_per_query", C.c_int32), ("reserved", C.c_int32)]


class hsdl_loadgen_opts(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("consumers", C.c_int32), ("n", C.c_int64), ("g", C.c_void_p),
                ("s", C.c_void_p), ("t", C.c_void_p), ("k", C.c_void_p), ("answers", C.c_void_p),
                ("offered_qps", C.c_double), ("seed", C.c_uint64)]


class hsdl_loadgen_result(C.Structure):
    _fields_ = [("completed", C.c_int64), ("seconds", C.c_double), ("achieved_qps", C.c_double),
                ("offered_qps", C.c_double), ("p50_us", C.c_double), ("p90_us", C.c_double),
                ("p99_us", C.c_double), ("p999_us", C.c_double), ("max_us", C.c_double),
                ("ready_frac", C.c_double), ("mean_batch", C.c_double)]


class hsdl_query_loadgen_opts(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("max_batch", C.c_int32), ("n", C.c_int64), ("s", C.c_void_p),
                ("t", C.c_void_p), ("k", C.c_void_p), ("answers", C.c_void_p), ("offered_qps", C.c_double),
                ("seed", C.c_uint64), ("window_us", C.c_double)]


class hsdl_serve_counters(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("processed", C.c_int64), ("bad_requests", C.c_int64),
                ("resident_graphs", C.c_int64), ("pending_builds", C.c_int64), ("resident_bytes", C.c_int64),
                ("builds_done", C.c_int64), ("loop_running", C.c_int32), ("reserved", C.c_int32)]


class hsdl_query_tuning(C.Structure):
    _fields_ = [("struct_size", C.c_int32), ("block_threads", C.c_int32), ("prefetch_ahead", C.c_int32),
                ("lanes_per_query", C.c_int32)]


P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
PP = C.POINTER(C.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "hsdl_last_error": (C.c_char_p, []),
    "hsdl_version": (I32, []),
    "hsdl_launch_count": (I64, []),
    "hsdl_debug_inject_failure": (C.c_int, [I32, I32]),
    "hsdl_debug_pool_used_high": (C.c_int, [P, I32]),
    "hsdl_gen_erdos_renyi": (C.c_int, [I32, I64, I32, I32, C.c_uint64, PP]),
    "hsdl_gen_chung_lu": (C.c_int, [I32, C.c_double, C.c_double, C.c_double, I32, I32, C.c_uint64, PP]),
    "hsdl_gen_barabasi_albert": (C.c_int, [I32, I32, I32, I32, C.c_uint64, PP]),
    "hsdl_host_graph_from_edges": (C.c_int, [I32, I64, P, P, P, I32, PP]),
    "hsdl_read_graph_text": (C.c_int, [C.c_char_p, I32, PP]),
    "hsdl_host_graph_get": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), PP, PP, PP, PP]),
    "hsdl_host_graph_free": (None, [P]),
    "hsdl_validate_csr": (C.c_int, [I32, P, P, P]),
    "hsdl_graph_create": (C.c_int, [I32, P, P, P, PP]),
    "hsdl_graph_destroy": (C.c_int, [P]),
    "hsdl_graph_create_from_edges": (C.c_int, [I32, I64, P, P, P, I32, P, PP]),
    "hsdl_graph_get_csr": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), P, P, P]),
    "hsdl_group_lp": (C.c_int, [P, I32, I32, P, C.POINTER(I32), C.POINTER(I32)]),
    "hsdl_build_opts_default": (None, [C.POINTER(hsdl_build_opts)]),
    "hsdl_wave_bounds": (C.c_int, [I32, C.POINTER(hsdl_build_opts), P, I32, C.POINTER(I32)]),
    "hsdl_build": (C.c_int, [P, I32, C.POINTER(hsdl_build_opts), PP]),
    "hsdl_build_batched": (C.c_int, [I32, P, P, P, P, P, C.POINTER(hsdl_build_opts), P]),
    "hsdl_build_autotune": (C.c_int, [P, I32, I32, C.POINTER(hsdl_build_opts), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int32)]),
    "hsdl_build_batched_autotune": (C.c_int, [I32, P, P, P, P, P, I32, C.POINTER(hsdl_build_opts),
                                              C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "hsdl_clean": (C.c_int, [P]),
    "hsdl_query_batch": (C.c_int, [P, I64, P, P, P, P]),
    "hsdl_query_batch_device": (C.c_int, [P, I64, P, P, P, P, P]),
    "hsdl_query_batch_static": (C.c_int, [P, I64, P, P, P, P]),
    "hsdl_query_static_prepare": (C.c_int, []),
    "hsdl_extract_path": (C.c_int, [P, I32, I32, I32, P, I32, C.POINTER(I32)]),
    "hsdl_index_get_info": (C.c_int, [P, C.POINTER(hsdl_index_info)]),
    "hsdl_export": (C.c_int, [P, P, P]),
    "hsdl_import": (C.c_int, [I32, I32, P, P, PP]),
    "hsdl_save_labels": (C.c_int, [P, C.c_char_p]),
    "hsdl_load_labels": (C.c_int, [C.c_char_p, I32, PP]),
    "hsdl_index_destroy": (C.c_int, [P]),
    "hsdl_set_query_tuning": (C.c_int, [P, C.POINTER(hsdl_query_tuning)]),
    "hsdl_get_query_tuning": (C.c_int, [P, C.POINTER(hsdl_query_tuning)]),
    "hsdl_serve_opts_default": (None, [C.POINTER(hsdl_serve_opts)]),
    "hsdl_serve_create": (C.c_int, [C.POINTER(hsdl_serve_opts), PP]),
    "hsdl_serve_add_index": (C.c_int, [P, P, C.POINTER(I32)]),
    "hsdl_serve_submit_build": (C.c_int, [P, P, I32, C.POINTER(I32)]),
    "hsdl_serve_graph_state": (C.c_int, [P, I32, C.POINTER(I32), C.POINTER(I64)]),
    "hsdl_serve_wait_graph": (C.c_int, [P, I32, C.c_double]),
    "hsdl_serve_remove_graph": (C.c_int, [P, I32]),
    "hsdl_serve_submit": (C.c_int, [P, I64, P, P, P, P, C.POINTER(I64)]),
    "hsdl_serve_wait": (C.c_int, [P, I64, I64, P, C.c_double]),
    "hsdl_serve_loadgen": (C.c_int, [P, C.POINTER(hsdl_loadgen_opts), C.POINTER(hsdl_loadgen_result)]),
    "hsdl_query_loadgen": (C.c_int, [P, C.POINTER(hsdl_query_loadgen_opts), C.POINTER(hsdl_loadgen_result)]),
    "hsdl_serve_stats": (C.c_int, [P, C.POINTER(hsdl_serve_counters)]),
    "hsdl_serve_destroy": (C.c_int, [P]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Loads libhsdl.so from the package directory (raises if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                                   "`python -c 'import __graft_entry__ as g; g.build()'`")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(rc: int) -> None:
    if rc != HSDL_OK:
        msg = lib().hsdl_last_error()
        raise HsdlError(rc, msg.decode() if msg else "")


def last_error() -> str:
    m = lib().hsdl_last_error()
    return m.decode() if m else ""
