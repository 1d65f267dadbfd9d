"""GB300 hop-constrained shortest-distance 2-hop labeling (HSDL).

Label generation, canonical clean and (s,t,k) distance queries run as
hand-written sm_103a kernels in libhsdl.so (C ABI: include/hsdl.h); this
package is the Python host side over that ABI.
"""
from .hsdl import (INT_MAX, Graph, autotune_build, autotune_build_batched, HostGraph, Index, LabelLists, Server, build_opts, generate_Group_CDLP, gpu_query, group_lp,
                   hop_constrained_case_info, hop_constrained_clean_L, hop_constrained_extract_distance,
                   hop_constrained_extract_shortest_path, hop_constrained_two_hop_labels_generation, wave_bounds)
from ._native import HsdlError, lib

__all__ = [
    "INT_MAX", "Graph", "autotune_build", "autotune_build_batched", "HostGraph", "Index", "LabelLists", "Server", "build_opts", "generate_Group_CDLP", "gpu_query", "group_lp", "hop_constrained_case_info",
    "hop_constrained_clean_L", "hop_constrained_extract_distance", "hop_constrained_extract_shortest_path",
    "hop_constrained_two_hop_labels_generation", "wave_bounds", "HsdlError", "lib",
]
