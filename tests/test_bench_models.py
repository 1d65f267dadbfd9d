"""The byte models behind the bench line's roofline figures, on small inputs
computed by hand.  CPU only."""
import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_query_bytes_count_both_rows_and_the_offsets():
    off = np.array([0, 3, 3, 10, 12], np.int64)  # row lengths 3, 0, 7, 2
    s = np.array([0, 2, 1, 3], np.int32)
    t = np.array([2, 3, 1, 3], np.int32)  # the last two pairs are s == t: no row is read
    k = np.array([1, 2, 3, 4], np.int32)
    want = 12 * ((3 + 7) + (7 + 2)) + 32 * 4
    assert bench.algorithmic_bytes(off, s, t, k) == want
    assert bench.algorithmic_bytes(off, s, t, k, per_label=8) == 8 * 19 + 32 * 4


def test_build_byte_models():
    info = {"work_relaxations": 10, "work_join_reads": 100, "work_join_visible": 250,
            "work_labels_written": 7, "work_clean_reads": 40, "labels": 5}
    assert bench.build_algorithmic_bytes(info) == 16 * 10 + 8 * 100 + 12 * 7 + 8 * 40 + 24 * 5
    assert bench.scope_generation_bytes(info) == 8 * 10 + 12 * 250 + 16 * 7


def test_captured_traffic_is_read_from_the_committed_profile():
    args = argparse.Namespace(n=1_000_000, queries=10_000_000, K=5)
    v = bench.captured_traffic(args)
    assert isinstance(v["bytes"], int) and v["bytes"] > 0
    assert v["capture"].startswith("profiles/") and isinstance(v["current"], bool)
    args.n = 200_000
    assert bench.captured_traffic(args) is None


def test_reference_arm_runs_without_the_product_library():
    """bench.py --impl reference builds the index with the oracle on the CPU
    (the same seeded graph, generated by the oracle library) and never maps
    libhsdl.so; a time cap turns the build into a watchdog-capped sample."""
    import subprocess
    import sys

    code = ("import sys, json, argparse; sys.path.insert(0, %r); import bench; "
            "a = argparse.Namespace(n=3000, K=5, queries=20000, steps=1, warmup=1, ref_build_cap=0.0); "
            "r = bench.run_reference(a, None, 0, 1, 0); "
            "maps = open('/proc/self/maps').read(); "
            "print(json.dumps({'hsdl': 'libhsdl.so' in maps, 'oracle': 'liboracle.so' in maps, "
            "'hubs': r['build']['hubs_searched'], 'capped': r['build']['capped'], 'v': r['value']}))") % bench.ROOT
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout
    import json

    d = json.loads(out.strip().splitlines()[-1])
    assert d["oracle"] and not d["hsdl"]
    assert d["hubs"] == 3000 and not d["capped"] and d["v"] > 0
