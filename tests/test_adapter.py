"""The C++ drop-in adapter (include/hsdl_reference_adapter.hpp): its templates
bind to the reference's own graph_v_of_v / hop_constrained_case_info types
(compile check, where a reference checkout is at hand), and a program written
against them gets the same labels, answers and paths as the C ABI."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import gpu4hophl_code_gb300 as H

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "gpu4hophl_code_gb300")


def _ref_dir():
    from oracle.oracle import reference_dir

    return reference_dir()


def test_adapter_binds_to_the_reference_types():
    ref = _ref_dir()
    if not os.path.isdir(os.path.join(ref, "CPU_HopHL", "include")) or shutil.which("g++") is None:
        pytest.skip("no reference checkout here")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + os.path.join(ref, "CPU_HopHL", "include"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, "adapter", "adapter_binds_reference.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
@pytest.mark.parametrize("www", [False, True])
def test_adapter_program_matches_the_c_abi(tmp_path, www):
    """www: case_info.use_2023WWW_generation = true (the 2023WWW search);
    more labels before the clean, the same labels after it."""
    exe = str(tmp_path / "adapter_demo")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, "adapter", "adapter_demo.cpp"), "-L" + LIBDIR, "-lhsdl",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    g = H.HostGraph.chung_lu(3000, 8, 2.2, 300, 1, 100, seed=91)
    K = 5
    a, b, w = g.edges()
    rng = np.random.default_rng(4)
    q = 2000
    s = rng.integers(0, g.n, q).astype(np.int32)
    t = rng.integers(0, g.n, q).astype(np.int32)
    k = rng.integers(0, K + 1, q).astype(np.int32)
    lines = [f"{g.n} {len(a)} {K}"] + [f"{x} {y} {z}" for x, y, z in zip(a, b, w)] + [str(q)]
    lines += [f"{x} {y} {z}" for x, y, z in zip(s, t, k)]
    r = subprocess.run([exe] + (["www"] if www else []), input="\n".join(lines) + "\n", capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = r.stdout.split("\n")
    idx = H.Index.build(H.Graph(g), K, generation=1 if www else 0)
    info = idx.info()
    off, _ = idx.export()
    before, after = next(l for l in out if l.startswith("labels")).split()[1:]
    assert int(before) == info["labels_before_clean"] and int(after) == info["labels"]
    if www:
        assert info["labels"] == H.Index.build(H.Graph(g), K).info()["labels"]
    rows = np.array([int(l.split()[2]) for l in out if l.startswith("row ")])
    assert np.array_equal(rows, np.diff(off))
    want = idx.query(s, t, k)
    assert np.array_equal(np.array([int(l.split()[1]) for l in out if l.startswith("ans ")]), want)
    assert np.array_equal(np.array([int(l.split()[1]) for l in out if l.startswith("batch ")]), want)
    path = idx.path(int(s[0]), int(t[0]), int(k[0]))
    assert int(next(l for l in out if l.startswith("path ")).split()[1]) == len(path)
