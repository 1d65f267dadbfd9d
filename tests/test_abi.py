"""The C-ABI library on the CPU: it loads, exports every symbol the public
headers declare, and its host-side logic (seeded generators, rank relabel,
CSR validation, error reporting) behaves.  No compute call needs a GPU here."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(hsdl_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(built, n)]
    assert not missing, missing


def test_binding_table_covers_the_header(built):
    from gpu4hophl_code_gb300 import _native

    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_generators_are_deterministic_and_ranked(built):
    from gpu4hophl_code_gb300 import HostGraph

    for make in (lambda s: HostGraph.erdos_renyi(500, 2000, 1, 100, seed=s),
                 lambda s: HostGraph.chung_lu(3000, 10, 2.1, 300, 1, 100, seed=s),
                 lambda s: HostGraph.barabasi_albert(800, 3, 1, 1000, seed=s)):
        a, b, c = make(9), make(9), make(10)
        assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col) and np.array_equal(a.w, b.w)
        assert not (np.array_equal(a.col, c.col) and np.array_equal(a.w, c.w))
        a.validate()
        deg = np.diff(a.row_ptr)
        assert np.all(deg[:-1] >= deg[1:]), "ids must follow degree descending"
        # ties by original id: within equal degree, new_to_old increases
        same = deg[:-1] == deg[1:]
        assert np.all(a.new_to_old[:-1][same] < a.new_to_old[1:][same])


def test_generator_shapes(built):
    from gpu4hophl_code_gb300 import HostGraph

    er = HostGraph.erdos_renyi(1000, 5000, 1, 100, seed=1)
    assert er.num_edges == 5000 and er.w.min() >= 1 and er.w.max() <= 100
    cl = HostGraph.chung_lu(20000, 10, 2.1, 1000, 1, 100, seed=1)
    assert cl.num_edges == 100000
    assert np.diff(cl.row_ptr).max() > 100  # power-law head
    ba = HostGraph.barabasi_albert(1000, 3, 1, 1000, seed=1)
    assert abs(ba.num_edges - 3 * 1000) < 10


def test_chung_lu_matches_committed_checksum(built):
    """The generator is integer/IEEE-exact: the same seed gives the same graph
    on x86-64 and aarch64."""
    import hashlib

    from gpu4hophl_code_gb300 import HostGraph

    g = HostGraph.chung_lu(5000, 10, 2.1, 500, 1, 100, seed=0x48534C44)
    h = hashlib.sha256(g.row_ptr.tobytes() + g.col.tobytes() + g.w.tobytes()).hexdigest()
    assert h == open(os.path.join(ROOT, "tests", "golden", "chung_lu_5000.sha256")).read().strip()


def test_from_edges_and_text_reader(built, tmp_path):
    from gpu4hophl_code_gb300 import HostGraph

    p = tmp_path / "g.txt"
    p.write_text("|V|= 4\n|E|= 4\n\nEdge 0 1 5\nEdge 1 2 3\nEdge 2 3 1\nEdge 0 2 2\nEdge 0 1 7\n\nEOF\n")
    g = HostGraph.read_text(str(p), rank_by_degree=False)
    assert g.n == 4 and g.num_edges == 4
    # a repeated edge keeps its last weight (graph_v_of_v::add_edge updates it)
    assert g.w[g.row_ptr[0]] == 7
    r = HostGraph.read_text(str(p), rank_by_degree=True)
    assert list(np.diff(r.row_ptr)) == [3, 3, 2, 2][: r.n] or sorted(np.diff(r.row_ptr), reverse=True) == list(
        np.diff(r.row_ptr))
    r.validate()


@pytest.mark.parametrize("text", ["|V|= 4294967301\nEdge 0 1 5\n", "|V|= 5\nEdge 0 4294967299 5\n",
                                  "|V|= 5\nEdge -1 2 5\n", "|V|= 5\nEdge 0 1 1e12\n"])
def test_text_reader_rejects_values_outside_int32(built, tmp_path, text):
    """Ids, counts and weights are range-checked before they are narrowed to
    int32, so an oversized value cannot wrap into a valid small one."""
    from gpu4hophl_code_gb300 import HostGraph, HsdlError

    p = tmp_path / "g.txt"
    p.write_text(text)
    with pytest.raises(HsdlError) as e:
        HostGraph.read_text(str(p))
    assert e.value.code == 1 and "range" in str(e.value)


def test_label_file_with_a_corrupt_count_is_an_error(built, tmp_path):
    """A row count larger than the rest of the file is reported before any
    buffer is sized by it (no device is touched on this path)."""
    from gpu4hophl_code_gb300 import HsdlError, Index

    p = tmp_path / "labels.bin"
    p.write_bytes(np.array([2, 1], np.uint64).tobytes() + np.array([0, 0, 0, 0], np.int32).tobytes() +
                  np.array([1 << 39], np.uint64).tobytes())
    with pytest.raises(HsdlError) as e:
        Index.load(str(p), 3)
    assert e.value.code == 7 and "malformed" in str(e.value)


@pytest.mark.parametrize("case", ["selfloop", "asym", "unsorted", "weight0", "range"])
def test_malformed_csr_is_rejected_with_a_message(built, case):
    from gpu4hophl_code_gb300 import HostGraph, HsdlError

    g = HostGraph.erdos_renyi(20, 40, 1, 9, seed=2)
    rp, col, w = g.row_ptr.copy(), g.col.copy(), g.w.copy()
    if case == "selfloop":
        col[rp[3]] = 3
    elif case == "asym":
        w[0] += 1
    elif case == "unsorted":
        v = int(np.argmax(np.diff(rp) >= 2))
        col[rp[v]], col[rp[v] + 1] = col[rp[v] + 1], col[rp[v]]
    elif case == "weight0":
        w[:] = 0
    elif case == "range":
        col[0] = 99
    bad = HostGraph(g.n, rp, col, w)
    with pytest.raises(HsdlError) as e:
        bad.validate()
    assert e.value.code == 1 and str(e.value)


def test_bad_arguments_fail_without_a_device(built):
    from gpu4hophl_code_gb300 import HostGraph, HsdlError

    with pytest.raises(HsdlError):
        HostGraph.erdos_renyi(1, 0)
    with pytest.raises(HsdlError):
        HostGraph.chung_lu(100, 10, 0.5, 10)


def test_wave_schedule(built):
    from gpu4hophl_code_gb300 import wave_bounds

    b = wave_bounds(1000, first_wave=1, max_wave=64)
    assert b[0] == 0 and b[-1] == 1000
    w = np.diff(b)
    assert list(w[:7]) == [1, 2, 4, 8, 16, 32, 64] and w.max() == 64


def test_label_record_layout_matches_reference():
    """hsdl_label is the reference's 16-byte record {hub, parent, hop, distance}."""
    from gpu4hophl_code_gb300._native import hsdl_label

    assert C.sizeof(hsdl_label) == 16
    assert [f for f, _ in hsdl_label._fields_] == ["hub_vertex", "parent_vertex", "hop", "distance"]


def test_python_struct_mirrors_match_the_header(tmp_path):
    """Every ctypes mirror of a public struct has the header's size and field
    offsets (a C program compiled against include/hsdl.h prints them)."""
    import shutil
    import subprocess

    from gpu4hophl_code_gb300 import _native as N

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [getattr(N, name) for name in dir(N)
               if name.startswith("hsdl_") and isinstance(getattr(N, name), type)
               and issubclass(getattr(N, name), C.Structure)]
    assert len(structs) >= 8
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "hsdl.h"', "int main(void) {"]
    for cls in structs:
        t = cls.__name__
        lines.append(f'  printf("{t} sizeof %zu\\n", sizeof({t}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{t} {f} %zu\\n", offsetof({t}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c_layout = {(a, b): int(c) for a, b, c in (line.split() for line in out if line)}
    for cls in structs:
        t = cls.__name__
        assert c_layout[(t, "sizeof")] == C.sizeof(cls), t
        for f, _ in cls._fields_:
            assert c_layout[(t, f)] == getattr(cls, f).offset, (t, f)
