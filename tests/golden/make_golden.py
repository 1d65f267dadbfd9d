"""Generates the golden fixtures under tests/golden/ by running the reference's
own CPU implementation (CPU_HopHL, compiled in place into
oracle/_ref/libhsdl_ref.so by oracle/Makefile).

The reference ships no stored labels or answers, so these fixtures are its
outputs on seeded synthetic graphs plus its two fixture graphs
(data/simple_iterative_tests.txt, data/euroroad2.txt), converted to CSR.

Run from the repository root where a reference checkout exists:
    python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import hashlib
import os
import sys
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import gpu4hophl_code_gb300 as H  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def queries(n: int, K: int, count: int, seed: int):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, n, count).astype(np.int32)
    t = rng.integers(0, n, count).astype(np.int32)
    k = rng.integers(0, K + 1, count).astype(np.int32)  # includes k = 0 edge cases
    k[:8] = [-1, 0, 0, 1, 1, K, K, K]
    t[:4] = s[:4]  # s == t cases
    return s, t, k


def make(name: str, g, K: int, full: bool, nq: int = 4000, bf_sources: int = 20):
    R = O.Reference()
    lab = R.build(g, K, threads=1)
    s, t, k = queries(g.n, K, nq, seed=zlib.crc32(name.encode()))
    ans = R.query(s, t, k)
    rng = np.random.default_rng(11)
    srcs = rng.integers(0, g.n, bf_sources).astype(np.int32)
    hops = rng.integers(1, K + 1, bf_sources).astype(np.int32)
    bf = np.stack([R.bf(int(a), int(h)) for a, h in zip(srcs, hops)])
    arrays = dict(n=np.int32(g.n), K=np.int32(K), row_ptr=g.row_ptr, col=g.col, w=g.w, q_s=s, q_t=t, q_k=k,
                  q_ans=ans, bf_src=srcs, bf_hop=hops, bf_dist=bf,
                  hhd_digest=np.array(digest(lab.lab[:, [0, 2, 3]])), off_digest=np.array(digest(lab.off)),
                  n_labels=np.int64(len(lab.lab)))
    if full:
        arrays["off"] = lab.off
        arrays["labels"] = lab.lab
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)
    print(f"{name}: n={g.n} m={g.num_edges} K={K} labels={len(lab.lab)} full={full}")


def make_www(name: str, g, K: int):
    """The reference's 2023WWW generation (use_2023WWW_generation = 1,
    thread_num = 1): its labels before the clean (duplicates and parents
    included, per vertex sorted) and after."""
    R = O.Reference()
    raw = R.build(g, K, threads=1, clean=False, www=True)
    cln = R.build(g, K, threads=1, clean=True, www=True)
    os.makedirs(os.path.join(OUT, "www"), exist_ok=True)
    np.savez_compressed(os.path.join(OUT, "www", f"{name}.npz"), n=np.int32(g.n), K=np.int32(K), row_ptr=g.row_ptr,
                        col=g.col, w=g.w, raw_off=raw.off, raw_labels=raw.lab, off=cln.off, labels=cln.lab)
    print(f"www/{name}: n={g.n} m={g.num_edges} K={K} labels {len(raw.lab)} -> {len(cln.lab)}")


def lp_label_sets(n: int, gmax: int, seed: int) -> np.ndarray:
    """Propagation labels for the assembly: groups of random sizes up to
    gmax (half of them single vertices) with random label values in [0, n);
    values that collide merge groups, so some exceed gmax."""
    rng = np.random.default_rng(seed)
    lab = np.empty(n, np.int32)
    perm = rng.permutation(n)
    v = 0
    while v < n:
        sz = int(min(n - v, rng.integers(1, gmax + 1) if rng.random() < 0.5 else 1))
        lab[perm[v:v + sz]] = rng.integers(0, n)
        v += sz
    return lab


def make_lp():
    """The reference's LP group assembly (CDLP_group.cuh:39-100, compiled in
    place by oracle/Makefile into _ref/libcdlp_ref.so) on fixed propagation
    labels: the deterministic half of generate_Group_CDLP."""
    R = O.ReferenceLP()
    cases = {}
    for gseed in (0, 1):
        g = H.HostGraph.chung_lu(3000, 8, 2.2, 300, 1, 100, seed=gseed)
        for gmax in (1, 5, 64, 1024):
            lab = lp_label_sets(g.n, gmax, seed=100 * gseed + gmax)
            gov, ng = R.assemble(g, lab, gmax)
            key = f"g{gseed}_m{gmax}"
            cases[key + "_labels"] = lab
            cases[key + "_gov"] = gov
    os.makedirs(os.path.join(OUT, "lp"), exist_ok=True)
    np.savez_compressed(os.path.join(OUT, "lp", "assembly.npz"), **cases)
    print(f"lp/assembly: {len(cases) // 2} label sets")


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    O.build(ref_dir)
    # the reference's own fixture graphs (ids re-ranked by degree, ties by id)
    for fname, K in (("simple_iterative_tests.txt", 5), ("euroroad2.txt", 5)):
        p = os.path.join(ref_dir, "data", fname)
        if os.path.exists(p):
            g = H.HostGraph.read_text(p, rank_by_degree=True)
            make("ref_" + fname.split(".")[0], g, K, full=True)
    # config-1 shape: ER n=1000, m=5000, w in [1,100], K=5 (labels pinned by digest)
    make("er_1000_5000_k5", H.HostGraph.erdos_renyi(1000, 5000, 1, 100, seed=0x48534C44 ^ 1), 5, full=False,
         nq=10000)
    make("er_200_1000_k5", H.HostGraph.erdos_renyi(200, 1000, 1, 100, seed=5), 5, full=True)
    make("cl_2000_k4", H.HostGraph.chung_lu(2000, 8, 2.2, 200, 1, 100, seed=6), 4, full=True)
    make("ba_800_k6", H.HostGraph.barabasi_albert(800, 3, 1, 1000, seed=7), 6, full=True)
    make("er_300_unit_k3", H.HostGraph.erdos_renyi(300, 900, 1, 1, seed=8), 3, full=True)
    # the 2023WWW generation (generation.h:226-370)
    make_www("er_150_600_k4", H.HostGraph.erdos_renyi(150, 600, 1, 100, seed=9), 4)
    make_www("er_300_unit_k3", H.HostGraph.erdos_renyi(300, 900, 1, 1, seed=8), 3)
    make_www("cl_600_k5", H.HostGraph.chung_lu(600, 6, 2.2, 80, 1, 100, seed=10), 5)
    make_lp()


if __name__ == "__main__":
    main()
