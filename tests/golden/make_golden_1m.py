"""Generates tests/golden/chung_lu_1m_k5.npz: the reference's own output on the
1M-vertex Chung-Lu workload (n = 1,000,000, average degree 10, exponent 2.1,
maximum expected degree 10,000, weights uniform in [1, 100], K = 5, vertices
ranked by degree descending with ties by id - the graph bench.py builds).

The label set is ~520 M labels (8 GB), far too large to commit, so the fixture
holds what pins it:

* sha256 of the offsets (int64[n+1]) and of the (hub, hop, distance) triples
  (int32[total, 3], rows in the reference's order), the label count, and a
  64-bit digest per block of 1,000 vertices (to locate a mismatch);
* answers of the reference's hop_constrained_extract_distance
  (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144) on 100,000
  seeded uniform (s, t, k) queries;
* hop-bounded Bellman-Ford distances
  (CPU_HopHL/include/graph_v_of_v/graph_v_of_v_hop_constrained_shortest_distance.h:7-38)
  for 20,000 sampled (s, t, k): 200 sources x k = 1..5 x 20 targets;
* the reference's phase timers (generation, sortL, canonical repair;
  hop_constrained_two_hop_labels_generation.h:594-629) and the thread count.

It runs the reference's CPU_HopHL compiled in place (oracle/_ref/libhsdl_ref.so,
oracle/Makefile) with every host core, which takes tens of minutes.  Run from the
repository root where a reference checkout exists:
    python tests/golden/make_golden_1m.py [threads]
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "headline", "chung_lu_1m_k5.npz")
N, K = 1_000_000, 5
BF_SOURCES, BF_TARGETS = 200, 20
QUERIES = 100_000


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    O.build()
    R = O.Reference()
    g = bench.make_graph(N)
    t0 = time.time()
    lab = R.build(g, K, threads=threads, clean=True)
    wall = time.time() - t0
    print(f"reference build: {len(lab.lab)} labels in {wall:.1f} s ({lab.info})", flush=True)
    d = bench.label_digests(lab.off, lab.lab)
    s, t, k = bench.make_queries(N, QUERIES, K, seed=bench.PARITY_QUERY_SEED)
    ans = R.query(s, t, k, threads=threads)
    rng = np.random.default_rng(bench.PARITY_BF_SEED)
    srcs = rng.choice(N, BF_SOURCES, replace=False).astype(np.int32)
    bs, bt, bk, bd = [], [], [], []
    for a in srcs:
        for h in range(1, K + 1):
            dist = R.bf(int(a), h)
            tg = rng.integers(0, N, BF_TARGETS).astype(np.int32)
            bs.append(np.full(BF_TARGETS, a, np.int32))
            bt.append(tg)
            bk.append(np.full(BF_TARGETS, h, np.int32))
            bd.append(dist[tg])
    bs, bt, bk, bd = (np.concatenate(x) for x in (bs, bt, bk, bd))
    # the reference's own answers must agree with its Bellman-Ford
    chk = R.query(bs, bt, bk, threads=threads)
    assert np.array_equal(chk, bd), "reference labels disagree with its Bellman-Ford"
    times = np.array([lab.info["t_init"], lab.info["t_gen"], lab.info["t_sort"], lab.info["t_clean"]])
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    np.savez_compressed(OUT, n=np.int32(N), K=np.int32(K), graph_digest=np.array(bench.graph_digest(g)),
                        off_digest=np.array(d["off"]), hhd_digest=np.array(d["hhd"]), block_digests=d["blocks"],
                        n_labels=np.int64(len(lab.lab)), q_s=s, q_t=t, q_k=k, q_ans=ans, bf_s=bs, bf_t=bt,
                        bf_k=bk, bf_dist=bd, ref_times=times, ref_threads=np.int32(threads),
                        ref_wall_s=np.float64(wall))
    print(f"wrote {OUT}: {len(lab.lab)} labels, {len(bs)} Bellman-Ford pairs, times {times}")


if __name__ == "__main__":
    main()
