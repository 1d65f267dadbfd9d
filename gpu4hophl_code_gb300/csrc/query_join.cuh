// The (s, t, k) distance join on a resident label index, one warp per query.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222): the
// minimum d1 + d2 over label pairs of a common hub with h1 + h2 <= k;
// INT_MAX for k < 0, then 0 for s == t, then INT_MAX for k == 0, and INT_MAX
// when no pair qualifies.
//
// The merged hub order of the two rows is cut into 32 equal pieces (merge
// path: each lane finds its split with one binary search along its diagonal,
// A's labels ordered before B's on equal hubs), and every lane merges its
// piece with two pointers over the 8-byte label keys.  When the lane takes a
// label of A with hub w, B's run of hub w starts at the lane's B pointer; it
// is scanned with the reference's hop-sum break (possibly past the lane's
// piece).  A warp min combines the lanes.
#pragma once
#include <climits>

#include "hsdl_device.cuh"

namespace hsdl {

// One lane's share of the merge-path join of label rows A (la labels) and B
// (lb labels) under hop bound k >= 1, the merge split over a group of G lanes
// (G = 8, 16 or 32; gl = lane index in the group); returns the lane's minimum
// (INT_MAX if none).  Each label is one key - KT = uint64_t (hub:32 | hop:4 |
// distance:28, format Fmt64) or uint32_t (the compact key, Fmt32) - so hop and
// distance arrive with the hub id and a match needs no dependent load (a
// layout with hub ids and hop|distance words in separate arrays measured
// 238 M q/s against 322 M q/s for the 8-byte keys at n = 1M).  Distances are
// below 2^28 in both formats, so a pair's sum fits int32.  At n = 1M (10M
// queries, compact keys) the 32-bit minimum, the end-of-row sentinel below and
// a two-step unroll took the join from 426 to 465 M q/s; carrying the hubs
// instead of the keys (345), a one-key lookahead per row (463) and 16 or 8
// lanes per query (275 / 170) did not help.
template <int G, class KT, class F>
__device__ inline int lane_merge(const KT* A, int la, const KT* B, int lb, int k, int gl, F f) {
  int best = INT_MAX;
  const int tot = la + lb;
  const int d0 = (int)(((int64_t)tot * gl) / G), d1 = (int)(((int64_t)tot * (gl + 1)) / G);
  int lo = max(0, d0 - lb), hi = min(d0, la);
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (f.hub(A[mid]) <= f.hub(B[d0 - 1 - mid])) lo = mid + 1; else hi = mid;
  }
  // An exhausted row reads as kEnd, whose hub field is above every real hub
  // id (the compact key's H holds 0..n), so the other row's label goes first;
  // inside the piece at most one row is exhausted (it ends by d1 <= la + lb),
  // so equal hubs are always a common hub.
  constexpr KT kEnd = (KT)~(KT)0;
  int ia = lo, ib = d0 - lo;
  KT wa = ia < la ? A[ia] : kEnd;
  KT wb = ib < lb ? B[ib] : kEnd;
#pragma unroll 2
  for (int step = d0; step < d1; step++) {
    const uint32_t ha = f.hub(wa), hb = f.hub(wb);
    const bool take_a = ha <= hb;  // A's label first on equal hubs
    if (ha == hb) {                // a common hub: B's run of it starts at ib
      const int h1 = (int)f.hop(wa);
      if (h1 <= k) {
        const int da = (int)f.dist(wa);
        KT xb = wb;  // its hub is ha
        for (int p = ib;;) {
          if (h1 + (int)f.hop(xb) > k) break;  // rows are hop-sorted within a hub
          best = min(best, da + (int)f.dist(xb));
          if (++p >= lb) break;
          xb = B[p];
          if (f.hub(xb) != ha) break;
        }
      }
    }
    ia += take_a ? 1 : 0;
    ib += take_a ? 0 : 1;
    const int at = take_a ? ia : ib;
    const int lim = take_a ? la : lb;
    const KT nxt = at < lim ? (take_a ? A : B)[at] : kEnd;
    wa = take_a ? nxt : wa;
    wb = take_a ? wb : nxt;
  }
  return best;
}

// Min over the G lanes of each group (every lane of the warp must call it).
template <int G>
__device__ inline int group_min(int v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// TMA bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, multiple of 16).
// A prefetch changes no memory the program sees, so the asm carries no
// "memory" clobber: with one, it fenced the compiler's scheduling of the
// surrounding loads.
__device__ inline void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes));
}

// Prefetches the 16-byte aligned spans holding rows s and t of the key array
// (keys of KT) into L2 (one lane issues).  The key array carries padding so
// the spans stay inside the allocation.
template <class KT>
__device__ inline void prefetch_rows(const int64_t* __restrict__ off, const KT* __restrict__ key, int32_t n, int s,
                                     int t) {
  if (s < 0 || s >= n || t < 0 || t >= n || s == t) return;
  constexpr int64_t per16 = 16 / sizeof(KT);
  const int64_t r[2] = {s, t};
#pragma unroll
  for (int i = 0; i < 2; i++) {
    int64_t a = off[r[i]] & ~(per16 - 1), b = (off[r[i] + 1] + per16 - 1) & ~(per16 - 1);
    if (b > a) prefetch_l2(key + a, (uint32_t)(b - a) * (uint32_t)sizeof(KT));
  }
}

// Checks that decide an answer without a join; returns true and sets *ans.
__device__ inline bool trivial_answer(int32_t n, int s, int t, int k, int32_t* ans) {
  if (s < 0 || s >= n || t < 0 || t >= n) {
    *ans = INT_MAX;  // ids outside the index answer "unreachable"
    return true;
  }
  if (k < 0) {
    *ans = INT_MAX;
    return true;
  }
  if (s == t) {
    *ans = 0;
    return true;
  }
  if (k == 0) {
    *ans = INT_MAX;
    return true;
  }
  return false;
}

// Each group of G lanes answers its own (s, t, k), rows read from global
// memory; every lane of the warp must call it (inactive groups pass
// active = false).  Every lane of a group returns the group's answer.
template <int G, class KT, class F>
__device__ inline int32_t group_query(bool active, int32_t n, const int64_t* __restrict__ off,
                                      const KT* __restrict__ key, int s, int t, int k, F f) {
  int32_t ans = INT_MAX;
  int best = INT_MAX;
  const bool trivial = !active || trivial_answer(n, s, t, k, &ans);
  if (!trivial) {
    int64_t a0 = off[s], a1 = off[s + 1], b0 = off[t], b1 = off[t + 1];
    if (a1 - a0 > b1 - b0) {  // A = the shorter row
      int64_t x = a0; a0 = b0; b0 = x;
      x = a1; a1 = b1; b1 = x;
    }
    best = lane_merge<G>(key + a0, (int)(a1 - a0), key + b0, (int)(b1 - b0), k, lane_id() & (G - 1), f);
  }
  best = group_min<G>(best);
  return trivial ? ans : best;
}

template <int G>
__device__ inline int32_t group_query(bool active, int32_t n, const int64_t* __restrict__ off,
                                      const uint64_t* __restrict__ key, int s, int t, int k) {
  return group_query<G>(active, n, off, key, s, t, k, Fmt64{});
}

// The whole answer of one (s, t, k) by a full warp (every lane must call it).
__device__ inline int32_t warp_query(int32_t n, const int64_t* __restrict__ off, const uint64_t* __restrict__ key,
                                     const int s, const int t, const int k) {
  return group_query<32>(true, n, off, key, s, t, k);
}

}  // namespace hsdl
