// Degree ranking and CSR construction on the device.
//
// Reference: graph_v_of_v_update_vertexIDs_by_degrees_large_to_small
// (CPU_HopHL/include/graph_v_of_v/graph_v_of_v_update_vertexIDs_by_degrees_large_to_small.h:14-40)
// ranks vertices by degree, largest first, and toCSR / graph_v_of_v_to_CSR
// (Hybrid_Generation_Clean/include/graph/csr_graph.hpp:38-115,117-196) lays the
// relabelled graph out as CSR.  The reference's rank sort is std::sort, whose
// order among equal degrees is unspecified; here ties go by id (smaller
// first), the same rule as the host path (graph_gen.cpp: build_ranked_csr), and
// the CSR is bit-identical to the host path's: rows in rank order, each row
// sorted by neighbour.
//
// Steps, all on the device from an undirected edge list:
//   1. degrees (atomic adds) and the largest degree;
//   2. rank order: a stable least-significant-digit sort of the vertex ids by
//      inverted degree, one bit per pass (a stable partition through an
//      exclusive scan), over only the bits the largest degree needs; ids start
//      ascending, so equal degrees stay in id order;
//   3. row offsets: the degrees in rank order, exclusively scanned;
//   4. fill: both directions of every edge, placed by an atomic cursor per row;
//   5. each row sorted by (neighbour, weight) with the index's row sort, and
//      checked for repeated neighbours (the graph must be simple).
#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kGThreads = 256;

__global__ void k_check_edges(int32_t n, int64_t m, const int32_t* __restrict__ a, const int32_t* __restrict__ b,
                              const int32_t* __restrict__ w, unsigned long long* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t x = a[i], y = b[i];
    if (x < 0 || x >= n || y < 0 || y >= n || x == y || w[i] < 1) atomicMin(bad, (unsigned long long)i);
  }
}

__global__ void k_degrees(int64_t m, const int32_t* __restrict__ a, const int32_t* __restrict__ b,
                          int32_t* __restrict__ deg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    atomicAdd(&deg[a[i]], 1);
    atomicAdd(&deg[b[i]], 1);
  }
}

__global__ void k_max_deg(int32_t n, const int32_t* __restrict__ deg, int32_t* __restrict__ out) {
  int32_t mx = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    mx = max(mx, deg[v]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane_id() == 0) atomicMax(out, mx);
}

__global__ void k_iota(int32_t n, int32_t* __restrict__ ids) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    ids[v] = (int32_t)v;
}

// flag = bit `bit` of the id's inverted degree (set = goes after the clear ones)
__global__ void k_zero_flags(int32_t n, const int32_t* __restrict__ ids, const int32_t* __restrict__ deg,
                             int32_t maxdeg, int bit, int64_t* __restrict__ zero) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    zero[i] = (((maxdeg - deg[ids[i]]) >> bit) & 1) ? 0 : 1;
}

__global__ void k_partition(int32_t n, const int32_t* __restrict__ ids, const int64_t* __restrict__ zero,
                            const int64_t* __restrict__ zero_before, int32_t* __restrict__ out) {
  const int64_t zeros = zero_before[n];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t zb = zero_before[i];
    out[zero[i] ? zb : zeros + (i - zb)] = ids[i];
  }
}

__global__ void k_rank_tables(int32_t n, const int32_t* __restrict__ new_to_old, const int32_t* __restrict__ deg,
                              int32_t* __restrict__ old_to_new, int64_t* __restrict__ deg_new) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = new_to_old[i];
    old_to_new[v] = (int32_t)i;
    deg_new[i] = deg[v];
  }
}

__global__ void k_fill(int64_t m, const int32_t* __restrict__ a, const int32_t* __restrict__ b,
                       const int32_t* __restrict__ w, const int32_t* __restrict__ old_to_new,
                       unsigned long long* __restrict__ cursor, uint64_t* __restrict__ key) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t x = (uint32_t)old_to_new[a[i]], y = (uint32_t)old_to_new[b[i]], wt = (uint32_t)w[i];
    key[atomicAdd(&cursor[x], 1ull)] = ((uint64_t)y << 32) | wt;
    key[atomicAdd(&cursor[y], 1ull)] = ((uint64_t)x << 32) | wt;
  }
}

// Splits the sorted (neighbour << 32 | weight) keys into the adjacency array;
// records the first entry that repeats its predecessor's neighbour in its row.
__global__ void k_unpack(int32_t n, const int64_t* __restrict__ rp, const uint64_t* __restrict__ key,
                         int2* __restrict__ adj, unsigned long long* dup, int32_t* __restrict__ wmax) {
  int32_t mw = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t e = rp[v]; e < rp[v + 1]; e++) {
      const uint64_t k = key[e];
      const int32_t nb = (int32_t)(k >> 32), wt = (int32_t)(uint32_t)k;
      adj[e] = make_int2(nb, wt);
      mw = max(mw, wt);
      if (e > rp[v] && (int32_t)(key[e - 1] >> 32) == nb) atomicMin(dup, (unsigned long long)v);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mw = max(mw, __shfl_xor_sync(0xffffffffu, mw, o));
  if (lane_id() == 0) atomicMax(wmax, mw);
}

}  // namespace

int build_graph_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                           bool rank_by_degree, int32_t* h_new_to_old, hsdl_graph_impl* g) {
  cudaStream_t st = nullptr;  // the graph's buffers live on the default stream
  const int sms = device_sm_count();
  const int grid = sms * 8;
  DevBuf<int32_t> ea, eb, ew, deg, ids, ids2, o2n, scal;
  DevBuf<int64_t> zero, zero_before, deg_new;
  DevBuf<unsigned long long> cursor, flags;
  DevBuf<uint64_t> key;
  DevBuf<int32_t> dummy;
  auto release = [&]() {
    ea.release(); eb.release(); ew.release(); deg.release(); ids.release(); ids2.release(); o2n.release();
    scal.release(); zero.release(); zero_before.release(); deg_new.release(); cursor.release(); flags.release();
    key.release(); dummy.release();
  };
  struct Guard {
    std::function<void()> f;
    ~Guard() { f(); }
  } guard{release};
  const int64_t me = std::max<int64_t>(1, m);
  HSDL_TRY(ea.alloc(me, st));
  HSDL_TRY(eb.alloc(me, st));
  HSDL_TRY(ew.alloc(me, st));
  HSDL_TRY(flags.alloc(2, st));
  HSDL_TRY(scal.alloc(2, st));
  if (m > 0) {
    HSDL_CUDA(cudaMemcpyAsync(ea.p, a, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaMemcpyAsync(eb.p, b, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaMemcpyAsync(ew.p, w, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st));
  }
  HSDL_CUDA(cudaMemsetAsync(flags.p, 0xFF, 2 * sizeof(unsigned long long), st));
  HSDL_CUDA(cudaMemsetAsync(scal.p, 0, 2 * sizeof(int32_t), st));
  k_check_edges<<<grid, kGThreads, 0, st>>>(n, m, ea.p, eb.p, ew.p, flags.p);
  HSDL_LAUNCHED();
  unsigned long long bad = 0;
  HSDL_CUDA(cudaMemcpyAsync(&bad, flags.p, sizeof(bad), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  if (bad != ~0ull) {
    set_error("edge " + std::to_string(bad) + ": endpoints must be distinct ids in [0, n) and the weight >= 1");
    return HSDL_ERR_INVALID;
  }
  // 1. degrees
  HSDL_TRY(deg.alloc(n, st));
  HSDL_CUDA(cudaMemsetAsync(deg.p, 0, sizeof(int32_t) * n, st));
  k_degrees<<<grid, kGThreads, 0, st>>>(m, ea.p, eb.p, deg.p);
  HSDL_LAUNCHED();
  k_max_deg<<<grid, kGThreads, 0, st>>>(n, deg.p, scal.p);
  HSDL_LAUNCHED();
  int32_t maxdeg = 0;
  HSDL_CUDA(cudaMemcpyAsync(&maxdeg, scal.p, sizeof(maxdeg), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  // 2. rank order
  HSDL_TRY(ids.alloc(n, st));
  HSDL_TRY(ids2.alloc(n, st));
  k_iota<<<grid, kGThreads, 0, st>>>(n, ids.p);
  HSDL_LAUNCHED();
  if (rank_by_degree) {
    int bits = 0;
    while ((1ll << bits) <= (int64_t)maxdeg) bits++;
    HSDL_TRY(zero.alloc(n, st));
    HSDL_TRY(zero_before.alloc((int64_t)n + 1, st));
    for (int bit = 0; bit < bits; bit++) {
      k_zero_flags<<<grid, kGThreads, 0, st>>>(n, ids.p, deg.p, maxdeg, bit, zero.p);
      HSDL_LAUNCHED();
      HSDL_TRY(exclusive_scan_i64(zero.p, zero_before.p, n, st));
      k_partition<<<grid, kGThreads, 0, st>>>(n, ids.p, zero.p, zero_before.p, ids2.p);
      HSDL_LAUNCHED();
      std::swap(ids.p, ids2.p);
    }
  }
  // 3. row offsets in rank order
  HSDL_TRY(o2n.alloc(n, st));
  HSDL_TRY(deg_new.alloc(n, st));
  k_rank_tables<<<grid, kGThreads, 0, st>>>(n, ids.p, deg.p, o2n.p, deg_new.p);
  HSDL_LAUNCHED();
  HSDL_TRY(g->rp.alloc((int64_t)n + 1, st));
  HSDL_TRY(exclusive_scan_i64(deg_new.p, g->rp.p, n, st));
  // 4. fill both directions
  const int64_t m2 = 2 * m;
  HSDL_TRY(cursor.alloc((int64_t)n + 1, st));
  HSDL_CUDA(cudaMemcpyAsync(cursor.p, g->rp.p, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
  HSDL_TRY(key.alloc(std::max<int64_t>(1, m2) + kRowPad, st));
  k_fill<<<grid, kGThreads, 0, st>>>(m, ea.p, eb.p, ew.p, o2n.p, cursor.p, key.p);
  HSDL_LAUNCHED();
  // 5. rows sorted by (neighbour, weight); check the graph is simple
  HSDL_TRY(dummy.alloc(std::max<int64_t>(1, m2) + kRowPad, st));
  HSDL_TRY(sort_rows(n, g->rp.p, key.p, dummy.p, std::max(0, maxdeg), st));
  HSDL_TRY(g->adj.alloc(std::max<int64_t>(1, m2), st));
  k_unpack<<<grid, kGThreads, 0, st>>>(n, g->rp.p, key.p, g->adj.p, flags.p + 1, scal.p + 1);
  HSDL_LAUNCHED();
  unsigned long long dup = 0;
  int32_t wmax = 0;
  HSDL_CUDA(cudaMemcpyAsync(&dup, flags.p + 1, sizeof(dup), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaMemcpyAsync(&wmax, scal.p + 1, sizeof(wmax), cudaMemcpyDeviceToHost, st));
  g->h_rp.resize((size_t)n + 1);
  HSDL_CUDA(cudaMemcpyAsync(g->h_rp.data(), g->rp.p, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
  if (h_new_to_old) HSDL_CUDA(cudaMemcpyAsync(h_new_to_old, ids.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  if (dup != ~0ull) {
    set_error("the edge list repeats an edge (at ranked vertex " + std::to_string(dup) + ")");
    g->rp.release();
    g->adj.release();
    return HSDL_ERR_INVALID;
  }
  g->n = n;
  g->m2 = m2;
  g->max_w = wmax;
  return HSDL_OK;
}

}  // namespace hsdl
