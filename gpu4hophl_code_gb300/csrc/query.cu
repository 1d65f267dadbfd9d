// Batched (s, t, k) distance queries over a resident label index.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222), and the
// GPU gpu_query / get_dis (Query_mdnd/src/gpu_query.cu:5-36,84-178), which
// needs three launches and a synchronisation per query.
//
// One launch answers the whole batch; one warp answers one query with the
// merge-path join of query_join.cuh, reading both rows through L1/L2.  The
// join is a chain of dependent loads, so each warp hides its latency by
// issuing TMA bulk prefetches (cp.async.bulk.prefetch.L2) of the rows of the
// queries it will take next: by the time it gets there, their rows sit in
// L2.  No shared memory is used, so occupancy stays high.
#include <algorithm>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"
#include "query_join.cuh"

namespace hsdl {

namespace {

// Each group of G lanes answers one query; the warp takes 32/G queries per
// step in grid-stride order.  `ahead` > 0 makes the warp prefetch the rows of
// the queries `ahead` steps further on into L2.
template <int G>
__global__ void k_query(int32_t n, int64_t nq, const int32_t* __restrict__ qs, const int32_t* __restrict__ qt,
                        const int32_t* __restrict__ qk, const int64_t* __restrict__ off,
                        const uint32_t* __restrict__ hub, const uint32_t* __restrict__ hd, int32_t* __restrict__ out,
                        int ahead) {
  constexpr int Q = 32 / G;  // queries per warp step
  const int lane = lane_id(), grp = lane / G, gl = lane & (G - 1);
  const int64_t step = (((int64_t)gridDim.x * blockDim.x) >> 5) * Q;
  for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * Q; base < nq; base += step) {
    if (ahead > 0 && gl == 0) {
      const int64_t p = base + (int64_t)ahead * step + grp;
      if (p < nq) prefetch_rows(off, hub, n, qs[p], qt[p]);
    }
    const int64_t q = base + grp;
    const bool active = q < nq;
    const int s = active ? qs[q] : 0, t = active ? qt[q] : 0, k = active ? qk[q] : 0;
    const int32_t ans = group_query<G>(active, n, off, hub, hd, s, t, k);
    if (active && gl == 0) out[q] = ans;
  }
}

// Staged variant: the warp first copies the hub ids of both rows into its own
// shared-memory buffer of `cap` words - coalesced loads, eight per lane in
// flight, so a row costs one memory round trip instead of the merge-path
// search's chain of dependent loads - then joins there.  Pairs of rows longer
// than the buffer take the global-memory join.
__global__ void k_query_staged(int32_t n, int64_t nq, const int32_t* __restrict__ qs, const int32_t* __restrict__ qt,
                               const int32_t* __restrict__ qk, const int64_t* __restrict__ off,
                               const uint32_t* __restrict__ hub, const uint32_t* __restrict__ hd,
                               int32_t* __restrict__ out, int cap) {
  extern __shared__ uint32_t qbuf[];
  const int lane = lane_id();
  uint32_t* buf = qbuf + (int64_t)(threadIdx.x >> 5) * cap;
  const int64_t step = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nq; q += step) {
    const int s = qs[q], t = qt[q], k = qk[q];
    int32_t ans;
    if (!trivial_answer(n, s, t, k, &ans)) {  // uniform over the warp
      int64_t a0 = off[s], a1 = off[s + 1], b0 = off[t], b1 = off[t + 1];
      if (a1 - a0 > b1 - b0) {  // A = the shorter row
        int64_t x = a0; a0 = b0; b0 = x;
        x = a1; a1 = b1; b1 = x;
      }
      const int la = (int)(a1 - a0), lb = (int)(b1 - b0), tot = la + lb;
      long long best;
      if (tot <= cap) {
        for (int p0 = 0; p0 < tot; p0 += 256) {
          uint32_t v[8];
#pragma unroll
          for (int u = 0; u < 8; u++) {
            const int p = p0 + u * 32 + lane;
            v[u] = p < tot ? hub[p < la ? a0 + p : b0 + (p - la)] : 0u;
          }
#pragma unroll
          for (int u = 0; u < 8; u++) {
            const int p = p0 + u * 32 + lane;
            if (p < tot) buf[p] = v[u];
          }
        }
        __syncwarp();
        best = lane_merge<32>(buf, la, buf + la, lb, hd + a0, hd + b0, k, lane);
        __syncwarp();  // the buffer is rewritten by the next query
      } else {
        best = lane_merge<32>(hub + a0, la, hub + b0, lb, hd + a0, hd + b0, k, lane);
      }
      ans = clamp_answer(group_min<32>(best));
    }
    if (lane == 0) out[q] = ans;
  }
}

int launch_staged(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                  int32_t* out, cudaStream_t st) {
  const int sms = device_sm_count();
  const int threads = idx->q_threads, cap = idx->q_stage;
  const size_t smem = (size_t)(threads / 32) * cap * sizeof(uint32_t);
  HSDL_CUDA(cudaFuncSetAttribute(k_query_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t blocks = (nq * 32 + threads - 1) / threads;
  const int64_t max_blocks = (int64_t)sms * resident_blocks(k_query_staged, threads, smem);
  k_query_staged<<<(unsigned)std::min(blocks, max_blocks), threads, smem, st>>>(
      idx->n, nq, s, t, k, idx->off.p, idx->hub.p, idx->hd.p, out, cap);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

template <int G>
int launch_query(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k, int32_t* out,
                 cudaStream_t st) {
  const int sms = device_sm_count();
  const int threads = idx->q_threads;
  const int64_t warps = (nq + (32 / G) - 1) / (32 / G);
  int64_t blocks = (warps * 32 + threads - 1) / threads;
  int64_t max_blocks = (int64_t)sms * resident_blocks(k_query<G>, threads);
  k_query<G><<<(unsigned)std::min(blocks, max_blocks), threads, 0, st>>>(idx->n, nq, s, t, k, idx->off.p,
                                                                          idx->hub.p, idx->hd.p, out, idx->q_ahead);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

}  // namespace

int query_device(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                 int32_t* out, cudaStream_t st) {
  if (nq <= 0) return HSDL_OK;
  if (idx->q_stage > 0) return launch_staged(idx, nq, s, t, k, out, st);
  switch (idx->q_lanes) {
    case 8:
      return launch_query<8>(idx, nq, s, t, k, out, st);
    case 16:
      return launch_query<16>(idx, nq, s, t, k, out, st);
    default:
      return launch_query<32>(idx, nq, s, t, k, out, st);
  }
}

int query_error(hsdl_index_impl* idx) {
  if (!idx->qerr.p) return HSDL_OK;
  unsigned int e = 0;
  HSDL_CUDA(cudaMemcpy(&e, idx->qerr.p, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) {
    HSDL_CUDA(cudaMemset(idx->qerr.p, 0, sizeof(e)));
    set_error("a bounded wait for staged label rows ran out in the query kernel");
    return HSDL_ERR_TIMEOUT;
  }
  return HSDL_OK;
}

}  // namespace hsdl
