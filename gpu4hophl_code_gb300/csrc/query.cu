// Batched (s, t, k) distance queries over a resident label index.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222) - a
// merge-join on hub over the sorted rows L[s] and L[t] that takes the minimum
// d1 + d2 over label pairs of a common hub with h1 + h2 <= k; and the GPU
// gpu_query / get_dis (Query_mdnd/src/gpu_query.cu:5-36,84-178), which needs
// three launches and a synchronisation per query.
//
// Here one warp answers one query and a launch answers the whole batch.  The
// shorter row A is cut into 32 contiguous pieces, one per lane; each lane
// finds where its piece's first hub falls in the longer row B (one binary
// search) and then merges its piece against B with two pointers, streaming
// the 4-byte hub ids of both rows and reading hop and distance only on a hub
// match.  A hub's run in B is scanned with the reference's hop-sum break, and
// the warp reduces the lanes' minima.
#include <algorithm>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kQueryThreads = 256;

__device__ inline int64_t lower_bound_hub(const uint32_t* __restrict__ a, int64_t lo, int64_t hi, uint32_t w) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < w) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kQueryThreads) k_query(int32_t n, int64_t nq, const int32_t* __restrict__ qs,
                                                         const int32_t* __restrict__ qt,
                                                         const int32_t* __restrict__ qk,
                                                         const int64_t* __restrict__ off,
                                                         const uint32_t* __restrict__ hub,
                                                         const uint32_t* __restrict__ hd,
                                                         int32_t* __restrict__ out) {
  const int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t q = warp; q < nq; q += nwarps) {
    const int s = qs[q], t = qt[q], k = qk[q];
    long long best = INT_MAX;
    if (s < 0 || s >= n || t < 0 || t >= n) {
      best = INT_MAX;  // ids outside the index answer "unreachable"
    } else if (k < 0) {
      best = INT_MAX;
    } else if (s == t) {
      best = 0;
    } else if (k == 0) {
      best = INT_MAX;
    } else {
      int64_t a0 = off[s], a1 = off[s + 1], b0 = off[t], b1 = off[t + 1];
      if (a1 - a0 > b1 - b0) {  // A = the shorter row
        int64_t x = a0; a0 = b0; b0 = x;
        x = a1; a1 = b1; b1 = x;
      }
      const int64_t la = a1 - a0;
      const int64_t pa = a0 + (la * lane) / 32, pe = a0 + (la * (lane + 1)) / 32;
      if (pa < pe) {
        int64_t pb = lower_bound_hub(hub, b0, b1, __ldg(hub + pa));
        for (int64_t i = pa; i < pe && pb < b1; i++) {
          const uint32_t w = __ldg(hub + i);
          uint32_t hb = __ldg(hub + pb);
          while (hb < w && ++pb < b1) hb = __ldg(hub + pb);
          if (pb >= b1) break;
          if (hb != w) continue;
          const uint32_t xa = __ldg(hd + i);
          const int h1 = (int)hd_hop(xa);
          if (h1 > k) continue;
          const long long d1 = hd_dist(xa);
          for (int64_t p = pb; p < b1 && __ldg(hub + p) == w; p++) {
            const uint32_t xb = __ldg(hd + p);
            if (h1 + (int)hd_hop(xb) > k) break;  // rows are hop-sorted within a hub
            const long long c = d1 + hd_dist(xb);
            best = c < best ? c : best;
          }
        }
      }
      best = warp_min_ll(best);
    }
    if (lane == 0) out[q] = best >= INT_MAX ? INT_MAX : (int32_t)best;
  }
}

}  // namespace

int query_device(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                 int32_t* out, cudaStream_t st) {
  if (nq <= 0) return HSDL_OK;
  const int sms = device_sm_count();
  int64_t warps_needed = nq;
  int64_t blocks = (warps_needed * 32 + kQueryThreads - 1) / kQueryThreads;
  int64_t max_blocks = (int64_t)sms * 16;
  k_query<<<(unsigned)std::min(blocks, max_blocks), kQueryThreads, 0, st>>>(idx->n, nq, s, t, k, idx->off.p,
                                                                             idx->hub.p, idx->hd.p, out);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

}  // namespace hsdl
