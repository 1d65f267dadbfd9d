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
// lanes take 32 consecutive labels of the shorter row at a time; each lane
// finds its hub in the longer row by binary search on the packed keys (rows
// are sorted by key = (hub, hop, distance)), scans that hub's run, and the
// warp reduces with a min.  The search window of the next 32 labels starts
// where the last lane's search ended.
#include <algorithm>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kQueryThreads = 256;

__device__ inline int64_t lower_bound_key(const uint64_t* __restrict__ a, int64_t lo, int64_t hi, uint64_t key) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kQueryThreads) k_query(int32_t n, int64_t nq, const int32_t* __restrict__ qs,
                                                         const int32_t* __restrict__ qt,
                                                         const int32_t* __restrict__ qk,
                                                         const int64_t* __restrict__ off,
                                                         const uint64_t* __restrict__ keys,
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
      if (a1 - a0 > b1 - b0) {  // probe with the shorter row
        int64_t x = a0; a0 = b0; b0 = x;
        x = a1; a1 = b1; b1 = x;
      }
      int64_t window = b0;
      for (int64_t j0 = a0; j0 < a1; j0 += 32) {
        int64_t j = j0 + lane;
        int64_t pos = window;
        if (j < a1) {
          uint64_t ka = __ldg(keys + j);
          int h1 = (int)lkey_hop(ka);
          uint32_t w = lkey_hub(ka);
          pos = lower_bound_key(keys, window, b1, lkey(w, 0, 0));
          if (h1 <= k) {
            for (int64_t p = pos; p < b1; p++) {
              uint64_t kb = __ldg(keys + p);
              if (lkey_hub(kb) != w) break;
              if (h1 + (int)lkey_hop(kb) > k) break;  // rows are hop-sorted within a hub
              long long c = (long long)lkey_dist(ka) + lkey_dist(kb);
              best = c < best ? c : best;
            }
          }
        }
        // next chunk's hubs are larger: search from the largest position found
        int64_t mx = pos;
        for (int o = 16; o > 0; o >>= 1) {
          int64_t y = __shfl_xor_sync(0xffffffffu, mx, o);
          mx = y > mx ? y : mx;
        }
        window = mx;
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
                                                                             idx->keys.p, out);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

}  // namespace hsdl
