// Batched (s, t, k) distance queries over a resident label index.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222), and the
// GPU gpu_query / get_dis (Query_mdnd/src/gpu_query.cu:5-36,84-178), which
// needs three launches and a synchronisation per query.
//
// One launch answers the whole batch; a group of lanes (a warp by default)
// answers one query with the merge-path join of query_join.cuh, reading both
// rows through L1/L2.  No shared memory is used, so occupancy stays high; the
// grid is one resident wave with a grid-stride loop.  Optionally each warp
// issues TMA bulk prefetches (cp.async.bulk.prefetch.L2) of the rows of the
// queries it will take a few steps later.  Staging both rows in shared memory
// first (coalesced loads into per-warp buffers) measured 81-195 M q/s against
// 238 M q/s for the global-memory join: the buffers cut occupancy more than
// the shorter load chains gained.
#include <algorithm>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"
#include "query_join.cuh"

namespace hsdl {

namespace {

// Each group of G lanes answers one query; the warp takes 32/G queries per
// step in grid-stride order.  With PF, the warp prefetches the rows of the
// queries `ahead` steps further on into L2 (a separate instantiation, so the
// plain kernel carries no prefetch code at all).
// (Capping it at 32 registers for 64 resident warps per SM, against 38 and 48
// warps, cut the rate from 322 M to 221 M q/s at n = 1M.)
// Over 4-byte keys the kernel is held to 32 registers (two blocks of 1,024
// threads, 64 warps per SM; it compiles without spills): at n = 1M 426 M q/s
// against 391 M at 38 registers (48 warps).  Over 8-byte keys the same cap
// spills and cost a third of the rate, so that join keeps its registers.
template <int G, bool PF, class KT, class F>
__global__ void __launch_bounds__(1024, sizeof(KT) == 4 ? 2 : 1)
    k_query(int32_t n, int64_t nq, const int32_t* __restrict__ qs, const int32_t* __restrict__ qt,
            const int32_t* __restrict__ qk, const int64_t* __restrict__ off, const KT* __restrict__ key,
            int32_t* __restrict__ out, int ahead, F f) {
  constexpr int Q = 32 / G;  // queries per warp step
  const int lane = lane_id(), grp = lane / G, gl = lane & (G - 1);
  const int64_t step = (((int64_t)gridDim.x * blockDim.x) >> 5) * Q;
  for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * Q; base < nq; base += step) {
    if (PF && gl == 0) {
      const int64_t p = base + (int64_t)ahead * step + grp;
      if (p < nq) prefetch_rows(off, key, n, qs[p], qt[p]);
    }
    const int64_t q = base + grp;
    const bool active = q < nq;
    const int s = active ? qs[q] : 0, t = active ? qt[q] : 0, k = active ? qk[q] : 0;
    const int32_t ans = group_query<G>(active, n, off, key, s, t, k, f);
    if (active && gl == 0) out[q] = ans;
  }
}

template <int G, bool PF, class KT, class F>
int launch_query(hsdl_index_impl* idx, const KT* key, F f, int64_t nq, const int32_t* s, const int32_t* t,
                 const int32_t* k, int32_t* out, cudaStream_t st) {
  const int sms = device_sm_count();
  const int64_t warps = (nq + (32 / G) - 1) / (32 / G);
  // a batch too small to give every SM a block runs in smaller blocks, so
  // that it spreads over all SMs instead of crowding a few (a 1,024-thread
  // block puts 32 of the batch's queries on one SM)
  int threads = idx->q_threads;
  if (warps * 32 < (int64_t)sms * threads)
    threads = (int)std::max<int64_t>(64, std::min<int64_t>(threads, (warps * 32 / sms) & ~(int64_t)31));
  int64_t blocks = (warps * 32 + threads - 1) / threads;
  int64_t max_blocks = (int64_t)sms * resident_blocks(k_query<G, PF, KT, F>, threads);
  k_query<G, PF, KT, F><<<(unsigned)std::min(blocks, max_blocks), threads, 0, st>>>(idx->n, nq, s, t, k, idx->off.p,
                                                                                     key, out, idx->q_ahead, f);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

template <int G, bool PF>
int launch_query(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k, int32_t* out,
                 cudaStream_t st) {
  if (idx->key32.p) return launch_query<G, PF>(idx, idx->key32.p, idx->fmt32, nq, s, t, k, out, st);
  return launch_query<G, PF>(idx, idx->key.p, Fmt64{}, nq, s, t, k, out, st);
}

// Largest distance field over the 8-byte keys.
__global__ void k_max_dist(int64_t total, const uint64_t* __restrict__ key, unsigned int* out) {
  uint32_t m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, lkey_dist(key[i]));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane_id() == 0) atomicMax(out, m);
}

__global__ void k_pack32(int64_t total, const uint64_t* __restrict__ key, uint32_t* __restrict__ key32, Fmt32 f) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t x = key[i];
    key32[i] = f.pack(lkey_hub(x), lkey_hop(x), lkey_dist(x));
  }
}

int bits_for(uint32_t v) {  // bits needed to hold 0..v (at least 1)
  int b = 1;
  while (b < 32 && (v >> b) != 0) b++;
  return b;
}

// Smallest index of a query naming a vertex outside [0, n) (stays all-ones if none).
__global__ void k_first_bad_id(int32_t n, int64_t nq, const int32_t* __restrict__ qs, const int32_t* __restrict__ qt,
                               unsigned long long* first) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = qs[i], t = qt[i];
    if (s < 0 || s >= n || t < 0 || t >= n) atomicMin(first, (unsigned long long)i);
  }
}

}  // namespace

int first_bad_query(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, unsigned long long* d_first,
                    cudaStream_t st) {
  HSDL_CUDA(cudaMemsetAsync(d_first, 0xFF, sizeof(unsigned long long), st));
  if (nq <= 0) return HSDL_OK;
  const int sms = device_sm_count();
  k_first_bad_id<<<sms * 4, 256, 0, st>>>(idx->n, nq, s, t, d_first);
  HSDL_LAUNCHED();
  return HSDL_OK;
}

template <int G, bool PF>
int preload_variant() {
  cudaFuncAttributes a;
  HSDL_CUDA(cudaFuncGetAttributes(&a, k_query<G, PF, uint64_t, Fmt64>));
  HSDL_CUDA(cudaFuncGetAttributes(&a, k_query<G, PF, uint32_t, Fmt32>));
  return HSDL_OK;
}

int preload_query_kernels() {
  HSDL_TRY((preload_variant<8, false>()));
  HSDL_TRY((preload_variant<8, true>()));
  HSDL_TRY((preload_variant<16, false>()));
  HSDL_TRY((preload_variant<16, true>()));
  HSDL_TRY((preload_variant<32, false>()));
  HSDL_TRY((preload_variant<32, true>()));
  cudaFuncAttributes a;
  HSDL_CUDA(cudaFuncGetAttributes(&a, k_first_bad_id));
  return HSDL_OK;
}

// Builds the compact 4-byte query keys of a finished index when its ranges fit
// (hub:H | hop:P | distance:D, see Fmt32), else releases them; the query
// kernels use them when present.  Synchronises the index's stream.
int make_query_keys(hsdl_index_impl* idx) {
  cudaStream_t st = idx->stream;
  idx->key32.release();
  if (!idx->q_tuned) {  // the 8-byte join's default shape
    idx->q_threads = 512;
    idx->q_ahead = 0;
  }
  // H holds 0..n, one more than the largest hub id, so an all-ones key reads
  // as a hub above every real one (the join's end-of-row sentinel)
  const int H = bits_for((uint32_t)std::max(0, idx->n)), P = bits_for((uint32_t)idx->K);
  const int D = 32 - H - P;
  if (D < 1 || idx->total <= 0) return HSDL_OK;
  const int sms = device_sm_count();
  DevBuf<unsigned int> mx;
  HSDL_TRY(mx.alloc(1, st));
  HSDL_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned int), st));
  k_max_dist<<<sms * 8, 256, 0, st>>>(idx->total, idx->key.p, mx.p);
  HSDL_LAUNCHED();
  unsigned int maxd = 0;
  HSDL_CUDA(cudaMemcpyAsync(&maxd, mx.p, sizeof(maxd), cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  mx.release();
  if (D < 32 && (maxd >> D) != 0) return HSDL_OK;
  // default launch shape of the join over 4-byte keys: 1,024 threads per block
  // (two blocks fill an SM's 64 warps at its 32 registers), no prefetch: at
  // n = 1M 426 M q/s, against 405 M for 512 threads and 406 M for 1,024 with
  // an L2 prefetch of the rows one query ahead (which also read 1.5x the
  // DRAM bytes: prefetched rows were evicted before their join)
  if (!idx->q_tuned) {
    idx->q_threads = 1024;
    idx->q_ahead = 0;
  }
  Fmt32 f{(uint32_t)(P + D), (uint32_t)D};
  HSDL_TRY(idx->key32.alloc(idx->total + kRowPad, st));
  HSDL_CUDA(cudaMemsetAsync(idx->key32.p + idx->total, 0xFF, sizeof(uint32_t) * kRowPad, st));
  k_pack32<<<sms * 8, 256, 0, st>>>(idx->total, idx->key.p, idx->key32.p, f);
  HSDL_LAUNCHED();
  idx->fmt32 = f;
  HSDL_CUDA(cudaStreamSynchronize(st));
  return HSDL_OK;
}

int query_device(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                 int32_t* out, cudaStream_t st) {
  if (nq <= 0) return HSDL_OK;
  const bool pf = idx->q_ahead > 0;
  switch (idx->q_lanes) {
    case 8:
      return pf ? launch_query<8, true>(idx, nq, s, t, k, out, st) : launch_query<8, false>(idx, nq, s, t, k, out, st);
    case 16:
      return pf ? launch_query<16, true>(idx, nq, s, t, k, out, st)
                : launch_query<16, false>(idx, nq, s, t, k, out, st);
    default:
      return pf ? launch_query<32, true>(idx, nq, s, t, k, out, st)
                : launch_query<32, false>(idx, nq, s, t, k, out, st);
  }
}

}  // namespace hsdl
