// Batched (s, t, k) distance queries over a resident label index.
//
// Reference: hop_constrained_extract_distance
// (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222), and the
// GPU gpu_query / get_dis (Query_mdnd/src/gpu_query.cu:5-36,84-178), which
// needs three launches and a synchronisation per query.
//
// One launch answers the whole batch; one warp answers one query with the
// merge-path join of query_join.cuh.  Each warp keeps a two-stage pipeline in
// shared memory: while it merges query i out of one stage, the hub rows of its
// next query are already arriving in the other stage through TMA bulk copies
// (cp.async.bulk global -> shared, completion on an mbarrier).  A row is
// copied as the 16-byte aligned span that contains it (the index arrays carry
// padding so the span never leaves the allocation).  Queries whose two rows do
// not fit a stage are joined straight from global memory.  Every mbarrier wait
// is bounded; a wait that runs out records an error the host turns into
// HSDL_ERR_TIMEOUT.
#include <algorithm>
#include <climits>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"
#include "query_join.cuh"

namespace hsdl {

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kStageCap = 2048;  // hub ids per stage per warp (8 KB)
constexpr int kWaitSpins = 1 << 22;

__device__ inline uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ inline void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ inline void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ inline void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ inline bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
__device__ inline void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// generic-proxy reads of a stage must be ordered before the next bulk write
__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ inline bool bounded_wait(uint64_t* bar, uint32_t phase) {
  for (int i = 0; i < kWaitSpins; i++)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

struct Plan {
  int32_t ans;     // answer when trivial
  int trivial;
  int staged;      // rows copied into the stage
  int64_t a0, b0;  // row starts (A = shorter row)
  int la, lb, k;
  int offA, offB;  // row starts inside the stage
  int spanA, spanB;
  int64_t sA, sB;  // aligned span starts in the hub array
};

__device__ inline Plan make_plan(int64_t q, int32_t n, const int32_t* __restrict__ qs, const int32_t* __restrict__ qt,
                                 const int32_t* __restrict__ qk, const int64_t* __restrict__ off) {
  Plan p;
  const int s = qs[q], t = qt[q], k = qk[q];
  p.k = k;
  p.staged = 0;
  p.trivial = trivial_answer(n, s, t, k, &p.ans) ? 1 : 0;
  if (p.trivial) return p;
  int64_t a0 = off[s], a1 = off[s + 1], b0 = off[t], b1 = off[t + 1];
  if (a1 - a0 > b1 - b0) {
    int64_t x = a0; a0 = b0; b0 = x;
    x = a1; a1 = b1; b1 = x;
  }
  p.a0 = a0;
  p.b0 = b0;
  p.la = (int)(a1 - a0);
  p.lb = (int)(b1 - b0);
  p.sA = a0 & ~(int64_t)3;
  p.sB = b0 & ~(int64_t)3;
  p.spanA = (int)(((a1 + 3) & ~(int64_t)3) - p.sA);
  p.spanB = (int)(((b1 + 3) & ~(int64_t)3) - p.sB);
  p.offA = (int)(a0 - p.sA);
  p.offB = p.spanA + (int)(b0 - p.sB);
  p.staged = (p.la > 0 && p.lb > 0 && p.spanA + p.spanB <= kStageCap) ? 1 : 0;
  return p;
}

__device__ inline void issue(const Plan& p, const uint32_t* __restrict__ hub, uint32_t* stage, uint64_t* bar) {
  if (p.trivial || !p.staged) return;
  if (lane_id() == 0) {
    mbar_expect_tx(bar, (uint32_t)(p.spanA + p.spanB) * 4u);
    bulk_g2s(stage, hub + p.sA, (uint32_t)p.spanA * 4u, bar);
    bulk_g2s(stage + p.spanA, hub + p.sB, (uint32_t)p.spanB * 4u, bar);
  }
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_query(int32_t n, int64_t nq, const int32_t* __restrict__ qs,
                                                               const int32_t* __restrict__ qt,
                                                               const int32_t* __restrict__ qk,
                                                               const int64_t* __restrict__ off,
                                                               const uint32_t* __restrict__ hub,
                                                               const uint32_t* __restrict__ hd,
                                                               int32_t* __restrict__ out, unsigned int* err) {
  extern __shared__ __align__(16) uint32_t smem_hubs[];
  __shared__ __align__(8) uint64_t bars[kWarpsPerBlock][2];
  const int lane = lane_id(), w = threadIdx.x >> 5;
  uint32_t* stage[2] = {smem_hubs + (size_t)w * 2 * kStageCap, smem_hubs + (size_t)w * 2 * kStageCap + kStageCap};
  if (lane == 0) {
    mbar_init(&bars[w][0], 1);
    mbar_init(&bars[w][1], 1);
    mbar_init_fence();
  }
  __syncwarp();
  uint32_t phase[2] = {0, 0};
  const int64_t step = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  int cur_stage = 0;
  Plan cur = make_plan(q, n, qs, qt, qk, off);
  issue(cur, hub, stage[0], &bars[w][0]);
  while (q < nq) {
    const int64_t qn = q + step;
    Plan nxt;
    nxt.trivial = 1;
    nxt.staged = 0;
    if (qn < nq) {
      nxt = make_plan(qn, n, qs, qt, qk, off);
      issue(nxt, hub, stage[cur_stage ^ 1], &bars[w][cur_stage ^ 1]);
    }
    int32_t ans = cur.ans;
    if (!cur.trivial) {
      const uint32_t *A, *B;
      if (cur.staged) {
        if (!bounded_wait(&bars[w][cur_stage], phase[cur_stage])) {
          // the copy never completed: report, let the next stage's copy land
          // (bounded), and leave without touching either stage again
          if (lane == 0) atomicExch(err, 1u);
          if (nxt.staged && !nxt.trivial) bounded_wait(&bars[w][cur_stage ^ 1], phase[cur_stage ^ 1]);
          return;
        }
        phase[cur_stage] ^= 1;
        A = stage[cur_stage] + cur.offA;
        B = stage[cur_stage] + cur.offB;
      } else {
        A = hub + cur.a0;
        B = hub + cur.b0;
      }
      long long best = lane_merge(A, cur.la, B, cur.lb, hd + cur.a0, hd + cur.b0, cur.k);
      ans = clamp_answer(warp_min_ll(best));
    }
    if (lane == 0) out[q] = ans;
    __syncwarp();
    fence_proxy_async();
    cur = nxt;
    q = qn;
    cur_stage ^= 1;
  }
}

}  // namespace

int query_device(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                 int32_t* out, cudaStream_t st) {
  if (nq <= 0) return HSDL_OK;
  const int sms = device_sm_count();
  const size_t smem = (size_t)kWarpsPerBlock * 2 * kStageCap * sizeof(uint32_t);
  static bool attr_set = false;
  if (!attr_set) {
    HSDL_CUDA(cudaFuncSetAttribute(k_query, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  int64_t blocks = (nq + kWarpsPerBlock - 1) / kWarpsPerBlock;
  int64_t max_blocks = (int64_t)sms * 3;
  k_query<<<(unsigned)std::min(blocks, max_blocks), kWarpsPerBlock * 32, smem, st>>>(
      idx->n, nq, s, t, k, idx->off.p, idx->hub.p, idx->hd.p, out, idx->qerr.p);
  HSDL_LAUNCHED();
  return HSDL_OK;
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
