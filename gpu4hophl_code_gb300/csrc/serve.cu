// Persistent, device-resident serving loop for (graph, s, t, k) queries over
// many resident label indexes, with index builds admitted concurrently.
//
// The reference answers queries one at a time on the host
// (hop_constrained_extract_distance, CPU_HopHL/include/HBPLL/
// hop_constrained_two_hop_labels.h:144) or with three launches and a sync per
// query (gpu_query, Query_mdnd/src/gpu_query.cu:84-178); it has no serving
// mode.  Here one kernel stays resident:
//
//  * Requests {graph, s, t, k} go into a ring in pinned host memory that the
//    GPU reads directly (mapped, coherent over NVLink-C2C on Grace systems).
//    The host publishes them by advancing `tail` with a release store.
//  * Every warp of the persistent kernel claims up to 32 published tickets at
//    a time with a CAS on the device-side `head` (continuous batching: a warp
//    takes whatever has arrived, across all resident graphs, as soon as it is
//    free), answers them one by one with the merge-path join
//    (query_join.cuh), and writes each answer with its ticket into a
//    completion ring in pinned host memory as one 8-byte store.
//  * Idle warps poll with __nanosleep.  Every wait is bounded: after
//    `idle_exit_s` without work, or when the host sets `stop`, the kernel
//    returns; the host relaunches it on the next submission.
//  * Resident indexes are described in a device table; builds requested
//    through the server run on a worker thread on their own stream while the
//    loop keeps serving, admitted when resident + pending estimated label
//    bytes fit the budget.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"
#include "query_join.cuh"

namespace hsdl {

namespace {

// Blocks of 256 threads per SM the loop is compiled for (40 registers) and
// runs with by default.  At n = 1M: 2 / 3 / 4 blocks per SM saturated at 147
// / 205 / 275-283 M q/s; 6 blocks at 315 M q/s, holding p99 at 314 us at
// 290 M/s offered (4 blocks: 3.2 ms).  Six blocks scale only because a
// request waits in 16 bytes of shared memory: with 48-byte slots the blocks'
// shared memory cost the SMs the L1 that holds the joins' rows, and 6 blocks
// saturated lower than 4 (266 M q/s).
constexpr int kServeBlocksPerSm = 6;
constexpr int kServeDefaultBlocksPerSm = 6;

struct IndexDesc {
  const int64_t* off;
  const uint64_t* key;
  const uint32_t* key32;  // compact query keys, or null
  int32_t n;
  int32_t valid;
  uint32_t fmt;  // compact key format: hub_shift | dist_bits << 8
  int32_t pad;
};

struct ServeReq {
  int32_t g, s, t, k;
};

// Copies of the mirrored tail, each on its own 128-byte line: the workers of
// block b poll copy b mod kTailCopies, so thousands of idle warps do not all
// poll one L2 line.  With one copy, p99 at n = 1M was 425 us at 100 M/s
// offered and 294 us at 200 M/s (at moderate load most workers are idle and
// polling); with 64, 188 and 210 us, and 318 against 426 us at 260 M/s.
constexpr int kTailCopies = 64;  // written two per lane by the dispatcher warp
constexpr int kTailStride = 16;  // u64 per 128-byte line

struct DevCtl {
  unsigned long long head;       // next ticket to claim
  unsigned long long processed;  // tickets answered
  unsigned long long bad;        // requests naming no resident graph
  unsigned int exit_reason;      // 1 idle, 2 stop
  unsigned int pad;
  unsigned long long dev_tail;   // device-side mirror of the host's tail
  unsigned long long pad2[11];
  unsigned long long tail_copy[kTailCopies * kTailStride];  // the mirror, fanned out
};

struct HostCtl {
  unsigned long long tail;  // tickets published by the host
  unsigned int stop;        // 1: return as soon as the claimed work is done
  unsigned int pad;
};

__device__ inline unsigned long long ld_acquire_sys(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline unsigned int ld_volatile_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline int4 ld_volatile_v4(const int4* p) {
  int4 v;
  asm volatile("ld.volatile.global.v4.s32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p)
               : "memory");
  return v;
}
__device__ inline void st_relaxed_sys(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ inline long long globaltimer_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ inline unsigned long long ld_acquire_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_relaxed_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ inline void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ inline void st_release_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ inline unsigned int ld_volatile_dev_u32(const unsigned int* p) {
  return *(const volatile unsigned int*)p;
}

// Warp 0 of block 0 is the dispatcher: it alone polls the host's tail and stop
// flag over the host link and mirrors the tail into device memory, and it
// decides the idle exit.  The other W warps are workers.  Tickets come in
// chunks of 8 (one 64-byte line of the completion ring); chunk c = (ticket -
// base) / 8 belongs to worker slot c mod W, and a block's warps pool their
// slots' chunks through one shared-memory counter, so no two warps contend for
// a request, every completion line is written once, by one coalesced store,
// and a chunk waits for the first free warp of its block rather than for one
// warp.  With a fixed chunk share per warp (each warp a single-server queue)
// p99 at n = 1M was 516-828 us at 260-290 M/s offered and the best rate
// under 1 ms 287.6 M q/s; pooled, 288-340 us and 299.0 M q/s on the same box.
// A warp reads the published requests of its chunk in parallel and answers
// them one after another.
// A worker's batch of requests waits in shared memory while it is answered
// (in registers, the 32 lanes' requests and index descriptors took the loop
// to 64 registers), one int4 per request: graph id (-1 when it names no
// resident index), s, t, k.  Only 16 bytes a request: the shared memory the
// blocks take comes out of the SMs' L1, which holds the rows the joins read
// (48-byte slots with the descriptors cost 6 blocks per SM a 100 KB carveout).

template <int G>
__global__ void __launch_bounds__(256, kServeBlocksPerSm) k_serve(DevCtl* ctl, const HostCtl* hctl, const int4* ring,
                                                                 unsigned long long* comp, unsigned long long mask,
                                                                 const IndexDesc* descs, int32_t max_idx,
                                                                 long long idle_ns, unsigned long long base) {
  constexpr int Q = 32 / G;  // requests answered at once by one warp
  const int lane = lane_id();
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  __shared__ unsigned long long s_claim;  // the block's next chunk to hand out
  if (threadIdx.x == 0) s_claim = 0;
  __syncthreads();
  if (gw == 0) {
    // the dispatcher warp: lane 0 polls the host; on a new tail every lane
    // writes two of the tail's copies
    unsigned long long last = 0;
    if (lane == 0) last = ld_acquire_gpu(&ctl->dev_tail);
    last = __shfl_sync(0xffffffffu, last, 0);
    long long idle_start = 0;
    if (lane == 0) idle_start = globaltimer_ns();
    for (;;) {
      unsigned long long t = 0;
      unsigned int stop = 0;
      if (lane == 0) {
        t = ld_acquire_sys(&hctl->tail);
        stop = ld_volatile_u32(&hctl->stop);
      }
      t = __shfl_sync(0xffffffffu, t, 0);
      stop = __shfl_sync(0xffffffffu, stop, 0);
      if (t != last) {
        // the warp barrier orders lane 0's acquire before every lane's fence,
        // and each fence makes its lane's relaxed stores release the tail
        // (and the ring entries the acquire made visible) to the workers
        __syncwarp();
        fence_acq_rel_gpu();
        for (int c = lane; c < kTailCopies; c += 32) st_relaxed_gpu(&ctl->tail_copy[c * kTailStride], t);
        if (lane == 0) {
          st_release_gpu(&ctl->dev_tail, t);
          idle_start = globaltimer_ns();
        }
        last = t;
      }
      if (stop) {
        if (lane == 0) atomicMax(&ctl->exit_reason, 2u);
        return;
      }
      int idle = 0;
      if (lane == 0)
        idle = globaltimer_ns() - idle_start > idle_ns && *(volatile unsigned long long*)&ctl->processed >= last;
      if (__shfl_sync(0xffffffffu, idle, 0)) {
        if (lane == 0) atomicMax(&ctl->exit_reason, 1u);
        return;
      }
      __nanosleep(100);
    }
  }
  __shared__ int4 s_req[256 / 32][32];
  int4* req = s_req[threadIdx.x >> 5];
  // Tickets come in chunks of 8 (one completion line).  The W worker warps
  // own the chunks in turn (chunk c belongs to worker slot c mod W, slot =
  // warp - 1), and a block's warps pool their slots' chunks: the block's j-th
  // chunk goes to whichever of its warps is free, so a warp held up by long
  // joins does not hold up the requests behind it.  A warp holds one chunk
  // at a time, claims the next (published or not) once its chunk is
  // answered, and answers a chunk's tickets as they are published.
  const unsigned long long W = (((unsigned long long)gridDim.x * blockDim.x) >> 5) - 1;
  const int wpb = (int)(blockDim.x >> 5);
  const int first_gw = max(1, (int)blockIdx.x * wpb);
  const unsigned long long s0 = (unsigned long long)(first_gw - 1);         // the block's first slot
  const unsigned long long nb = (unsigned long long)((int)blockIdx.x * wpb + wpb - first_gw);  // its slots
  const int grp = lane / G;
  unsigned long long t0 = 0;    // first ticket of the held chunk
  int got = 8;                  // tickets of it answered (8: none held)
  unsigned long long seen = 0;  // the latest tail this warp has acquired
  unsigned int backoff = 64;
  for (;;) {
    if (got == 8) {
      unsigned long long j = 0;
      if (lane == 0) j = atomicAdd(&s_claim, 1ull);
      j = __shfl_sync(0xffffffffu, j, 0);
      t0 = base + 8ull * ((j / nb) * W + s0 + j % nb);
      got = 0;
    }
    // The tail is acquired again only when the last one seen does not cover
    // the chunk: requests below a tail already acquired are visible to this
    // warp (the ring is read with volatile loads, past L1), and every gpu-scope
    // acquire also costs the SM's L1 the rows the joins had cached there.
    if (seen < t0 + 8) {
      unsigned long long tail = 0;
      if (lane == 0) tail = ld_acquire_gpu(&ctl->tail_copy[(blockIdx.x % kTailCopies) * kTailStride]);
      seen = __shfl_sync(0xffffffffu, tail, 0);
    }
    const unsigned long long pub = seen > t0 ? min(seen - t0, 8ull) : 0ull;  // published tickets of the chunk
    if (pub > (unsigned long long)got) {
      backoff = 64;
      const int cnt = (int)pub - got;
      const unsigned long long tk0 = t0 + (unsigned long long)got;
      // every lane reads its own request and checks its index.  (An L2 bulk
      // prefetch of the batch's rows here measured p99 410 against 297 us at
      // 260 M/s offered, n = 1M: the rows of up to 32 requests, joined one
      // after another, were partly evicted before use.)
      if (lane < cnt) {
        int4 r = ld_volatile_v4(ring + ((tk0 + (unsigned long long)lane) & mask));
        const bool valid = r.x >= 0 && r.x < max_idx && __ldcg(&descs[r.x].valid) != 0;
        if (!valid) {
          atomicAdd(&ctl->bad, 1ull);
          r.x = -1;
        }
        req[lane] = r;
      }
      __syncwarp();
      int32_t mine = INT_MAX;
      for (int r0 = 0; r0 < cnt; r0 += Q) {
        // group grp answers request r0 + grp (the lanes of a group read the
        // same slot and descriptor: broadcasts)
        const int4 q = req[min(r0 + grp, 31)];
        const bool active = r0 + grp < cnt && q.x >= 0;
        const IndexDesc* dp = descs + (active ? q.x : 0);
        const int64_t* off = (const int64_t*)__ldcg((const unsigned long long*)&dp->off);
        const void* k32 = (const void*)__ldcg((const unsigned long long*)&dp->key32);
        const bool is32 = k32 != nullptr;
        // groups of one warp may serve indexes of both key formats: each
        // format's join runs, warp-wide, only if some group needs it
        const unsigned m32 = __ballot_sync(0xffffffffu, active && is32);
        const unsigned m64 = __ballot_sync(0xffffffffu, active && !is32);
        const int n = __ldcg(&dp->n);
        int32_t ans = INT_MAX;
        if (m32) {
          const uint32_t fmt = __ldcg(&dp->fmt);
          const int32_t a = group_query<G>(active && is32, n, off, (const uint32_t*)k32, q.y, q.z, q.w,
                                           Fmt32{fmt & 0xFFu, fmt >> 8});
          if (is32) ans = a;
        }
        if (m64) {
          const uint64_t* k64 = (const uint64_t*)__ldcg((const unsigned long long*)&dp->key);
          const int32_t a = group_query<G>(active && !is32, n, off, k64, q.y, q.z, q.w, Fmt64{});
          if (!is32) ans = a;
        }
        // lane j takes the answer of the group that served it
        const int src = (lane >= r0 && lane < r0 + Q) ? (lane - r0) * G : 0;
        const int32_t a2 = __shfl_sync(0xffffffffu, ans, src);
        if (lane >= r0 && lane < r0 + Q) mine = a2;
      }
      __syncwarp();
      // one 8-byte store per answer carries its ticket, so the host needs no
      // ordering between slots
      if (lane < cnt) {
        const unsigned long long tk = tk0 + (unsigned long long)lane;
        st_relaxed_sys(comp + (tk & mask), ((unsigned long long)(uint32_t)(tk + 1) << 32) | (uint32_t)mine);
      }
      if (lane == 0) atomicAdd(&ctl->processed, (unsigned long long)cnt);
      got += cnt;
      continue;
    }
    unsigned int ex = 0;
    if (lane == 0) ex = ld_volatile_dev_u32(&ctl->exit_reason);
    ex = __shfl_sync(0xffffffffu, ex, 0);
    if (ex) return;  // the dispatcher left: every published ticket is answered
    __nanosleep(backoff);
    backoff = min(backoff * 2, 2048u);
  }
}

double mono_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
// Scheduled arrival times (ns from the run's start) of n requests of a
// Poisson stream of rate qps (SplitMix64 uniforms, exponential gaps); all at
// 0 for qps <= 0.
std::vector<int64_t> poisson_arrivals_ns(int64_t n, double qps, uint64_t seed) {
  std::vector<int64_t> arrive((size_t)n);
  uint64_t z = seed ? seed : 0x9E3779B97F4A7C15ull;
  double tcur = 0;
  for (int64_t i = 0; i < n; i++) {
    if (qps > 0) {
      z += 0x9E3779B97F4A7C15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      x ^= x >> 31;
      double u = ((double)(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
      tcur += -std::log(u) / qps;
    }
    arrive[i] = (int64_t)(tcur * 1e9);
  }
  return arrive;
}

// Rate and latency percentiles of a load run (latencies in ns).
void summarise_latency(const std::vector<int32_t>& lat_ns, int64_t first_arrival, int64_t last_done, double offered,
                       hsdl_loadgen_result* res) {
  std::vector<int32_t> sorted(lat_ns);
  std::sort(sorted.begin(), sorted.end());
  auto pct = [&](double p) { return sorted[std::min<size_t>(sorted.size() - 1, (size_t)(p * (sorted.size() - 1)))]; };
  const int64_t n = (int64_t)lat_ns.size();
  res->completed = n;
  res->seconds = (double)(last_done - first_arrival) / 1e9;
  res->achieved_qps = res->seconds > 0 ? (double)n / res->seconds : 0;
  res->offered_qps = offered;
  res->p50_us = pct(0.50) / 1e3;
  res->p90_us = pct(0.90) / 1e3;
  res->p99_us = pct(0.99) / 1e3;
  res->p999_us = pct(0.999) / 1e3;
  res->max_us = sorted.back() / 1e3;
}

int64_t mono_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

}  // namespace

struct ServerImpl {
  hsdl_serve_opts opts;
  int sms = 1;
  cudaStream_t stream = nullptr;   // the persistent kernel
  cudaStream_t side = nullptr;     // descriptor updates
  DevBuf<DevCtl> ctl;
  DevBuf<IndexDesc> descs;
  HostCtl* hctl = nullptr;         // pinned, mapped
  HostCtl* hctl_dev = nullptr;
  int4* ring = nullptr;            // pinned, mapped
  int4* ring_dev = nullptr;
  unsigned long long* comp = nullptr;  // pinned, mapped
  unsigned long long* comp_dev = nullptr;
  uint64_t cap = 0, mask = 0;
  uint64_t tail = 0;      // host copy of published tickets
  uint64_t consumed = 0;  // tickets whose answers the host has read
  bool running = false;
  std::mutex mu;          // submission / consumption / launch state
  // resident indexes
  struct Slot {
    hsdl_index* idx = nullptr;
    bool owned = false;
    int state = 0;  // 0 free, 1 pending build, 2 resident, 3 failed
    int64_t est_bytes = 0, bytes = 0;
    std::string error;
  };
  std::vector<Slot> slots;
  std::mutex slot_mu;
  std::condition_variable slot_cv;
  // build worker
  struct BuildJob {
    int32_t gid;
    hsdl_graph* g;
    int32_t K;
  };
  std::deque<BuildJob> jobs;
  std::thread worker;
  bool quit = false;
  int64_t builds_done = 0;
};

namespace {

int launch_if_needed(ServerImpl* S) {
  if (S->running) {
    cudaError_t q = cudaStreamQuery(S->stream);
    if (q == cudaErrorNotReady) return HSDL_OK;
    if (q != cudaSuccess) {
      set_error(std::string("serving kernel: ") + cudaGetErrorString(q));
      return HSDL_ERR_CUDA;
    }
    S->running = false;  // it returned (idle)
  }
  // tickets below `processed` are all answered and none above it is: the new
  // kernel's workers start there
  unsigned long long processed = 0;
  HSDL_CUDA(cudaMemcpyAsync(&processed, &S->ctl.p->processed, sizeof(processed), cudaMemcpyDeviceToHost,
                            S->stream));
  HSDL_CUDA(cudaMemsetAsync(&S->ctl.p->exit_reason, 0, sizeof(unsigned int), S->stream));
  HSDL_CUDA(cudaStreamSynchronize(S->stream));
  long long idle_ns = (long long)(S->opts.idle_exit_s * 1e9);
  if (S->opts.lanes_per_query == 8)
    k_serve<8><<<S->opts.ctas, 256, 0, S->stream>>>(S->ctl.p, S->hctl_dev, S->ring_dev, S->comp_dev, S->mask,
                                                    S->descs.p, S->opts.max_indexes, idle_ns, processed);
  else if (S->opts.lanes_per_query == 16)
    k_serve<16><<<S->opts.ctas, 256, 0, S->stream>>>(S->ctl.p, S->hctl_dev, S->ring_dev, S->comp_dev, S->mask,
                                                     S->descs.p, S->opts.max_indexes, idle_ns, processed);
  else
    k_serve<32><<<S->opts.ctas, 256, 0, S->stream>>>(S->ctl.p, S->hctl_dev, S->ring_dev, S->comp_dev, S->mask,
                                                     S->descs.p, S->opts.max_indexes, idle_ns, processed);
  HSDL_LAUNCHED();
  S->running = true;
  return HSDL_OK;
}

int write_desc(ServerImpl* S, int32_t gid, hsdl_index* idx, bool valid) {
  IndexDesc d{};
  if (idx) {
    d.off = idx->off.p;
    d.key = idx->key.p;
    d.key32 = idx->key32.p;
    d.fmt = idx->fmt32.hub_shift | (idx->fmt32.dist_bits << 8);
    d.n = idx->n;
  }
  d.valid = valid ? 1 : 0;
  HSDL_CUDA(cudaMemcpyAsync(S->descs.p + gid, &d, sizeof(d), cudaMemcpyHostToDevice, S->side));
  HSDL_CUDA(cudaStreamSynchronize(S->side));
  return HSDL_OK;
}

// Label bytes of an index of n vertices and m edges at hop bound K, for
// admission only: labels per vertex ~ 0.53 sqrt(n) (avg_deg/10) (K/5), capped
// by n (K+1), fitted on Chung-Lu graphs of 3*10^4 .. 10^6 vertices at K = 5;
// 12 bytes per label resident.  Replaced by the measured size once built.
int64_t estimate_label_bytes(int32_t n, int64_t m2, int32_t K) {
  double avg_deg = n ? (double)m2 / n : 0.0;
  double per_v = 0.53 * std::sqrt((double)n) * std::max(0.25, avg_deg / 10.0) * ((double)K / 5.0);
  per_v = std::min(per_v, (double)n * (K + 1));
  per_v = std::max(per_v, 1.0);
  return (int64_t)(12.0 * per_v * n) + 8 * ((int64_t)n + 1);
}

int64_t resident_bytes_locked(ServerImpl* S) {
  int64_t b = 0;
  for (auto& s : S->slots) {
    if (s.state == 1) b += s.est_bytes;
    if (s.state == 2) b += s.bytes;
  }
  return b;
}

void worker_main(ServerImpl* S) {
  for (;;) {
    ServerImpl::BuildJob job;
    {
      std::unique_lock<std::mutex> lk(S->slot_mu);
      S->slot_cv.wait(lk, [&] { return S->quit || !S->jobs.empty(); });
      if (S->quit) return;
      job = S->jobs.front();
      S->jobs.pop_front();
    }
    hsdl_build_opts o;
    hsdl_build_opts_default(&o);
    hsdl_index* idx = nullptr;
    int rc = hsdl_build(job.g, job.K, &o, &idx);
    std::string err = rc == HSDL_OK ? "" : hsdl_last_error();
    if (rc == HSDL_OK) rc = write_desc(S, job.gid, idx, true);
    {
      std::lock_guard<std::mutex> lk(S->slot_mu);
      auto& sl = S->slots[job.gid];
      if (rc == HSDL_OK) {
        hsdl_index_info info;
        hsdl_index_get_info(idx, &info);
        sl.idx = idx;
        sl.owned = true;
        sl.bytes = info.device_bytes;
        sl.state = 2;
      } else {
        if (idx) hsdl_index_destroy(idx);
        sl.state = 3;
        sl.error = err;
      }
      S->builds_done++;
    }
    S->slot_cv.notify_all();
  }
}

int alloc_slot_locked(ServerImpl* S, int32_t* gid) {
  for (size_t i = 0; i < S->slots.size(); i++) {
    if (S->slots[i].state == 0) {
      *gid = (int32_t)i;
      return HSDL_OK;
    }
  }
  set_error("no free graph slot (max_indexes reached)");
  return HSDL_ERR_FULL;
}

// Waits until every published ticket has been answered (used before an index
// is retired so no in-flight query reads it).
int drain(ServerImpl* S, double timeout_s) {
  double t0 = mono_s();
  for (;;) {
    unsigned long long processed = 0;
    HSDL_CUDA(cudaMemcpyAsync(&processed, &S->ctl.p->processed, sizeof(processed), cudaMemcpyDeviceToHost, S->side));
    HSDL_CUDA(cudaStreamSynchronize(S->side));
    if (processed >= S->tail) return HSDL_OK;
    if (mono_s() - t0 > timeout_s) {
      set_error("serving loop did not drain within the timeout");
      return HSDL_ERR_TIMEOUT;
    }
    HSDL_TRY(launch_if_needed(S));
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

}  // namespace

}  // namespace hsdl

using namespace hsdl;

struct hsdl_server : hsdl::ServerImpl {};

#define SRV_ARG(cond, msg)     \
  do {                         \
    if (!(cond)) {             \
      set_error(msg);          \
      return HSDL_ERR_INVALID; \
    }                          \
  } while (0)

extern "C" {

void hsdl_serve_opts_default(hsdl_serve_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->struct_size = (int32_t)sizeof(hsdl_serve_opts);
  o->ctas = 0;
  o->ring_log2 = 22;
  o->max_indexes = 1024;
  o->budget_bytes = (int64_t)120 << 30;
  o->idle_exit_s = 0.5;
  o->lanes_per_query = 32;
}

int hsdl_serve_create(const hsdl_serve_opts* opts, hsdl_server** out) {
  SRV_ARG(out, "null output");
  hsdl_serve_opts o;
  hsdl_serve_opts_default(&o);
  if (opts) {
    SRV_ARG(opts->struct_size == (int32_t)sizeof(hsdl_serve_opts), "hsdl_serve_opts.struct_size mismatch");
    o = *opts;
  }
  SRV_ARG(o.ring_log2 >= 10 && o.ring_log2 <= 26, "ring_log2 must be in [10, 26]");
  SRV_ARG(o.max_indexes >= 1 && o.max_indexes <= (1 << 20), "max_indexes out of range");
  SRV_ARG(o.idle_exit_s > 0 && o.idle_exit_s <= 60, "idle_exit_s must be in (0, 60]");
  SRV_ARG(o.lanes_per_query == 8 || o.lanes_per_query == 16 || o.lanes_per_query == 32,
          "lanes_per_query must be 8, 16 or 32");
  auto* S = new hsdl_server();
  S->opts = o;
  S->sms = device_sm_count();
  {
    // every block of the persistent loop must be resident at once (a block
    // left waiting for a slot would hold its share of the tickets)
    const int per_sm = o.lanes_per_query == 8    ? resident_blocks(k_serve<8>, 256)
                       : o.lanes_per_query == 16 ? resident_blocks(k_serve<16>, 256)
                                                 : resident_blocks(k_serve<32>, 256);
    const int most = S->sms * per_sm;
    if (S->opts.ctas <= 0) S->opts.ctas = std::min(most, S->sms * kServeDefaultBlocksPerSm);
    if (S->opts.ctas > most) {
      delete S;
      set_error("ctas must be at most " + std::to_string(most) + " (blocks of the loop that fit on the GPU at once)");
      return HSDL_ERR_INVALID;
    }
  }
  S->cap = 1ull << o.ring_log2;
  S->mask = S->cap - 1;
  auto fail = [&](int rc) {
    hsdl_serve_destroy(S);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&S->side, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return fail(HSDL_ERR_CUDA);
  }
  int rc = S->ctl.alloc(1, S->side);
  if (rc == HSDL_OK) rc = S->descs.alloc(o.max_indexes, S->side);
  if (rc == HSDL_OK && cudaStreamSynchronize(S->side) != cudaSuccess) rc = HSDL_ERR_CUDA;
  if (rc != HSDL_OK) return fail(rc);
  cudaError_t e = cudaHostAlloc((void**)&S->hctl, sizeof(HostCtl), cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess)
    e = cudaHostAlloc((void**)&S->ring, sizeof(int4) * S->cap, cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess)
    e = cudaHostAlloc((void**)&S->comp, sizeof(unsigned long long) * S->cap,
                      cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&S->hctl_dev, S->hctl, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&S->ring_dev, S->ring, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&S->comp_dev, S->comp, 0);
  if (e != cudaSuccess) {
    set_error(std::string("pinned ring allocation: ") + cudaGetErrorString(e));
    return fail(HSDL_ERR_NOMEM);
  }
  std::memset(S->hctl, 0, sizeof(HostCtl));
  std::memset(S->comp, 0, sizeof(unsigned long long) * S->cap);
  if (cudaMemset(S->ctl.p, 0, sizeof(DevCtl)) != cudaSuccess ||
      cudaMemset(S->descs.p, 0, sizeof(IndexDesc) * o.max_indexes) != cudaSuccess) {
    set_error("device control block initialisation failed");
    return fail(HSDL_ERR_CUDA);
  }
  S->slots.resize(o.max_indexes);
  S->worker = std::thread(worker_main, S);
  *out = S;
  return HSDL_OK;
}

int hsdl_serve_add_index(hsdl_server* S, hsdl_index* idx, int32_t* graph_id) {
  SRV_ARG(S && idx && graph_id, "null argument");
  int32_t gid = -1;
  {
    std::lock_guard<std::mutex> lk(S->slot_mu);
    HSDL_TRY(alloc_slot_locked(S, &gid));
    S->slots[gid].state = 1;
  }
  HSDL_CUDA(cudaStreamSynchronize(idx->stream));
  int rc = write_desc(S, gid, idx, true);
  std::lock_guard<std::mutex> lk(S->slot_mu);
  auto& sl = S->slots[gid];
  if (rc != HSDL_OK) {
    sl.state = 0;
    return rc;
  }
  hsdl_index_info info;
  hsdl_index_get_info(idx, &info);
  sl.idx = idx;
  sl.owned = false;
  sl.bytes = info.device_bytes;
  sl.state = 2;
  *graph_id = gid;
  return HSDL_OK;
}

int hsdl_serve_submit_build(hsdl_server* S, hsdl_graph* g, int32_t K, int32_t* graph_id) {
  SRV_ARG(S && g && graph_id, "null argument");
  SRV_ARG(K >= 1 && K <= kMaxK, "K must be in [1, 14]");
  int64_t est = estimate_label_bytes(g->n, g->m2, K);
  std::lock_guard<std::mutex> lk(S->slot_mu);
  if (resident_bytes_locked(S) + est > S->opts.budget_bytes) {
    set_error("build not admitted: resident + pending estimated label bytes would exceed the budget (" +
              std::to_string(resident_bytes_locked(S) + est) + " > " + std::to_string(S->opts.budget_bytes) + ")");
    return HSDL_ERR_FULL;
  }
  int32_t gid = -1;
  HSDL_TRY(alloc_slot_locked(S, &gid));
  auto& sl = S->slots[gid];
  sl.state = 1;
  sl.est_bytes = est;
  sl.error.clear();
  S->jobs.push_back({gid, g, K});
  S->slot_cv.notify_all();
  *graph_id = gid;
  return HSDL_OK;
}

int hsdl_serve_graph_state(hsdl_server* S, int32_t graph_id, int32_t* state, int64_t* bytes) {
  SRV_ARG(S && state, "null argument");
  SRV_ARG(graph_id >= 0 && graph_id < S->opts.max_indexes, "graph id out of range");
  std::lock_guard<std::mutex> lk(S->slot_mu);
  auto& sl = S->slots[graph_id];
  *state = sl.state;
  if (bytes) *bytes = sl.state == 2 ? sl.bytes : sl.est_bytes;
  if (sl.state == 3) set_error(sl.error);
  return HSDL_OK;
}

int hsdl_serve_wait_graph(hsdl_server* S, int32_t graph_id, double timeout_s) {
  SRV_ARG(S, "null server");
  SRV_ARG(graph_id >= 0 && graph_id < S->opts.max_indexes, "graph id out of range");
  std::unique_lock<std::mutex> lk(S->slot_mu);
  bool done = S->slot_cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                  [&] { return S->slots[graph_id].state != 1; });
  if (!done) {
    set_error("build still pending at the timeout");
    return HSDL_ERR_TIMEOUT;
  }
  if (S->slots[graph_id].state == 3) {
    set_error("build failed: " + S->slots[graph_id].error);
    return HSDL_ERR_STATE;
  }
  if (S->slots[graph_id].state != 2) {
    set_error("graph slot is not resident");
    return HSDL_ERR_STATE;
  }
  return HSDL_OK;
}

int hsdl_serve_remove_graph(hsdl_server* S, int32_t graph_id) {
  SRV_ARG(S, "null server");
  SRV_ARG(graph_id >= 0 && graph_id < S->opts.max_indexes, "graph id out of range");
  {
    std::lock_guard<std::mutex> lk(S->slot_mu);
    if (S->slots[graph_id].state != 2) {
      set_error("graph slot is not resident");
      return HSDL_ERR_STATE;
    }
  }
  HSDL_TRY(write_desc(S, graph_id, nullptr, false));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    HSDL_TRY(drain(S, 30.0));
  }
  std::lock_guard<std::mutex> lk(S->slot_mu);
  auto& sl = S->slots[graph_id];
  if (sl.owned && sl.idx) hsdl_index_destroy(sl.idx);
  sl = ServerImpl::Slot{};
  S->slot_cv.notify_all();
  return HSDL_OK;
}

// Publishes n requests; *first_ticket receives the ticket of the first.
// Blocks while the ring is full (answers not yet read by hsdl_serve_wait).
int hsdl_serve_submit(hsdl_server* S, int64_t n, const int32_t* g, const int32_t* s, const int32_t* t,
                      const int32_t* k, int64_t* first_ticket) {
  SRV_ARG(S && n >= 0 && first_ticket, "bad arguments");
  SRV_ARG(n == 0 || (g && s && t && k), "null request array");
  std::lock_guard<std::mutex> lk(S->mu);
  *first_ticket = (int64_t)S->tail;
  int64_t done = 0;
  double t0 = mono_s();
  while (done < n) {
    uint64_t room = S->cap - (S->tail - S->consumed);
    if (room == 0) {
      if (mono_s() - t0 > 30.0) {
        set_error("ring full: answers are not being consumed (call hsdl_serve_wait)");
        return HSDL_ERR_FULL;
      }
      HSDL_TRY(launch_if_needed(S));
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      continue;
    }
    int64_t chunk = std::min<int64_t>(n - done, (int64_t)room);
    for (int64_t i = 0; i < chunk; i++) {
      uint64_t tk = S->tail + i;
      S->ring[tk & S->mask] = make_int4(g[done + i], s[done + i], t[done + i], k[done + i]);
    }
    S->tail += chunk;
    __atomic_store_n(&S->hctl->tail, (unsigned long long)S->tail, __ATOMIC_RELEASE);
    done += chunk;
    HSDL_TRY(launch_if_needed(S));
  }
  return HSDL_OK;
}

// Waits for the answers of tickets [first_ticket, first_ticket + n), which
// must be the oldest unread ones, and copies them out.
int hsdl_serve_wait(hsdl_server* S, int64_t first_ticket, int64_t n, int32_t* answers, double timeout_s) {
  SRV_ARG(S && n >= 0 && (n == 0 || answers), "bad arguments");
  std::lock_guard<std::mutex> lk(S->mu);
  SRV_ARG((uint64_t)first_ticket == S->consumed, "tickets must be read in order, starting at the oldest unread one");
  SRV_ARG((uint64_t)(first_ticket + n) <= S->tail, "waiting for tickets that were never submitted");
  double t0 = mono_s();
  for (int64_t i = 0; i < n; i++) {
    uint64_t tk = (uint64_t)first_ticket + i;
    unsigned long long* slot = S->comp + (tk & S->mask);
    int spins = 0;
    for (;;) {
      unsigned long long v = __atomic_load_n(slot, __ATOMIC_ACQUIRE);
      if ((uint32_t)(v >> 32) == (uint32_t)(tk + 1)) {
        answers[i] = (int32_t)(uint32_t)v;
        break;
      }
      if (++spins > 4096) {
        spins = 0;
        if (mono_s() - t0 > timeout_s) {
          set_error("answers not complete at the timeout");
          return HSDL_ERR_TIMEOUT;
        }
        HSDL_TRY(launch_if_needed(S));
        std::this_thread::yield();
      }
    }
    S->consumed = tk + 1;
  }
  return HSDL_OK;
}

// Open-loop load generator: a producer thread publishes the given requests at
// Poisson arrival times of rate offered_qps (0 = as fast as the ring allows);
// a consumer thread reads the answers in order and records each request's
// latency from its scheduled arrival to the moment its answer is seen.
int hsdl_serve_loadgen(hsdl_server* S, const hsdl_loadgen_opts* o, hsdl_loadgen_result* res) {
  SRV_ARG(S && o && res, "null argument");
  SRV_ARG(o->struct_size == (int32_t)sizeof(hsdl_loadgen_opts), "hsdl_loadgen_opts.struct_size mismatch");
  const int64_t n = o->n;
  SRV_ARG(n >= 1 && o->g && o->s && o->t && o->k, "bad request arrays");
  std::lock_guard<std::mutex> lk(S->mu);
  const uint64_t base = S->tail;
  SRV_ARG(S->consumed == S->tail, "loadgen needs every earlier answer to be read first");
  std::vector<int64_t> arrive = poisson_arrivals_ns(n, o->offered_qps, o->seed);
  std::vector<int32_t> lat_ns((size_t)n);
  // Answers arrive in host memory over the host link; reading them one line
  // (8 answers) at a time from a single thread serialises a link round trip
  // per line.  Several consumer threads each own every R-th chunk of 64
  // tickets, so their line fetches overlap.  The producer's flow control
  // uses the slowest consumer's position.
  const int R = std::max(1, std::min(8, o->consumers > 0 ? o->consumers : 4));
  constexpr int64_t kChunk = 64;
  std::vector<std::atomic<int64_t>> cons_next(R);  // next index (relative) each consumer waits for
  for (int c = 0; c < R; c++) cons_next[c].store(c * kChunk);
  auto min_consumed = [&]() -> uint64_t {
    int64_t m = n;
    for (int c = 0; c < R; c++) m = std::min(m, cons_next[c].load(std::memory_order_acquire));
    return base + (uint64_t)m;
  };
  std::atomic<int> failed{0};
  std::atomic<int64_t> last_done_ns{0};
  std::atomic<int64_t> ready_first{0};
  // A loop that has sat idle can reach its idle exit just as the run starts,
  // and the watcher below relaunches it only milliseconds later, behind a
  // backlog (one sweep step saw p99 jump from 0.3 to 13 ms that way): nothing
  // is outstanding here, so stop it and start a fresh one whose idle clock
  // starts with the run.
  if (S->running) {
    __atomic_store_n(&S->hctl->stop, 1u, __ATOMIC_RELEASE);
    HSDL_CUDA(cudaStreamSynchronize(S->stream));
    S->running = false;
    __atomic_store_n(&S->hctl->stop, 0u, __ATOMIC_RELEASE);
  }
  HSDL_TRY(launch_if_needed(S));
  // The requests as the ring holds them, packed before the run: a client hands
  // the server whole requests, and gathering them from four arrays inside the
  // run made the one producer thread the ceiling (the loop then saturated near
  // 280 M requests/s whatever the GPU could do).
  std::vector<int4> packed((size_t)n);
  for (int64_t i = 0; i < n; i++) packed[i] = make_int4(o->g[i], o->s[i], o->t[i], o->k[i]);
  int64_t t_start = mono_ns() + 2000000;  // 2 ms to let the threads start
  std::thread producer([&] {
    int64_t i = 0;
    while (i < n && !failed.load(std::memory_order_relaxed)) {
      int64_t now = mono_ns() - t_start;
      if (now < arrive[i]) continue;
      uint64_t room = S->cap - (S->tail - min_consumed());
      if (room == 0) continue;
      // every request that has arrived, within the room left and 4,096 at a time
      const int64_t lim = std::min<int64_t>(n, i + (int64_t)std::min<uint64_t>(room, 4096));
      const int64_t j = std::upper_bound(arrive.begin() + i, arrive.begin() + lim, now) - arrive.begin();
      const uint64_t pos = S->tail & S->mask;
      const int64_t first = std::min<int64_t>(j - i, (int64_t)(S->cap - pos));
      std::memcpy(S->ring + pos, packed.data() + i, sizeof(int4) * (size_t)first);
      if (j - i > first) std::memcpy(S->ring, packed.data() + i + first, sizeof(int4) * (size_t)(j - i - first));
      S->tail += (uint64_t)(j - i);
      __atomic_store_n(&S->hctl->tail, (unsigned long long)S->tail, __ATOMIC_RELEASE);
      i = j;
    }
  });
  auto consumer = [&](int c) {
    int64_t ready = 0, latest = 0;
    for (int64_t c0 = (int64_t)c * kChunk; c0 < n; c0 += (int64_t)R * kChunk) {
      const int64_t c1 = std::min<int64_t>(n, c0 + kChunk);
      for (int64_t i = c0; i < c1; i++) {
        uint64_t tk = base + (uint64_t)i;
        unsigned long long* slot = S->comp + (tk & S->mask);
        bool first_look = true;
        int64_t spins = 0;
        unsigned long long v;
        for (;;) {
          v = __atomic_load_n(slot, __ATOMIC_ACQUIRE);
          if ((uint32_t)(v >> 32) == (uint32_t)(tk + 1)) break;
          first_look = false;
          if (failed.load(std::memory_order_relaxed)) return;
          if (++spins > (1 << 22)) {
            spins = 0;
            if (mono_ns() - t_start > (int64_t)120 * 1000000000) {
              failed = 1;  // two minutes without this answer: give up
              return;
            }
          }
        }
        ready += first_look;
        if (i == c0 || (tk & 7) == 0) latest = mono_ns() - t_start;  // one clock read per line
        lat_ns[i] = (int32_t)std::min<int64_t>(INT32_MAX, std::max<int64_t>(0, latest - arrive[i]));
        if (o->answers) o->answers[i] = (int32_t)(uint32_t)v;
      }
      cons_next[c].store(std::min<int64_t>(n, c0 + (int64_t)R * kChunk), std::memory_order_release);
    }
    cons_next[c].store(n, std::memory_order_release);
    ready_first.fetch_add(ready);
    int64_t prev = last_done_ns.load();
    while (latest > prev && !last_done_ns.compare_exchange_weak(prev, latest)) {
    }
  };
  std::vector<std::thread> consumers;
  for (int c = 1; c < R; c++) consumers.emplace_back(consumer, c);
  // this thread consumes chunk 0 mod R and watches the loop
  // relaunches the loop if it returned (it does so after idle_exit_s without
  // new requests) while answers are still outstanding
  std::thread watch([&] {
    while (!failed.load() && min_consumed() < base + (uint64_t)n) {
      std::this_thread::sleep_for(std::chrono::milliseconds(2));
      if (cudaStreamQuery(S->stream) != cudaErrorNotReady && launch_if_needed(S) != HSDL_OK) failed = 1;
    }
  });
  consumer(0);
  for (auto& th : consumers) th.join();
  watch.join();
  int64_t last_done = last_done_ns.load();
  S->consumed = base + (uint64_t)n;
  producer.join();
  if (failed.load()) {
    set_error("serving loop stopped answering during the load run");
    return HSDL_ERR_TIMEOUT;
  }
  summarise_latency(lat_ns, arrive[0], last_done, o->offered_qps, res);
  res->ready_frac = (double)ready_first.load() / (double)n;
  res->mean_batch = 0;
  return HSDL_OK;
}

// The plain path under the same open-loop Poisson stream: requests that have
// arrived are answered in batches by hsdl_query_batch (host arrays in, host
// arrays out, one call at a time).  A batch is dispatched once the oldest
// waiting request has waited window_us and the previous call has returned,
// and takes every request that has arrived by then (at most max_batch).  Latency runs from a
// request's scheduled arrival to the return of the call that answered it.
int hsdl_query_loadgen(hsdl_index* idx, const hsdl_query_loadgen_opts* o, hsdl_loadgen_result* res) {
  SRV_ARG(idx && o && res, "null argument");
  SRV_ARG(o->struct_size == (int32_t)sizeof(hsdl_query_loadgen_opts), "hsdl_query_loadgen_opts.struct_size mismatch");
  const int64_t n = o->n;
  SRV_ARG(n >= 1 && o->s && o->t && o->k && o->answers && o->window_us >= 0 && o->max_batch >= 0,
          "bad request arrays");
  std::vector<int64_t> arrive = poisson_arrivals_ns(n, o->offered_qps, o->seed);
  std::vector<int32_t> lat_ns((size_t)n);
  const int64_t window_ns = (int64_t)(o->window_us * 1e3);
  const int64_t t_start = mono_ns() + 1000000;
  int64_t done = 0, batches = 0;
  for (int64_t i = 0; i < n;) {
    const int64_t dispatch = std::max(done, arrive[i] + window_ns);
    int64_t now;
    while ((now = mono_ns() - t_start) < dispatch) {
    }
    int64_t j = std::upper_bound(arrive.begin() + i, arrive.end(), now) - arrive.begin();
    if (o->max_batch > 0) j = std::min<int64_t>(j, i + o->max_batch);
    HSDL_TRY(hsdl_query_batch(idx, j - i, o->s + i, o->t + i, o->k + i, o->answers + i));
    done = mono_ns() - t_start;
    for (int64_t r = i; r < j; r++) lat_ns[r] = (int32_t)std::min<int64_t>(INT32_MAX, done - arrive[r]);
    batches++;
    i = j;
  }
  summarise_latency(lat_ns, arrive[0], done, o->offered_qps, res);
  res->ready_frac = 0;
  res->mean_batch = (double)n / (double)batches;
  return HSDL_OK;
}

int hsdl_serve_stats(hsdl_server* S, hsdl_serve_counters* st) {
  SRV_ARG(S && st, "null argument");
  DevCtl c{};
  HSDL_CUDA(cudaMemcpyAsync(&c, S->ctl.p, sizeof(c), cudaMemcpyDeviceToHost, S->side));
  HSDL_CUDA(cudaStreamSynchronize(S->side));
  std::lock_guard<std::mutex> lk(S->slot_mu);
  st->submitted = (int64_t)S->tail;
  st->processed = (int64_t)c.processed;
  st->bad_requests = (int64_t)c.bad;
  st->resident_graphs = 0;
  st->pending_builds = 0;
  for (auto& s : S->slots) {
    st->resident_graphs += s.state == 2;
    st->pending_builds += s.state == 1;
  }
  st->resident_bytes = resident_bytes_locked(S);
  st->builds_done = S->builds_done;
  st->loop_running = S->running && cudaStreamQuery(S->stream) == cudaErrorNotReady;
  return HSDL_OK;
}

int hsdl_serve_destroy(hsdl_server* S) {
  if (!S) return HSDL_OK;
  {
    std::lock_guard<std::mutex> lk(S->slot_mu);
    S->quit = true;
  }
  S->slot_cv.notify_all();
  if (S->worker.joinable()) S->worker.join();
  if (S->hctl) __atomic_store_n(&S->hctl->stop, 1u, __ATOMIC_RELEASE);
  if (S->stream) cudaStreamSynchronize(S->stream);
  for (auto& s : S->slots)
    if (s.owned && s.idx) hsdl_index_destroy(s.idx);
  S->ctl.release();
  S->descs.release();
  if (S->side) cudaStreamSynchronize(S->side);
  if (S->hctl) cudaFreeHost(S->hctl);
  if (S->ring) cudaFreeHost(S->ring);
  if (S->comp) cudaFreeHost(S->comp);
  if (S->stream) cudaStreamDestroy(S->stream);
  if (S->side) cudaStreamDestroy(S->side);
  delete S;
  return HSDL_OK;
}

}  // extern "C"
