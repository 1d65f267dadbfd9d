// Device primitives: exclusive scan of int64 and per-row key/value sort.
#include <algorithm>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Per-tile exclusive scan; writes the tile total to sums[blockIdx.x].
__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                             int64_t* __restrict__ sums) {
  __shared__ int64_t sm[32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    local += v[i];
  }
  int64_t total;
  int64_t pre = block_exclusive_scan(local, sm, &total);
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ offs) {
  int64_t add = offs[blockIdx.x];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
    if (base + i < n) out[base + i] += add;
}

__global__ void k_set_total(const int64_t* in, const int64_t* out, int64_t n, int64_t* dst) {
  *dst = (n > 0) ? out[n - 1] + in[n - 1] : 0;
}

// ---------------------------------------------------------------------------
// Per-row sort of (key, parent) by the 64-bit label key.  Rows up to 32 labels: one warp per
// row, bitonic network on registers.  Longer rows: one block per row, bitonic
// network in shared memory (padded to a power of two with all-ones keys);
// rows longer than the shared-memory capacity use a global scratch buffer.
// ---------------------------------------------------------------------------
__global__ void k_sort_small(int32_t n, const int64_t* __restrict__ off, uint64_t* __restrict__ key,
                             int32_t* __restrict__ par) {
  int lane = lane_id();
  int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    int64_t lo = off[v], len = off[v + 1] - lo;
    if (len <= 1 || len > 32) continue;
    uint64_t k = lane < len ? key[lo + lane] : ~0ull;
    int32_t p = lane < len ? par[lo + lane] : 0;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        uint64_t ok = __shfl_xor_sync(0xffffffffu, k, stride);
        int32_t op = __shfl_xor_sync(0xffffffffu, p, stride);
        bool up = ((lane & size) == 0);
        bool lower = ((lane & stride) == 0);
        // keep the smaller key in the lower lane of an ascending pair
        bool take = lower == up ? (ok < k) : (ok > k);
        if (take) {
          k = ok;
          p = op;
        }
      }
    }
    if (lane < len) {
      key[lo + lane] = k;
      par[lo + lane] = p;
    }
  }
}

__device__ void block_bitonic(uint64_t* sk, int32_t* sp, int P) {
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
        int lo = 2 * i - (i & (stride - 1));
        int hi = lo + stride;
        bool up = ((lo & size) == 0);
        uint64_t a = sk[lo], b = sk[hi];
        if ((a > b) == up) {
          sk[lo] = b;
          sk[hi] = a;
          int32_t t = sp[lo];
          sp[lo] = sp[hi];
          sp[hi] = t;
        }
      }
    }
  }
  __syncthreads();
}

// rows listed in `rows` (count *nrows), each longer than 32
__global__ void k_sort_large(const int32_t* __restrict__ rows, const int32_t* nrows, const int64_t* __restrict__ off,
                             uint64_t* __restrict__ key, int32_t* __restrict__ par, int smem_cap,
                             uint64_t* __restrict__ gk, int32_t* __restrict__ gp) {
  extern __shared__ unsigned char smem_raw[];
  int cnt = *nrows;
  for (int r = blockIdx.x; r < cnt; r += gridDim.x) {
    int v = rows[r];
    int64_t lo = off[v], len = off[v + 1] - lo;
    int P = 1;
    while (P < len) P <<= 1;
    uint64_t* sk;
    int32_t* sp;
    if (P <= smem_cap) {
      sk = (uint64_t*)smem_raw;
      sp = (int32_t*)(sk + smem_cap);
    } else {
      // over-sized rows: launched with one block and a global scratch of P entries
      sk = gk;
      sp = gp;
    }
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      sk[i] = i < len ? key[lo + i] : ~0ull;
      sp[i] = i < len ? par[lo + i] : 0;
    }
    block_bitonic(sk, sp, P);
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      key[lo + i] = sk[i];
      par[lo + i] = sp[i];
    }
    __syncthreads();
  }
}

__global__ void k_list_large_rows(int32_t n, const int64_t* __restrict__ off, int32_t* rows, int32_t* count,
                                  int32_t min_len, int32_t max_len) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    int64_t len = off[v + 1] - off[v];
    if (len > min_len && len <= max_len) rows[atomicAdd(count, 1)] = (int32_t)v;
  }
}

}  // namespace

int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st) {
  // out[0..n-1] = exclusive prefix of in, out[n] = total
  if (n <= 0) {
    HSDL_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), st));
    return HSDL_OK;
  }
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  int64_t* sums = nullptr;
  int64_t* sums_scan = nullptr;
  HSDL_CUDA(cudaMallocAsync(&sums, (size_t)(tiles + 1) * sizeof(int64_t), st));
  HSDL_CUDA(cudaMallocAsync(&sums_scan, (size_t)(tiles + 1) * sizeof(int64_t), st));
  k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
  HSDL_LAUNCHED();
  if (tiles > 1) {
    HSDL_TRY(exclusive_scan_i64(sums, sums_scan, tiles, st));
    k_scan_add<<<(unsigned)tiles, 256, 0, st>>>(out, n, sums_scan);
    HSDL_LAUNCHED();
  }
  k_set_total<<<1, 1, 0, st>>>(in, out, n, out + n);
  HSDL_LAUNCHED();
  HSDL_CUDA(cudaFreeAsync(sums, st));
  HSDL_CUDA(cudaFreeAsync(sums_scan, st));
  return HSDL_OK;
}

int sort_rows(int32_t n, const int64_t* d_off, uint64_t* key, int32_t* par, int64_t max_row, cudaStream_t st) {
  int sms = device_sm_count();
  k_sort_small<<<sms * 8, 256, 0, st>>>(n, d_off, key, par);
  HSDL_LAUNCHED();
  if (max_row <= 32) return HSDL_OK;
  int32_t* rows = nullptr;
  int32_t* count = nullptr;
  HSDL_CUDA(cudaMallocAsync(&rows, (size_t)n * sizeof(int32_t), st));
  HSDL_CUDA(cudaMallocAsync(&count, sizeof(int32_t), st));
  // shared-memory rows: up to 1024 labels in 12 KB blocks of 256 threads (many
  // per SM), up to 8192 labels (96 KB) in blocks of 512
  const int small_cap = 1024, smem_cap = 8192;
  const size_t smem = (size_t)smem_cap * (sizeof(uint64_t) + sizeof(int32_t));
  const size_t small_smem = (size_t)small_cap * (sizeof(uint64_t) + sizeof(int32_t));
  HSDL_CUDA(cudaFuncSetAttribute(k_sort_large, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  HSDL_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), st));
  k_list_large_rows<<<sms * 4, 256, 0, st>>>(n, d_off, rows, count, 32, small_cap);
  HSDL_LAUNCHED();
  k_sort_large<<<sms * 8, 256, small_smem, st>>>(rows, count, d_off, key, par, small_cap, nullptr, nullptr);
  HSDL_LAUNCHED();
  if (max_row > small_cap) {
    HSDL_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), st));
    k_list_large_rows<<<sms * 4, 256, 0, st>>>(n, d_off, rows, count, small_cap, smem_cap);
    HSDL_LAUNCHED();
    k_sort_large<<<sms * 2, 512, smem, st>>>(rows, count, d_off, key, par, smem_cap, nullptr, nullptr);
    HSDL_LAUNCHED();
  }
  if (max_row > smem_cap) {
    int64_t P = 1;
    while (P < max_row) P <<= 1;
    uint64_t* gk = nullptr;
    int32_t* gp = nullptr;
    HSDL_CUDA(cudaMallocAsync(&gk, (size_t)P * sizeof(uint64_t), st));
    HSDL_CUDA(cudaMallocAsync(&gp, (size_t)P * sizeof(int32_t), st));
    HSDL_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), st));
    k_list_large_rows<<<sms * 4, 256, 0, st>>>(n, d_off, rows, count, smem_cap, (int32_t)max_row);
    HSDL_LAUNCHED();
    // one block walks the over-sized rows one after another through gk/gp
    k_sort_large<<<1, 1024, smem, st>>>(rows, count, d_off, key, par, smem_cap, gk, gp);
    HSDL_LAUNCHED();
    HSDL_CUDA(cudaFreeAsync(gk, st));
    HSDL_CUDA(cudaFreeAsync(gp, st));
  }
  HSDL_CUDA(cudaFreeAsync(rows, st));
  HSDL_CUDA(cudaFreeAsync(count, st));
  return HSDL_OK;
}

}  // namespace hsdl
