// Batched queries on host arrays without any device allocation.
//
// hsdl_query_batch stages the caller's (s, t, k) arrays and the answers in
// device memory it allocates for each call.  Some callers cannot allocate
// device memory at all:
//  * a thread answering queries next to long-running kernels (a serving loop,
//    a build on another stream): cudaMalloc / cudaFree can synchronise the
//    whole device and stall them, and pool growth can take locks;
//  * a process whose device memory belongs to another allocator with a hard
//    cap (a framework's caching pool), where allocations outside it fail or
//    fragment the pool;
//  * code running while another thread captures a CUDA graph in global
//    capture mode, where cudaMalloc is not permitted.
// For them, hsdl_query_batch_static stages through one file-scope device array
// of fixed size instead.  It calls no cudaMalloc, cudaFree or allocating
// library routine; it only copies, launches the query kernel and waits for its
// own stream.
//
// The array: HSDL_STATIC_QUERY_MAX queries x 4 int32 lanes (s, t, k, answer),
// 16 MiB, held by every GPU that loads the library until the process exits.
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it per device;
// make that first call before any stream capture begins.  All calls share the
// array and it keeps the last call's contents.  Nothing in it must start at
// zero: a call writes the first nq entries of the three input lanes before the
// kernel reads them, and the kernel writes every one of the nq answers.  Calls
// that overlap on the GPU would race on the array, so the entry point holds a
// process-wide lock until its copies back to the host have completed.
#include <mutex>
#include <string>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int64_t kStaticMax = HSDL_STATIC_QUERY_MAX;

// lanes: [0, max) s, [max, 2max) t, [2max, 3max) k, [3max, 4max) answers
static __device__ __align__(256) int32_t g_query_staging[4 * kStaticMax];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
int32_t* g_staging_addr[kMaxDevices] = {};

// Device address of g_query_staging on the current device (looked up once per
// device; the caller holds g_static_mu).
int staging_address(int32_t** out) {
  int dev = 0;
  HSDL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("hsdl_query_batch_static: device ordinal " + std::to_string(dev) + " out of range");
    return HSDL_ERR_INVALID;
  }
  if (g_staging_addr[dev] == nullptr) {
    void* p = nullptr;
    HSDL_CUDA(cudaGetSymbolAddress(&p, g_query_staging));
    g_staging_addr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_staging_addr[dev];
  return HSDL_OK;
}

}  // namespace

}  // namespace hsdl

using namespace hsdl;

extern "C" int hsdl_query_batch_static(hsdl_index* idx, int64_t nq, const int32_t* s, const int32_t* t,
                                       const int32_t* k, int32_t* out) {
  if (!idx || nq < 0) {
    set_error("hsdl_query_batch_static: null index or negative query count");
    return HSDL_ERR_INVALID;
  }
  if (nq > kStaticMax) {
    set_error("hsdl_query_batch_static: " + std::to_string(nq) + " queries exceed the static staging limit of " +
              std::to_string(kStaticMax) + " (HSDL_STATIC_QUERY_MAX); split the batch");
    return HSDL_ERR_INVALID;
  }
  if (nq == 0) return HSDL_OK;
  if (!s || !t || !k || !out) {
    set_error("hsdl_query_batch_static: null query array");
    return HSDL_ERR_INVALID;
  }
  for (int64_t i = 0; i < nq; i++) {
    if (s[i] < 0 || s[i] >= idx->n || t[i] < 0 || t[i] >= idx->n) {
      set_error("hsdl_query_batch_static: query vertex out of range at query " + std::to_string(i));
      return HSDL_ERR_INVALID;
    }
  }
  std::lock_guard<std::mutex> lock(g_static_mu);
  int32_t* base = nullptr;
  HSDL_TRY(staging_address(&base));
  cudaStream_t st = idx->stream;
  int32_t* ds = base;
  int32_t* dt = base + kStaticMax;
  int32_t* dk = base + 2 * kStaticMax;
  int32_t* dout = base + 3 * kStaticMax;
  const size_t bytes = sizeof(int32_t) * (size_t)nq;
  HSDL_CUDA(cudaMemcpyAsync(ds, s, bytes, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(dt, t, bytes, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(dk, k, bytes, cudaMemcpyHostToDevice, st));
  HSDL_TRY(query_device(idx, nq, ds, dt, dk, dout, st));
  HSDL_CUDA(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  return HSDL_OK;
}
