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
//    fragment the pool.
// For them, hsdl_query_batch_static stages through one file-scope device array
// of fixed size instead.  It calls no cudaMalloc, cudaFree or allocating
// library routine; it only copies, launches the id check and the query kernel
// and waits for its own stream.
//
// The array: HSDL_STATIC_QUERY_MAX queries x 4 int32 lanes (s, t, k, answer)
// plus one 256-byte tail holding the id check's result word, 16 MiB in all.
// The build loads modules lazily (CUDA's default), so a device gets the array
// when this file's module is first loaded there - at the set-up below, not
// when the library is loaded - and keeps it until the process exits.
//
// Set-up, once per device with that device current (hsdl_query_static_prepare,
// or the first hsdl_query_batch_static call on the device): look up the array's
// device address with cudaGetSymbolAddress (in host code the array's name is a
// host-side stand-in, not a device address) and load every variant of the
// query kernel and the id check, so that no later call - whatever query tuning
// is set - loads a module.  A module load may synchronise the device or
// allocate, so do the set-up before a serving loop starts or any stream
// capture begins.
//
// All calls share the array and it keeps the last call's contents.  Nothing
// in it must start at zero: a call writes the first nq entries of the three
// input lanes before the kernels read them, resets the id check's word, and
// the query kernel writes every one of the nq answers.  Calls that overlap on
// the GPU would race on the array, so the entry point holds a process-wide
// lock until its work on the stream has completed - on every return path,
// errors included.
#include <mutex>
#include <string>

#include "hsdl_device.cuh"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {

constexpr int64_t kStaticMax = HSDL_STATIC_QUERY_MAX;
constexpr int64_t kTail = 64;  // int32 words after the four lanes: the id check's result

// lanes: [0, max) s, [max, 2max) t, [2max, 3max) k, [3max, 4max) answers,
// then the id check's unsigned long long at [4max, 4max + 2)
static __device__ __align__(256) int32_t g_query_staging[4 * kStaticMax + kTail];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
int32_t* g_staging_addr[kMaxDevices] = {};

// Set-up on the current device (the caller holds g_static_mu): the array's
// device address, looked up once per device, and every query kernel loaded.
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
    HSDL_TRY(preload_query_kernels());
    g_staging_addr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_staging_addr[dev];
  return HSDL_OK;
}

// Waits for the stream on scope exit while armed.  Declared after the lock, so
// it runs before the lock is released: no work of a failed call can still be
// touching the array when the next call starts.  Its own status is ignored (a
// broken context reports its error through the call that broke it).
struct SyncOnExit {
  cudaStream_t st;
  bool armed = false;
  ~SyncOnExit() {
    if (armed) (void)cudaStreamSynchronize(st);
  }
};

}  // namespace

}  // namespace hsdl

using namespace hsdl;

extern "C" int hsdl_query_static_prepare(void) {
  std::lock_guard<std::mutex> lock(g_static_mu);
  int32_t* base = nullptr;
  return staging_address(&base);
}

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
  std::lock_guard<std::mutex> lock(g_static_mu);
  int32_t* base = nullptr;
  HSDL_TRY(staging_address(&base));
  cudaStream_t st = idx->stream;
  SyncOnExit sync{st};
  int32_t* ds = base;
  int32_t* dt = base + kStaticMax;
  int32_t* dk = base + 2 * kStaticMax;
  int32_t* dout = base + 3 * kStaticMax;
  unsigned long long* d_first = reinterpret_cast<unsigned long long*>(base + 4 * kStaticMax);
  const size_t bytes = sizeof(int32_t) * (size_t)nq;
  unsigned long long first = ~0ull;
  sync.armed = true;
  HSDL_CUDA(cudaMemcpyAsync(ds, s, bytes, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(dt, t, bytes, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(dk, k, bytes, cudaMemcpyHostToDevice, st));
  // ids are checked on the device, as in hsdl_query_batch; the query kernel
  // answers an id outside the index with INT32_MAX and reads nothing for it
  HSDL_TRY(first_bad_query(idx, nq, ds, dt, d_first, st));
  if (injected_failure(HSDL_FAIL_STATIC_QUERY)) return HSDL_ERR_CUDA;
  HSDL_TRY(query_device(idx, nq, ds, dt, dk, dout, st));
  HSDL_CUDA(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, st));
  HSDL_CUDA(cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, st));
  sync.armed = false;
  HSDL_CUDA(cudaStreamSynchronize(st));
  if (first != ~0ull) {
    set_error("hsdl_query_batch_static: query vertex out of range at query " + std::to_string(first));
    return HSDL_ERR_INVALID;
  }
  return HSDL_OK;
}
