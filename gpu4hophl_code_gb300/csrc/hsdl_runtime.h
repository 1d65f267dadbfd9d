// Host-side runtime shared by the CUDA translation units: handles, error
// plumbing, device allocation with accounting, launch counting.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/hsdl.h"
#include "hsdl_device.cuh"

namespace hsdl {

void set_error(const std::string& msg);
std::atomic<int64_t>& launch_counter();

// Status-returning error propagation.
struct Status {
  int code = HSDL_OK;
  bool ok() const { return code == HSDL_OK; }
};

#define HSDL_CUDA(call)                                                                             \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) {                                                                        \
      ::hsdl::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                        \
      return (e_ == cudaErrorMemoryAllocation) ? HSDL_ERR_NOMEM : HSDL_ERR_CUDA;                    \
    }                                                                                               \
  } while (0)

#define HSDL_TRY(expr)           \
  do {                           \
    int s_ = (expr);             \
    if (s_ != HSDL_OK) return s_; \
  } while (0)

#define HSDL_LAUNCHED()                                            \
  do {                                                             \
    ::hsdl::launch_counter().fetch_add(1, std::memory_order_relaxed); \
    cudaError_t e_ = cudaGetLastError();                           \
    if (e_ != cudaSuccess) {                                       \
      ::hsdl::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_)); \
      return HSDL_ERR_CUDA;                                        \
    }                                                              \
  } while (0)

// A device buffer, stream-ordered: allocated with cudaMallocAsync and freed
// with cudaFreeAsync on the stream that owns it, so that allocation never
// synchronises the device (a persistent serving kernel keeps running while a
// build allocates and frees).  The owning stream must outlive the buffer.
template <class T>
struct DevBuf {
  T* p = nullptr;
  int64_t cap = 0;  // elements
  cudaStream_t st = nullptr;
  int alloc(int64_t n, cudaStream_t s = nullptr) {
    release();
    st = s;
    if (n <= 0) return HSDL_OK;
    HSDL_CUDA(cudaMallocAsync((void**)&p, (size_t)n * sizeof(T), st));
    cap = n;
    return HSDL_OK;
  }
  // grows to at least n elements keeping the first `keep` elements
  int grow(int64_t n, int64_t keep, cudaStream_t s) {
    if (n <= cap) return HSDL_OK;
    T* q = nullptr;
    HSDL_CUDA(cudaMallocAsync((void**)&q, (size_t)n * sizeof(T), s));
    if (keep > 0 && p) HSDL_CUDA(cudaMemcpyAsync(q, p, (size_t)keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
    if (p) HSDL_CUDA(cudaFreeAsync(p, s));
    p = q;
    cap = n;
    st = s;
    return HSDL_OK;
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    cap = 0;
  }
  int64_t bytes() const { return cap * (int64_t)sizeof(T); }
};

struct hsdl_graph_impl {
  int32_t n = 0;
  int64_t m2 = 0;
  int32_t max_w = 0;
  DevBuf<int64_t> rp;
  DevBuf<int2> adj;  // (neighbour, weight)
  std::vector<int64_t> h_rp;  // host copy of row_ptr (for sizing decisions)
};

// A built (or imported) label index resident in HBM, per-vertex CSR in two
// parallel arrays: key[] (hub:32 | hop:4 | distance:28, one 8-byte word per
// label, so a join gets hop and distance with the hub id) and par[]
// (parent_vertex).  Rows are sorted by key, the reference's order.  The
// arrays carry kRowPad spare entries at the end so that 16-byte aligned bulk
// copies of any row stay inside the allocation.
constexpr int64_t kRowPad = 8;
struct hsdl_index_impl {
  int32_t n = 0, K = 0;
  bool cleaned = false;
  DevBuf<int64_t> off;    // n+1
  DevBuf<uint64_t> key;   // hub:32 | hop:4 | distance:28
  DevBuf<int32_t> par;    // parent_vertex
  DevBuf<int32_t> wave_lo;    // generated, not yet cleaned: first hub of each hub's wave
  DevBuf<uint32_t> key32;     // compact query keys (Fmt32), when the index's ranges fit; else empty
  Fmt32 fmt32{0, 0};
  int32_t q_threads = 512;    // query kernel: threads per block
  int32_t q_lanes = 32;       // query kernel: lanes per query (8, 16 or 32)
  int32_t q_ahead = 0;        // query kernel: queries prefetched ahead per warp (0 = none)
  bool q_tuned = false;       // set by hsdl_set_query_tuning: the defaults below no longer apply
  int64_t total = 0;
  int64_t before = 0, after = 0, max_row = 0;
  int32_t waves = 0;
  double t_gen = 0, t_sort = 0, t_clean = 0;
  // work counted on the device during the build (for the roofline)
  int64_t work_relax = 0, work_join_reads = 0, work_labels_written = 0, work_clean_reads = 0, work_candidates = 0;
  int64_t work_join_visible = 0;
  // device memory of the build
  int64_t build_peak = 0, build_pool = 0, build_max_cand = 0;
  int32_t wave_splits = 0, pool_chunks = 0;
  int32_t pool_key_bytes = 8;  // bytes per key in the generation's label pool
  cudaStream_t stream = nullptr;
  std::vector<int64_t> h_off;  // host copy of offsets (path extraction, export)
};

int device_sm_count();
// Blocks of `kernel` (with `threads` threads and `smem` dynamic shared memory)
// that fit on one SM at once; grids are sized as SMs x this, so that a
// grid-stride loop runs in a single wave.
template <class K>
int resident_blocks(K kernel, int threads, size_t smem = 0) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem) != cudaSuccess || b < 1) b = 1;
  return b;
}
int max_row_length(hsdl_index_impl* idx, int64_t* out);  // recomputes from h_off

// A batch of graphs built as one disjoint union (see batched.cu): explicit wave
// bounds over the union's ids, each vertex's id inside its own graph (lid,
// device), its graph's hop bound (vk, device) and its graph's size (comp_n,
// host).
struct BatchPlan {
  std::vector<int32_t> bounds;
  std::vector<int64_t> comp_n;
  const int32_t* lid = nullptr;
  const uint8_t* vk = nullptr;
};

// kernels / stages implemented in the .cu files
// hub_limit > 0: only hubs [0, hub_limit) search (a partial index, used to
// time a configuration on the widest searches)
int build_index(hsdl_graph_impl* g, int32_t K, const hsdl_build_opts& opts, hsdl_index_impl* idx,
                const BatchPlan* plan = nullptr, int32_t hub_limit = 0);
int clean_index(hsdl_index_impl* idx);
// Device degree ranking + CSR from a host edge list (graph_dev.cu).
int build_graph_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                           bool rank_by_degree, int32_t* h_new_to_old, hsdl_graph_impl* g);
int group_lp(hsdl_graph_impl* g, int32_t gmax, int32_t max_iter, int32_t* group_of_vertex, int32_t* num_groups,
             int32_t* iterations_run);
int query_device(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                 int32_t* out, cudaStream_t st);
// Device check of a query batch's vertex ids: *d_first (device) becomes the
// smallest index of a query with s or t outside [0, n), all-ones if none.
int first_bad_query(hsdl_index_impl* idx, int64_t nq, const int32_t* s, const int32_t* t, unsigned long long* d_first,
                    cudaStream_t st);
// Loads every variant of the query kernel and the id check on the current
// device (cudaFuncGetAttributes forces a lazily loaded kernel to load).
int preload_query_kernels();
// (Re)builds the compact query keys of a finished index (after a build, a
// clean, an import or a batched split).
int make_query_keys(hsdl_index_impl* idx);
// Host-side failure injection for tests (hsdl_debug_inject_failure): true if
// the pass through `site` must fail; the error text is set.
bool injected_failure(int site);
int sort_rows(int32_t n, const int64_t* d_off, uint64_t* key, int32_t* par, int64_t max_row, cudaStream_t st);
int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st);  // out[n] = total

}  // namespace hsdl

struct hsdl_graph : hsdl::hsdl_graph_impl {};
struct hsdl_index : hsdl::hsdl_index_impl {};
