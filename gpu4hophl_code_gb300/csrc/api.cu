// C ABI entry points (include/hsdl.h): handles, validation, host<->device
// copies and the calls into the generation / clean / query stages.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "hsdl_device.cuh"
#include "hsdl_internal.h"
#include "hsdl_runtime.h"

namespace hsdl {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

std::atomic<int32_t>* failure_budget() {
  static std::atomic<int32_t> budget[HSDL_FAIL_SITE_MAX + 1];
  return budget;
}

bool injected_failure(int site) {
  std::atomic<int32_t>& b = failure_budget()[site];
  int32_t c = b.load();
  while (c > 0) {
    if (b.compare_exchange_weak(c, c - 1)) {
      set_error("injected failure at site " + std::to_string(site));
      return true;
    }
  }
  return false;
}

std::atomic<int64_t>& launch_counter() {
  static std::atomic<int64_t> c{0};
  return c;
}

int device_sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      cached = v;
    else
      return 1;
  }
  return cached;
}

std::vector<int32_t> wave_schedule(int32_t n, int32_t first, int32_t max_wave);
int32_t auto_max_wave(int32_t n, int64_t budget_bytes);

}  // namespace hsdl

using namespace hsdl;

struct hsdl_host_graph {
  HostGraph g;
};

#define HSDL_CHECK_ARG(cond, msg)   \
  do {                              \
    if (!(cond)) {                  \
      set_error(msg);               \
      return HSDL_ERR_INVALID;      \
    }                               \
  } while (0)

namespace {

int finish_host_graph(HostGraph&& g, hsdl_host_graph** out) {
  auto* h = new hsdl_host_graph();
  h->g = std::move(g);
  *out = h;
  return HSDL_OK;
}

int new_index(hsdl_index** out) {
  auto* idx = new hsdl_index();
  cudaError_t e = cudaStreamCreateWithFlags(&idx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete idx;
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    return HSDL_ERR_CUDA;
  }
  *out = idx;
  return HSDL_OK;
}

void free_index(hsdl_index* idx) {
  if (!idx) return;
  if (idx->stream) cudaStreamSynchronize(idx->stream);
  idx->off.release();
  idx->key.release();
  idx->key32.release();
  idx->par.release();
  idx->wave_lo.release();
  if (idx->stream) {
    cudaStreamSynchronize(idx->stream);
    cudaStreamDestroy(idx->stream);
  }
  delete idx;
}

// Copies row v of an index to the host as label keys and parents.
int fetch_row(hsdl_index* idx, int32_t v, std::vector<uint64_t>& k, std::vector<int32_t>& p) {
  int64_t lo = idx->h_off[v], len = idx->h_off[v + 1] - lo;
  k.resize(len);
  p.resize(len);
  if (len == 0) return HSDL_OK;
  HSDL_CUDA(cudaMemcpy(k.data(), idx->key.p + lo, len * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  HSDL_CUDA(cudaMemcpy(p.data(), idx->par.p + lo, len * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return HSDL_OK;
}

// Largest label set an import accepts (2^36 labels = 1 TiB of 16-byte records).
constexpr int64_t kMaxImportLabels = int64_t(1) << 36;

int upload_index(int32_t n, int32_t K, const int64_t* offsets, const hsdl_label* labels, hsdl_index* idx) {
  HSDL_CHECK_ARG(n >= 1 && n <= (int32_t)kIdMask, "vertex count out of range");
  HSDL_CHECK_ARG(K >= 1 && K <= kMaxK, "K must be in [1, 14]");
  HSDL_CHECK_ARG(offsets && offsets[0] == 0, "offsets[0] must be 0");
  int64_t total = offsets[n];
  // bounds before any host allocation: a corrupt count must come back as an
  // error, not as an exception through the C ABI
  HSDL_CHECK_ARG(total >= 0 && total <= kMaxImportLabels, "label count out of range");
  HSDL_CHECK_ARG(total == 0 || labels, "null label array");
  std::vector<uint64_t> keys;
  std::vector<int32_t> par;
  try {
    keys.resize((size_t)total);
    par.resize((size_t)total);
  } catch (const std::exception&) {
    set_error("host memory for " + std::to_string(total) + " labels");
    return HSDL_ERR_NOMEM;
  }
  int64_t mr = 0;
  for (int32_t v = 0; v < n; v++) {
    HSDL_CHECK_ARG(offsets[v + 1] >= offsets[v], "offsets must be non-decreasing");
    mr = std::max(mr, offsets[v + 1] - offsets[v]);
    uint64_t prev = 0;
    for (int64_t i = offsets[v]; i < offsets[v + 1]; i++) {
      const hsdl_label& x = labels[i];
      HSDL_CHECK_ARG(x.hub_vertex >= 0 && x.hub_vertex < n && x.hop >= 0 && x.hop <= K && x.distance >= 0 &&
                         (uint32_t)x.distance <= kDistMask,
                     "label field out of range at entry " + std::to_string(i));
      uint64_t key = lkey((uint32_t)x.hub_vertex, (uint32_t)x.hop, (uint32_t)x.distance);
      // equal labels may repeat: the reference's 2023WWW generation pushes a
      // label once per improving relaxation (generation.h:276-336)
      HSDL_CHECK_ARG(i == offsets[v] || prev <= key,
                     "row " + std::to_string(v) + " is not sorted by (hub, hop, distance)");
      prev = key;
      keys[i] = key;
      par[i] = x.parent_vertex;
    }
  }
  idx->n = n;
  idx->K = K;
  idx->total = total;
  idx->before = idx->after = total;
  idx->max_row = mr;
  cudaStream_t st = idx->stream;
  HSDL_TRY(idx->off.alloc((int64_t)n + 1, st));
  HSDL_TRY(idx->key.alloc(total + kRowPad, st));
  HSDL_TRY(idx->par.alloc(total + kRowPad, st));
  HSDL_CUDA(cudaMemcpyAsync(idx->off.p, offsets, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
  if (total > 0) {
    HSDL_CUDA(cudaMemcpyAsync(idx->key.p, keys.data(), sizeof(uint64_t) * total, cudaMemcpyHostToDevice, st));
    HSDL_CUDA(cudaMemcpyAsync(idx->par.p, par.data(), sizeof(int32_t) * total, cudaMemcpyHostToDevice, st));
  }
  HSDL_CUDA(cudaStreamSynchronize(st));
  idx->h_off.assign(offsets, offsets + n + 1);
  return make_query_keys(idx);
}

}  // namespace

namespace hsdl {

int new_index_handle(hsdl_index** out) { return new_index(out); }
void free_index_handle(hsdl_index* idx) { free_index(idx); }

// Copies a (validated) host CSR into g's device buffers.
int upload_graph(int32_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* w, hsdl_graph_impl* g) {
  g->n = n;
  g->m2 = row_ptr[n];
  std::vector<int2> adj((size_t)g->m2);
  int32_t mw = 0;
  for (int64_t e = 0; e < g->m2; e++) {
    adj[e] = make_int2(col[e], w[e]);
    mw = std::max(mw, w[e]);
  }
  g->max_w = mw;
  int rc = g->rp.alloc((int64_t)n + 1, nullptr);
  if (rc == HSDL_OK) rc = g->adj.alloc(std::max<int64_t>(1, g->m2), nullptr);
  if (rc == HSDL_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) rc = HSDL_ERR_CUDA;
  if (rc == HSDL_OK) {
    cudaError_t e1 = cudaMemcpy(g->rp.p, row_ptr, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice);
    cudaError_t e2 = g->m2 ? cudaMemcpy(g->adj.p, adj.data(), sizeof(int2) * g->m2, cudaMemcpyHostToDevice)
                           : cudaSuccess;
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      set_error(std::string("graph upload: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
      rc = HSDL_ERR_CUDA;
    }
  }
  if (rc != HSDL_OK) {
    g->rp.release();
    g->adj.release();
  }
  return rc;
}

}  // namespace hsdl

extern "C" {

const char* hsdl_last_error(void) { return last_error_cstr(); }
int32_t hsdl_version(void) { return 1; }
int64_t hsdl_launch_count(void) { return launch_counter().load(); }

int hsdl_debug_pool_used_high(int64_t* bytes, int32_t reset) {
  HSDL_CHECK_ARG(bytes, "null argument");
  int dev = 0;
  HSDL_CUDA(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  HSDL_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  if (reset) {
    unsigned long long zero = 0;
    HSDL_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
  }
  unsigned long long v = 0;
  HSDL_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &v));
  *bytes = (int64_t)v;
  return HSDL_OK;
}

int hsdl_debug_inject_failure(int32_t site, int32_t count) {
  HSDL_CHECK_ARG(site >= 1 && site <= HSDL_FAIL_SITE_MAX && count >= 0, "unknown failure site or negative count");
  failure_budget()[site].store(count);
  return HSDL_OK;
}

// ---------------------------------------------------------------------------
// host graphs
// ---------------------------------------------------------------------------
int hsdl_gen_erdos_renyi(int32_t n, int64_t m, int32_t wmin, int32_t wmax, uint64_t seed, hsdl_host_graph** out) {
  HSDL_CHECK_ARG(out && n >= 2 && n <= (int32_t)kIdMask, "n must be in [2, 2^28)");
  HSDL_CHECK_ARG(m >= 0 && m <= (int64_t)n * (n - 1) / 2, "m out of range");
  HSDL_CHECK_ARG(wmin >= 1 && wmax >= wmin, "weights must satisfy 1 <= wmin <= wmax");
  HostGraph g;
  gen_erdos_renyi(n, m, wmin, wmax, seed, g);
  return finish_host_graph(std::move(g), out);
}

int hsdl_gen_chung_lu(int32_t n, double avg_degree, double exponent, double max_degree, int32_t wmin, int32_t wmax,
                      uint64_t seed, hsdl_host_graph** out) {
  HSDL_CHECK_ARG(out && n >= 2 && n <= (int32_t)kIdMask, "n must be in [2, 2^28)");
  HSDL_CHECK_ARG(avg_degree > 0 && avg_degree < n - 1, "avg_degree out of range");
  HSDL_CHECK_ARG(exponent > 1.0 && max_degree >= 1.0, "exponent must be > 1 and max_degree >= 1");
  HSDL_CHECK_ARG(wmin >= 1 && wmax >= wmin, "weights must satisfy 1 <= wmin <= wmax");
  HostGraph g;
  gen_chung_lu(n, avg_degree, exponent, max_degree, wmin, wmax, seed, g);
  return finish_host_graph(std::move(g), out);
}

int hsdl_gen_barabasi_albert(int32_t n, int32_t m0, int32_t wmin, int32_t wmax, uint64_t seed,
                             hsdl_host_graph** out) {
  HSDL_CHECK_ARG(out && n >= 2 && n <= (int32_t)kIdMask, "n must be in [2, 2^28)");
  HSDL_CHECK_ARG(m0 >= 1 && m0 < n, "m0 must be in [1, n)");
  HSDL_CHECK_ARG(wmin >= 1 && wmax >= wmin, "weights must satisfy 1 <= wmin <= wmax");
  HostGraph g;
  gen_barabasi_albert(n, m0, wmin, wmax, seed, g);
  return finish_host_graph(std::move(g), out);
}

int hsdl_host_graph_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                               int32_t rank_by_degree, hsdl_host_graph** out) {
  HSDL_CHECK_ARG(out && n >= 1 && n <= (int32_t)kIdMask, "n must be in [1, 2^28)");
  HSDL_CHECK_ARG(m >= 0 && (m == 0 || (a && b && w)), "edge arrays missing");
  // drop self loops and duplicate edges (the reference's add_edge keeps the
  // last weight of a repeated edge, graph_v_of_v.h:90-108)
  std::vector<std::pair<uint64_t, int64_t>> order;
  order.reserve((size_t)m);
  for (int64_t i = 0; i < m; i++) {
    HSDL_CHECK_ARG(a[i] >= 0 && a[i] < n && b[i] >= 0 && b[i] < n, "edge endpoint out of range");
    HSDL_CHECK_ARG(w[i] >= 1, "edge weights must be >= 1");
    if (a[i] == b[i]) continue;
    uint32_t x = (uint32_t)std::min(a[i], b[i]), y = (uint32_t)std::max(a[i], b[i]);
    order.push_back({((uint64_t)x << 32) | y, i});
  }
  std::stable_sort(order.begin(), order.end(), [](const auto& p, const auto& q) { return p.first < q.first; });
  std::vector<int32_t> ea, eb, ew;
  for (size_t i = 0; i < order.size(); i++) {
    if (i + 1 < order.size() && order[i + 1].first == order[i].first) continue;  // keep the last
    ea.push_back((int32_t)(order[i].first >> 32));
    eb.push_back((int32_t)(order[i].first & 0xffffffffu));
    ew.push_back(w[order[i].second]);
  }
  HostGraph g;
  build_ranked_csr(n, ea.data(), eb.data(), ew.data(), (int64_t)ea.size(), rank_by_degree != 0, g);
  return finish_host_graph(std::move(g), out);
}

int hsdl_read_graph_text(const char* path, int32_t rank_by_degree, hsdl_host_graph** out) {
  HSDL_CHECK_ARG(path && out, "null argument");
  std::ifstream f(path);
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return HSDL_ERR_IO;
  }
  int64_t n = -1;
  std::vector<int32_t> a, b, w;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string tag;
    if (!(ss >> tag)) continue;
    if (tag == "|V|=") {
      if (!(ss >> n) || n < 1 || n > (int64_t)kIdMask) {
        set_error("|V|= out of range [1, 2^28): " + line);
        return HSDL_ERR_INVALID;
      }
    } else if (tag == "Edge") {
      long long x, y;
      double wt;
      if (!(ss >> x >> y >> wt)) {
        set_error("malformed Edge line: " + line);
        return HSDL_ERR_IO;
      }
      // range-checked before the narrowing casts, so an oversized id cannot
      // wrap into a valid one
      if (x < 0 || y < 0 || x > INT32_MAX || y > INT32_MAX || !(wt >= INT32_MIN && wt <= INT32_MAX)) {
        set_error("Edge line out of the int32 range: " + line);
        return HSDL_ERR_INVALID;
      }
      a.push_back((int32_t)x);
      b.push_back((int32_t)y);
      w.push_back((int32_t)wt);  // the reference parses with stod into weight_type
    }
  }
  HSDL_CHECK_ARG(n >= 1, "missing |V|= line");
  return hsdl_host_graph_from_edges((int32_t)n, (int64_t)a.size(), a.data(), b.data(), w.data(), rank_by_degree, out);
}

int hsdl_host_graph_get(const hsdl_host_graph* g, int32_t* n, int64_t* adj_entries, const int64_t** row_ptr,
                        const int32_t** col, const int32_t** w, const int32_t** new_to_old) {
  HSDL_CHECK_ARG(g, "null graph");
  if (n) *n = g->g.n;
  if (adj_entries) *adj_entries = (int64_t)g->g.col.size();
  if (row_ptr) *row_ptr = g->g.row_ptr.data();
  if (col) *col = g->g.col.data();
  if (w) *w = g->g.w.data();
  if (new_to_old) *new_to_old = g->g.new_to_old.data();
  return HSDL_OK;
}

void hsdl_host_graph_free(hsdl_host_graph* g) { delete g; }

int hsdl_validate_csr(int32_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* w) {
  HSDL_CHECK_ARG(n >= 1 && n <= (int32_t)kIdMask, "vertex count must be in [1, 2^28)");
  HSDL_CHECK_ARG(row_ptr && (row_ptr[n] == 0 || (col && w)), "null CSR array");
  std::string err = validate_csr(n, row_ptr, col, w);
  if (!err.empty()) {
    set_error(err);
    return HSDL_ERR_INVALID;
  }
  return HSDL_OK;
}

// ---------------------------------------------------------------------------
// device graphs
// ---------------------------------------------------------------------------
int hsdl_graph_create(int32_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* w, hsdl_graph** out) {
  HSDL_CHECK_ARG(out, "null output");
  HSDL_TRY(hsdl_validate_csr(n, row_ptr, col, w));
  auto* g = new hsdl_graph();
  int rc = upload_graph(n, row_ptr, col, w, g);
  if (rc != HSDL_OK) {
    delete g;
    return rc;
  }
  g->h_rp.assign(row_ptr, row_ptr + n + 1);
  *out = g;
  return HSDL_OK;
}

int hsdl_graph_create_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                                 int32_t rank_by_degree, int32_t* new_to_old, hsdl_graph** out) {
  HSDL_CHECK_ARG(out, "null output");
  HSDL_CHECK_ARG(n >= 1 && n <= (int32_t)kIdMask, "vertex count out of range");
  HSDL_CHECK_ARG(m >= 0 && (m == 0 || (a && b && w)), "bad edge arrays");
  auto* g = new hsdl_graph();
  const int rc = build_graph_from_edges(n, m, a, b, w, rank_by_degree != 0, new_to_old, g);
  if (rc != HSDL_OK) {
    delete g;
    return rc;
  }
  *out = g;
  return HSDL_OK;
}

int hsdl_graph_get_csr(hsdl_graph* g, int32_t* n, int64_t* adj_entries, int64_t* row_ptr, int32_t* col, int32_t* w) {
  HSDL_CHECK_ARG(g, "null graph");
  if (n) *n = g->n;
  if (adj_entries) *adj_entries = g->m2;
  HSDL_CUDA(cudaDeviceSynchronize());
  if (row_ptr) std::copy(g->h_rp.begin(), g->h_rp.end(), row_ptr);
  if ((col || w) && g->m2 > 0) {
    std::vector<int2> adj((size_t)g->m2);
    HSDL_CUDA(cudaMemcpy(adj.data(), g->adj.p, sizeof(int2) * g->m2, cudaMemcpyDeviceToHost));
    for (int64_t e = 0; e < g->m2; e++) {
      if (col) col[e] = adj[e].x;
      if (w) w[e] = adj[e].y;
    }
  }
  return HSDL_OK;
}

int hsdl_graph_destroy(hsdl_graph* g) {
  if (!g) return HSDL_OK;
  g->rp.release();
  g->adj.release();
  delete g;
  return HSDL_OK;
}

int hsdl_group_lp(hsdl_graph* g, int32_t max_group, int32_t max_iterations, int32_t* group_of_vertex,
                  int32_t* num_groups, int32_t* iterations) {
  HSDL_CHECK_ARG(g && group_of_vertex && num_groups, "null argument");
  HSDL_CHECK_ARG(max_group >= 1, "max_group must be >= 1");
  HSDL_CHECK_ARG(max_iterations >= 0, "max_iterations must be >= 0");
  return group_lp(g, max_group, max_iterations, group_of_vertex, num_groups, iterations);
}

// ---------------------------------------------------------------------------
// build / clean
// ---------------------------------------------------------------------------
void hsdl_build_opts_default(hsdl_build_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->struct_size = (int32_t)sizeof(hsdl_build_opts);
  o->clean = 1;
  o->first_wave = 1;
}

static int resolve_opts(const hsdl_build_opts* in, hsdl_build_opts* o) {
  hsdl_build_opts_default(o);
  if (in) {
    HSDL_CHECK_ARG(in->struct_size == (int32_t)sizeof(hsdl_build_opts), "hsdl_build_opts.struct_size mismatch");
    *o = *in;
  }
  HSDL_CHECK_ARG(o->first_wave >= 0 && o->max_wave >= 0, "wave widths must be >= 0");
  HSDL_CHECK_ARG(o->device_budget_bytes >= 0, "device_budget_bytes must be >= 0");
  HSDL_CHECK_ARG(o->block_threads == 0 || o->block_threads == 128 || o->block_threads == 256 ||
                     o->block_threads == 512,
                 "block_threads must be 0, 128, 256 or 512");
  HSDL_CHECK_ARG(o->frontier_tile >= 0, "frontier_tile must be >= 0");
  HSDL_CHECK_ARG(o->prune_lanes == 0 || o->prune_lanes == 8 || o->prune_lanes == 16 || o->prune_lanes == 32,
                 "prune_lanes must be 0, 8, 16 or 32");
  HSDL_CHECK_ARG(o->prune_pairs >= 0 && o->prune_pairs <= 2, "prune_pairs must be 0, 1 or 2");
  HSDL_CHECK_ARG(o->generation == 0 || o->generation == 1, "generation must be 0 (HSDL) or 1 (2023WWW)");
  HSDL_CHECK_ARG(o->prune_order >= 0 && o->prune_order <= 2, "prune_order must be 0, 1 or 2");
  HSDL_CHECK_ARG(o->pool_key_bytes == 0 || o->pool_key_bytes == 8, "pool_key_bytes must be 0 (auto) or 8");
  return HSDL_OK;
}

int hsdl_wave_bounds(int32_t n, const hsdl_build_opts* opts, int32_t* bounds, int32_t cap, int32_t* count) {
  HSDL_CHECK_ARG(n >= 1 && count, "bad arguments");
  hsdl_build_opts o;
  HSDL_TRY(resolve_opts(opts, &o));
  int64_t budget = o.device_budget_bytes;
  if (budget == 0) {
    size_t fb = 0, tb = 0;
    if (cudaMemGetInfo(&fb, &tb) == cudaSuccess) budget = (int64_t)fb;
  }
  int32_t mw = o.max_wave > 0 ? o.max_wave : auto_max_wave(n, budget);
  std::vector<int32_t> b = wave_schedule(n, o.first_wave > 0 ? o.first_wave : 1, mw);
  *count = (int32_t)b.size();
  if (bounds) {
    HSDL_CHECK_ARG(cap >= (int32_t)b.size(), "bounds buffer too small");
    std::copy(b.begin(), b.end(), bounds);
  }
  return HSDL_OK;
}

int hsdl_build(hsdl_graph* g, int32_t K, const hsdl_build_opts* opts, hsdl_index** out) {
  HSDL_CHECK_ARG(g && out, "null argument");
  HSDL_CHECK_ARG(K >= 1 && K <= kMaxK, "K must be in [1, 14]");
  HSDL_CHECK_ARG((int64_t)K * g->max_w <= (int64_t)kDistMask, "K * max edge weight must be < 2^28");
  hsdl_build_opts o;
  HSDL_TRY(resolve_opts(opts, &o));
  hsdl_index* idx = nullptr;
  HSDL_TRY(new_index(&idx));
  int rc = build_index(g, K, o, idx);
  if (rc == HSDL_OK && o.clean) rc = clean_index(idx);
  if (rc == HSDL_OK) rc = make_query_keys(idx);
  if (rc != HSDL_OK) {
    free_index(idx);
    return rc;
  }
  *out = idx;
  return HSDL_OK;
}

int hsdl_clean(hsdl_index* idx) {
  HSDL_CHECK_ARG(idx, "null index");
  if (idx->cleaned) return HSDL_OK;
  HSDL_TRY(clean_index(idx));
  return make_query_keys(idx);
}

// ---------------------------------------------------------------------------
// queries
// ---------------------------------------------------------------------------
int hsdl_query_batch_device(hsdl_index* idx, int64_t nq, const int32_t* d_s, const int32_t* d_t, const int32_t* d_k,
                            int32_t* d_out, void* stream) {
  HSDL_CHECK_ARG(idx && nq >= 0, "bad arguments");
  if (nq == 0) return HSDL_OK;
  HSDL_CHECK_ARG(d_s && d_t && d_k && d_out, "null query array");
  cudaStream_t st = stream ? (cudaStream_t)stream : idx->stream;
  return query_device(idx, nq, d_s, d_t, d_k, d_out, st);
}

int hsdl_query_batch(hsdl_index* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                     int32_t* out) {
  HSDL_CHECK_ARG(idx && nq >= 0, "bad arguments");
  if (nq == 0) return HSDL_OK;
  HSDL_CHECK_ARG(s && t && k && out, "null query array");
  cudaStream_t st = idx->stream;
  // queries, answers and the id check's result in one allocation; the ids
  // are checked on the device (a host loop over 10M queries cost a quarter of
  // the call), and a batch naming a vertex outside the index is an error
  int32_t* d = nullptr;
  HSDL_CUDA(cudaMallocAsync(&d, sizeof(int32_t) * 4 * nq + sizeof(unsigned long long), st));
  unsigned long long* d_first = (unsigned long long*)(d + 4 * nq);
  HSDL_CUDA(cudaMemcpyAsync(d, s, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(d + nq, t, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, st));
  HSDL_CUDA(cudaMemcpyAsync(d + 2 * nq, k, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, st));
  int rc = first_bad_query(idx, nq, d, d + nq, d_first, st);
  if (rc == HSDL_OK) rc = query_device(idx, nq, d, d + nq, d + 2 * nq, d + 3 * nq, st);
  unsigned long long first = ~0ull;
  if (rc == HSDL_OK) {
    HSDL_CUDA(cudaMemcpyAsync(out, d + 3 * nq, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, st));
    HSDL_CUDA(cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, st));
  }
  HSDL_CUDA(cudaFreeAsync(d, st));
  HSDL_CUDA(cudaStreamSynchronize(st));
  if (rc == HSDL_OK && first != ~0ull) {
    set_error("query vertex out of range at query " + std::to_string(first));
    return HSDL_ERR_INVALID;
  }
  return rc;
}

// hop_constrained_extract_shortest_path (two_hop_labels.h:224-319): repeated
// merge-joins that step from s and t to the parents of the best label pair.
int hsdl_extract_path(hsdl_index* idx, int32_t s, int32_t t, int32_t k, int32_t* edges, int32_t cap,
                      int32_t* n_edges) {
  HSDL_CHECK_ARG(idx && n_edges && (cap == 0 || edges), "bad arguments");
  HSDL_CHECK_ARG(s >= 0 && s < idx->n && t >= 0 && t < idx->n, "vertex out of range");
  HSDL_CUDA(cudaStreamSynchronize(idx->stream));
  int32_t cnt = 0;
  std::vector<uint64_t> ks, kt;
  std::vector<int32_t> ps, pt;
  while (s != t) {
    HSDL_TRY(fetch_row(idx, s, ks, ps));
    HSDL_TRY(fetch_row(idx, t, kt, pt));
    long long best = INT_MAX;
    int32_t bs = -1, bt = -1;
    size_t i = 0, j = 0;
    while (i < ks.size() && j < kt.size()) {
      uint32_t hi = lkey_hub(ks[i]), hj = lkey_hub(kt[j]);
      if (hi == hj) {
        size_t ie = i, je = j;
        while (ie < ks.size() && lkey_hub(ks[ie]) == hi) ie++;
        while (je < kt.size() && lkey_hub(kt[je]) == hj) je++;
        for (size_t a = i; a < ie; a++) {
          for (size_t b = j; b < je; b++) {
            if ((int)(lkey_hop(kt[b]) + lkey_hop(ks[a])) <= k) {
              long long d = (long long)lkey_dist(ks[a]) + lkey_dist(kt[b]);
              if (best > d) {
                best = d;
                bs = ps[a];
                bt = pt[b];
              }
            } else {
              break;
            }
          }
        }
        i = ie;
        j = je;
      } else if (hi > hj) {
        j++;
      } else {
        i++;
      }
    }
    if (best >= INT_MAX) break;
    if (s != bs) {
      HSDL_CHECK_ARG(cnt < cap, "edge buffer too small");
      edges[2 * cnt] = s;
      edges[2 * cnt + 1] = bs;
      cnt++;
      s = bs;
      k--;
    }
    if (t != bt) {
      HSDL_CHECK_ARG(cnt < cap, "edge buffer too small");
      edges[2 * cnt] = t;
      edges[2 * cnt + 1] = bt;
      cnt++;
      t = bt;
      k--;
    }
  }
  *n_edges = cnt;
  return HSDL_OK;
}

// ---------------------------------------------------------------------------
// index contents
// ---------------------------------------------------------------------------
int hsdl_index_get_info(hsdl_index* idx, hsdl_index_info* info) {
  HSDL_CHECK_ARG(idx && info, "null argument");
  info->n = idx->n;
  info->K = idx->K;
  info->cleaned = idx->cleaned ? 1 : 0;
  info->waves = idx->waves;
  info->labels = idx->total;
  info->labels_before_clean = idx->before;
  info->labels_after_clean = idx->after;
  info->device_bytes = idx->off.bytes() + idx->key.bytes() + idx->key32.bytes() + idx->par.bytes();
  info->query_key_bytes = idx->key32.p ? 4 : 8;
  info->build_pool_key_bytes = idx->pool_key_bytes;
  info->query_key_hub_bits = idx->key32.p ? 32 - (int32_t)idx->fmt32.hub_shift : 0;
  info->time_generate_s = idx->t_gen;
  info->time_sort_s = idx->t_sort;
  info->time_clean_s = idx->t_clean;
  info->max_row = idx->max_row;
  info->work_relaxations = idx->work_relax;
  info->work_join_reads = idx->work_join_reads;
  info->work_labels_written = idx->work_labels_written;
  info->work_clean_reads = idx->work_clean_reads;
  info->work_candidates = idx->work_candidates;
  info->work_join_visible = idx->work_join_visible;
  info->build_peak_bytes = idx->build_peak;
  info->build_pool_entries = idx->build_pool;
  info->build_max_candidates = idx->build_max_cand;
  info->build_wave_splits = idx->wave_splits;
  info->build_pool_chunks = idx->pool_chunks;
  return HSDL_OK;
}

int hsdl_export(hsdl_index* idx, int64_t* offsets, hsdl_label* labels) {
  HSDL_CHECK_ARG(idx && offsets && (idx->total == 0 || labels), "null argument");
  HSDL_CUDA(cudaStreamSynchronize(idx->stream));
  std::vector<uint64_t> keys((size_t)idx->total);
  std::vector<int32_t> par((size_t)idx->total);
  if (idx->total > 0) {
    HSDL_CUDA(cudaMemcpy(keys.data(), idx->key.p, sizeof(uint64_t) * idx->total, cudaMemcpyDeviceToHost));
    HSDL_CUDA(cudaMemcpy(par.data(), idx->par.p, sizeof(int32_t) * idx->total, cudaMemcpyDeviceToHost));
  }
  std::copy(idx->h_off.begin(), idx->h_off.end(), offsets);
  for (int64_t i = 0; i < idx->total; i++) {
    labels[i].hub_vertex = (int32_t)lkey_hub(keys[i]);
    labels[i].parent_vertex = par[i];
    labels[i].hop = (int32_t)lkey_hop(keys[i]);
    labels[i].distance = (int32_t)lkey_dist(keys[i]);
  }
  return HSDL_OK;
}

int hsdl_import(int32_t n, int32_t K, const int64_t* offsets, const hsdl_label* labels, hsdl_index** out) {
  HSDL_CHECK_ARG(out && offsets, "null argument");
  hsdl_index* idx = nullptr;
  HSDL_TRY(new_index(&idx));
  int rc = upload_index(n, K, offsets, labels, idx);
  if (rc != HSDL_OK) {
    free_index(idx);
    return rc;
  }
  *out = idx;
  return HSDL_OK;
}

// Clean_pc/main.cu:11-34 (save_labels): size_t V, then per vertex size_t n and
// n records of 4 int32 (hub, parent, hop, distance).
int hsdl_save_labels(hsdl_index* idx, const char* path) {
  HSDL_CHECK_ARG(idx && path, "null argument");
  std::vector<int64_t> off((size_t)idx->n + 1);
  std::vector<hsdl_label> lab((size_t)std::max<int64_t>(1, idx->total));
  HSDL_TRY(hsdl_export(idx, off.data(), lab.data()));
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    set_error(std::string("cannot write ") + path);
    return HSDL_ERR_IO;
  }
  size_t V = (size_t)idx->n;
  bool ok = std::fwrite(&V, sizeof(size_t), 1, f) == 1;
  for (int32_t v = 0; ok && v < idx->n; v++) {
    size_t c = (size_t)(off[v + 1] - off[v]);
    ok = std::fwrite(&c, sizeof(size_t), 1, f) == 1;
    if (ok && c) ok = std::fwrite(lab.data() + off[v], sizeof(hsdl_label), c, f) == c;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    set_error(std::string("write failed: ") + path);
    return HSDL_ERR_IO;
  }
  return HSDL_OK;
}

// Clean_pc/main.cu:36-58 (load_labels).
int hsdl_load_labels(const char* path, int32_t K, hsdl_index** out) {
  HSDL_CHECK_ARG(path && out, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return HSDL_ERR_IO;
  }
  // every count is checked against the bytes left in the file before it
  // sizes anything, so a corrupt count is an error, not a huge allocation
  std::fseek(f, 0, SEEK_END);
  const long long file_bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  size_t V = 0;
  bool ok = file_bytes > 0 && std::fread(&V, sizeof(size_t), 1, f) == 1 && V >= 1 && V <= kIdMask &&
            (long long)(V * sizeof(size_t)) <= file_bytes;
  std::vector<int64_t> off;
  std::vector<hsdl_label> lab;
  try {
    off.assign(ok ? V + 1 : 1, 0);
    for (size_t v = 0; ok && v < V; v++) {
      size_t c = 0;
      ok = std::fread(&c, sizeof(size_t), 1, f) == 1;
      const long long left = file_bytes - std::ftell(f);
      ok = ok && c <= (size_t)std::max(0LL, left) / sizeof(hsdl_label);
      if (!ok) break;
      size_t at = lab.size();
      lab.resize(at + c);
      if (c) ok = std::fread(lab.data() + at, sizeof(hsdl_label), c, f) == c;
      off[v + 1] = (int64_t)lab.size();
    }
  } catch (const std::exception&) {
    std::fclose(f);
    set_error(std::string("host memory while reading ") + path);
    return HSDL_ERR_NOMEM;
  }
  std::fclose(f);
  if (!ok) {
    set_error(std::string("malformed label file: ") + path);
    return HSDL_ERR_IO;
  }
  return hsdl_import((int32_t)V, K, off.data(), lab.empty() ? nullptr : lab.data(), out);
}

int hsdl_set_query_tuning(hsdl_index* idx, const hsdl_query_tuning* t) {
  HSDL_CHECK_ARG(idx && t && t->struct_size == (int32_t)sizeof(hsdl_query_tuning), "bad tuning argument");
  HSDL_CHECK_ARG(t->block_threads >= 32 && t->block_threads <= 1024 && t->block_threads % 32 == 0,
                 "block_threads must be a multiple of 32 in [32, 1024]");
  HSDL_CHECK_ARG(t->prefetch_ahead >= 0 && t->prefetch_ahead <= 8, "prefetch_ahead must be in [0, 8]");
  HSDL_CHECK_ARG(t->lanes_per_query == 8 || t->lanes_per_query == 16 || t->lanes_per_query == 32,
                 "lanes_per_query must be 8, 16 or 32");
  idx->q_threads = t->block_threads;
  idx->q_ahead = t->prefetch_ahead;
  idx->q_lanes = t->lanes_per_query;
  idx->q_tuned = true;
  return HSDL_OK;
}

int hsdl_get_query_tuning(hsdl_index* idx, hsdl_query_tuning* t) {
  HSDL_CHECK_ARG(idx && t, "null argument");
  t->struct_size = (int32_t)sizeof(hsdl_query_tuning);
  t->block_threads = idx->q_threads;
  t->prefetch_ahead = idx->q_ahead;
  t->lanes_per_query = idx->q_lanes;
  return HSDL_OK;
}

int hsdl_index_destroy(hsdl_index* idx) {
  free_index(idx);
  return HSDL_OK;
}

}  // extern "C"
