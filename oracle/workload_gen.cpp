// The seeded synthetic workload graphs for the checkers (TEST INFRASTRUCTURE
// ONLY): the same generator source as the product library
// (gpu4hophl_code_gb300/csrc/graph_gen.cpp, compiled into liboracle.so too),
// so that the CPU arm of the benchmark builds exactly the GPU arm's graph
// without loading the product library.  Not part of the reference: it reads
// SNAP files instead.
#include <cstdint>
#include <cstring>

#include "../gpu4hophl_code_gb300/csrc/hsdl_internal.h"

extern "C" {

// Chung-Lu graph ranked by degree (ties by id), CSR rows sorted by neighbour;
// returns a handle, *adj_entries = 2m.
void* orc_gen_chung_lu(int32_t n, double avg_deg, double gamma, double max_deg, int32_t wmin, int32_t wmax,
                       uint64_t seed, int64_t* adj_entries) {
  auto* g = new hsdl::HostGraph();
  hsdl::gen_chung_lu(n, avg_deg, gamma, max_deg, wmin, wmax, seed, *g);
  *adj_entries = (int64_t)g->col.size();
  return g;
}

void orc_graph_copy(void* h, int64_t* row_ptr, int32_t* col, int32_t* w) {
  auto* g = static_cast<hsdl::HostGraph*>(h);
  std::memcpy(row_ptr, g->row_ptr.data(), sizeof(int64_t) * g->row_ptr.size());
  std::memcpy(col, g->col.data(), sizeof(int32_t) * g->col.size());
  std::memcpy(w, g->w.data(), sizeof(int32_t) * g->w.size());
}

void orc_graph_free(void* h) { delete static_cast<hsdl::HostGraph*>(h); }

}  // extern "C"
