// Internal declarations shared by the host-side translation units of libhsdl.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace hsdl {

// A host-side CSR graph, vertices in rank order (id 0 = highest rank).
struct HostGraph {
  int32_t n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col, w;
  std::vector<int32_t> new_to_old;  // rank id -> id before relabelling
};

void build_ranked_csr(int32_t n, const int32_t* ea, const int32_t* eb, const int32_t* ew, int64_t m,
                      bool rank_by_degree, HostGraph& out);
void gen_erdos_renyi(int32_t n, int64_t m, int32_t wmin, int32_t wmax, uint64_t seed, HostGraph& out);
void gen_chung_lu(int32_t n, double avg_deg, double gamma, double max_deg, int32_t wmin, int32_t wmax,
                  uint64_t seed, HostGraph& out);
void gen_barabasi_albert(int32_t n, int32_t m0, int32_t wmin, int32_t wmax, uint64_t seed, HostGraph& out);
std::string validate_csr(int32_t n, const int64_t* rp, const int32_t* col, const int32_t* w);

}  // namespace hsdl
