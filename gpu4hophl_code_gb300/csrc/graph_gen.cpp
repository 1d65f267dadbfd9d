// Seeded synthetic graphs and degree-rank relabelling (host side).
//
// The reference reads SNAP graphs and ranks vertices by degree with an
// unstable std::sort (CPU_HopHL/include/graph_v_of_v/graph_v_of_v_update_
// vertexIDs_by_degrees_large_to_small.h:14-40).  Here every generator returns
// an undirected, simple, loop-free graph already relabelled by degree
// descending with ties broken by the smaller original id, as CSR rows sorted
// by neighbour id (the order the reference's sorted adjacency vectors keep).
//
// Reproducibility: randomness is SplitMix64 driven by integer arithmetic only,
// and the one transcendental step (Chung-Lu weights) uses the series below
// built from IEEE +,-,*,/ so results are bit-identical on x86-64 and aarch64
// (compile with -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "hsdl_internal.h"

namespace hsdl {

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform integer in [0, bound) (Lemire's multiply-shift with rejection)
  uint64_t below(uint64_t bound) {
    for (;;) {
      uint64_t x = next();
      unsigned __int128 m = (unsigned __int128)x * bound;
      uint64_t lo = (uint64_t)m;
      if (lo >= bound || lo >= (0 - bound) % bound) return (uint64_t)(m >> 64);
    }
  }
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
};

// ln(x), x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)).
double det_log(double x) {
  int e = 0;
  double m = std::frexp(x, &e);  // exact, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    e -= 1;
  }
  double z = (m - 1.0) / (m + 1.0), z2 = z * z, term = z, sum = 0.0;
  for (int k = 1; k < 60; k += 2) {
    sum += term / (double)k;
    term *= z2;
  }
  return 2.0 * sum + (double)e * 0.69314718055994530942;
}

// e^y via y = k ln2 + r, |r| <= ln2/2, Taylor series of e^r.
double det_exp(double y) {
  const double ln2 = 0.69314718055994530942;
  double kf = std::floor(y / ln2 + 0.5);
  double r = y - kf * ln2;
  double sum = 1.0, term = 1.0;
  for (int i = 1; i < 30; i++) {
    term *= r / (double)i;
    sum += term;
  }
  return std::ldexp(sum, (int)kf);
}

double det_pow(double x, double y) { return det_exp(y * det_log(x)); }

// Open-addressing set of undirected edges (a < b).
struct EdgeSet {
  std::vector<uint64_t> slots;
  uint64_t mask;
  explicit EdgeSet(int64_t expected) {
    uint64_t cap = 1024;
    while (cap < (uint64_t)expected * 2) cap <<= 1;
    slots.assign(cap, ~0ull);
    mask = cap - 1;
  }
  bool insert(uint32_t a, uint32_t b) {
    uint64_t key = ((uint64_t)a << 32) | b;
    uint64_t h = key * 0x9E3779B97F4A7C15ull;
    for (uint64_t i = (h >> 20) & mask;; i = (i + 1) & mask) {
      if (slots[i] == key) return false;
      if (slots[i] == ~0ull) {
        slots[i] = key;
        return true;
      }
    }
  }
};

struct EdgeList {
  std::vector<int32_t> a, b, w;
  void add(int32_t x, int32_t y, int32_t wt) {
    a.push_back(x);
    b.push_back(y);
    w.push_back(wt);
  }
};

int32_t draw_weight(SplitMix64& r, int32_t wmin, int32_t wmax) {
  return wmin + (int32_t)r.below((uint64_t)(wmax - wmin) + 1);
}

}  // namespace

// Builds the ranked CSR from an undirected simple edge list.
void build_ranked_csr(int32_t n, const int32_t* ea, const int32_t* eb, const int32_t* ew, int64_t m,
                      bool rank_by_degree, HostGraph& out) {
  std::vector<int64_t> deg(n, 0);
  for (int64_t i = 0; i < m; i++) {
    deg[ea[i]]++;
    deg[eb[i]]++;
  }
  out.n = n;
  out.new_to_old.resize(n);
  std::iota(out.new_to_old.begin(), out.new_to_old.end(), 0);
  if (rank_by_degree) {
    std::stable_sort(out.new_to_old.begin(), out.new_to_old.end(),
                     [&](int32_t x, int32_t y) { return deg[x] > deg[y]; });
  }
  std::vector<int32_t> old_to_new(n);
  for (int32_t i = 0; i < n; i++) old_to_new[out.new_to_old[i]] = i;
  out.row_ptr.assign((size_t)n + 1, 0);
  for (int32_t v = 0; v < n; v++) out.row_ptr[old_to_new[v] + 1] = deg[v];
  for (int32_t v = 0; v < n; v++) out.row_ptr[v + 1] += out.row_ptr[v];
  out.col.resize(2 * m);
  out.w.resize(2 * m);
  std::vector<int64_t> fill(out.row_ptr.begin(), out.row_ptr.end() - 1);
  for (int64_t i = 0; i < m; i++) {
    int32_t x = old_to_new[ea[i]], y = old_to_new[eb[i]];
    out.col[fill[x]] = y;
    out.w[fill[x]++] = ew[i];
    out.col[fill[y]] = x;
    out.w[fill[y]++] = ew[i];
  }
  std::vector<std::pair<int32_t, int32_t>> row;
  for (int32_t v = 0; v < n; v++) {
    int64_t lo = out.row_ptr[v], hi = out.row_ptr[v + 1];
    row.clear();
    for (int64_t e = lo; e < hi; e++) row.push_back({out.col[e], out.w[e]});
    std::sort(row.begin(), row.end());
    for (int64_t e = lo; e < hi; e++) {
      out.col[e] = row[e - lo].first;
      out.w[e] = row[e - lo].second;
    }
  }
}

static void finish(int32_t n, EdgeList& E, HostGraph& out) {
  build_ranked_csr(n, E.a.data(), E.b.data(), E.w.data(), (int64_t)E.a.size(), true, out);
}

void gen_erdos_renyi(int32_t n, int64_t m, int32_t wmin, int32_t wmax, uint64_t seed, HostGraph& out) {
  SplitMix64 r(seed);
  EdgeSet set(m);
  EdgeList E;
  while ((int64_t)E.a.size() < m) {
    uint32_t x = (uint32_t)r.below(n), y = (uint32_t)r.below(n);
    if (x == y) continue;
    if (x > y) std::swap(x, y);
    if (set.insert(x, y)) E.add(x, y, draw_weight(r, wmin, wmax));
  }
  finish(n, E, out);
}

// Chung-Lu: expected degree of vertex i proportional to (i+1)^(-1/(gamma-1)),
// scaled to mean `avg_deg` and capped at `max_deg`; n*avg_deg/2 distinct edges
// are drawn with both endpoints chosen in proportion to these weights.
void gen_chung_lu(int32_t n, double avg_deg, double gamma, double max_deg, int32_t wmin, int32_t wmax,
                  uint64_t seed, HostGraph& out) {
  std::vector<double> W(n);
  double expo = -1.0 / (gamma - 1.0), sum = 0.0;
  for (int32_t i = 0; i < n; i++) {
    W[i] = det_pow((double)i + 1.0, expo);
    sum += W[i];
  }
  double scale = avg_deg * (double)n / sum;
  for (int32_t i = 0; i < n; i++) W[i] = std::min(W[i] * scale, max_deg);
  // Vose alias table
  double tot = 0.0;
  for (double x : W) tot += x;
  std::vector<double> prob(n);
  std::vector<int32_t> alias(n, 0), small, large;
  for (int32_t i = 0; i < n; i++) {
    prob[i] = W[i] * (double)n / tot;
    (prob[i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    int32_t s = small.back(), l = large.back();
    small.pop_back();
    alias[s] = l;
    prob[l] = (prob[l] + prob[s]) - 1.0;
    if (prob[l] < 1.0) {
      large.pop_back();
      small.push_back(l);
    }
  }
  for (int32_t i : large) prob[i] = 1.0;
  for (int32_t i : small) prob[i] = 1.0;
  SplitMix64 r(seed);
  auto sample = [&]() -> uint32_t {
    uint32_t i = (uint32_t)r.below(n);
    return r.unit() < prob[i] ? i : (uint32_t)alias[i];
  };
  int64_t m = (int64_t)(avg_deg * (double)n / 2.0);
  EdgeSet set(m);
  EdgeList E;
  int64_t tries = 0, max_tries = 64 * m + 1024;
  while ((int64_t)E.a.size() < m && tries < max_tries) {
    tries++;
    uint32_t x = sample(), y = sample();
    if (x == y) continue;
    if (x > y) std::swap(x, y);
    if (set.insert(x, y)) E.add(x, y, draw_weight(r, wmin, wmax));
  }
  finish(n, E, out);
}

// Barabasi-Albert: a clique on m0+1 vertices, then each new vertex attaches to
// m0 distinct earlier vertices chosen in proportion to their degree.
void gen_barabasi_albert(int32_t n, int32_t m0, int32_t wmin, int32_t wmax, uint64_t seed, HostGraph& out) {
  SplitMix64 r(seed);
  EdgeList E;
  std::vector<int32_t> ends;  // every edge endpoint once per incidence
  int32_t core = std::min(n, m0 + 1);
  for (int32_t x = 0; x < core; x++)
    for (int32_t y = x + 1; y < core; y++) {
      E.add(x, y, draw_weight(r, wmin, wmax));
      ends.push_back(x);
      ends.push_back(y);
    }
  std::vector<int32_t> pick;
  for (int32_t v = core; v < n; v++) {
    pick.clear();
    while ((int32_t)pick.size() < std::min(m0, v)) {
      int32_t t = ends.empty() ? (int32_t)r.below(v) : ends[r.below(ends.size())];
      if (std::find(pick.begin(), pick.end(), t) == pick.end()) pick.push_back(t);
    }
    for (int32_t t : pick) {
      E.add(t, v, draw_weight(r, wmin, wmax));
      ends.push_back(t);
      ends.push_back(v);
    }
  }
  finish(n, E, out);
}

// Checks a CSR for the form every entry point requires.  Returns "" if valid.
std::string validate_csr(int32_t n, const int64_t* rp, const int32_t* col, const int32_t* w) {
  if (n < 1) return "graph must have at least one vertex";
  if (rp[0] != 0) return "row_ptr[0] must be 0";
  for (int32_t v = 0; v < n; v++) {
    if (rp[v + 1] < rp[v]) return "row_ptr is not non-decreasing at vertex " + std::to_string(v);
    for (int64_t e = rp[v]; e < rp[v + 1]; e++) {
      int32_t u = col[e];
      if (u < 0 || u >= n) return "neighbour id out of range at edge " + std::to_string(e);
      if (u == v) return "self loop at vertex " + std::to_string(v);
      if (w[e] < 1) return "edge weight below 1 at edge " + std::to_string(e);
      if (e > rp[v] && col[e - 1] >= u)
        return "row " + std::to_string(v) + " is not sorted by neighbour id or has a duplicate";
      // symmetry: (u -> v) with the same weight
      const int32_t* b = col + rp[u];
      const int32_t* f = std::lower_bound(b, col + rp[u + 1], v);
      if (f == col + rp[u + 1] || *f != v) return "edge " + std::to_string(v) + "-" + std::to_string(u) + " has no reverse";
      if (w[rp[u] + (f - b)] != w[e]) return "edge " + std::to_string(v) + "-" + std::to_string(u) + " has asymmetric weight";
    }
  }
  if (rp[n] > (int64_t)INT32_MAX) return "more than 2^31-1 adjacency entries";
  return "";
}

}  // namespace hsdl
