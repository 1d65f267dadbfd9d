// HSDL oracle: a CPU restatement of the reference's hop-constrained 2-hop
// labeling path.
//
// TEST INFRASTRUCTURE ONLY.  Only the test suite, the smoke check and the CPU
// baseline leg of the benchmark load this library, and only as the checker or
// as the timed CPU baseline.  The product (libhsdl) never links or calls it.
//
// What it restates (reference file:line, paths inside the reference project):
//   orc_build (generation)  CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:45-224
//                           (HSDL_thread_function) and :513-632 (driver); variant 1:
//                           same file :226-370 (_2023WWW_thread_function)
//   sortL                   same file :373-419
//   clean                   same file :422-511 (hop_constrained_clean_L)
//   orc_query               CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144-222
//   orc_path                same file :224-319 (hop_constrained_extract_shortest_path)
//   orc_bf                  CPU_HopHL/include/graph_v_of_v/graph_v_of_v_hop_constrained_shortest_distance.h:7-38
//   orc_lp_group            Hybrid_Generation_Clean/include/vgroup/CDLP/GPU_Community_Detection.cuh:29-213
//                           and Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20-107,
//                           in the deterministic form this project defines (see orc_lp_group).
//
// Two deliberate, documented choices:
//  * parent_vertex on ties.  When several predecessors reach a (vertex, hop)
//    state with the same minimal distance, the reference keeps the first one
//    pushed, which depends on its heap's pop order among equal keys.  This
//    restatement keeps the smallest vertex id.  (hub, hop, distance) never
//    depends on it; the reference's own test pins parent only through path
//    validity (CPU_HopHL/include/HBPLL/test.h:105-131).
//  * wave mode.  With `wave_bounds` given, hubs are processed in waves
//    [b_i, b_{i+1}); every hub of a wave sees exactly the labels of hubs of
//    earlier waves, and a state (v,h,d) is dropped when an earlier-hop state of
//    the same hub at v already has distance <= d.  With waves of one hub this
//    is the reference's sequential run; with wider waves it yields the
//    superset that the GPU generation produces, and the clean then removes
//    exactly the extra labels.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

namespace {

struct Label {
  int32_t hub, parent, hop, dist;
};

static_assert(sizeof(Label) == 16, "label record is 4 x int32");

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Graph {
  int n;
  const int64_t* rp;
  const int32_t* col;
  const int32_t* w;
};

// Addressable binary heap over state ids, ordered by (distance, hop) ascending.
struct StateHeap {
  std::vector<int64_t> heap;  // state ids
  std::vector<int32_t>* pos;  // pos[state] = index in heap, -1 if absent
  const int32_t* dist;
  int kp1;
  bool less(int64_t a, int64_t b) const {
    if (dist[a] != dist[b]) return dist[a] < dist[b];
    return (a % kp1) < (b % kp1);
  }
  void set(size_t i, int64_t s) {
    heap[i] = s;
    (*pos)[s] = (int32_t)i;
  }
  void up(size_t i) {
    int64_t s = heap[i];
    while (i > 0) {
      size_t p = (i - 1) / 2;
      if (!less(s, heap[p])) break;
      set(i, heap[p]);
      i = p;
    }
    set(i, s);
  }
  void down(size_t i) {
    int64_t s = heap[i];
    size_t n = heap.size();
    for (;;) {
      size_t l = 2 * i + 1;
      if (l >= n) break;
      size_t c = l;
      if (l + 1 < n && less(heap[l + 1], heap[l])) c = l + 1;
      if (!less(heap[c], s)) break;
      set(i, heap[c]);
      i = c;
    }
    set(i, s);
  }
  void push(int64_t s) {
    heap.push_back(s);
    up(heap.size() - 1);
  }
  int64_t pop() {
    int64_t top = heap[0];
    (*pos)[top] = -1;
    int64_t last = heap.back();
    heap.pop_back();
    if (!heap.empty()) {
      heap[0] = last;
      (*pos)[last] = 0;
      down(0);
    }
    return top;
  }
};

struct Index {
  int n = 0, K = 0;
  std::vector<std::vector<Label>> L;
  double t_gen = 0, t_sort = 0, t_clean = 0;
  int64_t before = 0, after = 0;
  // work counters of the last generation
  int64_t popped = 0, relaxed = 0, query_reads = 0;
  int64_t hubs_searched = 0;  // hubs whose search ran (n unless a time cap stopped the generation)
};

// Time cap of the generation with the reference schedule (seconds, 0 = none):
// the watchdog pattern of the reference's experiment drivers
// (GPU4HSDL_EXP/CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:67-83):
// once it passes, workers start no further hub; the labels of the hubs
// searched so far are sorted and cleaned as usual.
double g_time_cap_s = 0;

// Per-worker scratch of the generation.
struct Scratch {
  std::vector<int32_t> dist, parent, pos;  // per (v,h) state
  std::vector<std::vector<std::pair<int32_t, int32_t>>> hubtab;  // per hub w: (dist, hop) of L[hub]
  std::vector<int64_t> touched_states;
  std::vector<int32_t> touched_hubs;
  Scratch(int n, int K) : dist((int64_t)n * (K + 1), INT_MAX), parent((int64_t)n * (K + 1), -1),
                          pos((int64_t)n * (K + 1), -1), hubtab(n) {}
};

bool label_less(const Label& a, const Label& b) {
  // compare_hop_constrained_two_hop_label (generation.h:373-387)
  if (a.hub != b.hub) return a.hub < b.hub;
  if (a.hop != b.hop) return a.hop < b.hop;
  return a.dist < b.dist;
}

// One hub's search (HSDL_thread_function, generation.h:45-224).
//  lock_scan(u, fn): calls fn(L_u) with the label list of u the pruning query
//                    reads, under whatever lock the caller needs.
//  emit(u, label):   records a new label of u.
//  wave: true = own-dominance by earlier-hop states instead of own labels.
template <class LockScan, class Emit>
void hub_search(const Graph& g, int K, int hub, Scratch& S, const std::vector<Label>& hub_labels,
                LockScan lock_scan, Emit emit, bool wave, Index* stats) {
  const int kp1 = K + 1;
  // Temp_L_vk: the hub's labels (plus its self label) indexed by their hub.
  for (const Label& x : hub_labels) {
    if (S.hubtab[x.hub].empty()) S.touched_hubs.push_back(x.hub);
    S.hubtab[x.hub].push_back({x.dist, x.hop});
  }
  if (S.hubtab[hub].empty()) S.touched_hubs.push_back(hub);
  S.hubtab[hub].push_back({0, 0});

  StateHeap Q;
  Q.pos = &S.pos;
  Q.dist = S.dist.data();
  Q.kp1 = kp1;
  int64_t s0 = (int64_t)hub * kp1;
  S.dist[s0] = 0;
  S.parent[s0] = hub;
  S.touched_states.push_back(s0);
  Q.push(s0);
  int64_t popped = 0, relaxed = 0, qreads = 0;

  while (!Q.heap.empty()) {
    int64_t st = Q.pop();
    popped++;
    int u = (int)(st / kp1), h = (int)(st % kp1);
    int P_u = S.dist[st];
    if (hub > u) continue;  // rank prune (generation.h:107-110)
    if (wave && h > 0) {
      // Own-dominance: a state of this hub at u with fewer hops and distance
      // <= P_u (pruned or not) drops this one.  States pop in (distance, hop)
      // order, so every such state is already final in S.dist.
      int m = INT_MAX;
      for (int hh = 0; hh < h; hh++) m = std::min(m, S.dist[(int64_t)u * kp1 + hh]);
      if (m <= P_u) continue;
    }
    bool label, expand;
    if (st == s0) {
      // The hub itself: its self label is already in place, the query
      // returns 0 and the state is expanded without a new label.
      label = false;
      expand = true;
    } else {
      // pruning query (generation.h:127-144)
      int q = INT_MAX;
      lock_scan(u, [&](const std::vector<Label>& Lu) {
        qreads += (int64_t)Lu.size();
        for (const Label& xx : Lu) {
          for (const auto& yy : S.hubtab[xx.hub]) {
            if (xx.hop + yy.second <= h) {
              long long d = (long long)xx.dist + yy.first;
              if (q > d) q = (int)d;
            }
          }
        }
      });
      label = P_u < q;
      expand = label || q == 0;
    }
    if (!expand) continue;
    if (label) emit(u, Label{hub, S.parent[st], h, P_u});
    if (h + 1 > K) continue;
    for (int64_t e = g.rp[u]; e < g.rp[u + 1]; e++) {
      int v = g.col[e];
      int nd = P_u + g.w[e];
      int64_t sv = (int64_t)v * kp1 + h + 1;
      relaxed++;
      if (S.dist[sv] == INT_MAX) {
        S.dist[sv] = nd;
        S.parent[sv] = u;
        S.touched_states.push_back(sv);
        Q.push(sv);
      } else if (nd < S.dist[sv]) {
        S.dist[sv] = nd;
        S.parent[sv] = u;
        if (S.pos[sv] >= 0) Q.up(S.pos[sv]);
      } else if (nd == S.dist[sv] && u < S.parent[sv] && S.pos[sv] >= 0) {
        S.parent[sv] = u;  // tie rule: smallest predecessor id
      }
    }
  }
  for (int64_t s : S.touched_states) {
    S.dist[s] = INT_MAX;
    S.parent[s] = -1;
    S.pos[s] = -1;
  }
  S.touched_states.clear();
  for (int x : S.touched_hubs) S.hubtab[x].clear();
  S.touched_hubs.clear();
  if (stats) {
    stats->popped += popped;
    stats->relaxed += relaxed;
    stats->query_reads += qreads;
  }
}

// Per-worker scratch of the 2023WWW search.
struct WwwScratch {
  std::vector<int32_t> dist, pred;                               // dist_hop: best distance so far, its predecessor
  std::vector<std::vector<std::pair<int32_t, int32_t>>> hubtab;  // Temp_L_vk: (dist, hop) of L[hub] per hub
  std::vector<int32_t> touched, touched_hubs;
  WwwScratch(int n) : dist(n, INT_MAX), pred(n, 0), hubtab(n) {}
};

// One hub's 2023WWW search (_2023WWW_thread_function, generation.h:226-370):
// hop-synchronous, no rank prune.  Vh[h] lists the vertices whose best
// distance improved in hop h - 1 (once per improving relaxation, so a vertex
// can appear, and be labelled, more than once); the improvements of a hop are
// applied in order at the start of the next (:282-291), and a vertex of Vh[h]
// gets the label (hub, h, dist_hop) iff that distance is below the pruning
// query at hop bound h (:304-336), and only then relaxes its neighbours
// (:338-347).  hub_labels are the hub's labels from earlier hubs (its own
// self label comes from hop 0 of this search).
template <class LockScan, class Emit>
void www_search(const Graph& g, int K, int hub, WwwScratch& S, const std::vector<Label>& hub_labels,
                LockScan lock_scan, Emit emit, Index* stats) {
  for (const Label& x : hub_labels) {
    if (S.hubtab[x.hub].empty()) S.touched_hubs.push_back(x.hub);
    S.hubtab[x.hub].push_back({x.dist, x.hop});
  }
  std::vector<std::vector<int32_t>> Vh((size_t)K + 2);
  Vh[0].push_back(hub);
  S.dist[hub] = 0;
  S.pred[hub] = hub;
  S.touched.push_back(hub);
  struct Update {
    int32_t v, d, p;
  };
  std::vector<Update> upd;
  int64_t popped = 0, relaxed = 0, qreads = 0;
  for (int h = 0; h <= K; h++) {
    for (const Update& x : upd) {
      if (S.dist[x.v] > x.d) {
        if (S.dist[x.v] == INT_MAX) S.touched.push_back(x.v);
        S.dist[x.v] = x.d;
        S.pred[x.v] = x.p;
      }
    }
    upd.clear();
    for (int u : Vh[h]) {
      popped++;
      const int P_u = S.dist[u];
      int q = INT_MAX;
      lock_scan(u, [&](const std::vector<Label>& Lu) {
        qreads += (int64_t)Lu.size();
        for (const Label& xx : Lu) {
          for (const auto& yy : S.hubtab[xx.hub]) {
            if (xx.hop + yy.second <= h) {
              long long d = (long long)xx.dist + yy.first;
              if (q > d) q = (int)d;
            }
          }
        }
      });
      if (!(P_u < q)) continue;
      emit(u, Label{hub, S.pred[u], h, P_u});
      for (int64_t e = g.rp[u]; e < g.rp[u + 1]; e++) {
        const int v = g.col[e], nd = P_u + g.w[e];
        relaxed++;
        if (nd < S.dist[v]) {
          Vh[h + 1].push_back(v);
          upd.push_back({v, nd, u});
        }
      }
    }
  }
  for (int v : S.touched) S.dist[v] = INT_MAX;
  S.touched.clear();
  for (int x : S.touched_hubs) S.hubtab[x].clear();
  S.touched_hubs.clear();
  if (stats) {
    stats->popped += popped;
    stats->relaxed += relaxed;
    stats->query_reads += qreads;
  }
}

void sort_all(Index& I) {
  for (auto& Lv : I.L) std::sort(Lv.begin(), Lv.end(), label_less);
}

// hop_constrained_clean_L (generation.h:422-511) on the sorted labels `in`.
// mode 0: vertices in order 0..n-1 with in-place replacement (the reference's
//         single-thread schedule).
// mode 1: every vertex reads the uncleaned input (any thread count).
void clean_labels(int n, const std::vector<std::vector<Label>>& in, std::vector<std::vector<Label>>& out,
                  int threads, int mode) {
  out.assign(n, {});
  auto one = [&](int v, std::vector<std::vector<std::pair<int32_t, int32_t>>>& T,
                 const std::vector<std::vector<Label>>& Lsrc) {
    std::vector<Label> fin;
    const std::vector<Label>& Lv = in[v];
    for (const Label& x : Lv) {
      int u = x.hub, uh = x.hop;
      const std::vector<Label>& Lu = (u == v) ? in[v] : Lsrc[u];
      int min_dis = INT_MAX;
      for (const Label& l1 : Lu) {
        for (const auto& l2 : T[l1.hub]) {
          if (l1.hop + l2.second <= uh) {
            long long qd = l1.dist + (long long)l2.first;
            if (qd < min_dis) min_dis = (int)qd;
          }
        }
      }
      if (min_dis > x.dist) {
        fin.push_back(x);
        T[u].push_back({x.dist, x.hop});
      }
    }
    for (const Label& x : fin) T[x.hub].clear();
    out[v].swap(fin);
  };
  if (mode == 0) {
    std::vector<std::vector<std::pair<int32_t, int32_t>>> T(n);
    for (int v = 0; v < n; v++) one(v, T, out);  // out[u<v] is already cleaned
    return;
  }
  std::atomic<int> next{0};
  auto worker = [&]() {
    std::vector<std::vector<std::pair<int32_t, int32_t>>> T(n);
    for (;;) {
      int v = next.fetch_add(64);
      if (v >= n) break;
      for (int x = v; x < std::min(n, v + 64); x++) one(x, T, in);
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < std::max(1, threads); i++) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
}

int query_one(const std::vector<Label>& Ls, const std::vector<Label>& Lt, int s, int t, int k) {
  // hop_constrained_extract_distance (two_hop_labels.h:144-222)
  if (k < 0) return INT_MAX;
  if (s == t) return 0;
  if (k == 0) return INT_MAX;
  long long best = INT_MAX;
  size_t i = 0, j = 0;
  while (i < Ls.size() && j < Lt.size()) {
    if (Ls[i].hub == Lt[j].hub) {
      size_t ie = i, je = j;
      while (ie < Ls.size() && Ls[ie].hub == Ls[i].hub) ie++;
      while (je < Lt.size() && Lt[je].hub == Lt[j].hub) je++;
      for (size_t a = i; a < ie; a++) {
        for (size_t b = j; b < je; b++) {
          if (Ls[a].hop + Lt[b].hop <= k) {
            long long d = (long long)Ls[a].dist + Lt[b].dist;
            if (best > d) best = d;
          } else {
            break;
          }
        }
      }
      i = ie;
      j = je;
    } else if (Ls[i].hub > Lt[j].hub) {
      j++;
    } else {
      i++;
    }
  }
  return (int)best;
}

thread_local char g_err[256];

}  // namespace

extern "C" {

// Builds labels.  threads: worker count (reference-style shared pool; results
// of generation before clean depend on scheduling when threads > 1).
// wave_bounds/n_bounds: optional wave schedule (see header comment); when
// given, generation is deterministic for any thread count.
// clean: 0 none, 1 clean (mode chosen by threads: 1 -> mode 0, else mode 1).
// variant: 0 HSDL_thread_function, 1 _2023WWW_thread_function (run with one
// thread in rank order, or in wave mode with any thread count).
void* orc_build(int n, const int64_t* rp, const int32_t* col, const int32_t* w, int K, int threads,
                const int32_t* wave_bounds, int n_bounds, int clean, int variant) {
  Graph g{n, rp, col, w};
  Index* I = new Index();
  I->n = n;
  I->K = K;
  I->L.assign(n, {});
  threads = std::max(1, threads);
  double t0 = now_s();
  const bool waves = wave_bounds && n_bounds >= 2;
  if (variant == 1) {
    std::vector<Index> stats(threads);
    if (!waves) {
      // rank order, labels visible as soon as they are written (generation.h:568-574 with one worker)
      WwwScratch S(n);
      std::vector<Label> snap;
      for (int hub = 0; hub < n; hub++) {
        snap = I->L[hub];
        www_search(
            g, K, hub, S, snap, [&](int u, auto fn) { fn(I->L[u]); },
            [&](int u, const Label& x) { I->L[u].push_back(x); }, &stats[0]);
      }
    } else {
      std::vector<std::vector<Label>> pending(n);
      std::vector<std::mutex> mtx(n);
      for (int b = 0; b + 1 < n_bounds; b++) {
        int lo = wave_bounds[b], hi = wave_bounds[b + 1];
        std::atomic<int> next{lo};
        auto worker = [&](int tid) {
          WwwScratch S(n);
          for (;;) {
            int hub = next.fetch_add(1);
            if (hub >= hi) break;
            www_search(
                g, K, hub, S, I->L[hub], [&](int u, auto fn) { fn(I->L[u]); },
                [&](int u, const Label& x) {
                  std::lock_guard<std::mutex> lk(mtx[u]);
                  pending[u].push_back(x);
                },
                &stats[tid]);
          }
        };
        std::vector<std::thread> pool;
        for (int i = 0; i < threads; i++) pool.emplace_back(worker, i);
        for (auto& t : pool) t.join();
        for (int v = 0; v < n; v++) {
          if (pending[v].empty()) continue;
          I->L[v].insert(I->L[v].end(), pending[v].begin(), pending[v].end());
          pending[v].clear();
        }
      }
    }
    for (auto& st : stats) {
      I->popped += st.popped;
      I->relaxed += st.relaxed;
      I->query_reads += st.query_reads;
    }
  } else if (waves) {
    // wave mode: every hub of a wave reads the labels of earlier waves only
    std::vector<std::vector<Label>> pending(n);
    std::vector<std::mutex> mtx(n);
    std::vector<Scratch*> scr;
    for (int i = 0; i < threads; i++) scr.push_back(new Scratch(n, K));
    std::vector<Index> stats(threads);
    for (int b = 0; b + 1 < n_bounds; b++) {
      int lo = wave_bounds[b], hi = wave_bounds[b + 1];
      std::atomic<int> next{lo};
      auto worker = [&](int tid) {
        for (;;) {
          int hub = next.fetch_add(1);
          if (hub >= hi) break;
          hub_search(
              g, K, hub, *scr[tid], I->L[hub], [&](int u, auto fn) { fn(I->L[u]); },
              [&](int u, const Label& x) {
                std::lock_guard<std::mutex> lk(mtx[u]);
                pending[u].push_back(x);
              },
              true, &stats[tid]);
        }
      };
      std::vector<std::thread> pool;
      for (int i = 0; i < threads; i++) pool.emplace_back(worker, i);
      for (auto& t : pool) t.join();
      for (int v = 0; v < n; v++) {
        if (pending[v].empty()) continue;
        I->L[v].insert(I->L[v].end(), pending[v].begin(), pending[v].end());
        pending[v].clear();
      }
    }
    for (auto* s : scr) delete s;
    for (auto& s : stats) {
      I->popped += s.popped;
      I->relaxed += s.relaxed;
      I->query_reads += s.query_reads;
    }
  } else {
    // reference schedule: hubs in rank order from a shared pool, labels
    // visible as soon as they are written (generation.h:586-595)
    std::vector<std::mutex> mtx(n);
    std::atomic<int> next{0};
    std::atomic<int64_t> searched{0};
    std::vector<Index> stats(threads);
    const double cap = g_time_cap_s;
    auto worker = [&](int tid) {
      Scratch S(n, K);
      std::vector<Label> snap;
      for (;;) {
        if (cap > 0 && now_s() - t0 > cap) break;
        int hub = next.fetch_add(1);
        if (hub >= n) break;
        searched.fetch_add(1);
        {
          std::lock_guard<std::mutex> lk(mtx[hub]);
          I->L[hub].push_back(Label{hub, hub, 0, 0});  // self label (generation.h:83-92)
          snap = I->L[hub];
        }
        snap.pop_back();  // hub_search adds the self entry to the hub table itself
        hub_search(
            g, K, hub, S, snap,
            [&](int u, auto fn) {
              std::lock_guard<std::mutex> lk(mtx[u]);
              fn(I->L[u]);
            },
            [&](int u, const Label& x) {
              std::lock_guard<std::mutex> lk(mtx[u]);
              I->L[u].push_back(x);
            },
            false, &stats[tid]);
      }
    };
    if (threads == 1) {
      // single thread: no copies needed, labels are read in place
      Scratch S(n, K);
      std::vector<Label> snap;
      for (int hub = 0; hub < n; hub++) {
        if (cap > 0 && now_s() - t0 > cap) break;
        searched.fetch_add(1);
        I->L[hub].push_back(Label{hub, hub, 0, 0});
        snap.assign(I->L[hub].begin(), I->L[hub].end() - 1);
        hub_search(
            g, K, hub, S, snap, [&](int u, auto fn) { fn(I->L[u]); },
            [&](int u, const Label& x) { I->L[u].push_back(x); }, false, &stats[0]);
      }
    } else {
      std::vector<std::thread> pool;
      for (int i = 0; i < threads; i++) pool.emplace_back(worker, i);
      for (auto& t : pool) t.join();
    }
    for (auto& s : stats) {
      I->popped += s.popped;
      I->relaxed += s.relaxed;
      I->query_reads += s.query_reads;
    }
    I->hubs_searched = searched.load();
  }
  if (variant != 1 && waves) {
    // in wave mode the self label is emitted by no search; add it per vertex
    // (the reference pushes it at the start of the hub's own search).
    for (int v = 0; v < n; v++) I->L[v].push_back(Label{v, v, 0, 0});
  }
  double t1 = now_s();
  sort_all(*I);
  double t2 = now_s();
  I->t_gen = t1 - t0;
  I->t_sort = t2 - t1;
  for (auto& x : I->L) I->before += (int64_t)x.size();
  I->after = I->before;
  if (clean) {
    std::vector<std::vector<Label>> out;
    clean_labels(n, I->L, out, threads, threads == 1 ? 0 : 1);
    I->L.swap(out);
    I->after = 0;
    for (auto& x : I->L) I->after += (int64_t)x.size();
  }
  I->t_clean = now_s() - t2;
  return I;
}

// Wraps externally supplied labels (per-vertex rows, each sorted by
// (hub, hop, distance)) as an oracle index.
void* orc_from_labels(int n, int K, const int64_t* offsets, const int32_t* labels) {
  Index* I = new Index();
  I->n = n;
  I->K = K;
  I->L.assign(n, {});
  for (int v = 0; v < n; v++) {
    for (int64_t i = offsets[v]; i < offsets[v + 1]; i++) {
      const int32_t* x = labels + 4 * i;
      I->L[v].push_back(Label{x[0], x[1], x[2], x[3]});
    }
  }
  for (auto& x : I->L) I->before += (int64_t)x.size();
  I->after = I->before;
  return I;
}

// Cleans the index in place.  mode 0 = reference single-thread schedule,
// 1 = every vertex against the uncleaned input.
void orc_clean(void* h, int threads, int mode) {
  Index* I = (Index*)h;
  sort_all(*I);
  double t0 = now_s();
  std::vector<std::vector<Label>> out;
  clean_labels(I->n, I->L, out, threads, mode);
  I->L.swap(out);
  I->t_clean = now_s() - t0;
  I->after = 0;
  for (auto& x : I->L) I->after += (int64_t)x.size();
}

// Time cap (seconds, 0 = none) of later builds with the reference schedule.
void orc_set_time_cap(double seconds) { g_time_cap_s = seconds > 0 ? seconds : 0; }

int64_t orc_size(void* h) {
  Index* I = (Index*)h;
  int64_t t = 0;
  for (auto& x : I->L) t += (int64_t)x.size();
  return t;
}

// info[0..5] = t_gen, t_sort, t_clean, before, after, hubs searched ; work[0..2] = popped, relaxed, query_reads
void orc_info(void* h, double* info, int64_t* work) {
  Index* I = (Index*)h;
  info[0] = I->t_gen;
  info[1] = I->t_sort;
  info[2] = I->t_clean;
  info[3] = (double)I->before;
  info[4] = (double)I->after;
  info[5] = (double)I->hubs_searched;
  if (work) {
    work[0] = I->popped;
    work[1] = I->relaxed;
    work[2] = I->query_reads;
  }
}

void orc_export(void* h, int64_t* offsets, int32_t* labels) {
  Index* I = (Index*)h;
  int64_t p = 0;
  offsets[0] = 0;
  for (int v = 0; v < I->n; v++) {
    for (const Label& x : I->L[v]) {
      labels[4 * p + 0] = x.hub;
      labels[4 * p + 1] = x.parent;
      labels[4 * p + 2] = x.hop;
      labels[4 * p + 3] = x.dist;
      p++;
    }
    offsets[v + 1] = p;
  }
}

void orc_query(void* h, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k, int32_t* out,
               int threads) {
  Index* I = (Index*)h;
  auto work = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; i++) out[i] = query_one(I->L[s[i]], I->L[t[i]], s[i], t[i], k[i]);
  };
  if (threads <= 1) {
    work(0, nq);
    return;
  }
  std::vector<std::thread> pool;
  int64_t chunk = (nq + threads - 1) / threads;
  for (int i = 0; i < threads; i++) {
    int64_t lo = i * chunk, hi = std::min<int64_t>(nq, lo + chunk);
    if (lo < hi) pool.emplace_back(work, lo, hi);
  }
  for (auto& th : pool) th.join();
}

// hop_constrained_extract_shortest_path (two_hop_labels.h:224-319), written
// iteratively.  Writes edges as (a,b) pairs; returns the count, -1 if `cap` is
// too small.
int orc_path(void* h, int s, int t, int k, int32_t* edges, int cap) {
  Index* I = (Index*)h;
  int cnt = 0;
  while (s != t) {
    const auto& Ls = I->L[s];
    const auto& Lt = I->L[t];
    long long best = INT_MAX;
    int ps = -1, pt = -1;
    size_t i = 0, j = 0;
    while (i < Ls.size() && j < Lt.size()) {
      if (Ls[i].hub == Lt[j].hub) {
        size_t ie = i, je = j;
        while (ie < Ls.size() && Ls[ie].hub == Ls[i].hub) ie++;
        while (je < Lt.size() && Lt[je].hub == Lt[j].hub) je++;
        for (size_t a = i; a < ie; a++) {
          for (size_t b = j; b < je; b++) {
            if (Lt[b].hop + Ls[a].hop <= k) {
              long long d = (long long)Ls[a].dist + Lt[b].dist;
              if (best > d) {
                best = d;
                ps = Ls[a].parent;
                pt = Lt[b].parent;
              }
            } else {
              break;
            }
          }
        }
        i = ie;
        j = je;
      } else if (Ls[i].hub > Lt[j].hub) {
        j++;
      } else {
        i++;
      }
    }
    if (best >= INT_MAX) break;
    if (s != ps) {
      if (cnt >= cap) return -1;
      edges[2 * cnt] = s;
      edges[2 * cnt + 1] = ps;
      cnt++;
      s = ps;
      k--;
    }
    if (t != pt) {
      if (cnt >= cap) return -1;
      edges[2 * cnt] = t;
      edges[2 * cnt + 1] = pt;
      cnt++;
      t = pt;
      k--;
    }
  }
  return cnt;
}

void orc_free(void* h) { delete (Index*)h; }

// graph_v_of_v_hop_constrained_shortest_distance (..._hop_constrained_shortest_distance.h:7-38)
void orc_bf(int n, const int64_t* rp, const int32_t* col, const int32_t* w, int src, int k, int32_t* dist) {
  std::vector<std::vector<std::pair<int, int>>> Q(k + 2);
  Q[0].push_back({src, 0});
  for (int i = 0; i < n; i++) dist[i] = INT_MAX;
  dist[src] = 0;
  for (int h = 0; h <= k; h++) {
    for (auto& xx : Q[h]) {
      int v = xx.first, dv = xx.second;
      if (v == src || dist[v] > dv) {
        dist[v] = dv;
        for (int64_t e = rp[v]; e < rp[v + 1]; e++) {
          if (dv + w[e] < dist[col[e]]) Q[h + 1].push_back({col[e], dv + w[e]});
        }
      }
    }
  }
}

const char* orc_last_error() { return g_err; }

}  // extern "C"

namespace {

struct OrcGroup {
  int64_t id, size;
  std::vector<int32_t> nodes;
  bool operator<(const OrcGroup& b) const { return size == b.size ? id < b.id : size < b.size; }
};

}  // namespace

extern "C" {

int orc_lp_assemble(int n, const int64_t* rp, const int32_t* label, int gmax, int32_t* group_of_vertex);

// Deterministic capped label propagation + the reference's group assembly.
//  Propagation (GPU_Community_Detection.cuh:29-91, made deterministic):
//   size[c] = |{v : label v = c}|; every vertex takes the most frequent label
//   among its neighbours that is its own or has size < gmax (ties: smaller
//   label; no eligible neighbour label: keep its own); the vertices proposing
//   label c != their own move iff size[c] + their number <= gmax; stop when
//   nothing moves or after max_iter rounds.
//  Assembly (CDLP_group.cuh:39-100): bucket by label in label order, drop
//   empty buckets; repeatedly take the largest group (by (size, id)) and merge
//   it with the largest other group that fits in gmax, else emit it; order the
//   emitted groups by total degree, largest first.
// group_of_vertex[v] = group index; returns the number of groups.
int orc_lp_group(int n, const int64_t* rp, const int32_t* col, int gmax, int max_iter, int32_t* group_of_vertex,
                 int32_t* iterations) {
  std::vector<int32_t> label(n), size(n), join(n), prop(n), nl(n);
  for (int v = 0; v < n; v++) label[v] = v;
  std::vector<uint32_t> nb;
  int it = 0;
  for (; it < max_iter; it++) {
    std::fill(size.begin(), size.end(), 0);
    std::fill(join.begin(), join.end(), 0);
    for (int v = 0; v < n; v++) size[label[v]]++;
    for (int v = 0; v < n; v++) {
      nb.clear();
      for (int64_t e = rp[v]; e < rp[v + 1]; e++) nb.push_back((uint32_t)label[col[e]]);
      std::sort(nb.begin(), nb.end());
      int32_t best = label[v];
      int64_t best_cnt = 0;
      for (size_t i = 0; i < nb.size();) {
        size_t j = i + 1;
        while (j < nb.size() && nb[j] == nb[i]) j++;
        int32_t c = (int32_t)nb[i];
        if ((c == label[v] || size[c] < gmax) && (int64_t)(j - i) > best_cnt) {
          best_cnt = (int64_t)(j - i);
          best = c;
        }
        i = j;
      }
      prop[v] = best;
      if (best != label[v]) join[best]++;
    }
    int64_t changed = 0;
    for (int v = 0; v < n; v++) {
      int32_t c = prop[v];
      nl[v] = (c != label[v] && size[c] + join[c] <= gmax) ? c : label[v];
      changed += nl[v] != label[v];
    }
    label.swap(nl);
    if (changed == 0) {
      it++;
      break;
    }
  }
  if (iterations) *iterations = it;
  return orc_lp_assemble(n, rp, label.data(), gmax, group_of_vertex);
}

// The reference's group assembly alone (CDLP_group.cuh:39-100) on given
// propagation labels (each in [0, n)).
int orc_lp_assemble(int n, const int64_t* rp, const int32_t* label, int gmax, int32_t* group_of_vertex) {
  std::vector<std::vector<int32_t>> buckets(n), groups;
  for (int v = 0; v < n; v++) buckets[label[v]].push_back(v);
  for (auto& b : buckets)
    if (!b.empty()) groups.push_back(b);
  std::set<OrcGroup> se;
  for (size_t g = 0; g < groups.size(); g++) se.insert(OrcGroup{(int64_t)g, (int64_t)groups[g].size(), groups[g]});
  std::vector<std::vector<int32_t>> after;
  while (!se.empty()) {
    auto it1 = std::prev(se.end());
    auto it2 = se.upper_bound(OrcGroup{(int64_t)groups.size(), gmax - it1->size, {}});
    bool merged = false;
    if (it2 != se.begin()) {
      --it2;
      if (it2 == it1) it2 = (it2 == se.begin()) ? se.end() : std::prev(it2);
      if (it2 != se.end() && it2 != it1 && it1->size + it2->size <= gmax) {
        OrcGroup a = *it1;
        a.size += it2->size;
        a.nodes.insert(a.nodes.end(), it2->nodes.begin(), it2->nodes.end());
        se.erase(it1);
        se.erase(it2);
        se.insert(a);
        merged = true;
      }
    }
    if (!merged) {
      after.push_back(it1->nodes);
      se.erase(it1);
    }
  }
  std::vector<OrcGroup> order;
  for (size_t g = 0; g < after.size(); g++) {
    int64_t tot = 0;
    for (int32_t v : after[g]) tot -= rp[v + 1] - rp[v];
    order.push_back(OrcGroup{(int64_t)g, tot, after[g]});
  }
  std::sort(order.begin(), order.end());
  for (size_t g = 0; g < order.size(); g++)
    for (int32_t v : order[g].nodes) group_of_vertex[v] = (int32_t)g;
  return (int)order.size();
}

}  // extern "C"
