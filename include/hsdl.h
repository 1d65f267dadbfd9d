/*
 * hsdl.h - C ABI of the GB300 hop-constrained shortest-distance 2-hop
 * labeling (HSDL) engine: label generation, canonical clean and (s,t,k)
 * distance queries on one GPU.
 *
 * Every function returns an int status (HSDL_OK = 0); on failure
 * hsdl_last_error() returns a message for the calling thread.  Handles are
 * opaque.  A handle may be used from one thread at a time; different handles
 * may be used concurrently.  No torch or CUDA types appear in the signatures:
 * streams are passed as `void*` (a cudaStream_t, NULL = the handle's own).
 *
 * Each entry point names the reference interface it replaces, as
 * file:line inside the reference project (rucdatascience/GPU4HopHL_code).
 *
 * Limits (checked, HSDL_ERR_INVALID when exceeded): vertex count < 2^28,
 * hop bound 1 <= K <= 14, edge weights >= 1 and K * max weight < 2^28.
 */
#ifndef HSDL_H
#define HSDL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HSDL_OK 0
#define HSDL_ERR_INVALID 1 /* bad argument or malformed input */
#define HSDL_ERR_CUDA 2    /* CUDA runtime failure (no device, launch error) */
#define HSDL_ERR_NOMEM 3   /* allocation failed or over the caller's budget */
#define HSDL_ERR_TIMEOUT 4 /* a bounded wait ran out (hsdl_serve_wait, hsdl_serve_wait_graph, the loop draining) */
#define HSDL_ERR_STATE 5   /* call not valid in the handle's current state */
#define HSDL_ERR_FULL 6    /* a queue or slot table is full */
#define HSDL_ERR_IO 7      /* file could not be read or written */

/* One label, byte-identical to the reference record
 * hop_constrained_two_hop_label {hub_vertex, parent_vertex, hop, distance}
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:6-21). */
typedef struct hsdl_label {
  int32_t hub_vertex;
  int32_t parent_vertex;
  int32_t hop;
  int32_t distance;
} hsdl_label;

/* Message of the last failing call on this thread ("" if none). */
const char* hsdl_last_error(void);
/* ABI version of this library. */
int32_t hsdl_version(void);
/* Number of CUDA kernels this library has launched in this process. */
int64_t hsdl_launch_count(void);
/* Host-side failure injection, for tests of error paths (no counterpart in
 * the reference): the next `count` passes through failure site `site` return
 * HSDL_ERR_CUDA with the message "injected failure at site <site>", without
 * touching the GPU.  Sites: HSDL_FAIL_STATIC_QUERY = inside
 * hsdl_query_batch_static, after its input copies and id check are queued
 * and before the query kernel.  count = 0 disarms. */
#define HSDL_FAIL_STATIC_QUERY 1
#define HSDL_FAIL_SITE_MAX 1
int hsdl_debug_inject_failure(int32_t site, int32_t count);
/* High-water mark, in bytes, of the current device's default memory pool
 * (the pool the library's stream-ordered allocations draw from) since the last
 * reset; reset != 0 first resets it to the memory in use.  For tests that
 * check an entry point allocates nothing (no counterpart in the reference). */
int hsdl_debug_pool_used_high(int64_t* bytes, int32_t reset);

/* ------------------------------------------------------------------------
 * Host graphs: seeded synthetic generators and loaders.  The result is an
 * undirected simple graph relabelled by degree descending (ties: smaller
 * original id first), as CSR rows sorted by neighbour id.  Replaces
 * graph_v_of_v_update_vertexIDs_by_degrees_large_to_small
 * (CPU_HopHL/include/graph_v_of_v/graph_v_of_v_update_vertexIDs_by_degrees_
 * large_to_small.h:14-40, whose std::sort leaves ties unordered) and
 * graph_v_of_v::txt_read (CPU_HopHL/include/graph_v_of_v/graph_v_of_v.h:242).
 * ---------------------------------------------------------------------- */
typedef struct hsdl_host_graph hsdl_host_graph;

int hsdl_gen_erdos_renyi(int32_t n, int64_t m, int32_t wmin, int32_t wmax, uint64_t seed,
                         hsdl_host_graph** out);
int hsdl_gen_chung_lu(int32_t n, double avg_degree, double exponent, double max_degree, int32_t wmin,
                      int32_t wmax, uint64_t seed, hsdl_host_graph** out);
int hsdl_gen_barabasi_albert(int32_t n, int32_t m0, int32_t wmin, int32_t wmax, uint64_t seed,
                             hsdl_host_graph** out);
/* Undirected edge list (a[i], b[i], w[i]); rank_by_degree = 0 keeps ids. */
int hsdl_host_graph_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                               int32_t rank_by_degree, hsdl_host_graph** out);
/* graph_v_of_v text format ("|V|= n", "Edge a b w" lines). */
int hsdl_read_graph_text(const char* path, int32_t rank_by_degree, hsdl_host_graph** out);
/* Pointers stay valid until hsdl_host_graph_free.  new_to_old may be NULL. */
int hsdl_host_graph_get(const hsdl_host_graph* g, int32_t* n, int64_t* adj_entries, const int64_t** row_ptr,
                        const int32_t** col, const int32_t** w, const int32_t** new_to_old);
void hsdl_host_graph_free(hsdl_host_graph* g);
/* Checks the CSR form every device entry point requires. */
int hsdl_validate_csr(int32_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* w);

/* ------------------------------------------------------------------------
 * Device graphs.  Copies a host CSR (ids = ranks, 0 highest) to HBM.  Plays
 * the role of toCSR / graph_v_of_v_to_CSR + the managed-memory copy
 * (Hybrid_Generation_Clean/include/graph/csr_graph.hpp:38,117).
 * ---------------------------------------------------------------------- */
typedef struct hsdl_graph hsdl_graph;

int hsdl_graph_create(int32_t n, const int64_t* row_ptr, const int32_t* col, const int32_t* w,
                      hsdl_graph** out);
int hsdl_graph_destroy(hsdl_graph* g);
/* Builds the device graph from an undirected simple edge list (a[i], b[i],
 * w[i], host arrays) on the GPU: degree ranking, largest degree first and ties
 * by smaller id, then the CSR with rows sorted by neighbour - bit-identical to
 * hsdl_host_graph_from_edges followed by hsdl_graph_create, without the host
 * work.  Replaces graph_v_of_v_update_vertexIDs_by_degrees_large_to_small
 * (CPU_HopHL/include/graph_v_of_v/graph_v_of_v_update_vertexIDs_by_degrees_large_to_small.h:14-40)
 * and toCSR (Hybrid_Generation_Clean/include/graph/csr_graph.hpp:38-115) run
 * on the host.  rank_by_degree = 0 keeps the ids.  new_to_old (n entries, may
 * be NULL) receives the original id of each ranked vertex. */
int hsdl_graph_create_from_edges(int32_t n, int64_t m, const int32_t* a, const int32_t* b, const int32_t* w,
                                 int32_t rank_by_degree, int32_t* new_to_old, hsdl_graph** out);
/* Copies a device graph's CSR to host arrays: row_ptr[n+1], col[adj], w[adj]
 * (any of the three may be NULL to skip it); *n and *adj_entries receive the
 * sizes. */
int hsdl_graph_get_csr(hsdl_graph* g, int32_t* n, int64_t* adj_entries, int64_t* row_ptr, int32_t* col, int32_t* w);

/* ------------------------------------------------------------------------
 * Label-propagation grouping.  Replaces generate_Group_CDLP(graph, groups,
 * G_max) (Hybrid_Generation_Clean/include/vgroup/CDLP_group.cuh:20) and its
 * CDLP_GPU kernels (.../vgroup/CDLP/GPU_Community_Detection.cuh:29-213), in
 * a deterministic form: capped label propagation (a label's joiners move only
 * if they all fit under max_group), then the reference's greedy merge of small
 * groups and ordering by total degree.  group_of_vertex[v] = index of v's
 * group in that order; *num_groups = groups; *iterations = rounds run.
 * ---------------------------------------------------------------------- */
int hsdl_group_lp(hsdl_graph* g, int32_t max_group, int32_t max_iterations, int32_t* group_of_vertex,
                  int32_t* num_groups, int32_t* iterations);

/* ------------------------------------------------------------------------
 * Label generation.  Replaces hop_constrained_two_hop_labels_generation
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:513)
 * and the GPU label_gen (Hybrid_Generation_Clean/src/label_gen.cu:603).
 * Hubs are processed in rank order in waves; a wave's hubs see the labels of
 * all earlier waves.  The result (before clean) is a superset of the
 * canonical labels; with opts->clean = 1 the canonical set is returned.
 * ---------------------------------------------------------------------- */
typedef struct hsdl_build_opts {
  int32_t struct_size;    /* sizeof(hsdl_build_opts) */
  int32_t clean;          /* 1: run hsdl_clean after generation (default 1) */
  int32_t first_wave;     /* hubs in the first wave (default 1) */
  int32_t max_wave;       /* widest wave; waves double up to it (0 = auto) */
  int32_t block_threads;  /* threads per expansion block: 128, 256 or 512 (0 = 256) */
  int32_t frontier_tile;  /* frontier entries an expansion block takes at a time (0 = one block's worth) */
  int32_t prune_lanes;    /* lanes per candidate in the pruning join: 8, 16 or 32 (0 = per wave, by mean row length) */
  int32_t prune_pairs;    /* label pairs each lane of the pruning join loads per step: 1 or 2 (0 = 1) */
  int32_t generation;     /* 0 = the HSDL search (HSDL_thread_function, generation.h:45-224; default);
                             1 = the 2023WWW search (_2023WWW_thread_function, generation.h:226-370;
                             the reference's use_2023WWW_generation): no rank prune, so more labels
                             before the clean; the cleaned labels are the same */
  int32_t prune_order;    /* 0 = each hop's candidates grouped by vertex-id range before the pruning join,
                             so joins of one vertex's candidates read its row while L2 holds it (default);
                             1 = expansion order.  Neither changes a label */
  int32_t pool_key_bytes; /* bytes per label key in the generation's label pool: 0 = 4 when every hub id,
                             hop and distance fit a 32-bit key (hub:H | hop:P | distance:D), else 8;
                             8 = always 8.  Changes no label */
  int32_t reserved;       /* 0 */
  int64_t device_budget_bytes; /* 0 = no limit beyond free HBM */
} hsdl_build_opts;

void hsdl_build_opts_default(hsdl_build_opts* opts);
/* Wave boundaries [b0=0, b1, ..., bW=n] the build uses for these options. */
int hsdl_wave_bounds(int32_t n, const hsdl_build_opts* opts, int32_t* bounds, int32_t cap, int32_t* count);

typedef struct hsdl_index hsdl_index;

int hsdl_build(hsdl_graph* g, int32_t K, const hsdl_build_opts* opts, hsdl_index** out);

/* Builds (and cleans) many graphs at once: graph i is the CSR (n[i],
 * row_ptr[i], col[i], w[i]) with hop bound K[i]; out[i] receives its index,
 * bit-identical to hsdl_build of that graph alone.  The graphs run as one
 * disjoint union whose waves hold the same ranks of many graphs together;
 * graphs are grouped, in input order, into sub-batches whose estimated build
 * bytes fit opts->device_budget_bytes (0 = 45% of the HBM free when the
 * sub-batch starts; the indexes already built stay resident), and a
 * sub-batch that runs out of memory is built again as two halves.  A batched wave holds at
 * most 64 rank layers and opts->max_wave hubs (0 = 262144).  No counterpart
 * in the reference, which builds one graph per run. */
int hsdl_build_batched(int32_t num_graphs, const int32_t* n, const int64_t* const* row_ptr,
                       const int32_t* const* col, const int32_t* const* w, const int32_t* K,
                       const hsdl_build_opts* opts, hsdl_index** out);

/* Autotuning of the launch shapes above (block_threads, frontier_tile,
 * prune_lanes, max_wave); the labels never depend on them.  Times the
 * generation of the graph's first sample_hubs hubs (0 = all of them up to 2M
 * vertices, else 262144), the highest-ranked and widest searches first,
 * under candidate settings by coordinate
 * descent, and writes the fastest into *opts (its other fields are kept).
 * best_seconds and trials (either may be NULL) receive the fastest sample
 * time and the number of timed runs.  No counterpart in the reference, whose
 * launch shapes are compile-time constants. */
int hsdl_build_autotune(hsdl_graph* g, int32_t K, int32_t sample_hubs, hsdl_build_opts* opts, double* best_seconds,
                        int32_t* trials);
/* Same for hsdl_build_batched: times batched builds of sample_graphs graphs
 * (0 = 256) spread evenly over the input.  max_wave is then the hub cap of a
 * batched wave. */
int hsdl_build_batched_autotune(int32_t num_graphs, const int32_t* n, const int64_t* const* row_ptr,
                                const int32_t* const* col, const int32_t* const* w, const int32_t* K,
                                int32_t sample_graphs, hsdl_build_opts* opts, double* best_seconds,
                                int32_t* trials);

/* ------------------------------------------------------------------------
 * Canonical repair.  Replaces hop_constrained_clean_L
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:422)
 * and gpu_clean (Clean_mdnd/src/gpu_clean.cu:180,
 * Hybrid_Generation_Clean/src/label_clean.cu:244).  Keeps label (u,h,d) of v
 * iff no pair of labels through a hub ranked at or above u reaches v from u
 * within h hops at distance <= d (the reference's rule, generation.h:451-482).
 * ---------------------------------------------------------------------- */
int hsdl_clean(hsdl_index* idx);

/* ------------------------------------------------------------------------
 * Queries.  Replace hop_constrained_extract_distance
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:144) and gpu_query
 * (Query_mdnd/src/gpu_query.cu:84).  out[i] = min over common hubs of
 * d1 + d2 with h1 + h2 <= k[i], INT32_MAX if no pair exists; checked first,
 * as in the reference: k < 0 -> INT32_MAX, then s == t -> 0, then
 * k == 0 -> INT32_MAX.
 * ---------------------------------------------------------------------- */
int hsdl_query_batch(hsdl_index* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                     int32_t* out);
/* Same on device arrays, asynchronous on `stream`. */
int hsdl_query_batch_device(hsdl_index* idx, int64_t nq, const int32_t* d_s, const int32_t* d_t,
                            const int32_t* d_k, int32_t* d_out, void* stream);

/* Same as hsdl_query_batch, but allocates no device memory: the queries and
 * answers are staged in one fixed-size device array inside the library
 * instead of per-call allocations.  For callers that cannot allocate device
 * memory - next to running serving or build kernels (cudaMalloc/cudaFree can
 * synchronise the device), or under another allocator's hard cap.  This entry
 * point has no counterpart in the reference.  At most HSDL_STATIC_QUERY_MAX
 * queries per call (larger batches: HSDL_ERR_INVALID); a batch naming a vertex
 * outside the index is HSDL_ERR_INVALID after the call, as in
 * hsdl_query_batch.  The array (16 MiB) is placed on a device when the
 * library's module is loaded there - at the set-up, since modules load lazily
 * - and held until exit.  Set-up, once per device with the device current:
 * hsdl_query_static_prepare, or else the first hsdl_query_batch_static call;
 * it looks up the array's address and loads every query kernel variant, and a
 * module load may synchronise the device, so run it before a serving loop
 * starts or any stream capture begins.  Calls share the array and are
 * serialised by a process-wide lock that is held until the call's work on the
 * stream has finished, on error paths too (overlapping calls would race). */
#define HSDL_STATIC_QUERY_MAX (1 << 20)
int hsdl_query_batch_static(hsdl_index* idx, int64_t nq, const int32_t* s, const int32_t* t, const int32_t* k,
                            int32_t* out);
/* The set-up of hsdl_query_batch_static on the current device (idempotent). */
int hsdl_query_static_prepare(void);

/* Launch parameters of the query kernel for one index (the autotuner's
 * knobs): threads per block (multiple of 32, 32..1024), how many queries
 * ahead each warp prefetches rows into L2 (0..8), and lanes per query (8, 16
 * or 32: a warp answers 32/lanes queries at once). */
typedef struct hsdl_query_tuning {
  int32_t struct_size;
  int32_t block_threads;
  int32_t prefetch_ahead;
  int32_t lanes_per_query;
} hsdl_query_tuning;
int hsdl_set_query_tuning(hsdl_index* idx, const hsdl_query_tuning* tuning);
int hsdl_get_query_tuning(hsdl_index* idx, hsdl_query_tuning* tuning);

/* Path extraction: hop_constrained_extract_shortest_path
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels.h:224).  Writes
 * edges as (a,b) pairs into edges[2*cap]; *n_edges = count. */
int hsdl_extract_path(hsdl_index* idx, int32_t s, int32_t t, int32_t k, int32_t* edges, int32_t cap,
                      int32_t* n_edges);

/* ------------------------------------------------------------------------
 * Index contents.
 * ---------------------------------------------------------------------- */
typedef struct hsdl_index_info {
  int32_t n;
  int32_t K;
  int32_t cleaned;               /* 1 after hsdl_clean */
  int32_t waves;                 /* waves the generation ran */
  int64_t labels;                /* current label count */
  int64_t labels_before_clean;   /* label_size_before_canonical_repair */
  int64_t labels_after_clean;    /* label_size_after_canonical_repair */
  int64_t device_bytes;          /* HBM held by the index */
  double time_generate_s;        /* time_generate_labels */
  double time_sort_s;            /* time_sortL */
  double time_clean_s;           /* time_canonical_repair */
  int64_t max_row;               /* longest label list */
  /* work counted on the device during the build */
  int64_t work_relaxations;      /* edges relaxed by the searches */
  int64_t work_join_reads;       /* committed labels read by the pruning joins */
  int64_t work_labels_written;   /* labels generated (before clean) */
  int64_t work_clean_reads;      /* labels read by the clean's joins */
  int64_t work_candidates;       /* (hub, vertex) candidates the pruning joins decided */
  int64_t work_join_visible;     /* committed labels in the rows of those candidates (what a join without
                                    early exit reads; the joins stop at a dominating label) */
  /* device memory of the build */
  int64_t build_peak_bytes;      /* most HBM the build's buffers held at once */
  int64_t build_pool_entries;    /* label-pool entries the generation's rows occupied (labels and row slack) */
  int64_t build_max_candidates;  /* longest candidate list of one wave */
  int32_t build_wave_splits;     /* waves split in two because their candidates outgrew the memory left */
  int32_t build_pool_chunks;     /* device allocations the label pool grew by */
  int32_t query_key_bytes;       /* bytes per label the query joins stream: 4 when the index's ranges fit the
                                    compact key hub:H | hop:P | distance:D (H = bits of n, P = bits of K,
                                    D = 32 - H - P), else 8 */
  int32_t query_key_hub_bits;    /* H of the compact key (0 with 8-byte keys) */
  int32_t build_pool_key_bytes;  /* bytes per label key in the generation's label pool (4 or 8) */
  int32_t reserved;
} hsdl_index_info;

int hsdl_index_get_info(hsdl_index* idx, hsdl_index_info* info);
/* offsets[n+1], labels[offsets[n]]: each vertex's labels sorted by
 * (hub, hop, distance), the reference's sortL order
 * (CPU_HopHL/include/HBPLL/hop_constrained_two_hop_labels_generation.h:373-419). */
int hsdl_export(hsdl_index* idx, int64_t* offsets, hsdl_label* labels);
/* Builds an index from host labels (each row sorted as above; equal labels
 * may repeat, as in the reference's 2023WWW output before its clean, and the
 * clean drops the repeats). */
int hsdl_import(int32_t n, int32_t K, const int64_t* offsets, const hsdl_label* labels, hsdl_index** out);
/* Binary label file of Clean_pc/main.cu:11-58 (save_labels / load_labels):
 * size_t V; per vertex size_t count, then count x {hub, parent, hop, dist}. */
int hsdl_save_labels(hsdl_index* idx, const char* path);
int hsdl_load_labels(const char* path, int32_t K, hsdl_index** out);
int hsdl_index_destroy(hsdl_index* idx);

/* ------------------------------------------------------------------------
 * Serving loop (no counterpart in the reference, which answers queries one
 * at a time: two_hop_labels.h:144, Query_mdnd/src/gpu_query.cu:84).  A
 * persistent kernel answers (graph, s, t, k) requests published into a ring
 * in pinned host memory, batching across all resident indexes as requests
 * arrive; index builds run concurrently and are admitted by estimated label
 * bytes under a budget.  Answers are bit-identical to hsdl_query_batch on
 * the same index.
 * ---------------------------------------------------------------------- */
typedef struct hsdl_server hsdl_server;

typedef struct hsdl_serve_opts {
  int32_t struct_size;  /* sizeof(hsdl_serve_opts) */
  int32_t ctas;         /* blocks of the persistent kernel (0 = 6 per SM; at most what fits at once) */
  int32_t ring_log2;    /* request/answer ring capacity = 2^ring_log2 */
  int32_t max_indexes;  /* graph slots */
  int64_t budget_bytes; /* admission budget for resident + pending label bytes */
  double idle_exit_s;   /* the loop returns after this long without requests */
  int32_t lanes_per_query; /* 8, 16 or 32 lanes answer one request (default 32) */
  int32_t reserved;
} hsdl_serve_opts;

typedef struct hsdl_loadgen_opts {
  int32_t struct_size; /* sizeof(hsdl_loadgen_opts) */
  int32_t consumers;   /* host threads reading answers (0 = 4, at most 8) */
  int64_t n;           /* requests */
  const int32_t* g;    /* graph id, source, target, hop bound per request */
  const int32_t* s;
  const int32_t* t;
  const int32_t* k;
  int32_t* answers;    /* optional: answers, in request order */
  double offered_qps;  /* Poisson arrival rate; 0 = as fast as the ring allows */
  uint64_t seed;
} hsdl_loadgen_opts;

typedef struct hsdl_loadgen_result {
  int64_t completed;
  double seconds;      /* first scheduled arrival to last answer */
  double achieved_qps;
  double offered_qps;
  double p50_us, p90_us, p99_us, p999_us, max_us; /* arrival -> answer seen */
  double ready_frac;   /* answers already present when the host first looked */
  double mean_batch;   /* hsdl_query_loadgen: mean requests per hsdl_query_batch call */
} hsdl_loadgen_result;

/* The plain path under the same Poisson stream (hsdl_query_loadgen). */
typedef struct hsdl_query_loadgen_opts {
  int32_t struct_size; /* sizeof(hsdl_query_loadgen_opts) */
  int32_t max_batch;   /* most requests per call (0 = no limit; 1 = one call per request) */
  int64_t n;           /* requests (all on the one index) */
  const int32_t* s;    /* source, target, hop bound per request (pinned host memory for a fair rate) */
  const int32_t* t;
  const int32_t* k;
  int32_t* answers;    /* answers, in request order */
  double offered_qps;  /* Poisson arrival rate (the serving loadgen's stream for the same seed) */
  uint64_t seed;
  double window_us;    /* a batch leaves once its oldest request has waited this long and the GPU is free */
} hsdl_query_loadgen_opts;

typedef struct hsdl_serve_counters {
  int64_t submitted, processed, bad_requests;
  int64_t resident_graphs, pending_builds, resident_bytes, builds_done;
  int32_t loop_running;
  int32_t reserved;
} hsdl_serve_counters;

void hsdl_serve_opts_default(hsdl_serve_opts* opts);
int hsdl_serve_create(const hsdl_serve_opts* opts, hsdl_server** out);
/* Registers a built index (the caller keeps it alive) as a graph slot. */
int hsdl_serve_add_index(hsdl_server* srv, hsdl_index* idx, int32_t* graph_id);
/* Queues a build of g (kept alive by the caller until the build completes);
 * HSDL_ERR_FULL if its estimated label bytes do not fit the budget. */
int hsdl_serve_submit_build(hsdl_server* srv, hsdl_graph* g, int32_t K, int32_t* graph_id);
/* state: 0 free, 1 building, 2 resident, 3 failed; bytes: resident or estimated */
int hsdl_serve_graph_state(hsdl_server* srv, int32_t graph_id, int32_t* state, int64_t* bytes);
int hsdl_serve_wait_graph(hsdl_server* srv, int32_t graph_id, double timeout_s);
int hsdl_serve_remove_graph(hsdl_server* srv, int32_t graph_id);
/* Publishes n requests (g[i], s[i], t[i], k[i]); tickets are consecutive. */
int hsdl_serve_submit(hsdl_server* srv, int64_t n, const int32_t* g, const int32_t* s, const int32_t* t,
                      const int32_t* k, int64_t* first_ticket);
/* Reads the answers of the oldest unread tickets [first_ticket, +n). */
int hsdl_serve_wait(hsdl_server* srv, int64_t first_ticket, int64_t n, int32_t* answers, double timeout_s);
int hsdl_serve_loadgen(hsdl_server* srv, const hsdl_loadgen_opts* opts, hsdl_loadgen_result* result);
/* Open-loop load on the plain path: the same Poisson arrivals answered in
 * batches by hsdl_query_batch, one call at a time; latency from scheduled
 * arrival to the return of the answering call.  No counterpart in the
 * reference (its gpu_query answers one query per three launches,
 * Query_mdnd/src/gpu_query.cu:139-155). */
int hsdl_query_loadgen(hsdl_index* idx, const hsdl_query_loadgen_opts* opts, hsdl_loadgen_result* result);
int hsdl_serve_stats(hsdl_server* srv, hsdl_serve_counters* stats);
int hsdl_serve_destroy(hsdl_server* srv);

#ifdef __cplusplus
}
#endif

#endif /* HSDL_H */
