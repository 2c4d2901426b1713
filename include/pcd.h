/*
 * libpcd — GB300-native (sm_103a) Par-CD refine / merge / score path.
 *
 * C ABI: plain pointers and sizes; no CUDA or C++ types in the signatures.
 * Every entry point returns a pcd_status and never exits the process (the
 * reference's CUDA_CHECK calls exit(); src/cuda-common.cuh:96-106).
 *
 * Threading and ordering: one host thread per pcd_ctx.  A context owns one
 * CUDA stream (or borrows the caller's, pcd_set_stream); every call is ordered
 * on it.  Calls that return host-visible results (pcd_compress's num_labels,
 * pcd_score, pcd_labels_get, pcd_stats_get, pcd_triangles, pcd_contract)
 * synchronise that stream; pcd_refine and pcd_merge are asynchronous and
 * capturable.
 *
 * Labels are int32.  NEW_LABEL (-1, the reference's ~0 in src/common.hpp:20)
 * marks a vertex that a propagation sweep moved to a fresh singleton
 * community; pcd_compress renumbers such labels exactly as compress_labels
 * does (src/framework.cpp:146-170).
 */
#ifndef PCD_H
#define PCD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCD_NEW_LABEL (-1)

typedef enum pcd_status {
    PCD_OK = 0,
    PCD_ERR_INVALID_ARGUMENT = 1, /* null pointer, size out of range, unknown rule */
    PCD_ERR_CUDA = 2,             /* a CUDA runtime call failed; see pcd_last_error */
    PCD_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed */
    PCD_ERR_FORMAT = 4,           /* graph arrays are not a valid "PCD" CSR */
    PCD_ERR_DEVICE_TIMEOUT = 5,   /* a bounded device-side wait gave up */
    PCD_ERR_NOT_READY = 6,        /* call order violated (e.g. WCC before labels) */
    PCD_ERR_UNSUPPORTED = 7
} pcd_status;

typedef enum pcd_rule_kind {
    PCD_RULE_MODULARITY = 0, /* ModularityRule  src/rules.cpp:9-56   */
    PCD_RULE_CPM = 1,        /* CPMRule         src/rules.cpp:121-148 */
    PCD_RULE_WCC = 2         /* WCCRule         src/rules.cpp:150-436 */
} pcd_rule_kind;

/* Replaces the reference's Rule / CudaRule objects (src/rules.hpp:9-19,
 * src/rules-cuda.cuh:23-30): which objective, plus CPM's resolution. */
typedef struct pcd_rule {
    int32_t kind;  /* pcd_rule_kind */
    double lambda; /* CPM resolution; ignored otherwise */
} pcd_rule;

typedef struct pcd_ctx pcd_ctx;
typedef struct pcd_graph pcd_graph;

/* Counters of the last pcd_refine / pcd_merge on a graph (host-visible after
 * the next synchronising call, or pcd_synchronize). */
typedef struct pcd_sweep_info {
    int64_t draws;         /* rand_r calls the sweep consumed */
    int32_t fallback;      /* vertices re-evaluated in FP64 (the exact integer key could not order them) */
    int32_t resolved;      /* vertices / communities whose tie list was replayed */
    int32_t kernels;       /* kernel launches issued by the call */
    int32_t merge_pairs;   /* contracted (a, b) pairs (merge only) */
    int64_t kernels_total; /* kernel launches issued by every call on this graph so far */
} pcd_sweep_info;

const char *pcd_status_string(pcd_status s);
/* Last detailed error message of a context (never NULL). */
const char *pcd_last_error(const pcd_ctx *ctx);

/* cuda_init (src/framework-cuda.cu:59-73, declared src/framework-cuda.cuh:14).
 * Selects `device`, creates the context's stream, uploads constant tables,
 * and lets the device's default memory pool keep up to a quarter of the
 * device's memory after frees (graphs are allocated stream-ordered from it;
 * kept memory makes the next load cheap; trim the pool to return it). */
pcd_status pcd_init(pcd_ctx **ctx, int32_t device);
/* cuda_deinit (src/framework-cuda.cu:75-78).  Frees every graph of the ctx. */
pcd_status pcd_destroy(pcd_ctx *ctx);
/* Order all later work on a caller-owned cudaStream_t (passed as void*);
 * NULL restores the context's own stream. */
pcd_status pcd_set_stream(pcd_ctx *ctx, void *cuda_stream);
pcd_status pcd_synchronize(pcd_ctx *ctx);
/* No counterpart in the reference (its sweep is one kernel sequence).  on = 1:
 * the degree classes of a refine sweep run concurrently on side streams
 * forked from the context's stream and joined before the sweep continues
 * (they read only the old labels and write disjoint outputs, so results are
 * the same); on = 0 (default): one after another on the context's stream. */
pcd_status pcd_set_class_streams(pcd_ctx *ctx, int32_t on);

/* cuda_transfer_graph (src/framework-cuda.cu:89-133) with Graph::read's
 * semantics (src/graph.cpp:40-105): n vertices, m undirected edges,
 * indices[n+1], adj[2m] in HOST memory; rows sorted, no loops, symmetric.
 * The arrays are copied; the caller keeps ownership.  Validates offsets,
 * ranges, sortedness and loops (PCD_ERR_FORMAT). */
pcd_status pcd_load_csr(pcd_ctx *ctx, int32_t n, int32_t m, const int32_t *indices,
                        const int32_t *adj, pcd_graph **out);
/* Same, from DEVICE pointers already resident on the context's device. */
pcd_status pcd_load_csr_device(pcd_ctx *ctx, int32_t n, int32_t m, const int32_t *d_indices,
                               const int32_t *d_adj, pcd_graph **out);
pcd_status pcd_graph_free(pcd_graph *g);

/* No counterpart in the reference (its GPU path sorts all edges at once).
 * Degree classes of the sweep kernels: vertices of degree <= max_deg[i] (and
 * above max_deg[i-1]) run in class i: 0..3 one thread per vertex with the row
 * in registers (up to 4/8/16/32 neighbours), 4 a warp per vertex, 5 a
 * 256-thread block, 6 a 512- or 1024-thread block (shared-memory tables sized
 * to each degree sub-range), and everything above max_deg[6] the hub kernel
 * (1024-thread blocks, labels split into hash parts).  Bounds must be
 * non-decreasing and at most {4, 8, 16, 32, 256, 2048, 8192} (the kernels'
 * capacities).  Results do not depend on the classes; the autotuner
 * (par-cd_gb300/tune.py) and the tests move them. */
pcd_status pcd_graph_set_bins(pcd_graph *g, const int32_t max_deg[7]);
pcd_status pcd_graph_get_bins(pcd_graph *g, int32_t max_deg[7], int64_t counts[8]);
/* No counterpart in the reference.  Size of a hash part of the hub kernel:
 * a hub row's entries whose neighbour is not alone in its community are split
 * into ceil(entries / labels) parts by label hash, each histogrammed in the
 * 16384-slot shared table (default 6144, range [1024, 8192]: a part's labels
 * must fit half of the table).  Results do not depend on it; the autotuner
 * moves it. */
pcd_status pcd_graph_set_hub_part(pcd_graph *g, int32_t labels);

/* Device memory a graph or batch holds right now (every buffer libpcd
 * allocated for it, merge buffers and seed tables included).  No counterpart
 * in the reference (its device buffers come from one global allocator,
 * framework-cuda.cu:14). */
pcd_status pcd_graph_device_bytes(pcd_graph *g, int64_t *bytes);

/* Upper bound of the device memory that loading and running a graph (or a
 * packed batch of num_graphs graphs with n vertices and nnz adjacency entries
 * in all) needs at its peak, from sizes known before loading: the largest
 * degree, the number of vertices above 8192 neighbours, the iteration cap of
 * pcd_batch_run (n_iter, or 1000 in threshold mode), whether merges run, and
 * the device's SM count.  Used for HBM admission in the serving loop. */
pcd_status pcd_estimate_device_bytes(int32_t n, int64_t nnz, int32_t max_deg, int64_t num_hubs, int32_t num_graphs,
                                     int32_t iteration_cap, int32_t merges, int32_t num_sms, int64_t *bytes);

/* SM count of the context's device. */
pcd_status pcd_device_sm_count(pcd_ctx *ctx, int32_t *sms);

/* cuda_labels_to_device / cuda_labels_from_device
 * (src/framework-cuda.cu:135-143).  Host arrays of n labels. */
pcd_status pcd_labels_set(pcd_graph *g, const int32_t *labels);
pcd_status pcd_labels_get(pcd_graph *g, int32_t *labels);
/* Device-pointer variants (n int32 on the context's device). */
pcd_status pcd_labels_set_device(pcd_graph *g, const int32_t *d_labels);
pcd_status pcd_labels_get_device(pcd_graph *g, int32_t *d_labels);

/* compress_labels + collect_statistics (src/framework.cpp:146-170, 69-143;
 * cuda_collect_statistics src/framework-cuda.cu:235-323): renumber labels by
 * first occurrence and collect per-community size, internal and external
 * volume.  num_labels may be NULL (then the call does not synchronise). */
pcd_status pcd_compress(pcd_graph *g, int32_t *num_labels);
/* Statistics of the current compressed partition (host arrays of capacity
 * >= num_labels; any may be NULL). */
pcd_status pcd_stats_get(pcd_graph *g, int32_t *sizes, int32_t *int_volume, int32_t *ext_volume);

/* Graph::count_triangles (src/graph.cpp:107-175): tri[v] (twice the
 * triangles through v), tri_deg[v] (edges of v in a triangle) and the mean
 * local clustering coefficient.  Any output may be NULL.  WCC needs this; the
 * first WCC call computes it if it has not been. */
pcd_status pcd_triangles(pcd_graph *g, int32_t *tri, int32_t *tri_deg, double *clustering_coef);

/* Rule::calculate (src/rules.cpp:9-22, 121-129, 150-235;
 * cuda_calculate_metric src/framework-cuda.cu:164-172) of the current
 * partition, reduced in FP64.  Compresses first if the labels changed. */
pcd_status pcd_score(pcd_graph *g, const pcd_rule *rule, double *out);

/* One synchronous label-propagation sweep: PropagationRefinement::refine
 * (src/refinement.cpp:114-182; cuda_propagation_step
 * src/framework-cuda.cu:465-633).  `seed` is the rand_r state the reference
 * draws with rand() at the start of the call; ties and the frac test replay
 * the same rand_r stream, so labels are bit-exact with the reference's -p 1
 * schedule.  Compresses first if needed.  Writes the new labels (NEW_LABEL
 * allowed) to the graph; asynchronous. */
pcd_status pcd_refine(pcd_graph *g, const pcd_rule *rule, double frac, uint32_t seed);

/* Mutual-best community merging: MergingRefinement::refine
 * (src/refinement.cpp:185-288; cuda_merging_step
 * src/framework-cuda.cu:744-892), built as a sort by (a, b) community pair
 * plus segmented reduce (the contracted edge weights), then `rounds` rounds of
 * best-partner selection and matching.  Asynchronous. */
pcd_status pcd_merge(pcd_graph *g, const pcd_rule *rule, int32_t rounds, uint32_t seed);

/* Contracted edge weights of the current compressed partition: every ordered
 * pair (a, b), a != b, of communities joined by w > 0 edges, sorted by
 * (a, b).  Writes min(cap, pairs) triples and the pair count. */
pcd_status pcd_contract(pcd_graph *g, int64_t cap, int32_t *a, int32_t *b, int32_t *w,
                        int64_t *num_pairs);

pcd_status pcd_sweep_info_get(pcd_graph *g, pcd_sweep_info *info);

/* Per-phase device timing (the reference's CudaTimer spans,
 * src/cuda-common.cuh:253-316): while enabled, pcd_refine / pcd_merge /
 * pcd_compress / pcd_load_csr record CUDA events between their kernel groups
 * on the context's stream.  pcd_profile_read synchronises and writes up to `cap`
 * (phase name, milliseconds) pairs of the most recent call; returns the number
 * of phases (or -1 on error).  Names are static strings. */
pcd_status pcd_profile_enable(pcd_ctx *ctx, int32_t on);
int32_t pcd_profile_read(pcd_ctx *ctx, const char **names, double *ms, int32_t cap);

/* ------------------------------------------------------------------------
 * Batched path (no counterpart in the reference, which handles one graph per
 * process).  A batch is many graphs loaded as one packed CSR: graph g owns
 * vertices [vertex_offsets[g], vertex_offsets[g+1]) (every graph at least one
 * vertex); indices[N+1] are row offsets into the packed adjacency
 * (N = vertex_offsets[G]); adj holds each graph's LOCAL neighbour ids.  The
 * returned handle is a pcd_graph; per-graph results use local labels.  Every
 * graph gets exactly the labels and scores it gets alone through the
 * single-graph calls with the same seeds.
 * ------------------------------------------------------------------------ */
pcd_status pcd_batch_load(pcd_ctx *ctx, int32_t num_graphs, const int32_t *vertex_offsets,
                          const int32_t *indices, const int32_t *adj, pcd_graph **out);
/* Same with indices / adj in device memory (vertex_offsets on the host). */
pcd_status pcd_batch_load_device(pcd_ctx *ctx, int32_t num_graphs, const int32_t *vertex_offsets,
                                 const int32_t *d_indices, const int32_t *d_adj, pcd_graph **out);
pcd_status pcd_batch_num_graphs(pcd_graph *batch, int32_t *num_graphs);
/* Host arrays of N labels, each graph's labels local to it ([-1, n_g)). */
pcd_status pcd_batch_labels_set(pcd_graph *batch, const int32_t *labels);
pcd_status pcd_batch_labels_get(pcd_graph *batch, int32_t *labels);
/* Per-graph community counts / scores (host arrays of num_graphs). */
pcd_status pcd_batch_compress(pcd_graph *batch, int32_t *per_graph_k);
pcd_status pcd_batch_score(pcd_graph *batch, const pcd_rule *rule, double *per_graph);
/* One sweep / one merge of every graph, with per-graph rand_r seeds. */
pcd_status pcd_batch_refine(pcd_graph *batch, const pcd_rule *rule, double frac, const uint32_t *seeds);
pcd_status pcd_batch_merge(pcd_graph *batch, const pcd_rule *rule, int32_t rounds, const uint32_t *seeds);
/* The reference driver loop (src/main.cpp:199-266, singleton start, -s
 * strategy, -f frac, -r rounds, -n n_iter or -t threshold when n_iter == -1)
 * for every graph at once, each graph with its own glibc seed stream and stop
 * test.  With use_cuda_graph, each propagation iteration of the whole batch is
 * one captured CUDA graph replay.  Threshold mode stops a graph after 1000
 * iterations at the latest (the reference's loop never ends for a graph whose
 * score stays <= 0).  Writes each graph's final score and iteration count
 * (host arrays, may be NULL). */
pcd_status pcd_batch_run(pcd_graph *batch, const pcd_rule *rule, int32_t strategy, double frac,
                         int32_t rounds, int32_t n_iter, double threshold, int32_t use_cuda_graph,
                         double *scores, int32_t *iterations);

/* Edge list -> graph, on the device, with the semantics of the reference
 * converter (src/convert.cpp:76-196): loops dropped, both directions,
 * duplicates removed, vertices renumbered by (degree, id) descending, rows
 * sorted, vertices without neighbours dropped.  src/dst: num_edges host int32
 * ids >= 0; num_nodes = -1 takes the largest id + 1 (src/convert.cpp:61).
 * map (host, may be NULL, room for num_nodes or the largest id + 1): the
 * original id of each new vertex.  The result is loaded as a graph;
 * pcd_graph_size / pcd_graph_csr_get read it back (e.g. to write a "PCD"
 * file).  Replaces the reference's host converter for large inputs. */
pcd_status pcd_convert_edges(pcd_ctx *ctx, int64_t num_edges, const int32_t *src, const int32_t *dst,
                             int32_t num_nodes, int32_t *map, pcd_graph **out);
pcd_status pcd_graph_size(pcd_graph *g, int32_t *n, int32_t *m);
/* Host arrays of n + 1 and 2m int32. */
pcd_status pcd_graph_csr_get(pcd_graph *g, int32_t *indices, int32_t *adj);

/* ------------------------------------------------------------------------
 * Serving loop.  No counterpart in the reference (its drivers run one graph
 * per process, src/main.cpp).  Requests -- a graph and a driver schedule --
 * queue in arrival order; `workers` threads, each with its own context and
 * stream, take batches of requests that share a schedule (at most
 * max_batch_graphs graphs and max_batch_edges adjacency entries) and run them
 * with pcd_batch_run, so batches of different workers overlap on the GPU.  A
 * batch is admitted only while the device memory of every batch in flight,
 * counted with pcd_estimate_device_bytes, stays within hbm_budget_bytes; a
 * request that alone exceeds the budget fails with PCD_ERR_OUT_OF_MEMORY.  A
 * batch smaller than max_batch_graphs starts once its oldest request has
 * waited max_wait_ms.  A batch holds one size class (small / medium / large
 * by adjacency entries; a large graph runs alone), and at most workers - 1
 * batches of medium or large graphs run at once, so small requests always
 * have a worker.  Every graph gets exactly its result alone.
 * ------------------------------------------------------------------------ */
typedef struct pcd_server pcd_server;
typedef struct pcd_schedule {
    pcd_rule rule;      /* Modularity or CPM (WCC needs the clustering start) */
    int32_t strategy;   /* -s: 0 propagation, 1 merging, 2 alternate          */
    double frac;        /* -f                                                 */
    int32_t rounds;     /* -r                                                 */
    int32_t n_iter;     /* -n, or -1: stop on -t threshold                    */
    double threshold;   /* -t                                                 */
} pcd_schedule;
typedef struct pcd_serve_config {
    int32_t device;
    int32_t workers;
    int32_t max_batch_graphs;
    int64_t max_batch_edges;
    int64_t hbm_budget_bytes;
    double max_wait_ms;
    int32_t use_cuda_graph;     /* passed to pcd_batch_run */
    int64_t small_graph_edges;  /* size classes by adjacency entries: small <= this,   */
    int64_t large_graph_edges;  /* medium <= this, large above (one graph per batch)   */
    int32_t continuous;         /* 1: a batch runs iteration by iteration; a graph whose
                                 * schedule ends returns at that iteration and leaves,
                                 * queued requests of the same schedule and size class
                                 * join between iterations as slots and memory free up
                                 * (for -s 2 at even iterations, so that all graphs of a
                                 * batch sweep alike).  0: each batch runs to its end
                                 * through pcd_batch_run (CUDA-graph iterations). */
} pcd_serve_config;
typedef struct pcd_serve_stats {
    int64_t submitted, completed, failed, batches, batched_graphs, queue_len;
    int64_t bytes_in_flight;     /* estimated bytes of the batches running now */
    int64_t bytes_peak;          /* largest estimated total in flight so far   */
    int64_t bytes_measured_peak; /* largest pcd_graph_device_bytes of a batch  */
    int64_t estimate_exceeded;   /* batches that held more than their estimate */
    int64_t admitted_running;    /* requests that joined a batch already running */
    int64_t released_early;      /* requests returned while their batch ran on   */
} pcd_serve_stats;
typedef struct pcd_serve_timing {
    double queue_ms;        /* submit -> its batch started */
    double latency_ms;      /* submit -> result ready      */
    int64_t batch_graphs;   /* graphs in its batch          */
} pcd_serve_timing;
pcd_status pcd_serve_start(const pcd_serve_config *cfg, pcd_server **out);
/* Copies the graph (host CSR, checked here) and queues it; returns at once. */
pcd_status pcd_serve_submit(pcd_server *s, int32_t n, int32_t m, const int32_t *indices, const int32_t *adj,
                            const pcd_schedule *sched, uint64_t *ticket);
pcd_status pcd_serve_poll(pcd_server *s, uint64_t ticket, int32_t *done);
/* Blocks until the request is done and releases its ticket; labels: n host
 * int32 (may be NULL); returns the request's own status. */
pcd_status pcd_serve_wait(pcd_server *s, uint64_t ticket, int32_t *labels, double *score, int32_t *iterations,
                          pcd_serve_timing *timing);
pcd_status pcd_serve_stats_get(pcd_server *s, pcd_serve_stats *out);
/* Runs what is queued, stops the workers, frees the server (no call may use
 * it afterwards, including pending waits). */
pcd_status pcd_serve_stop(pcd_server *s);

/* compress_labels on caller-owned device buffers, with no device allocation.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc where they relabel (inside another framework's memory arena,
 * allocation-free serving loops, hosts that reserve all device memory up
 * front).  d_labels_in / d_labels_out: n int32 on the current device, distinct
 * buffers; labels in [-1, n), -1 = NEW_LABEL (out-of-range values get a fresh
 * id like NEW_LABEL); *d_num_labels (device) receives the community count.
 * Scratch is a fixed file-scope device array sized for PCD_NOALLOC_MAX_LABELS
 * labels (about 8 MiB per GPU, held until the process exits); larger n is
 * rejected with PCD_ERR_INVALID_ARGUMENT.  The first call on a device, with
 * that device current, looks up the array's address (again after a
 * cudaDeviceReset); make that first call before any stream capture.  Calls
 * share the array: calls that overlap on the GPU race.  A CUDA error already
 * pending on the calling thread is left pending and returned as PCD_ERR_CUDA
 * with nothing launched.  Asynchronous on `cuda_stream` (NULL = legacy
 * default stream). */
#define PCD_NOALLOC_MAX_LABELS (1 << 20)
pcd_status pcd_compress_labels_noalloc(const int32_t *d_labels_in, int32_t n, int32_t *d_labels_out,
                                       int32_t *d_num_labels, void *cuda_stream);

/* Host-side seed stream: glibc rand() restated (default seed 1 = never
 * srand'ed), so a driver can hand pcd_refine / pcd_merge the same seed the
 * reference draws at src/refinement.cpp:123-124 and :217-218.  Replaces the
 * reference's use of the process-wide libc generator. */
typedef struct pcd_rand {
    uint32_t r[34];
    int32_t pos;
} pcd_rand;
void pcd_rand_seed(pcd_rand *s, uint32_t seed);   /* srand(seed) */
int32_t pcd_rand_next(pcd_rand *s);               /* rand()      */
void pcd_rand_skip(pcd_rand *s, int64_t count);   /* count x rand() */

/* Initial partitions, computed on the host as the reference does:
 * create_singleton_partition (src/framework.cpp:14-24) draws n values from s;
 * create_clustering_partition (src/framework.cpp:27-59) needs tri[] from
 * pcd_triangles.  Host arrays. */
pcd_status pcd_singleton_partition(pcd_rand *s, int32_t n, int32_t *labels);
pcd_status pcd_clustering_partition(int32_t n, const int32_t *indices, const int32_t *adj,
                                    const int32_t *tri, int32_t *labels);

/* create_clustering_partition (src/framework.cpp:27-59) on the device: the
 * graph's labels become the same partition as pcd_clustering_partition
 * (vertices by decreasing tri / (deg (deg - 1)), the product in 32-bit int,
 * then decreasing degree, then id; each unlabelled vertex opens a community
 * and claims its unlabelled neighbours).  Computes the triangles if they are
 * not yet known.  Labels are 0..k-1 in the order the communities open;
 * *num_labels (may be NULL) receives k.  Synchronises. */
pcd_status pcd_clustering_partition_device(pcd_graph *g, int32_t *num_labels);

/* FindConnectedRefinement::refine (src/refinement.cpp:291-322): the graph's
 * labels become, for every vertex, the smallest vertex id in its connected
 * component (the fixed point the reference's min-label rounds reach); the
 * current labels are not read.  Asynchronous unless num_components is
 * non-NULL, which receives the number of components and synchronises. */
pcd_status pcd_find_connected(pcd_graph *g, int32_t *num_components);

/* norm_mutual_info (src/common.cpp:75-125) of the confusion counts of count
 * label pairs (a[i], b[i]), normalised by n vertices: compare_communities(g,
 * a, b) (src/common.cpp:163-173) is count = n = g.n; the ground-truth file
 * form (src/common.cpp:127-160) passes one (community line, label) pair per
 * listed vertex and n = g.n.  Labels must be >= 0.  FP64; the sums run in a
 * fixed order that differs from the reference's map walk, so the value
 * agrees to rounding.  pcd_nmi_device takes device arrays, pcd_nmi host
 * arrays.  Synchronise. */
pcd_status pcd_nmi_device(pcd_ctx *ctx, int64_t count, const int32_t *a, const int32_t *b, int32_t n,
                          double *nmi);
pcd_status pcd_nmi(pcd_ctx *ctx, int64_t count, const int32_t *a, const int32_t *b, int32_t n, double *nmi);

#ifdef __cplusplus
}
#endif
#endif /* PCD_H */
