// Host-side state of libpcd and the launchers each translation unit exports.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pcd.h"
#include "pcd_types.h"

struct pcd_ctx {
    int32_t device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;  // own_stream or the caller's
    int32_t num_sms = 0;
    size_t smem_optin = 0;
    std::string last_error;
    std::vector<pcd_graph *> graphs;
    // profiling: spans (name, start event, end event), each on one stream;
    // a span starts where the previous mark on the same stream ended
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_pool;
    size_t prof_used = 0;
    struct ProfSpan {
        const char *name;
        int32_t ev0, ev1;
    };
    std::vector<ProfSpan> prof_spans;
    std::vector<std::pair<cudaStream_t, int32_t>> prof_last;  // stream -> its last event
    // side streams on which the sweep's degree classes run concurrently
    // (created on first use with the priority of `stream`), and the
    // fork/join events between them and `stream`
    static constexpr int kSide = 3;
    bool class_streams = false;  // pcd_set_class_streams
    cudaStream_t side[kSide] = {nullptr, nullptr, nullptr};
    int32_t side_prio = 0;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kSide] = {nullptr, nullptr, nullptr};
    // a graph load copies the neighbour array in up to kCopyChunks pieces and
    // records one of these after each, so its rows are checked as they arrive
    static constexpr int kCopyChunks = 8;
    cudaEvent_t ev_copy[kCopyChunks] = {};
    pcd::DevCounters *h_ctr = nullptr;  // pinned copy of a graph's counters (shared by its graphs)
    // multiplies the resident-block caps of the sweep grids: above 1 the warp,
    // block and thread classes launch more blocks than fit at once, so blocks
    // retire (and free SMs for other streams' work) throughout the kernel
    int32_t grid_scale = 1;
};

// Per-graph state of a batch: many graphs refined as one disjoint union whose
// vertices (and, after compress, communities) are grouped graph by graph.
struct BatchState {
    int32_t G = 0;
    std::vector<int32_t> h_voff;   // vertex offsets (G + 1)
    std::vector<int32_t> h_m;      // edges per graph
    int32_t *voff = nullptr;       // device copy of h_voff
    int32_t *vgid = nullptr;       // graph of each vertex
    int32_t *cgid = nullptr;       // graph of each community (after compress)
    int32_t *gK = nullptr;         // first community of each graph, gK[G] = k (after compress)
    int32_t *gm = nullptr;         // edges per graph
    double *gcc = nullptr;         // clustering coefficient per graph (WCC)
    uint32_t *gseed = nullptr;     // rand_r seed of each graph for the current call
    uint32_t *gbase = nullptr;     // each graph's offset in the scanned draw stream
    uint32_t *gtotal = nullptr;    // merge: draws of earlier rounds, per graph
    int32_t *gdone = nullptr;      // graph finished its schedule (labels frozen)
    double *gscore = nullptr, *gprev = nullptr;
    double *tile_part = nullptr;   // per-tile partial sums of the score (2 doubles each)
    int64_t tile_cap = 0;
    int32_t *gtile = nullptr;      // first score tile of each graph (G + 1)
    int32_t *iter = nullptr;       // device iteration counter (captured runs)
    uint32_t *seed_table = nullptr;  // [iters][G] seeds for captured runs
    int32_t seed_iters = 0;
};

struct pcd_graph {
    pcd_ctx *ctx = nullptr;
    BatchState *batch = nullptr;   // non-null for a batch (see pcd_batch_* in pcd.h)
    int32_t n = 0, m = 0;
    int64_t nnz = 0;  // 2m
    int32_t max_deg = 0;

    // CSR (device)
    int32_t *indices = nullptr, *adj = nullptr;
    // partition state (device, capacity n)
    int32_t *labels = nullptr;      // current labels
    int32_t *labels_alt = nullptr;  // sweep output / compress scratch
    int32_t *first = nullptr;       // compress: first vertex of each old label
    int32_t *sizes = nullptr, *intv = nullptr, *extv = nullptr, *vol = nullptr;
    // sweep scratch
    uint32_t *ndraw = nullptr;        // per vertex: rand_r calls; then draw offsets
    uint32_t *tile_sums = nullptr;    // scan scratch
    uint32_t *scan_total = nullptr;   // scan result (1 word)
    pcd::ScanScratch scan{};          // tile_sums + scan_total + overflow flag
    int32_t scan_overflow = 0;        // host: a scan did not fit its scratch
    int32_t *tiebuf = nullptr;
    int64_t tiebuf_cap = 0;
    pcd::TieRecord *recs = nullptr;   // capacity max(n, k)
    int32_t *nties = nullptr;         // per vertex: final-level ties of the last sweep
    int32_t *amb = nullptr;           // ambiguous vertex list, capacity n
    pcd::DevCounters *ctr = nullptr;  // device counters
    void *small = nullptr;            // 64 KiB of reduction scratch
    double *d_score = nullptr;        // device result of pcd_score
    pcd::DevCounters *h_ctr = nullptr;  // pinned mirror
    // FP64 re-evaluation: per block an HBM table of fb_slots entries (kept
    // empty between vertices) and a position array of max_deg entries
    int32_t *fb_scratch = nullptr;
    int64_t fb_slots = 0;    // power of two >= 2 * max_deg
    int32_t fb_blocks = 0;
    // hub kernel: one slice per hub block (hub_stride(max_deg) ints: packed
    // keys, labels and (position, label) buckets of the row being refined)
    int32_t *hub_scratch = nullptr;
    int32_t hub_blocks = 0;
    int32_t hub_part_labels = 6144;  // distinct labels per hash part (pcd_graph_set_hub_part)
    size_t hub_bytes = 0;
    size_t dev_bytes = 0;             // device memory held through dev_alloc and the hub slices
    // degree bins
    int32_t *bin_list = nullptr;          // vertices grouped by bin
    int64_t bin_off[pcd::NBINS + 1] = {0};
    int32_t bin_maxdeg[pcd::NBINS] = {0};  // largest degree in each class
    // degree sub-ranges inside the classes (each launched with tables sized to
    // its own largest degree); a class's sub-ranges tile its part of bin_list
    struct SubRange {
        int32_t bin, lo, hi;  // degrees in (lo, hi]
        int64_t off, cnt;
        int32_t maxdeg;
    };
    std::vector<SubRange> subs;
    pcd::BinConfig bins{};
    // triangles (WCC)
    int32_t *tri = nullptr, *tri_deg = nullptr;
    double cc = 0.0;
    bool have_tri = false;
    // merge scratch (grown on demand)
    void *merge_buf = nullptr;
    size_t merge_bytes = 0;
    // bookkeeping
    int32_t k = 0;           // communities (valid when compressed)
    bool compressed = false; // labels renumbered and statistics current
    bool labels_vertex_space = false;  // batch: labels still hold vertex ids (set, not compressed)
    pcd_sweep_info info{};
    std::vector<void *> allocs;
};

namespace pcd {

// api.cu
pcd_status set_error(pcd_ctx *ctx, pcd_status s, const std::string &msg);
pcd_status check_cuda(pcd_ctx *ctx, cudaError_t e, const char *what);
pcd_status dev_alloc(pcd_graph *g, void **p, size_t bytes);

// partition.cu
int launch_compress(pcd_graph *g, cudaStream_t st);   // relabel + stats; k to ctr->k
int launch_stats(pcd_graph *g, cudaStream_t st, bool after_compress = false);
int launch_score(pcd_graph *g, int32_t kind, double lambda, double *d_out, cudaStream_t st);
// CSR checks: offsets (flag bits 1, 2) and the largest degree (d_flag[1]) from
// `indices` alone; then the rows (bit 4), over offsets that passed
int launch_check_offsets(const int32_t *indices, int32_t n, int32_t m, int32_t *d_flag, cudaStream_t st);
// by degree class (needs the bins): the rows whose last neighbour lies in
// (lo, hi] of the neighbour array (rows ending at 0 with lo < 0)
int launch_validate_rows(pcd_graph *g, int32_t *d_flag, int64_t lo, int64_t hi, cudaStream_t st);
// fills bin_list, bin_off, subs (syncs); active_only (batches): vertices of
// graphs whose schedule has finished are left out of every class
int launch_bins(pcd_graph *g, cudaStream_t st, bool active_only = false);
// Stable LSD radix sort of (uint64 key, uint32 value) pairs on bits [0, bits),
// 8 bits per pass, ping-ponging between A and B; true if the result is in B.
// hist: 256 * grid words; sc: scratch for scans of 256 * grid items.
bool radix_sort(unsigned long long *ka, uint32_t *va, unsigned long long *kb, uint32_t *vb, int64_t n, int bits,
                uint32_t *hist, const pcd::ScanScratch &sc, int grid, cudaStream_t st, int *launches);
// hub kernel: shared table slots, distinct labels per part, per-block slice in int32 units
constexpr int32_t HUB_TABLE_CAP = 16384;  // 192 KiB of table: one 1024-thread block per SM
constexpr int32_t HUB_PART_LABELS = 6144;
constexpr int32_t HUB_MAX_PARTS = 1024;   // rows above HUB_MAX_PARTS * HUB_PART_LABELS labels fill parts faster
// per position: an 8-byte key, a 4-byte label and an 8-byte (position, label) bucket entry
inline int64_t hub_stride(int64_t max_deg) { return (5 * std::max<int64_t>(max_deg, 1) + 3) & ~1ll; }

// propagate.cu
int launch_refine(pcd_graph *g, int32_t kind, double lambda, double frac, uint32_t seed,
                  cudaStream_t st);
void launch_resolve(const TieRecord *recs, const DevCounters *ctr, const uint32_t *endpos, const uint32_t *base,
                    const int32_t *tiebuf, int32_t *out, uint32_t seed, int32_t mod_base, int grid,
                    cudaStream_t st, const int32_t *ugid = nullptr, const uint32_t *gseed = nullptr,
                    const uint32_t *gbase = nullptr, const uint32_t *gextra = nullptr);
void launch_graph_base(const int32_t *first_unit, int32_t G, const uint32_t *endpos, uint32_t *gbase,
                       cudaStream_t st);

// merge.cu
pcd_status run_merge(pcd_graph *g, int32_t kind, double lambda, int32_t rounds, uint32_t seed,
                     cudaStream_t st, int *launches);
pcd_status run_contract(pcd_graph *g, int64_t cap, int32_t *a, int32_t *b, int32_t *w,
                        int64_t *num_pairs, cudaStream_t st);

// triangles.cu
int launch_triangles(pcd_graph *g, cudaStream_t st);
int launch_wcc_score(pcd_graph *g, double *d_out, cudaStream_t st);

}  // namespace pcd

// api.cu helpers shared with batch.cu
pcd_status scan_guard(pcd_graph *g);
pcd_status sync_and_check(pcd_graph *g);
pcd_status ensure_compressed(pcd_graph *g, int *launches);
pcd_status ensure_triangles(pcd_graph *g);
pcd_status check_rule(pcd_graph *g, const pcd_rule *r);

namespace pcd {

// jump table upload (propagate.cu)
void upload_jump_table(cudaStream_t st);

// profiling marks (api.cu): prof_begin clears the span list and records the
// start on `st`; prof_mark closes the phase `name` on stream st (the span
// runs from the previous mark on st); prof_fork starts stream `side` at the
// current point of `from`.  No-ops unless enabled.
void prof_begin(pcd_ctx *ctx, cudaStream_t st);
void prof_mark(pcd_ctx *ctx, const char *name, cudaStream_t st);
void prof_fork(pcd_ctx *ctx, cudaStream_t side);

// side streams (api.cu): fork `k` side streams off ctx->stream (they wait for
// everything issued on it so far) and return them; join makes ctx->stream
// wait for everything issued on them.  Capture-safe (events only).
pcd_status side_fork(pcd_ctx *ctx, int k, cudaStream_t *out);
void side_join(pcd_ctx *ctx, int k);

}  // namespace pcd
