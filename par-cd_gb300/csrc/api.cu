// The C ABI of libpcd (include/pcd.h): contexts, graphs, and the phase
// entry points that replace the reference's GPU host API
// (src/framework-cuda.cuh:14-23) and its CPU phase functions.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "pcd_internal.h"

using namespace pcd;

namespace pcd {

pcd_status set_error(pcd_ctx *ctx, pcd_status s, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

pcd_status check_cuda(pcd_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PCD_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_error(ctx, e == cudaErrorMemoryAllocation ? PCD_ERR_OUT_OF_MEMORY : PCD_ERR_CUDA, m);
}

pcd_status dev_alloc(pcd_graph *g, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    // stream-ordered: no device-wide synchronisation, so contexts on other
    // streams (the serving workers) keep running while graphs come and go
    cudaError_t e = cudaMallocAsync(p, bytes, g->ctx->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        return check_cuda(g->ctx, e, "cudaMallocAsync");
    }
    g->allocs.push_back(*p);
    g->dev_bytes += bytes;
    return PCD_OK;
}

// one more event of the pool recorded on st; returns its index (-1 on failure)
static int32_t prof_record(pcd_ctx *ctx, cudaStream_t st) {
    if (ctx->prof_used == ctx->prof_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        ctx->prof_pool.push_back(e);
    }
    cudaEventRecord(ctx->prof_pool[ctx->prof_used], st);
    return (int32_t)ctx->prof_used++;
}

static int32_t &prof_last_of(pcd_ctx *ctx, cudaStream_t st) {
    for (auto &p : ctx->prof_last)
        if (p.first == st) return p.second;
    ctx->prof_last.emplace_back(st, -1);
    return ctx->prof_last.back().second;
}

void prof_begin(pcd_ctx *ctx, cudaStream_t st) {
    if (!ctx->prof_on) return;
    ctx->prof_used = 0;
    ctx->prof_spans.clear();
    ctx->prof_last.clear();
    prof_last_of(ctx, st) = prof_record(ctx, st);
}

void prof_mark(pcd_ctx *ctx, const char *name, cudaStream_t st) {
    if (!ctx->prof_on || ctx->prof_used == 0) return;
    int32_t &last = prof_last_of(ctx, st);
    const int32_t e = prof_record(ctx, st);
    if (last >= 0 && e >= 0) ctx->prof_spans.push_back({name, last, e});
    last = e;
}

void prof_fork(pcd_ctx *ctx, cudaStream_t side) {
    if (!ctx->prof_on || ctx->prof_used == 0) return;
    prof_last_of(ctx, side) = prof_record(ctx, side);
}

pcd_status side_fork(pcd_ctx *ctx, int k, cudaStream_t *out) {
    if (k > pcd_ctx::kSide) k = pcd_ctx::kSide;
    int prio = 0;
    if (cudaStreamGetPriority(ctx->stream, &prio) != cudaSuccess) prio = 0;
    if (!ctx->ev_fork) {
        if (cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess)
            return check_cuda(ctx, cudaGetLastError(), "side streams");
        for (auto &e : ctx->ev_join)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                return check_cuda(ctx, cudaGetLastError(), "side streams");
    }
    if (!ctx->side[0] || prio != ctx->side_prio) {
        for (auto &s : ctx->side) {
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
            s = nullptr;
        }
        for (auto &s : ctx->side)
            if (cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio) != cudaSuccess)
                return check_cuda(ctx, cudaGetLastError(), "side streams");
        ctx->side_prio = prio;
    }
    cudaEventRecord(ctx->ev_fork, ctx->stream);
    for (int i = 0; i < k; ++i) {
        cudaStreamWaitEvent(ctx->side[i], ctx->ev_fork, 0);
        prof_fork(ctx, ctx->side[i]);
        out[i] = ctx->side[i];
    }
    return PCD_OK;
}

void side_join(pcd_ctx *ctx, int k) {
    if (k > pcd_ctx::kSide) k = pcd_ctx::kSide;
    for (int i = 0; i < k; ++i) {
        cudaEventRecord(ctx->ev_join[i], ctx->side[i]);
        cudaStreamWaitEvent(ctx->stream, ctx->ev_join[i], 0);
    }
}

}  // namespace pcd

#define CK(call, what)                                          \
    do {                                                        \
        pcd_status _s = check_cuda(ctx, (call), what);          \
        if (_s != PCD_OK) return _s;                            \
    } while (0)

#define TRY(expr)                          \
    do {                                   \
        pcd_status _s = (expr);            \
        if (_s != PCD_OK) return _s;       \
    } while (0)

pcd_status scan_guard(pcd_graph *g) {
    if (!g->scan_overflow) return PCD_OK;
    g->scan_overflow = 0;
    return set_error(g->ctx, PCD_ERR_CUDA, "internal: a device scan exceeded its scratch (nothing was launched)");
}

pcd_status sync_and_check(pcd_graph *g) {
    pcd_ctx *ctx = g->ctx;
    TRY(scan_guard(g));
    CK(cudaMemcpyAsync(g->h_ctr, g->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, ctx->stream),
       "counters");
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    int32_t err = g->h_ctr->error;
    if (err) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "device error flags 0x%x (1 tie buffer, 2 wait limit, 4 scratch, 8 label range, 16 check 0x%x)",
                 (unsigned)err, (unsigned)g->h_ctr->check_where);
        cudaMemsetAsync(&g->ctr->error, 0, sizeof(int32_t), ctx->stream);
        cudaMemsetAsync(&g->ctr->check_where, 0, sizeof(int32_t), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        pcd_status s = (err & ERR_WAIT_TIMEOUT) ? PCD_ERR_DEVICE_TIMEOUT
                       : (err & ERR_LABEL_RANGE) ? PCD_ERR_INVALID_ARGUMENT
                                                 : PCD_ERR_CUDA;
        return set_error(ctx, s, buf);
    }
    g->info.draws = g->h_ctr->total_draws;
    g->info.fallback = g->h_ctr->n_ambiguous + g->h_ctr->n_amb_large;
    g->info.resolved = g->h_ctr->n_resolve;
    g->info.merge_pairs = g->h_ctr->n_pairs;
    return PCD_OK;
}

pcd_status ensure_compressed(pcd_graph *g, int *launches) {
    if (g->compressed) return PCD_OK;
    if (g->n > 0) *launches += launch_compress(g, g->ctx->stream);
    g->compressed = true;
    return check_cuda(g->ctx, cudaGetLastError(), "compress launch");
}

pcd_status ensure_triangles(pcd_graph *g) {
    if (g->have_tri) return PCD_OK;
    pcd_ctx *ctx = g->ctx;
    const size_t nn = (size_t)std::max(g->n, 1);
    if (!g->tri) {
        TRY(dev_alloc(g, (void **)&g->tri, sizeof(int32_t) * nn));
        TRY(dev_alloc(g, (void **)&g->tri_deg, sizeof(int32_t) * nn));
    }
    double cc = 0.0;
    if (g->n > 0) {
        launch_triangles(g, ctx->stream);
        if (!g->batch)
            CK(cudaMemcpyAsync(&cc, g->d_score, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "triangles");
    }
    CK(cudaStreamSynchronize(ctx->stream), "triangles");
    g->cc = cc;
    g->have_tri = true;
    return PCD_OK;
}

pcd_status check_rule(pcd_graph *g, const pcd_rule *r) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    if (!r || r->kind < 0 || r->kind > 2) return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "unknown rule");
    return PCD_OK;
}

namespace pcd {
// Lets the device's default memory pool keep up to `bytes` of freed memory
// mapped, so that graphs loaded one after another reuse it instead of mapping
// and releasing device memory each time (used by the serving loop).
pcd_status keep_pool_memory(int32_t device, int64_t bytes) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return PCD_ERR_CUDA;
    uint64_t thr = (uint64_t)std::max<int64_t>(bytes, 0);
    return cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr) == cudaSuccess ? PCD_OK
                                                                                                : PCD_ERR_CUDA;
}
}  // namespace pcd

extern "C" {

const char *pcd_status_string(pcd_status s) {
    switch (s) {
        case PCD_OK: return "ok";
        case PCD_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PCD_ERR_CUDA: return "CUDA error";
        case PCD_ERR_OUT_OF_MEMORY: return "out of device memory";
        case PCD_ERR_FORMAT: return "invalid graph format";
        case PCD_ERR_DEVICE_TIMEOUT: return "device wait limit reached";
        case PCD_ERR_NOT_READY: return "call order violated";
        case PCD_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char *pcd_last_error(const pcd_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

pcd_status pcd_init(pcd_ctx **out, int32_t device) {
    if (!out) return PCD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pcd_ctx *ctx = new (std::nothrow) pcd_ctx;
    if (!ctx) return PCD_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    pcd_status s = check_cuda(ctx, cudaSetDevice(device), "cudaSetDevice");
    if (s == PCD_OK) s = check_cuda(ctx, cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking),
                                    "cudaStreamCreate");
    if (s == PCD_OK)
        s = check_cuda(ctx, cudaMallocHost((void **)&ctx->h_ctr, sizeof(DevCounters)), "cudaMallocHost");
    if (s == PCD_OK) {
        ctx->stream = ctx->own_stream;
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        ctx->num_sms = sms > 0 ? sms : 1;
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
        ctx->smem_optin = (size_t)optin;
        upload_jump_table(ctx->stream);
        // graphs are loaded and freed stream-ordered: let the device's default
        // pool keep up to a quarter of the device's memory after frees, so the
        // next graph reuses mapped memory instead of mapping it again
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
            cudaMemPool_t pool;
            uint64_t cur = 0;
            if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess &&
                cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur) == cudaSuccess &&
                cur < total_b / 4)
                keep_pool_memory(device, (int64_t)(total_b / 4));
        }
        cudaGetLastError();
        s = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "pcd_init");
    }
    if (s != PCD_OK) {
        // keep the context so the caller can read the message, but mark it unusable
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        ctx->own_stream = ctx->stream = nullptr;
        *out = ctx;
        return s;
    }
    *out = ctx;
    return PCD_OK;
}

pcd_status pcd_graph_free(pcd_graph *g) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaStream_t fs = ctx ? ctx->stream : nullptr;
    for (void *p : g->allocs)
        if (p) cudaFreeAsync(p, fs);
    if (g->hub_scratch) cudaFreeAsync(g->hub_scratch, fs);
    if (g->merge_buf) cudaFreeAsync(g->merge_buf, fs);
    if (g->batch && g->batch->seed_table) cudaFreeAsync(g->batch->seed_table, fs);
    delete g->batch;
    if (ctx) ctx->graphs.erase(std::remove(ctx->graphs.begin(), ctx->graphs.end(), g), ctx->graphs.end());
    delete g;
    return PCD_OK;
}

pcd_status pcd_destroy(pcd_ctx *ctx) {
    if (!ctx) return PCD_ERR_INVALID_ARGUMENT;
    while (!ctx->graphs.empty()) pcd_graph_free(ctx->graphs.back());
    for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
    for (auto &sd : ctx->side)
        if (sd) {
            cudaStreamSynchronize(sd);
            cudaStreamDestroy(sd);
        }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    for (auto &e : ctx->ev_join)
        if (e) cudaEventDestroy(e);
    for (auto &e : ctx->ev_copy)
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->own_stream);
        cudaStreamDestroy(ctx->own_stream);
    }
    if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
    delete ctx;
    return PCD_OK;
}

pcd_status pcd_set_stream(pcd_ctx *ctx, void *stream) {
    if (!ctx || !ctx->own_stream) return PCD_ERR_INVALID_ARGUMENT;
    CK(cudaStreamSynchronize(ctx->stream), "pcd_set_stream");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return PCD_OK;
}

pcd_status pcd_set_class_streams(pcd_ctx *ctx, int32_t on) {
    if (!ctx || !ctx->stream) return PCD_ERR_INVALID_ARGUMENT;
    ctx->class_streams = on != 0;
    return PCD_OK;
}

pcd_status pcd_profile_enable(pcd_ctx *ctx, int32_t on) {
    if (!ctx) return PCD_ERR_INVALID_ARGUMENT;
    ctx->prof_on = on != 0;
    ctx->prof_used = 0;
    return PCD_OK;
}

int32_t pcd_profile_read(pcd_ctx *ctx, const char **names, double *ms, int32_t cap) {
    if (!ctx || !ctx->stream) return -1;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return -1;
    const int32_t nph = (int32_t)ctx->prof_spans.size();
    for (int32_t i = 0; i < nph && i < cap; ++i) {
        const auto &sp = ctx->prof_spans[(size_t)i];
        float t = 0.f;
        cudaEventSynchronize(ctx->prof_pool[(size_t)sp.ev1]);
        cudaEventElapsedTime(&t, ctx->prof_pool[(size_t)sp.ev0], ctx->prof_pool[(size_t)sp.ev1]);
        if (names) names[i] = sp.name;
        if (ms) ms[i] = t;
    }
    return nph;
}

pcd_status pcd_synchronize(pcd_ctx *ctx) {
    if (!ctx || !ctx->stream) return PCD_ERR_INVALID_ARGUMENT;
    CK(cudaStreamSynchronize(ctx->stream), "pcd_synchronize");
    return PCD_OK;
}

// Hub slices: per block, a packed key and a label for every position of the
// largest row; as many blocks as there are hub vertices (at most one per SM);
// grown when the degree classes change.  No initial contents are needed.
static pcd_status ensure_hub_scratch(pcd_graph *g) {
    pcd_ctx *ctx = g->ctx;
    const int64_t hubs = g->bin_off[NBINS] - g->bin_off[BIN_HUB];
    const int32_t want = (int32_t)std::min<int64_t>(ctx->num_sms, hubs);
    if (want <= g->hub_blocks) return PCD_OK;
    const int64_t stride = hub_stride(g->max_deg);
    cudaStream_t st = ctx->stream;
    CK(cudaStreamSynchronize(st), "hub scratch");
    if (g->hub_scratch) {
        cudaFreeAsync(g->hub_scratch, st);
        g->dev_bytes -= g->hub_bytes;
    }
    g->hub_scratch = nullptr;
    g->hub_blocks = 0;
    g->hub_bytes = 0;
    const size_t bytes = sizeof(int32_t) * (size_t)(stride * want);
    CK(cudaMallocAsync((void **)&g->hub_scratch, bytes, st), "hub scratch");
    g->hub_blocks = want;
    g->hub_bytes = bytes;
    g->dev_bytes += bytes;
    return PCD_OK;
}

// Partition state and sweep scratch sized by n and 2m: allocated before the
// copies, so that the side stream of graph_setup may use them.
static pcd_status alloc_state(pcd_ctx *ctx, pcd_graph *g) {
    const int64_t n = g->n, nn = std::max<int64_t>(n, 1);
    TRY(dev_alloc(g, (void **)&g->labels, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->labels_alt, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->first, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->sizes, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->intv, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->extv, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->vol, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->ndraw, sizeof(uint32_t) * nn));
    // scans run over vertices, communities, edges (merge) and radix histograms
    const int64_t scan_items = std::max<int64_t>({n, g->nnz, 256ll * 2 * ctx->num_sms, 1});
    const int64_t tile_cap = (scan_items + 2047) / 2048 + 2;
    TRY(dev_alloc(g, (void **)&g->tile_sums, sizeof(uint32_t) * (size_t)tile_cap));
    TRY(dev_alloc(g, (void **)&g->scan_total, sizeof(uint32_t) * 4));
    g->scan = ScanScratch{g->tile_sums, tile_cap, g->scan_total, &g->scan_overflow};
    g->tiebuf_cap = g->nnz + n + 16;
    TRY(dev_alloc(g, (void **)&g->tiebuf, sizeof(int32_t) * (size_t)g->tiebuf_cap));
    TRY(dev_alloc(g, (void **)&g->recs, sizeof(TieRecord) * nn));
    TRY(dev_alloc(g, (void **)&g->nties, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->amb, sizeof(int32_t) * nn));
    TRY(dev_alloc(g, (void **)&g->ctr, sizeof(DevCounters)));
    TRY(dev_alloc(g, (void **)&g->small, 65536));
    TRY(dev_alloc(g, (void **)&g->d_score, 64));
    TRY(dev_alloc(g, (void **)&g->bin_list, sizeof(int32_t) * nn));
    g->h_ctr = ctx->h_ctr;  // pinned, one per context (calls on a context come from one thread)
    return PCD_OK;
}

// After the row offsets have arrived, while the neighbour array is still in
// flight on the context's stream in `nch` pieces ([cut[k], cut[k + 1]),
// piece k complete at ctx->ev_copy[k]): on `side`, the offsets, the largest
// degree, the degree classes, then the rows of each piece as it lands; on the
// context's stream, behind the copy, the counters and the FP64 re-evaluation
// tables.  `flag` holds two zeroed words.  The caller joins `side` back into
// the context's stream.
static pcd_status graph_setup(pcd_ctx *ctx, pcd_graph *g, int32_t *flag, cudaStream_t side, const int64_t *cut,
                              int nch) {
    const int64_t n = g->n;
    cudaStream_t st = ctx->stream;
    if (n > 0) launch_check_offsets(g->indices, g->n, g->m, flag, side);
    int32_t h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, flag, sizeof h, cudaMemcpyDeviceToHost, side), "validate");
    CK(cudaStreamSynchronize(side), "validate");
    if (h[0]) {
        char buf[128];
        snprintf(buf, sizeof buf, "graph arrays are not a valid CSR (flags 0x%x: 1 span, 2 offsets, 4 rows)", h[0]);
        return set_error(ctx, PCD_ERR_FORMAT, buf);
    }
    g->max_deg = h[1];
    g->bins = BinConfig{{4, 8, 16, 32, 256, 2048, 8192}};
    if (n > 0) launch_bins(g, side);
    prof_mark(ctx, "load.bins", side);
    CK(cudaGetLastError(), "degree classes");
    for (int k = 0; k < nch; ++k) {
        CK(cudaStreamWaitEvent(side, ctx->ev_copy[k], 0), "validate");
        if (n > 0) launch_validate_rows(g, flag, k ? cut[k] : -1, cut[k + 1], side);
    }
    // the context's stream, behind the copy
    CK(cudaMemsetAsync(g->ctr, 0, sizeof(DevCounters), st), "memset");
    // FP64 re-evaluation tables: one HBM slice per block, empty between uses
    // (keys -1, counts 0, first positions 0xffffffff; position arrays need no init)
    int64_t slots = 64;
    while (slots < 2 * (int64_t)std::max(g->max_deg, 1)) slots <<= 1;
    g->fb_slots = slots;
    const int64_t fb_stride = 3 * slots + g->max_deg;
    g->fb_blocks = (int32_t)std::min<int64_t>(8, std::max<int64_t>(1, (int64_t)(1ll << 29) / (4 * fb_stride)));
    TRY(dev_alloc(g, (void **)&g->fb_scratch, sizeof(int32_t) * (size_t)(fb_stride * g->fb_blocks)));
    for (int32_t bk = 0; bk < g->fb_blocks; ++bk) {
        int32_t *base = g->fb_scratch + (int64_t)bk * fb_stride;
        CK(cudaMemsetAsync(base, 0xff, sizeof(int32_t) * (size_t)slots, st), "fallback scratch");
        CK(cudaMemsetAsync(base + slots, 0, sizeof(int32_t) * (size_t)slots, st), "fallback scratch");
        CK(cudaMemsetAsync(base + 2 * slots, 0xff, sizeof(int32_t) * (size_t)slots, st), "fallback scratch");
    }
    prof_mark(ctx, "load.state", st);
    // the rows' verdict (a copy to pageable memory returns once it is done)
    prof_mark(ctx, "load.validate", side);
    CK(cudaMemcpyAsync(h, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, side), "validate");
    CK(cudaStreamSynchronize(side), "validate");
    if (h[0]) {
        char buf[128];
        snprintf(buf, sizeof buf, "graph arrays are not a valid CSR (flags 0x%x: 1 span, 2 offsets, 4 rows)", h[0]);
        return set_error(ctx, PCD_ERR_FORMAT, buf);
    }
    // the hub slices (the same tables plus labels and counts by position)
    TRY(ensure_hub_scratch(g));
    // initial labels: singletons 0..n-1 (already compressed)
    g->k = g->n;
    g->compressed = false;
    return PCD_OK;
}

__global__ void k_label_range(const int32_t *__restrict__ labels, int32_t n, int32_t *bad) {
    int32_t b = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = labels[i];
        b |= (l < -1) | (l >= n);
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

__global__ void k_iota(int32_t *p, int32_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

static pcd_status load_common(pcd_ctx *ctx, int32_t n, int32_t m, const int32_t *indices, const int32_t *adj,
                              cudaMemcpyKind kind, pcd_graph **out) {
    if (!ctx || !ctx->stream || !out) return PCD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (n < 0 || m < 0 || (int64_t)2 * m > INT32_MAX) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "n or m out of range");
    if (!indices || (m > 0 && !adj)) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "null CSR array");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    pcd_graph *g = new (std::nothrow) pcd_graph;
    if (!g) return PCD_ERR_OUT_OF_MEMORY;
    g->ctx = ctx;
    g->n = n;
    g->m = m;
    g->nnz = 2 * (int64_t)m;
    prof_begin(ctx, ctx->stream);
    cudaStream_t st = ctx->stream, side = nullptr;
    int32_t *flag = nullptr;
    pcd_status s = dev_alloc(g, (void **)&g->indices, sizeof(int32_t) * ((size_t)n + 1));
    if (s == PCD_OK) s = dev_alloc(g, (void **)&g->adj, sizeof(int32_t) * (size_t)std::max<int64_t>(g->nnz, 1));
    if (s == PCD_OK) s = dev_alloc(g, (void **)&flag, 2 * sizeof(int32_t));
    if (s == PCD_OK) s = alloc_state(ctx, g);
    if (s == PCD_OK) s = check_cuda(ctx, cudaMemsetAsync(flag, 0, 2 * sizeof(int32_t), st), "memset");
    if (s == PCD_OK)
        s = check_cuda(ctx, cudaMemcpyAsync(g->indices, indices, sizeof(int32_t) * ((size_t)n + 1), kind, st),
                       "copy indices");
    // the side stream starts behind the allocations and the row offsets
    if (s == PCD_OK) s = side_fork(ctx, 1, &side);
    const bool forked = s == PCD_OK;
    // the neighbour array in pieces of about 256 MB (16-byte boundaries), an
    // event after each
    int64_t cut[pcd_ctx::kCopyChunks + 1] = {0};
    const int nch = (int)std::min<int64_t>(pcd_ctx::kCopyChunks, std::max<int64_t>(1, (4 * g->nnz) >> 28));
    for (int k = 1; k < nch; ++k) cut[k] = (g->nnz * k / nch) & ~3ll;
    cut[nch] = g->nnz;
    for (int k = 0; k < nch && s == PCD_OK; ++k) {
        if (!ctx->ev_copy[k])
            s = check_cuda(ctx, cudaEventCreateWithFlags(&ctx->ev_copy[k], cudaEventDisableTiming), "copy events");
        if (s == PCD_OK && cut[k + 1] > cut[k])
            s = check_cuda(ctx,
                           cudaMemcpyAsync(g->adj + cut[k], adj + cut[k], sizeof(int32_t) * (size_t)(cut[k + 1] - cut[k]),
                                           kind, st),
                           "copy adj");
        if (s == PCD_OK) s = check_cuda(ctx, cudaEventRecord(ctx->ev_copy[k], st), "copy events");
    }
    if (s == PCD_OK) prof_mark(ctx, "load.copy", st);
    if (s == PCD_OK) s = graph_setup(ctx, g, flag, side, cut, nch);
    if (forked) side_join(ctx, 1);
    if (s == PCD_OK && n > 0) {
        k_iota<<<std::max(1, std::min<int>((n + 255) / 256, ctx->num_sms * 8)), 256, 0, ctx->stream>>>(g->labels, n);
        prof_mark(ctx, "load.labels", ctx->stream);
        s = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "init labels");
    }
    if (s != PCD_OK) {
        cudaStreamSynchronize(ctx->stream);
        for (void *p : g->allocs)
            if (p) cudaFreeAsync(p, ctx->stream);
        if (g->hub_scratch) cudaFreeAsync(g->hub_scratch, ctx->stream);
        delete g;
        return s;
    }
    ctx->graphs.push_back(g);
    *out = g;
    return PCD_OK;
}

pcd_status pcd_load_csr(pcd_ctx *ctx, int32_t n, int32_t m, const int32_t *indices, const int32_t *adj,
                        pcd_graph **out) {
    return load_common(ctx, n, m, indices, adj, cudaMemcpyHostToDevice, out);
}

pcd_status pcd_load_csr_device(pcd_ctx *ctx, int32_t n, int32_t m, const int32_t *d_indices, const int32_t *d_adj,
                               pcd_graph **out) {
    return load_common(ctx, n, m, d_indices, d_adj, cudaMemcpyDeviceToDevice, out);
}


pcd_status pcd_device_sm_count(pcd_ctx *ctx, int32_t *sms) {
    if (!ctx || !sms) return PCD_ERR_INVALID_ARGUMENT;
    *sms = ctx->num_sms;
    return PCD_OK;
}

pcd_status pcd_graph_device_bytes(pcd_graph *g, int64_t *bytes) {
    if (!g || !bytes) return PCD_ERR_INVALID_ARGUMENT;
    int64_t b = (int64_t)g->dev_bytes + (int64_t)g->merge_bytes;
    if (g->batch) b += 4ll * g->batch->seed_iters * g->batch->G;
    *bytes = b;
    return PCD_OK;
}

// Upper bound of what pcd_batch_load + pcd_batch_run (or pcd_load_csr and the
// phase calls, num_graphs = 1) hold on the device at their peak, from sizes
// the caller knows before loading.  Mirrors the allocations of graph_setup,
// ensure_hub_scratch, batch_setup, the batch staging copies, the seed table
// of pcd_batch_run (iteration cap) and the merge buffers.
pcd_status pcd_estimate_device_bytes(int32_t n, int64_t nnz, int32_t max_deg, int64_t num_hubs, int32_t num_graphs,
                                     int32_t iteration_cap, int32_t merges, int32_t num_sms, int64_t *bytes) {
    if (!bytes || n < 0 || nnz < 0 || max_deg < 0 || num_hubs < 0 || num_graphs < 1 || num_sms < 1)
        return PCD_ERR_INVALID_ARGUMENT;
    const int64_t nn = std::max<int64_t>(n, 1), e = std::max<int64_t>(nnz, 1), G = num_graphs;
    int64_t b = 4 * (nn + 1) + 4 * e;                                                  // CSR
    b += 60 * nn;                                                                      // per-vertex state
    b += 4 * ((std::max<int64_t>({nn, e, 512ll * num_sms}) + 2047) / 2048 + 2) + 16;  // scan tiles
    b += 4 * (e + nn + 16);                                                            // tie slots
    b += 8 * nn;                                                                       // triangles (WCC)
    b += 65536 + 64 + 64 + 256;                                                        // counters, reductions
    int64_t slots = 64;
    while (slots < 2 * (int64_t)std::max(max_deg, 1)) slots <<= 1;
    const int64_t fb_stride = 3 * slots + max_deg;
    b += 4 * fb_stride * std::min<int64_t>(8, std::max<int64_t>(1, (1ll << 29) / (4 * fb_stride)));
    b += 4 * hub_stride(max_deg) * std::min<int64_t>(num_sms, num_hubs);
    // batch state, the staging copies of a batch load, the seed table of a run
    b += 8 * nn + 8 * (G + 1) + 52 * G + 64;
    b += 4 * (nn + 1) + 4 * e + 8 + 4 * (G + 1) + 4 * nn;
    b += 4 * G * std::max(iteration_cap, 1) + 12 * G + 64;
    if (merges) b += 60 * e + 24 * nn + 4 + 1024ll * 2 * num_sms + 256 * 21;
    b += 40 * 512;  // allocation granularity
    *bytes = b;
    return PCD_OK;
}

pcd_status pcd_graph_set_bins(pcd_graph *g, const int32_t max_deg[7]) {
    if (!g || !max_deg) return PCD_ERR_INVALID_ARGUMENT;
    static const int32_t cap[7] = {4, 8, 16, 32, 256, 2048, 8192};
    for (int i = 0; i < 7; ++i) {
        if (max_deg[i] < 0 || max_deg[i] > cap[i] || (i && max_deg[i] < max_deg[i - 1]))
            return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "degree classes out of range");
    }
    pcd_ctx *ctx = g->ctx;
    CK(cudaStreamSynchronize(ctx->stream), "set_bins");
    for (int i = 0; i < 7; ++i) g->bins.max_deg[i] = max_deg[i];
    if (g->n > 0) launch_bins(g, ctx->stream);
    TRY(ensure_hub_scratch(g));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "set_bins");
}

pcd_status pcd_graph_set_hub_part(pcd_graph *g, int32_t labels) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    if (labels < 1024 || labels > HUB_TABLE_CAP / 2)
        return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "hub part size out of range [1024, 8192]");
    g->hub_part_labels = labels;
    return PCD_OK;
}

pcd_status pcd_graph_get_bins(pcd_graph *g, int32_t max_deg[7], int64_t counts[8]) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 7; ++i)
        if (max_deg) max_deg[i] = g->bins.max_deg[i];
    for (int i = 0; i < 8; ++i)
        if (counts) counts[i] = g->bin_off[i + 1] - g->bin_off[i];
    return PCD_OK;
}

pcd_status pcd_labels_set(pcd_graph *g, const int32_t *labels) {
    if (!g || (!labels && g->n)) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    CK(cudaMemcpyAsync(g->labels, labels, sizeof(int32_t) * (size_t)g->n, cudaMemcpyHostToDevice, ctx->stream),
       "labels_set");
    g->compressed = false;
    // range check on the device (NEW_LABEL = -1 allowed), reported here
    int32_t *bad = static_cast<int32_t *>(g->small);
    CK(cudaMemsetAsync(bad, 0, sizeof(int32_t), ctx->stream), "labels_set");
    if (g->n > 0)
        k_label_range<<<std::max(1, std::min<int>((g->n + 255) / 256, ctx->num_sms * 8)), 256, 0, ctx->stream>>>(
            g->labels, g->n, bad);
    int32_t h_bad = 0;
    CK(cudaMemcpyAsync(&h_bad, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream), "labels_set");
    CK(cudaStreamSynchronize(ctx->stream), "labels_set");
    if (h_bad) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "label out of range [-1, n)");
    return PCD_OK;
}

pcd_status pcd_labels_set_device(pcd_graph *g, const int32_t *d_labels) {
    if (!g || (!d_labels && g->n)) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    CK(cudaMemcpyAsync(g->labels, d_labels, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToDevice, ctx->stream),
       "labels_set_device");
    g->compressed = false;  // range checked on the device by the next compress
    return PCD_OK;
}

pcd_status pcd_labels_get(pcd_graph *g, int32_t *labels) {
    if (!g || (!labels && g->n)) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    CK(cudaMemcpyAsync(labels, g->labels, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, ctx->stream),
       "labels_get");
    return sync_and_check(g);
}

pcd_status pcd_labels_get_device(pcd_graph *g, int32_t *d_labels) {
    if (!g || (!d_labels && g->n)) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    CK(cudaMemcpyAsync(d_labels, g->labels, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToDevice, ctx->stream),
       "labels_get_device");
    return PCD_OK;
}


pcd_status pcd_compress(pcd_graph *g, int32_t *num_labels) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    int launches = 0;
    if (!g->compressed) prof_begin(g->ctx, g->ctx->stream);
    TRY(ensure_compressed(g, &launches));
    g->info.kernels_total += launches;
    if (num_labels) {
        TRY(sync_and_check(g));
        g->k = g->n > 0 ? g->h_ctr->k : 0;
        *num_labels = g->k;
    }
    return PCD_OK;
}

pcd_status pcd_stats_get(pcd_graph *g, int32_t *sizes, int32_t *int_volume, int32_t *ext_volume) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    int32_t k;
    TRY(pcd_compress(g, &k));
    pcd_ctx *ctx = g->ctx;
    size_t b = sizeof(int32_t) * (size_t)k;
    if (sizes) CK(cudaMemcpyAsync(sizes, g->sizes, b, cudaMemcpyDeviceToHost, ctx->stream), "stats");
    if (int_volume) CK(cudaMemcpyAsync(int_volume, g->intv, b, cudaMemcpyDeviceToHost, ctx->stream), "stats");
    if (ext_volume) CK(cudaMemcpyAsync(ext_volume, g->extv, b, cudaMemcpyDeviceToHost, ctx->stream), "stats");
    CK(cudaStreamSynchronize(ctx->stream), "stats");
    return PCD_OK;
}


pcd_status pcd_triangles(pcd_graph *g, int32_t *tri, int32_t *tri_deg, double *clustering_coef) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    TRY(ensure_triangles(g));
    pcd_ctx *ctx = g->ctx;
    size_t b = sizeof(int32_t) * (size_t)g->n;
    if (tri) CK(cudaMemcpyAsync(tri, g->tri, b, cudaMemcpyDeviceToHost, ctx->stream), "tri");
    if (tri_deg) CK(cudaMemcpyAsync(tri_deg, g->tri_deg, b, cudaMemcpyDeviceToHost, ctx->stream), "tri_deg");
    CK(cudaStreamSynchronize(ctx->stream), "tri");
    if (clustering_coef) *clustering_coef = g->cc;
    return PCD_OK;
}


pcd_status pcd_score(pcd_graph *g, const pcd_rule *rule, double *out) {
    TRY(check_rule(g, rule));
    if (!out) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    if (rule->kind == PCD_RULE_WCC) TRY(ensure_triangles(g));
    int launches = 0;
    TRY(ensure_compressed(g, &launches));
    if (g->n == 0) {
        *out = 0.0;
        return PCD_OK;
    }
    if (rule->kind == PCD_RULE_WCC)
        launch_wcc_score(g, g->d_score, ctx->stream);
    else
        launch_score(g, rule->kind, rule->lambda, g->d_score, ctx->stream);
    CK(cudaMemcpyAsync(out, g->d_score, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "score");
    return sync_and_check(g);
}

pcd_status pcd_refine(pcd_graph *g, const pcd_rule *rule, double frac, uint32_t seed) {
    TRY(check_rule(g, rule));
    if (!(frac > 0.0 && frac <= 1.0))
        return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "fraction should be in (0, 1]");
    if (rule->kind == PCD_RULE_WCC) TRY(ensure_triangles(g));
    int launches = 0;
    prof_begin(g->ctx, g->ctx->stream);
    TRY(ensure_compressed(g, &launches));
    if (g->n > 0) {
        launches += launch_refine(g, rule->kind, rule->lambda, frac, seed, g->ctx->stream);
        std::swap(g->labels, g->labels_alt);
    }
    g->compressed = false;
    g->info.kernels = launches;
    g->info.kernels_total += launches;
    TRY(scan_guard(g));
    return check_cuda(g->ctx, cudaGetLastError(), "refine launch");
}

pcd_status pcd_merge(pcd_graph *g, const pcd_rule *rule, int32_t rounds, uint32_t seed) {
    TRY(check_rule(g, rule));
    if (rounds <= 0) return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "number of rounds should be positive");
    if (rule->kind == PCD_RULE_WCC) TRY(ensure_triangles(g));
    int launches = 0;
    prof_begin(g->ctx, g->ctx->stream);
    TRY(ensure_compressed(g, &launches));
    if (g->n > 0) {
        TRY(run_merge(g, rule->kind, rule->lambda, rounds, seed, g->ctx->stream, &launches));
        std::swap(g->labels, g->labels_alt);
    }
    g->compressed = false;
    g->info.kernels = launches;
    g->info.kernels_total += launches;
    TRY(scan_guard(g));
    return check_cuda(g->ctx, cudaGetLastError(), "merge launch");
}

pcd_status pcd_contract(pcd_graph *g, int64_t cap, int32_t *a, int32_t *b, int32_t *w, int64_t *num_pairs) {
    if (!g || !num_pairs || cap < 0 || (cap > 0 && (!a || !b || !w))) return PCD_ERR_INVALID_ARGUMENT;
    int launches = 0;
    TRY(ensure_compressed(g, &launches));
    return run_contract(g, cap, a, b, w, num_pairs, g->ctx->stream);
}

pcd_status pcd_sweep_info_get(pcd_graph *g, pcd_sweep_info *info) {
    if (!g || !info) return PCD_ERR_INVALID_ARGUMENT;
    TRY(sync_and_check(g));
    *info = g->info;
    return PCD_OK;
}

}  // extern "C"
