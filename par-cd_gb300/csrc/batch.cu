// The batched path: many graphs of uneven size refined and merged together.
//
// A batch is the disjoint union of its graphs, stored as one packed CSR with a
// vertex-offset table: graph g owns vertices [voff[g], voff[g+1]) and, after
// every compress, communities [gK[g], gK[g+1]) (first-occurrence numbering
// over the union numbers each graph's communities consecutively, in the same
// order as compressing that graph alone).  The sweep, merge, statistics and
// score kernels of the single-graph path run once over the whole union; what
// differs per graph -- the edge count m in the gains, the rand_r seed and
// stream offset, the clustering coefficient, the stop test -- is looked up
// per vertex or community through small per-graph arrays.  So a graph's labels
// and scores are the same as when it runs alone, and a whole iteration of
// every graph is one fixed launch sequence, captured once in a CUDA graph and
// replayed (pcd_batch_run).
#include <algorithm>
#include <cstring>
#include <vector>

#include "pcd_internal.h"

using namespace pcd;

namespace pcd {

__global__ void k_fill_vgid(const int32_t *voff, int32_t G, int32_t *vgid) {
    for (int64_t g = blockIdx.x; g < G; g += gridDim.x)
        for (int32_t v = voff[g] + threadIdx.x; v < voff[g + 1]; v += blockDim.x) vgid[v] = (int32_t)g;
}

// local neighbour ids -> union ids; flags neighbours outside their graph
__global__ void k_globalize_adj(const int32_t *indices, const int32_t *vgid, const int32_t *voff, int32_t n,
                                int32_t *adj, int32_t *flag) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < n; v += nw) {
        const int32_t g = vgid[v], base = voff[g], ng = voff[g + 1] - base;
        for (int32_t j = indices[v] + lane; j < indices[v + 1]; j += 32) {
            const int32_t u = adj[j];
            if (u < 0 || u >= ng) atomicOr(flag, 1);
            adj[j] = u + base;
        }
    }
}

__global__ void k_labels_to_union(const int32_t *local, const int32_t *vgid, const int32_t *voff, int32_t n,
                                  int32_t *out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = local[v];
        out[v] = l < 0 ? -1 : l + voff[vgid[v]];
    }
}

// community space (after compress / refine / merge): subtract gK[g];
// vertex space (right after labels_set): subtract voff[g]
__global__ void k_labels_to_local(const int32_t *in, const int32_t *vgid, const int32_t *base, int32_t n,
                                  int32_t *local) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = in[v];
        local[v] = l < 0 ? -1 : l - base[vgid[v]];
    }
}

__global__ void k_iota_union(int32_t *labels, int32_t n) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        labels[v] = (int32_t)v;
}

// The reference driver's stop test per graph (src/main.cpp:241-242), run after
// each graph's score of iteration *it is in gscore.
// Threshold mode stops a graph after `cap` iterations at the latest (the
// reference would loop forever on a graph whose score never turns positive).
__global__ void k_batch_stop(int32_t G, const double *score, double *prev, int32_t *done, int32_t *iters,
                             double *final_score, const int32_t *it_ptr, int32_t n_iter, double threshold,
                             int32_t cap) {
    const int32_t it = *it_ptr;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
        if (done[g]) continue;
        const double s = score[g];
        const bool d = n_iter != -1 ? it >= n_iter
                                    : ((prev[g] > 0 && s > 0 && s / prev[g] - 1 <= threshold) || it >= cap - 1);
        final_score[g] = s;
        iters[g] = it;
        if (d) done[g] = 1;
        prev[g] = s;
    }
}

__global__ void k_batch_seeds(int32_t G, const uint32_t *table, int32_t cap, const int32_t *it_ptr, uint32_t *gseed) {
    const int32_t it = min(*it_ptr, cap - 1);
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x)
        gseed[g] = table[(int64_t)it * G + g];
}

__global__ void k_count_done(int32_t G, const int32_t *done, int32_t *out) {
    int32_t c = 0;
    for (int64_t g = threadIdx.x; g < G; g += blockDim.x) c += done[g] ? 1 : 0;
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, c);
}

__global__ void k_incr(int32_t *p) { *p += 1; }

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

static unsigned grid_of(int64_t n, int sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16));
}

static pcd_status batch_setup(pcd_ctx *ctx, pcd_graph *g, int32_t G, const int32_t *h_voff) {
    BatchState *B = new (std::nothrow) BatchState;
    if (!B) return PCD_ERR_OUT_OF_MEMORY;
    g->batch = B;
    B->G = G;
    B->h_voff.assign(h_voff, h_voff + G + 1);
    cudaStream_t st = ctx->stream;
    TRY(dev_alloc(g, (void **)&B->voff, sizeof(int32_t) * (G + 1)));
    TRY(dev_alloc(g, (void **)&B->vgid, sizeof(int32_t) * std::max(g->n, 1)));
    TRY(dev_alloc(g, (void **)&B->cgid, sizeof(int32_t) * std::max(g->n, 1)));
    TRY(dev_alloc(g, (void **)&B->gK, sizeof(int32_t) * (G + 1)));
    TRY(dev_alloc(g, (void **)&B->gm, sizeof(int32_t) * G));
    TRY(dev_alloc(g, (void **)&B->gcc, sizeof(double) * G));
    TRY(dev_alloc(g, (void **)&B->gseed, sizeof(uint32_t) * G));
    TRY(dev_alloc(g, (void **)&B->gbase, sizeof(uint32_t) * G));
    TRY(dev_alloc(g, (void **)&B->gtotal, sizeof(uint32_t) * G));
    TRY(dev_alloc(g, (void **)&B->gdone, sizeof(int32_t) * G));
    TRY(dev_alloc(g, (void **)&B->gscore, sizeof(double) * G));
    TRY(dev_alloc(g, (void **)&B->gprev, sizeof(double) * G));
    TRY(dev_alloc(g, (void **)&B->iter, sizeof(int32_t) * 4));
    CK(cudaMemcpyAsync(B->voff, h_voff, sizeof(int32_t) * (G + 1), cudaMemcpyHostToDevice, st), "voff");
    CK(cudaMemsetAsync(B->gdone, 0, sizeof(int32_t) * G, st), "batch");
    CK(cudaMemsetAsync(B->gcc, 0, sizeof(double) * G, st), "batch");
    k_fill_vgid<<<(unsigned)std::min<int32_t>(G, 65535), 256, 0, st>>>(B->voff, G, B->vgid);
    return check_cuda(ctx, cudaGetLastError(), "batch setup");
}

// Loads the packed CSR: indices[N+1] are union row offsets, adj holds each
// graph's LOCAL neighbour ids.  kind: copy direction of indices/adj.
static pcd_status batch_load(pcd_ctx *ctx, int32_t G, const int32_t *voff, const int32_t *indices,
                             const int32_t *adj, cudaMemcpyKind kind, pcd_graph **out) {
    if (!ctx || !ctx->stream || !out || G < 1 || !voff || !indices) return PCD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (voff[0] != 0) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "vertex offsets must start at 0");
    for (int32_t g = 0; g < G; ++g)
        if (voff[g + 1] <= voff[g]) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "every graph needs a vertex");
    const int32_t N = voff[G];
    // row offsets at each graph boundary give m_g
    std::vector<int32_t> rows((size_t)G + 1);
    for (int32_t g = 0; g <= G; ++g) {
        if (kind == cudaMemcpyHostToDevice) {
            rows[(size_t)g] = indices[voff[g]];
        } else {
            CK(cudaMemcpy(&rows[(size_t)g], indices + voff[g], sizeof(int32_t), cudaMemcpyDeviceToHost), "rows");
        }
    }
    const int64_t nnz = rows[(size_t)G];
    if (rows[0] != 0 || nnz % 2) return set_error(ctx, PCD_ERR_FORMAT, "row offsets do not form a CSR");
    std::vector<int32_t> hm((size_t)G);
    for (int32_t g = 0; g < G; ++g) {
        const int32_t e = rows[(size_t)g + 1] - rows[(size_t)g];
        if (e < 0 || e % 2) return set_error(ctx, PCD_ERR_FORMAT, "a graph has an odd number of adjacency entries");
        hm[(size_t)g] = e / 2;
    }
    // union ids on the device (temporary copies), then the single-graph loader
    int32_t *d_ind = nullptr, *d_adj = nullptr, *d_flag = nullptr, *d_voff = nullptr, *d_vgid = nullptr;
    cudaStream_t st = ctx->stream;
    auto cleanup = [&]() {
        for (int32_t *p : {d_ind, d_adj, d_flag, d_voff, d_vgid})
            if (p) cudaFreeAsync(p, st);
    };
    if (cudaMallocAsync(&d_ind, sizeof(int32_t) * ((size_t)N + 1), st) != cudaSuccess ||
        cudaMallocAsync(&d_adj, sizeof(int32_t) * std::max<int64_t>(nnz, 1), st) != cudaSuccess ||
        cudaMallocAsync(&d_flag, sizeof(int32_t), st) != cudaSuccess ||
        cudaMallocAsync(&d_voff, sizeof(int32_t) * ((size_t)G + 1), st) != cudaSuccess ||
        cudaMallocAsync(&d_vgid, sizeof(int32_t) * std::max(N, 1), st) != cudaSuccess) {
        cleanup();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "batch staging buffers");
    }
    cudaMemcpyAsync(d_ind, indices, sizeof(int32_t) * ((size_t)N + 1), kind, st);
    if (nnz) cudaMemcpyAsync(d_adj, adj, sizeof(int32_t) * nnz, kind, st);
    cudaMemcpyAsync(d_voff, voff, sizeof(int32_t) * ((size_t)G + 1), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_flag, 0, sizeof(int32_t), st);
    k_fill_vgid<<<(unsigned)std::min<int32_t>(G, 65535), 256, 0, st>>>(d_voff, G, d_vgid);
    k_globalize_adj<<<grid_of((int64_t)N * 32, ctx->num_sms), 256, 0, st>>>(d_ind, d_vgid, d_voff, N, d_adj, d_flag);
    int32_t flag = 0;
    cudaMemcpyAsync(&flag, d_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    pcd_status s = check_cuda(ctx, cudaStreamSynchronize(st), "batch staging");
    if (s == PCD_OK && flag) s = set_error(ctx, PCD_ERR_FORMAT, "a neighbour id lies outside its graph");
    pcd_graph *g = nullptr;
    if (s == PCD_OK) s = pcd_load_csr_device(ctx, N, (int32_t)(nnz / 2), d_ind, d_adj, &g);
    cleanup();
    if (s != PCD_OK) return s;
    s = batch_setup(ctx, g, G, voff);
    if (s == PCD_OK) {
        s = check_cuda(ctx, cudaMemcpyAsync(g->batch->gm, hm.data(), sizeof(int32_t) * G, cudaMemcpyHostToDevice, st),
                       "gm");
        g->batch->h_m = hm;
    }
    if (s == PCD_OK) s = check_cuda(ctx, cudaStreamSynchronize(st), "batch load");
    if (s != PCD_OK) {
        pcd_graph_free(g);
        return s;
    }
    *out = g;
    return PCD_OK;
}

extern "C" {

pcd_status pcd_batch_load(pcd_ctx *ctx, int32_t num_graphs, const int32_t *vertex_offsets, const int32_t *indices,
                          const int32_t *adj, pcd_graph **out) {
    return batch_load(ctx, num_graphs, vertex_offsets, indices, adj, cudaMemcpyHostToDevice, out);
}

pcd_status pcd_batch_load_device(pcd_ctx *ctx, int32_t num_graphs, const int32_t *vertex_offsets,
                                 const int32_t *d_indices, const int32_t *d_adj, pcd_graph **out) {
    return batch_load(ctx, num_graphs, vertex_offsets, d_indices, d_adj, cudaMemcpyDeviceToDevice, out);
}

pcd_status pcd_batch_num_graphs(pcd_graph *g, int32_t *num_graphs) {
    if (!g || !g->batch || !num_graphs) return PCD_ERR_INVALID_ARGUMENT;
    *num_graphs = g->batch->G;
    return PCD_OK;
}

pcd_status pcd_batch_labels_set(pcd_graph *g, const int32_t *labels) {
    if (!g || !g->batch || !labels) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    BatchState *B = g->batch;
    for (int32_t gi = 0; gi < B->G; ++gi) {
        const int32_t ng = B->h_voff[(size_t)gi + 1] - B->h_voff[(size_t)gi];
        for (int32_t v = B->h_voff[(size_t)gi]; v < B->h_voff[(size_t)gi + 1]; ++v)
            if (labels[v] < -1 || labels[v] >= ng)
                return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "label out of range [-1, n_g)");
    }
    CK(cudaMemcpyAsync(g->labels_alt, labels, sizeof(int32_t) * (size_t)g->n, cudaMemcpyHostToDevice, ctx->stream),
       "labels");
    k_labels_to_union<<<grid_of(g->n, ctx->num_sms), 256, 0, ctx->stream>>>(g->labels_alt, B->vgid, B->voff, g->n,
                                                                            g->labels);
    g->compressed = false;
    g->labels_vertex_space = true;
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "labels");
}

pcd_status pcd_batch_labels_get(pcd_graph *g, int32_t *labels) {
    if (!g || !g->batch || !labels) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    BatchState *B = g->batch;
    k_labels_to_local<<<grid_of(g->n, ctx->num_sms), 256, 0, ctx->stream>>>(
        g->labels, B->vgid, g->labels_vertex_space ? B->voff : B->gK, g->n, g->first);
    CK(cudaMemcpyAsync(labels, g->first, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, ctx->stream),
       "labels");
    return sync_and_check(g);
}

pcd_status pcd_batch_compress(pcd_graph *g, int32_t *per_graph_k) {
    if (!g || !g->batch) return PCD_ERR_INVALID_ARGUMENT;
    int launches = 0;
    TRY(ensure_compressed(g, &launches));
    g->labels_vertex_space = false;
    if (per_graph_k) {
        pcd_ctx *ctx = g->ctx;
        BatchState *B = g->batch;
        std::vector<int32_t> K((size_t)B->G + 1);
        CK(cudaMemcpyAsync(K.data(), B->gK, sizeof(int32_t) * (B->G + 1), cudaMemcpyDeviceToHost, ctx->stream), "gK");
        TRY(sync_and_check(g));
        for (int32_t i = 0; i < B->G; ++i) per_graph_k[i] = K[(size_t)i + 1] - K[(size_t)i];
    }
    return PCD_OK;
}

pcd_status pcd_batch_score(pcd_graph *g, const pcd_rule *rule, double *per_graph) {
    TRY(check_rule(g, rule));
    if (!g->batch || !per_graph) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    if (rule->kind == PCD_RULE_WCC) TRY(ensure_triangles(g));
    int launches = 0;
    TRY(ensure_compressed(g, &launches));
    g->labels_vertex_space = false;
    if (rule->kind == PCD_RULE_WCC)
        launch_wcc_score(g, nullptr, ctx->stream);
    else
        launch_score(g, rule->kind, rule->lambda, nullptr, ctx->stream);
    CK(cudaMemcpyAsync(per_graph, g->batch->gscore, sizeof(double) * g->batch->G, cudaMemcpyDeviceToHost,
                       ctx->stream),
       "scores");
    return sync_and_check(g);
}

static pcd_status batch_step(pcd_graph *g, const pcd_rule *rule, bool merge, double frac, int32_t rounds,
                             const uint32_t *seeds) {
    TRY(check_rule(g, rule));
    if (!g->batch || !seeds) return PCD_ERR_INVALID_ARGUMENT;
    if (!merge && !(frac > 0.0 && frac <= 1.0))
        return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "fraction should be in (0, 1]");
    if (merge && rounds <= 0) return set_error(g->ctx, PCD_ERR_INVALID_ARGUMENT, "rounds should be positive");
    pcd_ctx *ctx = g->ctx;
    if (rule->kind == PCD_RULE_WCC) TRY(ensure_triangles(g));
    int launches = 0;
    prof_begin(ctx, ctx->stream);
    TRY(ensure_compressed(g, &launches));
    g->labels_vertex_space = false;
    CK(cudaMemcpyAsync(g->batch->gseed, seeds, sizeof(uint32_t) * g->batch->G, cudaMemcpyHostToDevice, ctx->stream),
       "seeds");
    // a single step refines or merges every graph of the batch
    CK(cudaMemsetAsync(g->batch->gdone, 0, sizeof(int32_t) * g->batch->G, ctx->stream), "batch step");
    if (merge)
        TRY(run_merge(g, rule->kind, rule->lambda, rounds, 0, ctx->stream, &launches));
    else
        launches += launch_refine(g, rule->kind, rule->lambda, frac, 0, ctx->stream);
    std::swap(g->labels, g->labels_alt);
    g->compressed = false;
    g->info.kernels = launches;
    g->info.kernels_total += launches;
    TRY(scan_guard(g));
    return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "batch step");
}

pcd_status pcd_batch_refine(pcd_graph *g, const pcd_rule *rule, double frac, const uint32_t *seeds) {
    return batch_step(g, rule, false, frac, 0, seeds);
}

pcd_status pcd_batch_merge(pcd_graph *g, const pcd_rule *rule, int32_t rounds, const uint32_t *seeds) {
    return batch_step(g, rule, true, 0.0, rounds, seeds);
}

pcd_status pcd_batch_run(pcd_graph *g, const pcd_rule *rule, int32_t strategy, double frac, int32_t rounds,
                         int32_t n_iter, double threshold, int32_t use_cuda_graph, double *scores,
                         int32_t *iterations) {
    TRY(check_rule(g, rule));
    if (!g->batch) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    BatchState *B = g->batch;
    const int32_t G = B->G;
    if (!(frac > 0.0 && frac <= 1.0) || rounds <= 0 || strategy < 0 || strategy > 2)
        return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "bad schedule parameters");
    if (rule->kind == PCD_RULE_WCC)
        return set_error(ctx, PCD_ERR_UNSUPPORTED, "batched runs start from singletons; WCC needs -i 1");
    cudaStream_t st = ctx->stream;
    // each graph's seed stream: the reference driver seeds rand() with 1,
    // draws n_g values for the singleton partition, then one per refinement
    // call.  Every graph reads the same stream, so it is drawn once, up to
    // the largest graph plus the iteration cap: graph g's seed of iteration
    // it is value n_g + it.
    const int32_t cap = n_iter >= 0 ? std::max(n_iter, 1) : 1000;
    int32_t max_n = 0;
    for (int32_t gi = 0; gi < G; ++gi)
        max_n = std::max(max_n, B->h_voff[(size_t)gi + 1] - B->h_voff[(size_t)gi]);
    std::vector<uint32_t> stream((size_t)max_n + (size_t)cap);
    {
        pcd_rand r;
        pcd_rand_seed(&r, 1);
        for (auto &x : stream) x = (uint32_t)pcd_rand_next(&r);
    }
    std::vector<uint32_t> table((size_t)cap * G);
    for (int32_t gi = 0; gi < G; ++gi) {
        const size_t ng = (size_t)(B->h_voff[(size_t)gi + 1] - B->h_voff[(size_t)gi]);
        for (int32_t it = 0; it < cap; ++it) table[(size_t)it * G + gi] = stream[ng + (size_t)it];
    }
    if (B->seed_iters < cap) {
        if (B->seed_table) cudaFreeAsync(B->seed_table, st);
        B->seed_table = nullptr;
        CK(cudaMallocAsync(&B->seed_table, sizeof(uint32_t) * table.size(), st), "seed table");
        B->seed_iters = cap;
    }
    int32_t *iters_d = nullptr;
    double *final_d = nullptr;
    CK(cudaMallocAsync(&iters_d, sizeof(int32_t) * G + sizeof(double) * G + 64, st), "run buffers");
    final_d = reinterpret_cast<double *>(reinterpret_cast<char *>(iters_d) + ((sizeof(int32_t) * G + 63) & ~63ull));
    CK(cudaMemcpyAsync(B->seed_table, table.data(), sizeof(uint32_t) * table.size(), cudaMemcpyHostToDevice, st),
       "seeds");
    CK(cudaMemsetAsync(B->gdone, 0, sizeof(int32_t) * G, st), "run");
    CK(cudaMemsetAsync(B->gprev, 0, sizeof(double) * G, st), "run");
    CK(cudaMemsetAsync(B->iter, 0, sizeof(int32_t) * 4, st), "run");
    k_iota_union<<<grid_of(g->n, ctx->num_sms), 256, 0, st>>>(g->labels, g->n);
    g->compressed = false;
    const bool prof = ctx->prof_on;
    ctx->prof_on = false;
    const int32_t kind = rule->kind;
    const double lambda = rule->lambda;
    // one iteration: compress, score, stop test, this iteration's seeds, then
    // (when `refine`) a propagation sweep; labels stay in g->labels
    auto iteration_head = [&]() {
        launch_compress(g, st);
        launch_score(g, kind, lambda, nullptr, st);
        k_batch_stop<<<(G + 255) / 256, 256, 0, st>>>(G, B->gscore, B->gprev, B->gdone, iters_d, final_d, B->iter,
                                                      n_iter, threshold, cap);
        k_batch_seeds<<<(G + 255) / 256, 256, 0, st>>>(G, B->seed_table, cap, B->iter, B->gseed);
    };
    auto prop_tail = [&]() {
        launch_refine(g, kind, lambda, frac, 0, st);
        cudaMemcpyAsync(g->labels, g->labels_alt, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToDevice, st);
        k_incr<<<1, 1, 0, st>>>(B->iter);
    };
    cudaGraphExec_t exec = nullptr;
    const int32_t max_it = n_iter >= 0 ? n_iter : cap - 1;
    pcd_status s = PCD_OK;
    int32_t done_count = 0, done_at_bins = 0;
    int32_t *d_count = B->iter + 2;
    for (int32_t it = 0; it <= max_it && s == PCD_OK; ++it) {
        const bool is_prop = strategy == 0 || (strategy == 2 && it % 2 == 0);
        const bool last = it == max_it && n_iter >= 0;
        if (last) {  // only the stop test of the final iteration remains
            iteration_head();
            break;
        }
        if (is_prop && use_cuda_graph) {
            if (!exec) {
                // run the first propagation iteration eagerly: it also sets the
                // kernels' shared-memory attributes outside capture
                iteration_head();
                prop_tail();
                s = check_cuda(ctx, cudaStreamSynchronize(st), "batch iteration");
                if (s != PCD_OK) break;
                cudaGraph_t graph = nullptr;
                s = check_cuda(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "capture");
                if (s != PCD_OK) break;
                iteration_head();
                prop_tail();
                s = check_cuda(ctx, cudaStreamEndCapture(st, &graph), "capture");
                if (s != PCD_OK) break;
                s = check_cuda(ctx, cudaGraphInstantiate(&exec, graph, 0), "instantiate");
                cudaGraphDestroy(graph);
                if (s != PCD_OK) break;
                continue;  // the eager run was this iteration
            }
            s = check_cuda(ctx, cudaGraphLaunch(exec, st), "graph launch");
        } else {
            iteration_head();
            if (is_prop) {
                prop_tail();
            } else {
                int launches = 0;
                g->compressed = true;
                s = run_merge(g, kind, lambda, rounds, 0, st, &launches);
                if (s != PCD_OK) break;
                cudaMemcpyAsync(g->labels, g->labels_alt, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToDevice,
                                st);
                k_incr<<<1, 1, 0, st>>>(B->iter);
            }
        }
        if (n_iter < 0) {  // threshold mode: stop when every graph is done
            cudaMemsetAsync(d_count, 0, sizeof(int32_t), st);
            k_count_done<<<1, 1024, 0, st>>>(G, B->gdone, d_count);
            cudaMemcpyAsync(&done_count, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            s = check_cuda(ctx, cudaStreamSynchronize(st), "batch iteration");
            if (done_count == G) break;
            // finished graphs keep their labels: once an eighth more of them have
            // finished, the degree classes are rebuilt over the others, so the
            // sweeps and statistics skip them (a captured iteration is re-captured)
            if (s == PCD_OK && done_count - done_at_bins >= std::max(1, G / 8)) {
                launch_bins(g, st, true);
                done_at_bins = done_count;
                if (exec) {
                    cudaGraphExecDestroy(exec);
                    exec = nullptr;
                }
            }
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (done_at_bins > 0) {
        // every vertex back in its class; the last statistics pass skipped the
        // graphs that had left the classes, so recompute them for all graphs
        launch_bins(g, st);
        launch_stats(g, st);
    }
    // graphs are "done" only inside a run: later single steps refine every graph
    cudaMemsetAsync(B->gdone, 0, sizeof(int32_t) * G, st);
    ctx->prof_on = prof;
    g->compressed = true;
    g->labels_vertex_space = false;
    if (s == PCD_OK && scores)
        s = check_cuda(ctx, cudaMemcpyAsync(scores, final_d, sizeof(double) * G, cudaMemcpyDeviceToHost, st), "scores");
    if (s == PCD_OK && iterations)
        s = check_cuda(ctx, cudaMemcpyAsync(iterations, iters_d, sizeof(int32_t) * G, cudaMemcpyDeviceToHost, st),
                       "iterations");
    if (s == PCD_OK) s = sync_and_check(g);
    cudaFreeAsync(iters_d, st);
    return s;
}

}  // extern "C"
