// Triangle statistics for WCC:
//   * Graph::count_triangles (src/graph.cpp:107-175): for every edge the
//     number of triangles through it; tri[v] sums it over v's edges (twice the
//     triangles at v) and tri_deg[v] counts v's edges that close a triangle;
//     the clustering coefficient is summed in vertex order, as the reference's
//     single-threaded call does (src/main.cpp:195), so it is bit-exact;
//   * WCCRule::calculate (src/rules.cpp:150-235): the same counts restricted
//     to triangles inside one community, then the per-vertex WCC terms.
// Each undirected edge (v, u), u < v, is handled once by the warp that owns v:
// lanes take different u and intersect the two sorted rows, walking the
// shorter row and binary-searching the longer one.
#include "pcd_device.cuh"
#include "pcd_internal.h"

namespace pcd {

__device__ __forceinline__ int32_t lower_bound_i32(const int32_t *__restrict__ a, int32_t lo, int32_t hi,
                                                   int32_t x) {
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (a[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// |N(v) cap N(u)|, optionally only common neighbours w with labels[w] == l.
__device__ int32_t intersect(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj, int32_t v,
                             int32_t u, const int32_t *__restrict__ labels, int32_t l) {
    int32_t bv = indices[v], ev = indices[v + 1], bu = indices[u], eu = indices[u + 1];
    if (ev - bv > eu - bu) {
        int32_t t;
        t = bv; bv = bu; bu = t;
        t = ev; ev = eu; eu = t;
    }
    int32_t c = 0, pos = bu;
    for (int32_t j = bv; j < ev && pos < eu; ++j) {
        int32_t w = adj[j];
        pos = lower_bound_i32(adj, pos, eu, w);
        if (pos < eu && adj[pos] == w && (!labels || labels[w] == l)) ++c;
    }
    return c;
}

__global__ void k_triangles(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj, int32_t n,
                            const int32_t *__restrict__ labels, int32_t *tri, int32_t *tri_deg) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < n; v += nwarps) {
        const int32_t b = indices[v], e = indices[v + 1];
        const int32_t l = labels ? labels[v] : 0;
        int32_t my_t = 0, my_td = 0;
        for (int32_t j = b + lane; j < e; j += 32) {
            const int32_t u = adj[j];
            if (u >= v) continue;  // rows are sorted: u < v is a prefix
            if (labels && labels[u] != l) continue;
            const int32_t c = intersect(indices, adj, (int32_t)v, u, labels, l);
            if (c > 0) {
                my_t += c;
                my_td += 1;
                atomicAdd(tri + u, c);
                atomicAdd(tri_deg + u, 1);
            }
        }
        my_t = __reduce_add_sync(FULL, my_t);
        my_td = __reduce_add_sync(FULL, my_td);
        if (lane == 0 && my_t) {
            atomicAdd(tri + v, my_t);
            atomicAdd(tri_deg + v, my_td);
        }
    }
}

// clustering_coef = sum over v of (tri / (deg (deg - 1.0))) / n, in vertex
// order (src/graph.cpp:491-499 with one thread).  One warp per graph (voff
// null: one graph [0, n)); lanes compute the terms, every lane adds them in
// order, lane 0 writes.
__global__ void k_clustering_coef(const int32_t *__restrict__ indices, const int32_t *__restrict__ tri, int32_t n,
                                  const int32_t *__restrict__ voff, int32_t G, double *out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (warp >= G) return;
    const int32_t v0 = voff ? voff[warp] : 0, v1 = voff ? voff[warp + 1] : n;
    const int32_t ng = v1 - v0;
    double cc = 0;
    for (int32_t base = v0; base < v1; base += 32) {
        const int32_t v = base + lane;
        double term = 0.0;
        bool has = false;
        if (v < v1) {
            int32_t deg = indices[v + 1] - indices[v];
            if (deg > 1) {
                term = (tri[v] / (deg * (deg - 1.0))) / ng;
                has = true;
            }
        }
        unsigned hm = __ballot_sync(FULL, has);
        for (int i = 0; i < 32; ++i) {
            double x = __shfl_sync(FULL, term, i);
            if ((hm >> i) & 1u) cc += x;
        }
    }
    if (lane == 0) out[warp] = cc;
}

int launch_triangles(pcd_graph *g, cudaStream_t st) {
    cudaMemsetAsync(g->tri, 0, sizeof(int32_t) * (size_t)g->n, st);
    cudaMemsetAsync(g->tri_deg, 0, sizeof(int32_t) * (size_t)g->n, st);
    int64_t warps = g->n;
    unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
    unsigned cap = (unsigned)g->ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_triangles<<<blocks, 256, 0, st>>>(g->indices, g->adj, g->n, nullptr, g->tri, g->tri_deg);
    if (g->batch)
        k_clustering_coef<<<(g->batch->G + 7) / 8, 256, 0, st>>>(g->indices, g->tri, g->n, g->batch->voff,
                                                                  g->batch->G, g->batch->gcc);
    else
        k_clustering_coef<<<1, 32, 0, st>>>(g->indices, g->tri, g->n, nullptr, 1, g->d_score);
    return 2;
}

// ---------------------------------------------------------------------------
// WCCRule::calculate: intra-community triangles, then
// sum_v [tri[v] > 0] (it/tri) * (dt / (size - 1 + dt - dit)) / n, reduced in
// a fixed double-double tree.  The reference sums with an OpenMP reduction
// whose order depends on the thread count, so this agrees within rounding.
// ---------------------------------------------------------------------------
struct DD2 {
    double hi, lo;
};

__device__ __forceinline__ DD2 dd2_add(DD2 a, double b) {
    double s = a.hi + b;
    double bb = s - a.hi;
    double err = (a.hi - (s - bb)) + (b - bb);
    double lo = a.lo + err;
    double hi = s + lo;
    lo = lo - (hi - s);
    return {hi, lo};
}

// One block per graph over its vertex range, like k_score_graph.
constexpr int WCC_THREADS = 1024;

__global__ void __launch_bounds__(WCC_THREADS) k_wcc_graph(int32_t n, const int32_t *__restrict__ voff,
                                                          const int32_t *__restrict__ labels,
                                                          const int32_t *__restrict__ sizes,
                                                          const int32_t *__restrict__ tri,
                                                          const int32_t *__restrict__ tri_deg,
                                                          const int32_t *__restrict__ it,
                                                          const int32_t *__restrict__ itd, double *out) {
    const int g = blockIdx.x;
    const int32_t v0 = voff ? voff[g] : 0, v1 = voff ? voff[g + 1] : n;
    const int32_t ng = v1 - v0;
    DD2 acc{0.0, 0.0};
    for (int32_t v = v0 + threadIdx.x; v < v1; v += WCC_THREADS) {
        int32_t t = tri[v];
        if (t > 0) {
            int32_t size = sizes[labels[v]];
            double a = it[v] / (double)t;
            double b = tri_deg[v] / (double)(size - 1 + tri_deg[v] - itd[v]);
            acc = dd2_add(acc, (a * b) / ng);
        }
    }
    __shared__ DD2 sh[WCC_THREADS];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = WCC_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            DD2 x = dd2_add(sh[threadIdx.x], sh[threadIdx.x + s].hi);
            sh[threadIdx.x] = dd2_add(x, sh[threadIdx.x + s].lo);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[g] = sh[0].hi + sh[0].lo;
}

int launch_wcc_score(pcd_graph *g, double *d_out, cudaStream_t st) {
    // intra-community counts reuse the propagation scratch: ndraw and first
    int32_t *it = reinterpret_cast<int32_t *>(g->ndraw);
    int32_t *itd = g->first;
    cudaMemsetAsync(it, 0, sizeof(int32_t) * (size_t)g->n, st);
    cudaMemsetAsync(itd, 0, sizeof(int32_t) * (size_t)g->n, st);
    int64_t warps = g->n;
    unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
    unsigned cap = (unsigned)g->ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_triangles<<<blocks, 256, 0, st>>>(g->indices, g->adj, g->n, g->labels, it, itd);
    BatchState *B = g->batch;
    k_wcc_graph<<<B ? B->G : 1, WCC_THREADS, 0, st>>>(g->n, B ? B->voff : nullptr, g->labels, g->sizes, g->tri,
                                                      g->tri_deg, it, itd, B ? B->gscore : d_out);
    return 2;
}

}  // namespace pcd
