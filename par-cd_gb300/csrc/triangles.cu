// Triangle statistics for WCC:
//   * Graph::count_triangles (src/graph.cpp:107-175): for every edge the
//     number of triangles through it; tri[v] sums it over v's edges (twice the
//     triangles at v) and tri_deg[v] counts v's edges that close a triangle;
//     the clustering coefficient is summed in vertex order, as the reference's
//     single-threaded call does (src/main.cpp:195), so it is bit-exact;
//   * WCCRule::calculate (src/rules.cpp:150-235): the same counts restricted
//     to triangles inside one community, then the per-vertex WCC terms.
// The reference's orientation: a triangle w < u < v is found once, from the
// edge (v, u) of v's row prefix (neighbours below v), by intersecting v's
// neighbours below u with u's neighbours below u; the edge counts live at
// each edge's position in its higher endpoint's row.  On the device a warp
// owns v and its lanes take different u; a lane walks the shorter of the two
// lists and binary-searches the longer.  A second pass turns the edge counts
// into tri / tri_deg.  The edge counts use the tie buffer (>= 2m ints), which
// no sweep holds while triangles are counted or WCC is scored.
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

// Edge counts of the triangles closed through the prefix edges of each v
// (labels non-null: only triangles whose three vertices share a label).
__global__ void __launch_bounds__(256) k_tri_edges(const int32_t *__restrict__ indices,
                                                   const int32_t *__restrict__ adj, int32_t n,
                                                   const int32_t *__restrict__ labels, int32_t *et) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t vv = warp; vv < n; vv += nwarps) {
        const int32_t v = (int32_t)vv;
        const int32_t bv = indices[v], ev = indices[v + 1];
        const int32_t l = labels ? labels[v] : 0;
        for (int32_t j0 = bv; j0 < ev; j0 += 32) {
            const int32_t r = j0 + lane;
            const int32_t u = r < ev ? adj[r] : INT32_MAX;
            if (!__any_sync(FULL, u < v)) break;  // rows are sorted: the prefix has ended
            if (u >= v || (labels && labels[u] != l)) continue;
            const int32_t bu = indices[u], eu = lower_bound_i32(adj, bu, indices[u + 1], u);
            // A = v's neighbours below u = [bv, r); B = u's neighbours below u = [bu, eu)
            int32_t c = 0;
            if (r - bv <= eu - bu) {
                int32_t y = bu;
                for (int32_t x = bv; x < r && y < eu; ++x) {
                    const int32_t w = adj[x];
                    y = lower_bound_i32(adj, y, eu, w);
                    if (y < eu && adj[y] == w && (!labels || labels[w] == l)) {
                        atomicAdd(et + x, 1);
                        atomicAdd(et + y, 1);
                        ++c;
                    }
                }
            } else {
                int32_t x = bv;
                for (int32_t y = bu; y < eu && x < r; ++y) {
                    const int32_t w = adj[y];
                    x = lower_bound_i32(adj, x, r, w);
                    if (x < r && adj[x] == w && (!labels || labels[w] == l)) {
                        atomicAdd(et + x, 1);
                        atomicAdd(et + y, 1);
                        ++c;
                    }
                }
            }
            if (c) atomicAdd(et + r, c);
        }
    }
}

// tri[v] / tri_deg[v] from the edge counts at the prefix positions.
__global__ void __launch_bounds__(256) k_tri_vertices(const int32_t *__restrict__ indices,
                                                      const int32_t *__restrict__ adj, int32_t n,
                                                      const int32_t *__restrict__ et, int32_t *tri,
                                                      int32_t *tri_deg) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t vv = warp; vv < n; vv += nwarps) {
        const int32_t v = (int32_t)vv;
        const int32_t bv = indices[v], ev = indices[v + 1];
        int32_t my_t = 0, my_td = 0;
        for (int32_t j0 = bv; j0 < ev; j0 += 32) {
            const int32_t r = j0 + lane;
            const int32_t u = r < ev ? adj[r] : INT32_MAX;
            if (!__any_sync(FULL, u < v)) break;
            if (u >= v) continue;
            const int32_t c = et[r];
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

static void launch_tri_counts(pcd_graph *g, const int32_t *labels, int32_t *tri, int32_t *tri_deg,
                              cudaStream_t st) {
    int32_t *et = g->tiebuf;  // >= 2m ints
    cudaMemsetAsync(et, 0, sizeof(int32_t) * (size_t)g->nnz, st);
    cudaMemsetAsync(tri, 0, sizeof(int32_t) * (size_t)g->n, st);
    cudaMemsetAsync(tri_deg, 0, sizeof(int32_t) * (size_t)g->n, st);
    int64_t blocks = ((int64_t)g->n * 32 + 255) / 256;
    const int64_t cap = (int64_t)g->ctx->num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_tri_edges<<<(unsigned)blocks, 256, 0, st>>>(g->indices, g->adj, g->n, labels, et);
    k_tri_vertices<<<(unsigned)blocks, 256, 0, st>>>(g->indices, g->adj, g->n, et, tri, tri_deg);
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
    launch_tri_counts(g, nullptr, g->tri, g->tri_deg, st);
    if (g->batch)
        k_clustering_coef<<<(g->batch->G + 7) / 8, 256, 0, st>>>(g->indices, g->tri, g->n, g->batch->voff,
                                                                  g->batch->G, g->batch->gcc);
    else
        k_clustering_coef<<<1, 32, 0, st>>>(g->indices, g->tri, g->n, nullptr, 1, g->d_score);
    return 3;
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
    launch_tri_counts(g, g->labels, it, itd, st);
    BatchState *B = g->batch;
    k_wcc_graph<<<B ? B->G : 1, WCC_THREADS, 0, st>>>(g->n, B ? B->voff : nullptr, g->labels, g->sizes, g->tri,
                                                      g->tri_deg, it, itd, B ? B->gscore : d_out);
    return 3;
}

}  // namespace pcd
