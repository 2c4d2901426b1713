// Connected components (pcd_find_connected): the fixed point of
// FindConnectedRefinement::refine (src/refinement.cpp:291-322), whose Jacobi
// rounds give every vertex the smallest vertex id of its component.  Here by
// union-find with hooking of the larger root under the smaller one, so a
// root is always the minimum of its tree and the result is the same fixed
// point, in one pass over the edges instead of one pass per diameter step.
//   1. parent[v] = v
//   2. edge pass: the adjacency is cut into equal chunks, one per thread; a
//      thread finds the row of its first entry by binary search and walks
//      on.  Each edge (v, u) with u < v unites the two trees.
//   3. parent[v] = root(v)
// Parent pointers only ever point to smaller ids, so every walk to a root
// ends; the hooking CAS retries only when another thread hooked the same
// root, and is bounded all the same (ERR_WAIT_TIMEOUT, never expected).
#include <algorithm>

#include "pcd_device.cuh"
#include "pcd_internal.h"

using namespace pcd;

namespace {

constexpr int CC_THREADS = 256;
constexpr int CC_CHUNK = 16;  // adjacency entries per thread
constexpr int CC_MAX_RETRIES = 1 << 24;

// Reads go to L2 (other SMs hook and halve concurrently; L1 is not coherent).
__device__ __forceinline__ int32_t cc_root(int32_t *parent, int32_t x) {
    int32_t p = __ldcg(parent + x);
    while (p != x) {  // path halving: parent[x] <- grandparent (still in the tree, still smaller)
        const int32_t gp = __ldcg(parent + p);
        if (gp != p) parent[x] = gp;
        x = p;
        p = gp;
    }
    return x;
}

__global__ void k_cc_init(int32_t *parent, int32_t n) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        parent[v] = (int32_t)v;
}

__global__ void __launch_bounds__(CC_THREADS) k_cc_hook(const int32_t *__restrict__ indices,
                                                        const int32_t *__restrict__ adj, int32_t n, int64_t nnz,
                                                        int32_t *parent, DevCounters *ctr) {
    const int64_t nchunks = (nnz + CC_CHUNK - 1) / CC_CHUNK;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nchunks;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j0 = c * CC_CHUNK, j1 = min(nnz, j0 + CC_CHUNK);
        // row of entry j0: the last v with indices[v] <= j0
        int32_t lo = 0, hi = n - 1;
        while (lo < hi) {
            const int32_t mid = lo + (hi - lo + 1) / 2;
            if (indices[mid] <= j0)
                lo = mid;
            else
                hi = mid - 1;
        }
        int32_t v = lo;
        int64_t vend = indices[v + 1];
        for (int64_t j = j0; j < j1; ++j) {
            while (j >= vend) vend = indices[++v + 1];
            const int32_t u = adj[j];
            if (u >= v) continue;  // each undirected edge once
            int32_t a = u, b = v;
            for (int it = 0;; ++it) {
                const int32_t ra = cc_root(parent, a), rb = cc_root(parent, b);
                if (ra == rb) break;
                const int32_t hi_r = max(ra, rb), lo_r = min(ra, rb);
                const int32_t old = atomicCAS(parent + hi_r, hi_r, lo_r);
                if (old == hi_r) break;
                if (it >= CC_MAX_RETRIES) {
                    atomicOr(&ctr->error, ERR_WAIT_TIMEOUT);
                    break;
                }
                a = hi_r;  // hi_r was hooked meanwhile: retry from its new root
                b = lo_r;
            }
        }
    }
}

__global__ void k_cc_flatten(int32_t *parent, int32_t n, int32_t *num_roots) {
    int32_t c = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = cc_root(parent, (int32_t)v);
        parent[v] = r;
        c += r == (int32_t)v;
    }
    c = __reduce_add_sync(FULL, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(num_roots, c);
}

unsigned grid_for(int64_t items, int sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((items + CC_THREADS - 1) / CC_THREADS, (int64_t)sms * 8));
}

}  // namespace

extern "C" pcd_status pcd_find_connected(pcd_graph *g, int32_t *num_components) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    if (g->batch) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "find_connected works on single graphs");
    const int32_t n = g->n;
    int32_t *parent = g->labels;
    int32_t *d_count = static_cast<int32_t *>(g->small);
    if (n > 0) {
        k_cc_init<<<grid_for(n, ctx->num_sms), CC_THREADS, 0, st>>>(parent, n);
        if (g->nnz > 0)
            k_cc_hook<<<grid_for((g->nnz + CC_CHUNK - 1) / CC_CHUNK, ctx->num_sms), CC_THREADS, 0, st>>>(
                g->indices, g->adj, n, g->nnz, parent, g->ctr);
        cudaMemsetAsync(d_count, 0, sizeof(int32_t), st);
        k_cc_flatten<<<grid_for(n, ctx->num_sms), CC_THREADS, 0, st>>>(parent, n, d_count);
    }
    g->compressed = false;
    g->labels_vertex_space = false;
    pcd_status s = check_cuda(ctx, cudaGetLastError(), "find_connected launch");
    if (s != PCD_OK || !num_components) return s;
    int32_t k = 0;
    if (n > 0) {
        s = check_cuda(ctx, cudaMemcpyAsync(&k, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st),
                       "find_connected count");
        if (s == PCD_OK) s = sync_and_check(g);
    }
    if (s == PCD_OK) *num_components = k;
    return s;
}
