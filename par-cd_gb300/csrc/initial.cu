// Triangle-based initial partition on the device
// (pcd_clustering_partition_device), the same labels as
// create_clustering_partition (src/framework.cpp:27-59):
//   order: by (-cc, -deg, id) ascending, cc = tri / double(deg * (deg - 1))
//          with the product in 32-bit int, as the reference computes it;
//          two stable radix sorts: (max_deg - deg, id), then the order-
//          preserving bits of -cc (-0.0 folded onto 0.0, which the
//          reference's pair comparison treats as equal);
//   claim: walking that order, an unlabelled vertex opens a community and
//          claims its unlabelled neighbours.  The vertices that open one are
//          the lexicographically first maximal independent set of that
//          order, found in rounds: an undecided vertex opens one when every
//          earlier neighbour is claimed, and is claimed as soon as an
//          earlier neighbour has opened one.  Every round decides at least
//          the earliest undecided vertex.  A warp scans a vertex's row from
//          the first earlier neighbour that was still undecided;
//   labels: an opener's label is the number of openers before it in the
//          order (a scan); a claimed vertex takes the label of its earliest
//          opener neighbour (atomicMin of ranks over the openers' rows).
#include <algorithm>
#include <climits>
#include <vector>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

using namespace pcd;

namespace {

constexpr int CP_THREADS = 256;
constexpr int CP_CHUNK = 16;
constexpr int32_t CP_UNDECIDED = 0, CP_OPENS = 1, CP_CLAIMED = 2;

int bit_len(uint64_t x) {
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

unsigned grid_for(int64_t items, int sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((items + CP_THREADS - 1) / CP_THREADS, (int64_t)sms * 8));
}

__global__ void k_cp_deg_keys(const int32_t *__restrict__ indices, int32_t n, int32_t max_deg, int vbits,
                              unsigned long long *keys, uint32_t *vals) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t deg = indices[v + 1] - indices[v];
        keys[v] = ((unsigned long long)(uint32_t)(max_deg - deg) << vbits) | (unsigned long long)v;
        vals[v] = (uint32_t)v;
    }
}

// -cc as bits that sort like the value (src/framework.cpp:33-37)
__global__ void k_cp_cc_keys(const int32_t *__restrict__ indices, const int32_t *__restrict__ tri, int32_t n,
                             const uint32_t *__restrict__ order, unsigned long long *keys, uint32_t *vals) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = (int32_t)order[s];
        const int32_t deg = indices[v + 1] - indices[v];
        const int32_t prod = (int32_t)((uint32_t)deg * (uint32_t)(deg - 1));
        const double cc = deg > 1 ? (double)tri[v] / (double)prod : 0.0;
        double x = -cc;
        if (x == 0.0) x = 0.0;
        const unsigned long long u = (unsigned long long)__double_as_longlong(x);
        keys[s] = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
        vals[s] = (uint32_t)v;
    }
}

__global__ void k_cp_rank(const uint32_t *__restrict__ order, int32_t n, int32_t *rank, int32_t *state,
                          int32_t *resume, const int32_t *__restrict__ indices, int32_t *list) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        rank[order[s]] = (int32_t)s;
        state[s] = CP_UNDECIDED;
        resume[s] = indices[s];
        list[s] = (int32_t)s;
    }
}

// One round over the undecided vertices, a warp per vertex.
__global__ void __launch_bounds__(CP_THREADS) k_cp_round(const int32_t *__restrict__ list_in,
                                                         const int32_t *__restrict__ count_in, int32_t *list_out,
                                                         int32_t *count_out, const int32_t *__restrict__ indices,
                                                         const int32_t *__restrict__ adj,
                                                         const int32_t *__restrict__ rank, int32_t *state,
                                                         int32_t *resume) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int32_t cnt = *count_in;
    for (int64_t w = gw; w < cnt; w += nw) {
        const int32_t v = list_in[w];
        const int32_t rv = rank[v], e = indices[v + 1];
        int32_t pending = -1;
        bool claimed = false;
        for (int32_t base = resume[v]; base < e; base += 32) {
            const int32_t j = base + lane;
            int32_t su = CP_CLAIMED;
            if (j < e) {
                const int32_t u = adj[j];
                if (rank[u] < rv) su = __ldcg(state + u);  // written by other warps this round
            }
            if (__any_sync(FULL, su == CP_OPENS)) {
                claimed = true;
                break;
            }
            const unsigned pm = __ballot_sync(FULL, su == CP_UNDECIDED);
            if (pm && pending < 0) pending = base + __ffs(pm) - 1;
        }
        if (lane == 0) {
            if (claimed) {
                state[v] = CP_CLAIMED;
            } else if (pending < 0) {
                state[v] = CP_OPENS;
            } else {
                resume[v] = pending;
                list_out[atomicAdd(count_out, 1)] = v;
            }
        }
    }
}

struct OpenLoad {
    const uint32_t *order;
    const int32_t *state;
    __device__ uint32_t operator()(int64_t s) const { return state[order[s]] == CP_OPENS ? 1u : 0u; }
};
struct OpenStore {
    const uint32_t *order;
    int32_t *clabel;
    __device__ void operator()(int64_t s, uint32_t ex, uint32_t val) const {
        if (val) clabel[order[s]] = (int32_t)ex;
    }
};

// best[u] = smallest rank of an opener next to u (edges of openers only)
__global__ void __launch_bounds__(CP_THREADS) k_cp_best(const int32_t *__restrict__ indices,
                                                        const int32_t *__restrict__ adj, int32_t n, int64_t nnz,
                                                        const int32_t *__restrict__ state,
                                                        const int32_t *__restrict__ rank, int32_t *best) {
    const int64_t nchunks = (nnz + CP_CHUNK - 1) / CP_CHUNK;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nchunks;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j0 = c * CP_CHUNK, j1 = min(nnz, j0 + CP_CHUNK);
        int32_t lo = 0, hi = n - 1;  // row of j0: the last v with indices[v] <= j0
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
            if (state[v] == CP_OPENS) atomicMin(best + adj[j], rank[v]);
        }
    }
}

__global__ void k_cp_labels(int32_t n, const int32_t *__restrict__ state, const int32_t *__restrict__ best,
                            const uint32_t *__restrict__ order, const int32_t *__restrict__ clabel, int32_t *labels,
                            DevCounters *ctr) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        if (state[v] == CP_OPENS) {
            labels[v] = clabel[v];
        } else {
            const int32_t b = best[v];
            if (state[v] != CP_CLAIMED || b < 0 || b >= n) {  // every claimed vertex has an opener neighbour
                atomicOr(&ctr->error, ERR_CHECK);
                atomicOr(&ctr->check_where, 64);
                labels[v] = -1;
            } else {
                labels[v] = clabel[order[b]];
            }
        }
    }
}

}  // namespace

extern "C" pcd_status pcd_clustering_partition_device(pcd_graph *g, int32_t *num_labels) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    if (g->batch) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "clustering partition works on single graphs");
    pcd_status s = ensure_triangles(g);
    if (s != PCD_OK) return s;
    cudaStream_t st = ctx->stream;
    const int32_t n = g->n;
    if (n == 0) {
        g->compressed = false;
        if (num_labels) *num_labels = 0;
        return PCD_OK;
    }
    const int sms = ctx->num_sms;
    std::vector<void *> bufs;
    auto alloc = [&](void **p, size_t bytes) {
        if (cudaMallocAsync(p, std::max<size_t>(bytes, 16), st) != cudaSuccess) return false;
        bufs.push_back(*p);
        return true;
    };
    auto release = [&]() {
        for (void *p : bufs) cudaFreeAsync(p, st);
        bufs.clear();
    };
    const size_t nn = (size_t)n;
    const int grid = sms * 2;
    const int64_t tile_cap = (std::max<int64_t>({(int64_t)n, 256ll * grid, 1}) + 2047) / 2048 + 2;
    unsigned long long *ka = nullptr, *kb = nullptr;
    uint32_t *va = nullptr, *vb = nullptr, *hist = nullptr, *tiles = nullptr;
    int32_t *rank = nullptr, *state = nullptr, *resume = nullptr, *list0 = nullptr, *list1 = nullptr,
            *counts = nullptr;
    if (!alloc((void **)&ka, 8 * nn) || !alloc((void **)&kb, 8 * nn) || !alloc((void **)&va, 4 * nn) ||
        !alloc((void **)&vb, 4 * nn) || !alloc((void **)&hist, 4ull * 256 * grid) ||
        !alloc((void **)&tiles, 4 * (size_t)tile_cap + 64) || !alloc((void **)&rank, 4 * nn) ||
        !alloc((void **)&state, 4 * nn) || !alloc((void **)&resume, 4 * nn) || !alloc((void **)&list0, 4 * nn) ||
        !alloc((void **)&list1, 4 * nn) || !alloc((void **)&counts, 64)) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "clustering partition buffers");
    }
    int32_t scan_overflow = 0;
    const ScanScratch sc{tiles, tile_cap, tiles + tile_cap, &scan_overflow};
    int launches = 0;
    // 1. the order: stable sort by (max_deg - deg, id), then by the bits of -cc
    const int vbits = std::max(1, bit_len((uint64_t)(n - 1)));
    k_cp_deg_keys<<<grid_for(n, sms), CP_THREADS, 0, st>>>(g->indices, n, g->max_deg, vbits, ka, va);
    const bool in1 = radix_sort(ka, va, kb, vb, n, vbits + bit_len((uint64_t)g->max_deg), hist, sc, grid, st,
                                &launches);
    const uint32_t *order1 = in1 ? vb : va;
    unsigned long long *k2 = in1 ? ka : kb;  // the free key buffer
    uint32_t *v2 = in1 ? va : vb;           // the free value buffer
    k_cp_cc_keys<<<grid_for(n, sms), CP_THREADS, 0, st>>>(g->indices, g->tri, n, order1, k2, v2);
    unsigned long long *k2o = k2 == ka ? kb : ka;
    uint32_t *v2o = v2 == va ? vb : va;
    const bool in2 = radix_sort(k2, v2, k2o, v2o, n, 64, hist, sc, grid, st, &launches);
    const uint32_t *order = in2 ? v2o : v2;
    // 2. rounds of the first maximal independent set of that order
    k_cp_rank<<<grid_for(n, sms), CP_THREADS, 0, st>>>(order, n, rank, state, resume, g->indices, list0);
    int32_t h_count = n;
    cudaMemcpyAsync(counts, &h_count, sizeof(int32_t), cudaMemcpyHostToDevice, st);
    s = check_cuda(ctx, cudaGetLastError(), "clustering partition launch");
    int32_t rounds = 0;
    int32_t *lin = list0, *lout = list1;
    int cur = 0;
    while (s == PCD_OK && h_count > 0) {
        if (rounds++ > n) {  // each round decides the earliest undecided vertex
            s = set_error(ctx, PCD_ERR_CUDA, "internal: clustering partition did not converge");
            break;
        }
        cudaMemsetAsync(counts + (1 - cur), 0, sizeof(int32_t), st);
        const unsigned blocks = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>(((int64_t)h_count + 7) / 8, (int64_t)sms * 16));
        k_cp_round<<<blocks, CP_THREADS, 0, st>>>(lin, counts + cur, lout, counts + (1 - cur), g->indices, g->adj,
                                                  rank, state, resume);
        cudaMemcpyAsync(&h_count, counts + (1 - cur), sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        s = check_cuda(ctx, cudaStreamSynchronize(st), "clustering partition round");
        std::swap(lin, lout);
        cur = 1 - cur;
    }
    // 3. labels: openers by a scan in order, claimed vertices from their earliest opener
    int32_t *clabel = resume, *best = list0;  // both free now
    if (s == PCD_OK) {
        launches += scan_exclusive(OpenLoad{order, state}, OpenStore{order, clabel}, n, sc, st);
        cudaMemsetAsync(best, 0x7f, 4 * nn, st);
        if (g->nnz > 0)
            k_cp_best<<<grid_for((g->nnz + CP_CHUNK - 1) / CP_CHUNK, sms), CP_THREADS, 0, st>>>(
                g->indices, g->adj, n, g->nnz, state, rank, best);
        k_cp_labels<<<grid_for(n, sms), CP_THREADS, 0, st>>>(n, state, best, order, clabel, g->labels, g->ctr);
        uint32_t opened = 0;
        cudaMemcpyAsync(&opened, tiles + tile_cap, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        release();
        s = sync_and_check(g);
        if (s == PCD_OK && scan_overflow) s = set_error(ctx, PCD_ERR_CUDA, "internal: clustering partition scan");
        if (s == PCD_OK && num_labels) *num_labels = (int32_t)opened;
    } else {
        release();
    }
    g->compressed = false;
    g->labels_vertex_space = false;
    return s;
}
