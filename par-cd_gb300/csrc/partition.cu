// Partition bookkeeping on the device:
//   * compress  : first-occurrence relabel  (compress_labels, src/framework.cpp:146-170)
//   * stats     : per-community size / internal / external volume
//                 (collect_statistics, src/framework.cpp:69-143)
//   * score     : Rule::calculate for Modularity and CPM (src/rules.cpp:9-22, 121-129)
//   * validate  : the CSR checks Graph::read leaves implicit
//   * bins      : vertices grouped by degree class for the sweep kernels
#include <algorithm>
#include <climits>
#include <vector>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

namespace pcd {

// ---------------------------------------------------------------------------
// scan of tile sums (declared in pcd_scan.cuh)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_scan_tile_sums(uint32_t *tile_sums, int64_t ntiles, uint32_t *total) {
    uint32_t carry = 0;
    for (int64_t base = 0; base < ntiles; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        uint32_t x = i < ntiles ? tile_sums[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_sum_u32(x, &tot);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_fill_i32(int32_t *p, int32_t v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

static inline unsigned grid_for(int64_t n, int threads, int cap = 152 * 32) {
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// ---------------------------------------------------------------------------
// compress_labels: label L keeps the rank of its first vertex among all
// "first occurrences" (first vertex of each label, and every NEW_LABEL vertex).
// ---------------------------------------------------------------------------
__global__ void k_first_occurrence(const int32_t *__restrict__ labels, int32_t n, int32_t *first,
                                   DevCounters *ctr) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int32_t L = labels[v];
        if (L >= 0 && L < n)
            atomicMin(first + L, (int32_t)v);
        else if (L != -1)
            atomicOr(&ctr->error, ERR_LABEL_RANGE);
    }
}

struct FirstFlag {
    const int32_t *labels;
    const int32_t *first;
    int32_t n;
    __device__ uint32_t operator()(int64_t v) const {
        int32_t L = labels[v];
        if (L < 0 || L >= n) return 1u;
        return first[L] == (int32_t)v ? 1u : 0u;
    }
};

struct StoreRank {
    int32_t *rank;
    __device__ void operator()(int64_t v, uint32_t x, uint32_t) const { rank[v] = (int32_t)x; }
};

__global__ void k_relabel(int32_t *labels, const int32_t *__restrict__ rank, const int32_t *__restrict__ first,
                          int32_t n) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int32_t L = labels[v];
        labels[v] = (L < 0 || L >= n) ? rank[v] : rank[first[L]];
    }
}

__global__ void k_set_k(DevCounters *ctr, const uint32_t *total) { ctr->k = (int32_t)*total; }

// ---------------------------------------------------------------------------
// collect_statistics.  sizes[l] += 1, intv[l] += d_int, extv[l] += d_ext,
// vol[l] += deg.  Integer sums: the result does not depend on order.
// ---------------------------------------------------------------------------
// Lanes of the warp that share a community add once, through their leader.
// The leader sums its group's counts from shared memory (a loop as long as
// the largest group; warp reductions over per-group masks would run once per
// distinct community of the warp).  `wsh`: this warp's 32 slots.
__device__ __forceinline__ void add_stats(int32_t l, int32_t di, int32_t de, int32_t *intv, int32_t *extv,
                                          int32_t *vol, bool valid, int2 *wsh) {
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(FULL, valid ? l : -1 - lane);
    wsh[lane] = make_int2(di, de);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) {
        int32_t a = 0, b = 0;
        for (unsigned m = peers; m; m &= m - 1) {
            const int2 x = wsh[__ffs(m) - 1];
            a += x.x;
            b += x.y;
        }
        atomicAdd(intv + l, a);
        atomicAdd(extv + l, b);
        atomicAdd(vol + l, a + b);
    }
    __syncwarp();
}

// Community sizes first (one pass over the listed vertices), so that the
// volume kernels skip the neighbour labels of a vertex alone in its community:
// it has no internal edge (no loops), all its edges are external.
__global__ void k_stat_sizes(const int32_t *__restrict__ list, int64_t count, const int32_t *__restrict__ labels,
                             int32_t *sizes) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(sizes + labels[list[i]], 1);
}

// `singles`: the partition has one vertex per community (k == n right after a
// compress; see launch_stats), so no neighbour shares a vertex's label (the
// graph has no loops) and the neighbour labels need not be read.
__global__ void k_stats_thread(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj,
                               const int32_t *__restrict__ labels, const int32_t *__restrict__ list,
                               int64_t count, int32_t *sizes, int32_t *intv, int32_t *extv, int32_t *vol,
                               const int32_t *k_dev, int32_t n_all) {
    __shared__ int2 sh[1024];
    const bool singles = k_dev && *k_dev == n_all;
    int2 *wsh = sh + (threadIdx.x & ~31u);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rounds = (count + stride - 1) / stride;
    for (int64_t r = 0; r < rounds; ++r) {
        int64_t idx = start + r * stride;
        bool valid = idx < count;
        int32_t l = 0, di = 0, de = 0;
        if (valid) {
            int32_t v = list[idx];
            l = labels[v];
            int32_t b = indices[v], e = indices[v + 1];
            const bool alone = singles || sizes[l] == 1;
            for (int32_t j = b; j < (alone ? b : e); j += 4) {  // four gathers in flight
                int32_t u[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) u[k] = j + k < e ? adj[j + k] : -1;
#pragma unroll
                for (int k = 0; k < 4; ++k) di += u[k] >= 0 && labels[u[k]] == l;
            }
            de = (e - b) - di;
        }
        add_stats(l, di, de, intv, extv, vol, valid, wsh);
    }
}

// Warp per vertex for the larger degrees; lane 0 adds the vertex's counts.
// Neighbour ids are >= 0 in a validated graph, so -1 marks a lane past the row.
__global__ void k_stats_warp(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj,
                             const int32_t *__restrict__ labels, const int32_t *__restrict__ list,
                             int64_t count, int32_t *sizes, int32_t *intv, int32_t *extv, int32_t *vol,
                             const int32_t *k_dev, int32_t n_all) {
    const int lane = threadIdx.x & 31;
    const bool singles = k_dev && *k_dev == n_all;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t idx = warp; idx < count; idx += nwarps) {
        int32_t v = list[idx];
        int32_t l = labels[v];
        int32_t b = indices[v], e = indices[v + 1];
        int32_t di = 0;
        const bool alone = singles || sizes[l] == 1;
        for (int32_t j = b + lane; j < (alone ? b : e); j += 4 * 32) {  // four gathers in flight per lane
            int32_t u[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) u[k] = j + 32 * k < e ? adj[j + 32 * k] : -1;
#pragma unroll
            for (int k = 0; k < 4; ++k) di += u[k] >= 0 && labels[u[k]] == l;
        }
#pragma unroll
        for (int d = 16; d; d >>= 1) di += __shfl_xor_sync(FULL, di, d);
        if (lane == 0) {
            int32_t de = (e - b) - di;
            atomicAdd(intv + l, di);
            atomicAdd(extv + l, de);
            atomicAdd(vol + l, e - b);
        }
    }
}

// Block per vertex for rows above 2048 neighbours (one warp would walk them
// alone): BT threads with four label gathers in flight each, one set of
// atomics per vertex.  (256-thread blocks for 257..2048 were slower than a
// warp per row there.)
template <int BT>
__global__ void __launch_bounds__(BT) k_stats_block(const int32_t *__restrict__ indices,
                                                    const int32_t *__restrict__ adj,
                                                    const int32_t *__restrict__ labels,
                                                    const int32_t *__restrict__ list, int64_t count, int32_t *sizes,
                                                    int32_t *intv, int32_t *extv, int32_t *vol,
                                                    const int32_t *k_dev, int32_t n_all) {
    constexpr int NW = BT / 32;
    const bool singles = k_dev && *k_dev == n_all;
    __shared__ int32_t part[NW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t idx = blockIdx.x; idx < count; idx += gridDim.x) {
        const int32_t v = list[idx];
        const int32_t l = labels[v];
        const int32_t b = indices[v], e = indices[v + 1];
        int32_t di = 0;
        const bool alone = singles || sizes[l] == 1;
        for (int32_t j0 = b + (int32_t)threadIdx.x; j0 < (alone ? b : e); j0 += 4 * BT) {
            int32_t u[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) u[k] = j0 + k * BT < e ? adj[j0 + k * BT] : -1;
#pragma unroll
            for (int k = 0; k < 4; ++k) di += u[k] >= 0 && labels[u[k]] == l;
        }
        di = __reduce_add_sync(FULL, di);
        if (lane == 0) part[wid] = di;
        __syncthreads();
        if (threadIdx.x == 0) {
            int32_t t = 0;
            for (int w = 0; w < NW; ++w) t += part[w];
            atomicAdd(intv + l, t);
            atomicAdd(extv + l, (e - b) - t);
            atomicAdd(vol + l, e - b);
        }
        __syncthreads();
    }
}

// after_compress: ctr->k holds the community count of the current labels
// (launch_compress has just set it), so a partition of single vertices can be
// recognised on the device; other callers pass false.
int launch_stats(pcd_graph *g, cudaStream_t st, bool after_compress) {
    int launches = 0;
    const int32_t *k_dev = after_compress ? &g->ctr->k : nullptr;
    size_t bytes = sizeof(int32_t) * (size_t)(g->n > 0 ? g->n : 1);
    cudaMemsetAsync(g->sizes, 0, bytes, st);
    cudaMemsetAsync(g->intv, 0, bytes, st);
    cudaMemsetAsync(g->extv, 0, bytes, st);
    cudaMemsetAsync(g->vol, 0, bytes, st);
    const int64_t listed = g->bin_off[NBINS] - g->bin_off[0];
    if (listed > 0) {
        k_stat_sizes<<<grid_for(listed, 256), 256, 0, st>>>(g->bin_list + g->bin_off[0], listed, g->labels, g->sizes);
        prof_mark(g->ctx, "stats.sizes", st);
        ++launches;
    }
    int64_t nt = g->bin_off[BIN_WARP] - g->bin_off[0];
    if (nt > 0) {
        k_stats_thread<<<grid_for(nt, 256), 256, 0, st>>>(g->indices, g->adj, g->labels,
                                                           g->bin_list + g->bin_off[0], nt, g->sizes,
                                                           g->intv, g->extv, g->vol, k_dev, g->n);
        prof_mark(g->ctx, "stats.thread", st);
        ++launches;
    }
    int64_t nw = g->bin_off[BIN_BLOCK_L] - g->bin_off[BIN_WARP];
    if (nw > 0) {
        k_stats_warp<<<grid_for(nw * 32, 256), 256, 0, st>>>(g->indices, g->adj, g->labels,
                                                             g->bin_list + g->bin_off[BIN_WARP], nw, g->sizes,
                                                             g->intv, g->extv, g->vol, k_dev, g->n);
        prof_mark(g->ctx, "stats.warp", st);
        ++launches;
    }
    int64_t nl = g->bin_off[NBINS] - g->bin_off[BIN_BLOCK_L];
    if (nl > 0) {
        const unsigned blocks = (unsigned)std::min<int64_t>(nl, (int64_t)g->ctx->num_sms * 4);
        k_stats_block<512><<<blocks, 512, 0, st>>>(g->indices, g->adj, g->labels,
                                                   g->bin_list + g->bin_off[BIN_BLOCK_L], nl, g->sizes, g->intv,
                                                   g->extv, g->vol, k_dev, g->n);
        prof_mark(g->ctx, "stats.block_l", st);
        ++launches;
    }
    return launches;
}

// Batch: community -> graph, and the first community of each graph (the label
// of its first vertex: compress numbers communities by first occurrence).
__global__ void k_batch_comm(const int32_t *__restrict__ labels, const int32_t *__restrict__ vgid,
                             const int32_t *__restrict__ voff, int32_t G, int32_t n, int32_t *cgid, int32_t *gK,
                             const DevCounters *ctr) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        cgid[labels[v]] = vgid[v];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= G; i += (int64_t)gridDim.x * blockDim.x)
        gK[i] = i < G ? labels[voff[i]] : ctr->k;
}

int launch_compress(pcd_graph *g, cudaStream_t st) {
    int launches = 0;
    const int32_t n = g->n;
    k_fill_i32<<<grid_for(n, 256), 256, 0, st>>>(g->first, INT_MAX, n);
    k_first_occurrence<<<grid_for(n, 256), 256, 0, st>>>(g->labels, n, g->first, g->ctr);
    launches += 2;
    launches += scan_exclusive(FirstFlag{g->labels, g->first, n}, StoreRank{g->labels_alt}, n, g->scan, st);
    k_relabel<<<grid_for(n, 256), 256, 0, st>>>(g->labels, g->labels_alt, g->first, n);
    k_set_k<<<1, 1, 0, st>>>(g->ctr, g->scan_total);
    launches += 2;
    if (g->batch) {
        k_batch_comm<<<grid_for(n, 256), 256, 0, st>>>(g->labels, g->batch->vgid, g->batch->voff, g->batch->G, n,
                                                        g->batch->cgid, g->batch->gK, g->ctr);
        ++launches;
    }
    prof_mark(g->ctx, "compress", st);
    launches += launch_stats(g, st, true);
    return launches;
}

// ---------------------------------------------------------------------------
// Rule::calculate for Modularity / CPM (src/rules.cpp:9-22, 121-129).  The
// per-community terms are rational with denominator 2m (CPM) or (2m)^2
// (Modularity), so the sums are taken exactly in integers,
//     Modularity = I / 2m - S / (2m)^2,   I = sum int_c, S = sum vol_c^2,
//     CPM        = (I - lambda * P) / 2m, P = sum size_c (size_c - 1),
// and rounded once at the end (the reference rounds every term and the
// running sum; the two agree to the reference's own rounding error).  Integer
// sums do not depend on the order or grouping of the additions, so a graph
// gets the same score alone or in a batch, from one block or from many.
// S <= (2m)^2 < 2^64 and P <= n^2 < 2^62 for 32-bit sizes.
// ---------------------------------------------------------------------------
struct ScoreSums {
    unsigned long long a, b;
};

__device__ __forceinline__ ScoreSums score_terms(int32_t kind, int64_t i, const int32_t *__restrict__ sizes,
                                                 const int32_t *__restrict__ intv, const int32_t *__restrict__ vol) {
    if (kind == 0) {
        const unsigned long long v = (unsigned)vol[i];
        return {(unsigned long long)(unsigned)intv[i], v * v};
    }
    const long long sz = sizes[i];
    return {(unsigned long long)(unsigned)intv[i], (unsigned long long)(sz * (sz - 1))};
}

__device__ __forceinline__ double score_value(int32_t kind, double lambda, int32_t m, bool empty,
                                              unsigned long long a, unsigned long long b) {
    const double tm = 2.0 * (double)m;
    if (kind == 0) return empty ? 0.0 : (double)a / tm - (double)b / (tm * tm);
    return ((double)a - lambda * (double)b) / tm;
}

__device__ __forceinline__ ScoreSums block_sum(ScoreSums x) {
    __shared__ unsigned long long sa[32], sb[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o; o >>= 1) {
        x.a += __shfl_down_sync(0xffffffffu, x.a, o);
        x.b += __shfl_down_sync(0xffffffffu, x.b, o);
    }
    if (lane == 0) {
        sa[w] = x.a;
        sb[w] = x.b;
    }
    __syncthreads();
    ScoreSums r{0, 0};
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            r.a += sa[i];
            r.b += sb[i];
        }
    return r;  // valid in thread 0
}

// batch: one block per graph, community range [gK[g], gK[g + 1])
__global__ void __launch_bounds__(256) k_score_graphs(int32_t kind, double lambda, const int32_t *__restrict__ gm,
                                                      const int32_t *__restrict__ gK,
                                                      const int32_t *__restrict__ sizes,
                                                      const int32_t *__restrict__ intv,
                                                      const int32_t *__restrict__ vol, double *out) {
    const int g = blockIdx.x;
    const int32_t c0 = gK[g], c1 = gK[g + 1];
    ScoreSums acc{0, 0};
    for (int32_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
        const ScoreSums t = score_terms(kind, i, sizes, intv, vol);
        acc.a += t.a;
        acc.b += t.b;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) out[g] = score_value(kind, lambda, gm[g], c1 <= c0, acc.a, acc.b);
}

// one graph: every block adds its partial sums into acc[0..1]
__global__ void __launch_bounds__(256) k_score_single(int32_t kind, const int32_t *__restrict__ sizes,
                                                      const int32_t *__restrict__ intv,
                                                      const int32_t *__restrict__ vol, const DevCounters *ctr,
                                                      unsigned long long *acc_out) {
    const int32_t k = ctr->k;
    ScoreSums acc{0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
        const ScoreSums t = score_terms(kind, i, sizes, intv, vol);
        acc.a += t.a;
        acc.b += t.b;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0 && (acc.a | acc.b)) {
        atomicAdd(acc_out, acc.a);
        atomicAdd(acc_out + 1, acc.b);
    }
}

__global__ void k_score_final(int32_t kind, double lambda, int32_t m, const DevCounters *ctr,
                              const unsigned long long *acc, double *out) {
    *out = score_value(kind, lambda, m, ctr->k <= 0, acc[0], acc[1]);
}

int launch_score(pcd_graph *g, int32_t kind, double lambda, double *d_out, cudaStream_t st) {
    BatchState *B = g->batch;
    if (B) {
        k_score_graphs<<<B->G, 256, 0, st>>>(kind, lambda, B->gm, B->gK, g->sizes, g->intv, g->vol, B->gscore);
        return 1;
    }
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(g->small);
    cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), st);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((g->n + 255) / 256, g->ctx->num_sms * 4ll));
    k_score_single<<<grid, 256, 0, st>>>(kind, g->sizes, g->intv, g->vol, g->ctr, acc);
    k_score_final<<<1, 1, 0, st>>>(kind, lambda, g->m, g->ctr, acc, d_out);
    return 2;
}

// ---------------------------------------------------------------------------
// CSR validation in two parts.  The row offsets alone (monotone, spanning
// [0, 2m]; flag bits 1 and 2) and the largest degree need only `indices`, so
// they run while the neighbour array is still being copied; the rows
// (neighbours in range, strictly increasing, no loops; bit 4) follow once it
// has arrived, and only over offsets that passed.
// ---------------------------------------------------------------------------
__global__ void k_check_offsets(const int32_t *__restrict__ indices, int32_t n, int32_t m, int32_t *flag) {
    int32_t bad = 0, mx = 0;
    const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t0 == 0 && (indices[0] != 0 || (int64_t)indices[n] != 2 * (int64_t)m)) bad |= 1;
    for (int64_t v = t0; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = indices[v], e = indices[v + 1];
        if (b > e || b < 0 || (int64_t)e > 2 * (int64_t)m) bad |= 2;
        mx = max(mx, e - b);
    }
    bad = __reduce_or_sync(FULL, bad);
    mx = __reduce_max_sync(FULL, mx);
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(flag, bad);
        atomicMax(flag + 1, mx);
    }
}

// Rows (bit 4 of flag), by degree class from the class lists (bin_list), so
// that no thread walks a long row alone: a thread per row up to 32 neighbours,
// a warp per row up to 2048, a 512-thread block per longer row; four loads in
// flight per thread.  Within a row the neighbours must increase strictly, lie
// in [0, n) and differ from the row's vertex.  One launch checks the rows
// whose end offset lies in (lo, hi]: the neighbour array arrives in pieces,
// and a row is checked once its last neighbour has.  The offsets have passed
// k_check_offsets.
__global__ void k_validate_thread(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj, int32_t n,
                                  const int32_t *__restrict__ list, int64_t count, int64_t lo, int64_t hi,
                                  int32_t *flag) {
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = list[i];
        const int32_t e = indices[v + 1];
        if (e <= lo || e > hi) continue;
        const int32_t b = indices[v];
        int32_t prev = -1;  // ids are >= 0, so the first neighbour always exceeds it
        for (int32_t j = b; j < e; j += 4) {
            int32_t u[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) u[k] = j + k < e ? adj[j + k] : INT_MAX;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (j + k < e) {
                    bad |= u[k] < 0 || u[k] >= n || u[k] == v || u[k] <= prev;
                    prev = u[k];
                }
            }
        }
    }
    if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 4);
}

// `nw` warps walk row [b, e) of vertex v in 32-entry chunks (chunk c of the
// row to warp c % nw); the neighbour before each lane's entry comes from the
// lane below, or from memory for lane 0.
__device__ __forceinline__ bool check_row_warps(const int32_t *__restrict__ adj, int32_t n, int32_t v, int32_t b,
                                                int32_t e, int wid, int nw, int lane) {
    bool bad = false;
    for (int64_t c0 = (int64_t)b + 32 * wid; c0 < e; c0 += 4ll * 32 * nw) {
        int32_t u[4], p0[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t c = c0 + 32ll * nw * k, j = c + lane;
            u[k] = j < e ? adj[j] : 0;
            p0[k] = lane == 0 && c < e && c > b ? adj[c - 1] : -1;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int64_t j = c0 + 32ll * nw * k + lane;
            int32_t prev = __shfl_up_sync(FULL, u[k], 1);
            if (lane == 0) prev = p0[k];
            if (j < e) bad |= u[k] < 0 || u[k] >= n || u[k] == v || (j > b && prev >= u[k]);
        }
    }
    return bad;
}

__global__ void k_validate_warp(const int32_t *__restrict__ indices, const int32_t *__restrict__ adj, int32_t n,
                                const int32_t *__restrict__ list, int64_t count, int64_t lo, int64_t hi,
                                int32_t *flag) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    bool bad = false;
    for (int64_t i = warp; i < count; i += nwarps) {
        const int32_t v = list[i];
        const int32_t e = indices[v + 1];
        if (e <= lo || e > hi) continue;
        bad |= check_row_warps(adj, n, v, indices[v], e, 0, 1, lane);
    }
    if (__any_sync(FULL, bad) && lane == 0) atomicOr(flag, 4);
}

__global__ void __launch_bounds__(512) k_validate_block(const int32_t *__restrict__ indices,
                                                        const int32_t *__restrict__ adj, int32_t n,
                                                        const int32_t *__restrict__ list, int64_t count,
                                                        int64_t lo, int64_t hi, int32_t *flag) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    bool bad = false;
    for (int64_t i = blockIdx.x; i < count; i += gridDim.x) {
        const int32_t v = list[i];
        const int32_t e = indices[v + 1];
        if (e <= lo || e > hi) continue;
        bad |= check_row_warps(adj, n, v, indices[v], e, wid, 16, lane);
    }
    if (__any_sync(FULL, bad) && lane == 0) atomicOr(flag, 4);
}

int launch_check_offsets(const int32_t *indices, int32_t n, int32_t m, int32_t *d_flag, cudaStream_t st) {
    k_check_offsets<<<grid_for(std::max<int64_t>(n, 1), 256), 256, 0, st>>>(indices, n, m, d_flag);
    return 1;
}

int launch_validate_rows(pcd_graph *g, int32_t *d_flag, int64_t lo, int64_t hi, cudaStream_t st) {
    int launches = 0;
    const int64_t nt = g->bin_off[BIN_WARP] - g->bin_off[0];
    const int64_t nw = g->bin_off[BIN_BLOCK_L] - g->bin_off[BIN_WARP];
    const int64_t nb = g->bin_off[NBINS] - g->bin_off[BIN_BLOCK_L];
    if (nt > 0) {
        k_validate_thread<<<grid_for(nt, 256), 256, 0, st>>>(g->indices, g->adj, g->n, g->bin_list + g->bin_off[0],
                                                              nt, lo, hi, d_flag);
        ++launches;
    }
    if (nw > 0) {
        k_validate_warp<<<grid_for(nw * 32, 256), 256, 0, st>>>(g->indices, g->adj, g->n,
                                                                 g->bin_list + g->bin_off[BIN_WARP], nw, lo, hi,
                                                                 d_flag);
        ++launches;
    }
    if (nb > 0) {
        const unsigned blocks = (unsigned)std::min<int64_t>(nb, (int64_t)g->ctx->num_sms * 4);
        k_validate_block<<<blocks, 512, 0, st>>>(g->indices, g->adj, g->n, g->bin_list + g->bin_off[BIN_BLOCK_L], nb,
                                                 lo, hi, d_flag);
        ++launches;
    }
    return launches;
}

// ---------------------------------------------------------------------------
// degree bins: stable compaction of the vertices of each class
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t bin_of(int32_t d, const BinConfig &b) {
    for (int i = 0; i < NBINS - 1; ++i)
        if (d <= b.max_deg[i]) return i;
    return NBINS - 1;
}

constexpr int MAX_SUBS = 16;
constexpr int BIN_TILE = 256;  // vertices per block of the count and scatter passes
struct SubBounds {
    int32_t count;
    int32_t lo[MAX_SUBS], hi[MAX_SUBS];
};

// The sub-range of vertex v (degree class cut at powers of two), or -1 when v
// is left out (a batch's finished graph).
__device__ __forceinline__ int sub_of(const int32_t *__restrict__ indices, int64_t v, const SubBounds &sb,
                                      const int32_t *__restrict__ vgid, const int32_t *__restrict__ gdone,
                                      int32_t &d) {
    d = indices[v + 1] - indices[v];
    if (gdone && gdone[vgid[v]]) return -1;
    for (int s = 0; s < sb.count; ++s)
        if (d > sb.lo[s] && d <= sb.hi[s]) return s;
    return -1;
}

// Per tile of BIN_TILE vertices: its count in every sub-range (written
// sub-major, cnt[s * ntiles + tile], so one exclusive scan gives every tile's
// place in the class list) and the largest degree of every sub-range.
__global__ void __launch_bounds__(BIN_TILE) k_bins_count(const int32_t *__restrict__ indices, int32_t n,
                                                         SubBounds sb, const int32_t *__restrict__ vgid,
                                                         const int32_t *__restrict__ gdone, int64_t ntiles,
                                                         uint32_t *cnt, int32_t *maxdeg) {
    __shared__ uint32_t c[MAX_SUBS];
    __shared__ int32_t mx[MAX_SUBS];
    if (threadIdx.x < MAX_SUBS) {
        c[threadIdx.x] = 0;
        mx[threadIdx.x] = 0;
    }
    __syncthreads();
    const int64_t v = blockIdx.x * (int64_t)BIN_TILE + threadIdx.x;
    if (v < n) {
        int32_t d;
        const int sv = sub_of(indices, v, sb, vgid, gdone, d);
        if (sv >= 0) {
            atomicAdd(&c[sv], 1u);
            atomicMax(&mx[sv], d);
        }
    }
    __syncthreads();
    if (threadIdx.x < sb.count) {
        cnt[threadIdx.x * ntiles + blockIdx.x] = c[threadIdx.x];
        if (mx[threadIdx.x] > 0) atomicMax(&maxdeg[threadIdx.x], mx[threadIdx.x]);
    }
}

// Each vertex to its place: the tile's offset in its sub-range, plus the
// vertices of the same sub-range before it in the tile (warps in order, lanes
// in order), so every class list is in vertex order.
__global__ void __launch_bounds__(BIN_TILE) k_bins_scatter(const int32_t *__restrict__ indices, int32_t n,
                                                           SubBounds sb, const int32_t *__restrict__ vgid,
                                                           const int32_t *__restrict__ gdone, int64_t ntiles,
                                                           const uint32_t *__restrict__ off, int32_t *list) {
    constexpr int NW = BIN_TILE / 32;
    __shared__ uint32_t wc[NW][MAX_SUBS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < NW * MAX_SUBS; i += BIN_TILE) wc[i / MAX_SUBS][i % MAX_SUBS] = 0;
    __syncthreads();
    const int64_t v = blockIdx.x * (int64_t)BIN_TILE + threadIdx.x;
    int sv = -1;
    if (v < n) {
        int32_t d;
        sv = sub_of(indices, v, sb, vgid, gdone, d);
    }
    const unsigned peers = __match_any_sync(FULL, sv);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (sv >= 0 && rank == 0) wc[wid][sv] = __popc(peers);
    __syncthreads();
    if (threadIdx.x < sb.count) {  // exclusive prefix over the warps, per sub-range
        uint32_t run = 0;
        for (int w = 0; w < NW; ++w) {
            const uint32_t x = wc[w][threadIdx.x];
            wc[w][threadIdx.x] = run;
            run += x;
        }
    }
    __syncthreads();
    if (sv >= 0) list[off[sv * ntiles + blockIdx.x] + wc[wid][sv] + rank] = (int32_t)v;
}

// sub-range starts in the class list (first tile of each), and the total
__global__ void k_bins_heads(const uint32_t *__restrict__ off, int64_t ntiles, int32_t subs,
                             const uint32_t *total, int32_t *out) {
    const int s = threadIdx.x;
    if (s < subs) out[s] = (int32_t)off[s * ntiles];
    if (s == subs) out[s] = (int32_t)*total;
}

struct CntLoad {
    const uint32_t *cnt;
    __device__ uint32_t operator()(int64_t i) const { return cnt[i]; }
};
struct CntStore {
    uint32_t *off;
    __device__ void operator()(int64_t i, uint32_t x, uint32_t) const { off[i] = x; }
};

// Classes, and inside the warp and block classes sub-ranges at powers of two
// (warp: 64, 128; block: 512, 1024; large block: 4096), each a stable
// compaction of the vertices with that degree range: one count pass, one
// scan, one scatter pass and one read-back.  The tie buffer is the count
// array (no sweep is in flight while the classes are built).
int launch_bins(pcd_graph *g, cudaStream_t st, bool active_only) {
    int launches = 0;
    const int32_t *vgid = active_only && g->batch ? g->batch->vgid : nullptr;
    const int32_t *gdone = active_only && g->batch ? g->batch->gdone : nullptr;
    std::vector<pcd_graph::SubRange> subs;
    for (int b = 0; b < NBINS; ++b) {
        const int32_t lo = b == 0 ? -1 : g->bins.max_deg[b - 1];
        const int32_t hi = b == NBINS - 1 ? INT_MAX : g->bins.max_deg[b];
        std::vector<int32_t> cuts;
        if (b == BIN_WARP) cuts = {64, 128};
        if (b == BIN_BLOCK) cuts = {512, 1024};
        if (b == BIN_BLOCK_L) cuts = {4096};
        int32_t s_lo = lo;
        for (int32_t c : cuts)
            if (c > lo && c < hi) {
                subs.push_back({b, s_lo, c, 0, 0, 0});
                s_lo = c;
            }
        subs.push_back({b, s_lo, hi, 0, 0, 0});
    }
    SubBounds sb{};
    sb.count = (int32_t)subs.size();
    for (int s = 0; s < sb.count; ++s) {
        sb.lo[s] = subs[(size_t)s].lo;
        sb.hi[s] = subs[(size_t)s].hi;
    }
    const int64_t ntiles = ((int64_t)g->n + BIN_TILE - 1) / BIN_TILE;
    uint32_t *cnt = reinterpret_cast<uint32_t *>(g->tiebuf);  // sb.count * ntiles <= n / 16 + 16 words
    int32_t *d_small = reinterpret_cast<int32_t *>(g->small);  // [0, 16): largest degrees; [16, 33): heads
    cudaMemsetAsync(d_small, 0, MAX_SUBS * sizeof(int32_t), st);
    k_bins_count<<<(unsigned)ntiles, BIN_TILE, 0, st>>>(g->indices, g->n, sb, vgid, gdone, ntiles, cnt, d_small);
    launches += 2 + scan_exclusive(CntLoad{cnt}, CntStore{cnt}, sb.count * ntiles, g->scan, st);
    k_bins_scatter<<<(unsigned)ntiles, BIN_TILE, 0, st>>>(g->indices, g->n, sb, vgid, gdone, ntiles, cnt,
                                                          g->bin_list);
    k_bins_heads<<<1, 32, 0, st>>>(cnt, ntiles, sb.count, g->scan_total, d_small + MAX_SUBS);
    int32_t h[2 * MAX_SUBS + 1] = {0};
    cudaMemcpyAsync(h, d_small, sizeof(int32_t) * (2 * MAX_SUBS + 1), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    for (int b = 0; b < NBINS; ++b) g->bin_maxdeg[b] = 0;
    for (int s = 0; s < sb.count; ++s) {
        auto &r = subs[(size_t)s];
        r.off = h[MAX_SUBS + s];
        r.cnt = h[MAX_SUBS + s + 1] - h[MAX_SUBS + s];
        r.maxdeg = h[s];
        g->bin_maxdeg[r.bin] = std::max(g->bin_maxdeg[r.bin], r.maxdeg);
    }
    g->bin_off[0] = 0;
    for (int b = 0; b < NBINS; ++b) {
        int64_t end = g->bin_off[b];
        for (const auto &r : subs)
            if (r.bin == b) end = r.off + r.cnt;
        g->bin_off[b + 1] = end;
    }
    g->subs = subs;
    return launches;
}

}  // namespace pcd
