// Community merging (MergingRefinement::refine, src/refinement.cpp:185-288)
// and the contracted edge weights it is built on.
//
// Contraction: every directed edge e = (v, u) whose endpoints lie in different
// communities (a, b) emits the key (a, b) with value e, in CSR order; a stable
// LSD radix sort by key followed by a segmented reduce gives one record per
// community pair: the integer weight w(a, b) (the number of such edges) and
// the first edge position, which is where the reference's per-community hash
// table first meets b (members are visited in vertex order and each member's
// row in order, so insertion order = increasing CSR position).  A second sort
// by (a, first position) puts every community's candidates in that insertion
// order.
//
// Matching: each round, one warp per community walks its candidates in order,
// skipping matched communities, with the same running-maximum / tie-count
// analysis as the propagation sweep but the merge tie rule
// (`rand_r % count++`, count from 1, ties tested before improvements,
// src/refinement.cpp:249-257).  Draw positions come from a scan over
// communities in order (the single-threaded round order), rounds continue the
// same rand_r stream, and the final level of ties is replayed to pick each
// community's best partner.  Mutual best partners are matched
// (src/refinement.cpp:264-274) and vertices relabelled to min(l, partner)
// (src/refinement.cpp:277-286).
#include <algorithm>
#include <climits>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

namespace pcd {

static inline int bits_for(int64_t x) {  // bits to hold values 0..x
    int b = 0;
    while (b < 63 && (1ll << b) <= x) ++b;
    return b;
}

// ---------------------------------------------------------------------------
// stable LSD radix sort of (uint64 key, uint32 value), 8-bit digits
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const unsigned long long *__restrict__ keys, int64_t n,
                                                       int shift, int64_t chunk, uint32_t *hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t b = blockIdx.x * chunk, e = min(n, b + chunk);
    for (int64_t i = b + threadIdx.x; i < e; i += RS_THREADS) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    __syncthreads();
    hist[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];  // digit-major
}

struct HistLoad {
    const uint32_t *h;
    __device__ uint32_t operator()(int64_t i) const { return h[i]; }
};
struct HistStore {
    uint32_t *h;
    __device__ void operator()(int64_t i, uint32_t ex, uint32_t) const { h[i] = ex; }
};

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const unsigned long long *__restrict__ keys_in,
                                                          const uint32_t *__restrict__ vals_in,
                                                          unsigned long long *keys_out, uint32_t *vals_out,
                                                          int64_t n, int shift, int64_t chunk,
                                                          const uint32_t *__restrict__ offsets) {
    constexpr int NW = RS_THREADS / 32;
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[NW][256];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    base[threadIdx.x] = offsets[(int64_t)threadIdx.x * gridDim.x + blockIdx.x];
    const int64_t b = blockIdx.x * chunk, e = min(n, b + chunk);
    for (int64_t t0 = b; t0 < e; t0 += RS_THREADS) {
        for (int w = 0; w < NW; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const int64_t i = t0 + threadIdx.x;
        const bool valid = i < e;
        unsigned long long k = 0;
        uint32_t v = 0, dg = 256 + lane;  // invalid lanes: distinct dummy digits
        if (valid) {
            k = keys_in[i];
            v = vals_in[i];
            dg = (uint32_t)((k >> shift) & 255u);
        }
        const unsigned peers = __match_any_sync(FULL, dg);
        const int rank = __popc(peers & lanemask_lt());
        if (valid && lane == __ffs(peers) - 1) wcnt[wid][dg] = __popc(peers);
        __syncthreads();
        // per digit (thread = digit): exclusive over warps, in place
        {
            uint32_t run = 0;
            for (int w = 0; w < NW; ++w) {
                uint32_t c = wcnt[w][threadIdx.x];
                wcnt[w][threadIdx.x] = run;
                run += c;
            }
            __syncthreads();
            if (valid) {
                uint32_t pos = base[dg] + wcnt[wid][dg] + rank;
                keys_out[pos] = k;
                vals_out[pos] = v;
            }
            __syncthreads();
            base[threadIdx.x] += run;
        }
        __syncthreads();
    }
}

// Sorts keys/vals (n items, significant bits [0, bits)); ping-pongs between
// the A and B buffers and returns true if the result ended in B.
bool radix_sort(unsigned long long *ka, uint32_t *va, unsigned long long *kb, uint32_t *vb, int64_t n, int bits,
                uint32_t *hist, const ScanScratch &sc, int grid, cudaStream_t st, int *launches) {
    if (n <= 1 || bits <= 0) return false;
    const int64_t chunk = ((n + grid - 1) / grid + RS_THREADS - 1) / RS_THREADS * RS_THREADS;
    const int g = (int)((n + chunk - 1) / chunk);
    bool inB = false;
    for (int shift = 0; shift < bits; shift += 8) {
        const unsigned long long *ki = inB ? kb : ka;
        const uint32_t *vi = inB ? vb : va;
        unsigned long long *ko = inB ? ka : kb;
        uint32_t *vo = inB ? va : vb;
        k_rs_hist<<<g, RS_THREADS, 0, st>>>(ki, n, shift, chunk, hist);
        *launches += 1 + scan_exclusive(HistLoad{hist}, HistStore{hist}, 256ll * g, sc, st);
        k_rs_scatter<<<g, RS_THREADS, 0, st>>>(ki, vi, ko, vo, n, shift, chunk, hist);
        *launches += 1;
        inB = !inB;
    }
    return inB;
}

// ---------------------------------------------------------------------------
// contraction
// ---------------------------------------------------------------------------
struct ExtLoad {  // inter-community endpoints of v
    const int32_t *indices, *adj, *labels;
    __device__ uint32_t operator()(int64_t v) const {
        const int32_t l = labels[v];
        uint32_t c = 0;
        for (int32_t j = indices[v]; j < indices[v + 1]; ++j) c += labels[adj[j]] != l;
        return c;
    }
};

struct ExtEmit {  // writes key (a << b | c) and value e for each, in row order
    const int32_t *indices, *adj, *labels;
    int b;
    unsigned long long *keys;
    uint32_t *vals;
    __device__ void operator()(int64_t v, uint32_t off, uint32_t cnt) const {
        if (!cnt) return;
        const int32_t l = labels[v];
        for (int32_t j = indices[v]; j < indices[v + 1]; ++j) {
            const int32_t k = labels[adj[j]];
            if (k != l) {
                keys[off] = ((unsigned long long)l << b) | (unsigned long long)k;
                vals[off] = (uint32_t)j;
                ++off;
            }
        }
    }
};

struct HeadLoad {
    const unsigned long long *keys;
    __device__ uint32_t operator()(int64_t i) const { return (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u; }
};

struct HeadStore {  // pair j starts at sorted position i
    const unsigned long long *keys;
    int32_t *ppos;
    __device__ void operator()(int64_t i, uint32_t ex, uint32_t val) const {
        if (val) ppos[ex] = (int32_t)i;
    }
};

__global__ void k_pairs(const unsigned long long *__restrict__ keys, const uint32_t *__restrict__ vals,
                        const int32_t *__restrict__ ppos, int64_t P, int64_t E, int b, int32_t *pa, int32_t *pb,
                        int32_t *pw, int32_t *pfirst) {
    const unsigned long long mask = (1ull << b) - 1;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < P; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = ppos[j];
        const int64_t nx = j + 1 < P ? ppos[j + 1] : E;
        const unsigned long long k = keys[i];
        pa[j] = (int32_t)(k >> b);
        pb[j] = (int32_t)(k & mask);
        pw[j] = (int32_t)(nx - i);
        pfirst[j] = (int32_t)vals[i];  // stable sort: the head holds the smallest edge position
    }
}

__global__ void k_order_keys(const int32_t *__restrict__ pa, const int32_t *__restrict__ pfirst, int64_t P, int be,
                             unsigned long long *keys, uint32_t *vals) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < P; j += (int64_t)gridDim.x * blockDim.x) {
        keys[j] = ((unsigned long long)pa[j] << be) | (unsigned long long)pfirst[j];
        vals[j] = (uint32_t)j;
    }
}

__global__ void k_gather_pairs(const uint32_t *__restrict__ idx, int64_t P, const int32_t *__restrict__ pa,
                               const int32_t *__restrict__ pb, const int32_t *__restrict__ pw, int32_t *oa,
                               int32_t *ob, int32_t *ow) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < P; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = idx[j];
        oa[j] = pa[s];
        ob[j] = pb[s];
        ow[j] = pw[s];
    }
}

__global__ void k_segments(const int32_t *__restrict__ pa, int64_t P, int32_t *seg_start, int32_t *seg_end) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < P; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = pa[j];
        if (j == 0 || pa[j - 1] != a) seg_start[a] = (int32_t)j;
        if (j == P - 1 || pa[j + 1] != a) seg_end[a] = (int32_t)j + 1;
    }
}

// ---------------------------------------------------------------------------
// matching rounds
// ---------------------------------------------------------------------------
struct MergeArgs {
    CommView cm;
    const int32_t *seg_start, *seg_end;
    const int32_t *cb, *cw;  // candidates in insertion order
    int32_t *best;
    int32_t *found;
    uint32_t *ndraw;  // per community: draws this round
    int32_t *tiebuf;  // community l owns [seg_start[l] + l, seg_end[l] + l + 1)
    TieRecord *recs;
    DevCounters *ctr;
    int32_t k;
    const int32_t *cgid;   // batch: graph of each community (else null)
    const int32_t *gdone;  // batch: graphs whose schedule has ended
};

template <class R>
__global__ void __launch_bounds__(256) k_merge_analyze(MergeArgs a, R rule) {
    using E = Elem<double>;
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const double ident = R::identity();
    for (int64_t li = gw; li < a.k; li += nw) {
        const int32_t l = (int32_t)li;
        const int32_t bp = a.best[l];
        const bool active = !a.found[l] && (bp == -1 || a.found[bp]) && !(a.gdone && a.gdone[a.cgid[l]]);
        const R vr = rule.at_comm(l);
        if (!active) {
            if (lane == 0) a.ndraw[l] = 0;
            continue;
        }
        const int32_t s0 = a.seg_start[l], s1 = a.seg_end[l];
        int32_t *ties = a.tiebuf + s0 + l + 1;
        E carry{0.0, -1};
        int32_t holder = -1;
        uint32_t t = 0;
        int32_t r = 0;
        for (int32_t base = s0; base < s1; base += 32) {
            const int32_t i = base + lane;
            const bool valid = i < s1;
            int32_t c = -1, w = 0;
            bool sc = false;
            double key = ident;
            if (valid) {
                c = a.cb[i];
                w = a.cw[i];
                sc = !a.found[c];
                if (sc) {
                    key = vr.merge(l, c, w, a.cm);
                    if (key != key) {  // NaN: neither ties nor wins
                        sc = false;
                        key = ident;
                    }
                }
            }
            const E inc = warp_scan_max<R>(E{key, sc ? i : -2}, lane);
            E ex = shfl_up_any(inc, 1);
            if (lane == 0) ex = E{ident, -2};
            const E pre = combine<R>(carry, ex);
            const bool tie = sc && key == pre.key;
            t += __popc(__ballot_sync(FULL, tie));
            const E nxt = combine<R>(carry, shfl_any(inc, 31));
            if (nxt.ord != carry.ord) {
                r = 0;
                holder = __shfl_sync(FULL, c, nxt.ord - base);
            }
            const bool inrun = tie && pre.ord == nxt.ord;
            const unsigned run = __ballot_sync(FULL, inrun);
            if (inrun) ties[r + __popc(run & lanemask_lt())] = c;
            r += __popc(run);
            carry = nxt;
        }
        if (lane == 0) {
            a.ndraw[l] = t;
            a.best[l] = holder;  // -1 when no candidate beat 0.0
            if (r > 0) {
                a.tiebuf[s0 + l] = holder;
                const int32_t ri = atomicAdd(&a.ctr->n_resolve, 1);
                a.recs[ri] = TieRecord{l, r, (long long)(s0 + l)};
            }
        }
        __syncwarp();
    }
}

__global__ void k_round_reset(DevCounters *ctr) { ctr->n_resolve = 0; }

struct CommDrawLoad {
    const uint32_t *nd;
    __device__ uint32_t operator()(int64_t i) const { return nd[i]; }
};
struct CommDrawStore {
    uint32_t *endpos;
    __device__ void operator()(int64_t i, uint32_t ex, uint32_t v) const { endpos[i] = ex + v; }
};

__global__ void k_round_advance(DevCounters *ctr, const uint32_t *total) { ctr->total_draws += *total; }

// Batch: each graph's draws this round (its communities' span of the scan).
__global__ void k_round_advance_graphs(const int32_t *gK, int32_t G, const uint32_t *endpos, const uint32_t *gbase,
                                       uint32_t *gtotal) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x)
        if (gK[g + 1] > gK[g]) gtotal[g] += endpos[gK[g + 1] - 1] - gbase[g];
}

__global__ void k_found(const int32_t *__restrict__ best, int32_t *found, int32_t k) {
    for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = best[l];
        if (!found[l] && (b == -1 || best[b] == (int32_t)l)) found[l] = 1;
    }
}

__global__ void k_merge_relabel(const int32_t *__restrict__ labels, const int32_t *__restrict__ best,
                                const int32_t *__restrict__ found, int32_t n, int32_t *out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = labels[v];
        const int32_t b = best[l];
        out[v] = (found[l] && b != -1) ? min(l, b) : l;
    }
}

__global__ void k_merge_init(int32_t *best, int32_t *found, int32_t *seg_start, int32_t *seg_end, int32_t k) {
    for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x) {
        best[l] = -1;
        found[l] = 0;
        seg_start[l] = 0;
        seg_end[l] = 0;
    }
}

__global__ void k_set_pairs(DevCounters *ctr, const uint32_t *total) { ctr->n_pairs = (int32_t)*total; }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct MergeBuffers {
    unsigned long long *ka, *kb;
    uint32_t *va, *vb;
    int32_t *ppos, *pa, *pb, *pw, *pfirst;
    int32_t *oa, *ob, *ow;
    int32_t *seg_start, *seg_end, *best, *found, *tiebuf;
    uint32_t *ndraw, *hist;
};

static pcd_status merge_buffers(pcd_graph *g, int64_t E, int64_t k, int grid, MergeBuffers *mb) {
    const int64_t e = std::max<int64_t>(E, 1), kk = std::max<int64_t>(k, 1);
    size_t need = 0;
    auto take = [&](size_t bytes) {
        size_t off = need;
        need += (bytes + 255) & ~size_t(255);
        return off;
    };
    size_t o_ka = take(8 * e), o_kb = take(8 * e), o_va = take(4 * e), o_vb = take(4 * e);
    size_t o_ppos = take(4 * e), o_pa = take(4 * e), o_pb = take(4 * e), o_pw = take(4 * e), o_pf = take(4 * e);
    size_t o_oa = take(4 * e), o_ob = take(4 * e), o_ow = take(4 * e);
    size_t o_ss = take(4 * kk), o_se = take(4 * kk), o_best = take(4 * kk), o_found = take(4 * kk);
    size_t o_tie = take(4 * (e + kk + 1)), o_nd = take(4 * kk), o_hist = take(4ull * 256 * grid);
    if (need > g->merge_bytes) {
        if (g->merge_buf) cudaFreeAsync(g->merge_buf, g->ctx->stream);
        g->merge_buf = nullptr;
        g->merge_bytes = 0;
        cudaError_t err = cudaMallocAsync(&g->merge_buf, need, g->ctx->stream);
        if (err != cudaSuccess) return check_cuda(g->ctx, err, "merge buffers");
        g->merge_bytes = need;
    }
    char *p = (char *)g->merge_buf;
    mb->ka = (unsigned long long *)(p + o_ka);
    mb->kb = (unsigned long long *)(p + o_kb);
    mb->va = (uint32_t *)(p + o_va);
    mb->vb = (uint32_t *)(p + o_vb);
    mb->ppos = (int32_t *)(p + o_ppos);
    mb->pa = (int32_t *)(p + o_pa);
    mb->pb = (int32_t *)(p + o_pb);
    mb->pw = (int32_t *)(p + o_pw);
    mb->pfirst = (int32_t *)(p + o_pf);
    mb->oa = (int32_t *)(p + o_oa);
    mb->ob = (int32_t *)(p + o_ob);
    mb->ow = (int32_t *)(p + o_ow);
    mb->seg_start = (int32_t *)(p + o_ss);
    mb->seg_end = (int32_t *)(p + o_se);
    mb->best = (int32_t *)(p + o_best);
    mb->found = (int32_t *)(p + o_found);
    mb->tiebuf = (int32_t *)(p + o_tie);
    mb->ndraw = (uint32_t *)(p + o_nd);
    mb->hist = (uint32_t *)(p + o_hist);
    return PCD_OK;
}

static unsigned grid_n(int64_t n, int sms) {
    int64_t g = (n + 255) / 256;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sms * 16));
}

struct StoreNone {
    __device__ void operator()(int64_t, uint32_t, uint32_t) const {}
};

static pcd_status read_counters(pcd_graph *g, cudaStream_t st) {
    cudaMemcpyAsync(g->h_ctr, g->ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, st);
    return check_cuda(g->ctx, cudaStreamSynchronize(st), "merge counters");
}

static pcd_status read_total(pcd_graph *g, cudaStream_t st, uint32_t *out) {
    cudaMemcpyAsync(out, g->scan_total, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    return check_cuda(g->ctx, cudaStreamSynchronize(st), "merge total");
}

// Builds the contracted pairs of the current compressed partition: on return
// mb->pa / pb / pw / pfirst hold the P pairs sorted by (a, b).
static pcd_status contract(pcd_graph *g, cudaStream_t st, MergeBuffers *mb, int64_t *P_out, int32_t *k_out,
                           int *launches) {
    pcd_ctx *ctx = g->ctx;
    const int grid = ctx->num_sms * 2;
    pcd_status s = read_counters(g, st);
    if (s != PCD_OK) return s;
    const int32_t k = g->h_ctr->k;
    *k_out = k;
    // inter-community endpoints
    const ExtLoad ext{g->indices, g->adj, g->labels};
    *launches += scan_exclusive(ext, StoreNone{}, g->n, g->scan, st);
    uint32_t E32 = 0;
    if ((s = read_total(g, st, &E32)) != PCD_OK) return s;
    const int64_t E = E32;
    if ((s = merge_buffers(g, E, k, grid, mb)) != PCD_OK) return s;
    if (E == 0) {
        *P_out = 0;
        return PCD_OK;
    }
    const int b = std::max(1, bits_for((int64_t)k - 1));
    *launches += scan_exclusive(ext, ExtEmit{g->indices, g->adj, g->labels, b, mb->ka, mb->va}, g->n, g->scan, st);
    const bool inB = radix_sort(mb->ka, mb->va, mb->kb, mb->vb, E, 2 * b, mb->hist, g->scan,
                                grid, st, launches);
    const unsigned long long *keys = inB ? mb->kb : mb->ka;
    const uint32_t *vals = inB ? mb->vb : mb->va;
    *launches += scan_exclusive(HeadLoad{keys}, HeadStore{keys, mb->ppos}, E, g->scan, st);
    uint32_t P32 = 0;
    if ((s = read_total(g, st, &P32)) != PCD_OK) return s;
    const int64_t P = P32;
    k_pairs<<<grid_n(P, ctx->num_sms), 256, 0, st>>>(keys, vals, mb->ppos, P, E, b, mb->pa, mb->pb, mb->pw,
                                                    mb->pfirst);
    *launches += 1;
    *P_out = P;
    return check_cuda(ctx, cudaGetLastError(), "contract");
}

pcd_status run_contract(pcd_graph *g, int64_t cap, int32_t *a, int32_t *b, int32_t *w, int64_t *num_pairs,
                        cudaStream_t st) {
    MergeBuffers mb;
    int64_t P = 0;
    int32_t k = 0;
    int launches = 0;
    pcd_status s = contract(g, st, &mb, &P, &k, &launches);
    if (s != PCD_OK) return s;
    const int64_t c = std::min(cap, P);
    if (c > 0) {
        cudaMemcpyAsync(a, mb.pa, sizeof(int32_t) * c, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(b, mb.pb, sizeof(int32_t) * c, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(w, mb.pw, sizeof(int32_t) * c, cudaMemcpyDeviceToHost, st);
    }
    s = check_cuda(g->ctx, cudaStreamSynchronize(st), "contract copy");
    *num_pairs = P;
    return s;
}

__global__ void k_merge_reset(DevCounters *ctr, const uint32_t *npairs) {
    ctr->total_draws = 0;
    ctr->n_resolve = 0;
    ctr->n_pairs = npairs ? (int32_t)*npairs : 0;
}

template <class R>
static void merge_rounds(pcd_graph *g, const MergeArgs &ma, const R &rule, int32_t rounds, uint32_t seed,
                         cudaStream_t st, int *launches) {
    const int sms = g->ctx->num_sms;
    const int64_t k = ma.k;
    const unsigned wgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((k + 7) / 8, (int64_t)sms * 16));
    for (int32_t rnd = 0; rnd < rounds; ++rnd) {
        k_round_reset<<<1, 1, 0, st>>>(g->ctr);
        k_merge_analyze<R><<<wgrid, 256, 0, st>>>(ma, rule);
        *launches += 2;
        *launches += scan_exclusive(CommDrawLoad{ma.ndraw}, CommDrawStore{ma.ndraw}, k, g->scan, st);
        BatchState *B = g->batch;
        if (B) {
            launch_graph_base(B->gK, B->G, ma.ndraw, B->gbase, st);
            launch_resolve(ma.recs, g->ctr, ma.ndraw, nullptr, ma.tiebuf, ma.best, seed, 1, sms * 4, st, B->cgid,
                           B->gseed, B->gbase, B->gtotal);
            k_round_advance_graphs<<<(B->G + 255) / 256, 256, 0, st>>>(B->gK, B->G, ma.ndraw, B->gbase, B->gtotal);
            *launches += 3;
        } else {
            launch_resolve(ma.recs, g->ctr, ma.ndraw, &g->ctr->total_draws, ma.tiebuf, ma.best, seed, 1, sms * 4,
                           st);
        }
        k_round_advance<<<1, 1, 0, st>>>(g->ctr, g->scan_total);
        k_found<<<grid_n(k, sms), 256, 0, st>>>(ma.best, ma.found, (int32_t)k);
        *launches += 3;
    }
}

pcd_status run_merge(pcd_graph *g, int32_t kind, double lambda, int32_t rounds, uint32_t seed, cudaStream_t st,
                     int *launches) {
    pcd_ctx *ctx = g->ctx;
    const int sms = ctx->num_sms;
    MergeBuffers mb;
    int64_t P = 0;
    int32_t k = 0;
    pcd_status s = contract(g, st, &mb, &P, &k, launches);
    if (s != PCD_OK) return s;
    // candidates of each community in insertion order
    const int b = std::max(1, bits_for((int64_t)k - 1));
    const int be = std::max(1, bits_for(g->nnz));
    k_merge_init<<<grid_n(k, sms), 256, 0, st>>>(mb.best, mb.found, mb.seg_start, mb.seg_end, k);
    *launches += 1;
    if (P > 0) {
        k_order_keys<<<grid_n(P, sms), 256, 0, st>>>(mb.pa, mb.pfirst, P, be, mb.ka, mb.va);
        const bool inB = radix_sort(mb.ka, mb.va, mb.kb, mb.vb, P, b + be, mb.hist, g->scan,
                                    sms * 2, st, launches);
        k_gather_pairs<<<grid_n(P, sms), 256, 0, st>>>(inB ? mb.vb : mb.va, P, mb.pa, mb.pb, mb.pw, mb.oa, mb.ob,
                                                       mb.ow);
        k_segments<<<grid_n(P, sms), 256, 0, st>>>(mb.oa, P, mb.seg_start, mb.seg_end);
        *launches += 3;
    }
    k_merge_reset<<<1, 1, 0, st>>>(g->ctr, nullptr);
    *launches += 1;
    MergeArgs ma;
    ma.cm = CommView{g->sizes, g->intv, g->extv, g->vol};
    ma.seg_start = mb.seg_start;
    ma.seg_end = mb.seg_end;
    ma.cb = mb.ob;
    ma.cw = mb.ow;
    ma.best = mb.best;
    ma.found = mb.found;
    ma.ndraw = mb.ndraw;
    ma.tiebuf = mb.tiebuf;
    ma.recs = g->recs;
    ma.ctr = g->ctr;
    ma.k = k;
    BatchState *B = g->batch;
    ma.cgid = B ? B->cgid : nullptr;
    ma.gdone = B ? B->gdone : nullptr;
    const BatchView bv = B ? BatchView{B->vgid, B->cgid, B->gm, B->gcc} : BatchView{};
    if (B) cudaMemsetAsync(B->gtotal, 0, sizeof(uint32_t) * B->G, st);
    if (kind == PCD_RULE_MODULARITY) {
        RuleModF64 r;
        r.m = g->m;
        r.bv = bv;
        merge_rounds(g, ma, r, rounds, seed, st, launches);
    } else if (kind == PCD_RULE_CPM) {
        RuleCPM r;
        r.lambda = lambda;
        r.bv = bv;
        merge_rounds(g, ma, r, rounds, seed, st, launches);
    } else {
        RuleWCC r;
        r.cc = g->cc;
        r.bv = bv;
        merge_rounds(g, ma, r, rounds, seed, st, launches);
    }
    k_merge_relabel<<<grid_n(g->n, sms), 256, 0, st>>>(g->labels, mb.best, mb.found, g->n, g->labels_alt);
    *launches += 1;
    g->info.merge_pairs = (int32_t)P;
    return check_cuda(ctx, cudaGetLastError(), "merge");
}

}  // namespace pcd
