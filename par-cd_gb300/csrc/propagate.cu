// One synchronous label-propagation sweep (PropagationRefinement::refine,
// src/refinement.cpp:114-182), bit-exact with the reference's -p 1 schedule.
//
// Per vertex v the reference builds the histogram of its neighbours' labels
// in first-occurrence order (FastHashTable iterates in insertion order,
// src/refinement.cpp:24-110), scores every label but its own in that order,
// keeps the first candidate of the running maximum (starting from 0.0) and
// draws rand_r once for every candidate that EQUALS the running maximum
// (reservoir sampling, :158-161), after one rand_r draw for the frac test
// (:129).  The number of draws of v does not depend on the random values, so
// the sweep runs in three passes:
//   1. candidate analysis (degree-binned kernels: thread / warp / block per
//      vertex with a shared-memory hash, hubs with their table in HBM):
//      per vertex the draw count t(v), the decision, and -- when the winner is
//      drawn among ties -- the holder plus the final level's ties in order;
//   2. an exclusive scan of 1 + t(v) over vertices (their -p 1 order) gives
//      every vertex its position in the single rand_r stream;
//   3. replay: jump the LCG to that position and redo the reservoir draws of
//      the final level (the last r draws of v) to pick the winner.
// With frac < 1 the frac test decides whether v draws at all, so step 2
// becomes a sequential walk of the stream (k_walk).
//
// Modularity is analysed with the exact integer key of RuleModInt; vertices
// whose outcome the key cannot decide are queued and re-analysed in FP64.
#include <climits>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

namespace pcd {

__constant__ JumpTable c_jump;

// State after `calls` rand_r calls starting from `seed` (calls taken mod 2^32:
// the LCG has period 2^32 and 3 is odd, so the call stream has period 2^32).
__device__ __forceinline__ uint32_t rand_r_jump(uint32_t seed, uint32_t calls) {
    uint32_t x = seed;
#pragma unroll 1
    for (int i = 0; calls; ++i, calls >>= 1)
        if (calls & 1u) x = c_jump.a[i] * x + c_jump.c[i];
    return x;
}

void upload_jump_table(cudaStream_t st) {
    JumpTable t;
    // one call: three steps of x -> 1103515245 x + 12345
    uint32_t a = 1, c = 0;
    for (int s = 0; s < 3; ++s) {
        c = 1103515245u * c + 12345u;
        a = 1103515245u * a;
    }
    for (int i = 0; i < 32; ++i) {
        t.a[i] = a;
        t.c[i] = c;
        c = a * c + c;
        a = a * a;
    }
    cudaMemcpyToSymbolAsync(c_jump, &t, sizeof(t), 0, cudaMemcpyHostToDevice, st);
}

struct SweepArgs {
    GraphView g;
    CommView cm;
    const int32_t *__restrict__ labels;
    int32_t *new_labels;
    uint32_t *ndraw;
    int32_t *tiebuf;
    long long tiebuf_cap;
    TieRecord *recs;
    int32_t *amb;
    DevCounters *ctr;
};

// ---------------------------------------------------------------------------
// output of one analysed vertex
// ---------------------------------------------------------------------------
__device__ __forceinline__ void push_ambiguous(const SweepArgs &a, int32_t v) {
    int32_t i = atomicAdd(&a.ctr->n_ambiguous, 1);
    a.amb[i] = v;
}

// Allocates the tie record of a MOVE vertex with r >= 1 ties; returns the
// buffer offset (or -1 on overflow, flagged).
__device__ __forceinline__ long long alloc_ties(const SweepArgs &a, int32_t v, int32_t r, int32_t holder) {
    unsigned long long off = atomicAdd(&a.ctr->tie_used, (unsigned long long)(r + 1));
    if ((long long)(off + r + 1) > a.tiebuf_cap) {
        atomicOr(&a.ctr->error, ERR_TIEBUF_OVERFLOW);
        return -1;
    }
    a.tiebuf[off] = holder;
    int32_t ri = atomicAdd(&a.ctr->n_resolve, 1);
    a.recs[ri] = TieRecord{v, r, (long long)off};
    return (long long)off;
}

__device__ __forceinline__ void write_decision(const SweepArgs &a, int32_t v, int32_t dec, int32_t holder,
                                               int32_t curr) {
    a.new_labels[v] = dec == DEC_MOVE ? holder : (dec == DEC_NEW ? -1 : curr);
}

// ---------------------------------------------------------------------------
// thread per vertex (deg <= CAP): the reference loop, one vertex per thread,
// candidates in a per-thread slice of shared memory (stride blockDim).
// ---------------------------------------------------------------------------
template <class R, int CAP>
__global__ void __launch_bounds__(128) k_prop_thread(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                     int64_t count) {
    extern __shared__ int32_t smem[];
    const int T = blockDim.x;
    int32_t *cl = smem + threadIdx.x;
    int32_t *cc = smem + T * CAP + threadIdx.x;
    using Key = typename R::Key;
    for (int64_t idx = blockIdx.x * (int64_t)T + threadIdx.x; idx < count; idx += (int64_t)gridDim.x * T) {
        const int32_t v = list[idx];
        const int32_t b = a.g.indices[v], e = a.g.indices[v + 1], d = e - b;
        const int32_t curr = a.labels[v];
        if (rule.vertex_ambiguous(d)) {
            push_ambiguous(a, v);
            continue;
        }
        int32_t nc = 0;
        for (int32_t j = b; j < e; ++j) {
            int32_t l = a.labels[a.g.adj[j]];
            int32_t i = 0;
            while (i < nc && cl[i * T] != l) ++i;
            if (i < nc) {
                cc[i * T] += 1;
            } else {
                cl[nc * T] = l;
                cc[nc * T] = 1;
                ++nc;
            }
        }
        Key M = R::initial();
        bool has = false, amb = false;
        int32_t hl = -1, r = 0, curr_freq = 0;
        uint32_t t = 0;
        for (int32_t i = 0; i < nc; ++i) {
            int32_t l = cl[i * T], k = cc[i * T];
            if (l == curr) {
                curr_freq = k;
                continue;
            }
            Key s = rule.join(v, d, l, k, a.cm);
            if (!R::usable(s)) continue;
            if (R::gt(s, M)) {
                M = s;
                hl = l;
                has = true;
                r = 0;
            } else if (R::eq(s, M)) {
                ++t;
                amb |= R::ambiguous_tie(s, M, has);
                cl[r * T] = l;  // r <= i: candidate r was already read
                ++r;
            }
        }
        if (amb) {
            push_ambiguous(a, v);
            continue;
        }
        int32_t dec = rule.decide(M, has, v, d, curr, curr_freq, a.cm);
        if (dec == DEC_AMBIGUOUS) {
            push_ambiguous(a, v);
            continue;
        }
        a.ndraw[v] = t;
        write_decision(a, v, dec, hl, curr);
        if (dec == DEC_MOVE && r > 0) {
            long long off = alloc_ties(a, v, r, hl);
            if (off >= 0)
                for (int32_t j = 0; j < r; ++j) a.tiebuf[off + 1 + j] = cl[j * T];
        }
    }
}

// ---------------------------------------------------------------------------
// warp per vertex (deg <= WCAP): adjacency in chunks of 32 in order; lanes
// holding the same label are merged with match_any and the lowest lane (the
// first occurrence) inserts; new labels get consecutive ordinals in lane
// order, so ordinals are first-occurrence order.  Then an ordered warp scan
// of the gains with the running maximum carried across chunks.
// ---------------------------------------------------------------------------
template <class R, int WCAP>
__global__ void __launch_bounds__(256) k_prop_warp(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                   int64_t count) {
    constexpr int TS = 2 * WCAP;
    extern __shared__ int32_t smem[];
    using Key = typename R::Key;
    using E = Elem<Key>;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t *keys = smem + wid * (2 * TS + 3 * WCAP);
    int32_t *ords = keys + TS;
    int32_t *clab = ords + TS;
    int32_t *ccnt = clab + WCAP;
    int32_t *ties = ccnt + WCAP;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t idx = gw; idx < count; idx += nw) {
        const int32_t v = list[idx];
        const int32_t b = a.g.indices[v], e = a.g.indices[v + 1], d = e - b;
        const int32_t curr = a.labels[v];
        if (rule.vertex_ambiguous(d)) {
            if (lane == 0) push_ambiguous(a, v);
            continue;
        }
        for (int i = lane; i < TS; i += 32) keys[i] = -1;
        __syncwarp();
        int32_t nc = 0;
        for (int32_t base = b; base < e; base += 32) {
            const int32_t j = base + lane;
            const bool valid = j < e;
            const int32_t l = valid ? a.labels[a.g.adj[j]] : -2;
            const unsigned peers = __match_any_sync(FULL, l);
            const bool leader = valid && lane == __ffs(peers) - 1;
            bool isnew = false;
            uint32_t h = 0;
            if (leader) {
                h = hash_label(l) & (TS - 1);
                for (;;) {
                    int32_t kk = keys[h];
                    if (kk == l) break;
                    if (kk == -1) {
                        int32_t old = atomicCAS(&keys[h], -1, l);
                        if (old == -1) {
                            isnew = true;
                            break;
                        }
                        if (old == l) break;
                    }
                    h = (h + 1) & (TS - 1);
                }
            }
            const unsigned newmask = __ballot_sync(FULL, isnew);
            if (isnew) {
                int32_t ord = nc + __popc(newmask & lanemask_lt());
                ords[h] = ord;
                clab[ord] = l;
                ccnt[ord] = __popc(peers);
            }
            __syncwarp();
            if (leader && !isnew) ccnt[ords[h]] += __popc(peers);
            nc += __popc(newmask);
            __syncwarp();
        }
        // ordered scoring
        E carry{R::initial(), -1, -1};
        uint32_t t = 0;
        int32_t r = 0, my_curr = 0;
        bool amb = false;
        for (int32_t base = 0; base < nc; base += 32) {
            const int32_t i = base + lane;
            const bool valid = i < nc;
            const int32_t l = valid ? clab[i] : -1;
            const int32_t k = valid ? ccnt[i] : 0;
            const bool is_curr = valid && l == curr;
            if (is_curr) my_curr = k;
            bool sc = valid && !is_curr;
            Key key = R::identity();
            if (sc) {
                key = rule.join(v, d, l, k, a.cm);
                if (!R::usable(key)) {
                    sc = false;
                    key = R::identity();
                }
            }
            E x{key, sc ? i : -2, l};
            E inc = warp_scan_max<R>(x, lane);
            E ex = shfl_up_any(inc, 1);
            if (lane == 0) ex = E{R::identity(), -2, -1};
            E pre = combine<R>(carry, ex);
            const bool tie = sc && R::eq(key, pre.key);
            if (tie && R::ambiguous_tie(key, pre.key, pre.ord >= 0)) amb = true;
            t += __popc(__ballot_sync(FULL, tie));
            E tot = shfl_any(inc, 31);
            E nxt = combine<R>(carry, tot);
            if (nxt.ord != carry.ord) r = 0;
            const bool inrun = tie && pre.ord == nxt.ord;
            const unsigned run = __ballot_sync(FULL, inrun);
            if (inrun) ties[r + __popc(run & lanemask_lt())] = l;
            r += __popc(run);
            carry = nxt;
        }
        __syncwarp();
        amb = __any_sync(FULL, amb);
        const int32_t curr_freq = __reduce_add_sync(FULL, my_curr);
        if (amb) {
            if (lane == 0) push_ambiguous(a, v);
            continue;
        }
        const bool has = carry.ord >= 0;
        const int32_t dec = rule.decide(carry.key, has, v, d, curr, curr_freq, a.cm);
        if (dec == DEC_AMBIGUOUS) {
            if (lane == 0) push_ambiguous(a, v);
            continue;
        }
        long long off = -1;
        if (lane == 0) {
            a.ndraw[v] = t;
            write_decision(a, v, dec, carry.label, curr);
            if (dec == DEC_MOVE && r > 0) off = alloc_ties(a, v, r, carry.label);
        }
        off = __shfl_sync(FULL, off, 0);
        if (off >= 0)
            for (int32_t j = lane; j < r; j += 32) a.tiebuf[off + 1 + j] = ties[j];
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// block per vertex.  Table (key, count, first position) with atomicMin on the
// first position; then position -> slot, and an ordered block scan over
// positions (empty positions are identity) reproduces insertion order.
// The table lives in shared memory (block bins) or in a per-block HBM slice
// (hubs, FP64 re-evaluation).
// ---------------------------------------------------------------------------
template <class R>
struct BlockScratch {
    Elem<typename R::Key> warp_tot[32];
    Elem<typename R::Key> blk_total;
    Elem<typename R::Key> run_carry;
    int32_t warp_cnt[32];
    int32_t r;
    uint32_t t;
    int32_t amb;
    int32_t curr_freq;
    long long off;
};

// Block-wide running-max scan (keep-left).  Returns this thread's exclusive
// prefix; *total receives the block aggregate.  Contains __syncthreads.
template <class R>
__device__ __forceinline__ Elem<typename R::Key> block_scan_max(Elem<typename R::Key> x, BlockScratch<R> &s,
                                                                Elem<typename R::Key> *total) {
    using E = Elem<typename R::Key>;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    E inc = warp_scan_max<R>(x, lane);
    E ex = shfl_up_any(inc, 1);
    if (lane == 0) ex = E{R::identity(), -2, -1};
    if (lane == 31) s.warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        E wt = lane < nw ? s.warp_tot[lane] : E{R::identity(), -2, -1};
        E wi = warp_scan_max<R>(wt, lane);
        E we = shfl_up_any(wi, 1);
        if (lane == 0) we = E{R::identity(), -2, -1};
        if (lane < nw) s.warp_tot[lane] = we;
        if (lane == 31) s.blk_total = wi;
    }
    __syncthreads();
    E res = combine<R>(s.warp_tot[wid], ex);
    *total = s.blk_total;
    __syncthreads();
    return res;
}

// Exclusive count of `f` over the block in thread order.  Contains __syncthreads.
__device__ __forceinline__ int block_excl_count(bool f, int32_t *warp_cnt, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned m = __ballot_sync(FULL, f);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    int before = 0, tot = 0;
    for (int w = 0; w < nw; ++w) {
        int c = warp_cnt[w];
        before += w < wid ? c : 0;
        tot += c;
    }
    __syncthreads();
    *total = tot;
    return before + __popc(m & lanemask_lt());
}

template <class R, bool GLOBAL>
__global__ void k_prop_block(SweepArgs a, R rule, const int32_t *__restrict__ list, int64_t count,
                             const int32_t *count_dev, int32_t table_cap, int32_t *gscratch, int64_t gstride) {
    using Key = typename R::Key;
    using E = Elem<Key>;
    extern __shared__ int32_t smem[];
    __shared__ BlockScratch<R> s;
    int32_t *keys = GLOBAL ? gscratch + (int64_t)blockIdx.x * gstride : smem;
    int32_t *cnts = keys + table_cap;
    int32_t *fpos = cnts + table_cap;
    int32_t *posarr = fpos + table_cap;  // position -> slot; reused for the tie list
    if (count_dev) count = *count_dev;
    const int tid = threadIdx.x, BT = blockDim.x, lane = threadIdx.x & 31;
    for (int64_t vi = blockIdx.x; vi < count; vi += gridDim.x) {
        const int32_t v = list[vi];
        const int32_t b = a.g.indices[v], e = a.g.indices[v + 1], d = e - b;
        const int32_t curr = a.labels[v];
        if (rule.vertex_ambiguous(d)) {
            if (tid == 0) push_ambiguous(a, v);
            continue;
        }
        int32_t ts = 64;
        while (ts < 2 * d) ts <<= 1;
        if (ts > table_cap) {  // a vertex binned past its table: never expected
            if (tid == 0) atomicOr(&a.ctr->error, ERR_SCRATCH_OVERFLOW);
            continue;
        }
        for (int32_t i = tid; i < ts; i += BT) {
            keys[i] = -1;
            cnts[i] = 0;
            fpos[i] = INT_MAX;
        }
        for (int32_t p = tid; p < d; p += BT) posarr[p] = -1;
        if (tid == 0) {
            s.run_carry = E{R::initial(), -1, -1};
            s.r = 0;
            s.t = 0;
            s.amb = 0;
            s.curr_freq = 0;
        }
        __syncthreads();
        // histogram with first positions
        for (int32_t p0 = 0; p0 < d; p0 += BT) {
            const int32_t p = p0 + tid;
            const bool valid = p < d;
            const int32_t l = valid ? a.labels[a.g.adj[b + p]] : -2;
            const unsigned peers = __match_any_sync(FULL, l);
            if (valid && lane == __ffs(peers) - 1) {
                uint32_t h = hash_label(l) & (uint32_t)(ts - 1);
                for (;;) {
                    int32_t kk = keys[h];
                    if (kk == l) break;
                    if (kk == -1) {
                        int32_t old = atomicCAS(&keys[h], -1, l);
                        if (old == -1 || old == l) break;
                    }
                    h = (h + 1) & (uint32_t)(ts - 1);
                }
                atomicAdd(&cnts[h], __popc(peers));
                atomicMin(&fpos[h], p);  // leader = lowest lane = first position of the group
            }
        }
        __syncthreads();
        for (int32_t i = tid; i < ts; i += BT)
            if (keys[i] != -1) posarr[fpos[i]] = i;
        __syncthreads();
        // ordered scoring over positions
        for (int32_t p0 = 0; p0 < d; p0 += BT) {
            const int32_t p = p0 + tid;
            const int32_t slot = p < d ? posarr[p] : -1;
            const bool valid = slot >= 0;
            const int32_t l = valid ? keys[slot] : -1;
            const int32_t k = valid ? cnts[slot] : 0;
            const bool is_curr = valid && l == curr;
            if (is_curr) s.curr_freq = k;
            bool sc = valid && !is_curr;
            Key key = R::identity();
            if (sc) {
                key = rule.join(v, d, l, k, a.cm);
                if (!R::usable(key)) {
                    sc = false;
                    key = R::identity();
                }
            }
            E tot;
            const E ex = block_scan_max<R>(E{key, sc ? p : -2, l}, s, &tot);  // all posarr reads are done
            const E carry = s.run_carry;
            const E pre = combine<R>(carry, ex);
            const bool tie = sc && R::eq(key, pre.key);
            if (tie && R::ambiguous_tie(key, pre.key, pre.ord >= 0)) s.amb = 1;
            const unsigned tm = __ballot_sync(FULL, tie);
            if (lane == 0 && tm) atomicAdd(&s.t, (uint32_t)__popc(tm));
            const E nxt = combine<R>(carry, tot);
            const bool inrun = tie && pre.ord == nxt.ord;
            int run_total;
            const int rank = block_excl_count(inrun, s.warp_cnt, &run_total);
            const int32_t r0 = nxt.ord != carry.ord ? 0 : s.r;
            // r0 + rank < candidates seen so far <= p0 + BT: only positions already read are overwritten
            if (inrun) posarr[r0 + rank] = l;
            __syncthreads();
            if (tid == 0) {
                s.r = r0 + run_total;
                s.run_carry = nxt;
            }
            __syncthreads();
        }
        if (tid == 0) {
            s.off = -1;
            const E c = s.run_carry;
            int32_t dec = DEC_AMBIGUOUS;
            if (!s.amb) dec = rule.decide(c.key, c.ord >= 0, v, d, curr, s.curr_freq, a.cm);
            if (dec == DEC_AMBIGUOUS) {
                push_ambiguous(a, v);
            } else {
                a.ndraw[v] = s.t;
                write_decision(a, v, dec, c.label, curr);
                if (dec == DEC_MOVE && s.r > 0) s.off = alloc_ties(a, v, s.r, c.label);
            }
        }
        __syncthreads();
        const long long off = s.off;
        const int32_t r = s.r;
        if (off >= 0)
            for (int32_t j = tid; j < r; j += BT) a.tiebuf[off + 1 + j] = posarr[j];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// stream positions
// ---------------------------------------------------------------------------
struct DrawLoad {
    const uint32_t *ndraw;
    __device__ uint32_t operator()(int64_t v) const { return 1u + ndraw[v]; }
};
struct DrawStore {
    uint32_t *endpos;
    __device__ void operator()(int64_t v, uint32_t ex, uint32_t val) const { endpos[v] = ex + val; }
};

__global__ void k_total_draws(DevCounters *ctr, const uint32_t *total) { ctr->total_draws = *total; }

// frac < 1: whether v draws its ties depends on its frac draw, which depends
// on every earlier vertex's draw count, so one thread walks the stream in
// vertex order (src/refinement.cpp:127-132 with one thread).
__global__ void k_walk(uint32_t seed, int32_t f, int32_t n, uint32_t *ndraw, const int32_t *__restrict__ labels,
                       int32_t *new_labels, int32_t *skip, DevCounters *ctr) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t x = seed, pos = 0;
    for (int32_t v = 0; v < n; ++v) {
        int32_t val = rand_r_dev(x);
        pos += 1;
        uint32_t t = ndraw[v];
        if (val > f) {
            skip[v] = 1;
            new_labels[v] = labels[v];
        } else {
            skip[v] = 0;
            if (t < 8) {
                for (uint32_t j = 0; j < t; ++j) (void)rand_r_dev(x);
            } else {
                x = rand_r_jump(x, t);
            }
            pos += t;
        }
        ndraw[v] = pos;
    }
    ctr->total_draws = pos;
}

// Replay the final level of ties of each recorded vertex/community: the j-th
// tie (0-based) replaces the holder when rand_r % (j + mod_base) == 0.
// Propagation: mod_base 2 (src/refinement.cpp:159, ++best_count from 1);
// merging: mod_base 1 (src/refinement.cpp:250, count++ from 1).
__global__ void k_resolve(const TieRecord *__restrict__ recs, const DevCounters *ctr,
                          const uint32_t *__restrict__ endpos, const uint32_t *base,
                          const int32_t *__restrict__ tiebuf, int32_t *out, uint32_t seed, int32_t mod_base,
                          const int32_t *skip) {
    const int32_t nrec = ctr->n_resolve;
    const uint32_t b0 = base ? *base : 0u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrec; i += (int64_t)gridDim.x * blockDim.x) {
        const TieRecord rec = recs[i];
        if (skip && skip[rec.v]) continue;
        uint32_t x = rand_r_jump(seed, b0 + endpos[rec.v] - (uint32_t)rec.r);
        int32_t best = tiebuf[rec.off];
        for (int32_t j = 0; j < rec.r; ++j) {
            int32_t val = rand_r_dev(x);
            if (val % (j + mod_base) == 0) best = tiebuf[rec.off + 1 + j];
        }
        out[rec.v] = best;
    }
}

__global__ void k_reset_sweep(DevCounters *ctr) {
    ctr->tie_used = 0;
    ctr->n_resolve = 0;
    ctr->n_ambiguous = 0;
    ctr->error = 0;
    ctr->total_draws = 0;
}

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------
constexpr int THREAD_CAP = 16;
constexpr int WARP_CAP = 128;
constexpr int BLOCK_CAP = 1024;    // table 2048
constexpr int BLOCK_L_CAP = 4096;  // table 8192

static inline unsigned cap_grid(int64_t want, int64_t cap) {
    if (want < 1) want = 1;
    return (unsigned)(want < cap ? want : cap);
}

template <class R>
static int launch_bins_rule(pcd_graph *g, const SweepArgs &a, const R &rule, cudaStream_t st) {
    const int sms = g->ctx->num_sms;
    int launches = 0;
    const int32_t *L = g->bin_list;
    int64_t c;
    if ((c = g->bin_off[BIN_THREAD + 1] - g->bin_off[BIN_THREAD]) > 0) {
        size_t smem = 2ull * 128 * THREAD_CAP * sizeof(int32_t);
        k_prop_thread<R, THREAD_CAP><<<cap_grid((c + 127) / 128, sms * 16), 128, smem, st>>>(
            a, rule, L + g->bin_off[BIN_THREAD], c);
        ++launches;
        prof_mark(g->ctx, "sweep.thread", st);
    }
    if ((c = g->bin_off[BIN_WARP + 1] - g->bin_off[BIN_WARP]) > 0) {
        size_t smem = 8ull * (2 * 2 * WARP_CAP + 3 * WARP_CAP) * sizeof(int32_t);
        k_prop_warp<R, WARP_CAP><<<cap_grid((c + 7) / 8, sms * 8), 256, smem, st>>>(a, rule,
                                                                                L + g->bin_off[BIN_WARP], c);
        ++launches;
        prof_mark(g->ctx, "sweep.warp", st);
    }
    if ((c = g->bin_off[BIN_BLOCK + 1] - g->bin_off[BIN_BLOCK]) > 0) {
        size_t smem = (3ull * 2 * BLOCK_CAP + BLOCK_CAP) * sizeof(int32_t);
        k_prop_block<R, false><<<cap_grid(c, sms * 6), 256, smem, st>>>(
            a, rule, L + g->bin_off[BIN_BLOCK], c, nullptr, 2 * BLOCK_CAP, nullptr, 0);
        ++launches;
        prof_mark(g->ctx, "sweep.block", st);
    }
    if ((c = g->bin_off[BIN_BLOCK_L + 1] - g->bin_off[BIN_BLOCK_L]) > 0) {
        size_t smem = (3ull * 2 * BLOCK_L_CAP + BLOCK_L_CAP) * sizeof(int32_t);
        cudaFuncSetAttribute(k_prop_block<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_prop_block<R, false><<<cap_grid(c, sms * 2), 512, smem, st>>>(
            a, rule, L + g->bin_off[BIN_BLOCK_L], c, nullptr, 2 * BLOCK_L_CAP, nullptr, 0);
        ++launches;
        prof_mark(g->ctx, "sweep.block_l", st);
    }
    if ((c = g->bin_off[BIN_HUB + 1] - g->bin_off[BIN_HUB]) > 0) {
        k_prop_block<R, true><<<cap_grid(c, g->hub_blocks), 512, 0, st>>>(
            a, rule, L + g->bin_off[BIN_HUB], c, nullptr, (int32_t)g->hub_slots, g->hub_scratch,
            3 * g->hub_slots + g->max_deg);
        ++launches;
        prof_mark(g->ctx, "sweep.hub", st);
    }
    return launches;
}

void propagate_configure(pcd_ctx *) {}

int launch_refine(pcd_graph *g, int32_t kind, double lambda, double frac, uint32_t seed, cudaStream_t st) {
    int launches = 0;
    SweepArgs a;
    a.g = GraphView{g->n, g->m, g->indices, g->adj, g->tri, g->tri_deg, g->cc};
    a.cm = CommView{g->sizes, g->intv, g->extv, g->vol};
    a.labels = g->labels;
    a.new_labels = g->labels_alt;
    a.ndraw = g->ndraw;
    a.tiebuf = g->tiebuf;
    a.tiebuf_cap = g->tiebuf_cap;
    a.recs = g->recs;
    a.amb = g->amb;
    a.ctr = g->ctr;
    k_reset_sweep<<<1, 1, 0, st>>>(g->ctr);
    ++launches;
    prof_mark(g->ctx, "sweep.reset", st);
    if (kind == PCD_RULE_MODULARITY) {
        RuleModInt r;
        r.m = g->m;
        r.two_m = 2LL * g->m;
        launches += launch_bins_rule(g, a, r, st);
        RuleModF64 rf;
        rf.m = g->m;
        k_prop_block<RuleModF64, true><<<g->hub_blocks, 512, 0, st>>>(
            a, rf, g->amb, 0, &g->ctr->n_ambiguous, (int32_t)g->hub_slots, g->hub_scratch,
            3 * g->hub_slots + g->max_deg);
        ++launches;
        prof_mark(g->ctx, "sweep.fp64_recheck", st);
    } else if (kind == PCD_RULE_CPM) {
        RuleCPM r;
        r.lambda = lambda;
        launches += launch_bins_rule(g, a, r, st);
    } else {
        RuleWCC r;
        r.cc = g->cc;
        launches += launch_bins_rule(g, a, r, st);
    }
    const int32_t f = (int32_t)((frac < 1.0 ? frac : 1.0) * 2147483647.0);
    const int32_t *skip = nullptr;
    if (f == 2147483647) {
        launches += scan_exclusive(DrawLoad{g->ndraw}, DrawStore{g->ndraw}, g->n, g->scan, st);
        k_total_draws<<<1, 1, 0, st>>>(g->ctr, g->scan_total);
        ++launches;
        prof_mark(g->ctx, "sweep.draw_scan", st);
    } else {
        k_walk<<<1, 1, 0, st>>>(seed, f, g->n, g->ndraw, g->labels, g->labels_alt, g->first, g->ctr);
        skip = g->first;
        ++launches;
        prof_mark(g->ctx, "sweep.draw_walk", st);
    }
    k_resolve<<<g->ctx->num_sms * 4, 256, 0, st>>>(g->recs, g->ctr, g->ndraw, nullptr, g->tiebuf, g->labels_alt,
                                                  seed, 2, skip);
    ++launches;
    prof_mark(g->ctx, "sweep.resolve", st);
    return launches;
}

void launch_resolve(const TieRecord *recs, const DevCounters *ctr, const uint32_t *endpos, const uint32_t *base,
                    const int32_t *tiebuf, int32_t *out, uint32_t seed, int32_t mod_base, int grid,
                    cudaStream_t st) {
    k_resolve<<<grid, 256, 0, st>>>(recs, ctr, endpos, base, tiebuf, out, seed, mod_base, nullptr);
}

}  // namespace pcd
