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
#include <type_traits>

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
    // labels again, except that a vertex whose community is itself alone
    // holds that community's volume with bit 31 set (written by k_flag_single
    // before the class kernels; not used for a partition of single vertices)
    const int32_t *__restrict__ nlab;
    int32_t *new_labels;
    uint32_t *ndraw;
    int32_t *tiebuf;
    long long tiebuf_cap;
    TieRecord *recs;
    int32_t *nties;  // per vertex: final-level ties to replay (0: none)
    int32_t *amb;
    DevCounters *ctr;
};

// ---------------------------------------------------------------------------
// output of one analysed vertex
// ---------------------------------------------------------------------------
// Vertices the integer key cannot decide go to one list (capacity n) filled
// from both ends: degree <= AMB_WARP_MAX from the front (re-evaluated one warp
// per vertex), larger ones from the back (one block per vertex).
constexpr int AMB_WARP_MAX = 256;

__device__ __forceinline__ void push_ambiguous(const SweepArgs &a, int32_t v, int32_t d) {
    if (d <= AMB_WARP_MAX) {
        const int32_t i = atomicAdd(&a.ctr->n_ambiguous, 1);
        a.amb[i] = v;
    } else {
        const int32_t i = atomicAdd(&a.ctr->n_amb_large, 1);
        a.amb[a.g.n - 1 - i] = v;
    }
}

// The final-level ties of vertex v live in its own slots of the tie buffer,
// [indices[v] + v, indices[v + 1] + v + 1): the holder, then the r tied
// labels in row order (r <= degree).  nties[v] = r tells the replay which
// vertices to visit; fixed slots need no allocation, so analysing kernels
// share no counter.  Returns the slot offset, or -1 when nothing is recorded.
__device__ __forceinline__ long long record_ties(const SweepArgs &a, int32_t v, int32_t row, bool rec, int32_t r,
                                                 int32_t holder) {
    a.nties[v] = rec ? r : 0;
    if (!rec) return -1;
    const long long off = (long long)row + v;
    a.tiebuf[off] = holder;
    return off;
}

__device__ __forceinline__ void write_decision(const SweepArgs &a, int32_t v, int32_t dec, int32_t holder,
                                               int32_t curr) {
    a.new_labels[v] = dec == DEC_MOVE ? holder : (dec == DEC_NEW ? -1 : curr);
}

// Final-level candidates are listed as labels, or, for a single vertex's
// community (whose gain came from the volume in its flag word), as the row
// position with bit 31 set: the label is read from the row only where a
// decision or a tie record needs it.  `row` = indices[v].
__device__ __forceinline__ int32_t fin_entry(int32_t label, int32_t pos) {
    return label >= 0 ? label : (int32_t)(0x80000000u | (uint32_t)pos);
}
__device__ __forceinline__ int32_t fin_label(const SweepArgs &a, int32_t row, int32_t x) {
    return x >= 0 ? x : a.labels[a.g.adj[row + (x & 0x7fffffff)]];
}

// Warp-aggregated allocation of tie records: every lane that passes
// want = r + 1 > 0 gets its own offset in the tie buffer and a record slot.
// Returns the offset (or -1).  All lanes of the warp must call it.
__device__ __forceinline__ long long alloc_ties_warp(const SweepArgs &a, int32_t v, int32_t r, int32_t holder,
                                                    bool want) {
    const int lane = threadIdx.x & 31;
    const unsigned wm = __ballot_sync(FULL, want);
    if (!wm) return -1;
    int tot;
    const int words = want ? r + 1 : 0;
    const int ex = warp_excl_sum(words, lane, &tot);
    const int leader = __ffs(wm) - 1;
    unsigned long long base = 0;
    int32_t rbase = 0;
    if (lane == leader) {
        base = atomicAdd(&a.ctr->tie_used, (unsigned long long)tot);
        rbase = atomicAdd(&a.ctr->n_resolve, __popc(wm));
    }
    base = __shfl_sync(FULL, base, leader);
    rbase = __shfl_sync(FULL, rbase, leader);
    if (!want) return -1;
    const long long off = (long long)(base + ex);
    if (off + r + 1 > a.tiebuf_cap) {
        atomicOr(&a.ctr->error, ERR_TIEBUF_OVERFLOW);
        return -1;
    }
    a.tiebuf[off] = holder;
    a.recs[rbase + __popc(wm & lanemask_lt())] = TieRecord{v, r, off};
    return off;
}

// ---------------------------------------------------------------------------
// One thread per vertex (deg <= MAXD): the reference's candidate loop run as
// it is written, on a row held in registers.  Counting is a pass over the
// pairs i < j of the row (an equal later label adds to the earlier one's
// count and is not a first occurrence), so a label's count sits at its first
// position; then the first occurrences are scored in row order with the
// running maximum, its ties (every tie is one rand_r draw) and the positions
// tied with the final holder (a bit mask).  No lane talks to another, so a
// warp analyses 32 vertices at once.
// ---------------------------------------------------------------------------
// True when every vertex is its own community: k == n, set by the compress
// that precedes every sweep (the first sweep of every schedule from the
// singleton partition).  A row's labels are then distinct (rows hold no
// duplicate neighbours), each counted once, and a label's first occurrence is
// its row position, so the kernels score the row as it stands, without a
// histogram.  Compress numbers communities by their first vertex, so every
// label is then its vertex's id and a neighbour's label needs no gather.
// The flag is the same for every thread of a launch.
__device__ __forceinline__ bool singleton_partition(const SweepArgs &a) { return a.ctr->k == a.g.n; }

template <class R, int MAXD>
__global__ void __launch_bounds__(256) k_prop_thread(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                     int64_t count) {
    using Key = typename R::Key;
    const bool singles = singleton_partition(a);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < count;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = list[idx];
        const int32_t b = a.g.indices[v], d = a.g.indices[v + 1] - b;
        const int32_t curr = a.labels[v];
        const R vr = rule.at(v);
        int32_t lab[MAXD];
        int32_t cnt[MAXD];
#pragma unroll
        for (int j = 0; j < MAXD; ++j) lab[j] = j < d ? a.g.adj[b + j] : -1;
#pragma unroll
        for (int j = 0; j < MAXD; ++j) {
            lab[j] = j < d ? (singles ? lab[j] : a.labels[lab[j]]) : -2 - j;  // distinct negative fillers never match
            cnt[j] = 1;
        }
        uint32_t later = 0;  // bit j: lab[j] occurred at an earlier position
        if (!singles) {
#pragma unroll
            for (int j = 1; j < MAXD; ++j) {
#pragma unroll
                for (int i = 0; i < j; ++i) {
                    const bool e = lab[i] == lab[j];
                    cnt[i] += e ? 1 : 0;
                    later |= e ? (1u << j) : 0u;
                }
            }
        }
        Key best = R::initial();
        int32_t best_j = -1;
        Tag htag{0, 0};
        uint32_t run = 0;  // positions tied with the current holder
        uint32_t t = 0;
        bool amb = false;
        int32_t curr_freq = 0;
#pragma unroll
        for (int j = 0; j < MAXD; ++j) {
            if (j < d && !((later >> j) & 1u)) {
                if (lab[j] == curr) {
                    curr_freq = cnt[j];
                } else {
                    Tag tag{0, 0};
                    const Key key = vr.join(v, d, lab[j], cnt[j], a.cm, tag);
                    if (R::usable(key)) {
                        if (R::gt(key, best)) {
                            best = key;
                            best_j = j;
                            htag = tag;
                            run = 0;
                        } else if (R::eq(key, best)) {
                            ++t;
                            run |= 1u << j;
                            if (R::ambiguous_tie(tag, htag, best_j >= 0)) amb = true;
                        }
                    }
                }
            }
        }
        amb = amb || vr.vertex_ambiguous(d);
        const int32_t dec = amb ? DEC_AMBIGUOUS : vr.decide(best, best_j >= 0, v, d, curr, curr_freq, a.cm);
        if (dec == DEC_AMBIGUOUS) {
            push_ambiguous(a, v, d);
            continue;
        }
        int32_t holder = -1;
#pragma unroll
        for (int j = 0; j < MAXD; ++j)
            if (j == best_j) holder = lab[j];
        const int32_t r = __popc(run);
        a.ndraw[v] = t;
        write_decision(a, v, dec, holder, curr);
        const long long off = record_ties(a, v, b, dec == DEC_MOVE && r > 0, r, holder);
        if (off >= 0) {
            int32_t o = 1;
#pragma unroll
            for (int j = 0; j < MAXD; ++j)
                if ((run >> j) & 1u) a.tiebuf[off + o++] = lab[j];
        }
    }
}

template <class R>
struct PackedKey {
    using K = double;
    __device__ static K ident() { return -__longlong_as_double(0x7ff0000000000000LL); }
    __device__ static K init() { return 0.0; }
    __device__ static K make(typename R::Key raw, int32_t) { return raw; }
    __device__ static double level(K x) { return x; }
    __device__ static bool tie_ambiguous(K, K) { return false; }
    __device__ static typename R::Key raw_level(K x) { return x; }
};

template <>
struct PackedKey<RuleModInt> {
    using K = long long;
    __device__ static K ident() { return LLONG_MIN; }
    __device__ static K init() { return 0; }
    __device__ static K make(long long n, int32_t k) { return (long long)((unsigned long long)n << 14) | k; }
    __device__ static long long level(K x) { return x >> 14; }
    __device__ static bool tie_ambiguous(K c, K pre) { return ((c ^ pre) & 0x3FFF) != 0; }
    __device__ static long long raw_level(K x) { return x >> 14; }
};

template <class K>
__device__ __forceinline__ K kmax(K a, K b) {
    return a > b ? a : b;
}

// One 32-candidate step of the ordered pass (src/refinement.cpp:150-166 over
// packed keys: `score > best` takes the candidate, `score == best` is a tie
// and one rand_r draw).  carry: the packed running maximum before the step
// (equal levels keep the larger count); t: the ties so far; amb: a tie whose
// two gains the integer key cannot tell apart; lfin: the level of the final
// maximum.  A lane whose level is below the carry's can neither tie nor raise
// it, so only the other ("active") lanes are looked at:
//   * none: nothing to do;
//   * the carry already at the final level: no candidate can pass it, so
//     every active lane ties with it.  The carry is left as it is: once its
//     level is final, a tie is ambiguous exactly when its count differs from
//     the carry's (an earlier tie with another count already was);
//   * up to three: walked one by one in lane order, as the reference loop;
//   * more: an inclusive max-scan over the warp.
// Every branch is warp-uniform (carry, lfin and the ballot are).
template <class PK, class L>
__device__ __forceinline__ void ordered_step(typename PK::K key, bool cand, L lfin, typename PK::K &carry,
                                             uint32_t &t, bool &amb, int lane) {
    using K = typename PK::K;
    const unsigned act = __ballot_sync(FULL, cand && PK::level(key) >= PK::level(carry));
    if (!act) return;
    if (PK::level(carry) == lfin) {
        t += __popc(act);
        if (((act >> lane) & 1u) && PK::tie_ambiguous(key, carry)) amb = true;
        return;
    }
    if (__popc(act) <= 3) {
        unsigned rest = act;
        while (rest) {
            const int j = __ffs(rest) - 1;
            rest &= rest - 1;
            const K kj = __shfl_sync(FULL, key, j);
            if (PK::level(kj) == PK::level(carry)) {
                ++t;
                if (PK::tie_ambiguous(kj, carry)) amb = true;
            }
            carry = kmax(carry, kj);
        }
        return;
    }
    K inc = key;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const K y = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc = kmax(inc, y);
    }
    K ex = __shfl_up_sync(FULL, inc, 1);
    if (lane == 0) ex = PK::ident();
    const K pre = kmax(carry, ex);
    const bool tie = cand && PK::level(key) == PK::level(pre);
    if (tie && PK::tie_ambiguous(key, pre)) amb = true;
    t += __popc(__ballot_sync(FULL, tie));
    carry = kmax(carry, __shfl_sync(FULL, inc, 31));
}

// The same step with per-lane tallies: when no candidate of the step passes
// the running maximum (the usual case once a few have been seen), every
// candidate at the carry's level ties with it; the lane counts its own in
// t_lane / a_lane, and the caller reduces them once after the pass.  A step
// in which one passes runs in order (ordered_step).
template <class PK, class L>
__device__ __forceinline__ void tally_step(typename PK::K key, bool cand, L lfin, typename PK::K &carry,
                                           uint32_t &t, bool &amb, uint32_t &t_lane, bool &a_lane, int lane) {
    const auto cl = PK::level(carry);
    const auto lv = PK::level(key);
    if (__any_sync(FULL, cand && lv > cl)) {
        ordered_step<PK>(key, cand, lfin, carry, t, amb, lane);
    } else {
        const bool eq = cand && lv == cl;
        t_lane += eq;
        a_lane |= eq && PK::tie_ambiguous(key, carry);
    }
}

// Per-warp results of a block, combined by every warp from one shared load
// per lane and a shuffle scan (rather than every thread reading all NW
// entries).  carry: the maximum of `init` and the maxima of the warps before
// `wid`; mreal: the maximum over all warps.
// Maximum over the warp.  Integer keys: two 32-bit warp reductions, the high
// words (signed) and then the low words (unsigned) of the lanes that hold the
// top high word, which orders like the signed 64-bit value; FP64 keys: a
// butterfly of shuffles.
__device__ __forceinline__ long long warp_max(long long x) {
    const int hi = (int)(x >> 32);
    const int top = __reduce_max_sync(FULL, hi);
    const unsigned lo = __reduce_max_sync(FULL, hi == top ? (unsigned)x : 0u);
    return (long long)(((unsigned long long)(unsigned)top << 32) | lo);
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
    for (int o = 16; o; o >>= 1) x = kmax(x, __shfl_xor_sync(FULL, x, o));
    return x;
}

template <class PK, int NW>
__device__ __forceinline__ void warp_carry_in(const typename PK::K *s_agg, int wid, int lane, typename PK::K &carry,
                                              typename PK::K &mreal) {
    static_assert(NW <= 32, "one lane per warp");
    using K = typename PK::K;
    const K mine = lane < NW ? s_agg[lane] : PK::ident();
    if constexpr (std::is_same<K, long long>::value) {  // two reductions instead of a scan
        mreal = warp_max(mine);
        const K before = warp_max(lane < wid ? mine : PK::ident());
        carry = wid > 0 ? kmax(PK::init(), before) : PK::init();
    } else {
        K inc = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const K y = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc = kmax(inc, y);
        }
        mreal = __shfl_sync(FULL, inc, 31);
        const K before = __shfl_sync(FULL, inc, wid > 0 ? wid - 1 : 0);
        carry = wid > 0 ? kmax(PK::init(), before) : PK::init();
    }
}

// tt: the sum of the warps' tie counts (mod 2^32); nf: the final-level
// candidates of all warps; before: those of the warps before `wid`; hw: the
// first warp with one (-1: none).
template <int NW>
__device__ __forceinline__ void warp_totals(const uint32_t *s_t, const int32_t *s_nfin, int wid, int lane,
                                            uint32_t &tt, int32_t &nf, int32_t &before, int32_t &hw) {
    const uint32_t t = lane < NW ? s_t[lane] : 0u;
    const int32_t c = lane < NW ? s_nfin[lane] : 0;
    tt = __reduce_add_sync(FULL, t);
    int32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += y;
    }
    nf = __shfl_sync(FULL, inc, 31);
    before = __shfl_sync(FULL, inc - c, wid);
    const unsigned nz = __ballot_sync(FULL, c > 0);
    hw = nz ? __ffs(nz) - 1 : -1;
}

// ---------------------------------------------------------------------------
// warp per vertex (deg <= WCAP): adjacency in chunks of 32 in order; lanes
// holding the same label are merged with match_any and the lowest lane (the
// first occurrence) inserts into the warp's shared hash; new labels get
// consecutive ordinals in lane order, so ordinals are first-occurrence order.
// The candidates are then scored in ordinal order with packed keys, as in the
// one-pass block kernel: their maximum first, then one ordered pass from the
// initial 0.0 for the ties with the running maximum and the final level.
// ---------------------------------------------------------------------------
// Shared memory of one warp of k_prop_warp: the label table (int32, 2 WCAP
// slots; the scoring pass reuses it for the tie list), first-occurrence
// labels (int32), counts (uint16, <= WCAP) and slot ordinals (uint8, < WCAP).
template <int WCAP>
constexpr size_t warp_bytes() {
    static_assert(WCAP <= 256, "ordinals are stored in 8 bits");
    return 8 * WCAP + 4 * WCAP + 2 * WCAP + 2 * WCAP;
}

template <class R, int WCAP>
__global__ void __launch_bounds__(256) k_prop_warp(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                   int64_t count, const int32_t *count_dev) {
    constexpr int TS = 2 * WCAP;
    extern __shared__ int32_t smem[];
    using Key = typename R::Key;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned char *wbase = reinterpret_cast<unsigned char *>(smem) + wid * warp_bytes<WCAP>();
    int32_t *keys = reinterpret_cast<int32_t *>(wbase);
    int32_t *ties = keys;  // the table is dead once the histogram is done
    int32_t *clab = keys + TS;
    uint16_t *ccnt = reinterpret_cast<uint16_t *>(clab + WCAP);
    uint8_t *ords = reinterpret_cast<uint8_t *>(ccnt + WCAP);
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (count_dev) count = *count_dev;
    const bool singles = singleton_partition(a);
    for (int64_t idx = gw; idx < count; idx += nw) {
        const int32_t v = list[idx];
        const int32_t b = a.g.indices[v], e = a.g.indices[v + 1], d = e - b;
        const int32_t curr = a.labels[v];
        const R vr = rule.at(v);
        if (vr.vertex_ambiguous(d)) {
            if (lane == 0) push_ambiguous(a, v, d);
            continue;
        }
        int32_t nc = 0;
        if (singles) {  // the row as it stands: every position a candidate of count 1
            for (int32_t i = lane; i < d; i += 32) {
                clab[i] = a.g.adj[b + i];
                ccnt[i] = 1;
            }
            nc = d;
            __syncwarp();
        }
        int32_t ts = 64;
        while (ts < 2 * d) ts <<= 1;
        if (!singles)
            for (int i = lane; i < ts; i += 32) keys[i] = -1;
        __syncwarp();
        for (int32_t base = b; base < (singles ? b : e); base += 32) {
            const int32_t j = base + lane;
            const bool valid = j < e;
            // flagged entries: a single vertex's community occurs once in the
            // row, a new candidate of count 1 without a table slot; such lanes
            // meet in one dummy group of the match.  Its candidate entry keeps
            // the flag word (the volume) and, in place of the count, the row
            // position, from which the label is read back if it is needed.
            const int32_t l = valid ? a.nlab[a.g.adj[j]] : -2;
            const bool one = valid && l < 0;
            const unsigned peers = __match_any_sync(FULL, one ? INT_MIN : l);
            const bool leader = valid && !one && lane == __ffs(peers) - 1;
            bool isnew = one;
            uint32_t h = 0;
            if (leader) {
                h = hash_label(l) & (uint32_t)(ts - 1);
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
                    h = (h + 1) & (uint32_t)(ts - 1);
                }
            }
            const unsigned newmask = __ballot_sync(FULL, isnew);
            if (isnew) {
                int32_t ord = nc + __popc(newmask & lanemask_lt());
                if (!one) ords[h] = (uint8_t)ord;
                clab[ord] = l;
                ccnt[ord] = one ? (uint16_t)(j - b) : (uint16_t)__popc(peers);
            }
            __syncwarp();
            if (leader && !isnew) ccnt[ords[h]] += (uint16_t)__popc(peers);
            nc += __popc(newmask);
            __syncwarp();
        }
        // scoring over the candidates in first-occurrence order, with packed
        // keys as in the one-pass block kernel: A the keys (registers) and their
        // maximum, B the ordered pass from the initial 0.0 (ties with the running
        // maximum, FP64 ambiguity, the final level's labels in order)
        using PK = PackedKey<R>;
        using K = typename PK::K;
        constexpr int CH = WCAP / 32;
        K key[CH];
        int32_t my_curr = 0;
        K wmax = PK::ident();
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const int32_t i = 32 * c + lane;
            key[c] = PK::ident();
            if (i < nc) {
                const int32_t l = clab[i], k = ccnt[i];
                if (l < 0) {  // a single vertex's community: count 1, volume in the flag word
                    Tag tag{0, 0};
                    const Key raw = vr.join_one(v, d, l & 0x7fffffff, tag);
                    if (R::usable(raw)) key[c] = PK::make(raw, 1);
                } else if (l == curr) {
                    my_curr = k;
                } else {
                    Tag tag{0, 0};
                    const Key raw = vr.join(v, d, l, k, a.cm, tag);
                    if (R::usable(raw)) key[c] = PK::make(raw, k);
                }
            }
            wmax = kmax(wmax, key[c]);
        }
        wmax = warp_max(wmax);
        const K mreal = wmax;
        const auto lfin = PK::level(kmax(PK::init(), mreal));
        K carry = PK::init();
        uint32_t t = 0;
        int32_t nfin = 0;
        bool amb = false;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            if (32 * c >= nc) break;
            const int32_t i = 32 * c + lane;
            const bool cand = key[c] != PK::ident();
            const bool fin = cand && PK::level(key[c]) == lfin;
            const unsigned fm = __ballot_sync(FULL, fin);
            if (fin) ties[nfin + __popc(fm & lanemask_lt())] = fin_entry(clab[i], ccnt[i]);
            nfin += __popc(fm);
            ordered_step<PK>(key[c], cand, lfin, carry, t, amb, lane);
        }
        __syncwarp();
        amb = __any_sync(FULL, amb);
        const int32_t curr_freq = __reduce_add_sync(FULL, my_curr);
        const bool has = mreal != PK::ident() && PK::level(mreal) > PK::level(PK::init());
        const int32_t holder = has ? ties[0] : -1;  // a fin_entry: resolved where it is used
        const int32_t r = has ? nfin - 1 : 0;
        int32_t dec = DEC_AMBIGUOUS;
        if constexpr (R::kExactInt) {  // integer decision: cheaper in every lane than a broadcast
            if (!amb) dec = vr.decide(has ? PK::raw_level(mreal) : R::initial(), has, v, d, curr, curr_freq, a.cm);
        } else {  // FP64 leave gain: one lane evaluates it, the warp takes its decision
            if (!amb && lane == 0)
                dec = vr.decide(has ? PK::raw_level(mreal) : R::initial(), has, v, d, curr, curr_freq, a.cm);
            dec = __shfl_sync(FULL, dec, 0);
        }
        if (dec == DEC_AMBIGUOUS) {
            if (lane == 0) push_ambiguous(a, v, d);
            continue;
        }
        const bool rec = dec == DEC_MOVE && r > 0;
        const long long off = rec ? (long long)b + v : -1;
        if (lane == 0) {
            const int32_t hl = dec == DEC_MOVE ? fin_label(a, b, holder) : holder;
            a.ndraw[v] = t;
            write_decision(a, v, dec, hl, curr);
            record_ties(a, v, b, rec, r, hl);
        }
        if (off >= 0)
            for (int32_t j = lane; j < r; j += 32) a.tiebuf[off + 1 + j] = fin_label(a, b, ties[1 + j]);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// block per vertex.  Histogram into a table (label, count, first position)
// with atomicMin on the first position; position -> slot; then an ordered
// reduce-then-scan over positions: every warp owns a contiguous range, pass A
// takes each range's running maximum, one warp combines them into each
// range's carry-in (starting from the initial 0.0), pass B finds the ties.
// The table lives in shared memory (block bins) or in a per-block HBM slice
// (hubs, FP64 re-evaluation).
// ---------------------------------------------------------------------------
template <class R>
struct BlockScratch {
    Elem<typename R::Key> warp_tot[32];
    Elem<typename R::Key> carry_in[32];
    Tag carry_tag[32];
    int32_t warp_label[32];
    Elem<typename R::Key> fin;
    int32_t fin_label;
    int32_t warp_ties[32];
    int32_t tie_off[32];
    uint32_t t;
    int32_t amb;
    int32_t curr_freq;
    int32_t holder;
    int32_t r;
    long long off;
};

// Warp-wide maximum of a key (all lanes get it).
template <class R>
__device__ __forceinline__ typename R::Key warp_max_key(typename R::Key k) {
#pragma unroll
    for (int d = 16; d; d >>= 1) {
        typename R::Key o = shfl_any(k, (threadIdx.x & 31) ^ d);
        if (R::gt(o, k)) k = o;
    }
    return k;
}

// The table of a block: keys (-1 = empty), counts, first positions (unsigned,
// 0xffffffff = none), then the position -> slot array.  Between vertices the
// table is left empty: pass B clears every slot it reads, and every slot is
// read exactly once (at its label's first position).  Tables live in shared
// memory (one per block), in per-block HBM slices (stride gstride), or in a
// per-vertex HBM region (region_off[list index], hubs: all of them at once).
// Every loop over positions handles U chunks of 32 per warp step so that U
// independent gathers are in flight.
template <class R, bool GLOBAL, int BT, int U>
__global__ void __launch_bounds__(BT) k_prop_block(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                   int64_t count, const int32_t *count_dev, int32_t table_cap,
                                                   int32_t *gscratch, int64_t gstride,
                                                   const long long *__restrict__ region_off, int from_end) {
    using Key = typename R::Key;
    using E = Elem<Key>;
    constexpr int NW = BT / 32;
    extern __shared__ int32_t smem[];
    __shared__ BlockScratch<R> s;
    if (count_dev) count = *count_dev;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (!GLOBAL) {  // shared tables start empty once per block
        uint32_t *f = reinterpret_cast<uint32_t *>(smem + 2 * table_cap);
        for (int32_t i = tid; i < table_cap; i += BT) {
            smem[i] = -1;
            smem[table_cap + i] = 0;
            f[i] = 0xffffffffu;
        }
    }
    for (int64_t vi = blockIdx.x; vi < count; vi += gridDim.x) {
        const int32_t v = from_end ? list[-1 - vi] : list[vi];
        const int32_t b = a.g.indices[v], e = a.g.indices[v + 1], d = e - b;
        const int32_t curr = a.labels[v];
        const R vr = rule.at(v);
        if (vr.vertex_ambiguous(d)) {
            if (tid == 0) push_ambiguous(a, v, d);
            continue;
        }
        int32_t ts = 64;
        while (ts < 2 * d) ts <<= 1;
        int32_t cap = table_cap;
        int32_t *keys = smem;
        if (GLOBAL) {
            if (region_off) {
                keys = gscratch + region_off[vi];
                cap = ts;
            } else {
                keys = gscratch + (int64_t)blockIdx.x * gstride;
            }
        }
        if (ts > cap) {  // a vertex binned past its table: never expected
            if (tid == 0) atomicOr(&a.ctr->error, ERR_SCRATCH_OVERFLOW);
            continue;
        }
        int32_t *cnts = keys + cap;
        uint32_t *fpos = reinterpret_cast<uint32_t *>(cnts + cap);
        int32_t *posarr = cnts + 2 * cap;  // position -> slot; then each warp's final-level ties
        for (int32_t p = tid; p < d; p += BT) posarr[p] = -1;
        if (tid == 0) {
            s.t = 0;
            s.amb = 0;
            s.curr_freq = 0;
        }
        __syncthreads();
        // histogram with first positions
        for (int32_t p0 = 0; p0 < d; p0 += BT * U) {
            int32_t lab[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t p = p0 + u * BT + tid;
                lab[u] = p < d ? a.g.adj[b + p] : -1;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) lab[u] = lab[u] >= 0 ? a.labels[lab[u]] : -2;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int32_t p = p0 + u * BT + tid;
                const int32_t l = lab[u];
                const unsigned peers = __match_any_sync(FULL, l);
                if (p < d && lane == __ffs(peers) - 1) {
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
                    atomicMin(&fpos[h], (uint32_t)p);  // leader = lowest lane = first position of the group
                }
            }
        }
        __syncthreads();
        for (int32_t i = tid; i < ts; i += BT)
            if (keys[i] != -1) posarr[fpos[i]] = i;
        __syncthreads();
        // each warp owns positions [lo, hi)
        const int32_t span = ((d + NW - 1) / NW + 32 * U - 1) / (32 * U) * (32 * U);
        const int32_t lo = min(d, wid * span), hi = min(d, lo + span);
        // pass A: each range's maximum (first position holding it)
        {
            E carry{R::identity(), -2};
            Tag ctag{0, 0};
            int32_t clabel = -1;
            for (int32_t base0 = lo; base0 < hi; base0 += 32 * U) {
                int32_t slot[U], l[U];
                Key key[U];
                Tag tag[U];
                bool sc[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int32_t p = base0 + 32 * u + lane;
                    slot[u] = p < hi ? posarr[p] : -1;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    l[u] = slot[u] >= 0 ? keys[slot[u]] : -1;
                    const int32_t k = slot[u] >= 0 ? cnts[slot[u]] : 0;
                    if (slot[u] >= 0 && l[u] == curr) s.curr_freq = k;
                    sc[u] = slot[u] >= 0 && l[u] != curr;
                    tag[u] = Tag{0, 0};
                    key[u] = R::identity();
                    if (sc[u]) {
                        key[u] = vr.join(v, d, l[u], k, a.cm, tag[u]);
                        if (!R::usable(key[u])) {
                            sc[u] = false;
                            key[u] = R::identity();
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (!__any_sync(FULL, sc[u] && R::gt(key[u], carry.key))) continue;
                    const Key wm = warp_max_key<R>(key[u]);
                    const int fl = __ffs(__ballot_sync(FULL, sc[u] && R::eq(key[u], wm))) - 1;
                    carry = E{wm, base0 + 32 * u + fl};
                    ctag = Tag{__shfl_sync(FULL, tag[u].k, fl), __shfl_sync(FULL, tag[u].V, fl)};
                    clabel = __shfl_sync(FULL, l[u], fl);
                }
            }
            if (lane == 0) {
                s.warp_tot[wid] = carry;
                s.carry_tag[wid] = ctag;  // tag and label of this range's maximum
                s.warp_label[wid] = clabel;
            }
        }
        __syncthreads();
        if (wid == 0) {
            const E wt = lane < NW ? s.warp_tot[lane] : E{R::identity(), -2};
            const Tag wtag = lane < NW ? s.carry_tag[lane] : Tag{0, 0};
            const E wi = warp_scan_max<R>(wt, lane);
            E we = shfl_up_any(wi, 1);
            if (lane == 0) we = E{R::identity(), -2};
            const E init{R::initial(), -1};
            const E cin = combine<R>(init, we);
            const E fin = combine<R>(init, shfl_any(wi, 31));
            int src = lane, fsrc = 0;
            for (int w2 = 0; w2 < NW; ++w2) {
                const int32_t o = __shfl_sync(FULL, wt.ord, w2);
                if (cin.ord >= 0 && o == cin.ord) src = w2;
                if (fin.ord >= 0 && o == fin.ord) fsrc = w2;
            }
            const Tag ct{__shfl_sync(FULL, wtag.k, src), __shfl_sync(FULL, wtag.V, src)};
            const int32_t wl = lane < NW ? s.warp_label[lane] : -1;
            const int32_t fl = __shfl_sync(FULL, wl, fsrc);
            __syncwarp();
            if (lane < NW) {
                s.carry_in[lane] = cin;
                s.carry_tag[lane] = ct;
            }
            if (lane == 0) {
                s.fin = fin;
                s.fin_label = fin.ord >= 0 ? fl : -1;
            }
        }
        __syncthreads();
        // pass B: ties against the true running maximum; clears the table
        {
            E carry = s.carry_in[wid];
            Tag ctag = s.carry_tag[wid];
            const E fin = s.fin;
            uint32_t t = 0;
            int32_t nt = 0;  // this warp's final-level ties so far
            bool amb = false;
            for (int32_t base0 = lo; base0 < hi; base0 += 32 * U) {
                int32_t slot[U], l[U];
                Key key[U];
                Tag tag[U];
                bool sc[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int32_t p = base0 + 32 * u + lane;
                    slot[u] = p < hi ? posarr[p] : -1;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    l[u] = -1;
                    int32_t k = 0;
                    if (slot[u] >= 0) {
                        l[u] = keys[slot[u]];
                        k = cnts[slot[u]];
                        keys[slot[u]] = -1;
                        cnts[slot[u]] = 0;
                        fpos[slot[u]] = 0xffffffffu;
                    }
                    sc[u] = slot[u] >= 0 && l[u] != curr;
                    tag[u] = Tag{0, 0};
                    key[u] = R::identity();
                    if (sc[u]) {
                        key[u] = vr.join(v, d, l[u], k, a.cm, tag[u]);
                        if (!R::usable(key[u])) {
                            sc[u] = false;
                            key[u] = R::identity();
                        }
                    }
                }
                __syncwarp();  // all lanes have read posarr[base0, base0 + 32 U)
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (!__any_sync(FULL, sc[u] && !R::gt(carry.key, key[u]))) continue;  // below the maximum
                    const int32_t base = base0 + 32 * u;
                    const E inc = warp_scan_max<R>(E{key[u], sc[u] ? base + lane : -2}, lane);
                    E ex = shfl_up_any(inc, 1);
                    if (lane == 0) ex = E{R::identity(), -2};
                    const E pre = combine<R>(carry, ex);
                    const bool tie = sc[u] && R::eq(key[u], pre.key);
                    const bool in_chunk = pre.ord >= base;
                    const int src = in_chunk ? pre.ord - base : lane;
                    const Tag lt{__shfl_sync(FULL, tag[u].k, src), __shfl_sync(FULL, tag[u].V, src)};
                    const Tag htag = in_chunk ? lt : ctag;
                    if (tie && R::ambiguous_tie(tag[u], htag, pre.ord >= 0)) amb = true;
                    t += __popc(__ballot_sync(FULL, tie));
                    const E nxt = combine<R>(carry, shfl_any(inc, 31));
                    if (nxt.ord != carry.ord) {
                        const int hs = nxt.ord - base;
                        ctag = Tag{__shfl_sync(FULL, tag[u].k, hs), __shfl_sync(FULL, tag[u].V, hs)};
                    }
                    const bool inrun = tie && pre.ord == fin.ord;
                    const unsigned run = __ballot_sync(FULL, inrun);
                    // nt + rank < positions of this range already read: overwrites only consumed slots
                    if (inrun) posarr[lo + nt + __popc(run & lanemask_lt())] = l[u];
                    nt += __popc(run);
                    carry = nxt;
                }
            }
            amb = __any_sync(FULL, amb);
            if (lane == 0) {
                s.warp_ties[wid] = nt;
                if (t) atomicAdd(&s.t, t);
                if (amb) s.amb = 1;
            }
        }
        __syncthreads();
        if (tid == 0) {
            const E c = s.fin;
            int32_t r = 0;
            for (int w = 0; w < NW; ++w) {
                s.tie_off[w] = r;
                r += s.warp_ties[w];
            }
            s.r = r;
            s.off = -1;
            const int32_t dec = s.amb ? DEC_AMBIGUOUS : vr.decide(c.key, c.ord >= 0, v, d, curr, s.curr_freq, a.cm);
            if (dec == DEC_AMBIGUOUS) {
                push_ambiguous(a, v, d);
            } else {
                a.ndraw[v] = s.t;
                write_decision(a, v, dec, s.fin_label, curr);
                s.off = record_ties(a, v, b, dec == DEC_MOVE && r > 0, r, s.fin_label);
            }
        }
        __syncthreads();
        {
            const long long off = s.off;
            if (off >= 0) {
                const int32_t nt = s.warp_ties[wid], o = s.tie_off[wid];
                for (int32_t j = lane; j < nt; j += 32) a.tiebuf[off + 1 + o + j] = posarr[lo + j];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Packed candidate keys for the one-pass block kernels.  A key must order
// candidates by gain and let a plain maximum carry what the tie logic needs:
//   Modularity (exact integer gain N): (N << 14) | k.  |N| <= 2m d <= 2^48
//     (larger m d goes to the FP64 path first), so the shift cannot overflow,
//     and k <= d <= 8192 fits the low 14 bits exactly (a hub whose count
//     passes 14 bits is decided in FP64).  Among keys of one
//     gain level the maximum carries the largest k seen; a tie whose k differs
//     from it meets a holder with another (k, volume) pair -- equal integer
//     gain, possibly unequal FP64 gains -- and is re-evaluated in FP64.  The
//     initial 0.0 packs as k = 0, which no real candidate has.
//   FP64 rules: the gain itself (NaN gains are not candidates).
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// block per vertex, one keyed pass (degrees up to NW * 32 * RPL).  Every warp
// owns a contiguous range of the row, RPL positions per lane in registers
// (p = lo + 32 i + lane: each step of a warp reads 32 consecutive neighbours).
//   H  the range's neighbour labels, all RPL gathers in flight; a single
//      vertex's community (flag word) is a candidate of count 1 at once, its
//      key from the volume in the flag word; every other label is inserted
//      into the shared table (positions with one label meet in one slot, one
//      CAS wins; count and first position by shared-memory atomics).
//      (Pre-aggregating equal labels across the warp with match_any cost more
//      than the atomics it saved: R-MAT scale 24, large-block class 4.99 ->
//      4.54 ms without it.)
//   K  one barrier, then a table position is a candidate iff first[slot] ==
//      p; packed keys and the range maximum; one barrier, then every warp
//      knows its carry-in (the initial 0.0 and the maxima of the ranges
//      before it) and the final maximum.
//   S  ordered pass over the range from the carry-in: ties with the running
//      maximum (one rand_r draw each), FP64 ambiguity and the number of the
//      final level's candidates.  A range whose maximum is below its
//      carry-in has none; once the carry holds the final level, every
//      final-level candidate ties with it (in larger blocks tallied per lane
//      and reduced once).  The table slots are cleared here.
//   Every warp then derives the same decision from the per-warp totals.  For
//   a move, each range lists its final-level candidates from its registers:
//   the first of all (the holder) is the new label, and with ties every one
//   goes to the tie buffer at its rank.  No barrier closes a vertex: the
//   next vertex's H only touches the table (cleared before the S barrier)
//   and registers, so warps that finish early start loading the next row;
//   the per-vertex flags alternate by parity.
// ---------------------------------------------------------------------------
// Blocks per SM the register budget is set for: 512-thread variants two (64
// registers a thread), 256-thread ones with three or four positions per lane
// five (48); the others, and WCC's FP64 gain, leave it to the compiler
template <class R>
constexpr int block1_min_blocks(int bt, int rpl) {
    return std::is_same<R, RuleWCC>::value ? 0 : bt == 512 ? 2 : bt == 256 && (rpl == 3 || rpl == 4) ? 5 : 0;
}
template <class R>
constexpr bool block1_lists_in_pass(int bt) {
    return bt == 256 || std::is_same<R, RuleWCC>::value;
}

template <class R, int BT, int RPL>
__global__ void __launch_bounds__(BT, block1_min_blocks<R>(BT, RPL)) k_prop_block1(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                    int64_t count, int32_t table_cap) {
    using PK = PackedKey<R>;
    using K = typename PK::K;
    constexpr int NW = BT / 32;
    extern __shared__ int32_t smem[];
    int32_t *keys = smem;
    int32_t *cnts = smem + table_cap;
    uint32_t *first = reinterpret_cast<uint32_t *>(smem + 2 * table_cap);
    // 256-thread blocks (and WCC, whose FP64 gain needs the registers) list
    // the final level's candidates in the ordered pass (fin_all: each range's
    // list at its own positions), so their keys and labels need not stay in
    // registers until the decision; larger blocks, whose ordered pass holds
    // most of their time, list them only for a move
    constexpr bool kListInS = block1_lists_in_pass<R>(BT);
    // WCC keys every candidate in K: its gain is an out-of-line FP64
    // function, and calls from both passes would each save the live registers
    constexpr bool kOneKeyInK = std::is_same<R, RuleWCC>::value;
    int32_t *fin_all = smem + 3 * table_cap;  // NW * 32 * RPL entries when kListInS
    __shared__ K s_agg[NW];
    __shared__ uint32_t s_t[NW];
    __shared__ int32_t s_nfin[NW];
    __shared__ int32_t s_amb[2], s_curr_freq[2];  // by the parity of the analysed vertex
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const bool singles = singleton_partition(a);
    for (int32_t i = tid; i < table_cap; i += BT) {
        keys[i] = -1;
        cnts[i] = 0;
        first[i] = 0xffffffffu;
    }
    if (tid == 0) {
        s_amb[0] = 0;
        s_curr_freq[0] = 0;
    }
    __syncthreads();
    int par = 0;
    for (int64_t vi = blockIdx.x; vi < count; vi += gridDim.x) {
        const int32_t v = list[vi];
        const int32_t b = a.g.indices[v], d = a.g.indices[v + 1] - b;
        const int32_t curr = a.labels[v];
        const R vr = rule.at(v);
        if (vr.vertex_ambiguous(d)) {
            if (tid == 0) push_ambiguous(a, v, d);
            continue;
        }
        int32_t ts = 64;
        while (ts < 2 * d) ts <<= 1;
        if (ts > table_cap || d > NW * 32 * RPL) {  // binned past its table: never expected
            if (tid == 0) atomicOr(&a.ctr->error, ERR_SCRATCH_OVERFLOW);
            continue;
        }
        const int32_t span = ((d + NW - 1) / NW + 31) & ~31;
        const int32_t lo = min(d, wid * span), hi = min(d, lo + span);
        // H: labels of the range (a partition of single vertices: the row as
        // it stands, every position a candidate of count 1)
        int32_t lab[RPL], slot[RPL];
        K key[RPL];
        uint32_t one_mask = 0;  // kOneKeyInK: positions holding a flag word
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            const int32_t p = lo + 32 * i + lane;
            lab[i] = p < hi ? a.g.adj[b + p] : -1;
        }
        if (!singles) {
#pragma unroll
            for (int i = 0; i < RPL; ++i) lab[i] = lab[i] >= 0 ? a.nlab[lab[i]] : -1;
        }
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            const int32_t p = lo + 32 * i + lane;
            key[i] = PK::ident();
            slot[i] = -1;
            if (p >= hi) {
                lab[i] = -1;
            } else if (!singles) {
                const int32_t l = lab[i];
                if (l < 0) {  // a single vertex's community: count 1, first here
                    if constexpr (kOneKeyInK) {
                        one_mask |= 1u << i;  // keyed in K, beside the table's candidates
                    } else {
                        Tag tag{0, 0};
                        const typename R::Key raw = vr.join_one(v, d, l & 0x7fffffff, tag);
                        if (R::usable(raw)) key[i] = PK::make(raw, 1);
                        lab[i] = -2;  // listed by its position if it reaches the final level
                    }
                } else {
                    uint32_t h = hash_label(l) & (uint32_t)(ts - 1);
                    for (;;) {
                        const int32_t kk = keys[h];
                        if (kk == l) break;
                        if (kk == -1) {
                            const int32_t old = atomicCAS(&keys[h], -1, l);
                            if (old == -1 || old == l) break;
                        }
                        h = (h + 1) & (uint32_t)(ts - 1);
                    }
                    atomicAdd(&cnts[h], 1);
                    atomicMin(&first[h], (uint32_t)p);
                    slot[i] = (int32_t)h;
                }
            }
        }
        __syncthreads();
        if (tid == 0) {  // the next vertex's flags (the last reads of this parity were before the barrier)
            s_amb[par ^ 1] = 0;
            s_curr_freq[par ^ 1] = 0;
        }
        // K: the table's candidates (a label's first position), their keys
        // and the range maximum
        K wmax = PK::ident();
        int32_t kc[RPL];
#pragma unroll
        for (int i = 0; i < RPL; ++i) {
            const int32_t p = lo + 32 * i + lane;
            kc[i] = 0;
            if (singles) {
                if (p < hi) kc[i] = 1;
            } else if (slot[i] >= 0) {
                if (first[slot[i]] == (uint32_t)p)
                    kc[i] = cnts[slot[i]];
                else
                    slot[i] = -1;  // cleared by the label's first position
            }
        }
        if constexpr (std::is_same<R, RuleModInt>::value && RPL <= 4) {
            // the integer Modularity key, the community volumes loaded together
            int32_t vv[RPL];
#pragma unroll
            for (int i = 0; i < RPL; ++i) vv[i] = kc[i] > 0 && lab[i] != curr ? a.cm.vol[lab[i]] : 0;
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                if (kc[i] > 0) {
                    if (lab[i] == curr)
                        s_curr_freq[par] = kc[i];
                    else
                        key[i] = PK::make(vr.two_m * kc[i] - (long long)vv[i] * d, kc[i]);
                }
                wmax = kmax(wmax, key[i]);
            }
        } else {
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                if (kOneKeyInK && ((one_mask >> i) & 1u)) {
                    Tag tag{0, 0};
                    const typename R::Key raw = vr.join_one(v, d, lab[i] & 0x7fffffff, tag);
                    if (R::usable(raw)) key[i] = PK::make(raw, 1);
                    lab[i] = -2;
                }
                if (kc[i] > 0) {
                    if (lab[i] == curr) {
                        s_curr_freq[par] = kc[i];
                    } else {
                        Tag tag{0, 0};
                        const typename R::Key raw = vr.join(v, d, lab[i], kc[i], a.cm, tag);
                        if (R::usable(raw)) key[i] = PK::make(raw, kc[i]);
                    }
                }
                wmax = kmax(wmax, key[i]);
            }
        }
        wmax = warp_max(wmax);
        if (lane == 0) s_agg[wid] = wmax;
        __syncthreads();
        K carry, mreal;
        warp_carry_in<PK, NW>(s_agg, wid, lane, carry, mreal);
        const auto lfin = PK::level(kmax(PK::init(), mreal));
        // S: table clearing; ties with the running maximum and the final
        // level's candidates of this range (listed in the tail, and only when
        // the vertex moves).  A range whose maximum is below the carry-in has
        // neither; once the carry holds the final level, the final level's
        // candidates all tie with it, tallied per lane and reduced once.
#pragma unroll
        for (int i = 0; i < RPL; ++i)
            if (slot[i] >= 0) {
                keys[slot[i]] = -1;
                cnts[slot[i]] = 0;
                first[slot[i]] = 0xffffffffu;
            }
        uint32_t t = 0;
        int32_t nfin = 0;
        bool amb = false;
        if (wmax != PK::ident() && PK::level(wmax) >= PK::level(carry)) {
            int32_t c_fin = 0;
            bool a_fin = false;
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                if (lo + 32 * i >= hi) break;
                const bool cand = key[i] != PK::ident();
                const bool fin = cand && PK::level(key[i]) == lfin;
                if constexpr (kListInS) {  // a single vertex's community (lab -2) is listed by its position
                    const unsigned fm = __ballot_sync(FULL, fin);
                    if (fm) {
                        if (fin) fin_all[lo + nfin + __popc(fm & lanemask_lt())] = fin_entry(lab[i], lo + 32 * i + lane);
                        nfin += __popc(fm);
                    }
                    if (PK::level(carry) == lfin) {  // nothing passes the carry: the final level ties with it
                        t += __popc(fm);
                        if (fin && PK::tie_ambiguous(key[i], carry)) amb = true;
                    } else {
                        ordered_step<PK>(key[i], cand, lfin, carry, t, amb, lane);
                    }
                } else if (PK::level(carry) == lfin) {  // the same, tallied per lane and reduced once
                    c_fin += fin;
                    a_fin |= fin && PK::tie_ambiguous(key[i], carry);
                } else {
                    nfin += __popc(__ballot_sync(FULL, fin));
                    ordered_step<PK>(key[i], cand, lfin, carry, t, amb, lane);
                }
            }
            if (!kListInS) {
                c_fin = __reduce_add_sync(FULL, c_fin);
                nfin += c_fin;
                t += (uint32_t)c_fin;
                amb |= a_fin;
            }
        }
        amb = __any_sync(FULL, amb);
        if (lane == 0) {
            s_t[wid] = t;
            s_nfin[wid] = nfin;
            if (amb) s_amb[par] = 1;
        }
        __syncthreads();
        // every warp: the same totals and decision
        uint32_t tt;
        int32_t nf, before, hw;
        warp_totals<NW>(s_t, s_nfin, wid, lane, tt, nf, before, hw);
        const bool has_best = mreal != PK::ident() && PK::level(mreal) > PK::level(PK::init());
        const int32_t r = has_best ? nf - 1 : 0;
        const int32_t curr_freq = s_curr_freq[par];
        const bool any_amb = s_amb[par] != 0;
        int32_t dec = DEC_AMBIGUOUS;
        if constexpr (R::kExactInt) {  // integer decision: cheaper in every lane than a broadcast
            if (!any_amb) {
                const typename R::Key best = has_best ? PK::raw_level(mreal) : R::initial();
                dec = vr.decide(best, has_best, v, d, curr, curr_freq, a.cm);
            }
        } else {  // FP64 leave gain: one lane per warp evaluates it
            if (!any_amb && lane == 0) {
                const typename R::Key best = has_best ? PK::raw_level(mreal) : R::initial();
                dec = vr.decide(best, has_best, v, d, curr, curr_freq, a.cm);
            }
            dec = __shfl_sync(FULL, dec, 0);
        }
        const bool rec = dec == DEC_MOVE && r > 0;
        if constexpr (kListInS) {
            // the holder is the first final-level candidate: entry 0 of the
            // first range that has one (a fin_entry)
            const int32_t holder = has_best ? fin_all[hw * span] : -1;
            if (tid == 0) {
                if (dec == DEC_AMBIGUOUS) {
                    push_ambiguous(a, v, d);
                } else {
                    const int32_t hl = dec == DEC_MOVE ? fin_label(a, b, holder) : holder;
                    a.ndraw[v] = tt;
                    write_decision(a, v, dec, hl, curr);
                    record_ties(a, v, b, rec, r, hl);
                }
            }
            if (rec) {  // the same number of iterations in every lane
                const long long off = (long long)b + v;  // record_ties' slots: holder, then the ties
                for (int32_t j0 = 0; j0 < nfin; j0 += 32) {
                    const int32_t j = j0 + lane, gi = before + j;  // 0 is the holder
                    if (j < nfin && gi > 0) a.tiebuf[off + gi] = fin_label(a, b, fin_all[lo + j]);
                }
            }
            par ^= 1;
            continue;
        }
        if (tid == 0) {
            if (dec == DEC_AMBIGUOUS) {
                push_ambiguous(a, v, d);
            } else {
                a.ndraw[v] = tt;
                a.nties[v] = rec ? r : 0;
                if (dec != DEC_MOVE) write_decision(a, v, dec, -1, curr);
            }
        }
        // a move: the final level's candidates in row order, the first (the
        // holder, in the first range that has one) is the new label, and with
        // ties every one goes to the vertex's slots of the tie buffer
        // ([indices[v] + v, ...): the holder, then the ties)
        if (dec == DEC_MOVE && nfin > 0 && (rec || wid == hw)) {
            // ranks first, then every needed label read at once (a neighbour's
            // current label), then the writes
            const long long off = (long long)b + v;
            int32_t gi[RPL];
            int32_t j = before;
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                const bool fin = key[i] != PK::ident() && PK::level(key[i]) == lfin;
                const unsigned fm = __ballot_sync(FULL, fin);
                const int32_t g = j + __popc(fm & lanemask_lt());
                gi[i] = fin && (rec || g == 0) ? g : -1;
                j += __popc(fm);
            }
            int32_t L[RPL];
#pragma unroll
            for (int i = 0; i < RPL; ++i) L[i] = gi[i] >= 0 ? a.g.adj[b + lo + 32 * i + lane] : -1;
#pragma unroll
            for (int i = 0; i < RPL; ++i) L[i] = L[i] >= 0 ? a.labels[L[i]] : -1;
#pragma unroll
            for (int i = 0; i < RPL; ++i) {
                if (gi[i] == 0) a.new_labels[v] = L[i];
                if (gi[i] >= 0 && rec) a.tiebuf[off + gi[i]] = L[i];
            }
        }
        par ^= 1;
    }
}

// ---------------------------------------------------------------------------
// Hubs: 1024-thread blocks (one per SM) that take hubs from a queue in list
// order (largest first), so one very large hub does not leave the others to a
// fixed share of the blocks.  The gather pass keys every single vertex's
// community at once (count 1, volume in its flag word) and counts the other
// entries; those are split by hash into P parts of at most part_labels of
// them (one part, the usual case once most neighbours are single vertices,
// reads the positions straight from pos_lab; more parts are bucketed first);
// each part is histogrammed in the shared
// table (label, count, first position: every entry inserts itself,
// with shared-memory atomics for the count and the minimum position, since
// bucket order is not position order), then the table is walked once in slot
// order: each label's packed key is written at its first position and the
// slot is cleared in the same walk.  Position-indexed arrays in a per-block
// global slice carry the row between parts: pos_lab[p] (the label at position
// p, gathered once) and pos_key[p] (the identity, then the packed key at each
// candidate's first position).  The ordered pass of the one-pass kernel then
// runs over pos_key: range maxima, carry-ins, ties and the final level.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hub_part(uint32_t hv, int32_t parts) {
    return (uint32_t)(((unsigned long long)hv * (uint32_t)parts) >> 32);
}

template <class R>
__global__ void __launch_bounds__(1024) k_prop_hub_parts(SweepArgs a, R rule, const int32_t *__restrict__ list,
                                                         int64_t count, int32_t table_cap, int32_t part_labels,
                                                         int32_t *gscratch, int64_t gstride, int32_t pos_cap) {
    using PK = PackedKey<R>;
    using K = typename PK::K;
    constexpr int BT = 1024, NW = 32;
    extern __shared__ int32_t smem[];
    int32_t *keys = smem;
    int32_t *cnts = smem + table_cap;
    uint32_t *first = reinterpret_cast<uint32_t *>(smem + 2 * table_cap);
    __shared__ int32_t s_start[HUB_MAX_PARTS + 1], s_cur[HUB_MAX_PARTS];
    __shared__ K s_agg[NW];
    __shared__ uint32_t s_t[NW];
    __shared__ int32_t s_nfin[NW];
    __shared__ int32_t s_amb, s_curr_freq, s_nrest;
    __shared__ int32_t s_vi[2];  // by iteration parity: a slot is rewritten only after every thread read it
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const bool singles = singleton_partition(a);
    K *pos_key = reinterpret_cast<K *>(gscratch + (int64_t)blockIdx.x * gstride);
    int32_t *pos_lab = reinterpret_cast<int32_t *>(pos_key + pos_cap);
    constexpr bool kHubKeyOnRead = !std::is_same<R, RuleWCC>::value;
    // (position, label) grouped by part; starts on an 8-byte boundary whatever pos_cap is
    int2 *bucket = reinterpret_cast<int2 *>(pos_lab + ((pos_cap + 1) & ~1));
    for (int32_t i = tid; i < table_cap; i += BT) {
        keys[i] = -1;
        cnts[i] = 0;
        first[i] = 0xffffffffu;
    }
    __syncthreads();
    for (int it = 0;; ++it) {
        if (tid == 0) s_vi[it & 1] = atomicAdd(&a.ctr->hub_next, 1);
        __syncthreads();
        const int64_t vi = s_vi[it & 1];
        if (vi >= count) break;
        const int32_t v = list[vi];
        const int32_t b = a.g.indices[v], d = a.g.indices[v + 1] - b;
        const int32_t curr = a.labels[v];
        const R vr = rule.at(v);
        // the packed key of a single vertex's community from its flag word,
        // and a position's key (formed from pos_lab, or stored in pos_key)
        auto flag_key = [&](int32_t lw) -> K {
            Tag tag{0, 0};
            const typename R::Key raw = vr.join_one(v, d, lw & 0x7fffffff, tag);
            return R::usable(raw) ? PK::make(raw, 1) : PK::ident();
        };
        auto pos_key_at = [&](int32_t p) -> K {
            if (kHubKeyOnRead) {
                const int32_t lp = pos_lab[p];
                if (lp < 0) return flag_key(lp);
            }
            return pos_key[p];
        };
        if (vr.vertex_ambiguous(d)) {
            if (tid == 0) push_ambiguous(a, v, d);
            continue;
        }
        if (d > pos_cap) {  // the slices hold the largest degree: never expected
            if (tid == 0) atomicOr(&a.ctr->error, ERR_SCRATCH_OVERFLOW);
            continue;
        }
        if (tid == 0) {
            s_amb = 0;
            s_curr_freq = 0;
            s_nrest = 0;
        }
        __syncthreads();
        // the row's labels by position (gathered once), and how many are not
        // a single vertex's community (those go through the parts)
        int32_t nrest = 0;
        for (int32_t p0 = 0; p0 < d; p0 += BT * 4) {
            int32_t l[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int32_t p = p0 + u * BT + tid;
                l[u] = p < d ? a.g.adj[b + p] : -1;
            }
            if (!singles) {  // flagged labels: bit 31 set for a single vertex's community
#pragma unroll
                for (int u = 0; u < 4; ++u) l[u] = l[u] >= 0 ? a.nlab[l[u]] : 0;  // four gathers in flight
            }
            if (singles) {  // every position is its label's first, count 1: its key at once
                typename R::Key raw[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    Tag tag{0, 0};
                    const int32_t p = p0 + u * BT + tid;
                    raw[u] = p < d && l[u] != curr ? vr.join(v, d, l[u], 1, a.cm, tag) : R::identity();
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int32_t p = p0 + u * BT + tid;
                    if (p < d) {
                        pos_lab[p] = l[u];
                        pos_key[p] = l[u] != curr && R::usable(raw[u]) ? PK::make(raw[u], 1) : PK::ident();
                        if (l[u] == curr) s_curr_freq = 1;
                    }
                }
                continue;
            }
            // a single vertex's community occurs once in any row and is never
            // the vertex's own: count 1, first at p, its key from the volume
            // in the flag word; pos_lab keeps the flag word, the parts below
            // skip it, and its label is read back at the final level.  Its key
            // is formed again where it is read (kHubKeyOnRead) rather than
            // stored, except for WCC, whose gain is too costly to form twice.
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int32_t p = p0 + u * BT + tid;
                if (p < d) {
                    pos_lab[p] = l[u];
                    if (!kHubKeyOnRead || l[u] >= 0) pos_key[p] = l[u] < 0 ? flag_key(l[u]) : PK::ident();
                    nrest += l[u] >= 0;
                }
            }
        }
        if (!singles) {
            nrest = __reduce_add_sync(FULL, nrest);
            if (lane == 0 && nrest) atomicAdd(&s_nrest, nrest);
        }
        __syncthreads();
        // parts of at most part_labels labels, by hash; one part needs no buckets
        const int32_t nr = s_nrest;
        const int32_t parts = min(HUB_MAX_PARTS, max(1, (nr + part_labels - 1) / part_labels));
        if (!singles && nr > 0 && parts > 1) {  // part sizes
            for (int32_t i = tid; i < parts; i += BT) s_cur[i] = 0;
            __syncthreads();
            for (int32_t p0 = 0; p0 < d; p0 += BT) {
                const int32_t p = p0 + tid;
                const int32_t lp = p < d ? pos_lab[p] : -1;
                const int32_t pt = lp >= 0 ? (int32_t)hub_part(hash_label(lp), parts) : -1 - lane;
                const unsigned peers = __match_any_sync(FULL, pt);
                if (pt >= 0 && lane == __ffs(peers) - 1) atomicAdd(&s_cur[pt], __popc(peers));
            }
            __syncthreads();
        }
        if (!singles && nr > 0) {  // parts: buckets, histograms and the slot walk
            if (parts == 1) {
                if (tid == 0) {
                    s_start[0] = 0;
                    s_start[1] = d;  // the positions themselves, read straight from pos_lab
                }
            } else if (wid == 0) {  // exclusive scan of the part sizes
                int32_t carry = 0;
                for (int32_t i0 = 0; i0 < parts; i0 += 32) {
                    const int32_t i = i0 + lane;
                    const int32_t c = i < parts ? s_cur[i] : 0;
                    int32_t inc = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int32_t y = __shfl_up_sync(FULL, inc, o);
                        if (lane >= o) inc += y;
                    }
                    if (i < parts) s_start[i] = carry + inc - c;
                    carry += __shfl_sync(FULL, inc, 31);
                }
                if (lane == 0) s_start[parts] = carry;
            }
            __syncthreads();
            if (parts > 1) {
                for (int32_t i = tid; i < parts; i += BT) s_cur[i] = s_start[i];
                __syncthreads();
                for (int32_t p0 = 0; p0 < d; p0 += BT) {  // positions into their part's bucket
                    const int32_t p = p0 + tid;
                    const int32_t lp = p < d ? pos_lab[p] : -1;  // < 0: a single vertex's label, no bucket
                    const int32_t pt = lp >= 0 ? (int32_t)hub_part(hash_label(lp), parts) : -1 - lane;
                    const unsigned peers = __match_any_sync(FULL, pt);
                    int32_t base = 0;
                    if (lp >= 0 && lane == __ffs(peers) - 1) base = atomicAdd(&s_cur[pt], __popc(peers));
                    base = __shfl_sync(FULL, base, __ffs(peers) - 1);
                    if (lp >= 0) bucket[base + __popc(peers & lanemask_lt())] = make_int2(p, lp);
                }
                __syncthreads();
            }
            for (int32_t part = 0; part < parts; ++part) {
                // one part: the row's positions [0, d), its single vertices skipped
                const int32_t i0 = s_start[part], i1 = s_start[part + 1];
                int32_t ts = 64;
                while (ts < 2 * (parts == 1 ? nr : i1 - i0) && ts < table_cap) ts <<= 1;
                // histogram of this part's labels, four entries in flight per thread
                for (int32_t j0 = i0; j0 < i1; j0 += 4 * BT) {
                  int2 eq[4];
#pragma unroll
                  for (int u = 0; u < 4; ++u) {
                      const int32_t j = j0 + u * BT + tid;
                      if (parts == 1) {
                          const int32_t lp = j < i1 ? pos_lab[j] : -1;
                          eq[u] = make_int2(lp >= 0 ? j : -1, lp);
                      } else {
                          eq[u] = j < i1 ? bucket[j] : make_int2(-1, -2);
                      }
                  }
#pragma unroll
                  for (int u = 0; u < 4; ++u) {
                    const int32_t p = eq[u].x, l = eq[u].y;
                    if (p >= 0) {
                        uint32_t h = hash_label(l) & (uint32_t)(ts - 1);
                        int32_t probes = 0;
                        for (; probes < ts; ++probes) {
                            const int32_t kk = keys[h];
                            if (kk == l) break;
                            if (kk == -1) {
                                const int32_t old = atomicCAS(&keys[h], -1, l);
                                if (old == -1 || old == l) break;
                            }
                            h = (h + 1) & (uint32_t)(ts - 1);
                        }
                        if (probes < ts) {
                            atomicAdd(&cnts[h], 1);
                            atomicMin(&first[h], (uint32_t)p);
                        } else {
                            atomicOr(&a.ctr->error, ERR_SCRATCH_OVERFLOW);  // a part overfilled the table
                        }
                    }
                  }
                }
                __syncthreads();
                // slot walk: each label's key at its first position; the slot is
                // cleared.  Four slots per thread at a time, so that their
                // community statistics gathers (in join) are in flight together.
                for (int32_t i0 = tid; i0 < ts; i0 += 4 * BT) {
                    int32_t lw[4], kw[4];
                    uint32_t pw[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int32_t i = i0 + u * BT;
                        lw[u] = i < ts ? keys[i] : -1;
                        kw[u] = 0;
                        pw[u] = 0;
                        if (lw[u] != -1) {
                            kw[u] = cnts[i];
                            pw[u] = first[i];
                            keys[i] = -1;
                            cnts[i] = 0;
                            first[i] = 0xffffffffu;
                        }
                    }
                    typename R::Key raw[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        Tag tag{0, 0};
                        raw[u] = lw[u] != -1 && lw[u] != curr ? vr.join(v, d, lw[u], kw[u], a.cm, tag) : R::identity();
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (lw[u] == -1) continue;
                        if (lw[u] == curr)
                            s_curr_freq = kw[u];
                        else if (R::usable(raw[u]))
                            pos_key[pw[u]] = PK::make(raw[u], kw[u]);
                        // a candidate's count past the packed key's 14 bits:
                        // the vertex is decided in FP64 (its keys are not used)
                        if (std::is_same<R, RuleModInt>::value && lw[u] != curr && kw[u] > 0x3FFF) s_amb = 1;
                    }
                }
                __syncthreads();
            }
        }
        // ordered pass over the keyed positions, one contiguous range per warp
        const int32_t span = ((d + NW - 1) / NW + 31) & ~31;
        const int32_t lo = min(d, wid * span), hi = min(d, lo + span);
        K wmax = PK::ident();
        for (int32_t p = lo + lane; p < hi; p += 32) wmax = kmax(wmax, pos_key_at(p));
        wmax = warp_max(wmax);
        if (lane == 0) s_agg[wid] = wmax;
        __syncthreads();
        K carry, mreal;
        warp_carry_in<PK, NW>(s_agg, wid, lane, carry, mreal);
        const auto lfin = PK::level(kmax(PK::init(), mreal));
        uint32_t t = 0, t_lane = 0;
        int32_t nfin = 0;
        bool amb = false, a_lane = false;
        int32_t *fin_list = pos_lab + lo;  // entries already read are overwritten
        constexpr int UO = 4;  // 32-position steps whose loads are issued together
        for (int32_t base0 = lo; base0 < hi; base0 += 32 * UO) {
            K kq[UO];
            int32_t lq[UO];
#pragma unroll
            for (int u = 0; u < UO; ++u) {
                const int32_t p = base0 + 32 * u + lane;
                lq[u] = p < hi ? pos_lab[p] : -1;  // < 0: a single vertex's flag word
            }
#pragma unroll
            for (int u = 0; u < UO; ++u) {
                const int32_t p = base0 + 32 * u + lane;
                kq[u] = p >= hi ? PK::ident() : (kHubKeyOnRead && lq[u] < 0 ? flag_key(lq[u]) : pos_key[p]);
            }
            __syncwarp();  // these steps' labels are read before fin_list overwrites read entries
#pragma unroll
            for (int u = 0; u < UO; ++u) {
                const K key = kq[u];
                const bool cand = key != PK::ident();
                const bool fin = cand && PK::level(key) == lfin;
                const unsigned fm = __ballot_sync(FULL, fin);
                if (fin)  // a single vertex's community is listed by its position
                    fin_list[nfin + __popc(fm & lanemask_lt())] = fin_entry(lq[u], base0 + 32 * u + lane);
                nfin += __popc(fm);
                tally_step<PK>(key, cand, lfin, carry, t, amb, t_lane, a_lane, lane);
            }
        }
        t += __reduce_add_sync(FULL, t_lane);
        amb = __any_sync(FULL, amb || a_lane);
        if (lane == 0) {
            s_t[wid] = t;
            s_nfin[wid] = nfin;
            if (amb) s_amb = 1;
        }
        __syncthreads();
        uint32_t tt;
        int32_t nf, before, hw;
        warp_totals<NW>(s_t, s_nfin, wid, lane, tt, nf, before, hw);
        const bool has_best = mreal != PK::ident() && PK::level(mreal) > PK::level(PK::init());
        const int32_t holder = has_best && hw >= 0 ? pos_lab[hw * span] : -1;  // a fin_entry
        const int32_t r = has_best ? nf - 1 : 0;
        int32_t dec = DEC_AMBIGUOUS;
        if constexpr (R::kExactInt) {  // integer decision: cheaper in every lane than a broadcast
            if (!s_amb) {
                const typename R::Key best = has_best ? PK::raw_level(mreal) : R::initial();
                dec = vr.decide(best, has_best, v, d, curr, s_curr_freq, a.cm);
            }
        } else {  // FP64 leave gain: one lane per warp evaluates it
            if (!s_amb && lane == 0) {
                const typename R::Key best = has_best ? PK::raw_level(mreal) : R::initial();
                dec = vr.decide(best, has_best, v, d, curr, s_curr_freq, a.cm);
            }
            dec = __shfl_sync(FULL, dec, 0);
        }
        const bool rec = dec == DEC_MOVE && r > 0;
        if (tid == 0) {
            if (dec == DEC_AMBIGUOUS) {
                push_ambiguous(a, v, d);
            } else {
                const int32_t hl = dec == DEC_MOVE ? fin_label(a, b, holder) : holder;
                a.ndraw[v] = tt;
                write_decision(a, v, dec, hl, curr);
                record_ties(a, v, b, rec, r, hl);
            }
        }
        if (rec) {  // the same number of iterations in every lane
            const long long off = (long long)b + v;
            for (int32_t j0 = 0; j0 < nfin; j0 += 32) {
                const int32_t j = j0 + lane, gi = before + j;  // 0 is the holder
                if (j < nfin && gi > 0) a.tiebuf[off + gi] = fin_label(a, b, fin_list[j]);
            }
        }
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

// nlab[v] = labels[v], or, when v's community is v alone, its volume with bit
// 31 set (the community's statistics are then size 1, no internal edge and
// that volume, so a candidate's gain needs nothing else; its label is read
// back only if it reaches the final level); not needed (nothing written) for
// a partition of single vertices
__global__ void k_flag_single(const int32_t *__restrict__ labels, const int32_t *__restrict__ size,
                              const int32_t *__restrict__ vol, int32_t n, const DevCounters *ctr, int32_t *nlab) {
    if (ctr->k == n) return;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = labels[v];
        nlab[v] = size[l] == 1 ? (int32_t)((uint32_t)vol[l] | 0x80000000u) : l;
    }
}

// frac < 1: whether v draws its ties depends on its frac draw, which depends
// on every earlier vertex's draw count, so each graph's stream is walked in
// vertex order (src/refinement.cpp:127-132 with one thread).  One warp per
// graph: for a chunk of 32 vertices every lane loads its vertex's tie-draw
// count t and composes the affine map of t rand_r calls (independent of the
// stream state); then the whole warp steps the state through the chunk in
// lock-step, so the sequential part is a few integer operations per vertex
// (the frac draw's three LCG steps are evaluated in parallel from the state).
// voff null: one graph [0, n) with `seed`; else graph g = [voff[g], voff[g+1])
// with gseed[g].  Writes each vertex's end position relative to its graph.
__device__ __forceinline__ void calls_map(uint32_t calls, uint32_t &a, uint32_t &c) {
    a = 1u;
    c = 0u;
#pragma unroll 1
    for (int i = 0; calls; ++i, calls >>= 1)
        if (calls & 1u) {
            c = c_jump.a[i] * c + c_jump.c[i];
            a = c_jump.a[i] * a;
        }
}

// One vertex of the walk: the frac draw from state x (its three LCG steps
// evaluated side by side from x; s1 is kept pre-shifted by 4 bits so the 11
// high-order output bits land in place), then, when the vertex draws, the
// affine map (ta, tc) of its t tie draws.
struct WalkStep {
    static constexpr uint32_t A1 = 1103515245u, C1 = 12345u;
    static constexpr uint32_t A2 = A1 * A1, C2 = A1 * C1 + C1;
    static constexpr uint32_t A3 = A1 * A2, C3 = A1 * C2 + C1;
    // The draw is val = hi | lo with hi = its bits 20..30; when hi differs
    // from f's bits 20..30 (all but one case in 2048, the same in every lane)
    // hi alone decides val <= f.
    __device__ __forceinline__ static bool step(uint32_t &x, uint32_t f, uint32_t fhi, uint32_t ta, uint32_t tc) {
        const uint32_t s1 = (16u * A1) * x + 16u * C1;
        const uint32_t s3 = A3 * x + C3;
        const uint32_t hi = s1 & 0x7FF00000u;
        bool draws;
        if (__builtin_expect(hi != fhi, 1)) {
            draws = hi < fhi;
        } else {
            const uint32_t s2 = A2 * x + C2;
            draws = (hi | ((s2 >> 6) & 0x000FFC00u) | ((s3 >> 16) & 0x3FFu)) <= f;
        }
        x = draws ? ta * s3 + tc : s3;
        return draws;
    }
    // One vertex on the sequential chain, without branches: both outcomes of
    // the frac test are formed and selected (a vertex without ties has
    // t = 0 and the identity tie map, so its outcome moves neither the
    // state nor the position); lane `mine` keeps the state it saw, its end
    // position and its outcome.
    __device__ __forceinline__ static void chain(uint32_t &x, uint32_t &pos, uint32_t f, uint32_t fhi, uint32_t ta,
                                                 uint32_t tc, uint32_t t, bool mine, uint32_t &my_x,
                                                 uint32_t &my_pos, bool &my_d) {
        if (mine) my_x = x;
        const uint32_t s1 = (16u * A1) * x + 16u * C1;
        const uint32_t s2 = A2 * x + C2;
        const uint32_t s3 = A3 * x + C3;
        const uint32_t hi = s1 & 0x7FF00000u;
        const uint32_t val = hi | ((s2 >> 6) & 0x000FFC00u) | ((s3 >> 16) & 0x3FFu);
        const bool d = hi != fhi ? hi < fhi : val <= f;
        const uint32_t xd = ta * s3 + tc;
        x = d ? xd : s3;
        pos += d ? 1u + t : 1u;
        if (mine) {
            my_pos = pos;
            my_d = d;
        }
    }
};

// The walk only branches at vertices with ties: a vertex without ties makes
// one call whether or not it passes the frac test.  Per chunk of 32
// vertices, two exact ways, picked by how many of them have ties:
//   few: the vertices with ties are walked in order (the calls of the
//        vertices between them are jumped over with the map of k calls),
//        then every lane evaluates its own frac test from the state after
//        the last vertex with ties before it;
//   many: the chain runs over all 32 vertices, one LCG step (three steps of
//        the generator folded into one affine map) for a vertex without
//        ties, the full step (frac draw, then the jump over its tie draws
//        when it draws) for one with ties; the frac tests of the vertices
//        without ties are evaluated afterwards in their own lanes.
constexpr int WALK_SPARSE = 4;  // at most this many vertices with ties: walk only those

__global__ void __launch_bounds__(128) k_walk(uint32_t seed, const uint32_t *gseed, const int32_t *voff, int32_t G,
                                              int32_t f, int32_t n, uint32_t *ndraw, int32_t *skip,
                                              DevCounters *ctr, const int32_t *gdone) {
    __shared__ uint32_t sh[4][5][32];
    __shared__ uint32_t jA[32], jC[32];
    __shared__ uint32_t kA[33], kC[33];  // map of k calls, k = 0..32
    if (threadIdx.x < 32) {
        jA[threadIdx.x] = c_jump.a[threadIdx.x];
        jC[threadIdx.x] = c_jump.c[threadIdx.x];
    }
    if (threadIdx.x == 0) {
        uint32_t a = 1u, c = 0u;
        for (int k = 0; k <= 32; ++k) {
            kA[k] = a;
            kC[k] = c;
            c = WalkStep::A3 * c + WalkStep::C3;
            a = WalkStep::A3 * a;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t uf = (uint32_t)f, fhi = uf & 0x7FF00000u;
    uint32_t *st = sh[wib][0], *sa = sh[wib][1], *sc = sh[wib][2], *xa = sh[wib][3], *pa = sh[wib][4];
    for (int64_t g = warp; g < G; g += nw) {
        if (gdone && gdone[g]) continue;  // a finished graph keeps its labels: nothing to walk
        const int32_t v0 = voff ? voff[g] : 0, v1 = voff ? voff[g + 1] : n;
        uint32_t x = voff ? gseed[g] : seed, pos = 0;
        // tie counts of the next WQ chunks in flight: each chunk's load is
        // issued WQ chunks before the chain reaches it (ndraw is overwritten
        // only at the chunk being walked)
        constexpr int WQ = 8;
        uint32_t tq[WQ];
#pragma unroll
        for (int q = 0; q < WQ; ++q) {
            const int32_t u = v0 + 32 * q + lane;
            tq[q] = u < v1 ? ndraw[u] : 0u;
        }
        for (int32_t c0 = v0; c0 < v1; c0 += 32) {
            const int32_t v = c0 + lane;
            const bool valid = v < v1;
            const uint32_t t = tq[0];
#pragma unroll
            for (int q = 0; q < WQ - 1; ++q) tq[q] = tq[q + 1];
            tq[WQ - 1] = v + 32 * WQ < v1 ? ndraw[v + 32 * WQ] : 0u;
            uint32_t ta = 1u, tc = 0u;
#pragma unroll 1
            for (uint32_t rem = t, i = 0; rem; ++i, rem >>= 1)
                if (rem & 1u) {
                    tc = jA[i] * tc + jC[i];
                    ta = jA[i] * ta;
                }
            __syncwarp();
            st[lane] = t;
            sa[lane] = ta;
            sc[lane] = tc;
            __syncwarp();
            const unsigned bm = __ballot_sync(FULL, valid && t > 0u);
            const bool has_ties = (bm >> lane) & 1u;
            const int cnt = min(32, v1 - c0);
            uint32_t my_x = 0, my_pos = 0;  // the state before its frac draw, its end position
            bool my_d = false;
            const bool sparse = __popc(bm) <= WALK_SPARSE;
            if (sparse) {
                uint32_t xs = x, ps = pos;
                int prev = -1;
                for (unsigned rest = bm; rest; rest &= rest - 1) {
                    const int j = __ffs(rest) - 1;
                    const int gap = j - prev - 1;  // vertices without ties in between: one call each
                    xs = kA[gap] * xs + kC[gap];
                    ps += (uint32_t)gap;
                    const bool d = WalkStep::step(xs, uf, fhi, sa[j], sc[j]);
                    ps += d ? 1u + st[j] : 1u;
                    if (lane == j) {
                        xa[j] = xs;  // the state and position after vertex j
                        pa[j] = ps;
                        my_d = d;
                    }
                    prev = j;
                }
                __syncwarp();
                const unsigned before = bm & lanemask_lt();
                const int p = before ? 31 - __clz(before) : -1;
                const uint32_t xb = p >= 0 ? xa[p] : x, pb = p >= 0 ? pa[p] : pos;
                const int k = lane - p - 1;
                my_x = kA[k] * xb + kC[k];
                my_pos = has_ties ? pa[lane] : pb + (uint32_t)k + 1u;
                // the chunk's end: after its last vertex
                const int last = cnt - 1;
                const unsigned bl = bm & (last == 31 ? FULL : ((2u << last) - 1u));
                const int pl = bl ? 31 - __clz(bl) : -1;
                const int m = last - pl;
                const uint32_t xe = pl >= 0 ? xa[pl] : x, pe = pl >= 0 ? pa[pl] : pos;
                x = kA[m] * xe + kC[m];
                pos = pe + (uint32_t)m;
                __syncwarp();
            } else if (cnt == 32) {
#pragma unroll
                for (int j = 0; j < 32; ++j) WalkStep::chain(x, pos, uf, fhi, sa[j], sc[j], st[j], lane == j, my_x,
                                                             my_pos, my_d);
            } else {
                for (int j = 0; j < cnt; ++j)
                    WalkStep::chain(x, pos, uf, fhi, sa[j], sc[j], st[j], lane == j, my_x, my_pos, my_d);
            }
            if (valid) {
                if (sparse && !has_ties) my_d = WalkStep::step(my_x, uf, fhi, 1u, 0u);  // its frac test
                ndraw[v] = my_pos;
                skip[v] = my_d ? 0 : 1;
            }
        }
        if (!voff && lane == 0) ctr->total_draws = pos;
    }
}

// Each graph's offset in the scanned stream: the end position of the unit
// before its first one (units are vertices, or communities for merging).
__global__ void k_graph_base(const int32_t *first_unit, int32_t G, const uint32_t *endpos, uint32_t *gbase) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = first_unit[g];
        gbase[g] = u > 0 ? endpos[u - 1] : 0u;
    }
}

// Graphs whose schedule has ended keep their labels.
__global__ void k_done_fixup(const int32_t *__restrict__ vgid, const int32_t *__restrict__ gdone,
                             const int32_t *__restrict__ labels, int32_t *new_labels, int32_t n) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (gdone[vgid[v]]) new_labels[v] = labels[v];
}

// Replay the final level of ties of each recorded vertex/community: the j-th
// tie (0-based) replaces the holder when rand_r % (j + mod_base) == 0.
// Propagation: mod_base 2 (src/refinement.cpp:159, ++best_count from 1);
// merging: mod_base 1 (src/refinement.cpp:250, count++ from 1).
// Batched: ugid maps a unit to its graph, whose seed is gseed[g] and whose
// positions are endpos - gbase[g] (+ gextra[g], merge rounds already drawn).
__global__ void k_resolve(const TieRecord *__restrict__ recs, const DevCounters *ctr,
                          const uint32_t *__restrict__ endpos, const uint32_t *base,
                          const int32_t *__restrict__ tiebuf, int32_t *out, uint32_t seed, int32_t mod_base,
                          const int32_t *skip, const int32_t *__restrict__ ugid, const uint32_t *__restrict__ gseed,
                          const uint32_t *__restrict__ gbase, const uint32_t *__restrict__ gextra) {
    const int32_t nrec = ctr->n_resolve;
    const uint32_t b0 = base ? *base : 0u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrec; i += (int64_t)gridDim.x * blockDim.x) {
        const TieRecord rec = recs[i];
        if (skip && skip[rec.v]) continue;
        uint32_t sd = seed, bb = b0;
        if (ugid) {
            const int32_t g = ugid[rec.v];
            sd = gseed[g];
            bb = (gextra ? gextra[g] : 0u) - gbase[g];
        }
        uint32_t x = rand_r_jump(sd, bb + endpos[rec.v] - (uint32_t)rec.r);
        int32_t best = tiebuf[rec.off];
        for (int32_t j = 0; j < rec.r; ++j) {
            int32_t val = rand_r_dev(x);
            if (val % (j + mod_base) == 0) best = tiebuf[rec.off + 1 + j];
        }
        out[rec.v] = best;
    }
}

// Propagation replay over every vertex (mod_base 2): vertices with nties[v] > 0
// redo the reservoir draws of their final level from their own slots.
__global__ void __launch_bounds__(256) k_resolve_vertices(
    int32_t n, const int32_t *__restrict__ nties, const int32_t *__restrict__ indices,
    const uint32_t *__restrict__ endpos, const int32_t *__restrict__ tiebuf, const int32_t *__restrict__ labels,
    int32_t *out, uint32_t seed, const int32_t *skip, const int32_t *__restrict__ vgid, const uint32_t *__restrict__ gseed,
    const uint32_t *__restrict__ gbase, DevCounters *ctr) {
    int32_t replayed = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        if (skip && skip[v]) {  // no frac draw: the vertex keeps its label
            out[v] = labels[v];
            continue;
        }
        const int32_t r = nties[v];
        if (r <= 0) continue;
        if (r > indices[v + 1] - indices[v]) {  // more ties than neighbours: an internal error
            atomicOr(&ctr->check_where, 32);
            atomicOr(&ctr->error, ERR_CHECK);
            continue;
        }
        uint32_t sd = seed, bb = 0u;
        if (vgid) {
            const int32_t g = vgid[v];
            sd = gseed[g];
            bb = 0u - gbase[g];
        }
        uint32_t x = rand_r_jump(sd, bb + endpos[v] - (uint32_t)r);
        const long long off = (long long)indices[v] + v;
        int32_t best = tiebuf[off];
        for (int32_t j = 0; j < r; ++j) {
            const int32_t val = rand_r_dev(x);
            if (val % (j + 2) == 0) best = tiebuf[off + 1 + j];
        }
        out[v] = best;
        ++replayed;
    }
    __shared__ int32_t block_count;
    if (threadIdx.x == 0) block_count = 0;
    __syncthreads();
    replayed = __reduce_add_sync(0xffffffffu, replayed);
    if ((threadIdx.x & 31) == 0 && replayed) atomicAdd(&block_count, replayed);
    __syncthreads();
    if (threadIdx.x == 0 && block_count) atomicAdd(&ctr->n_resolve, block_count);
}

__global__ void k_reset_sweep(DevCounters *ctr) {
    ctr->tie_used = 0;
    ctr->n_resolve = 0;
    ctr->n_ambiguous = 0;
    ctr->n_amb_large = 0;
    ctr->check_where = 0;
    ctr->error = 0;
    ctr->total_draws = 0;
    ctr->hub_next = 0;
}

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------
constexpr int WARP_CAP = 256;

static inline unsigned cap_grid(int64_t want, int64_t cap) {
    if (want < 1) want = 1;
    return (unsigned)(want < cap ? want : cap);
}

// Warp per vertex for degrees up to WCAP: shared tables of 8 warps per block.
template <class R, int WCAP>
static void launch_warp(pcd_graph *g, const SweepArgs &a, const R &rule, const int32_t *list, int64_t c,
                        cudaStream_t st) {
    const size_t smem = 8 * warp_bytes<WCAP>();
    cudaFuncSetAttribute(k_prop_warp<R, WCAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_prop_warp<R, WCAP>, 256, smem);
    k_prop_warp<R, WCAP><<<cap_grid((c + 7) / 8, (int64_t)g->ctx->num_sms * std::max(1, per_sm) * g->ctx->grid_scale),
                           256, smem, st>>>(
        a, rule, list, c, nullptr);
}

// One-pass block kernel for a class whose largest degree is dmax: the table
// holds 2 dmax slots rounded up to a power of two, so small classes keep many
// blocks resident per SM.
template <class R, int BT, int RPL>
static void launch_block1(pcd_graph *g, const SweepArgs &a, const R &rule, const int32_t *list, int64_t c,
                          int32_t dmax, cudaStream_t st) {
    int32_t cap = 64;
    while (cap < 2 * dmax) cap <<= 1;
    const size_t smem = (3ull * cap + (block1_lists_in_pass<R>(BT) ? (size_t)BT * RPL : 0)) * sizeof(int32_t);
    cudaFuncSetAttribute(k_prop_block1<R, BT, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_prop_block1<R, BT, RPL>, BT, smem);
    k_prop_block1<R, BT, RPL><<<cap_grid(c, (int64_t)g->ctx->num_sms * std::max(1, per_sm) * g->ctx->grid_scale), BT,
                                smem, st>>>(
        a, rule, list, c, cap);
}

template <class R, int MAXD>
static void launch_thread(pcd_graph *g, const SweepArgs &a, const R &rule, int bin, const char *name,
                          cudaStream_t st, int *launches) {
    const int64_t c = g->bin_off[bin + 1] - g->bin_off[bin];
    if (c <= 0) return;
    k_prop_thread<R, MAXD><<<cap_grid((c + 255) / 256, (int64_t)g->ctx->num_sms * 16 * g->ctx->grid_scale), 256, 0, st>>>(
        a, rule, g->bin_list + g->bin_off[bin], c);
    ++*launches;
    prof_mark(g->ctx, name, st);
}

// The degree classes of one sweep are independent (each reads only the old
// labels and writes its own vertices' outputs), so they run concurrently:
// hubs, the large-block and the block classes each on a side stream forked
// from `st`, the warp and thread classes on `st`; `st` then waits for all.
// The longest classes are issued first.
template <class R>
static int launch_bins_rule(pcd_graph *g, const SweepArgs &a, const R &rule, cudaStream_t st) {
    int launches = 0;
    const int32_t *L = g->bin_list;
    int64_t c;
    cudaStream_t side[pcd_ctx::kSide];
    const bool forked = g->ctx->class_streams && side_fork(g->ctx, pcd_ctx::kSide, side) == PCD_OK;
    cudaStream_t s_hub = forked ? side[0] : st, s_bl = forked ? side[1] : st, s_b = forked ? side[2] : st;
    if ((c = g->bin_off[BIN_HUB + 1] - g->bin_off[BIN_HUB]) > 0) {
        // hubs: 1024-thread blocks (one per SM), shared tables filled part by
        // part, position arrays in per-block slices of hub_scratch
        constexpr int32_t cap = HUB_TABLE_CAP;
        const size_t smem = 3ull * cap * sizeof(int32_t);
        cudaFuncSetAttribute(k_prop_hub_parts<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_prop_hub_parts<R><<<cap_grid(c, g->hub_blocks), 1024, smem, s_hub>>>(
            a, rule, L + g->bin_off[BIN_HUB], c, cap, g->hub_part_labels, g->hub_scratch, hub_stride(g->max_deg),
            g->max_deg);
        ++launches;
        prof_mark(g->ctx, "sweep.hub", s_hub);
    }
    // warp and block classes: one launch per degree sub-range, tables sized to
    // its largest degree, larger sub-ranges first
    for (size_t k = g->subs.size(); k-- > 0;) {
        const auto &sr = g->subs[k];
        if (sr.cnt <= 0 || sr.bin < BIN_WARP || sr.bin > BIN_BLOCK_L) continue;
        const int32_t dm = std::max(1, sr.maxdeg), *lst = L + sr.off;
        c = sr.cnt;
        const cudaStream_t ss = sr.bin == BIN_BLOCK_L ? s_bl : (sr.bin == BIN_BLOCK ? s_b : st);
        if (sr.bin == BIN_WARP) {
            if (dm <= 64)
                launch_warp<R, 64>(g, a, rule, lst, c, ss);
            else if (dm <= 128)
                launch_warp<R, 128>(g, a, rule, lst, c, ss);
            else
                launch_warp<R, WARP_CAP>(g, a, rule, lst, c, ss);
        } else if (dm <= 512) {  // positions per lane (RPL) fitted to the sub-range's largest degree
            launch_block1<R, 256, 2>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 768) {
            launch_block1<R, 256, 3>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 1024) {
            launch_block1<R, 256, 4>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 1536) {
            launch_block1<R, 256, 6>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 2048) {
            launch_block1<R, 256, 8>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 2560) {
            launch_block1<R, 512, 5>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 3072) {
            launch_block1<R, 512, 6>(g, a, rule, lst, c, dm, ss);
        } else if (dm <= 4096) {
            launch_block1<R, 512, 8>(g, a, rule, lst, c, dm, ss);
        } else {
            launch_block1<R, 1024, 8>(g, a, rule, lst, c, dm, ss);
        }
        ++launches;
        prof_mark(g->ctx, sr.bin == BIN_WARP ? "sweep.warp" : (sr.bin == BIN_BLOCK ? "sweep.block" : "sweep.block_l"),
                  ss);
    }
    launch_thread<R, 32>(g, a, rule, BIN_G32, "sweep.g32", st, &launches);
    launch_thread<R, 16>(g, a, rule, BIN_G16, "sweep.g16", st, &launches);
    launch_thread<R, 8>(g, a, rule, BIN_G8, "sweep.g8", st, &launches);
    launch_thread<R, 4>(g, a, rule, BIN_G4, "sweep.g4", st, &launches);
    if (forked) {
        side_join(g->ctx, pcd_ctx::kSide);
        prof_mark(g->ctx, "sweep.join", st);  // the wait for the side streams' classes
    }
    return launches;
}

int launch_refine(pcd_graph *g, int32_t kind, double lambda, double frac, uint32_t seed, cudaStream_t st) {
    int launches = 0;
    BatchState *B = g->batch;
    const BatchView bv = B ? BatchView{B->vgid, B->cgid, B->gm, B->gcc} : BatchView{};
    SweepArgs a;
    a.g = GraphView{g->n, g->m, g->indices, g->adj, g->tri, g->tri_deg, g->cc};
    a.cm = CommView{g->sizes, g->intv, g->extv, g->vol};
    a.labels = g->labels;
    a.nlab = g->first;  // free until the frac < 1 walk, after the class kernels
    a.new_labels = g->labels_alt;
    a.ndraw = g->ndraw;
    a.tiebuf = g->tiebuf;
    a.tiebuf_cap = g->tiebuf_cap;
    a.recs = g->recs;
    a.nties = g->nties;
    a.amb = g->amb;
    a.ctr = g->ctr;
    k_reset_sweep<<<1, 1, 0, st>>>(g->ctr);
    if (g->n > 0)
        k_flag_single<<<std::max(1, std::min<int>((g->n + 255) / 256, g->ctx->num_sms * 8)), 256, 0, st>>>(
            g->labels, g->sizes, g->vol, g->n, g->ctr, g->first);
    launches += 2;
    prof_mark(g->ctx, "sweep.reset", st);
    if (kind == PCD_RULE_MODULARITY) {
        RuleModInt r;
        r.m = g->m;
        r.two_m = 2LL * g->m;
        r.bv = bv;
        launches += launch_bins_rule(g, a, r, st);
        // FP64 re-evaluation of the vertices the integer key left open; the
        // list lengths are only known on the device, so both grids stride
        RuleModF64 rf;
        rf.m = g->m;
        rf.bv = bv;
        const size_t smem = 8 * warp_bytes<WARP_CAP>();
        cudaFuncSetAttribute(k_prop_warp<RuleModF64, WARP_CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        k_prop_warp<RuleModF64, WARP_CAP><<<g->ctx->num_sms * 8, 256, smem, st>>>(a, rf, g->amb, 0,
                                                                                  &g->ctr->n_ambiguous);
        k_prop_block<RuleModF64, true, 512, 2><<<g->fb_blocks, 512, 0, st>>>(
            a, rf, g->amb + g->n, 0, &g->ctr->n_amb_large, (int32_t)g->fb_slots, g->fb_scratch,
            3 * g->fb_slots + g->max_deg, nullptr, 1);
        launches += 2;
        prof_mark(g->ctx, "sweep.fp64_recheck", st);
    } else if (kind == PCD_RULE_CPM) {
        RuleCPM r;
        r.lambda = lambda;
        r.bv = bv;
        launches += launch_bins_rule(g, a, r, st);
    } else {
        RuleWCC r;
        r.cc = g->cc;
        r.bv = bv;
        launches += launch_bins_rule(g, a, r, st);
    }
    const int32_t f = (int32_t)((frac < 1.0 ? frac : 1.0) * 2147483647.0);
    const int32_t *skip = nullptr;
    if (f == 2147483647) {
        launches += scan_exclusive(DrawLoad{g->ndraw}, DrawStore{g->ndraw}, g->n, g->scan, st);
        k_total_draws<<<1, 1, 0, st>>>(g->ctr, g->scan_total);
        ++launches;
        if (B) {
            launch_graph_base(B->voff, B->G, g->ndraw, B->gbase, st);
            ++launches;
        }
        prof_mark(g->ctx, "sweep.draw_scan", st);
    } else {
        const int32_t G = B ? B->G : 1;
        k_walk<<<(unsigned)((G + 3) / 4), 128, 0, st>>>(seed, B ? B->gseed : nullptr, B ? B->voff : nullptr, G, f,
                                                         g->n, g->ndraw, g->first, g->ctr, B ? B->gdone : nullptr);
        if (B) cudaMemsetAsync(B->gbase, 0, sizeof(uint32_t) * B->G, st);
        skip = g->first;
        ++launches;
        prof_mark(g->ctx, "sweep.draw_walk", st);
    }
    k_resolve_vertices<<<g->ctx->num_sms * 8, 256, 0, st>>>(g->n, g->nties, g->indices, g->ndraw, g->tiebuf,
                                                           g->labels, g->labels_alt, seed, skip, B ? B->vgid : nullptr,
                                                           B ? B->gseed : nullptr, B ? B->gbase : nullptr, g->ctr);
    ++launches;
    if (B) {
        k_done_fixup<<<g->ctx->num_sms * 8, 256, 0, st>>>(B->vgid, B->gdone, g->labels, g->labels_alt, g->n);
        ++launches;
    }
    prof_mark(g->ctx, "sweep.resolve", st);
    return launches;
}

void launch_resolve(const TieRecord *recs, const DevCounters *ctr, const uint32_t *endpos, const uint32_t *base,
                    const int32_t *tiebuf, int32_t *out, uint32_t seed, int32_t mod_base, int grid,
                    cudaStream_t st, const int32_t *ugid, const uint32_t *gseed, const uint32_t *gbase,
                    const uint32_t *gextra) {
    k_resolve<<<grid, 256, 0, st>>>(recs, ctr, endpos, base, tiebuf, out, seed, mod_base, nullptr, ugid, gseed, gbase,
                                    gextra);
}

void launch_graph_base(const int32_t *first_unit, int32_t G, const uint32_t *endpos, uint32_t *gbase,
                       cudaStream_t st) {
    k_graph_base<<<(G + 255) / 256, 256, 0, st>>>(first_unit, G, endpos, gbase);
}

}  // namespace pcd
