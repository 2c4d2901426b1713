// Device-side building blocks shared by every kernel of libpcd:
//   * rand_r stream replay with O(log n) jump-ahead,
//   * the gain rules (Modularity, CPM, WCC) in the reference's FP64
//     expression order, plus the exact-integer Modularity ordering key,
//   * warp/block "running maximum, first holder kept" scans that reproduce the
//     reference's sequential best-candidate loop.
//
// All translation units are compiled with -fmad=false so that FP64 products
// and sums are never contracted into FMAs: every double below is the IEEE
// result of the same operation sequence as the reference source.
#pragma once

#include <cstdint>
#include <climits>
#include <cuda_runtime.h>

#include "pcd_types.h"

namespace pcd {

constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// rand_r (glibc) on the device.  The reference draws every tie-break and
// every frac test with rand_r (src/refinement.cpp:129,159,250).  One rand_r
// call advances the 32-bit LCG x -> 1103515245 x + 12345 three times and
// assembles 11 + 10 + 10 bits taken from bit 16 of the successive states.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lcg(uint32_t x) { return x * 1103515245u + 12345u; }

__device__ __forceinline__ int32_t rand_r_dev(uint32_t &x) {
    x = lcg(x);
    int32_t r = (int32_t)((x >> 16) & 2047u);
    x = lcg(x);
    r = (r << 10) ^ (int32_t)((x >> 16) & 1023u);
    x = lcg(x);
    r = (r << 10) ^ (int32_t)((x >> 16) & 1023u);
    return r;
}

// Affine maps x -> a x + c of 3 * 2^i LCG steps (one rand_r call = 3 steps),
// i = 0..31; the table itself lives in propagate.cu's constant bank.
struct JumpTable {
    uint32_t a[32];
    uint32_t c[32];
};

// ---------------------------------------------------------------------------
// Graph / partition views handed to kernels.
// ---------------------------------------------------------------------------
struct GraphView {
    int32_t n, m;
    const int32_t *__restrict__ indices;
    const int32_t *__restrict__ adj;
    const int32_t *__restrict__ tri;     // WCC
    const int32_t *__restrict__ tri_deg; // WCC
    double cc;                           // WCC clustering coefficient
};

struct CommView {
    const int32_t *__restrict__ size;
    const int32_t *__restrict__ intv;
    const int32_t *__restrict__ extv;
    const int32_t *__restrict__ vol;  // intv + extv
};

// ---------------------------------------------------------------------------
// WCC improvement, src/rules.cpp:240-389, term by term.  Products the
// reference computes in `int` wrap modulo 2^32 (imul_wrap); every other
// operation is the same IEEE double operation in the same order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t imul_wrap(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}

static __device__ __noinline__ double wcc_improvement(int32_t n_x, int32_t n_y, int32_t c_x, int32_t c_y,
                                               int32_t m_x, int32_t m_y, int32_t m_xy, int32_t b_x,
                                               int32_t b_y, double cc) {
    double p_x = n_x > 1 ? m_x / (n_x * (n_x - 1.0) / 2.0) : 0.0;
    double p_y = n_y > 1 ? m_y / (n_y * (n_y - 1.0) / 2.0) : 0.0;
    double p_xy = c_x > 0 && c_y > 0 ? m_xy / (double)imul_wrap(c_x, c_y) : 0.0;
    double q_x = n_x > 0 ? (b_x - m_xy) / (double)n_x : 0;
    double q_y = n_y > 0 ? (b_y - m_xy) / (double)n_y : 0;
    double score = 0.0;
    if (c_x > 0) {
        double t_x = (imul_wrap(n_x - 1, n_x - 2) / 2) * p_x * p_x * p_x;
        double t_xy = t_x + imul_wrap(c_x - 1, c_y) * p_x * p_y * p_xy
                      + (imul_wrap(c_y, c_y - 1) / 2) * p_xy * p_xy * p_y;
        double t_v = t_xy + q_x * (q_x - 1) / 2 * cc + q_x * (n_x - 1) * p_x * cc
                     + c_y * q_x * p_xy * cc;
        double vt_xy = q_x;
        double vt_x = vt_xy + p_xy * c_y;
        double vt_v = vt_x + p_x * (n_x - 1);
        double tr = (vt_v / t_v) * (t_xy / (n_x + n_y - 1 + vt_xy))
                    - (vt_v / t_v) * (t_x / (n_x - 1 + vt_x));
        if (t_v > 0) score += c_x * tr;
    }
    if (c_x < n_x) {
        double t_x = (imul_wrap(n_x - 1, n_x - 2) / 2) * p_x * p_x * p_x;
        double t_xy = t_x;
        double t_v = t_xy + q_x * (q_x - 1) / 2 * cc + q_x * (n_x - 1) * p_x * cc;
        double vt_xy = q_x;
        double vt_x = vt_xy;
        double vt_v = vt_x + p_x * (n_x - 1);
        double tr = (vt_v / t_v) * (t_xy / (n_x + n_y - 1 + vt_xy))
                    - (vt_v / t_v) * (t_x / (n_x - 1 + vt_x));
        if (t_v > 0) score += (n_x - c_x) * tr;
    }
    if (c_y > 0) {
        double t_y = (imul_wrap(n_y - 1, n_y - 2) / 2) * p_y * p_y * p_y;
        double t_xy = t_y + imul_wrap(c_y - 1, c_x) * p_y * p_x * p_xy
                      + (imul_wrap(c_x, c_x - 1) / 2) * p_xy * p_xy * p_x;
        double t_v = t_xy + q_y * (q_y - 1) / 2 * cc + q_y * (n_y - 1) * p_y * cc
                     + c_x * q_y * p_xy * cc;
        double vt_xy = q_y;
        double vt_y = vt_xy + p_xy * c_x;
        double vt_v = vt_y + p_y * (n_y - 1);
        double tr = (vt_v / t_v) * (t_xy / (n_y + n_x - 1 + vt_xy))
                    - (vt_v / t_v) * (t_y / (n_y - 1 + vt_y));
        if (t_v > 0) score += c_y * tr;
    }
    if (c_y < n_y) {
        double t_y = (imul_wrap(n_y - 1, n_y - 2) / 2) * p_y * p_y * p_y;
        double t_xy = t_y;
        double t_v = t_xy + q_y * (q_y - 1) / 2 * cc + q_y * (n_y - 1) * p_y * cc;
        double vt_xy = q_y;
        double vt_y = vt_xy;
        double vt_v = vt_y + p_y * (n_y - 1);
        double tr = (vt_v / t_v) * (t_xy / (n_y + n_x - 1 + vt_xy))
                    - (vt_v / t_v) * (t_y / (n_y - 1 + vt_y));
        if (t_v > 0) score += (n_y - c_y) * tr;
    }
    return score;
}

// Per-graph parameters when many graphs are refined as one disjoint union
// (the batched path).  All pointers are null for a single graph.
struct BatchView {
    const int32_t *__restrict__ vgid;  // graph of each vertex
    const int32_t *__restrict__ cgid;  // graph of each community
    const int32_t *__restrict__ gm;    // edges of each graph
    const double *__restrict__ gcc;    // clustering coefficient of each graph (WCC)
};

// ---------------------------------------------------------------------------
// Rules.  Each rule defines a scan Key and its order, the join gain of a
// candidate (vertex v of degree d, community c, k neighbours in c) and the
// final move decision.  A Tag carries what the exact-integer Modularity key
// needs to tell equal keys apart (k and the community volume V).
// ---------------------------------------------------------------------------
enum : int32_t { DEC_STAY = 0, DEC_MOVE = 1, DEC_NEW = 2, DEC_AMBIGUOUS = 3 };

struct Tag {
    int32_t k;
    int32_t V;
};

// The FP64 rules: CPM, WCC, and Modularity when re-evaluated exactly.
template <class Derived>
struct RuleF64Base {
    using Key = double;
    static constexpr bool kExactInt = false;
    BatchView bv{};
    // the rule as seen by vertex v / community c (batched: that graph's parameters)
    __device__ Derived at(int32_t v) const {
        Derived r = *static_cast<const Derived *>(this);
        if (bv.vgid) r.set_graph(bv.vgid[v]);
        return r;
    }
    __device__ Derived at_comm(int32_t c) const {
        Derived r = *static_cast<const Derived *>(this);
        if (bv.cgid) r.set_graph(bv.cgid[c]);
        return r;
    }
    __device__ void set_graph(int32_t) {}
    __device__ static Key identity() { return -__longlong_as_double(0x7ff0000000000000LL); }
    __device__ static Key initial() { return 0.0; }
    __device__ static bool gt(Key a, Key b) { return a > b; }
    __device__ static bool eq(Key a, Key b) { return a == b; }
    // NaN gains compare false against everything in the reference loop:
    // they never win and never tie, exactly like an absent candidate.
    __device__ static bool usable(Key a) { return a == a; }
    __device__ static bool ambiguous_tie(const Tag &, const Tag &, bool) { return false; }
    __device__ bool vertex_ambiguous(int32_t) const { return false; }
    // src/refinement.cpp:169-179
    __device__ int32_t decide(Key best, bool has_best, int32_t v, int32_t d, int32_t curr,
                              int32_t curr_freq, const CommView &cm) const {
        (void)has_best;
        double leave = static_cast<const Derived *>(this)->leave(v, d, curr, curr_freq, cm);
        double best_score = best;
        best_score += leave;
        if (best_score > 0 && best_score > leave) return DEC_MOVE;
        if (leave > 0) return DEC_NEW;
        return DEC_STAY;
    }
};

// ModularityRule, src/rules.cpp:24-56.
struct RuleModF64 : RuleF64Base<RuleModF64> {
    int32_t m;
    __device__ void set_graph(int32_t g) { m = bv.gm[g]; }
    __device__ Key join(int32_t, int32_t d, int32_t c, int32_t k, const CommView &cm, Tag &) const {
        double e_ij = k / (double)m;
        double a_i = cm.vol[c] / (2.0 * m);
        double a_j = d / (2.0 * m);
        return e_ij - 2 * a_i * a_j;
    }
    // join of a community that is one vertex (size 1, no internal edge,
    // volume V = that vertex's degree) with k = 1: the same operations as
    // join() with those statistics, which the caller already holds
    __device__ Key join_one(int32_t, int32_t d, int32_t V, Tag &) const {
        double e_ij = 1 / (double)m;
        double a_i = V / (2.0 * m);
        double a_j = d / (2.0 * m);
        return e_ij - 2 * a_i * a_j;
    }
    __device__ double leave(int32_t, int32_t d, int32_t c, int32_t k, const CommView &cm) const {
        double e_ij = k / (double)m;
        double a_i = (cm.vol[c] - d) / (2.0 * m);
        double a_j = d / (2.0 * m);
        return -(e_ij - 2 * a_i * a_j);
    }
    __device__ double merge(int32_t i, int32_t j, int32_t w, const CommView &cm) const {
        double e_ij = w / (double)m;
        double a_i = cm.vol[i] / (2.0 * m);
        double a_j = cm.vol[j] / (2.0 * m);
        return e_ij - 2 * a_i * a_j;
    }
};

// CPMRule, src/rules.cpp:131-144.
struct RuleCPM : RuleF64Base<RuleCPM> {
    double lambda;
    __device__ Key join(int32_t, int32_t, int32_t c, int32_t k, const CommView &cm, Tag &) const {
        return k - lambda * cm.size[c];
    }
    __device__ Key join_one(int32_t, int32_t, int32_t, Tag &) const { return 1 - lambda * 1; }
    __device__ double leave(int32_t, int32_t, int32_t c, int32_t k, const CommView &cm) const {
        return -(k - lambda * (cm.size[c] - 1));
    }
    __device__ double merge(int32_t i, int32_t j, int32_t w, const CommView &cm) const {
        return w - lambda * cm.size[i] * cm.size[j];
    }
};

// WCCRule, src/rules.cpp:391-436.
struct RuleWCC : RuleF64Base<RuleWCC> {
    double cc;
    __device__ void set_graph(int32_t g) { cc = bv.gcc[g]; }
    __device__ Key join(int32_t, int32_t d, int32_t c, int32_t k, const CommView &cm, Tag &) const {
        return wcc_improvement(1, cm.size[c], 1, k, 0, cm.intv[c] / 2, k, d, cm.extv[c], cc);
    }
    // a one-vertex community: size 1, internal volume 0, external volume V
    __device__ Key join_one(int32_t, int32_t d, int32_t V, Tag &) const {
        return wcc_improvement(1, 1, 1, 1, 0, 0, 1, d, V, cc);
    }
    __device__ double leave(int32_t, int32_t d, int32_t c, int32_t k, const CommView &cm) const {
        return -wcc_improvement(1, cm.size[c] - 1, 1, k, 0, cm.intv[c] / 2 - k, k, d,
                                cm.extv[c] - d + 2 * k, cc);
    }
    __device__ double merge(int32_t i, int32_t j, int32_t w, const CommView &cm) const {
        int32_t si = cm.size[i], sj = cm.size[j];
        return wcc_improvement(si, sj, w < si ? w : si, w < sj ? w : sj, cm.intv[i] / 2,
                               cm.intv[j] / 2, w, cm.extv[i], cm.extv[j], cc);
    }
};

// Modularity ordered by an exact integer key.
//
// With e = RN(k/m), a_i = RN(V/2m), a_j = RN(d/2m) the reference's join gain
// is s = RN(e - RN(2 a_i a_j)), and s * 2m^2 = N + delta with
// N = 2m k - V d (exact, int64) and |delta| <= 8.0002 m d 2^-53.  When
// m d <= 2^47 this gives |delta| <= 1/8 and |N| <= 2^48, so ulp(s)*2m^2 <=
// 1/8 and two gains with different N compare the same way as their N (and
// never round to equal), signs follow N, and the final move test
// RN(s_best + leave) > 0 follows N_best > J (J = the leave key).  Equal N with
// the same (k, V) are bit-identical doubles.  Everything else -- equal N from
// different (k, V), N == 0 against the initial 0.0, N_best == J, J == 0, or
// m d > 2^47 -- is flagged and the vertex is re-evaluated in FP64
// (RuleModF64), so the labels are always those of the FP64 computation.
struct RuleModInt {
    using Key = long long;
    static constexpr bool kExactInt = true;
    int32_t m;
    long long two_m;
    BatchView bv{};
    __device__ RuleModInt at(int32_t v) const {
        RuleModInt r = *this;
        if (bv.vgid) {
            r.m = bv.gm[bv.vgid[v]];
            r.two_m = 2LL * r.m;
        }
        return r;
    }
    __device__ static Key identity() { return LLONG_MIN; }
    __device__ static Key initial() { return 0; }
    __device__ static bool gt(Key a, Key b) { return a > b; }
    __device__ static bool eq(Key a, Key b) { return a == b; }
    __device__ static bool usable(Key) { return true; }
    __device__ static bool ambiguous_tie(const Tag &cand, const Tag &holder, bool holder_real) {
        return !holder_real || cand.k != holder.k || cand.V != holder.V;
    }
    __device__ bool vertex_ambiguous(int32_t d) const {
        return (long long)m * (long long)d > (1LL << 47);
    }
    __device__ Key join(int32_t, int32_t d, int32_t c, int32_t k, const CommView &cm, Tag &tag) const {
        const int32_t V = cm.vol[c];
        tag.k = k;
        tag.V = V;
        return two_m * k - (long long)V * d;
    }
    __device__ Key join_one(int32_t, int32_t d, int32_t V, Tag &tag) const {
        tag.k = 1;
        tag.V = V;
        return two_m - (long long)V * d;
    }
    __device__ int32_t decide(Key best, bool has_best, int32_t, int32_t d, int32_t curr, int32_t curr_freq,
                              const CommView &cm) const {
        long long J = two_m * curr_freq - (long long)(cm.vol[curr] - d) * d;
        if (has_best) {
            if (best > J) return DEC_MOVE;
            if (best == J) return DEC_AMBIGUOUS;
            return DEC_STAY;
        }
        if (J < 0) return DEC_NEW;
        if (J == 0) return DEC_AMBIGUOUS;
        return DEC_STAY;
    }
};

// ---------------------------------------------------------------------------
// Ordered running-maximum scan.  An element is (key, ord); combining keeps the
// LEFT element unless the right key is strictly greater -- the reference's
// `if (score > best_score)` with the first holder of a level kept.
// ord: candidate position, -1 for the initial 0.0, -2 for the identity.
// ---------------------------------------------------------------------------
template <class Key>
struct Elem {
    Key key;
    int32_t ord;
};

template <class R>
__device__ __forceinline__ Elem<typename R::Key> combine(const Elem<typename R::Key> &l,
                                                         const Elem<typename R::Key> &r) {
    return R::gt(r.key, l.key) ? r : l;
}

template <class T>
__device__ __forceinline__ T shfl_up_any(const T &v, int delta, int width = 32) {
    static_assert(sizeof(T) % 4 == 0, "word-sized");
    T out;
    const int *s = reinterpret_cast<const int *>(&v);
    int *d = reinterpret_cast<int *>(&out);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); ++i) d[i] = __shfl_up_sync(FULL, s[i], delta, width);
    return out;
}

template <class T>
__device__ __forceinline__ T shfl_any(const T &v, int src, int width = 32) {
    static_assert(sizeof(T) % 4 == 0, "word-sized");
    T out;
    const int *s = reinterpret_cast<const int *>(&v);
    int *d = reinterpret_cast<int *>(&out);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); ++i) d[i] = __shfl_sync(FULL, s[i], src, width);
    return out;
}

// Inclusive scan within aligned groups of `width` lanes; every lane calls it.
template <class R, int WIDTH = 32>
__device__ __forceinline__ Elem<typename R::Key> warp_scan_max(Elem<typename R::Key> x, int lane_in_group) {
#pragma unroll
    for (int d = 1; d < WIDTH; d <<= 1) {
        Elem<typename R::Key> o = shfl_up_any(x, d, WIDTH);
        if (lane_in_group >= d) x = combine<R>(o, x);
    }
    return x;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

// Exclusive warp prefix sum of small ints.
__device__ __forceinline__ int warp_excl_sum(int x, int lane, int *total) {
    int inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int o = __shfl_up_sync(FULL, inc, d);
        if (lane >= d) inc += o;
    }
    *total = __shfl_sync(FULL, inc, 31);
    return inc - x;
}

__device__ __forceinline__ uint32_t hash_label(int32_t l) {
    return (uint32_t)l * 2654435761u;
}

}  // namespace pcd
