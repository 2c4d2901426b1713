/* CPU restatement of the reference's refine / merge / score path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  The product never links or calls this file.  Its parity with the
 * reference is pinned by tests/test_oracle_pin.py (the reference's own CPU
 * objects, built from the reference sources into oracle/_ref/, run beside it
 * on seeded graphs) and by the hashes in tests/golden/.
 *
 * Each function cites the reference lines it restates.  Arithmetic follows the
 * reference's expression order in IEEE double with no contraction
 * (built with -ffp-contract=off -fno-fast-math).  Signed int products that
 * the reference computes in `int` are computed with 32-bit wrap-around here
 * (what the reference's compiled code does when they overflow).
 */
#include "pcd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RAND_MAX_GLIBC 2147483647
#define NEW_LABEL (-1)

static inline int32_t imul_wrap(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}

static inline int32_t degree(const pcdo_graph *g, int32_t v) {
    return g->indices[v + 1] - g->indices[v];
}

/* ------------------------------------------------------------------------ */
/* glibc rand() / rand_r(), restated from the published algorithm.          */
/* rand(): TYPE_3 additive lagged-Fibonacci generator, r[i] = r[i-3] +      */
/* r[i-31] mod 2^32 over a state seeded by the Park-Miller LCG (16807 mod    */
/* 2^31-1); the first 310 values are discarded; each output is r >> 1.       */
/* rand_r(): three steps of x = x * 1103515245 + 12345 mod 2^32, taking 11,  */
/* 10 and 10 bits (bits 16..) of the successive states.                      */
/* ------------------------------------------------------------------------ */

void pcdo_srand(pcdo_rand_state *s, uint32_t seed) {
    int64_t w = (int32_t)(seed == 0 ? 1u : seed);
    s->r[0] = (uint32_t)w;
    for (int i = 1; i < 31; i++) {
        int64_t x = (16807 * w) % 2147483647;
        if (x < 0) x += 2147483647;
        w = x;
        s->r[i] = (uint32_t)w;
    }
    for (int i = 31; i < 34; i++) s->r[i] = s->r[i - 31];
    s->pos = 0; /* ring slot of value 34 (the next one produced) */
    for (int i = 0; i < 310; i++) (void)pcdo_rand(s);
}

int32_t pcdo_rand(pcdo_rand_state *s) {
    /* ring of the last 34 values: r[i] = r[i-31] + r[i-3]; slot i-31 is
     * (pos + 3) mod 34 and slot i-3 is (pos + 31) mod 34 */
    int32_t i = s->pos;
    uint32_t v = s->r[(i + 3) % 34] + s->r[(i + 31) % 34];
    s->r[i] = v;
    s->pos = (i + 1) % 34;
    return (int32_t)(v >> 1);
}

int32_t pcdo_rand_r(uint32_t *seed) {
    uint32_t x = *seed;
    int32_t result;
    x = x * 1103515245u + 12345u;
    result = (int32_t)((x >> 16) % 2048u);
    x = x * 1103515245u + 12345u;
    result = (result << 10) ^ (int32_t)((x >> 16) % 1024u);
    x = x * 1103515245u + 12345u;
    result = (result << 10) ^ (int32_t)((x >> 16) % 1024u);
    *seed = x;
    return result;
}

/* ------------------------------------------------------------------------ */
/* Insertion-ordered open-addressing table: label -> count.  Same contract  */
/* as the reference's FastHashTable (src/refinement.cpp:24-110): linear      */
/* probing on key & mask, load factor 1/2, starts at 4096 slots, iteration   */
/* in first-insertion order.                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    int32_t *keys;
    int32_t *vals;
    int32_t *order;
    int32_t cap, mask, size;
} otab;

static void otab_init(otab *t) {
    t->cap = 4096;
    t->mask = t->cap - 1;
    t->size = 0;
    t->keys = (int32_t *)malloc(sizeof(int32_t) * t->cap);
    t->vals = (int32_t *)malloc(sizeof(int32_t) * t->cap);
    t->order = (int32_t *)malloc(sizeof(int32_t) * t->cap);
    for (int i = 0; i < t->cap; i++) t->keys[i] = -1;
}

static void otab_free(otab *t) {
    free(t->keys);
    free(t->vals);
    free(t->order);
}

static void otab_grow(otab *t) {
    int32_t ncap = t->cap * 2;
    int32_t *nk = (int32_t *)malloc(sizeof(int32_t) * ncap);
    int32_t *nv = (int32_t *)malloc(sizeof(int32_t) * ncap);
    int32_t *no = (int32_t *)malloc(sizeof(int32_t) * ncap);
    for (int i = 0; i < ncap; i++) nk[i] = -1;
    for (int i = 0; i < t->size; i++) {
        int32_t key = t->keys[t->order[i]];
        int32_t h = key & (ncap - 1);
        while (nk[h] != -1) h = (h + 1) & (ncap - 1);
        nk[h] = key;
        nv[h] = t->vals[t->order[i]];
        no[i] = h;
    }
    free(t->keys);
    free(t->vals);
    free(t->order);
    t->keys = nk;
    t->vals = nv;
    t->order = no;
    t->cap = ncap;
    t->mask = ncap - 1;
}

static inline void otab_insert(otab *t, int32_t key) {
    int32_t h = key & t->mask;
    for (;;) {
        int32_t k = t->keys[h];
        if (k == key) {
            t->vals[h] += 1;
            return;
        }
        if (k == -1) {
            t->keys[h] = key;
            t->vals[h] = 1;
            t->order[t->size++] = h;
            break;
        }
        h = (h + 1) & t->mask;
    }
    if (t->size * 2 > t->cap) otab_grow(t);
}

static inline void otab_clear(otab *t) {
    for (int i = 0; i < t->size; i++) t->keys[t->order[i]] = -1;
    t->size = 0;
}

/* ------------------------------------------------------------------------ */
/* framework.cpp                                                             */
/* ------------------------------------------------------------------------ */

/* framework.cpp:14-24 */
void pcdo_singleton_partition(const pcdo_graph *g, pcdo_rand_state *rs, int32_t *labels) {
    int32_t n = g->n;
    for (int32_t v = 0; v < n; v++) labels[v] = v;
    for (int32_t v = 0; v < n; v++) {
        int32_t j = pcdo_rand(rs) % n;
        int32_t t = labels[v];
        labels[v] = labels[j];
        labels[j] = t;
    }
}

typedef struct {
    double ncc;
    int32_t ndeg;
    int32_t v;
} cc_key;

static int cc_key_cmp(const void *a, const void *b) {
    const cc_key *x = (const cc_key *)a, *y = (const cc_key *)b;
    if (x->ncc < y->ncc) return -1;
    if (y->ncc < x->ncc) return 1;
    if (x->ndeg != y->ndeg) return x->ndeg < y->ndeg ? -1 : 1;
    return x->v < y->v ? -1 : (x->v > y->v);
}

/* framework.cpp:27-59 (needs g->tri) */
void pcdo_clustering_partition(const pcdo_graph *g, int32_t *labels) {
    int32_t n = g->n;
    cc_key *pairs = (cc_key *)malloc(sizeof(cc_key) * (n ? n : 1));
    for (int32_t v = 0; v < n; v++) {
        int32_t tri = g->tri[v];
        int32_t deg = degree(g, v);
        double cc = deg > 1 ? tri / (double)imul_wrap(deg, deg - 1) : 0.0;
        pairs[v].ncc = -cc;
        pairs[v].ndeg = -deg;
        pairs[v].v = v;
    }
    qsort(pairs, n, sizeof(cc_key), cc_key_cmp);
    int32_t num = 0;
    for (int32_t v = 0; v < n; v++) labels[v] = NEW_LABEL;
    for (int32_t i = 0; i < n; i++) {
        int32_t v = pairs[i].v;
        if (labels[v] == NEW_LABEL) {
            labels[v] = num;
            for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++)
                if (labels[g->adj[e]] == NEW_LABEL) labels[g->adj[e]] = num;
            num++;
        }
    }
    free(pairs);
}

/* refinement.cpp:291-322: tags start as vertex ids; each round every vertex
 * takes the minimum of its own and its neighbours' tags (read from the
 * previous round) until no tag changes. */
void pcdo_find_connected(const pcdo_graph *g, int32_t *labels) {
    int32_t n = g->n;
    int32_t *tags = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    int32_t *next = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    for (int32_t i = 0; i < n; i++) tags[i] = i;
    int done = 0;
    while (!done) {
        done = 1;
        for (int32_t v = 0; v < n; v++) {
            int32_t t = tags[v];
            for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++)
                if (tags[g->adj[e]] < t) t = tags[g->adj[e]];
            next[v] = t;
            if (tags[v] != t) done = 0;
        }
        int32_t *tmp = tags;
        tags = next;
        next = tmp;
    }
    memcpy(labels, tags, sizeof(int32_t) * (size_t)n);
    free(tags);
    free(next);
}

typedef struct {
    int32_t i, j;
} nmi_pair;

static int nmi_pair_cmp(const void *a, const void *b) {
    const nmi_pair *x = (const nmi_pair *)a, *y = (const nmi_pair *)b;
    if (x->i != y->i) return x->i < y->i ? -1 : 1;
    return x->j < y->j ? -1 : (x->j > y->j);
}

/* common.cpp:75-125 with the map of common.cpp:163-173: the distinct pairs
 * in (i, j) order with their counts; sums in that order, i then j for den. */
double pcdo_norm_mutual_info(int64_t count, const int32_t *a, const int32_t *b, int32_t n) {
    nmi_pair *pr = (nmi_pair *)malloc(sizeof(nmi_pair) * (size_t)(count ? count : 1));
    int32_t ca = 0, cb = 0;
    for (int64_t k = 0; k < count; k++) {
        pr[k].i = a[k];
        pr[k].j = b[k];
        if (a[k] + 1 > ca) ca = a[k] + 1;
        if (b[k] + 1 > cb) cb = b[k] + 1;
    }
    qsort(pr, (size_t)count, sizeof(nmi_pair), nmi_pair_cmp);
    int32_t *ni = (int32_t *)calloc((size_t)(ca ? ca : 1), sizeof(int32_t));
    int32_t *nj = (int32_t *)calloc((size_t)(cb ? cb : 1), sizeof(int32_t));
    for (int64_t k = 0; k < count; k++) {
        ni[pr[k].i] += 1;
        nj[pr[k].j] += 1;
    }
    double nom = 0.0, den = 0.0;
    for (int64_t k = 0; k < count;) {
        int64_t e = k + 1;
        while (e < count && pr[e].i == pr[k].i && pr[e].j == pr[k].j) e++;
        int32_t val = (int32_t)(e - k);
        int32_t i = pr[k].i, j = pr[k].j;
        nom += val * log(((double)val * n) / imul_wrap(ni[i], nj[j]));
        k = e;
    }
    for (int32_t i = 0; i < ca; i++)
        if (ni[i] != 0) den += ni[i] * log(ni[i] / ((double)n));
    for (int32_t j = 0; j < cb; j++)
        if (nj[j] != 0) den += nj[j] * log(nj[j] / ((double)n));
    free(pr);
    free(ni);
    free(nj);
    return -2 * nom / den;
}

/* framework.cpp:146-170: first-occurrence renumbering; every NEW_LABEL
 * vertex gets a fresh id. */
int32_t pcdo_compress_labels(int32_t n, int32_t *labels) {
    int32_t mx = -1;
    for (int32_t v = 0; v < n; v++)
        if (labels[v] > mx) mx = labels[v];
    int32_t num_labels = mx + 1;
    int32_t *relabel = (int32_t *)malloc(sizeof(int32_t) * (num_labels > 0 ? num_labels : 1));
    for (int32_t i = 0; i < num_labels; i++) relabel[i] = NEW_LABEL;
    int32_t next = 0;
    for (int32_t v = 0; v < n; v++) {
        int32_t old = labels[v];
        int32_t nl;
        if (old == NEW_LABEL)
            nl = next++;
        else if (relabel[old] != NEW_LABEL)
            nl = relabel[old];
        else
            nl = relabel[old] = next++;
        labels[v] = nl;
    }
    free(relabel);
    return next;
}

/* framework.cpp:69-100 (collect_statistics_noatomic) */
int32_t pcdo_collect_statistics(const pcdo_graph *g, const int32_t *labels, int32_t *sizes,
                                int32_t *int_volume, int32_t *ext_volume) {
    int32_t n = g->n;
    int32_t k = -1;
    for (int32_t v = 0; v < n; v++)
        if (labels[v] > k) k = labels[v];
    k += 1;
    for (int32_t i = 0; i < k; i++) sizes[i] = int_volume[i] = ext_volume[i] = 0;
    for (int32_t v = 0; v < n; v++) {
        int32_t l = labels[v], di = 0, de = 0;
        for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
            if (labels[g->adj[e]] == l)
                di++;
            else
                de++;
        }
        sizes[l]++;
        int_volume[l] += di;
        ext_volume[l] += de;
    }
    return k;
}

/* ------------------------------------------------------------------------ */
/* graph.cpp:107-175: triangles per vertex (twice the number of triangles    */
/* through v), edges in at least one triangle, mean local clustering         */
/* coefficient summed in vertex order.                                       */
/* ------------------------------------------------------------------------ */

static int32_t intersect_count(const pcdo_graph *g, int32_t a, int32_t b, const int32_t *labels,
                               int32_t need_label) {
    const int32_t *x = g->adj + g->indices[a], *xe = g->adj + g->indices[a + 1];
    const int32_t *y = g->adj + g->indices[b], *ye = g->adj + g->indices[b + 1];
    int32_t c = 0;
    while (x != xe && y != ye) {
        int32_t d = *x - *y;
        if (d == 0 && (!labels || labels[*x] == need_label)) c++;
        if (d <= 0) x++;
        if (d >= 0) y++;
    }
    return c;
}

void pcdo_count_triangles(const pcdo_graph *g, int32_t *tri, int32_t *tri_deg, double *cc_out) {
    int32_t n = g->n;
    for (int32_t v = 0; v < n; v++) tri[v] = tri_deg[v] = 0;
    for (int32_t v = 0; v < n; v++) {
        for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
            int32_t u = g->adj[e];
            if (u >= v) continue;
            int32_t c = intersect_count(g, v, u, NULL, 0);
            if (c > 0) {
                tri[v] += c;
                tri[u] += c;
                tri_deg[v]++;
                tri_deg[u]++;
            }
        }
    }
    double cc = 0;
    for (int32_t v = 0; v < n; v++) {
        int32_t t = tri[v], deg = degree(g, v);
        if (deg > 1) cc += (t / (deg * (deg - 1.0))) / n;
    }
    *cc_out = cc;
}

/* The same counts with the edge loop on `threads` OpenMP threads: integer
 * sums (atomic adds) do not depend on the order, and the clustering
 * coefficient is still summed in vertex order, so the results are identical
 * to pcdo_count_triangles'. */
void pcdo_count_triangles_mt(const pcdo_graph *g, int32_t *tri, int32_t *tri_deg, double *cc_out,
                             int32_t threads) {
    int32_t n = g->n;
    if (threads < 1) threads = 1;
    for (int32_t v = 0; v < n; v++) tri[v] = tri_deg[v] = 0;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
    for (int32_t v = 0; v < n; v++) {
        for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
            int32_t u = g->adj[e];
            if (u >= v) continue;
            int32_t c = intersect_count(g, v, u, NULL, 0);
            if (c > 0) {
#pragma omp atomic
                tri[v] += c;
#pragma omp atomic
                tri[u] += c;
#pragma omp atomic
                tri_deg[v]++;
#pragma omp atomic
                tri_deg[u]++;
            }
        }
    }
    double cc = 0;
    for (int32_t v = 0; v < n; v++) {
        int32_t t = tri[v], deg = degree(g, v);
        if (deg > 1) cc += (t / (deg * (deg - 1.0))) / n;
    }
    *cc_out = cc;
}

/* ------------------------------------------------------------------------ */
/* rules.cpp                                                                 */
/* ------------------------------------------------------------------------ */

/* rules.cpp:240-389, term by term in the reference's order and types. */
static double wcc_improvement(int32_t n_x, int32_t n_y, int32_t c_x, int32_t c_y, int32_t m_x,
                              int32_t m_y, int32_t m_xy, int32_t b_x, int32_t b_y, double cc) {
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

/* ModularityRule::score_join rules.cpp:34-43; CPMRule rules.cpp:136-139;
 * WCCRule rules.cpp:403-417 */
double pcdo_score_join(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                       int32_t v, int32_t c, int32_t k) {
    if (rule == PCDO_MODULARITY) {
        int32_t m = g->m;
        double e_ij = k / (double)m;
        double a_i = (p->int_volume[c] + p->ext_volume[c]) / (2.0 * m);
        double a_j = degree(g, v) / (2.0 * m);
        return e_ij - 2 * a_i * a_j;
    } else if (rule == PCDO_CPM) {
        return k - lambda * p->sizes[c];
    } else {
        int32_t deg = degree(g, v);
        int32_t size = p->sizes[c];
        int32_t int_edge = p->int_volume[c] / 2;
        int32_t ext_edge = p->ext_volume[c];
        return wcc_improvement(1, size, 1, k, 0, int_edge, k, deg, ext_edge, g->clustering_coef);
    }
}

/* ModularityRule::score_leave rules.cpp:45-56; CPM rules.cpp:141-144;
 * WCC rules.cpp:419-436 */
double pcdo_score_leave(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                        int32_t v, int32_t k) {
    int32_t c = p->labels[v];
    if (rule == PCDO_MODULARITY) {
        int32_t m = g->m;
        int32_t deg = degree(g, v);
        double e_ij = k / (double)m;
        double a_i = (p->int_volume[c] + p->ext_volume[c] - deg) / (2.0 * m);
        double a_j = degree(g, v) / (2.0 * m);
        return -(e_ij - 2 * a_i * a_j);
    } else if (rule == PCDO_CPM) {
        return -(k - lambda * (p->sizes[c] - 1));
    } else {
        int32_t deg = degree(g, v);
        int32_t size = p->sizes[c];
        int32_t int_edge = p->int_volume[c] / 2;
        int32_t ext_edge = p->ext_volume[c];
        return -wcc_improvement(1, size - 1, 1, k, 0, int_edge - k, k, deg, ext_edge - deg + 2 * k,
                                g->clustering_coef);
    }
}

/* ModularityRule::score_merge rules.cpp:24-32; CPM rules.cpp:131-134;
 * WCC rules.cpp:391-401 */
double pcdo_score_merge(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                        int32_t i, int32_t j, int32_t w) {
    if (rule == PCDO_MODULARITY) {
        int32_t m = g->m;
        double e_ij = w / (double)m;
        double a_i = (p->int_volume[i] + p->ext_volume[i]) / (2.0 * m);
        double a_j = (p->int_volume[j] + p->ext_volume[j]) / (2.0 * m);
        return e_ij - 2 * a_i * a_j;
    } else if (rule == PCDO_CPM) {
        return w - lambda * p->sizes[i] * p->sizes[j];
    } else {
        int32_t si = p->sizes[i], sj = p->sizes[j];
        return wcc_improvement(si, sj, w < si ? w : si, w < sj ? w : sj, p->int_volume[i] / 2,
                               p->int_volume[j] / 2, w, p->ext_volume[i], p->ext_volume[j],
                               g->clustering_coef);
    }
}

/* rules.cpp:9-22 (pow(x, 2) is x * x), 121-129, 150-235 */
double pcdo_calculate(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p) {
    int32_t c = p->num_labels;
    if (rule == PCDO_MODULARITY) {
        int32_t m = g->m;
        double mod = 0.0;
        for (int32_t i = 0; i < c; i++) {
            double actual = p->int_volume[i] / (2.0 * m);
            double x = (p->int_volume[i] + p->ext_volume[i]) / (2.0 * m);
            double expect = x * x;
            mod += actual - expect;
        }
        return mod;
    } else if (rule == PCDO_CPM) {
        double score = 0.0;
        for (int32_t i = 0; i < c; i++)
            score += p->int_volume[i] - lambda * p->sizes[i] * (p->sizes[i] - 1);
        return score / (double)(2 * g->m);
    } else {
        int32_t n = g->n;
        const int32_t *labels = p->labels;
        int32_t *it = (int32_t *)calloc(n ? n : 1, sizeof(int32_t));
        int32_t *itd = (int32_t *)calloc(n ? n : 1, sizeof(int32_t));
        for (int32_t v = 0; v < n; v++) {
            int32_t l = labels[v];
            for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
                int32_t u = g->adj[e];
                if (u >= v) break;
                if (labels[u] != l) continue;
                int32_t cnt = intersect_count(g, v, u, labels, l);
                if (cnt > 0) {
                    it[v] += cnt;
                    it[u] += cnt;
                    itd[v]++;
                    itd[u]++;
                }
            }
        }
        double score = 0.0;
        for (int32_t v = 0; v < n; v++) {
            int32_t size = p->sizes[labels[v]];
            int32_t t = g->tri[v], dt = g->tri_deg[v], ti = it[v], dti = itd[v];
            if (t > 0) {
                double a = ti / (double)t;
                double b = dt / (double)(size - 1 + dt - dti);
                score += (a * b) / n;
            }
        }
        free(it);
        free(itd);
        return score;
    }
}

/* pcdo_calculate with WCC's intra-community intersections on `threads` OpenMP
 * threads (atomic integer adds); every FP64 sum keeps pcdo_calculate's order,
 * so the value is identical. */
double pcdo_calculate_mt(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                         int32_t threads) {
    if (threads < 1) threads = 1;
    int32_t c = p->num_labels;
    if (rule == PCDO_MODULARITY) {
        int32_t m = g->m;
        double mod = 0.0;
        for (int32_t i = 0; i < c; i++) {
            double actual = p->int_volume[i] / (2.0 * m);
            double x = (p->int_volume[i] + p->ext_volume[i]) / (2.0 * m);
            double expect = x * x;
            mod += actual - expect;
        }
        return mod;
    } else if (rule == PCDO_CPM) {
        double score = 0.0;
        for (int32_t i = 0; i < c; i++)
            score += p->int_volume[i] - lambda * p->sizes[i] * (p->sizes[i] - 1);
        return score / (double)(2 * g->m);
    } else {
        int32_t n = g->n;
        const int32_t *labels = p->labels;
        int32_t *it = (int32_t *)calloc(n ? n : 1, sizeof(int32_t));
        int32_t *itd = (int32_t *)calloc(n ? n : 1, sizeof(int32_t));
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
        for (int32_t v = 0; v < n; v++) {
            int32_t l = labels[v];
            for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
                int32_t u = g->adj[e];
                if (u >= v) break;
                if (labels[u] != l) continue;
                int32_t cnt = intersect_count(g, v, u, labels, l);
                if (cnt > 0) {
#pragma omp atomic
                    it[v] += cnt;
#pragma omp atomic
                    it[u] += cnt;
#pragma omp atomic
                    itd[v]++;
#pragma omp atomic
                    itd[u]++;
                }
            }
        }
        double score = 0.0;
        for (int32_t v = 0; v < n; v++) {
            int32_t size = p->sizes[labels[v]];
            int32_t t = g->tri[v], dt = g->tri_deg[v], ti = it[v], dti = itd[v];
            if (t > 0) {
                double a = ti / (double)t;
                double b = dt / (double)(size - 1 + dt - dti);
                score += (a * b) / n;
            }
        }
        free(it);
        free(itd);
        return score;
    }
}

/* ------------------------------------------------------------------------ */
/* refinement.cpp:114-182 PropagationRefinement::refine                      */
/* ------------------------------------------------------------------------ */

void pcdo_propagation_refine(int32_t rule, double lambda, const pcdo_graph *g,
                             const pcdo_partition *p, double frac, uint32_t seed0,
                             int32_t threads, int32_t *new_labels, int32_t *draws) {
    const int32_t n = g->n;
    const int32_t f = (int32_t)((frac < 1.0 ? frac : 1.0) * RAND_MAX_GLIBC);
    const int32_t *labels = p->labels;
    if (threads < 1) threads = 1;

#pragma omp parallel num_threads(threads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        uint32_t seed = seed0 ^ (uint32_t)(tid * 0x9E3779B9u);
        otab t;
        otab_init(&t);

#pragma omp for schedule(static, 512)
        for (int32_t v = 0; v < n; v++) {
            int32_t nd = 1;
            if (pcdo_rand_r(&seed) > f) {
                new_labels[v] = labels[v];
                if (draws) draws[v] = nd;
                continue;
            }
            for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++)
                otab_insert(&t, labels[g->adj[e]]);

            int32_t curr = labels[v];
            int32_t best_label = -1, best_count = 0, curr_freq = 0;
            double best_score = 0.0, leave_score;
            for (int32_t i = 0; i < t.size; i++) {
                int32_t label = t.keys[t.order[i]];
                int32_t freq = t.vals[t.order[i]];
                if (label != curr) {
                    double s = pcdo_score_join(rule, lambda, g, p, v, label, freq);
                    if (s > best_score) {
                        best_label = label;
                        best_score = s;
                        best_count = 1;
                    } else if (s == best_score) {
                        nd++;
                        if (pcdo_rand_r(&seed) % (++best_count) == 0) best_label = label;
                    }
                } else {
                    curr_freq = freq;
                }
            }
            otab_clear(&t);
            leave_score = pcdo_score_leave(rule, lambda, g, p, v, curr_freq);
            best_score += leave_score;
            if (best_score > 0 && best_score > leave_score)
                new_labels[v] = best_label;
            else if (leave_score > 0)
                new_labels[v] = NEW_LABEL;
            else
                new_labels[v] = curr;
            if (draws) draws[v] = nd;
        }
        otab_free(&t);
    }
}

/* ------------------------------------------------------------------------ */
/* refinement.cpp:185-288 MergingRefinement::refine                          */
/* ------------------------------------------------------------------------ */

void pcdo_merging_refine(int32_t rule, double lambda, const pcdo_graph *g,
                         const pcdo_partition *p, int32_t rounds, uint32_t seed0,
                         int32_t threads, int32_t *new_labels, int32_t *best_out) {
    const int32_t n = g->n;
    const int32_t k = p->num_labels;
    const int32_t *labels = p->labels;
    if (threads < 1) threads = 1;

    /* members of each community in vertex order (refinement.cpp:190-202) */
    int32_t *members = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    int32_t *start = (int32_t *)malloc(sizeof(int32_t) * (k + 2));
    start[0] = 0;
    start[1] = 0;
    for (int32_t i = 2; i < k + 1; i++) start[i] = start[i - 1] + p->sizes[i - 2];
    for (int32_t v = 0; v < n; v++) members[start[labels[v] + 1]++] = v;

    int32_t *best = (int32_t *)malloc(sizeof(int32_t) * (k ? k : 1));
    char *found = (char *)malloc(k ? k : 1);
    for (int32_t i = 0; i < k; i++) {
        best[i] = -1;
        found[i] = 0;
    }
    int all_done = 0;

#pragma omp parallel num_threads(threads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        uint32_t seed = seed0 ^ (uint32_t)(tid * 0x9E3779B9u);
        otab t;
        otab_init(&t);

        for (int32_t rnd = 0; rnd < rounds && !all_done; rnd++) {
#pragma omp for schedule(dynamic, 256)
            for (int32_t l = 0; l < k; l++) {
                if (found[l] || (best[l] != -1 && !found[best[l]])) continue;
                for (int32_t i = start[l]; i != start[l + 1]; i++) {
                    int32_t v = members[i];
                    for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
                        int32_t kk = labels[g->adj[e]];
                        if (kk != l && !found[kk]) otab_insert(&t, kk);
                    }
                }
                int32_t best_label = -1, count = 1;
                double best_score = 0;
                for (int32_t i = 0; i < t.size; i++) {
                    int32_t label = t.keys[t.order[i]];
                    int32_t freq = t.vals[t.order[i]];
                    double s = pcdo_score_merge(rule, lambda, g, p, l, label, freq);
                    if (s == best_score) {
                        if (pcdo_rand_r(&seed) % (count++) == 0) best_label = label;
                    } else if (s > best_score) {
                        best_label = label;
                        best_score = s;
                        count = 1;
                    }
                }
                best[l] = best_label;
                otab_clear(&t);
            }
#pragma omp single
            all_done = 1;
            int local_done = 1;
#pragma omp for schedule(static, 512)
            for (int32_t l = 0; l < k; l++) {
                if (!found[l] && (best[l] == -1 || best[best[l]] == l)) found[l] = 1;
                local_done &= found[l];
            }
#pragma omp atomic
            all_done &= local_done;
#pragma omp barrier
        }

#pragma omp for schedule(static, 512)
        for (int32_t v = 0; v < n; v++) {
            int32_t l = labels[v];
            if (found[l] && best[l] != -1)
                new_labels[v] = l < best[l] ? l : best[l];
            else
                new_labels[v] = l;
        }
        otab_free(&t);
    }
    if (best_out)
        for (int32_t i = 0; i < k; i++) best_out[i] = found[i] ? best[i] : -2;
    free(members);
    free(start);
    free(best);
    free(found);
}

/* ------------------------------------------------------------------------ */
/* contracted edge weights (the per-pair counts the merge phase histograms,   */
/* refinement.cpp:228-238, over every community at once)                     */
/* ------------------------------------------------------------------------ */

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : (x > y);
}

int64_t pcdo_contract(const pcdo_graph *g, const pcdo_partition *p, int64_t cap, int32_t *ca,
                      int32_t *cb, int32_t *w) {
    int64_t ne = 0;
    const int32_t *labels = p->labels;
    for (int32_t v = 0; v < g->n; v++)
        for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++)
            if (labels[g->adj[e]] != labels[v]) ne++;
    int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (ne ? ne : 1));
    int64_t j = 0;
    for (int32_t v = 0; v < g->n; v++)
        for (int32_t e = g->indices[v]; e < g->indices[v + 1]; e++) {
            int32_t a = labels[v], b = labels[g->adj[e]];
            if (a != b) keys[j++] = ((int64_t)a << 32) | (uint32_t)b;
        }
    qsort(keys, ne, sizeof(int64_t), cmp_i64);
    int64_t np = 0;
    for (int64_t i = 0; i < ne;) {
        int64_t s = i;
        while (i < ne && keys[i] == keys[s]) i++;
        if (np < cap) {
            ca[np] = (int32_t)(keys[s] >> 32);
            cb[np] = (int32_t)(keys[s] & 0xffffffff);
            w[np] = (int32_t)(i - s);
        }
        np++;
    }
    free(keys);
    return np;
}
