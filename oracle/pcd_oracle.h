/* CPU restatement of the reference's refine / merge / score path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU path is
 * compared against (tests/, __graft_entry__.smoke) and the timed CPU baseline
 * (bench.py's cpu_baseline leg and its reference arm).  The product never
 * links, loads or calls it.
 *
 * Parity is pinned: tests/test_oracle_pin.py runs the reference's own CPU
 * objects (built from the reference sources by oracle/Makefile into
 * oracle/_ref/) beside this file on seeded graphs and requires identical
 * labels after every sweep, identical statistics and identical FP64 gains;
 * tests/golden/ holds the hashes produced by the reference itself.
 *
 * All functions take plain arrays.  Labels are int32; NEW_LABEL is -1
 * (src/common.hpp:20 defines it as ~0).
 */
#ifndef PCD_ORACLE_H
#define PCD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { PCDO_MODULARITY = 0, PCDO_CPM = 1, PCDO_WCC = 2 };

typedef struct {
    int32_t n, m;
    const int32_t *indices; /* n + 1 */
    const int32_t *adj;     /* 2m    */
    const int32_t *tri;     /* n, WCC only (may be NULL otherwise) */
    const int32_t *tri_deg; /* n, WCC only */
    double clustering_coef; /* WCC only */
} pcdo_graph;

typedef struct {
    int32_t num_labels;
    const int32_t *labels; /* n, compressed */
    const int32_t *sizes;  /* num_labels */
    const int32_t *int_volume;
    const int32_t *ext_volume;
} pcdo_partition;

/* glibc rand() (TYPE_3 additive feedback) and rand_r() restated. */
typedef struct {
    uint32_t r[34];
    int32_t pos;
} pcdo_rand_state;
void pcdo_srand(pcdo_rand_state *s, uint32_t seed);
int32_t pcdo_rand(pcdo_rand_state *s);
int32_t pcdo_rand_r(uint32_t *seed);

/* framework.cpp */
void pcdo_singleton_partition(const pcdo_graph *g, pcdo_rand_state *rs, int32_t *labels);
void pcdo_clustering_partition(const pcdo_graph *g, int32_t *labels);
/* FindConnectedRefinement::refine (refinement.cpp:291-322) */
void pcdo_find_connected(const pcdo_graph *g, int32_t *labels);
/* norm_mutual_info over the (a[i], b[i]) confusion map (common.cpp:75-125,
 * 163-173); n is g.n.  Labels >= 0. */
double pcdo_norm_mutual_info(int64_t count, const int32_t *a, const int32_t *b, int32_t n);
int32_t pcdo_compress_labels(int32_t n, int32_t *labels);
int32_t pcdo_collect_statistics(const pcdo_graph *g, const int32_t *labels, int32_t *sizes,
                                int32_t *int_volume, int32_t *ext_volume);

/* graph.cpp */
void pcdo_count_triangles(const pcdo_graph *g, int32_t *tri, int32_t *tri_deg, double *cc);
/* the same results with the edge loop on `threads` OpenMP threads */
void pcdo_count_triangles_mt(const pcdo_graph *g, int32_t *tri, int32_t *tri_deg, double *cc, int32_t threads);

/* rules.cpp */
double pcdo_calculate(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p);
/* the same value with WCC's intersections on `threads` OpenMP threads */
double pcdo_calculate_mt(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                         int32_t threads);
double pcdo_score_join(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                       int32_t v, int32_t c, int32_t k);
double pcdo_score_leave(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                        int32_t v, int32_t k);
double pcdo_score_merge(int32_t rule, double lambda, const pcdo_graph *g, const pcdo_partition *p,
                        int32_t a, int32_t b, int32_t w);

/* refinement.cpp.  `seed` is the value the reference draws with rand() at the
 * start of the call.  threads == 1 is the reference's -p 1 schedule (bit-exact);
 * threads > 1 runs the same loops in parallel for timing (per-thread seeds are
 * derived from `seed`, so labels differ, as they do for the reference at -p > 1).
 * draws (optional, n entries for propagation / num_labels for merging) receives
 * the number of rand_r calls each vertex / community made. */
void pcdo_propagation_refine(int32_t rule, double lambda, const pcdo_graph *g,
                             const pcdo_partition *p, double frac, uint32_t seed,
                             int32_t threads, int32_t *new_labels, int32_t *draws);
void pcdo_merging_refine(int32_t rule, double lambda, const pcdo_graph *g,
                         const pcdo_partition *p, int32_t rounds, uint32_t seed,
                         int32_t threads, int32_t *new_labels, int32_t *best_partner);

/* Contracted edge weights of a partition: every ordered pair (a, b), a != b,
 * of communities joined by w > 0 edges, sorted by (a, b).  Returns the pair
 * count; writes at most `cap` triples. */
int64_t pcdo_contract(const pcdo_graph *g, const pcdo_partition *p, int64_t cap,
                      int32_t *ca, int32_t *cb, int32_t *w);

#ifdef __cplusplus
}
#endif
#endif
