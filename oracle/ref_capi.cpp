// C shim over the reference's own CPU objects (graph.o common.o rules.o
// framework.o refinement.o, compiled from the reference sources by
// oracle/Makefile).  It exists only so that tests can drive the reference one
// phase at a time from Python (ctypes) and read every intermediate array.
//
// Test infrastructure: nothing in the product links or loads this file.
//
// Every function calls the reference implementation unmodified:
//   ref_compress        -> compress_labels            src/framework.cpp:146-170
//   ref_stats           -> collect_statistics         src/framework.cpp:69-143
//   ref_score           -> Rule::calculate            src/rules.cpp:9-22,121-129,150-235
//   ref_refine_prop     -> PropagationRefinement      src/refinement.cpp:114-182
//   ref_refine_merge    -> MergingRefinement          src/refinement.cpp:185-288
//   ref_count_triangles -> Graph::count_triangles     src/graph.cpp:107-175
//   ref_singleton / ref_clustering -> framework.cpp:14-24 / 27-59
//   ref_gain_*          -> Rule::score_join/leave/merge (rules.cpp)
//   ref_find_connected  -> FindConnectedRefinement    src/refinement.cpp:291-322
//   ref_compare         -> compare_communities(g,a,b) src/common.cpp:75-125,163-173
//   ref_compare_file    -> compare_communities(g,l,f) src/common.cpp:127-160
// glibc rand() is the process-global stream the reference draws its seeds
// from; ref_srand / ref_rand expose it.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>

#include "graph.hpp"
#include "common.hpp"
#include "framework.hpp"
#include "refinement.hpp"
#include "rules.hpp"

namespace {

struct RefGraph {
    Graph *g;
};

Rule *make_rule(int kind, double lambda) {
    switch (kind) {
        case 0: return new ModularityRule();
        case 1: return new CPMRule(lambda);
        case 2: return new WCCRule();
        default: return 0;
    }
}

// Partition over a private copy of `labels`, with statistics collected the
// way main.cpp does it (compress first is the caller's business).
Partition *make_partition(const Graph *g, const int *labels, int threads) {
    int *l = new int[g->n];
    std::memcpy(l, labels, sizeof(int) * g->n);
    Partition *p = new Partition(l);
    collect_statistics(*g, *p, threads);
    return p;
}

}  // namespace

extern "C" {

void *ref_graph_new(int n, int m, const int *indices, const int *adj) {
    int *ind = new int[n + 1];
    int *a = new int[2 * (size_t)m > 0 ? 2 * (size_t)m : 1];
    std::memcpy(ind, indices, sizeof(int) * (n + 1));
    std::memcpy(a, adj, sizeof(int) * 2 * (size_t)m);
    RefGraph *rg = new RefGraph;
    rg->g = new Graph(n, m, a, ind, NULL, NULL, NULL);
    return rg;
}

void ref_graph_free(void *h) {
    RefGraph *rg = (RefGraph *)h;
    delete rg->g;
    delete rg;
}

void ref_count_triangles(void *h, int threads, int *tri, int *tri_deg, double *cc) {
    const Graph *g = ((RefGraph *)h)->g;
    g->count_triangles(threads);
    if (tri) std::memcpy(tri, g->tri, sizeof(int) * g->n);
    if (tri_deg) std::memcpy(tri_deg, g->tri_deg, sizeof(int) * g->n);
    if (cc) *cc = g->clustering_coef;
}

void ref_srand(unsigned s) { srand(s); }
int ref_rand(void) { return rand(); }
int ref_rand_r(unsigned *state) { return rand_r(state); }

void ref_singleton(void *h, int *labels) {
    create_singleton_partition(*((RefGraph *)h)->g, labels);
}

void ref_clustering(void *h, int *labels) {
    create_clustering_partition(*((RefGraph *)h)->g, labels);
}

int ref_compress(void *h, int *labels) {
    return compress_labels(*((RefGraph *)h)->g, labels);
}

// labels must already be compressed (0..k-1); writes k and the three arrays
// (each of capacity >= k).
int ref_stats(void *h, const int *labels, int threads, int *sizes, int *int_vol, int *ext_vol) {
    const Graph *g = ((RefGraph *)h)->g;
    Partition *p = make_partition(g, labels, threads);
    int k = p->num_labels;
    if (sizes) std::memcpy(sizes, p->sizes, sizeof(int) * k);
    if (int_vol) std::memcpy(int_vol, p->int_volume, sizeof(int) * k);
    if (ext_vol) std::memcpy(ext_vol, p->ext_volume, sizeof(int) * k);
    delete p;
    return k;
}

double ref_score(void *h, int rule, double lambda, const int *labels, int threads) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, threads);
    double s = r->calculate(*g, *p);
    delete p;
    delete r;
    return s;
}

void ref_refine_prop(void *h, int rule, double lambda, const int *labels, double frac,
                     int threads, int *new_labels) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, threads);
    PropagationRefinement pr(frac, threads);
    pr.refine(*g, *p, *r, new_labels);
    delete p;
    delete r;
}

void ref_refine_merge(void *h, int rule, double lambda, const int *labels, int rounds,
                      int threads, int *new_labels) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, threads);
    MergingRefinement mr(rounds, threads);
    mr.refine(*g, *p, *r, new_labels);
    delete p;
    delete r;
}

void ref_find_connected(void *h, const int *labels, int threads, int *new_labels) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(0, 0.0);
    Partition *p = make_partition(g, labels, threads);
    FindConnectedRefinement fc(threads);
    fc.refine(*g, *p, *r, new_labels);
    delete p;
    delete r;
}

double ref_compare(void *h, int *a, int *b) {
    return compare_communities(*((RefGraph *)h)->g, a, b);
}

double ref_compare_file(void *h, int *labels, const char *path) {
    return compare_communities(*((RefGraph *)h)->g, labels, std::string(path));
}

// Single gain evaluations on a partition (for rule-level unit checks).
double ref_gain_join(void *h, int rule, double lambda, const int *labels, int v, int c, int k) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, 1);
    double s = r->score_join(*g, *p, v, c, k);
    delete p;
    delete r;
    return s;
}

double ref_gain_leave(void *h, int rule, double lambda, const int *labels, int v, int k) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, 1);
    double s = r->score_leave(*g, *p, v, k);
    delete p;
    delete r;
    return s;
}

double ref_gain_merge(void *h, int rule, double lambda, const int *labels, int a, int b, int w) {
    const Graph *g = ((RefGraph *)h)->g;
    Rule *r = make_rule(rule, lambda);
    Partition *p = make_partition(g, labels, 1);
    double s = r->score_merge(*g, *p, a, b, w);
    delete p;
    delete r;
    return s;
}

}  // extern "C"
