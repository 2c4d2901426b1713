// The reference's GPU host API (src/framework-cuda.cuh:14-23) implemented
// over libpcd, as a maintainer switching src/main-cuda.cu to this library
// would write it, plus a small driver that runs the reference's schedule
// (src/main.cpp:226-266) through those functions and writes every sweep's
// labels.  Compiled by the tests against the reference's own graph.hpp where
// the reference sources are present, and otherwise against a minimal
// stand-in Graph with the same members (tests/shim/graph_stand_in/).
//
// Differences from the reference's declarations: a rule is the plain
// pcd_rule descriptor instead of the CudaRule class hierarchy
// (src/rules-cuda.cuh:23-30, whose GPU code is not part of this library), and
// the propagation / merge seeds are drawn inside, from the same glibc rand()
// stream the reference CPU driver draws them from (seed 1, after the
// singleton partition's n values; src/refinement.cpp:123-124, 217-218).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "graph.hpp"
#include "pcd.h"

static pcd_ctx *ctx = nullptr;
static pcd_graph *dev_graph = nullptr;
static pcd_rand seeds;

bool cuda_init(int device_id, int group_size) {  // framework-cuda.cu:59
    (void)group_size;
    return pcd_init(&ctx, device_id) == PCD_OK;
}

bool cuda_deinit(void) { return pcd_destroy(ctx) == PCD_OK; }

bool cuda_transfer_graph(const Graph &g) {  // framework-cuda.cu:89
    if (dev_graph) pcd_graph_free(dev_graph);
    pcd_rand_seed(&seeds, 1);
    pcd_rand_skip(&seeds, g.n);  // create_singleton_partition's draws
    return pcd_load_csr(ctx, g.n, g.m, g.indices, g.adj, &dev_graph) == PCD_OK;
}

bool cuda_labels_to_device(int *labels) { return pcd_labels_set(dev_graph, labels) == PCD_OK; }
bool cuda_labels_from_device(int *labels) { return pcd_labels_get(dev_graph, labels) == PCD_OK; }
bool cuda_collect_statistics(void) { return pcd_compress(dev_graph, nullptr) == PCD_OK; }

bool cuda_propagation_step(double frac, const pcd_rule &r) {
    return pcd_refine(dev_graph, &r, frac, (uint32_t)pcd_rand_next(&seeds)) == PCD_OK;
}

bool cuda_merging_step(int rounds, const pcd_rule &r) {
    return pcd_merge(dev_graph, &r, rounds, (uint32_t)pcd_rand_next(&seeds)) == PCD_OK;
}

float cuda_calculate_metric(const pcd_rule &r) {
    double s = 0.0;
    pcd_score(dev_graph, &r, &s);
    return (float)s;
}

// driver: shim <csr file> <out file> <rule 0|1> <lambda> <strategy> <iterations>
// csr file: int32 n, int32 m, indices[n + 1], adj[2m]; out: per sweep, n int32 labels
int main(int argc, char **argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s csr out rule lambda strategy iterations\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t nm[2];
    if (std::fread(nm, sizeof(int32_t), 2, f) != 2) return 2;
    int *indices = new int[(size_t)nm[0] + 1];
    int *adj = new int[2 * (size_t)nm[1] + 1];
    if (std::fread(indices, sizeof(int32_t), (size_t)nm[0] + 1, f) != (size_t)nm[0] + 1 ||
        std::fread(adj, sizeof(int32_t), 2 * (size_t)nm[1], f) != 2 * (size_t)nm[1])
        return 2;
    std::fclose(f);
    // the reference's Graph owns (and frees) its arrays
    const Graph *g = new Graph(nm[0], nm[1], adj, indices, nullptr, nullptr);
    const pcd_rule rule{std::atoi(argv[3]), std::atof(argv[4])};
    const int strategy = std::atoi(argv[5]), iters = std::atoi(argv[6]);
    if (!cuda_init(0, 1) || !cuda_transfer_graph(*g)) return 1;
    std::vector<int> labels((size_t)g->n);
    pcd_rand start;
    pcd_rand_seed(&start, 1);
    pcd_singleton_partition(&start, g->n, labels.data());  // create_singleton_partition
    if (!cuda_labels_to_device(labels.data())) return 1;
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    for (int it = 0; it < iters; ++it) {
        if (!cuda_collect_statistics()) return 1;
        (void)cuda_calculate_metric(rule);
        const bool prop = strategy == 0 || (strategy == 2 && it % 2 == 0);
        if (!(prop ? cuda_propagation_step(1.0, rule) : cuda_merging_step(1, rule))) return 1;
        if (!cuda_labels_from_device(labels.data())) return 1;
        std::fwrite(labels.data(), sizeof(int32_t), labels.size(), out);
    }
    std::fclose(out);
    delete g;
    return cuda_deinit() ? 0 : 1;
}
