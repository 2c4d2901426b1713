// main-cuda: the drop-in driver.  Command line and output of the reference's
// CPU driver (src/main.cpp:20-287, a superset of src/main-cuda.cu:11-102's
// flags), with every phase on the GPU through libpcd:
//
//   main-cuda <graph> [-m mod|wcc|cpm-<gamma>] [-f frac] [-r rounds] [-t thr]
//             [-n iters] [-i 0|1] [-s 0|1|2] [-p threads (accepted, unused)]
//
// The seed stream is the reference's (glibc rand() from the default seed: n
// draws for the singleton partition, one per refinement call), so labels and
// scores match the reference CPU driver run with -p 1.  Final labels go to
// stderr as "map[v] label[v]" lines (src/main.cpp:282-284).
#include <sys/time.h>
#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/pcd.h"

namespace {

double now() {
    struct timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + t.tv_usec / 1e6;
}

struct Timer {
    std::vector<double> stack;
    void start() { stack.push_back(now()); }
    double end() {
        if (stack.empty()) return 0.0;
        double t = now() - stack.back();
        stack.pop_back();
        return t;
    }
};

struct HostGraph {
    int32_t n = 0, m = 0;
    std::vector<int32_t> indices, adj, map;
};

// Graph::read (src/graph.cpp:40-105): "PCD", n, m, indices[n+1], adj[2m],
// map[n], and nothing after.
bool read_graph(const char *path, HostGraph &g) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        std::cerr << "failed to open " << path << std::endl;
        return false;
    }
    char magic[3];
    bool ok = fread(magic, 1, 3, f) == 3 && memcmp(magic, "PCD", 3) == 0;
    if (!ok) {
        std::cerr << "invalid file type" << std::endl;
        fclose(f);
        return false;
    }
    ok = fread(&g.n, 4, 1, f) == 1 && fread(&g.m, 4, 1, f) == 1 && g.n >= 0 && g.m >= 0;
    if (ok) {
        g.indices.resize((size_t)g.n + 1);
        g.adj.resize(2 * (size_t)g.m);
        g.map.resize((size_t)g.n);
        ok = fread(g.indices.data(), 4, g.indices.size(), f) == g.indices.size() &&
             fread(g.adj.data(), 4, g.adj.size(), f) == g.adj.size() &&
             fread(g.map.data(), 4, g.map.size(), f) == g.map.size();
        char extra;
        ok = ok && fread(&extra, 1, 1, f) == 0;
    }
    fclose(f);
    if (!ok) std::cerr << "error while reading " << path << std::endl;
    return ok;
}

void usage(const char *prog) {
    std::cerr << "usage: " << prog << " <graph> [options]\n\n"
              << "options:\n"
              << "-m <metric>      mod | wcc | cpm-<gamma>\n"
              << "-p <#threads>    accepted for compatibility (the GPU path ignores it)\n"
              << "-f <fraction>    fraction of vertices to update per propagation sweep\n"
              << "-r <#rounds>     rounds of parallel merging\n"
              << "-t <threshold>   iteration threshold\n"
              << "-n <#iterations> total number of iterations (disables -t)\n"
              << "-i 0/1           initial partition: 0 unique labels, 1 triangle-based\n"
              << "-s <schedule>    0 propagation, 1 merging, 2 alternate\n"
              << "-d <device>      CUDA device (default 0)\n"
              << "-h               print this help message\n"
              << std::endl;
}

std::string rule_name(const pcd_rule &r) {
    if (r.kind == PCD_RULE_MODULARITY) return "modularity";
    if (r.kind == PCD_RULE_WCC) return "WCC";
    char buf[64];
    snprintf(buf, sizeof buf, "CPM (lambda=%g)", r.lambda);
    return buf;
}

#define CHECK(call)                                                                               \
    do {                                                                                          \
        pcd_status _s = (call);                                                                   \
        if (_s != PCD_OK) {                                                                       \
            std::cerr << #call << ": " << pcd_status_string(_s) << ": " << pcd_last_error(ctx)    \
                      << std::endl;                                                               \
            return 2;                                                                             \
        }                                                                                         \
    } while (0)

}  // namespace

int main(int argc, char **argv) {
    int c;
    double frac = 0.5, threshold = 0.0;
    int rounds = 1, max_iter = -1, initial = 0, strategy = 0, device = 0;
    pcd_rule rule{PCD_RULE_MODULARITY, 0.0};
    while ((c = getopt(argc, argv, "?hr:f:m:p:t:s:i:n:d:")) != -1) {
        switch (c) {
            case 'p':
                if (atoi(optarg) < 0) {
                    std::cerr << "number of threads should be positive" << std::endl;
                    return 255;
                }
                break;
            case 'r':
                rounds = atoi(optarg);
                if (rounds <= 0) {
                    std::cerr << "number of rounds should be positive" << std::endl;
                    return 255;
                }
                break;
            case 'n': max_iter = atoi(optarg); break;
            case 'i': initial = atoi(optarg); break;
            case 'd': device = atoi(optarg); break;
            case 'f':
                frac = atof(optarg);
                if (frac <= 0 || frac > 1) {
                    std::cerr << "fraction should be between 0.0 and 1.0" << std::endl;
                    return 255;
                }
                break;
            case 't':
                threshold = atof(optarg);
                if (threshold < 0 || threshold > 1) {
                    std::cerr << "threshold should be between 0.0 and 1.0" << std::endl;
                    return 255;
                }
                break;
            case 's': strategy = atoi(optarg); break;
            case 'm': {
                for (int i = 0; optarg[i]; i++) optarg[i] = (char)tolower(optarg[i]);
                if (!strcmp(optarg, "mod") || !strcmp(optarg, "modularity")) {
                    rule = pcd_rule{PCD_RULE_MODULARITY, 0.0};
                } else if (!strcmp(optarg, "wcc")) {
                    rule = pcd_rule{PCD_RULE_WCC, 0.0};
                } else if (!strncmp(optarg, "cpm-", 4) && optarg[4]) {
                    rule = pcd_rule{PCD_RULE_CPM, atof(optarg + 4)};
                } else {
                    std::cerr << "unknown metric: " << optarg << std::endl;
                    return 255;
                }
                break;
            }
            default:
                usage(argv[0]);
                return 255;
        }
    }
    if (optind >= argc) {
        usage(argv[0]);
        return 255;
    }
    if (initial != 0 && initial != 1) {
        std::cerr << "unknown partitioning strategy" << std::endl;
        return 255;
    }
    Timer timer;
    const char *path = argv[optind];
    std::cout << "loading graph..." << std::endl;
    timer.start();
    HostGraph hg;
    if (!read_graph(path, hg)) {
        std::cerr << "error while loading graph" << std::endl;
        return 255;
    }
    pcd_ctx *ctx = nullptr;
    if (pcd_init(&ctx, device) != PCD_OK) {
        std::cerr << "CUDA init failed: " << (ctx ? pcd_last_error(ctx) : "") << std::endl;
        return 2;
    }
    pcd_graph *g = nullptr;
    CHECK(pcd_load_csr(ctx, hg.n, hg.m, hg.indices.data(), hg.adj.data(), &g));
    const double time_load = timer.end();
    const int32_t n = hg.n;
    std::cout << "-------------------------------------------------" << std::endl;
    std::cout << "loaded graph from " << path << std::endl;
    std::cout << "num nodes: " << n << std::endl;
    std::cout << "num edges: " << hg.m << std::endl;
    std::cout << "avg. degree: " << double(2 * hg.m) / n << std::endl;
    std::cout << "max. degree: " << (n ? hg.indices[1] - hg.indices[0] : 0) << std::endl;
    std::cout << "-------------------------------------------------" << std::endl;

    std::vector<int32_t> labels((size_t)n);
    pcd_rand rnd;
    pcd_rand_seed(&rnd, 1);
    std::cout << "creating initial partitioning..." << std::endl;
    timer.start();
    if (initial == 1 || rule.kind == PCD_RULE_WCC) {
        timer.start();
        CHECK(pcd_triangles(g, nullptr, nullptr, nullptr));
        std::cout << "count triangles: " << timer.end() << std::endl;
    }
    if (initial == 0) {
        CHECK(pcd_singleton_partition(&rnd, n, labels.data()));
        CHECK(pcd_labels_set(g, labels.data()));
    } else {
        CHECK(pcd_clustering_partition_device(g, nullptr));  // create_clustering_partition's labels
    }
    const double time_initial = timer.end();

    double prev_score = 0.0, score = 0.0;
    bool done = false;
    int it = 0;
    int32_t k = 0;
    std::cout << "refining partitioning..." << std::endl;
    timer.start();
    while (!done) {
        timer.start();
        timer.start();
        CHECK(pcd_compress(g, &k));
        std::cout << " - collecting statistics: " << timer.end() << " sec" << std::endl;
        timer.start();
        CHECK(pcd_score(g, &rule, &score));
        std::cout << " - calculate metric: " << timer.end() << " sec" << std::endl;
        std::cout << " - " << rule_name(rule) << ": " << score << std::endl;
        std::cout << " - improv. of prev. iteration: " << (score / prev_score - 1) * 100 << "%" << std::endl;
        done = max_iter != -1 ? it >= max_iter
                              : (prev_score > 0 && score > 0 && score / prev_score - 1 <= threshold);
        if (!done) {
            const uint32_t seed = (uint32_t)pcd_rand_next(&rnd);
            if (strategy == 0 || (strategy == 2 && it % 2 == 0)) {
                timer.start();
                CHECK(pcd_refine(g, &rule, frac, seed));
                CHECK(pcd_synchronize(ctx));
                std::cout << " - label propagation: " << timer.end() << " sec" << std::endl;
            } else {
                timer.start();
                CHECK(pcd_merge(g, &rule, rounds, seed));
                CHECK(pcd_synchronize(ctx));
                std::cout << " - parallel merging: " << timer.end() << " sec" << std::endl;
            }
        }
        std::cout << "iteration " << (it + 1) << ": " << timer.end() << " sec" << std::endl;
        it++;
        prev_score = score;
    }
    const double time_refine = timer.end();
    std::vector<int32_t> sizes((size_t)std::max(k, 1));
    CHECK(pcd_stats_get(g, sizes.data(), nullptr, nullptr));
    CHECK(pcd_labels_get(g, labels.data()));
    std::cout << "-------------------------------------------------" << std::endl;
    std::cout << "time read graph: " << time_load << " sec" << std::endl;
    std::cout << "time initial partitioning: " << time_initial << " sec" << std::endl;
    std::cout << "time refinement phase: " << time_refine << " sec" << std::endl;
    std::cout << "refinement iterations: " << it << std::endl;
    std::cout << "avg. time per iteration: " << time_refine / it << " sec" << std::endl;
    std::cout << rule_name(rule) << ": " << prev_score << std::endl;
    std::cout << "num. communities: " << k << std::endl;
    std::cout << "avg. community size: " << double(n) / k << std::endl;
    std::cout << "largest community size: " << (k ? *std::max_element(sizes.begin(), sizes.begin() + k) : 0)
              << std::endl;
    std::cout << "-------------------------------------------------" << std::endl;
    for (int32_t i = 0; i < n; i++) std::cerr << hg.map[(size_t)i] << " " << labels[(size_t)i] << "\n";
    std::cerr.flush();
    pcd_destroy(ctx);
    return 1;  // the reference driver exits with 1 (src/main.cpp:286)
}
