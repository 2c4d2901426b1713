// Host-side parts of the driver loop that the reference also runs on the
// host: the glibc rand() seed stream and the two initial partitions
// (src/framework.cpp:14-59).
//
// Seed stream.  The reference driver seeds every
// refinement call with glibc rand() (src/refinement.cpp:123-124, 217-218) after
// create_singleton_partition consumed n values (src/framework.cpp:21-23), all
// from glibc's default seed.  This is that generator restated from its
// published description (TYPE_3 additive feedback: r[i] = r[i-3] + r[i-31]
// mod 2^32, state seeded by the 16807 multiplicative LCG mod 2^31 - 1, 310
// values discarded, outputs r >> 1), so a driver reproduces the reference's
// seeds without touching the process-wide libc state.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#include "../../include/pcd.h"

extern "C" {

void pcd_rand_seed(pcd_rand *s, uint32_t seed) {
    if (!s) return;
    int64_t w = (int32_t)(seed == 0 ? 1u : seed);
    s->r[0] = (uint32_t)w;
    for (int i = 1; i < 31; ++i) {
        int64_t x = (16807 * w) % 2147483647;
        if (x < 0) x += 2147483647;
        w = x;
        s->r[i] = (uint32_t)w;
    }
    for (int i = 31; i < 34; ++i) s->r[i] = s->r[i - 31];
    s->pos = 0;
    for (int i = 0; i < 310; ++i) (void)pcd_rand_next(s);
}

int32_t pcd_rand_next(pcd_rand *s) {
    const int32_t i = s->pos;
    const uint32_t v = s->r[(i + 3) % 34] + s->r[(i + 31) % 34];
    s->r[i] = v;
    s->pos = (i + 1) % 34;
    return (int32_t)(v >> 1);
}

void pcd_rand_skip(pcd_rand *s, int64_t count) {
    for (int64_t i = 0; i < count; ++i) (void)pcd_rand_next(s);
}

// create_singleton_partition (src/framework.cpp:14-24): identity, then n
// swaps with rand() % n.
pcd_status pcd_singleton_partition(pcd_rand *s, int32_t n, int32_t *labels) {
    if (!s || n < 0 || (n > 0 && !labels)) return PCD_ERR_INVALID_ARGUMENT;
    for (int32_t v = 0; v < n; ++v) labels[v] = v;
    for (int32_t v = 0; v < n; ++v) std::swap(labels[v], labels[pcd_rand_next(s) % n]);
    return PCD_OK;
}

// create_clustering_partition (src/framework.cpp:27-59): vertices by
// decreasing local clustering tri / (deg (deg - 1)) (the product in int, as
// the reference computes it), then decreasing degree, then id; each unlabelled
// vertex claims itself and its unlabelled neighbours.
pcd_status pcd_clustering_partition(int32_t n, const int32_t *indices, const int32_t *adj, const int32_t *tri,
                                    int32_t *labels) {
    if (n < 0 || (n > 0 && (!indices || !tri || !labels))) return PCD_ERR_INVALID_ARGUMENT;
    struct Key {
        double ncc;
        int32_t ndeg, v;
    };
    std::vector<Key> keys((size_t)n);
    for (int32_t v = 0; v < n; ++v) {
        const int32_t deg = indices[v + 1] - indices[v];
        const int32_t prod = (int32_t)((uint32_t)deg * (uint32_t)(deg - 1));
        const double cc = deg > 1 ? tri[v] / (double)prod : 0.0;
        keys[(size_t)v] = Key{-cc, -deg, v};
    }
    std::sort(keys.begin(), keys.end(), [](const Key &a, const Key &b) {
        if (a.ncc < b.ncc) return true;
        if (b.ncc < a.ncc) return false;
        if (a.ndeg != b.ndeg) return a.ndeg < b.ndeg;
        return a.v < b.v;
    });
    for (int32_t v = 0; v < n; ++v) labels[v] = PCD_NEW_LABEL;
    int32_t num = 0;
    for (const Key &k : keys) {
        if (labels[k.v] != PCD_NEW_LABEL) continue;
        labels[k.v] = num;
        for (int32_t j = indices[k.v]; j < indices[k.v + 1]; ++j)
            if (labels[adj[j]] == PCD_NEW_LABEL) labels[adj[j]] = num;
        ++num;
    }
    return PCD_OK;
}

}  // extern "C"
