// convert-cuda: the reference converter's command line (src/convert.cpp:281)
// with the CSR built on the GPU.  Reads a text edge list (one "a b" pair of
// non-negative ids per line, '#' comment lines and blank lines skipped, like
// src/convert.cpp:17-64) and writes the "PCD" file: magic, n, m, indices,
// adjacency, map (src/convert.cpp:244-278).
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pcd.h"

static bool read_edges(const char *path, std::vector<int32_t> &src, std::vector<int32_t> &dst) {
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        std::fprintf(stderr, "failed to open %s\n", path);
        return false;
    }
    std::vector<char> buf;
    char tmp[1 << 16];
    size_t r;
    while ((r = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    std::fclose(f);
    buf.push_back('\n');
    size_t i = 0;
    long line = 0;
    while (i < buf.size()) {
        ++line;
        size_t e = i;
        while (e < buf.size() && buf[e] != '\n') ++e;
        size_t p = i;
        while (p < e && std::isspace((unsigned char)buf[p])) ++p;
        if (p < e && buf[p] != '#') {
            int64_t v[2];
            for (int k = 0; k < 2; ++k) {
                if (p >= e || !std::isdigit((unsigned char)buf[p])) {
                    std::fprintf(stderr, "line %ld is corrupt\n", line);
                    return false;
                }
                int64_t a = 0;
                while (p < e && std::isdigit((unsigned char)buf[p])) {
                    a = 10 * a + (buf[p] - '0');
                    if (a > INT32_MAX) {
                        std::fprintf(stderr, "line %ld is corrupt\n", line);
                        return false;
                    }
                    ++p;
                }
                v[k] = a;
                while (k == 0 && p < e && std::isspace((unsigned char)buf[p])) ++p;
            }
            src.push_back((int32_t)v[0]);
            dst.push_back((int32_t)v[1]);
        }
        i = e + 1;
    }
    return true;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <input file> <output file>\n", argv[0]);
        return 255;
    }
    std::vector<int32_t> src, dst;
    std::printf("reading graph from file %s\n", argv[1]);
    if (!read_edges(argv[1], src, dst)) return 255;
    int32_t maxid = -1;
    for (size_t k = 0; k < src.size(); ++k) maxid = std::max(maxid, std::max(src[k], dst[k]));
    std::printf("found %d nodes and %zu edges\n", maxid + 1, src.size());
    pcd_ctx *ctx = nullptr;
    if (pcd_init(&ctx, 0) != PCD_OK) {
        std::fprintf(stderr, "CUDA initialisation failed: %s\n", pcd_last_error(ctx));
        return 255;
    }
    std::vector<int32_t> map((size_t)(maxid + 1) + 1);
    pcd_graph *g = nullptr;
    if (pcd_convert_edges(ctx, (int64_t)src.size(), src.data(), dst.data(), -1, map.data(), &g) != PCD_OK) {
        std::fprintf(stderr, "conversion failed: %s\n", pcd_last_error(ctx));
        pcd_destroy(ctx);
        return 255;
    }
    int32_t n = 0, m = 0;
    pcd_graph_size(g, &n, &m);
    std::vector<int32_t> ind((size_t)n + 1), adj((size_t)2 * m + 1);
    if (pcd_graph_csr_get(g, ind.data(), adj.data()) != PCD_OK) {
        std::fprintf(stderr, "reading the CSR failed: %s\n", pcd_last_error(ctx));
        pcd_destroy(ctx);
        return 255;
    }
    pcd_destroy(ctx);
    std::printf("writing %d nodes and %d edges to %s\n", n, m, argv[2]);
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) {
        std::fprintf(stderr, "failed to open %s\n", argv[2]);
        return 255;
    }
    bool ok = std::fwrite("PCD", 1, 3, f) == 3 && std::fwrite(&n, 4, 1, f) == 1 && std::fwrite(&m, 4, 1, f) == 1 &&
              std::fwrite(ind.data(), 4, (size_t)n + 1, f) == (size_t)n + 1 &&
              (m == 0 || std::fwrite(adj.data(), 4, (size_t)2 * m, f) == (size_t)2 * m) &&
              (n == 0 || std::fwrite(map.data(), 4, (size_t)n, f) == (size_t)n);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) {
        std::fprintf(stderr, "failed to write %s\n", argv[2]);
        return 255;
    }
    return 0;
}
