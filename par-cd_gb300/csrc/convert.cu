// Edge list -> the reference converter's CSR on the device (pcd_convert_edges),
// the pipeline of src/convert.cpp:76-196 without its O(E log E) host sorts:
//   loops dropped, both directions emitted as (u << 32 | v) keys, radix sorted,
//   duplicates removed; degrees; vertices ordered by (degree, id) descending
//   (a second radix sort of (DMAX - degree) << 32 | (n - 1 - id) keys);
//   edges renamed and sorted again; trailing isolated vertices dropped.
// One deliberate difference from the reference, as in the host restatement:
// loops are removed before the CSR is built (the reference's convert_to_csr
// writes a loop's slot twice, src/convert.cpp:97-102).
#include <algorithm>
#include <climits>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

using namespace pcd;

namespace {

__global__ void k_cv_check(const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t E,
                           int32_t *maxid, int32_t *bad) {
    int32_t mx = -1, b = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = src[i], v = dst[i];
        b |= (u < 0) | (v < 0);
        mx = max(mx, max(u, v));
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    b = __reduce_or_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxid, mx);
        if (b) atomicOr(bad, 1);
    }
}

// both directions of every non-loop edge; loops become the sentinel, which
// sorts after every real key
__global__ void k_cv_emit(const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t E,
                          unsigned long long sentinel, int32_t n, unsigned long long *keys, uint32_t *vals,
                          int32_t *bad) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = src[i], v = dst[i];
        if (u >= n || v >= n) atomicOr(bad, 2);
        const bool loop = u == v || u >= n || v >= n;
        keys[2 * i] = loop ? sentinel : ((unsigned long long)(uint32_t)u << 32) | (uint32_t)v;
        keys[2 * i + 1] = loop ? sentinel : ((unsigned long long)(uint32_t)v << 32) | (uint32_t)u;
        vals[2 * i] = 0;
        vals[2 * i + 1] = 0;
    }
}

struct UniqLoad {  // 1 for the first copy of each real key
    const unsigned long long *k;
    unsigned long long sentinel;
    __device__ uint32_t operator()(int64_t i) const {
        const unsigned long long x = k[i];
        return (x != sentinel && (i == 0 || k[i - 1] != x)) ? 1u : 0u;
    }
};
struct UniqStore {
    const unsigned long long *k;
    unsigned long long sentinel;
    unsigned long long *out;
    int32_t *deg;
    __device__ void operator()(int64_t i, uint32_t ex, uint32_t val) const {
        if (val) {
            const unsigned long long x = k[i];
            out[ex] = x;
            atomicAdd(deg + (int32_t)(x >> 32), 1);
        }
    }
};

__global__ void k_cv_vkeys(const int32_t *__restrict__ deg, int32_t n, unsigned long long *keys, uint32_t *vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = ((unsigned long long)(uint32_t)(INT32_MAX - deg[i]) << 32) | (uint32_t)(n - 1 - (int32_t)i);
        vals[i] = (uint32_t)i;
    }
}

__global__ void k_cv_rename(const uint32_t *__restrict__ order, int32_t n, const int32_t *__restrict__ deg,
                            int32_t *new_id, int32_t *deg2, int32_t *nz) {
    int32_t c = 0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = (int32_t)order[j];
        new_id[id] = (int32_t)j;
        deg2[j] = deg[id];
        c += deg[id] > 0 ? 1 : 0;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(nz, c);
}

__global__ void k_cv_remap(unsigned long long *keys, int64_t U, const int32_t *__restrict__ new_id) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < U; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long x = keys[i];
        keys[i] = ((unsigned long long)(uint32_t)new_id[(int32_t)(x >> 32)] << 32) |
                  (uint32_t)new_id[(int32_t)(x & 0xffffffffu)];
    }
}

__global__ void k_cv_adj(const unsigned long long *__restrict__ keys, int64_t U, int32_t *adj) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < U; i += (int64_t)gridDim.x * blockDim.x)
        adj[i] = (int32_t)(keys[i] & 0xffffffffu);
}

struct DegLoad {
    const int32_t *deg;
    __device__ uint32_t operator()(int64_t i) const { return (uint32_t)deg[i]; }
};
struct OffStore {
    int32_t *indices;
    __device__ void operator()(int64_t i, uint32_t ex, uint32_t) const { indices[i] = (int32_t)ex; }
};

int bit_length(uint64_t x) {
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

unsigned grid_of(int64_t n, int sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16));
}

}  // namespace

extern "C" {

pcd_status pcd_convert_edges(pcd_ctx *ctx, int64_t num_edges, const int32_t *src, const int32_t *dst,
                             int32_t num_nodes, int32_t *map, pcd_graph **out) {
    if (!ctx || !ctx->stream || !out || num_edges < 0 || (num_edges > 0 && (!src || !dst)))
        return PCD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (2 * num_edges > (int64_t)UINT32_MAX)
        return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "too many edges for 32-bit positions");
    cudaStream_t st = ctx->stream;
    const int sms = ctx->num_sms;
    const int64_t E = num_edges, E2 = std::max<int64_t>({2 * E, (int64_t)num_nodes, 1});
    // working memory (stream-ordered, freed on every exit)
    std::vector<void *> bufs;
    auto alloc = [&](void **p, size_t bytes) {
        if (cudaMallocAsync(p, std::max<size_t>(bytes, 16), st) != cudaSuccess) return false;
        bufs.push_back(*p);
        return true;
    };
    auto release = [&]() {
        for (void *p : bufs) cudaFreeAsync(p, st);
        bufs.clear();
    };
    int32_t *d_src = nullptr, *d_dst = nullptr, *d_small = nullptr;
    unsigned long long *ka = nullptr, *kb = nullptr;
    uint32_t *va = nullptr, *vb = nullptr, *hist = nullptr, *tiles = nullptr;
    const int grid = sms * 2;
    const int64_t tile_cap = (std::max<int64_t>({E2, 256ll * grid, 1}) + 2047) / 2048 + 2;
    if (!alloc((void **)&d_src, sizeof(int32_t) * std::max<int64_t>(E, 1)) ||
        !alloc((void **)&d_dst, sizeof(int32_t) * std::max<int64_t>(E, 1)) ||
        !alloc((void **)&d_small, 64) || !alloc((void **)&hist, 4ull * 256 * grid) ||
        !alloc((void **)&tiles, 4 * (size_t)tile_cap + 64)) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "converter buffers");
    }
    int32_t scan_overflow = 0;
    const ScanScratch sc{tiles, tile_cap, tiles + tile_cap, &scan_overflow};
    int launches = 0;
    if (E) {
        cudaMemcpyAsync(d_src, src, sizeof(int32_t) * E, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_dst, dst, sizeof(int32_t) * E, cudaMemcpyHostToDevice, st);
    }
    cudaMemsetAsync(d_small, 0, 64, st);
    int32_t h_small[4] = {-1, 0, 0, 0};
    cudaMemsetAsync(d_small, 0xff, sizeof(int32_t), st);  // max id starts at -1
    if (E) k_cv_check<<<grid_of(E, sms), 256, 0, st>>>(d_src, d_dst, E, d_small, d_small + 1);
    cudaMemcpyAsync(h_small, d_small, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    pcd_status s = check_cuda(ctx, cudaStreamSynchronize(st), "converter input");
    if (s == PCD_OK && h_small[1]) s = set_error(ctx, PCD_ERR_FORMAT, "negative vertex id");
    const int32_t n = num_nodes >= 0 ? num_nodes : h_small[0] + 1;  // src/convert.cpp:61
    if (s == PCD_OK && num_nodes >= 0 && h_small[0] >= num_nodes)
        s = set_error(ctx, PCD_ERR_FORMAT, "vertex id beyond num_nodes");
    if (s != PCD_OK) {
        release();
        return s;
    }
    // key and value buffers hold both directions of every edge, or one key per vertex
    const int64_t cap = std::max<int64_t>({2 * E, (int64_t)n, 1});
    if (!alloc((void **)&ka, 8 * (size_t)cap) || !alloc((void **)&kb, 8 * (size_t)cap) ||
        !alloc((void **)&va, 4 * (size_t)cap) || !alloc((void **)&vb, 4 * (size_t)cap)) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "converter buffers");
    }
    const int kbits = 32 + bit_length((uint64_t)std::max(n, 1));
    const unsigned long long sentinel = (unsigned long long)(uint32_t)n << 32;
    int32_t *deg = nullptr, *deg2 = nullptr, *new_id = nullptr, *ind = nullptr, *adj = nullptr;
    if (!alloc((void **)&deg, 4 * (size_t)std::max(n, 1)) || !alloc((void **)&deg2, 4 * (size_t)std::max(n, 1)) ||
        !alloc((void **)&new_id, 4 * (size_t)std::max(n, 1)) || !alloc((void **)&ind, 4 * ((size_t)n + 1))) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "converter buffers");
    }
    cudaMemsetAsync(deg, 0, 4 * (size_t)std::max(n, 1), st);
    // 1. keys of both directions, sorted; unique keys into the other buffer
    int64_t U = 0;
    unsigned long long *uk = kb;
    if (E) {
        k_cv_emit<<<grid_of(E, sms), 256, 0, st>>>(d_src, d_dst, E, sentinel, n, ka, va, d_small + 1);
        const bool inB = radix_sort(ka, va, kb, vb, 2 * E, kbits, hist, sc, grid, st, &launches);
        const unsigned long long *sorted = inB ? kb : ka;
        uk = inB ? ka : kb;
        launches += scan_exclusive(UniqLoad{sorted, sentinel}, UniqStore{sorted, sentinel, uk, deg}, 2 * E, sc, st);
        uint32_t total = 0;
        cudaMemcpyAsync(&total, tiles + tile_cap, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        s = check_cuda(ctx, cudaStreamSynchronize(st), "converter unique");
        U = total;
    }
    if (s == PCD_OK && scan_overflow) s = set_error(ctx, PCD_ERR_CUDA, "internal: converter scan scratch");
    if (s == PCD_OK && (U % 2 || U / 2 > INT32_MAX)) s = set_error(ctx, PCD_ERR_FORMAT, "edge count out of range");
    if (s != PCD_OK) {
        release();
        return s;
    }
    // 2. vertex order: (degree, id) descending  (src/convert.cpp:136-156)
    // vertex keys: the free key buffer and a second buffer of n keys
    unsigned long long *vk_a = uk == ka ? kb : ka;
    unsigned long long *vk_b2 = nullptr;
    uint32_t *vv_a = va, *vv_b = vb;
    if (!alloc((void **)&vk_b2, 8 * (size_t)std::max(n, 1))) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "converter buffers");
    }
    if (n > 0) k_cv_vkeys<<<grid_of(n, sms), 256, 0, st>>>(deg, n, vk_a, vv_a);
    const bool vInB = n > 1 && radix_sort(vk_a, vv_a, vk_b2, vv_b, n, 64, hist, sc, grid, st, &launches);
    const uint32_t *order = vInB ? vv_b : vv_a;
    cudaMemsetAsync(d_small + 2, 0, sizeof(int32_t), st);
    if (n > 0) k_cv_rename<<<grid_of(n, sms), 256, 0, st>>>(order, n, deg, new_id, deg2, d_small + 2);
    int32_t nz = 0;
    cudaMemcpyAsync(&nz, d_small + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (map && n > 0) {  // map[j] = original id of new vertex j, j < nz
        s = check_cuda(ctx, cudaStreamSynchronize(st), "converter order");
        if (s == PCD_OK && nz > 0)
            s = check_cuda(ctx, cudaMemcpyAsync(map, order, sizeof(int32_t) * (size_t)nz, cudaMemcpyDeviceToHost, st),
                           "converter map");
    }
    // 3. edges renamed and sorted by (new u, new v); the CSR
    if (s == PCD_OK && U > 0) {
        k_cv_remap<<<grid_of(U, sms), 256, 0, st>>>(uk, U, new_id);
        unsigned long long *other = uk == ka ? kb : ka;
        const bool inB = radix_sort(uk, va, other, vb, U, kbits, hist, sc, grid, st, &launches);
        uk = inB ? other : uk;
    }
    if (s == PCD_OK) s = check_cuda(ctx, cudaStreamSynchronize(st), "converter sort");
    if (s == PCD_OK) {
        launches += scan_exclusive(DegLoad{deg2}, OffStore{ind}, nz, sc, st);
        cudaMemcpyAsync(ind + nz, tiles + tile_cap, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
        if (!alloc((void **)&adj, 4 * (size_t)std::max<int64_t>(U, 1))) {
            cudaGetLastError();
            s = set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "converter buffers");
        }
    }
    if (s == PCD_OK && U > 0) k_cv_adj<<<grid_of(U, sms), 256, 0, st>>>(uk, U, adj);
    if (s == PCD_OK) s = check_cuda(ctx, cudaStreamSynchronize(st), "converter CSR");
    if (s == PCD_OK && scan_overflow) s = set_error(ctx, PCD_ERR_CUDA, "internal: converter scan scratch");
    if (s == PCD_OK) s = pcd_load_csr_device(ctx, nz, (int32_t)(U / 2), ind, adj, out);
    release();
    return s;
}

pcd_status pcd_graph_size(pcd_graph *g, int32_t *n, int32_t *m) {
    if (!g) return PCD_ERR_INVALID_ARGUMENT;
    if (n) *n = g->n;
    if (m) *m = g->m;
    return PCD_OK;
}

pcd_status pcd_graph_csr_get(pcd_graph *g, int32_t *indices, int32_t *adj) {
    if (!g || !indices || (g->nnz > 0 && !adj)) return PCD_ERR_INVALID_ARGUMENT;
    pcd_ctx *ctx = g->ctx;
    pcd_status s = check_cuda(
        ctx, cudaMemcpyAsync(indices, g->indices, sizeof(int32_t) * ((size_t)g->n + 1), cudaMemcpyDeviceToHost,
                             ctx->stream),
        "csr indices");
    if (s == PCD_OK && g->nnz > 0)
        s = check_cuda(ctx, cudaMemcpyAsync(adj, g->adj, sizeof(int32_t) * (size_t)g->nnz, cudaMemcpyDeviceToHost,
                                            ctx->stream),
                       "csr adj");
    if (s == PCD_OK) s = check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "csr get");
    return s;
}

}  // extern "C"
