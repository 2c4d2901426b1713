// Normalised mutual information on the device (pcd_nmi_device / pcd_nmi):
// norm_mutual_info (src/common.cpp:75-125) over the confusion counts of
// (a[i], b[i]) pairs, which compare_communities builds from two labelings
// (src/common.cpp:163-173) or from a ground-truth file (src/common.cpp:127-160).
//   ni, nj: label histograms; distinct pairs: one radix sort of
//   (a << bits(b)) | b keys, a pair's count is the length of its run;
//   nom = sum val * log(val * n / (ni * nj)), with ni * nj in 32-bit int as the
//   reference multiplies it; den = sum ni * log(ni / n) + sum nj * log(nj / n);
//   result -2 nom / den.
// Each term is the reference's expression in FP64; the sums run in a fixed
// tree order (deterministic from run to run) instead of the reference's map
// order, so the result agrees with it to rounding, not bit for bit.
#include <algorithm>
#include <climits>
#include <vector>

#include "pcd_device.cuh"
#include "pcd_internal.h"

using namespace pcd;

namespace {

constexpr int NM_THREADS = 256;

int bit_len(uint64_t x) {
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

__global__ void k_nm_check(const int32_t *__restrict__ a, const int32_t *__restrict__ b, int64_t count,
                           int32_t *small) {
    int32_t ma = -1, mb = -1, bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = a[i], y = b[i];
        bad |= (x < 0) | (y < 0);
        ma = max(ma, x);
        mb = max(mb, y);
    }
    ma = __reduce_max_sync(FULL, ma);
    mb = __reduce_max_sync(FULL, mb);
    bad = __reduce_or_sync(FULL, bad);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(small, ma);
        atomicMax(small + 1, mb);
        if (bad) atomicOr(small + 2, 1);
    }
}

__global__ void k_nm_hist(const int32_t *__restrict__ a, const int32_t *__restrict__ b, int64_t count, int bb,
                          int32_t *ni, int32_t *nj, unsigned long long *keys, uint32_t *vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = a[i], y = b[i];
        atomicAdd(ni + x, 1);
        atomicAdd(nj + y, 1);
        keys[i] = ((unsigned long long)(uint32_t)x << bb) | (uint32_t)y;
        vals[i] = 0;
    }
}

// Block sum of one double per thread in a fixed tree order.
__device__ double block_sum(double x) {
    __shared__ double part[NM_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_down_sync(FULL, x, o);
    if (lane == 0) part[wid] = x;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = lane < NM_THREADS / 32 ? part[lane] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_down_sync(FULL, t, o);
    }
    __syncthreads();
    return t;  // valid in thread 0
}

// nom terms, one per distinct pair (at the head of its run); partial sums per block
__global__ void __launch_bounds__(NM_THREADS) k_nm_nom(const unsigned long long *__restrict__ keys, int64_t count,
                                                       int bb, const int32_t *__restrict__ ni,
                                                       const int32_t *__restrict__ nj, int32_t n, double *partial) {
    double acc = 0.0;
    const unsigned long long mask = (1ull << bb) - 1;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < count;
         s += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[s];
        if (s > 0 && keys[s - 1] == k) continue;
        int64_t lo = s + 1, hi = count;  // first index past the run
        while (lo < hi) {
            const int64_t mid = lo + (hi - lo) / 2;
            if (keys[mid] == k)
                lo = mid + 1;
            else
                hi = mid;
        }
        const int32_t val = (int32_t)(lo - s);
        const int32_t i = (int32_t)(k >> bb), j = (int32_t)(k & mask);
        const int32_t prod = (int32_t)((uint32_t)ni[i] * (uint32_t)nj[j]);
        acc += val * log(((double)val * n) / prod);
    }
    const double t = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// den terms of one histogram; partial sums per block
__global__ void __launch_bounds__(NM_THREADS) k_nm_den(const int32_t *__restrict__ h, int32_t len, int32_t n,
                                                       double *partial) {
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = h[i];
        if (c != 0) acc += c * log(c / ((double)n));
    }
    const double t = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// the three totals, each summed over its block partials in block order
__global__ void k_nm_final(const double *__restrict__ partial, int nb, double *out) {
    const int which = threadIdx.x;
    if (which >= 3) return;
    double t = 0.0;
    for (int i = 0; i < nb; ++i) t += partial[which * nb + i];
    out[which] = t;
}

}  // namespace

extern "C" {

pcd_status pcd_nmi_device(pcd_ctx *ctx, int64_t count, const int32_t *a, const int32_t *b, int32_t n,
                          double *nmi) {
    if (!ctx || !nmi || count < 0 || n < 0 || (count > 0 && (!a || !b))) return PCD_ERR_INVALID_ARGUMENT;
    if (count > (int64_t)UINT32_MAX) return set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "too many pairs");
    cudaStream_t st = ctx->stream;
    if (count == 0) {  // no pairs: nom = den = 0, as in the reference
        const double zero = 0.0;
        *nmi = -2 * zero / zero;
        return PCD_OK;
    }
    const int sms = ctx->num_sms;
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
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, (int64_t)sms * 8));
    int32_t *small = nullptr;
    if (!alloc((void **)&small, 64)) {
        cudaGetLastError();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "nmi buffers");
    }
    int32_t h_small[3] = {-1, -1, 0};
    cudaMemcpyAsync(small, h_small, sizeof h_small, cudaMemcpyHostToDevice, st);
    k_nm_check<<<grid, NM_THREADS, 0, st>>>(a, b, count, small);
    cudaMemcpyAsync(h_small, small, sizeof h_small, cudaMemcpyDeviceToHost, st);
    pcd_status s = check_cuda(ctx, cudaStreamSynchronize(st), "nmi input");
    if (s == PCD_OK && h_small[2]) s = set_error(ctx, PCD_ERR_INVALID_ARGUMENT, "negative label");
    if (s != PCD_OK) {
        release();
        return s;
    }
    const int32_t ca = h_small[0] + 1, cb = h_small[1] + 1;
    const int ba = std::max(1, bit_len((uint64_t)h_small[0])), bb = std::max(1, bit_len((uint64_t)h_small[1]));
    const int64_t tile_cap = (std::max<int64_t>({count, 256ll * 2 * sms, 1}) + 2047) / 2048 + 2;
    const int rgrid = sms * 2;
    const unsigned dgrid = (unsigned)sms * 2;
    int32_t *ni = nullptr, *nj = nullptr;
    unsigned long long *ka = nullptr, *kb = nullptr;
    uint32_t *va = nullptr, *vb = nullptr, *hist = nullptr, *tiles = nullptr;
    double *partial = nullptr, *tot = nullptr;
    if (!alloc((void **)&ni, 4 * (size_t)ca) || !alloc((void **)&nj, 4 * (size_t)cb) ||
        !alloc((void **)&ka, 8 * (size_t)count) || !alloc((void **)&kb, 8 * (size_t)count) ||
        !alloc((void **)&va, 4 * (size_t)count) || !alloc((void **)&vb, 4 * (size_t)count) ||
        !alloc((void **)&hist, 4ull * 256 * rgrid) || !alloc((void **)&tiles, 4 * (size_t)tile_cap + 64) ||
        !alloc((void **)&partial, 8ull * 3 * dgrid) || !alloc((void **)&tot, 8 * 3)) {
        cudaGetLastError();
        release();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "nmi buffers");
    }
    int32_t scan_overflow = 0;
    const ScanScratch sc{tiles, tile_cap, tiles + tile_cap, &scan_overflow};
    int launches = 0;
    cudaMemsetAsync(ni, 0, 4 * (size_t)ca, st);
    cudaMemsetAsync(nj, 0, 4 * (size_t)cb, st);
    k_nm_hist<<<grid, NM_THREADS, 0, st>>>(a, b, count, bb, ni, nj, ka, va);
    const bool inB = radix_sort(ka, va, kb, vb, count, ba + bb, hist, sc, rgrid, st, &launches);
    k_nm_nom<<<dgrid, NM_THREADS, 0, st>>>(inB ? kb : ka, count, bb, ni, nj, n, partial);
    k_nm_den<<<dgrid, NM_THREADS, 0, st>>>(ni, ca, n, partial + dgrid);
    k_nm_den<<<dgrid, NM_THREADS, 0, st>>>(nj, cb, n, partial + 2 * dgrid);
    k_nm_final<<<1, 32, 0, st>>>(partial, (int)dgrid, tot);
    double h_tot[3] = {0, 0, 0};
    cudaMemcpyAsync(h_tot, tot, sizeof h_tot, cudaMemcpyDeviceToHost, st);
    s = check_cuda(ctx, cudaStreamSynchronize(st), "nmi");
    release();
    if (s == PCD_OK && scan_overflow) s = set_error(ctx, PCD_ERR_CUDA, "internal: nmi scan scratch");
    if (s == PCD_OK) *nmi = -2 * h_tot[0] / (h_tot[1] + h_tot[2]);
    return s;
}

pcd_status pcd_nmi(pcd_ctx *ctx, int64_t count, const int32_t *a, const int32_t *b, int32_t n, double *nmi) {
    if (!ctx || !nmi || count < 0 || (count > 0 && (!a || !b))) return PCD_ERR_INVALID_ARGUMENT;
    cudaStream_t st = ctx->stream;
    int32_t *d = nullptr;
    if (count > 0 && cudaMallocAsync((void **)&d, 8 * (size_t)count, st) != cudaSuccess) {
        cudaGetLastError();
        return set_error(ctx, PCD_ERR_OUT_OF_MEMORY, "nmi input");
    }
    if (count > 0) {
        cudaMemcpyAsync(d, a, 4 * (size_t)count, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d + count, b, 4 * (size_t)count, cudaMemcpyHostToDevice, st);
    }
    pcd_status s = pcd_nmi_device(ctx, count, d, count > 0 ? d + count : nullptr, n, nmi);
    if (d) cudaFreeAsync(d, st);
    return s;
}

}  // extern "C"
