// pcd_compress_labels_noalloc: first-occurrence relabelling of a label array
// that the caller already holds on the device, without any device allocation.
//
// Why it exists: every other entry point of this library sizes and allocates
// its working memory (cudaMalloc) when a graph is loaded.  Some callers
// cannot allocate at the point where they want to relabel: code running
// inside another framework's memory arena or allocator hooks, latency-critical
// loops that must not hit cudaMalloc's implicit device synchronisation, or
// hosts that pre-reserve all device memory at start-up.  This entry point
// takes device input and output buffers from the caller and keeps its own
// scratch in a fixed, file-scope device array instead.
//
// Limits and sharing rules:
//   * at most PCD_NOALLOC_MAX_LABELS labels per call (the array holds two
//     int32 per label plus the scan's tile sums: about 8 MiB, held by every
//     GPU that loads the library until the process exits);
//   * the first call on a device (with that device current) looks up the
//     array's device address with cudaGetSymbolAddress and the device's SM
//     count; make that first call before any stream capture that includes
//     this entry point.  The address is kept per CUDA context (keyed by the
//     context's unique id), so a call after cudaDeviceReset looks it up again
//     in the new context;
//   * a CUDA error already pending on the calling thread is left in place and
//     reported as PCD_ERR_CUDA before anything is launched; a launch error of
//     this call is cleared and reported as PCD_ERR_CUDA;
//   * every call uses the same array, and it keeps whatever the previous call
//     left there: each call re-initialises what it reads; two calls whose
//     work overlaps on the GPU (different streams, no ordering between them)
//     race on the array and give wrong results.
#include <algorithm>
#include <climits>
#include <mutex>

#include "pcd_internal.h"
#include "pcd_scan.cuh"

namespace pcd {
namespace {

constexpr int64_t kMax = PCD_NOALLOC_MAX_LABELS;
constexpr int64_t kTiles = (kMax + SCAN_TILE - 1) / SCAN_TILE + 2;
// layout: first[kMax] | rank[kMax] | tile_sums[kTiles] | total[4]
constexpr int64_t kWords = 2 * kMax + kTiles + 4;

static __device__ __align__(256) int32_t g_noalloc_scratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct DeviceSlot {
    int32_t *addr = nullptr;
    unsigned long long ctx_id = 0;  // the CUDA context the address belongs to
    int32_t sms = 0;
};
DeviceSlot g_slot[kMaxDevices];

// The current context's unique id through the driver API (resolved once);
// 0 when the driver does not offer it (the address is then looked up once).
using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
        resolved = true;
    }
    if (!get_current || !get_id) return 0;
    void *c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
    return id;
}

__global__ void k_na_fill(int32_t *first, int32_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        first[i] = INT_MAX;
}

__global__ void k_na_first(const int32_t *__restrict__ labels, int32_t n, int32_t *first) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t L = labels[v];
        if (L >= 0 && L < n) atomicMin(first + L, (int32_t)v);
    }
}

struct NaFlag {
    const int32_t *labels, *first;
    int32_t n;
    __device__ uint32_t operator()(int64_t v) const {
        const int32_t L = labels[v];
        if (L < 0 || L >= n) return 1u;
        return first[L] == (int32_t)v ? 1u : 0u;
    }
};

struct NaRank {
    int32_t *rank;
    __device__ void operator()(int64_t v, uint32_t x, uint32_t) const { rank[v] = (int32_t)x; }
};

__global__ void k_na_relabel(const int32_t *__restrict__ in, const int32_t *__restrict__ rank,
                             const int32_t *__restrict__ first, int32_t n, int32_t *out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t L = in[v];
        out[v] = (L < 0 || L >= n) ? rank[v] : rank[first[L]];
    }
}

__global__ void k_na_count(const uint32_t *total, int32_t *out) { *out = (int32_t)*total; }

}  // namespace
}  // namespace pcd

using namespace pcd;

extern "C" pcd_status pcd_compress_labels_noalloc(const int32_t *d_labels_in, int32_t n, int32_t *d_labels_out,
                                                  int32_t *d_num_labels, void *cuda_stream) {
    if (n < 0 || n > kMax) return PCD_ERR_INVALID_ARGUMENT;
    if (!d_num_labels || (n > 0 && (!d_labels_in || !d_labels_out))) return PCD_ERR_INVALID_ARGUMENT;
    if (d_labels_in == d_labels_out && n > 0) return PCD_ERR_INVALID_ARGUMENT;  // relabel reads other entries
    // an error the caller has not collected yet stays theirs: report it, launch nothing
    if (cudaPeekAtLastError() != cudaSuccess) return PCD_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PCD_ERR_CUDA;
    int32_t *base = nullptr;
    int32_t sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        DeviceSlot &ds = g_slot[dev];
        const unsigned long long cid = current_context_id();
        if (!ds.addr || (cid != 0 && cid != ds.ctx_id)) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return PCD_ERR_CUDA;
            }
            int count = 0;
            if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || count < 1) {
                cudaGetLastError();
                return PCD_ERR_CUDA;
            }
            ds.addr = static_cast<int32_t *>(p);
            ds.ctx_id = cid;
            ds.sms = count;
        }
        base = ds.addr;
        sms = ds.sms;
    }
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int32_t *first = base;
    int32_t *rank = base + kMax;
    uint32_t *tiles = reinterpret_cast<uint32_t *>(base + 2 * kMax);
    uint32_t *total = tiles + kTiles;
    if (n == 0) {
        cudaMemsetAsync(d_num_labels, 0, sizeof(int32_t), st);
        return cudaGetLastError() == cudaSuccess ? PCD_OK : PCD_ERR_CUDA;
    }
    // grid-stride kernels: up to 16 blocks of 256 threads per SM
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16);
    k_na_fill<<<grid, 256, 0, st>>>(first, n);
    k_na_first<<<grid, 256, 0, st>>>(d_labels_in, n, first);
    if (cudaGetLastError() != cudaSuccess) return PCD_ERR_CUDA;
    int32_t overflow = 0;
    scan_exclusive(NaFlag{d_labels_in, first, n}, NaRank{rank}, n, ScanScratch{tiles, kTiles, total, &overflow}, st);
    if (overflow) return PCD_ERR_INVALID_ARGUMENT;  // cannot happen for n <= kMax
    k_na_relabel<<<grid, 256, 0, st>>>(d_labels_in, rank, first, n, d_labels_out);
    k_na_count<<<1, 1, 0, st>>>(total, d_num_labels);
    return cudaGetLastError() == cudaSuccess ? PCD_OK : PCD_ERR_CUDA;
}
