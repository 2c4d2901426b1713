// Device-wide exclusive prefix sum of uint32 values (mod 2^32), built as three
// launches: per-tile sums, one block scanning the tile sums, and the per-tile
// scan that adds the tile's offset.  Values are produced and consumed through
// functors so the scan fuses into its producer and consumer:
//   Load : __device__ uint32_t operator()(int64_t i) const
//   Store: __device__ void operator()(int64_t i, uint32_t exclusive, uint32_t value) const
// Scratch: one uint32 per tile (scan_tiles(n)) plus one for the total.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pcd_device.cuh"

namespace pcd {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

inline int64_t scan_tiles(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// Exclusive block scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ uint32_t block_excl_sum_u32(uint32_t x, uint32_t *total) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t block_tot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(FULL, inc, d);
        if (lane >= d) inc += o;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < nw ? warp_tot[lane] : 0u;
        uint32_t ti = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t o = __shfl_up_sync(FULL, ti, d);
            if (lane >= d) ti += o;
        }
        if (lane < nw) warp_tot[lane] = ti - t;
        if (lane == 31) block_tot = ti;  // lanes >= nw add 0: lane 31 holds the total
    }
    __syncthreads();
    uint32_t res = warp_tot[wid] + inc - x;
    *total = block_tot;
    __syncthreads();
    return res;
}

template <class Load>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(Load load, int64_t n, uint32_t *tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        int64_t i = base + (int64_t)j * SCAN_THREADS + threadIdx.x;
        if (i < n) s += load(i);
    }
    uint32_t tot;
    (void)block_excl_sum_u32(s, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// One block: exclusive scan of tile_sums in place; writes the grand total.
__global__ void __launch_bounds__(1024) k_scan_tile_sums(uint32_t *tile_sums, int64_t ntiles, uint32_t *total);

template <class Load, class Store>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(Load load, Store store, int64_t n,
                                                             const uint32_t *tile_sums) {
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    // thread t owns items [base + t*ITEMS, base + (t+1)*ITEMS): contiguous per thread
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + j;
        v[j] = i < n ? load(i) : 0u;
        s += v[j];
    }
    uint32_t tot;
    uint32_t run = block_excl_sum_u32(s, &tot) + tile_sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + j;
        if (i < n) store(i, run, v[j]);
        run += v[j];
    }
}

// Host helper: launches the three kernels on `st`.  Returns the number of
// launches.  If n needs more tiles than the scratch holds, nothing is
// launched and *sc.overflow is set (the caller reports it).
template <class Load, class Store>
int scan_exclusive(Load load, Store store, int64_t n, const ScanScratch &sc, cudaStream_t st) {
    if (n <= 0) {
        cudaMemsetAsync(sc.total, 0, sizeof(uint32_t), st);
        return 0;
    }
    const int64_t nt = scan_tiles(n);
    if (nt > sc.tile_cap) {
        if (sc.overflow) *sc.overflow = 1;
        return 0;
    }
    uint32_t *tile_sums = sc.tile_sums;
    uint32_t *total = sc.total;
    k_scan_reduce<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(load, n, tile_sums);
    k_scan_tile_sums<<<1, 1024, 0, st>>>(tile_sums, nt, total);
    k_scan_down<<<(unsigned)nt, SCAN_THREADS, 0, st>>>(load, store, n, tile_sums);
    return 3;
}

}  // namespace pcd
