// Plain structs shared by the host orchestration and the kernels.
#pragma once

#include <cstdint>

namespace pcd {

// Device-resident counters of one sweep, reset at its start.  One per graph.
struct DevCounters {
    unsigned long long tie_used;  // words of the tie buffer handed out
    int32_t n_resolve;            // tie records appended
    int32_t n_ambiguous;          // vertices queued for FP64 re-evaluation
    int32_t k;                    // communities after the last compress
    int32_t error;                // ERR_* bits
    uint32_t total_draws;         // rand_r calls of the sweep (mod 2^32)
    int32_t n_pairs;              // contracted pairs (merge)
    int32_t all_found;            // merge: every community matched
    int32_t pad;
};

enum : int32_t {
    ERR_TIEBUF_OVERFLOW = 1,
    ERR_WAIT_TIMEOUT = 2,
    ERR_SCRATCH_OVERFLOW = 4,
    ERR_LABEL_RANGE = 8,
};

// A vertex (or community) whose winner is picked by replaying its final
// level of ties: holder label at tiebuf[off], then r tie labels.
struct TieRecord {
    int32_t v;
    int32_t r;
    long long off;
};

// Scratch of a device-wide scan: tile sums (capacity in tiles), the device
// total, and a host flag raised when a scan would not fit.
struct ScanScratch {
    uint32_t *tile_sums;
    int64_t tile_cap;
    uint32_t *total;
    int32_t *overflow;
};

// Degree bins (vertex counts are per graph, fixed at load).
enum Bin : int32_t { BIN_THREAD = 0, BIN_WARP = 1, BIN_BLOCK = 2, BIN_BLOCK_L = 3, BIN_HUB = 4, NBINS = 5 };

struct BinConfig {
    int32_t thread_max;   // deg <= thread_max       -> one thread per vertex
    int32_t warp_max;     // deg <= warp_max         -> one warp per vertex
    int32_t block_max;    // deg <= block_max        -> one 256-thread block, table in smem
    int32_t block_l_max;  // deg <= block_l_max      -> one 1024-thread block, large smem table
                          // else                    -> hub: block with its table in HBM
};

}  // namespace pcd
