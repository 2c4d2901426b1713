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
    int32_t n_amb_large;          // of those, vertices of degree > 256 (queued from the list's end)
    int32_t check_where;          // bits of failed internal consistency checks (ERR_CHECK)
    int32_t hub_next;             // next hub of the sweep's hub queue (blocks take hubs in list order)
};

enum : int32_t {
    ERR_TIEBUF_OVERFLOW = 1,
    ERR_WAIT_TIMEOUT = 2,
    ERR_SCRATCH_OVERFLOW = 4,
    ERR_LABEL_RANGE = 8,
    ERR_CHECK = 16,
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
enum Bin : int32_t {
    BIN_G4 = 0,    // deg <= 4     : 4 lanes per vertex, 8 vertices per warp
    BIN_G8 = 1,    // deg <= 8
    BIN_G16 = 2,   // deg <= 16
    BIN_G32 = 3,   // deg <= 32    : one warp, row in registers
    BIN_WARP = 4,  // deg <= 256   : one warp, hash in shared memory
    BIN_BLOCK = 5, // deg <= 2048  : 256-thread block, table in shared memory
    BIN_BLOCK_L = 6,  // deg <= 8192 : 1024-thread block, 224 KiB shared table
    BIN_HUB = 7,   // larger       : 1024-thread block, table in HBM
    NBINS = 8
};

struct BinConfig {
    int32_t max_deg[NBINS - 1];  // upper degree of each bin but the last
};

}  // namespace pcd
