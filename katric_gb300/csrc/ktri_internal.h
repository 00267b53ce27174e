// Internal declarations shared by the host code and the CUDA launchers.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "ktri.h"

struct ktri_graph {
    uint64_t n = 0;
    std::vector<uint64_t> first_out;
    std::vector<uint32_t> head;
};

namespace ktri {

// Resolved options (defaults filled in).
struct Options {
    int32_t method = KTRI_METHOD_AUTO;
    uint32_t small_outdegree = 32;   // owner bins and tile segment of the AUTO kernels
    uint32_t medium_outdegree = 256;
    uint32_t segment = 1024;
    bool collect_stats = false;
    uint64_t binary_cutoff = 1000;
    double hybrid_scale = 1.0;
    bool force_wide = false;
    uint32_t copy_wait_polls = 0;    // polls of the first wait for an owner chunk's bulk copy (0 = default)
    uint32_t tile_order = 0;         // 0: by streamed vertex / owner degree; KTRI_TILE_ORDER_COST: by tile work
};

// The device a context was created on, and its SM count.
int ctx_device(const ktri_ctx* ctx);
int ctx_num_sms(const ktri_ctx* ctx);

struct Control;
struct EngineJob;
// Serving engine: enqueue the preparation of a packed batch (orientation, descriptors, owner
// tiles) on ctx's workspace and `stream`, then publish its counting phase as job `job` with
// sequence number seq; done_word (device address of host-mapped memory) receives seq when the
// engine has counted it.  Per-vertex counts go to d_per_vertex; *ctl_out is the batch's control
// block (for the graph totals after completion).  Batches that need 64-bit descriptors return
// KTRI_ERR_UNSUPPORTED (count them with ktri_count_batch_device).
int engine_prepare_batch(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                         uint64_t nnz_total, uint64_t* d_per_vertex, void* stream, EngineJob* job,
                         unsigned long long seq, unsigned long long* done_word, Control** ctl_out);

// Device-side error bits written by the kernels (one u32 word in the control block).
enum : uint32_t {
    DEV_ERR_ID_RANGE = 1u << 0,   // head entry >= n
    DEV_ERR_SELF_LOOP = 1u << 1,  // head entry == owner
    DEV_ERR_DUPLICATE = 1u << 2,  // a list holds the same id twice
    DEV_ERR_DEGREE = 1u << 3,     // first_out not monotone, or a degree >= 2^32
    DEV_ERR_TIMEOUT = 1u << 4,    // a bounded wait (bulk-copy barrier) ran out
    DEV_ERR_COPY_INFLIGHT = 1u << 5,  // ... and its second wait too: a copy may have been in flight
                                      // into shared memory when the block left
    DEV_FLAG_UNSORTED = 1u << 8,  // some input list is not strictly increasing (not an error)
};

// Control block in device memory: counters and flags the kernels share.
struct Control {
    uint32_t err;              // DEV_ERR_* | DEV_FLAG_*
    uint32_t pad0;
    unsigned long long large_tiles;      // number of (owner, segment) tiles for large owners
    unsigned long long small_next;       // dynamic tile cursor of the small-owner kernel
    unsigned long long large_next;       // dynamic tile cursor of the large-owner kernel
    unsigned long long spanning;         // number of vertices whose out-list was assembled by several tiles
    unsigned long long edge_next;        // dynamic cursor of the per-edge kernels
    unsigned long long stat_wedge;       // collect_stats: sum of |N+(u)| over oriented (v,u)
    unsigned long long stat_isz;         // collect_stats: sum of |N+(v)|+|N+(u)|
    unsigned long long stat_streamed;    // collect_stats: entries streamed by the AUTO kernels
    unsigned long long stat_oriented;    // collect_stats: sum of out-degrees
    unsigned long long sort_mid;         // lists sorted by whole blocks in shared memory
    unsigned long long sort_big;         // lists sorted by whole blocks in global scratch
    unsigned long long medium_tiles;     // number of (owner, segment) tiles for medium owners
    unsigned long long medium_next;      // dynamic tile cursor of the medium-owner kernel
    unsigned long long stat_chunked;     // collect_stats: streamed entries times the owner's table chunks
    unsigned long long pad[1];
};

}  // namespace ktri
