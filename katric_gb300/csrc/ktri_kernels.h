// Launchers of the device kernels (host-callable, no torch types).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ktri_internal.h"

namespace ktri {

using u32 = uint32_t;
using u64 = unsigned long long;

constexpr int ORIENT_BLOCK = 256;   // 8 warps, one merge-path tile each
constexpr int ORIENT_IPT = 8;       // slots per lane of a tile: tiles of 256 diagonals
constexpr int SMALL_BLOCK = 256;
constexpr int SMALL_D = 48;          // largest out-degree bound of the small-owner kernel's owners
constexpr int SMALL_D_LOW = 32;      // bounds up to this run the small-owner kernel's instantiation for
                                     // 32, the others the one for SMALL_D (more table and bin space)
constexpr int MEDIUM_D = 256;        // out-degree bound of the warp-per-tile kernel's owners
constexpr int MEDIUM_BLOCK = 256;
constexpr int LARGE_BLOCK = 256;
constexpr int LARGE_CAP = 2048;      // keys per shared-memory table chunk of the vertex kernel
constexpr u32 LARGE_SEG = 1024;      // most adjacency slots per (owner, segment) tile
constexpr u32 MIN_SEG = 64;          // fewest adjacency slots per (owner, segment) tile
constexpr int LONG_LIST = 16;        // lists longer than this are streamed by a whole warp
constexpr u32 COPY_WAIT_POLLS = 1u << 22;  // polls of a bounded wait for a bulk copy into shared memory
constexpr u32 SMALL_WARP_DEG = 256;  // the small-owner kernel takes owners up to this degree; owners of
                                     // larger degree (and small out-degree) go to the medium kernel's tiles

// Merge-path tile boundaries are tabulated once per call at this granularity: entry k holds
// the vertex where diagonal k * TILE_BASE crosses the path.  One warp orients one base tile.
constexpr u64 TILE_BASE = 32ull * ORIENT_IPT;
inline u64 base_tiles(u64 n, u64 nnz) { return (n + nnz + TILE_BASE - 1) / TILE_BASE; }
// Each base tile records at most one split list (the one that starts in it and ends past it).
inline u64 spanning_capacity(u64 n, u64 nnz) { return base_tiles(n, nnz) + 2; }
// Owners above small_d hold more than small_d adjacency entries each, and owners routed to the
// tiles for their degree more than SMALL_WARP_DEG; every owner has at most deg / seg + 1 tiles.
inline u64 large_tile_capacity(u64 n, u64 nnz, u32 small_d, u32 seg) {
    u64 owners = nnz / ((u64)small_d + 1) + nnz / ((u64)SMALL_WARP_DEG + 1) + 1;
    if (owners > n) owners = n;
    return owners + nnz / seg + 1;
}

// Optional list of the triangles found by the edge-iterator kernel (debug listing): each
// triangle (v, u, w) is written, ids in increasing order, at the next position below cap.
struct TriangleSink {
    uint32_t* triples = nullptr;  // 3 * cap ids
    u64 cap = 0;
    unsigned long long* pos = nullptr;
#ifdef __CUDACC__
    __device__ __forceinline__ void emit(uint32_t a, uint32_t b, uint32_t c) const {
        if (!triples) return;
        const u64 p = atomicAdd(pos, 1ull);
        if (p >= cap) return;
        uint32_t x = a < b ? a : b, y = a < b ? b : a;
        uint32_t z = c;
        if (z < y) {
            const uint32_t t = y;
            y = z;
            z = t;
        }
        if (y < x) {
            const uint32_t t = x;
            x = y;
            y = t;
        }
        triples[3 * p] = x;
        triples[3 * p + 1] = y;
        triples[3 * p + 2] = z;
    }
#endif
};

void launch_prep(const u64* fo, u64 n, u64 nnz, u32* deg, u32* dplus, u64* cnt, u32* tile_i0, Control* ctl,
                 int num_sms, cudaStream_t st);
// Orientation over the blocks [tile_begin, tile_end) of ORIENT_TILE diagonals (all by
// default; a block holds ORIENT_BLOCK / 32 base tiles).  Block t reads adjacency slots below
// (t + 1) * ORIENT_TILE + 1 only, so it may run as soon as that prefix of head is on the device.
constexpr u64 ORIENT_TILE = (u64)ORIENT_BLOCK * ORIENT_IPT;
u64 orient_tiles(u64 n, u64 nnz);
void launch_orient(const u64* fo, const u32* head, u64 n, u64 nnz, const u32* deg, const u32* tile_i0, u32* headp,
                   u32* dplus, u32* spanning, Control* ctl, cudaStream_t st, u64 tile_begin = 0,
                   u64 tile_end = ~0ull);
// Owner tiles: medium owners' tiles are written to mtiles, large owners' to ltiles (each
// array holds large_tile_capacity entries).
// small_deg_max: owners up to small_d whose degree exceeds it get medium tiles too (the
// small-owner kernel's bound, SMALL_WARP_DEG).
template <typename OffT>
void launch_desc(const u64* fo, u64 n, const u32* dplus, void* vdesc, uint2* mtiles, uint2* ltiles, u32 small_d,
                 u32 medium_d, u32 seg, u32 small_deg_max, Control* ctl, int num_sms, cudaStream_t st);

// Owner tiles reordered (*count tiles on the device) by a counting sort on a 12-bit key:
// TILE_BY_VERTEX, the first vertex each segment streams (tiles that run together then stream
// from the same region of the list array); TILE_BY_DEGREE, the owner's out-degree, largest
// first; TILE_BY_COST, the tile's streamed entries (k_tile_cost writes them, log-scaled, into
// keys), heaviest first.  keys holds every tile's key between the two passes, so it needs the
// tiles' capacity in u32; hist needs tile_order_scratch_words() u32, sorted the same capacity
// as tiles.
enum : u32 { TILE_BY_VERTEX = 0, TILE_BY_DEGREE = 1, TILE_BY_COST = 2 };
u64 tile_order_scratch_words();
void launch_order_tiles(const u64* fo, const u32* head, const u32* dplus, u64 n, const uint2* tiles,
                        const unsigned long long* count, u32 seg, u32 mode, u32* keys, u32* hist, uint2* sorted,
                        Control* ctl, int num_sms, cudaStream_t st);

// Owner-side hash counting (KTRI_METHOD_AUTO).  partials needs small_grid + large_grid entries.
template <typename OffT>
int count_grid_small(int num_sms, u32 small_d);
template <typename OffT>
int count_grid_medium(int num_sms);
template <typename OffT>
int count_grid_large(int num_sms);
template <typename OffT>
int count_grid_auto(int num_sms, u32 small_d);  // small + medium + large, for this small-owner bound
template <typename OffT>
cudaError_t launch_count_auto(const u64* fo, const u32* head, u64 n, u64 nnz, const void* vdesc, const u32* headp,
                              const uint2* mtiles, const uint2* ltiles, u32 small_d, u32 seg, u64* cnt, u64* partials,
                              Control* ctl, int num_sms, cudaStream_t st, cudaEvent_t after_small,
                              cudaEvent_t after_large, u32 copy_wait_polls = COPY_WAIT_POLLS);
void launch_final(const u64* partials, u32 np, u64* total, Control* ctl, cudaStream_t st);
// The total of an AUTO count (the small-owner kernel's grid depends on n).
int small_grid_launched(u64 n, int cap);
template <typename OffT>
void launch_final_auto(const u64* partials, u64 n, u32 small_d, int num_sms, u64* total, Control* ctl,
                       cudaStream_t st);

// ---- the serving engine ------------------------------------------------------------------
// A prepared batch (orientation, descriptors and owner tiles done on its slot's stream) is
// published as a job; one persistent engine kernel per server drains the jobs' work units while
// the host keeps publishing: ENGINE_UNIT_ITEMS vertex batches of 32 (small owners, a run of
// ENGINE_REPS per warp), as many medium tiles (likewise) or one large tile (the whole block) per
// unit.  The block that finishes a
// job's last unit writes the job's sequence number into host-mapped memory.
struct EngineJob {
    const u64* fo;
    const u32* head;
    u64 n;
    const void* vdesc;  // Desc<u32>: jobs use 32-bit descriptors
    const u32* headp;
    const uint2* mtiles;
    const uint2* ltiles;
    u64* cnt;
    Control* ctl;
    u32 small_d, seg;
    unsigned long long units_small, units_medium, units;  // the rest are large tiles
    unsigned long long next;  // claim cursor
    unsigned long long done;  // finished units
    unsigned long long seq;   // nonzero while published (written last)
    unsigned long long pad[3];
};
constexpr int ENGINE_BLOCK = 256;
constexpr u32 ENGINE_REPS = 4;  // vertex batches or medium tiles per warp and unit
constexpr u32 ENGINE_UNIT_ITEMS = ENGINE_BLOCK / 32 * ENGINE_REPS;  // vertex batches or medium tiles per unit
// Publish a prepared batch as job slot `job` with sequence number seq (on the batch's stream,
// after its preparation).  A batch with nothing to count, or with invalid input, is marked done
// at once: done_word (host-mapped) receives seq.
void launch_publish(EngineJob* job, unsigned long long seq, const u64* fo, const u32* head, u64 n,
                    const void* vdesc, const u32* headp, const uint2* mtiles, const uint2* ltiles, u64* cnt,
                    Control* ctl, u32 small_d, u32 seg, unsigned long long* done_word, cudaStream_t st);
// The engine: blocks drain published jobs.  A block that has made idle_polls scans (about 2 us
// each) finding every published job finished sets *stop and leaves; every block leaves at its
// next scan once *stop is nonzero (set by a block or by the host), so a launch ends as a whole.
// *stop must be 0 when the engine is launched.  done_words[j] (host-mapped) receives job j's
// sequence number when its last unit is done.
int engine_grid(int num_sms);
size_t engine_smem_bytes();
void launch_engine(EngineJob* jobs, u32 njobs, unsigned long long* done_words, unsigned* stop, u32 idle_polls,
                   int grid, cudaStream_t st);

// u64 ids (the binary file format) -> u32 ids; ids above 2^32 - 1 become 0xFFFFFFFF.
void launch_narrow_ids(const u64* src, u64 count, u32* dst, int num_sms, cudaStream_t st);
// bytes from src to dst by a kernel (either side may be host memory the device can address).
// Both addresses 16-byte aligned (copy_by_kernel_ok), or at most 256 bytes; false (nothing
// launched) otherwise.
bool copy_by_kernel_ok(const void* src, const void* dst);
bool launch_copy(const void* src, void* dst, u64 bytes, int num_sms, cudaStream_t st);

// Oriented out-lists -> undirected CSR of their edges (fs: n + 1 offsets, hs: 2m ids).  cursor
// needs n u32 and sums dag_scan_chunks(n) u64 of scratch.
u64 dag_scan_chunks(u64 n);
void launch_scan_u64(u64* x, u64 len, u64* sums, cudaStream_t st);  // exclusive, in place
// Per-vertex cost (KTRI_COST_*) into cost[0..n), its exclusive prefix in place (cost[n] = total),
// and parts + 1 vertex boundaries of equal-cost ranges.  sums: dag_scan_chunks(n) u64.
void launch_cost_partition(const u64* fo, const u32* head, u64 n, const u32* deg, const u32* dplus, int fn, u32 parts,
                           u64* cost, u64* sums, u64* boundaries, int num_sms, cudaStream_t st);
// Contraction of a rank's lists after its local phase: local vertices 0..n_local-1 keep their
// ghost out-neighbours (ids n_local..n-1) in list order; vertices left without any are dropped
// and the rest renumbered.  cnt and keep need n_local + 1 entries, sums dag_scan_chunks(n_local),
// desc n_local Desc<u64> (for sorting the lists by id afterwards).
void launch_contract(const u64* fo, const u32* head, u64 n, u64 n_local, u64* cnt, u64* keep, u64* sums,
                     unsigned long long* maxlen, u32* kept, u64* out_fo, u32* out_head, void* desc, int num_sms,
                     cudaStream_t st);
void launch_dag_symmetrize(const u64* fo, const u32* head, u64 n, u64* fs, u32* hs, u32* cursor, u64* sums,
                           int num_sms, cudaStream_t st);
void launch_graph_totals(const u64* cnt, const u64* graph_first, u64 num_graphs, u64 n, u64* totals, Control* ctl,
                         int num_sms, cudaStream_t st);

// Work counters of the reference (wedge_checks, intersection_size_local) and of the AUTO
// kernels, accumulated into the control block.
template <typename OffT>
void launch_stats(const u64* fo, const u32* head, u64 n, const void* vdesc, const u32* headp, u32 medium_d,
                  Control* ctl, int num_sms, cudaStream_t st);

// Sorted-list strategies (merge, binary search, binary, hybrid): sort out-lists by id, then
// one warp per oriented edge.
template <typename OffT>
void launch_sort_lists(u64 n, const void* vdesc, u32* headp, u32* mid_list, u32* big_list, u32* scratch,
                       u64 scratch_per_block, int big_grid, Control* ctl, int num_sms, cudaStream_t st);
template <typename OffT>
void launch_count_edges(u64 n, const void* vdesc, const u32* headp, int method, u64 cutoff, double hybrid_scale,
                        u64* cnt, u64* partials, int grid, Control* ctl, TriangleSink sink, cudaStream_t st);
int count_grid_edges(int num_sms);

// Oriented CSR export: compact copy of the out-lists (after sorting).
template <typename OffT>
void launch_export(u64 n, const void* vdesc, const u32* headp, const u64* out_fo, u32* out_head, int num_sms,
                   cudaStream_t st);
template <typename OffT>
void launch_outdeg(u64 n, const void* vdesc, u64* out, int num_sms, cudaStream_t st);

// Batched pair intersection for known-answer tests of the strategies.
void launch_intersect_pairs(int method, const u32* a_vals, const u64* a_off, const u32* b_vals, const u64* b_off,
                            u64 npairs, u64 cutoff, double hybrid_scale, u64* counts, u32* members, int* err,
                            cudaStream_t st);

}  // namespace ktri
