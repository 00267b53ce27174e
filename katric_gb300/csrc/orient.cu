// Orientation: degrees, (degree, id) orientation with order-preserving compaction of every
// adjacency list to its out-neighbours, and the per-vertex out-list descriptors.
//
// Restates on the device what DistributedGraph::orient (distributed_graph.h:538-566) with
// node_ordering::degree_outward (distributed_graph.h:148-163) computes: u is kept in the
// out-list of v iff (deg(v), v) < (deg(u), u).  The reference partitions each list in place;
// here the input CSR is read-only and the out-lists are written to a separate gapped array.
// A list that one merge-path tile holds entirely keeps its input order.  A list that spans
// tiles is assembled from per-tile pieces and is recorded in the spanning list; the id sort
// (sort_neighborhoods, distributed_graph.h:578-593) runs only where a strategy needs sorted
// lists.
#include "ktri_device.cuh"
#include "ktri_kernels.h"

namespace ktri {

// deg[v] = first_out[v+1] - first_out[v]; zero the out-degrees and the per-vertex counts.
// Also tabulates the merge-path tile boundaries: vertex v covers the diagonals
// [first_out[v] + v, first_out[v+1] + v] (its slots and its end event), so every boundary
// k * TILE_BASE in that range crosses the path at vertex v.
__global__ void k_prep(const u64* __restrict__ fo, u64 n, u64 nnz, u32* __restrict__ deg, u32* __restrict__ dplus,
                       u64* __restrict__ cnt, u32* __restrict__ tile_i0, Control* ctl) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    const u64 nt = (n + nnz + TILE_BASE - 1) / TILE_BASE;
    u32 err = 0;
    for (u64 v = (u64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
        u64 a = fo[v], b = fo[v + 1];
        u32 d = 0;
        if (b < a || b - a > 0xFFFFFFFFull || b > nnz) {
            err |= DEV_ERR_DEGREE;
        } else {
            d = (u32)(b - a);
            const u64 k0 = (a + v + TILE_BASE - 1) / TILE_BASE, k1 = (b + v) / TILE_BASE;
            for (u64 k = k0; k <= k1 && k < nt; ++k) tile_i0[k] = (u32)v;
        }
        deg[v] = d;
        dplus[v] = 0;
        if (cnt) cnt[v] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        tile_i0[nt] = (u32)n;
        if (fo[0] != 0 || fo[n] != nnz) err |= DEV_ERR_DEGREE;
    }
    if (err) atomicOr(&ctl->err, err);
}

// Orientation of one merge-path tile of W = 32 * IPT diagonals per warp.  The tile holds the
// window vertices i0..i1 and the adjacency slots [j0, j1); every list with slots in the tile
// has one piece there.  Slots are taken 32 at a time, one per lane, so the owner of a slot,
// the rank of a kept entry among the tile's kept entries and the rank at a piece's ends all
// come from warp ballots and population counts: no block barrier, no per-thread path walk.
// Inside the tile all arithmetic is 32-bit (ids are below 2^32, slots relative to j0).
//   vertex pass  at the slot where each piece starts: (window index + 1, degree of its vertex)
//   pass 1       per slot: owner (the last piece start at or below the lane), deg[y] gather,
//                the (deg, id) decision, input checks; the tile rank at each piece's first
//                and past its last slot
//   piece pass   per window vertex, lanes in parallel: the piece's out-degree share (a plain
//                store, or an atomic reservation for a piece of a split list) and the
//                gapped-array index of its first kept entry
//   pass 2       kept entries written from registers, in slot order
// A list held by one tile keeps its input order.  A split list's pieces reserve their ranges
// with one atomic each and are recorded in the spanning list by the tile that holds the list's
// start.
template <int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK) k_orient(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                                                  u64 nnz, const u32* __restrict__ deg,
                                                  const u32* __restrict__ tile_i0, u32* __restrict__ headp,
                                                  u32* __restrict__ dplus, u32* __restrict__ spanning,
                                                  Control* ctl, u64 tile_begin) {
    constexpr int W = 32 * IPT;
    constexpr int WARPS = BLOCK / 32;
    constexpr u32 FULL = 0xFFFFFFFFu;
    __shared__ uint2 s_info_all[WARPS][W];  // at a piece's first slot: (window index + 1, degree)
    // at a piece's first slot: the tile ranks (at its first slot, past its last slot), then the
    // headp index of tile rank 0 for its entries
    __shared__ u64 s_base_all[WARPS][W];

    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const u64 total = n + nnz;
    const u64 tile = (tile_begin + blockIdx.x) * WARPS + wid;
    const u64 d0 = tile * W;
    if (d0 >= total) return;
    const u64 d1 = d0 + W < total ? d0 + W : total;
    uint2* s_info = s_info_all[wid];
    u64* s_base = s_base_all[wid];
    uint2* s_rank = reinterpret_cast<uint2*>(s_base);
    // tile_i0 holds base_tiles + 1 entries (the last is n), and tile + 1 <= base_tiles here
    const u64 i0 = tile_i0[tile], i1 = tile_i0[tile + 1];
    const u64 j0 = d0 - i0, j1 = d1 - i1;
    const u32 ns = (u32)(j1 - j0);
    if (ns == 0) return;  // only vertex ends: those lists have no slots here (out-degrees start at 0)
    const u32 n32 = (u32)n;  // n < 2^32: every id fits
    // every slot's neighbour and its degree, all in flight before the window is read
    u32 y_r[IPT], dy_r[IPT];
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const u32 s = (u32)it * 32 + lane;
        y_r[it] = s < ns ? __ldcs(head + j0 + s) : 0u;
    }
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const u32 s = (u32)it * 32 + lane;
        dy_r[it] = (s < ns && y_r[it] < n32) ? __ldg(deg + y_r[it]) : 0u;
    }
    for (u32 s = lane; s < ns; s += 32) s_info[s] = make_uint2(0u, 0u);
    __syncwarp();
    const u64 last_v = i1 < n ? i1 : n - 1;
    const u32 nwin = (u32)(last_v - i0) + 1;  // window vertices (at most W + 1)
    // the first 32 window vertices with every lane present (lane 0's list may begin before the
    // tile); their bounds stay in registers for the piece pass
    const bool have0 = (u32)lane < nwin;
    const u64 a0 = have0 ? fo[i0 + lane] : 0, b0 = have0 ? fo[i0 + lane + 1] : 0;
    const u64 fo_i0 = __shfl_sync(FULL, a0, 0), fo_i0_end = __shfl_sync(FULL, b0, 0);
    if (have0 && b0 > a0 && a0 < j1 && b0 > j0)
        s_info[a0 > j0 ? a0 - j0 : 0] = make_uint2((u32)lane + 1, (u32)(b0 - a0));
    for (u32 k = 32 + lane; k < nwin; k += 32) {
        const u64 v = i0 + k;
        const u64 a = fo[v], b = fo[v + 1];
        if (b > a && a < j1 && b > j0) s_info[a - j0] = make_uint2(k + 1, (u32)(b - a));
    }
    __syncwarp();
    const bool first_before = fo_i0 < j0;  // the first piece continues a list begun before the tile
    // the first vertex's list continues past the tile
    const bool first_past = fo_i0_end > j1;
    const u32 lt = (1u << lane) - 1u, le = lt | (1u << lane);
    const u32 i0_32 = (u32)i0;

    u32 s0_r[IPT], km_r[IPT];
    u32 rank = 0;                // kept entries of the tile before this iteration
    u32 s0c = 0, kc = 0, dc = 0;  // the piece open at the end of the previous iteration
    bool bad_id = false, self_loop = false, dup = false, unsorted = false;
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        s0_r[it] = 0;
        km_r[it] = 0;
        if ((u32)it * 32 >= ns) continue;
        const u32 s = (u32)it * 32 + lane;
        const bool valid = s < ns;
        const uint2 info = valid ? s_info[s] : make_uint2(0u, 0u);
        const u32 starts = __ballot_sync(FULL, info.x != 0);
        const u32 below = starts & le;
        const int src = 31 - __clz(below);  // -1 when no piece starts at or below this lane
        const u32 kx = __shfl_sync(FULL, info.x, src & 31);
        const u32 dxs = __shfl_sync(FULL, info.y, src & 31);
        const bool here = below != 0;
        const u32 s0 = here ? (u32)it * 32 + (u32)src : s0c;
        const u32 k1 = here ? kx : kc;
        const u32 dx = here ? dxs : dc;
        const u32 y = y_r[it];
        const u32 x = i0_32 + k1 - 1;
        const bool in_range = y < n32;
        bad_id |= valid && !in_range;
        self_loop |= valid && in_range && y == x;
        const u32 dy = dy_r[it];
        const bool kept = valid && in_range && y != x && (dx < dy || (dx == dy && x < y));
        const u32 km = __ballot_sync(FULL, kept);
        const bool last_slot = s + 1 == ns;
        bool next_start;
        if (lane < 31) next_start = (starts >> (lane + 1)) & 1u;
        else next_start = valid && !last_slot && s_info[s + 1].x != 0;
        // tile ranks at the piece's first slot and past its last slot
        if (valid && info.x != 0) s_rank[s].x = rank + __popc(km & lt);
        if (valid && (last_slot || next_start)) s_rank[s0].y = rank + __popc(km & le);
        // the next slot's neighbour (the next lane's, or lane 0's of the next iteration) when it
        // belongs to the same list: adjacent duplicates and order
        const u32 nd = __shfl_down_sync(FULL, y, 1);
        const u32 nn = __shfl_sync(FULL, y_r[it + 1 < IPT ? it + 1 : it], 0);
        const bool past = (k1 == 1 && first_before) ? first_past : dx > ns - s0;
        const bool same = valid && (last_slot ? past : !next_start);
        if (same) {
            const u32 nx = last_slot ? __ldcs(head + j1) : (lane < 31 ? nd : nn);
            unsorted |= nx < y;
            dup |= nx == y;
        }
        s0c = __shfl_sync(FULL, s0, 31);
        kc = __shfl_sync(FULL, k1, 31);
        dc = __shfl_sync(FULL, dx, 31);
        rank += __popc(km);
        s0_r[it] = s0;
        km_r[it] = km;
    }
    const u32 err = (bad_id ? DEV_ERR_ID_RANGE : 0u) | (self_loop ? DEV_ERR_SELF_LOOP : 0u) |
                    (dup ? DEV_ERR_DUPLICATE : 0u);
    if (err) atomicOr(&ctl->err, err);
    if (unsorted) atomicOr(&ctl->err, DEV_FLAG_UNSORTED);
    __syncwarp();
    // piece pass: out-degree shares and where each piece's kept entries go
    {
        auto settle = [&](u64 v, u64 a, u64 b) {
            if (!(b > a && a < j1 && b > j0)) return;
            const u32 s0 = a > j0 ? (u32)(a - j0) : 0u;
            const uint2 rk = s_rank[s0];
            const u32 cnt = rk.y - rk.x;
            u32 carry = 0;
            if (a < j0 || b > j1) {
                if (cnt) carry = atomicAdd(&dplus[v], cnt);
                if (a >= j0) spanning[atomicAdd(&ctl->spanning, 1ull)] = (u32)v;
            } else {
                dplus[v] = cnt;
            }
            s_base[s0] = oriented_start(a, v) + carry - rk.x;
        };
        if (have0) settle(i0 + lane, a0, b0);
        for (u32 k = 32 + lane; k < nwin; k += 32) {
            const u64 v = i0 + k;
            settle(v, fo[v], fo[v + 1]);
        }
    }
    __syncwarp();
    rank = 0;
#pragma unroll
    for (int it = 0; it < IPT; ++it) {
        const u32 km = km_r[it];
        if ((km >> lane) & 1u) __stcs(headp + s_base[s0_r[it]] + rank + __popc(km & lt), y_r[it]);
        rank += __popc(km);
    }
}

// Out-list descriptors, and the (owner, segment) tiles of owners above the small
// out-degree threshold.
template <typename OffT>
__global__ void k_desc(const u64* __restrict__ fo, u64 n, const u32* __restrict__ dplus, Desc<OffT>* __restrict__ vdesc,
                       uint2* __restrict__ mtiles, uint2* __restrict__ ltiles, u32 small_d, u32 medium_d, u32 seg,
                       u32 small_deg_max, Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31;
    const u64 warp_global = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 base = warp_global * 32; base < n; base += nwarps * 32) {
        const u64 v = base + lane;
        u32 nm = 0, nl = 0;
        if (v < n) {
            const u64 a = fo[v], b = fo[v + 1];
            const u32 d = dplus[v];
            Desc<OffT> ds;
            set_list_start(ds, oriented_start(a, v));
            ds.d = d;
            if constexpr (sizeof(OffT) == 8) ds.pad = 0;
            vdesc[v] = ds;
            // no tiles at all without tile arrays (the reference strategies pass none)
            const bool tiled = mtiles && ltiles && (d > small_d || (d > 0 && b - a > small_deg_max));
            const u32 nt = tiled ? (u32)((b - a + seg - 1) / seg) : 0u;
            if (d > medium_d) nl = nt;
            else nm = nt;
        }
        // warp-aggregated reservation of tile slots, one list per owner class
#pragma unroll
        for (int cls = 0; cls < 2; ++cls) {
            const u32 mine = cls == 0 ? nm : nl;
            u32 incl = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                u32 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += y;
            }
            const u32 wsum = __shfl_sync(0xFFFFFFFFu, incl, 31);
            u64 wbase = 0;
            if (lane == 31 && wsum) wbase = atomicAdd(cls == 0 ? &ctl->medium_tiles : &ctl->large_tiles, (u64)wsum);
            wbase = __shfl_sync(0xFFFFFFFFu, wbase, 31);
            const u64 my = wbase + incl - mine;
            uint2* out = cls == 0 ? mtiles : ltiles;
            for (u32 s = 0; s < mine; ++s) out[my + s] = make_uint2((u32)v, s);
        }
    }
}

// Large-owner tiles in the order of the first vertex each segment streams (a counting sort
// on the top id bits).  Input adjacency lists are mostly in id order, so tiles that run at the
// same time then stream out-lists from the same region of the list array, and the L2 cache
// serves the repeats.  Counts do not depend on the order.
constexpr u32 TILE_BUCKETS = 4096;

// Sort key of a tile (TILE_BY_VERTEX): the top id bits of the first vertex its segment
// streams; (TILE_BY_DEGREE): the owner's out-degree, largest first (longest tiles first);
// (TILE_BY_COST): the key k_tile_cost left in keys[t].
__device__ __forceinline__ u32 tile_key(const u64* fo, const u32* head, const u32* dplus, uint2 tl, u32 seg,
                                        u32 shift, u32 mode, const u32* keys, u64 t) {
    u32 key;
    if (mode == TILE_BY_COST) {
        key = keys[t];
    } else if (mode == TILE_BY_DEGREE) {
        const u32 d = dplus[tl.x];
        key = d >= TILE_BUCKETS ? 0u : TILE_BUCKETS - 1 - d;
    } else {
        key = __ldg(head + fo[tl.x] + (u64)tl.y * seg) >> shift;
    }
    return key < TILE_BUCKETS ? key : TILE_BUCKETS - 1;
}

// The work of each tile, for TILE_BY_COST: the entries its owner x streams over the tile's
// segment, sum of d+(y) over the neighbours y below x in (out-degree, id) -- the edge cost of
// the reference's DPD cost function (cost_function.h:287-376, cetric_edge_iterator.h:584-593)
// restated for owner-side tiles.  One warp per tile; the key orders heaviest first on a
// log scale (7 fractional bits).
__global__ void k_tile_cost(const u64* __restrict__ fo, const u32* __restrict__ head, const u32* __restrict__ dplus,
                            const uint2* __restrict__ tiles, const unsigned long long* count, u32 seg,
                            u32* __restrict__ keys, Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const u64 nt = *(volatile const unsigned long long*)count;
    const int lane = threadIdx.x & 31;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 t = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
        const uint2 tl = tiles[t];
        const u64 x = tl.x;
        const u32 dx = dplus[x];
        const u64 a = fo[x] + (u64)tl.y * seg, e1 = fo[x + 1], b = a + seg < e1 ? a + seg : e1;
        u64 cost = 0;
        for (u64 e = a + lane; e < b; e += 32) {
            const u32 y = __ldg(head + e);
            const u32 dy = __ldg(dplus + y);
            if (dy > 0 && key_less(dy, y, dx, x)) cost += dy;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cost += __shfl_down_sync(0xFFFFFFFFu, cost, o);
        if (lane == 0) {
            const u32 c = cost > 0xFFFFFFFFull ? 0xFFFFFFFFu : (u32)cost;
            const u32 lg = 31 - __clz(c | 1u);
            const u32 frac = lg >= 7 ? (c >> (lg - 7)) & 0x7Fu : (c << (7 - lg)) & 0x7Fu;
            const u32 bucket = lg * 128 + frac;  // < 32 * 128 = TILE_BUCKETS
            keys[t] = TILE_BUCKETS - 1 - bucket;
        }
    }
}

// Tiles [t0, t1) of block b when the tiles are cut into gridDim.x contiguous chunks.
__device__ __forceinline__ void tile_chunk(u64 nt, u64& t0, u64& t1) {
    const u64 per = (nt + gridDim.x - 1) / gridDim.x;
    t0 = (u64)blockIdx.x * per;
    t1 = t0 + per < nt ? t0 + per : nt;
    if (t0 > t1) t0 = t1;
}

// Histogram of the tiles' keys.  Each block counts its contiguous chunk in shared memory and
// adds the non-zero counts to the global histogram (one atomic per key present in the chunk,
// not per tile: the medium tiles' degree keys crowd onto a few hundred values).  The keys are
// left in keys[t] for the scatter (TILE_BY_COST finds them there already).
constexpr int TILE_ORDER_BLOCK = 256;
__global__ void __launch_bounds__(TILE_ORDER_BLOCK) k_tile_hist(const u64* __restrict__ fo,
                                                                const u32* __restrict__ head,
                                                                const u32* __restrict__ dplus,
                                                                const uint2* __restrict__ tiles,
                                                                const unsigned long long* count, u32 seg, u32 shift,
                                                                u32 mode, u32* __restrict__ keys, u32* hist,
                                                                Control* ctl) {
    __shared__ u32 s_cnt[TILE_BUCKETS];
    if (ctl->err & DEV_ERR_MASK) return;
    const u64 nt = *(volatile const unsigned long long*)count;
    u64 t0, t1;
    tile_chunk(nt, t0, t1);
    if (t0 == t1) return;
    for (u32 k = threadIdx.x; k < TILE_BUCKETS; k += TILE_ORDER_BLOCK) s_cnt[k] = 0;
    __syncthreads();
    for (u64 t = t0 + threadIdx.x; t < t1; t += TILE_ORDER_BLOCK) {
        const u32 key = tile_key(fo, head, dplus, tiles[t], seg, shift, mode, keys, t);
        if (mode != TILE_BY_COST) keys[t] = key;
        atomicAdd(&s_cnt[key], 1u);
    }
    __syncthreads();
    for (u32 k = threadIdx.x; k < TILE_BUCKETS; k += TILE_ORDER_BLOCK)
        if (s_cnt[k]) atomicAdd(&hist[k], s_cnt[k]);
}

// 256 threads: a block this small also fits beside the serving engine's resident blocks.
constexpr int TILE_SCAN_BLOCK = 256;
__global__ void __launch_bounds__(TILE_SCAN_BLOCK) k_tile_scan(u32* hist, Control* ctl) {
    constexpr int PER = TILE_BUCKETS / TILE_SCAN_BLOCK;
    __shared__ u32 s_warp[TILE_SCAN_BLOCK / 32];
    if (ctl->err & DEV_ERR_MASK) return;
    u32 v[PER], t = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        v[k] = hist[threadIdx.x * PER + k];
        t += v[k];
    }
    u32 total;
    u32 run = block_exclusive_scan<TILE_SCAN_BLOCK>(t, s_warp, &total);
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        hist[threadIdx.x * PER + k] = run;
        run += v[k];
    }
}

// Scatter of the tiles into key order (cursor = the scanned histogram).  Each block counts its
// chunk's keys again, reserves one range per key present with one atomic, and hands out the
// positions inside its ranges with shared-memory atomics.
__global__ void __launch_bounds__(TILE_ORDER_BLOCK) k_tile_scatter(const uint2* __restrict__ tiles,
                                                                   const unsigned long long* count,
                                                                   const u32* __restrict__ keys, u32* cursor,
                                                                   uint2* __restrict__ sorted, Control* ctl) {
    __shared__ u32 s_pos[TILE_BUCKETS];
    if (ctl->err & DEV_ERR_MASK) return;
    const u64 nt = *(volatile const unsigned long long*)count;
    u64 t0, t1;
    tile_chunk(nt, t0, t1);
    if (t0 == t1) return;
    for (u32 k = threadIdx.x; k < TILE_BUCKETS; k += TILE_ORDER_BLOCK) s_pos[k] = 0;
    __syncthreads();
    for (u64 t = t0 + threadIdx.x; t < t1; t += TILE_ORDER_BLOCK) atomicAdd(&s_pos[keys[t]], 1u);
    __syncthreads();
    for (u32 k = threadIdx.x; k < TILE_BUCKETS; k += TILE_ORDER_BLOCK) {
        const u32 c = s_pos[k];
        if (c) s_pos[k] = atomicAdd(&cursor[k], c);
    }
    __syncthreads();
    for (u64 t = t0 + threadIdx.x; t < t1; t += TILE_ORDER_BLOCK) sorted[atomicAdd(&s_pos[keys[t]], 1u)] = tiles[t];
}

// ---- launchers ------------------------------------------------------------------------

u64 tile_order_scratch_words() { return TILE_BUCKETS; }

void launch_order_tiles(const u64* fo, const u32* head, const u32* dplus, u64 n, const uint2* tiles,
                        const unsigned long long* count, u32 seg, u32 mode, u32* keys, u32* hist, uint2* sorted,
                        Control* ctl, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    u32 bits = 0;
    while ((1ull << bits) < n) ++bits;
    const u32 shift = bits > 12 ? bits - 12 : 0;
    cudaMemsetAsync(hist, 0, sizeof(u32) * TILE_BUCKETS, st);
    if (mode == TILE_BY_COST)
        k_tile_cost<<<num_sms * 8, 256, 0, st>>>(fo, head, dplus, tiles, count, seg, keys, ctl);
    k_tile_hist<<<num_sms * 4, TILE_ORDER_BLOCK, 0, st>>>(fo, head, dplus, tiles, count, seg, shift, mode, keys, hist,
                                                          ctl);
    k_tile_scan<<<1, TILE_SCAN_BLOCK, 0, st>>>(hist, ctl);
    k_tile_scatter<<<num_sms * 4, TILE_ORDER_BLOCK, 0, st>>>(tiles, count, keys, hist, sorted, ctl);
}

void launch_prep(const u64* fo, u64 n, u64 nnz, u32* deg, u32* dplus, u64* cnt, u32* tile_i0, Control* ctl,
                 int num_sms, cudaStream_t st) {
    if (n == 0) return;
    u64 blocks = (n + 255) / 256;
    u64 cap = (u64)num_sms * 8;
    k_prep<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(fo, n, nnz, deg, dplus, cnt, tile_i0, ctl);
}

u64 orient_tiles(u64 n, u64 nnz) { return (n + nnz + ORIENT_TILE - 1) / ORIENT_TILE; }

void launch_orient(const u64* fo, const u32* head, u64 n, u64 nnz, const u32* deg, const u32* tile_i0, u32* headp,
                   u32* dplus, u32* spanning, Control* ctl, cudaStream_t st, u64 tile_begin, u64 tile_end) {
    constexpr int BLOCK = ORIENT_BLOCK, IPT = ORIENT_IPT;
    const u64 tiles = orient_tiles(n, nnz);
    if (tile_end > tiles) tile_end = tiles;
    if (tile_begin >= tile_end) return;
    k_orient<BLOCK, IPT><<<(unsigned)(tile_end - tile_begin), BLOCK, 0, st>>>(fo, head, n, nnz, deg, tile_i0, headp,
                                                                             dplus, spanning, ctl, tile_begin);
}

template <typename OffT>
void launch_desc(const u64* fo, u64 n, const u32* dplus, void* vdesc, uint2* mtiles, uint2* ltiles, u32 small_d,
                 u32 medium_d, u32 seg, u32 small_deg_max, Control* ctl, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    u64 blocks = (n + 255) / 256;
    u64 cap = (u64)num_sms * 8;
    k_desc<OffT><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(
        fo, n, dplus, reinterpret_cast<Desc<OffT>*>(vdesc), mtiles, ltiles, small_d, medium_d, seg, small_deg_max,
        ctl);
}

template void launch_desc<u32>(const u64*, u64, const u32*, void*, uint2*, uint2*, u32, u32, u32, u32, Control*,
                               int, cudaStream_t);
template void launch_desc<u64>(const u64*, u64, const u32*, void*, uint2*, uint2*, u32, u32, u32, u32, Control*,
                               int, cudaStream_t);

}  // namespace ktri
