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

template <int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK) k_orient(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                                                  u64 nnz, const u32* __restrict__ deg,
                                                  const u32* __restrict__ tile_i0, u32* __restrict__ headp,
                                                  u32* __restrict__ dplus, u32* __restrict__ spanning,
                                                  Control* ctl, u64 tile_begin) {
    constexpr int TILE = BLOCK * IPT;
    // Everything inside a tile is addressed relative to its first vertex i0 and first slot j0,
    // in 32 bits.  s_fo[k] = first_out[i0 + k] - j0 clamped to [0, nslot]: only the first
    // vertex's start and the last one's end can lie outside the tile.
    __shared__ u32 s_fo[TILE + 2];
    __shared__ u32 s_deg[TILE + 2];
    __shared__ u32 s_head[TILE];
    __shared__ u32 s_cnt[TILE + 2];
    __shared__ u32 s_first[TILE + 2];
    __shared__ u32 s_warp[BLOCK / 32];
    __shared__ u64 s_b[3];   // i0, i1, first_out[i0]
    __shared__ u32 s_carry[2];
    __shared__ u32 s_flags;  // bit 0: the last window vertex's list continues past the tile

    if (ctl->err & DEV_ERR_MASK) return;
    const u64 total = n + nnz;
    const u64 tile = tile_begin + blockIdx.x;
    const u64 d0 = tile * TILE;
    if (d0 >= total) return;
    const u64 d1 = d0 + TILE < total ? d0 + TILE : total;
    if (threadIdx.x == 0) {
        const u64 nt = (total + TILE_BASE - 1) / TILE_BASE;
        const u64 k1 = ORIENT_PER_BASE * (tile + 1);
        s_b[0] = tile_i0[ORIENT_PER_BASE * tile];
        s_b[1] = tile_i0[k1 < nt ? k1 : nt];
    }
    __syncthreads();
    const u64 i0 = s_b[0], i1 = s_b[1];
    const u64 j0 = d0 - i0, j1 = d1 - i1;
    const u32 nslot = (u32)(j1 - j0);
    const u32 last = (u32)(i1 - i0);  // window vertices 0..last (last may be n - i0: no vertex)
    const u64 fo_last = i1 + 1 < n ? i1 + 1 : n;
    const u32 nfo = (u32)(fo_last - i0 + 1);
    for (u32 k = threadIdx.x; k < nfo; k += BLOCK) {
        const u64 f = fo[i0 + k];
        s_fo[k] = f < j0 ? 0u : (f > j1 ? nslot : (u32)(f - j0));
        s_cnt[k] = 0;
        if (k <= last && i0 + k < n) s_deg[k] = deg[i0 + k];
        if (k == 0) s_b[2] = f;
    }
    if (nfo <= last + 1) s_fo[last + 1] = nslot;  // the window ends at n
    for (u32 k = threadIdx.x; k < nslot; k += BLOCK) s_head[k] = head[j0 + k];
    if (threadIdx.x == 0) s_flags = (i1 < n && fo[i1 + 1] > j1) ? 1u : 0u;
    __syncthreads();

    // this thread's run of the merge path: items t .. te of the tile
    const u32 t = threadIdx.x * IPT < (u32)(d1 - d0) ? threadIdx.x * IPT : (u32)(d1 - d0);
    const u32 te = t + IPT < (u32)(d1 - d0) ? t + IPT : (u32)(d1 - d0);
    u32 i_start;  // largest i in [0, last] with s_fo[i] + i <= t
    {
        u32 lo = 0, hi = last;
        while (lo < hi) {
            const u32 mid = (lo + hi + 1) >> 1;
            if (s_fo[mid] + mid <= t) lo = mid;
            else hi = mid - 1;
        }
        i_start = lo;
    }
    const u32 j_start = t - i_start;
    const u32 nv = (u32)(n - i0);  // window vertices that exist: i < nv

    u32 own[IPT], yv[IPT];
    bool unsorted = false;
    u32 err = 0;
    {
        u32 i = i_start, j = j_start;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            own[k] = NONE;
            yv[k] = 0;
            if (t + k < te) {
                if (i < nv && j < s_fo[i + 1]) {
                    own[k] = i;
                    const u32 y = s_head[j];
                    yv[k] = y;
                    u32 nx = y;
                    bool has_next = false;
                    if (j + 1 < s_fo[i + 1]) {
                        nx = s_head[j + 1];
                        has_next = true;
                    } else if (i == last && (s_flags & 1u) && j + 1 == nslot) {
                        nx = __ldg(head + j0 + nslot);
                        has_next = true;
                    }
                    if (has_next) {
                        if (nx < y) unsorted = true;
                        if (nx == y) err |= DEV_ERR_DUPLICATE;
                    }
                    ++j;
                } else {
                    ++i;
                }
            }
        }
    }
    u32 dy[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) dy[k] = (own[k] != NONE && yv[k] < n) ? __ldg(deg + yv[k]) : 0u;

    u32 outbits = 0;
    {
        u32 run_owner = NONE, run = 0;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            if (own[k] == NONE) continue;
            const u64 x = i0 + own[k];
            const u32 y = yv[k];
            bool out = false;
            if (y >= n) err |= DEV_ERR_ID_RANGE;
            else if ((u64)y == x) err |= DEV_ERR_SELF_LOOP;
            else out = key_less(s_deg[own[k]], x, dy[k], y);
            if (own[k] != run_owner) {
                if (run) atomicAdd(&s_cnt[run_owner], run);
                run_owner = own[k];
                run = 0;
            }
            if (out) {
                outbits |= 1u << k;
                ++run;
            }
        }
        if (run) atomicAdd(&s_cnt[run_owner], run);
    }
    if (err) atomicOr(&ctl->err, err);
    if (unsorted) atomicOr(&ctl->err, DEV_FLAG_UNSORTED);

    u32 tot;
    const u32 base = block_exclusive_scan<BLOCK>((u32)__popc(outbits), s_warp, &tot);

    // first in-tile slot of every owner: record its scan position; lists wholly inside the
    // tile (every window vertex but possibly the first and the last) publish their out-degree
    const bool first_whole = s_b[2] >= j0 && (last > 0 || !(s_flags & 1u));
    {
        u32 run = base;
        u32 j = j_start;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            if (own[k] == NONE) continue;
            const u32 o = own[k];
            if (j == s_fo[o]) {
                s_first[o] = run;
                const bool whole = o == 0 ? first_whole : (o < last || !(s_flags & 1u));
                if (whole) dplus[i0 + o] = s_cnt[o];
            }
            if (outbits >> k & 1u) ++run;
            ++j;
        }
    }
    if (threadIdx.x == 0) {
        s_carry[0] = 0;
        s_carry[1] = 0;
        if (i0 < n) {
            const u64 a = fo[i0], b = fo[i0 + 1];
            const u64 lo = a > j0 ? a : j0, hi = b < j1 ? b : j1;
            if (lo < hi && (a < j0 || b > j1)) {
                s_carry[0] = atomicAdd(&dplus[i0], s_cnt[0]);
                if (a >= j0) spanning[atomicAdd(&ctl->spanning, 1ull)] = (u32)i0;
            }
        }
        if (i1 != i0 && i1 < n) {
            const u64 a = fo[i1], b = fo[i1 + 1];
            if (a < j1 && b > j1) {
                s_carry[1] = atomicAdd(&dplus[i1], s_cnt[last]);
                spanning[atomicAdd(&ctl->spanning, 1ull)] = (u32)i1;
            }
        }
    }
    __syncthreads();
    {
        u32 run = base;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            if (!(outbits >> k & 1u)) continue;
            const u32 o = own[k];
            const u32 carry = o == 0 ? s_carry[0] : (o == last ? s_carry[1] : 0u);
            const u32 pos = run - s_first[o] + carry;
            // every window vertex after the first starts inside the tile, at j0 + s_fo[o]
            const u64 fx = o == 0 ? s_b[2] : j0 + s_fo[o];
            headp[oriented_start(fx, i0 + o) + pos] = yv[k];
            ++run;
        }
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

__global__ void k_tile_hist(const u64* __restrict__ fo, const u32* __restrict__ head, const u32* __restrict__ dplus,
                            const uint2* __restrict__ tiles, const unsigned long long* count, u32 seg, u32 shift,
                            u32 mode, const u32* __restrict__ keys, u32* hist, Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const u64 nt = *(volatile const unsigned long long*)count;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += stride)
        atomicAdd(&hist[tile_key(fo, head, dplus, tiles[t], seg, shift, mode, keys, t)], 1u);
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

__global__ void k_tile_scatter(const u64* __restrict__ fo, const u32* __restrict__ head, const u32* __restrict__ dplus,
                               const uint2* __restrict__ tiles, const unsigned long long* count, u32 seg, u32 shift,
                               u32 mode, const u32* __restrict__ keys, u32* cursor, uint2* __restrict__ sorted,
                               Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const u64 nt = *(volatile const unsigned long long*)count;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += stride) {
        const uint2 tl = tiles[t];
        sorted[atomicAdd(&cursor[tile_key(fo, head, dplus, tl, seg, shift, mode, keys, t)], 1u)] = tl;
    }
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
    k_tile_hist<<<num_sms * 4, 256, 0, st>>>(fo, head, dplus, tiles, count, seg, shift, mode, keys, hist, ctl);
    k_tile_scan<<<1, TILE_SCAN_BLOCK, 0, st>>>(hist, ctl);
    k_tile_scatter<<<num_sms * 4, 256, 0, st>>>(fo, head, dplus, tiles, count, seg, shift, mode, keys, hist, sorted,
                                                ctl);
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
