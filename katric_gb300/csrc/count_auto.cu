// Owner-side hash counting (KTRI_METHOD_AUTO): the GPU form of CetricEdgeIterator::run_local
// (cetric_edge_iterator.h:889-1066) with intersection() (intersection.h:41-79).
//
// Every undirected edge {x,y} contributes |N+(x) ∩ N+(y)| triangles, where N+ is the
// out-list after orientation by (degree, id); the sum over all edges is the triangle total,
// exactly as the reference's sum over oriented edges (v,u) of |N+(v) ∩ N+(u)|.  The edge is
// evaluated once, at its "owner": the endpoint whose (out-degree, id) is larger.  The owner's
// out-list sits in a shared-memory hash table and the other endpoint's (shorter) out-list
// is streamed through it, so the work of an edge is min(|N+(x)|, |N+(y)|) probes.
//
// Per-vertex counts: a hit w of edge {x,y} is the triangle {x,y,w}.  w is a key of the
// owner's table: its hits accumulate in a shared-memory counter next to the key and are
// flushed once per table.  y gets one atomic per edge, x one per tile.
//
// Three kernels split the owners by out-degree (the bounds are runtime options, at most
// SMALL_D and MEDIUM_D):
//   k_count_small: owners with out-degree <= small_outdegree (instantiated for bounds up to
//     SMALL_D_LOW and up to SMALL_D, both five blocks per SM).  Merge-path tiles over the
//     adjacency (as in orientation) give every block the same number of slots; the tables of
//     all owners in a tile live side by side in shared memory.  Selected edges are queued,
//     counting-sorted by streamed-list length so that the lanes of a warp carry equal work,
//     then streamed one list per thread with uint4 loads.
//   k_count_medium: owners up to medium_outdegree, one warp per (owner, segment) tile with
//     the warp's own table, filter and survivor buffer, so tiles need no block barrier.
//   k_count_large: larger owners, one (owner, segment) tile per block iteration.  Short
//     streamed lists are handled one per thread while the segment is scanned; longer ones are
//     queued and taken one at a time by whole warps (one entry per lane, eight loads in
//     flight), so no block-wide barrier separates the lists.
// The medium and large kernels test every streamed entry against a one-hash filter of the
// owner's keys first and look up only the survivors, packed 32 at a time.
#include "ktri_device.cuh"
#include "ktri_kernels.h"

namespace ktri {

constexpr size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Bulk (TMA) copies into shared memory, completed on an mbarrier.  The copy engine moves a
// 16-byte-aligned run of bytes (a multiple of 16) from global to shared memory and counts the
// bytes against the barrier's expected transaction count.
__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, u32 bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, u32 parity) {
    u32 ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the barrier's phase of the given parity; gives up after `polls` polls (each poll
// itself blocks for a short hardware-defined time) and reports false.  polls = 0 gives up at
// once without looking.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, u32 parity, u32 polls) {
    for (u32 it = 0; it < polls; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Hit counters of the owners' tables are 16-bit, two per word: a key gets at most one hit per
// streamed list, and a tile streams at most LARGE_SEG (block and warp kernels) or one tile's
// slots (small-owner kernel) lists, so they cannot overflow.
__device__ __forceinline__ void hit16(u32* hits32, u32 slot) { atomicAdd(&hits32[slot >> 1], 1u << ((slot & 1u) << 4)); }
__device__ __forceinline__ u32 read16(const u32* hits32, u32 slot) { return (hits32[slot >> 1] >> ((slot & 1u) << 4)) & 0xFFFFu; }

// Lookup with a 16-bit hit counter (same table layout as bucket_probe).
__device__ __forceinline__ u32 bucket_probe16(const u32* keys, u32* hits32, u32 lg, u32 w) {
    const u32 nb_mask = (1u << (lg - 2)) - 1;
    u32 b = bucket_home(w, lg);
    for (u32 it = 0; it <= nb_mask; ++it) {
        const uint4 q = *reinterpret_cast<const uint4*>(keys + 4 * b);
        const bool m0 = q.x == w, m1 = q.y == w, m2 = q.z == w, m3 = q.w == w;
        if (m0 | m1 | m2 | m3) {
            hit16(hits32, 4 * b + (m0 ? 0u : (m1 ? 1u : (m2 ? 2u : 3u))));
            return 1u;
        }
        if (q.w == EMPTY_KEY) return 0u;
        b = (b + 1) & nb_mask;
    }
    return 0u;
}


// The same lookup without early exits: one bucket read, a walk along full buckets only when
// the home bucket is full and holds no w (rare at the tables' load factors), and a predicated
// hit count, so the lanes of a warp that look up 32 packed filter survivors stay together.
__device__ __forceinline__ u32 bucket_probe16_flat(const u32* keys, u32* hits32, u32 lg, u32 w) {
    const u32 nb_mask = (1u << (lg - 2)) - 1;
    u32 b = bucket_home(w, lg);
    uint4 q = *reinterpret_cast<const uint4*>(keys + 4 * b);
    for (u32 it = 0; it < nb_mask && q.w != EMPTY_KEY && q.x != w && q.y != w && q.z != w && q.w != w; ++it) {
        b = (b + 1) & nb_mask;
        q = *reinterpret_cast<const uint4*>(keys + 4 * b);
    }
    const u32 slot = q.x == w ? 0u : (q.y == w ? 1u : (q.z == w ? 2u : (q.w == w ? 3u : 4u)));
    if (slot < 4u) hit16(hits32, 4 * b + slot);
    return slot < 4u ? 1u : 0u;
}

template <int BLOCK, int IPT, int SD, typename OffT>
struct SmallLayout {
    static constexpr int TILE = BLOCK * IPT;
    static constexpr int TBL = 4 * (TILE + 2 * SD);  // sum of per-owner table sizes (pow2 >= max(4, 2d) <= 4d)
    static constexpr int WPT = (TILE + 1 + BLOCK - 1) / BLOCK;
    static_assert(TILE < 65536, "window offsets and hit counters are 16-bit");
    static constexpr size_t off_fo = 0;  // first_out of the window, clamped to the tile, relative to its first slot
    static constexpr size_t off_desc = align16(off_fo + sizeof(unsigned short) * (TILE + 2));
    static constexpr size_t off_tb = align16(off_desc + sizeof(Desc<OffT>) * (TILE + 2));
    // key offsets of the owners while the tables are filled, then the owners' hit totals
    static constexpr size_t off_ko = align16(off_tb + sizeof(u32) * (TILE + 2));
    static constexpr size_t off_keys = align16(off_ko + sizeof(u32) * (TILE + 2));
    static constexpr size_t off_hits = align16(off_keys + sizeof(u32) * TBL);  // two u16 counters per word
    static constexpr size_t off_qy = align16(off_hits + sizeof(u32) * (TBL / 2));
    static constexpr size_t off_qs = align16(off_qy + sizeof(u32) * TILE);
    static constexpr size_t off_qm = align16(off_qs + sizeof(OffT) * TILE);
    static constexpr size_t off_ord = align16(off_qm + sizeof(unsigned short) * TILE);
    static constexpr size_t bytes = align16(off_ord + sizeof(unsigned short) * TILE);
};

template <int BLOCK, int IPT, int SD, typename OffT>
__global__ void __launch_bounds__(BLOCK, 5) k_count_small(const u64* __restrict__ fo, const u32* __restrict__ head,
                                                       u64 n, u64 nnz, const Desc<OffT>* __restrict__ vdesc,
                                                       const u32* __restrict__ headp,
                                                       const u32* __restrict__ tile_i0, u32 sd,
                                                       u64* __restrict__ cnt, u64* __restrict__ partials,
                                                       Control* ctl) {
    using L = SmallLayout<BLOCK, IPT, SD, OffT>;
    static_assert(L::TILE == TILE_BASE, "one counting tile = one base tile");
    constexpr int TILE = L::TILE;
    constexpr int WPT = L::WPT;
    static_assert(SD < 64, "list length is packed in 6 bits");
    static_assert(TILE + 2 <= 1024, "window owner index is packed in 10 bits");
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned short* s_fo = reinterpret_cast<unsigned short*>(smem + L::off_fo);
    Desc<OffT>* s_desc = reinterpret_cast<Desc<OffT>*>(smem + L::off_desc);
    u32* s_tb = reinterpret_cast<u32*>(smem + L::off_tb);
    u32* s_ko = reinterpret_cast<u32*>(smem + L::off_ko);
    u32* s_own = reinterpret_cast<u32*>(smem + L::off_ko);  // after the tables are filled
    u32* s_keys = reinterpret_cast<u32*>(smem + L::off_keys);
    u32* s_hits = reinterpret_cast<u32*>(smem + L::off_hits);
    u32* q_y = reinterpret_cast<u32*>(smem + L::off_qy);
    OffT* q_s = reinterpret_cast<OffT*>(smem + L::off_qs);
    unsigned short* q_m = reinterpret_cast<unsigned short*>(smem + L::off_qm);  // (owner << 6) | list length
    unsigned short* q_ord = reinterpret_cast<unsigned short*>(smem + L::off_ord);
    __shared__ u32 s_warp[BLOCK / 32];
    __shared__ u64 s_red[BLOCK / 32];
    __shared__ u64 s_b[3];
    __shared__ u32 s_bins[SD + 2];
    __shared__ u32 s_qn, s_chunk;

    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31;
    const u64 total_items = n + nnz;
    const u64 ntiles = (total_items + TILE - 1) / TILE;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    u64 local_total = 0;
    u32 dup = 0;

    while (true) {
        if (threadIdx.x == 0) {
            const u64 t = atomicAdd(&ctl->small_next, 1ull);
            s_b[2] = t;
            if (t < ntiles) {
                s_b[0] = tile_i0[t];
                s_b[1] = tile_i0[t + 1];
            }
            s_qn = 0;
            s_chunk = 0;
        }
        if (threadIdx.x < SD + 2) s_bins[threadIdx.x] = 0;
        __syncthreads();
        const u64 tile = s_b[2];
        if (tile >= ntiles) break;
        const u64 d0 = tile * TILE;
        const u64 d1 = d0 + TILE < total_items ? d0 + TILE : total_items;
        const u64 i0 = s_b[0], i1 = s_b[1];
        if (i0 >= n) {  // only trailing vertex-end events: nothing to count
            __syncthreads();
            continue;
        }
        const u64 j0 = d0 - i0, j1 = d1 - i1;
        const u64 fo_last = i1 + 1 < n ? i1 + 1 : n;
        const u32 nw = (u32)(fo_last - i0);  // window vertices [i0, fo_last)
        for (u32 k = threadIdx.x; k <= nw; k += BLOCK) {
            u64 f = fo[i0 + k];
            f = f < j0 ? j0 : (f > j1 ? j1 : f);
            s_fo[k] = (unsigned short)(f - j0);
        }
        for (u32 k = threadIdx.x; k < nw; k += BLOCK) {
            s_desc[k] = load_desc(vdesc + i0 + k);
        }
        __syncthreads();

        // table sizes and key offsets of the owners in the window
        u32 packed[WPT];
        u32 tsum = 0;
#pragma unroll
        for (int r = 0; r < WPT; ++r) {
            const u32 k = threadIdx.x * WPT + r;
            packed[r] = 0;
            if (k < nw) {
                const u32 d = s_desc[k].d;
                if (s_fo[k] < s_fo[k + 1] && d > 0 && d <= sd) {
                    u32 lg = ceil_log2(2 * d);
                    if (lg < 2) lg = 2;
                    packed[r] = ((1u << lg) << 16) | d;
                }
            }
            tsum += packed[r];
        }
        u32 ptot;
        u32 pbase = block_exclusive_scan<BLOCK>(tsum, s_warp, &ptot);
#pragma unroll
        for (int r = 0; r < WPT; ++r) {
            const u32 k = threadIdx.x * WPT + r;
            if (k < nw) {
                const u32 p = packed[r];
                if (p) {
                    const u32 sz = p >> 16;
                    s_tb[k] = ((pbase >> 16) << 5) | (31 - __clz(sz));
                } else {
                    s_tb[k] = NONE;
                }
                s_ko[k] = pbase & 0xFFFFu;
            }
            pbase += packed[r];
        }
        const u32 table_slots = ptot >> 16, nkeys = ptot & 0xFFFFu;
        if (threadIdx.x == 0) s_ko[nw] = nkeys;
        for (u32 s = threadIdx.x; s < table_slots; s += BLOCK) s_keys[s] = EMPTY_KEY;
        for (u32 s = threadIdx.x; s < table_slots / 2; s += BLOCK) s_hits[s] = 0;
        __syncthreads();

        // insert the out-lists of the owners (one key per thread per step)
        for (u32 q = threadIdx.x; q < nkeys; q += BLOCK) {
            u32 lo = 0, hi = nw - 1;
            while (lo < hi) {
                u32 mid = (lo + hi + 1) >> 1;
                if (s_ko[mid] <= q) lo = mid; else hi = mid - 1;
            }
            const u32 tb = s_tb[lo];
            const u32 w = __ldg(headp + list_start(s_desc[lo]) + (q - s_ko[lo]));
            if (!bucket_insert(s_keys + (tb >> 5), tb & 31u, w)) dup = 1;
        }

        // walk this thread's items of the merge path and queue the edges this tile owns
        const u64 dt = d0 + (u64)threadIdx.x * IPT < d1 ? d0 + (u64)threadIdx.x * IPT : d1;
        const u64 dte = dt + IPT < d1 ? dt + IPT : d1;
        // merge-path search in the window: largest i in [i0, i1] with first_out[i] + i <= dt
        u64 i_start;
        {
            u64 lo = i0, hi = i1;
            while (lo < hi) {
                const u64 mid = (lo + hi + 1) >> 1;
                if ((u64)s_fo[mid - i0] + j0 + mid <= dt) lo = mid; else hi = mid - 1;
            }
            i_start = lo;
        }
        u32 own[IPT], yv[IPT];
        {
            u64 i = i_start;
            u32 j = (u32)(dt - i_start - j0);  // slot relative to the tile's first slot
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                own[k] = NONE;
                yv[k] = 0;
                if (dt + k < dte) {
                    if (i < n && j < s_fo[i + 1 - i0]) {
                        const u32 o = (u32)(i - i0);
                        const u32 d = s_desc[o].d;
                        if (d > 0 && d <= sd) {
                            own[k] = o;
                            yv[k] = __ldg(head + j0 + j);
                        }
                        ++j;
                    } else {
                        ++i;
                    }
                }
            }
        }
        Desc<OffT> vy[IPT];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            vy[k].start = 0;
            vy[k].d = 0;
            if (own[k] != NONE && yv[k] < n) vy[k] = load_desc(vdesc + yv[k]);
        }
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const u32 o = own[k];
            bool sel = false;
            if (o != NONE) {
                const u32 dy = vy[k].d;
                sel = dy > 0 && key_less(dy, yv[k], s_desc[o].d, i0 + o);
            }
            const u32 ball = __ballot_sync(0xFFFFFFFFu, sel);
            u32 base = 0;
            if (lane == 0 && ball) base = atomicAdd(&s_qn, (u32)__popc(ball));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (sel) {
                const u32 qi = base + __popc(ball & ((1u << lane) - 1));
                q_y[qi] = yv[k];
                q_s[qi] = (OffT)list_group(vy[k]);
                q_m[qi] = (unsigned short)((o << 6) | vy[k].d);
                atomicAdd(&s_bins[vy[k].d], 1u);
            }
        }
        __syncthreads();

        // counting sort of the queue by list length; the key offsets are no longer needed and
        // their words become the owners' hit totals
        for (u32 k = threadIdx.x; k < nw; k += BLOCK) s_own[k] = 0;
        const u32 qn = s_qn;
        if (threadIdx.x < 32) {
            u32 c0 = s_bins[lane], c1 = lane + 32 < SD + 2 ? s_bins[lane + 32] : 0;
            u32 x0 = c0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                u32 y = __shfl_up_sync(0xFFFFFFFFu, x0, o);
                if (lane >= o) x0 += y;
            }
            const u32 tot0 = __shfl_sync(0xFFFFFFFFu, x0, 31);
            u32 x1 = c1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                u32 y = __shfl_up_sync(0xFFFFFFFFu, x1, o);
                if (lane >= o) x1 += y;
            }
            s_bins[lane] = x0 - c0;
            if (lane + 32 < SD + 2) s_bins[lane + 32] = tot0 + x1 - c1;
        }
        __syncthreads();
        for (u32 qi = threadIdx.x; qi < qn; qi += BLOCK) {
            const u32 pos = atomicAdd(&s_bins[q_m[qi] & 63u], 1u);
            q_ord[pos] = (unsigned short)qi;
        }
        __syncthreads();

        // stream the queued lists: warps take chunks of 32 from the length-sorted queue, longest
        // first, so the lanes of a warp carry equal lengths and the warps finish together
        while (true) {
            u32 c32 = 0;
            if (lane == 0) c32 = atomicAdd(&s_chunk, 32u);
            c32 = __shfl_sync(0xFFFFFFFFu, c32, 0);
            if (c32 >= qn) break;
            const u32 r = c32 + lane;
            if (r >= qn) continue;
            const u32 qi = q_ord[qn - 1 - r];
            const u32 meta = q_m[qi];
            const u32 o = meta >> 6, dy = meta & 63u;
            const u32 tb = s_tb[o];
            const u32* keys = s_keys + (tb >> 5);
            u32* hitc = s_hits + ((tb >> 5) >> 1);  // table offsets are multiples of 4 slots
            const u32 lg = tb & 31u;
            const u64 q0 = (u64)q_s[qi];
            u32 hits = 0;
            // the list's 16-byte groups are loaded PRE at a time before any probe, so their
            // latencies overlap instead of adding up
            constexpr int PRE = 4;
#pragma unroll 1
            for (int c0 = 0; c0 < SD / 4; c0 += PRE) {
                if (4 * c0 >= (int)dy) break;
                uint4 qv[PRE];
#pragma unroll
                for (int c = 0; c < PRE; ++c)
                    qv[c] = 4 * (c0 + c) < (int)dy ? __ldg(headp4 + q0 + c0 + c)
                                                   : make_uint4(EMPTY_KEY, EMPTY_KEY, EMPTY_KEY, EMPTY_KEY);
#pragma unroll
                for (int c = 0; c < PRE; ++c) {
                    const int e = 4 * (c0 + c);
                    if (e < (int)dy) hits += bucket_probe16(keys, hitc, lg, qv[c].x);
                    if (e + 1 < (int)dy) hits += bucket_probe16(keys, hitc, lg, qv[c].y);
                    if (e + 2 < (int)dy) hits += bucket_probe16(keys, hitc, lg, qv[c].z);
                    if (e + 3 < (int)dy) hits += bucket_probe16(keys, hitc, lg, qv[c].w);
                }
            }
            if (hits) {
                atomicAdd(&cnt[q_y[qi]], (u64)hits);
                atomicAdd(&s_own[o], hits);
            }
        }
        __syncthreads();

        // flush: hits of every key (vertex w), then the owners' own counts
        for (u32 s = threadIdx.x; s < table_slots; s += BLOCK) {
            const u32 h = read16(s_hits, s);
            if (h) atomicAdd(&cnt[s_keys[s]], (u64)h);
        }
        for (u32 k = threadIdx.x; k < nw; k += BLOCK) {
            const u32 t = s_own[k];
            if (t) {
                atomicAdd(&cnt[i0 + k], (u64)t);
                local_total += t;
            }
        }
        __syncthreads();
    }
    if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
    const u64 bt = block_sum_u64<BLOCK>(local_total, s_red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bt;
}

// Small owners, one warp per owner (the form used when Options.small_kernel selects it): a
// warp takes 32 consecutive vertices at a time and, for each owner among them (out-degree
// 1..small_outdegree, degree at most SMALL_WARP_DEG; owners of larger degree go to the medium
// kernel's tiles), fills its own slice of shared memory with the owner's table and streams the
// out-list of every lower neighbour through it, one list per lane.  No block barrier: the warps
// of a block never wait for one another.
template <int SD>
struct SmallWarpLayout {
    static constexpr int TS = SD <= 32 ? 64 : 128;  // table slots: a power of two >= 2 * SD
    static constexpr int PER_WARP = TS + TS / 2;     // keys, then two 16-bit hit counters per word
};

template <int BLOCK, int SD, typename OffT>
__global__ void __launch_bounds__(BLOCK, 4) k_count_small_warp(const u64* __restrict__ fo, const u32* __restrict__ head,
                                                            u64 n, const Desc<OffT>* __restrict__ vdesc,
                                                            const u32* __restrict__ headp, u32 sd,
                                                            u64* __restrict__ cnt, u64* __restrict__ partials,
                                                            Control* ctl) {
    using L = SmallWarpLayout<SD>;
    constexpr int NW = BLOCK / 32;
    static_assert(2 * SD <= L::TS, "a table holds twice the owner's keys");
    __shared__ __align__(16) u32 s_tab[NW * L::PER_WARP];
    __shared__ u64 s_red[NW];
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32* keys = s_tab + warp * L::PER_WARP;
    u32* hitc = keys + L::TS;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    const u64 nbatch = (n + 31) / 32;
    u64 local_total = 0;
    u32 dup = 0;
    while (true) {
        unsigned long long bi = 0;
        if (lane == 0) bi = atomicAdd(&ctl->small_next, 1ull);
        bi = __shfl_sync(0xFFFFFFFFu, bi, 0);
        if (bi >= nbatch) break;
        const u64 v = bi * 32 + lane;
        Desc<OffT> dv;
        dv.start = 0;
        dv.d = 0;
        u64 a = 0, b = 0;
        bool own = false;
        if (v < n) {
            dv = load_desc(vdesc + v);
            a = fo[v];
            b = fo[v + 1];
            own = dv.d > 0 && dv.d <= sd && b - a <= (u64)SMALL_WARP_DEG;
        }
        const u64 vs = list_start(dv);
        u32 todo = __ballot_sync(0xFFFFFFFFu, own);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const u64 x = bi * 32 + src;
            const u32 dx = __shfl_sync(0xFFFFFFFFu, dv.d, src);
            const u64 xs = __shfl_sync(0xFFFFFFFFu, vs, src);
            const u64 xa = __shfl_sync(0xFFFFFFFFu, a, src);
            const u32 xdeg = (u32)(__shfl_sync(0xFFFFFFFFu, b, src) - xa);
            u32 lg = ceil_log2(2 * dx);
            if (lg < 2) lg = 2;
            const u32 size = 1u << lg;
            for (u32 i = lane; i < size; i += 32) keys[i] = EMPTY_KEY;
            for (u32 i = lane; i < size / 2; i += 32) hitc[i] = 0;
            __syncwarp();
            for (u32 q = lane; q < dx; q += 32)
                if (!bucket_insert(keys, lg, __ldg(headp + xs + q))) dup = 1;
            __syncwarp();
            u32 T = 0;
            for (u32 e0 = 0; e0 < xdeg; e0 += 32) {
                u32 hits = 0;
                if (e0 + lane < xdeg) {
                    const u32 y = __ldg(head + xa + e0 + lane);
                    if (y < n) {
                        const Desc<OffT> vy = load_desc(vdesc + y);
                        const u32 dy = vy.d;
                        if (dy > 0 && key_less(dy, y, dx, x)) {
                            // the list's 16-byte groups, four loads in flight before the probes
                            const u64 q0 = list_group(vy);
                            for (u32 g0 = 0; 4 * g0 < dy; g0 += 4) {
                                uint4 qv[4];
#pragma unroll
                                for (int c = 0; c < 4; ++c)
                                    qv[c] = 4 * (g0 + c) < dy ? __ldg(headp4 + q0 + g0 + c)
                                                              : make_uint4(EMPTY_KEY, EMPTY_KEY, EMPTY_KEY, EMPTY_KEY);
#pragma unroll
                                for (int c = 0; c < 4; ++c) {
                                    const u32 e = 4 * (g0 + c);
                                    if (e < dy) hits += bucket_probe16(keys, hitc, lg, qv[c].x);
                                    if (e + 1 < dy) hits += bucket_probe16(keys, hitc, lg, qv[c].y);
                                    if (e + 2 < dy) hits += bucket_probe16(keys, hitc, lg, qv[c].z);
                                    if (e + 3 < dy) hits += bucket_probe16(keys, hitc, lg, qv[c].w);
                                }
                            }
                            if (hits) atomicAdd(&cnt[y], (u64)hits);
                        }
                    }
                }
                T += hits;
            }
            __syncwarp();
            for (u32 i = lane; i < size; i += 32) {
                const u32 h = read16(hitc, i);
                if (h) atomicAdd(&cnt[keys[i]], (u64)h);
            }
            T = __reduce_add_sync(0xFFFFFFFFu, T);
            if (lane == 0 && T) {
                atomicAdd(&cnt[x], (u64)T);
                local_total += T;
            }
            __syncwarp();  // the next owner clears the table only after every lane has flushed
        }
    }
    if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
    const u64 bt = block_sum_u64<BLOCK>(local_total, s_red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bt;
}

template <int BLOCK, int CAP, typename OffT>
struct LargeLayout {
    static constexpr int TS = 2 * CAP;       // table slots (at most half full)
    static constexpr int FWORDS = CAP / 2;   // filter words: 16 bits per key at CAP keys
    static constexpr int WBUF = 64;          // per-warp buffer of filter survivors
    static constexpr size_t off_keys = 0;
    static constexpr size_t off_hits = align16(off_keys + sizeof(u32) * TS);         // two u16 counters per word
    static constexpr size_t off_filt = align16(off_hits + sizeof(u32) * (TS / 2));
    static constexpr size_t off_wbuf = align16(off_filt + sizeof(u32) * FWORDS);
    static constexpr size_t off_qy = align16(off_wbuf + sizeof(u32) * WBUF * (BLOCK / 32));
    static constexpr size_t off_qd = align16(off_qy + sizeof(u32) * LARGE_SEG);
    static constexpr size_t bytes = align16(off_qd + sizeof(Desc<OffT>) * LARGE_SEG);
};

// One-hash membership filter of the owner's keys (2^fl bits): a clear bit is a sure miss.
__device__ __forceinline__ u32 filter_bit(u32 w, u32 fl) { return (w * 0x85EBCA6Bu) >> (32 - fl); }
__device__ __forceinline__ bool filter_test(const u32* filt, u32 fl, u32 w) {
    const u32 h = filter_bit(w, fl);
    return (filt[h >> 5] >> (h & 31u)) & 1u;
}

// A whole warp streams one list (d entries at lst) through the owner's filter and table.
// Entries that pass the filter are packed into the warp's buffer (64 entries) and looked up
// 32 at a time.  Returns this lane's share of the hits.
template <int U>
__device__ __forceinline__ u32 warp_stream_list(const u32* __restrict__ lst, u32 d, const u32* keys, u32* hitc, u32 lg,
                                                const u32* filt, u32 fl, u32* wbuf, int lane, u32 lt_mask) {
    u32 hits = 0, nbuf = 0;
    // a running pointer and a running count of the entries left from this lane's position,
    // so each load is one instruction with an immediate offset and one compare
    const u32* lp = lst + lane;
    int rem = (int)d - lane;
    for (u32 p0 = 0; p0 < d; p0 += 32 * U, lp += 32 * U, rem -= 32 * U) {
        u32 w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) w[u] = rem > 32 * u ? __ldg(lp + 32 * u) : EMPTY_KEY;
        const int left = (int)(d - p0);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (left <= 32 * u) break;
            // both tests evaluated (no branch): past the list's end w[u] is EMPTY_KEY, a harmless
            // filter read whose result the range test masks
            const bool maybe = (rem > 32 * u) & filter_test(filt, fl, w[u]);
            const u32 ball = __ballot_sync(0xFFFFFFFFu, maybe);
            if (maybe) wbuf[nbuf + __popc(ball & lt_mask)] = w[u];
            nbuf += __popc(ball);
            if (nbuf >= 32) {
                __syncwarp();
                hits += bucket_probe16_flat(keys, hitc, lg, wbuf[lane]);
                const u32 rest = nbuf - 32;
                const u32 carry = lane < rest ? wbuf[32 + lane] : 0u;
                __syncwarp();
                if (lane < rest) wbuf[lane] = carry;
                __syncwarp();
                nbuf = rest;
            }
        }
    }
    __syncwarp();
    if (lane < nbuf) hits += bucket_probe16_flat(keys, hitc, lg, wbuf[lane]);
    __syncwarp();
    return hits;
}

// A lane streams one short list (d <= LONG_LIST entries, 16-byte aligned) through the owner's
// filter and table.
template <typename OffT>
__device__ __forceinline__ u32 lane_stream_short(const uint4* __restrict__ headp4, const Desc<OffT>& vy,
                                                 const u32* keys, u32* hitc, u32 lg, const u32* filt, u32 fl) {
    const u32 dy = vy.d;
    const u64 q0 = list_group(vy);
    uint4 qv[LONG_LIST / 4];
#pragma unroll
    for (int c = 0; c < LONG_LIST / 4; ++c)
        qv[c] = 4 * c < (int)dy ? __ldg(headp4 + q0 + c) : make_uint4(EMPTY_KEY, EMPTY_KEY, EMPTY_KEY, EMPTY_KEY);
    u32 hits = 0;
#pragma unroll
    for (int c = 0; c < LONG_LIST / 4; ++c) {
        if (4 * c < (int)dy) {
            const u32 wv[4] = {qv[c].x, qv[c].y, qv[c].z, qv[c].w};
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if ((4 * c + k < (int)dy) & filter_test(filt, fl, wv[k])) hits += bucket_probe16(keys, hitc, lg, wv[k]);
        }
    }
    return hits;
}

// Table and filter sizes of an owner chunk of klen keys: a quarter-full table (at most
// max_lg) and 16 filter bits per key (at most max_fl).
__device__ __forceinline__ void chunk_sizes(u32 klen, u32 max_lg, u32 max_fl, u32* lg, u32* fl) {
    u32 a = ceil_log2(4 * klen);
    if (a > max_lg) a = max_lg;
    if (a < 2) a = 2;
    u32 f = ceil_log2(16 * klen);
    if (f > max_fl) f = max_fl;
    if (f < 5) f = 5;
    *lg = a;
    *fl = f;
}

template <int BLOCK, int CAP, typename OffT>
__global__ void __launch_bounds__(BLOCK) k_count_large(const u64* __restrict__ fo, const u32* __restrict__ head,
                                                       u64 n, const Desc<OffT>* __restrict__ vdesc,
                                                       const u32* __restrict__ headp,
                                                       const uint2* __restrict__ ltiles, u32 seg,
                                                       u64* __restrict__ cnt, u64* __restrict__ partials,
                                                       Control* ctl, u32 first_wait_polls) {
    using L = LargeLayout<BLOCK, CAP, OffT>;
    constexpr int NW = BLOCK / 32;
    constexpr int U = 8;  // loads in flight per lane and list
    extern __shared__ __align__(16) unsigned char smem[];
    u32* keys = reinterpret_cast<u32*>(smem + L::off_keys);
    u32* hitc = reinterpret_cast<u32*>(smem + L::off_hits);
    u32* filt = reinterpret_cast<u32*>(smem + L::off_filt);
    u32* qy = reinterpret_cast<u32*>(smem + L::off_qy);
    Desc<OffT>* qd = reinterpret_cast<Desc<OffT>*>(smem + L::off_qd);
    __shared__ u64 s_red[NW];
    __shared__ u64 s_t;
    __shared__ u32 s_qn, s_next;
    __shared__ __align__(8) unsigned long long s_bar;  // completion of the owner-list bulk copy

    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) mbar_init(&s_bar, 1);
    fence_proxy_async_smem();
    __syncthreads();
    u32 phase = 0;
    bool timed_out = false, inflight = false;
    // the owner's keys are staged in the queue's descriptor region, which is free until the scan
    u32* stage = reinterpret_cast<u32*>(smem + L::off_qd);
    static_assert(sizeof(Desc<OffT>) * LARGE_SEG >= sizeof(u32) * CAP, "staging fits the queue region");
    u32* wbuf = reinterpret_cast<u32*>(smem + L::off_wbuf) + warp * L::WBUF;
    const u32 lt_mask = (1u << lane) - 1;
    const u64 ntiles = *(volatile unsigned long long*)&ctl->large_tiles;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    u64 local_total = 0;
    u32 dup = 0;

    while (true) {
        if (threadIdx.x == 0) s_t = atomicAdd(&ctl->large_next, 1ull);
        __syncthreads();
        const u64 t = s_t;
        if (t >= ntiles) break;
        const uint2 tl = ltiles[t];
        const u64 x = tl.x;
        const Desc<OffT> dxd = load_desc(vdesc + x);
        const u32 dx = dxd.d;
        const u64 fx1 = fo[x + 1];
        const u64 a = fo[x] + (u64)tl.y * seg;
        const u64 b = a + seg < fx1 ? a + seg : fx1;
        u64 T = 0;
        for (u32 c0 = 0; c0 < dx; c0 += CAP) {
            const u32 klen = dx - c0 < (u32)CAP ? dx - c0 : (u32)CAP;
            u32 lg, fl;
            chunk_sizes(klen, 31 - __clz((u32)L::TS), 31 - __clz((u32)(L::FWORDS * 32)), &lg, &fl);
            const u32 size = 1u << lg, fwords = (1u << fl) >> 5;
            for (u32 s = threadIdx.x; s < size; s += BLOCK) keys[s] = EMPTY_KEY;
            for (u32 s = threadIdx.x; s < size / 2; s += BLOCK) hitc[s] = 0;
            for (u32 s = threadIdx.x; s < fwords; s += BLOCK) filt[s] = 0;
            if (threadIdx.x == 0) {
                s_qn = 0;
                s_next = 0;
            }
            fence_proxy_async_smem();  // earlier generic accesses of the staging region come first
            __syncthreads();
            // one bulk copy of the chunk's keys (list starts are 16-byte aligned, and the gapped
            // layout leaves room to round the length up to whole 16-byte groups)
            if (threadIdx.x == 0) {
                const u32 bytes = ((klen + 3u) & ~3u) * (u32)sizeof(u32);
                mbar_expect_tx(&s_bar, bytes);
                bulk_copy_g2s(stage, headp + list_start(dxd) + c0, bytes, &s_bar);
            }
            const bool arrived = mbar_wait_bounded(&s_bar, phase, first_wait_polls);
            if (__syncthreads_or(!arrived)) {  // the same decision in every thread
                // give the copy in flight a second bounded wait, so that it does not land in
                // shared memory after the block has left; then report the timeout (and, if the
                // copy still has not landed, that it may be in flight as the block leaves)
                if (!__syncthreads_or(!mbar_wait_bounded(&s_bar, phase, COPY_WAIT_POLLS))) timed_out = true;
                else timed_out = inflight = true;
                break;
            }
            phase ^= 1u;
            for (u32 q = threadIdx.x; q < klen; q += BLOCK) {
                const u32 w = stage[q];
                if (!bucket_insert(keys, lg, w)) dup = 1;
                const u32 h = filter_bit(w, fl);
                atomicOr(&filt[h >> 5], 1u << (h & 31u));
            }
            __syncthreads();
            // scan the segment: short lists now, long lists into the queue
            for (u64 e0 = a + (u64)warp * 32; e0 < b; e0 += (u64)NW * 32) {
                const u64 e = e0 + lane;
                bool queue = false;
                u32 y = 0;
                Desc<OffT> vy;
                vy.start = 0;
                vy.d = 0;
                if (e < b) {
                    y = __ldg(head + e);
                    if (y < n) vy = load_desc(vdesc + y);
                    const u32 dy = vy.d;
                    if (dy > 0 && key_less(dy, y, dx, x)) {
                        if (dy <= (u32)LONG_LIST) {
                            const u32 hits = lane_stream_short<OffT>(headp4, vy, keys, hitc, lg, filt, fl);
                            if (hits) {
                                atomicAdd(&cnt[y], (u64)hits);
                                T += hits;
                            }
                        } else {
                            queue = true;
                        }
                    }
                }
                const u32 ball = __ballot_sync(0xFFFFFFFFu, queue);
                u32 base = 0;
                if (lane == 0 && ball) base = atomicAdd(&s_qn, (u32)__popc(ball));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (queue) {
                    const u32 qi = base + __popc(ball & lt_mask);
                    qy[qi] = y;
                    qd[qi] = vy;
                }
            }
            __syncthreads();
            // long lists: one warp per list, taken from the queue.  Every entry is tested against
            // the filter; the survivors are packed into the warp's buffer and looked up in the
            // table 32 at a time, so the lookups run with full warps.
            const u32 qn = s_qn;
            while (true) {
                u32 qi = 0;
                if (lane == 0) qi = atomicAdd(&s_next, 1u);
                qi = __shfl_sync(0xFFFFFFFFu, qi, 0);
                if (qi >= qn) break;
                const Desc<OffT> vy = qd[qi];
                u32 hits = warp_stream_list<U>(headp + list_start(vy), vy.d, keys, hitc, lg, filt, fl, wbuf, lane,
                                               lt_mask);
                hits = __reduce_add_sync(0xFFFFFFFFu, hits);
                if (lane == 0 && hits) {
                    atomicAdd(&cnt[qy[qi]], (u64)hits);
                    T += hits;
                }
            }
            __syncthreads();
            // flush the hits of every key
            for (u32 s = threadIdx.x; s < size; s += BLOCK) {
                const u32 h = read16(hitc, s);
                if (h) atomicAdd(&cnt[keys[s]], (u64)h);
            }
            __syncthreads();
        }
        const u64 bt = block_sum_u64<BLOCK>(T, s_red);
        if (threadIdx.x == 0 && bt) {
            atomicAdd(&cnt[x], bt);
            local_total += bt;
        }
        if (timed_out) break;
    }
    if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
    if (timed_out) atomicOr(&ctl->err, DEV_ERR_TIMEOUT | (inflight ? DEV_ERR_COPY_INFLIGHT : 0u));
    if (threadIdx.x == 0) partials[blockIdx.x] = local_total;
}

// Medium owners (small threshold < out-degree <= MEDIUM_D): one warp per (owner, segment)
// tile, with its own table, filter and buffer in shared memory, so a tile needs no block
// barrier.  Most owner tiles of skewed graphs are of this kind and carry little work each.
template <int BLOCK>
struct MediumLayout {
    static constexpr int NW = BLOCK / 32;
    static constexpr int TS = 2 * MEDIUM_D;  // table slots per warp (a quarter to half full)
    static constexpr int FW = MEDIUM_D / 2;  // filter words per warp (16 bits per key)
    static constexpr int WBUF = 64;
    static constexpr int PER_WARP = TS + TS / 2 + FW + WBUF;  // u32 words: keys, 16-bit hits, filter, buffer
    static constexpr size_t bytes = sizeof(u32) * PER_WARP * NW;
};

template <int BLOCK, typename OffT>
__global__ void __launch_bounds__(BLOCK)
    k_count_medium(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                   const Desc<OffT>* __restrict__ vdesc, const u32* __restrict__ headp,
                   const uint2* __restrict__ mtiles, u32 seg, u64* __restrict__ cnt,
                   u64* __restrict__ partials, Control* ctl) {
    using L = MediumLayout<BLOCK>;
    constexpr int U = 4;  // medium owners' streamed lists are shorter than 256 entries
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ u64 s_red[L::NW];
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32* keys = reinterpret_cast<u32*>(smem) + warp * L::PER_WARP;
    u32* hitc = keys + L::TS;
    u32* filt = hitc + L::TS / 2;
    u32* wbuf = filt + L::FW;
    const u32 lt_mask = (1u << lane) - 1;
    const u64 ntiles = *(volatile unsigned long long*)&ctl->medium_tiles;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    u64 local_total = 0;
    u32 dup = 0;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&ctl->medium_next, 1ull);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        if (t >= ntiles) break;
        const uint2 tl = mtiles[t];
        const u64 x = tl.x;
        const Desc<OffT> dxd = load_desc(vdesc + x);
        const u32 dx = dxd.d;
        const u64 fx1 = fo[x + 1];
        const u64 a = fo[x] + (u64)tl.y * seg;
        const u64 b = a + seg < fx1 ? a + seg : fx1;
        u32 lg, fl;
        chunk_sizes(dx, 31 - __clz((u32)L::TS), 31 - __clz((u32)(L::FW * 32)), &lg, &fl);
        const u32 size = 1u << lg, fwords = (1u << fl) >> 5;
        for (u32 i = lane; i < size; i += 32) keys[i] = EMPTY_KEY;
        for (u32 i = lane; i < size / 2; i += 32) hitc[i] = 0;
        for (u32 i = lane; i < fwords; i += 32) filt[i] = 0;
        __syncwarp();
        for (u32 q = lane; q < dx; q += 32) {
            const u32 w = __ldg(headp + list_start(dxd) + q);
            if (!bucket_insert(keys, lg, w)) dup = 1;
            const u32 h = filter_bit(w, fl);
            atomicOr(&filt[h >> 5], 1u << (h & 31u));
        }
        __syncwarp();
        u32 T = 0;
        for (u64 e0 = a; e0 < b; e0 += 32) {
            const u64 e = e0 + lane;
            u32 y = 0;
            Desc<OffT> vy;
            vy.start = 0;
            vy.d = 0;
            bool longl = false;
            if (e < b) {
                y = __ldg(head + e);
                vy = load_desc(vdesc + y);
                const u32 dy = vy.d;
                if (dy > 0 && key_less(dy, y, dx, x)) {
                    if (dy <= (u32)LONG_LIST) {
                        const u32 hits = lane_stream_short<OffT>(headp4, vy, keys, hitc, lg, filt, fl);
                        if (hits) {
                            atomicAdd(&cnt[y], (u64)hits);
                            T += hits;
                        }
                    } else {
                        longl = true;
                    }
                }
            }
            u32 ball = __ballot_sync(0xFFFFFFFFu, longl);
            while (ball) {  // the warp streams this chunk's long lists one at a time
                const int src = __ffs(ball) - 1;
                ball &= ball - 1;
                const u32 yy = __shfl_sync(0xFFFFFFFFu, y, src);
                const u64 ys = (u64)__shfl_sync(0xFFFFFFFFu, (unsigned long long)list_start(vy), src);
                const u32 yd = __shfl_sync(0xFFFFFFFFu, vy.d, src);
                u32 hits = warp_stream_list<U>(headp + ys, yd, keys, hitc, lg, filt, fl, wbuf, lane, lt_mask);
                hits = __reduce_add_sync(0xFFFFFFFFu, hits);
                if (lane == 0 && hits) {
                    atomicAdd(&cnt[yy], (u64)hits);
                    T += hits;
                }
            }
        }
        __syncwarp();
        for (u32 i = lane; i < size; i += 32) {
            const u32 h = read16(hitc, i);
            if (h) atomicAdd(&cnt[keys[i]], (u64)h);
        }
        const u32 wt = __reduce_add_sync(0xFFFFFFFFu, T);
        if (lane == 0 && wt) {
            atomicAdd(&cnt[x], (u64)wt);
            local_total += wt;
        }
        __syncwarp();
    }
    if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
    const u64 bt = block_sum_u64<BLOCK>(local_total, s_red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bt;
}

// Sum of the per-block partial totals (a u64 tree reduction in one block).  After a device
// error (invalid input, a bounded wait that ran out) the partials are incomplete or stale, so
// the total is written as 0.
__global__ void __launch_bounds__(1024) k_final(const u64* __restrict__ partials, u32 np, u64* total,
                                                const Control* ctl) {
    __shared__ u64 s_red[32];
    if (*(volatile const u32*)&ctl->err & DEV_ERR_MASK) {
        if (threadIdx.x == 0) *total = 0;
        return;
    }
    u64 s = 0;
    for (u32 i = threadIdx.x; i < np; i += 1024) s += partials[i];
    const u64 t = block_sum_u64<1024>(s, s_red);
    if (threadIdx.x == 0) *total = t;
}

// Batched counting: per-graph totals of a disjoint union (graph g owns the vertices
// [graph_first[g], graph_first[g+1])).  Every triangle adds one to each of its three corners,
// all inside one graph, so a graph's total is the sum of its per-vertex counts over three.
__global__ void __launch_bounds__(256) k_graph_totals(const u64* __restrict__ cnt, const u64* __restrict__ graph_first,
                                                      u64 num_graphs, u64 n, u64* __restrict__ totals, Control* ctl) {
    __shared__ u64 s_red[8];
    if (ctl->err & DEV_ERR_MASK) return;
    for (u64 g = blockIdx.x; g < num_graphs; g += gridDim.x) {
        const u64 a = graph_first[g], b = graph_first[g + 1];
        const bool ok = a <= b && b <= n;
        u64 s = 0;
        if (ok)
            for (u64 v = a + threadIdx.x; v < b; v += 256) s += cnt[v];
        s = block_sum_u64<256>(s, s_red);
        if (threadIdx.x == 0) {
            totals[g] = ok ? s / 3 : 0;
            if (!ok) atomicOr(&ctl->err, DEV_ERR_DEGREE);
        }
    }
}

// collect_stats: wedge_checks = sum over oriented (v,u) of |N+(u)|, the reference's counter
// (cetric_edge_iterator.h:279-281), plus the entries streamed by the AUTO kernels, also counted
// once per table chunk of their owner (owners above medium_d keep at most LARGE_CAP keys per
// chunk and stream their segment once per chunk).
template <typename OffT>
__global__ void k_stats(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                        const Desc<OffT>* __restrict__ vdesc, const u32* __restrict__ headp, u32 medium_d,
                        Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31;
    const u64 gw = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    u64 wedge = 0, isz = 0, streamed = 0, oriented = 0, chunked = 0;
    for (u64 v = gw; v < n; v += nwarps) {
        const Desc<OffT> dv = load_desc(vdesc + v);
        const u64 chunks = dv.d > medium_d ? (dv.d + LARGE_CAP - 1) / LARGE_CAP : 1;
        if (lane == 0) oriented += dv.d;
        for (u32 k = lane; k < dv.d; k += 32) {
            const u32 u = headp[list_start(dv) + k];
            const u32 du = load_desc(vdesc + u).d;
            wedge += du;
            isz += (u64)dv.d + du;
        }
        for (u64 e = fo[v] + lane; e < fo[v + 1]; e += 32) {
            const u32 y = head[e];
            const u32 dy = load_desc(vdesc + y).d;
            if (dy > 0 && key_less(dy, y, dv.d, v)) {
                streamed += dy;
                chunked += dy * chunks;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        wedge += __shfl_down_sync(0xFFFFFFFFu, wedge, o);
        isz += __shfl_down_sync(0xFFFFFFFFu, isz, o);
        streamed += __shfl_down_sync(0xFFFFFFFFu, streamed, o);
        oriented += __shfl_down_sync(0xFFFFFFFFu, oriented, o);
        chunked += __shfl_down_sync(0xFFFFFFFFu, chunked, o);
    }
    if (lane == 0) {
        atomicAdd(&ctl->stat_wedge, wedge);
        atomicAdd(&ctl->stat_isz, isz);
        atomicAdd(&ctl->stat_streamed, streamed);
        atomicAdd(&ctl->stat_oriented, oriented);
        atomicAdd(&ctl->stat_chunked, chunked);
    }
}

// ---- launchers ------------------------------------------------------------------------

namespace {
template <int SD, typename OffT>
using SmallL = SmallLayout<SMALL_BLOCK, SMALL_IPT, SD, OffT>;
template <typename OffT>
using LargeL = LargeLayout<LARGE_BLOCK, LARGE_CAP, OffT>;
using MediumL = MediumLayout<MEDIUM_BLOCK>;

template <int SD, typename OffT>
int occupancy_small() {
    static int occ = -1;
    if (occ < 0) {
        auto kern = k_count_small<SMALL_BLOCK, SMALL_IPT, SD, OffT>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SmallL<SD, OffT>::bytes);
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, SMALL_BLOCK, SmallL<SD, OffT>::bytes);
        occ = o > 0 ? o : 1;
    }
    return occ;
}
template <int SD, typename OffT>
int occupancy_small_warp() {
    static int occ = -1;
    if (occ < 0) {
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_count_small_warp<SMALL_BLOCK, SD, OffT>, SMALL_BLOCK, 0);
        occ = o > 0 ? o : 1;
    }
    return occ;
}
template <typename OffT>
int occupancy_medium() {
    static int occ = -1;
    if (occ < 0) {
        auto kern = k_count_medium<MEDIUM_BLOCK, OffT>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MediumL::bytes);
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, MEDIUM_BLOCK, MediumL::bytes);
        occ = o > 0 ? o : 1;
    }
    return occ;
}
template <typename OffT>
int occupancy_large() {
    static int occ = -1;
    if (occ < 0) {
        auto kern = k_count_large<LARGE_BLOCK, LARGE_CAP, OffT>;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LargeL<OffT>::bytes);
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, LARGE_BLOCK, LargeL<OffT>::bytes);
        occ = o > 0 ? o : 1;
    }
    return occ;
}
}  // namespace

template <typename OffT>
int count_grid_small(int num_sms, u32 small_d, bool warp) {
    if (warp)
        return num_sms * (small_d <= (u32)SMALL_D_LOW ? occupancy_small_warp<SMALL_D_LOW, OffT>()
                                                      : occupancy_small_warp<SMALL_D, OffT>());
    return num_sms * (small_d <= (u32)SMALL_D_LOW ? occupancy_small<SMALL_D_LOW, OffT>()
                                                  : occupancy_small<SMALL_D, OffT>());
}
template <typename OffT>
int count_grid_medium(int num_sms) {
    return num_sms * occupancy_medium<OffT>();
}
template <typename OffT>
int count_grid_large(int num_sms) {
    return num_sms * occupancy_large<OffT>();
}
template <typename OffT>
int count_grid_auto(int num_sms, u32 small_d, bool warp) {
    return count_grid_small<OffT>(num_sms, small_d, warp) + count_grid_medium<OffT>(num_sms) +
           count_grid_large<OffT>(num_sms);
}

template <typename OffT>
cudaError_t launch_count_auto(const u64* fo, const u32* head, u64 n, u64 nnz, const void* vdesc, const u32* headp,
                              const u32* tile_i0, const uint2* mtiles, const uint2* ltiles, u32 small_d, u32 seg,
                              u64* cnt, u64* partials, Control* ctl, int num_sms, cudaStream_t st,
                              cudaEvent_t after_small, cudaEvent_t after_large, u32 copy_wait_polls,
                              bool small_warp) {
    const int gs = count_grid_small<OffT>(num_sms, small_d, small_warp);
    const int gm = count_grid_medium<OffT>(num_sms);
    const int gl = count_grid_large<OffT>(num_sms);
    const auto* vd = reinterpret_cast<const Desc<OffT>*>(vdesc);
    if (small_warp && small_d <= (u32)SMALL_D_LOW)
        k_count_small_warp<SMALL_BLOCK, SMALL_D_LOW, OffT>
            <<<gs, SMALL_BLOCK, 0, st>>>(fo, head, n, vd, headp, small_d, cnt, partials, ctl);
    else if (small_warp)
        k_count_small_warp<SMALL_BLOCK, SMALL_D, OffT>
            <<<gs, SMALL_BLOCK, 0, st>>>(fo, head, n, vd, headp, small_d, cnt, partials, ctl);
    else if (small_d <= (u32)SMALL_D_LOW)
        k_count_small<SMALL_BLOCK, SMALL_IPT, SMALL_D_LOW, OffT><<<gs, SMALL_BLOCK, SmallL<SMALL_D_LOW, OffT>::bytes, st>>>(
            fo, head, n, nnz, vd, headp, tile_i0, small_d, cnt, partials, ctl);
    else
        k_count_small<SMALL_BLOCK, SMALL_IPT, SMALL_D, OffT><<<gs, SMALL_BLOCK, SmallL<SMALL_D, OffT>::bytes, st>>>(
            fo, head, n, nnz, vd, headp, tile_i0, small_d, cnt, partials, ctl);
    if (after_small) cudaEventRecord(after_small, st);
    k_count_medium<MEDIUM_BLOCK, OffT>
        <<<gm, MEDIUM_BLOCK, MediumL::bytes, st>>>(fo, head, n, vd, headp, mtiles, seg, cnt, partials + gs, ctl);
    k_count_large<LARGE_BLOCK, LARGE_CAP, OffT>
        <<<gl, LARGE_BLOCK, LargeL<OffT>::bytes, st>>>(fo, head, n, vd, headp, ltiles, seg, cnt, partials + gs + gm,
                                                       ctl, copy_wait_polls);
    if (after_large) cudaEventRecord(after_large, st);
    return cudaGetLastError();
}

void launch_graph_totals(const u64* cnt, const u64* graph_first, u64 num_graphs, u64 n, u64* totals, Control* ctl,
                         int num_sms, cudaStream_t st) {
    if (num_graphs == 0) return;
    u64 blocks = num_graphs < (u64)num_sms * 8 ? num_graphs : (u64)num_sms * 8;
    k_graph_totals<<<(unsigned)blocks, 256, 0, st>>>(cnt, graph_first, num_graphs, n, totals, ctl);
}

void launch_final(const u64* partials, u32 np, u64* total, Control* ctl, cudaStream_t st) {
    k_final<<<1, 1024, 0, st>>>(partials, np, total, ctl);
}

template <typename OffT>
void launch_stats(const u64* fo, const u32* head, u64 n, const void* vdesc, const u32* headp, u32 medium_d,
                  Control* ctl, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    k_stats<OffT><<<num_sms * 8, 256, 0, st>>>(fo, head, n, reinterpret_cast<const Desc<OffT>*>(vdesc), headp,
                                               medium_d, ctl);
}

template int count_grid_small<u32>(int, u32, bool);
template int count_grid_small<u64>(int, u32, bool);
template int count_grid_large<u32>(int);
template int count_grid_large<u64>(int);
template int count_grid_medium<u32>(int);
template int count_grid_medium<u64>(int);
template int count_grid_auto<u32>(int, u32, bool);
template int count_grid_auto<u64>(int, u32, bool);
template cudaError_t launch_count_auto<u32>(const u64*, const u32*, u64, u64, const void*, const u32*, const u32*,
                                            const uint2*, const uint2*, u32, u32,
                                            u64*, u64*, Control*, int, cudaStream_t, cudaEvent_t, cudaEvent_t, u32,
                                            bool);
template cudaError_t launch_count_auto<u64>(const u64*, const u32*, u64, u64, const void*, const u32*, const u32*,
                                            const uint2*, const uint2*, u32, u32,
                                            u64*, u64*, Control*, int, cudaStream_t, cudaEvent_t, cudaEvent_t, u32,
                                            bool);
template void launch_stats<u32>(const u64*, const u32*, u64, const void*, const u32*, u32, Control*, int,
                                cudaStream_t);
template void launch_stats<u64>(const u64*, const u32*, u64, const void*, const u32*, u32, Control*, int,
                                cudaStream_t);

}  // namespace ktri
