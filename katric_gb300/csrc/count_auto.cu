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
//   k_count_small: owners with out-degree <= small_outdegree and degree <= SMALL_WARP_DEG
//     (instantiated for bounds up to SMALL_D_LOW and up to SMALL_D).  A warp takes 32
//     consecutive vertices and counts their owners in groups of up to eight that share its
//     slice of shared memory: tables side by side, one flattened pass over all their keys, one
//     over all their adjacency slots (queueing the lower neighbours' lists), a counting sort of
//     the queue by list length, then one list per lane with uint4 loads.  No block barrier.
//   k_count_medium: owners up to medium_outdegree (and small-out-degree owners of larger
//     degree), one warp per (owner, segment) tile with the warp's own table, filter and
//     survivor buffer, so tiles need no block barrier.
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

// Loads of the counting bodies.  The standalone kernels read through the read-only path
// (CG = false): their inputs do not change while they run.  The serving engine (CG = true) runs
// across many batches whose buffers other kernels rewrite meanwhile, so it reads at L2 only,
// where those writes are visible, never from lines an SM cached earlier.
template <bool CG, typename T>
__device__ __forceinline__ T ld_in(const T* p) {
    if constexpr (CG) return __ldcg(p);
    else return __ldg(p);
}
template <bool CG, typename OffT>
__device__ __forceinline__ Desc<OffT> ld_desc(const Desc<OffT>* p) {
    if constexpr (!CG) {
        return load_desc(p);
    } else if constexpr (sizeof(OffT) == 4) {
        const uint2 v = __ldcg(reinterpret_cast<const uint2*>(p));
        return Desc<OffT>{v.x, v.y};
    } else {
        const uint4 v = __ldcg(reinterpret_cast<const uint4*>(p));
        return Desc<OffT>{(u64)v.x | ((u64)v.y << 32), v.z, 0};
    }
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

// Index of the segment holding item base + lane, for segments that start at strictly increasing
// positions: before = segments started at or below base (at least one), starts = bit p set when
// a segment starts at base + p (p in 1..31).
__device__ __forceinline__ u32 segment_of(u32 before, u32 starts, u32 le_mask) {
    return before - 1 + __popc(starts & le_mask);
}
// Bit (s - base) for a segment start s inside (base, base + 32), else 0.
__device__ __forceinline__ u32 start_bit(bool have, u32 s, u32 base) {
    return (have && s > base && s < base + 32) ? 1u << (s - base) : 0u;
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

// Small owners (k_count_small), warp-granular.  A warp takes
// 32 consecutive vertices at a time and counts their owners (out-degree 1..small_outdegree,
// degree at most SMALL_WARP_DEG; owners of larger degree go to the medium kernel's tiles) in
// groups: up to GROUP owners whose tables fit TAB slots and whose adjacency fits QCAP slots
// share the warp's slice of shared memory.  Each phase runs over the whole group at once (all
// keys, then all adjacency slots, then all queued lists), so one round of global loads serves
// every owner of the group; the queue is counting-sorted by list length and streamed one list
// per lane, longest first.  Only __syncwarp orders the phases: the warps of a block never wait
// for one another.
template <int SD, typename OffT>
struct SmallWarpLayout {
    static constexpr int GROUP = 8;      // owners per group
    static constexpr int TAB = 256;      // table slots of a group (each table a power of two >= 2 d+)
    static constexpr int QCAP = 256;     // adjacency slots of a group (the queue's capacity)
    static constexpr int NBIN = SD + 2;  // list lengths 0..SD
    static constexpr int OW = 10;        // words per owner record
    // u32 words per warp
    static constexpr int W_KEYS = 0;
    static constexpr int W_HITS = W_KEYS + TAB;                         // two 16-bit counters per word
    static constexpr int W_QY = W_HITS + TAB / 2;
    static constexpr int W_QS = W_QY + QCAP;                            // list starts (OffT)
    static constexpr int W_QM = W_QS + QCAP * (int)(sizeof(OffT) / 4);  // (owner << 8) | length
    static constexpr int W_ORD = W_QM + QCAP;                           // queue order by length (u16)
    static constexpr int W_BIN = W_ORD + QCAP / 2;                      // 64 length bins
    static constexpr int W_OWN = W_BIN + 64;
    static constexpr int PER_WARP = (W_OWN + OW * GROUP + 3) & ~3;
    static constexpr size_t bytes(int warps) { return sizeof(u32) * PER_WARP * warps; }
};

// One batch of 32 consecutive vertices (bi), counted by one warp in its slice of shared
// memory: the owners among them, in groups.
template <int SD, typename OffT, bool CG = false>
__device__ __forceinline__ void small_batch(u32* base, u64 bi, const u64* __restrict__ fo,
                                            const u32* __restrict__ head, u64 n,
                                            const Desc<OffT>* __restrict__ vdesc, const u32* __restrict__ headp,
                                            u32 sd, u64* __restrict__ cnt, u64& local_total, u32& dup) {
    using L = SmallWarpLayout<SD, OffT>;
    constexpr int OW = L::OW;
    static_assert(2 * SD <= L::TAB / 2, "two owners of the largest out-degree fit a group's tables");
    static_assert(SMALL_WARP_DEG <= (u32)L::QCAP, "one owner's adjacency fits the queue");
    static_assert(SD < 256 && L::NBIN <= 64, "list length is packed in 8 bits, bins two per lane");
    const int lane = threadIdx.x & 31;
    const u32 lt_mask = (1u << lane) - 1;
    u32* keys = base + L::W_KEYS;
    u32* hitc = base + L::W_HITS;
    u32* q_y = base + L::W_QY;
    OffT* q_s = reinterpret_cast<OffT*>(base + L::W_QS);
    u32* q_m = base + L::W_QM;
    unsigned short* q_ord = reinterpret_cast<unsigned short*>(base + L::W_ORD);
    u32* bins = base + L::W_BIN;
    // owner gi at own + OW * gi: [0] vertex, [1] (table offset << 5) | lg, [2] out-degree,
    // [3] key prefix, [4] adjacency prefix, [5] hit total, [6..7] first adjacency slot (u64),
    // [8..9] out-list start (u64)
    u32* own = base + L::W_OWN;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    const u64 v = bi * 32 + lane;
    Desc<OffT> dv;
    dv.start = 0;
    dv.d = 0;
    u64 a = 0;
    u32 deg = 0;
    bool is_owner = false;
    if (v < n) {
        dv = ld_desc<CG>(vdesc + v);
        a = ld_in<CG>(fo + v);
        const u64 b = ld_in<CG>(fo + v + 1);
        is_owner = dv.d > 0 && dv.d <= sd && b - a <= (u64)SMALL_WARP_DEG;
        deg = (u32)(b - a);
    }
    u32 lg = 0, tsz = 0;
    if (is_owner) {
        lg = ceil_log2(2 * dv.d);
        if (lg < 2) lg = 2;
        tsz = 1u << lg;
    }
    u32 todo = __ballot_sync(0xFFFFFFFFu, is_owner);
    while (todo) {
        // the group: the next owners in lane order while their tables and adjacency fit
        const bool cand = (todo >> lane) & 1u;
        u32 pk = cand ? (tsz << 16) | deg : 0u;  // inclusive prefix of (table slots, adjacency)
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xFFFFFFFFu, pk, o);
            if (lane >= o) pk += y;
        }
        const u32 rank = __popc(todo & lt_mask);
        const bool in = cand && (pk >> 16) <= (u32)L::TAB && (pk & 0xFFFFu) <= (u32)L::QCAP &&
                        rank < (u32)L::GROUP;
        const u32 gmask = __ballot_sync(0xFFFFFFFFu, in);
        todo &= ~gmask;
        const u32 G = __popc(gmask);
        const u32 last = 31 - __clz(gmask);  // the group's last member holds its totals
        const u32 tot_pk = __shfl_sync(0xFFFFFFFFu, pk, last);
        const u32 T = tot_pk >> 16, D = tot_pk & 0xFFFFu;
        u32 kk = in ? dv.d : 0u;  // inclusive prefix of the members' out-degrees
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(0xFFFFFFFFu, kk, o);
            if (lane >= o) kk += y;
        }
        const u32 K = __shfl_sync(0xFFFFFFFFu, kk, last);
        if (in) {
            const u32 gi = __popc(gmask & lt_mask);
            u32* o = own + OW * gi;
            const u64 ls = list_start(dv);
            o[0] = (u32)v;
            o[1] = (((pk >> 16) - tsz) << 5) | lg;
            o[2] = dv.d;
            o[3] = kk - dv.d;
            o[4] = (pk & 0xFFFFu) - deg;
            o[5] = 0;
            o[6] = (u32)a;
            o[7] = (u32)(a >> 32);
            o[8] = (u32)ls;
            o[9] = (u32)(ls >> 32);
        }
        for (u32 i = lane; i < T; i += 32) keys[i] = EMPTY_KEY;
        for (u32 i = lane; i < T / 2; i += 32) hitc[i] = 0;
        for (u32 i = lane; i < 64; i += 32) bins[i] = 0;
        __syncwarp();
        // member lane (< G) holds its key and adjacency prefixes: owners of items by start masks
        const u32 le_mask = lt_mask | (1u << lane);
        const bool mem = (u32)lane < G;
        const u32 kst = mem ? own[OW * lane + 3] : 0u, ast = mem ? own[OW * lane + 4] : 0u;
        // keys of every owner of the group
        for (u32 q0 = 0; q0 < K; q0 += 32) {
            const u32 before = __popc(__ballot_sync(0xFFFFFFFFu, mem && kst <= q0));
            const u32 starts = __reduce_or_sync(0xFFFFFFFFu, start_bit(mem, kst, q0));
            const u32 q = q0 + lane;
            if (q >= K) continue;
            const u32* o = own + OW * segment_of(before, starts, le_mask);
            const u64 xs = (u64)o[8] | ((u64)o[9] << 32);
            if (!bucket_insert(keys + (o[1] >> 5), o[1] & 31u, ld_in<CG>(headp + xs + (q - o[3])))) dup = 1;
        }
        // adjacency of every owner: queue the lower neighbours' lists (four slots in flight)
        u32 qn = 0;
        for (u32 e0 = 0; e0 < D; e0 += 128) {
            u32 yv[4], gv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const u32 eb = e0 + 32 * u;
                const u32 before = __popc(__ballot_sync(0xFFFFFFFFu, mem && ast <= eb));
                const u32 starts = __reduce_or_sync(0xFFFFFFFFu, start_bit(mem, ast, eb));
                const u32 e = eb + lane;
                yv[u] = NONE;
                gv[u] = 0;
                if (e < D) {
                    const u32 gi = segment_of(before, starts, le_mask);
                    const u64 xa = (u64)own[OW * gi + 6] | ((u64)own[OW * gi + 7] << 32);
                    gv[u] = gi;
                    yv[u] = ld_in<CG>(head + xa + (e - own[OW * gi + 4]));
                }
            }
            Desc<OffT> dyv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                dyv[u].start = 0;
                dyv[u].d = 0;
                if (yv[u] < n) dyv[u] = ld_desc<CG>(vdesc + yv[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const u32 gi = gv[u], dy = dyv[u].d;
                const bool sel = yv[u] < n && dy > 0 && key_less(dy, yv[u], own[OW * gi + 2], own[OW * gi]);
                const u32 ball = __ballot_sync(0xFFFFFFFFu, sel);
                if (sel) {
                    const u32 qi = qn + __popc(ball & lt_mask);
                    q_y[qi] = yv[u];
                    q_s[qi] = (OffT)list_group(dyv[u]);
                    q_m[qi] = (gi << 8) | dy;
                    atomicAdd(&bins[dy], 1u);
                }
                qn += __popc(ball);
            }
        }
        __syncwarp();
        // counting sort of the queue by list length (bins 2 lane and 2 lane + 1 in each lane)
        {
            const u32 c0 = bins[2 * lane], c1 = bins[2 * lane + 1];
            u32 x = c0 + c1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const u32 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            bins[2 * lane] = x - c0 - c1;
            bins[2 * lane + 1] = x - c1;
        }
        __syncwarp();
        for (u32 qi = lane; qi < qn; qi += 32) q_ord[atomicAdd(&bins[q_m[qi] & 0xFFu], 1u)] = (unsigned short)qi;
        __syncwarp();
        // stream the queued lists, one per lane, longest first
        for (u32 r = lane; r < qn; r += 32) {
            const u32 qi = q_ord[qn - 1 - r];
            const u32 meta = q_m[qi];
            const u32 gi = meta >> 8, dy = meta & 0xFFu;
            const u32 tb = own[OW * gi + 1];
            const u32* tk = keys + (tb >> 5);
            u32* th = hitc + ((tb >> 5) >> 1);  // table offsets are multiples of 4 slots
            const u32 tl = tb & 31u;
            const u64 q0 = (u64)q_s[qi];
            u32 hits = 0;
            // one 16-byte group of the list per iteration (groups are padded, so the load stays
            // inside the list's slots): four groups per iteration, loaded together, measured
            // slower, the loop body then holding sixteen inlined probes
            for (u32 g0 = 0; 4 * g0 < dy; ++g0) {
                const uint4 qv = ld_in<CG>(headp4 + q0 + g0);
                const u32 e = 4 * g0;
                hits += bucket_probe16(tk, th, tl, qv.x);
                if (e + 1 < dy) hits += bucket_probe16(tk, th, tl, qv.y);
                if (e + 2 < dy) hits += bucket_probe16(tk, th, tl, qv.z);
                if (e + 3 < dy) hits += bucket_probe16(tk, th, tl, qv.w);
            }
            if (hits) {
                atomicAdd(&cnt[q_y[qi]], (u64)hits);
                atomicAdd(&own[OW * gi + 5], hits);
            }
        }
        __syncwarp();
        // flush: every key's hits, then the owners' totals
        for (u32 i = lane; i < T; i += 32) {
            const u32 h = read16(hitc, i);
            if (h) atomicAdd(&cnt[keys[i]], (u64)h);
        }
        if ((u32)lane < G) {
            const u32 t = own[OW * lane + 5];
            if (t) {
                atomicAdd(&cnt[own[OW * lane]], (u64)t);
                local_total += t;
            }
        }
        __syncwarp();  // the next group reuses the slice only after every lane has flushed
    }
}

template <int BLOCK, int SD, typename OffT>
__global__ void __launch_bounds__(BLOCK, 4) k_count_small(const u64* __restrict__ fo, const u32* __restrict__ head,
                                                          u64 n, const Desc<OffT>* __restrict__ vdesc,
                                                          const u32* __restrict__ headp, u32 sd,
                                                          u64* __restrict__ cnt, u64* __restrict__ partials,
                                                          Control* ctl) {
    using L = SmallWarpLayout<SD, OffT>;
    constexpr int NW = BLOCK / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ u64 s_red[NW];
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32* base = reinterpret_cast<u32*>(smem) + warp * L::PER_WARP;
    const u64 nbatch = (n + 31) / 32;
    u64 local_total = 0;
    u32 dup = 0;
    while (true) {
        unsigned long long bi = 0;
        if (lane == 0) bi = atomicAdd(&ctl->small_next, 1ull);
        bi = __shfl_sync(0xFFFFFFFFu, bi, 0);
        if (bi >= nbatch) break;
        small_batch<SD, OffT>(base, bi, fo, head, n, vdesc, headp, sd, cnt, local_total, dup);
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
    // block scalars: reduction slots, queue length and cursor, the bulk copy's mbarrier
    static constexpr size_t off_red = align16(off_qd + sizeof(Desc<OffT>) * LARGE_SEG);
    static constexpr size_t off_qn = off_red + sizeof(u64) * (BLOCK / 32);
    static constexpr size_t off_next = off_qn + sizeof(u32);
    static constexpr size_t off_bar = align16(off_next + sizeof(u32));
    static constexpr size_t bytes = align16(off_bar + sizeof(unsigned long long));
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
template <int U, bool CG = false>
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
        for (int u = 0; u < U; ++u) w[u] = rem > 32 * u ? ld_in<CG>(lp + 32 * u) : EMPTY_KEY;
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
template <typename OffT, bool CG = false>
__device__ __forceinline__ u32 lane_stream_short(const uint4* __restrict__ headp4, const Desc<OffT>& vy,
                                                 const u32* keys, u32* hitc, u32 lg, const u32* filt, u32 fl) {
    const u32 dy = vy.d;
    const u64 q0 = list_group(vy);
    uint4 qv[LONG_LIST / 4];
#pragma unroll
    for (int c = 0; c < LONG_LIST / 4; ++c)
        qv[c] = 4 * c < (int)dy ? ld_in<CG>(headp4 + q0 + c) : make_uint4(EMPTY_KEY, EMPTY_KEY, EMPTY_KEY, EMPTY_KEY);
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

// One (owner, segment) tile of a large owner, counted by the whole block.  bar is the block's
// bulk-copy mbarrier, initialised once and kept where no other use of shared memory reaches.
// Returns true when a bounded wait for a bulk copy ran out (inflight: the second wait ran out too).
template <int BLOCK, int CAP, typename OffT, bool CG = false>
__device__ __forceinline__ bool large_tile(unsigned char* smem, unsigned long long* bar, uint2 tl,
                                           const u64* __restrict__ fo,
                                           const u32* __restrict__ head, u64 n, const Desc<OffT>* __restrict__ vdesc,
                                           const u32* __restrict__ headp, u32 seg, u64* __restrict__ cnt,
                                           u32 first_wait_polls, u32& phase, bool& inflight, u64& local_total,
                                           u32& dup) {
    using L = LargeLayout<BLOCK, CAP, OffT>;
    constexpr int NW = BLOCK / 32;
    constexpr int U = 8;  // loads in flight per lane and list
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 lt_mask = (1u << lane) - 1;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    u32* keys = reinterpret_cast<u32*>(smem + L::off_keys);
    u32* hitc = reinterpret_cast<u32*>(smem + L::off_hits);
    u32* filt = reinterpret_cast<u32*>(smem + L::off_filt);
    u32* qy = reinterpret_cast<u32*>(smem + L::off_qy);
    Desc<OffT>* qd = reinterpret_cast<Desc<OffT>*>(smem + L::off_qd);
    // the owner's keys are staged in the queue's descriptor region, which is free until the scan
    u32* stage = reinterpret_cast<u32*>(smem + L::off_qd);
    static_assert(sizeof(Desc<OffT>) * LARGE_SEG >= sizeof(u32) * CAP, "staging fits the queue region");
    u32* wbuf = reinterpret_cast<u32*>(smem + L::off_wbuf) + warp * L::WBUF;
    u64* s_red = reinterpret_cast<u64*>(smem + L::off_red);
    u32& s_qn = *reinterpret_cast<u32*>(smem + L::off_qn);
    u32& s_next = *reinterpret_cast<u32*>(smem + L::off_next);
    unsigned long long& s_bar = *bar;  // the block's bulk-copy barrier (its phase persists across tiles)
    bool timed_out = false;
    const u64 x = tl.x;
    const Desc<OffT> dxd = ld_desc<CG>(vdesc + x);
    const u32 dx = dxd.d;
    const u64 fx1 = ld_in<CG>(fo + x + 1);
    const u64 a = ld_in<CG>(fo + x) + (u64)tl.y * seg;
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
            if (!__syncthreads_or(!mbar_wait_bounded(&s_bar, phase, COPY_WAIT_POLLS))) {
                timed_out = true;
                phase ^= 1u;  // the copy landed: the barrier's phase completed (a block that goes on
                              // taking tiles, as the engine's do, waits on the next one)
            } else {
                timed_out = inflight = true;
            }
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
                y = ld_in<CG>(head + e);
                if (y < n) vy = ld_desc<CG>(vdesc + y);
                const u32 dy = vy.d;
                if (dy > 0 && key_less(dy, y, dx, x)) {
                    if (dy <= (u32)LONG_LIST) {
                        const u32 hits = lane_stream_short<OffT, CG>(headp4, vy, keys, hitc, lg, filt, fl);
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
            u32 hits = warp_stream_list<U, CG>(headp + list_start(vy), vy.d, keys, hitc, lg, filt, fl, wbuf, lane,
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
    return timed_out;
}

template <int BLOCK, int CAP, typename OffT>
__global__ void __launch_bounds__(BLOCK) k_count_large(const u64* __restrict__ fo, const u32* __restrict__ head,
                                                       u64 n, const Desc<OffT>* __restrict__ vdesc,
                                                       const u32* __restrict__ headp,
                                                       const uint2* __restrict__ ltiles, u32 seg,
                                                       u64* __restrict__ cnt, u64* __restrict__ partials,
                                                       Control* ctl, u32 first_wait_polls) {
    using L = LargeLayout<BLOCK, CAP, OffT>;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ u64 s_t;
    unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(smem + L::off_bar);  // the bulk copy's barrier

    if (ctl->err & DEV_ERR_MASK) return;
    if (threadIdx.x == 0) mbar_init(s_bar, 1);
    fence_proxy_async_smem();
    __syncthreads();
    u32 phase = 0;
    bool timed_out = false, inflight = false;
    const u64 ntiles = *(volatile unsigned long long*)&ctl->large_tiles;
    u64 local_total = 0;
    u32 dup = 0;
    while (true) {
        if (threadIdx.x == 0) s_t = atomicAdd(&ctl->large_next, 1ull);
        __syncthreads();
        const u64 t = s_t;
        if (t >= ntiles) break;
        timed_out = large_tile<BLOCK, CAP, OffT>(smem, s_bar, ltiles[t], fo, head, n, vdesc, headp, seg, cnt,
                                                 first_wait_polls, phase, inflight, local_total, dup);
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

// One (owner, segment) tile of a medium owner, counted by one warp in its slice of shared
// memory (keys at `keys`, then the hit counters, the filter and the survivor buffer).
template <int BLOCK, typename OffT, bool CG = false>
__device__ __forceinline__ void medium_tile(u32* keys, uint2 tl, const u64* __restrict__ fo,
                                            const u32* __restrict__ head, const Desc<OffT>* __restrict__ vdesc,
                                            const u32* __restrict__ headp, u32 seg, u64* __restrict__ cnt,
                                            u64& local_total, u32& dup) {
    using L = MediumLayout<BLOCK>;
    constexpr int U = 4;  // medium owners' streamed lists are shorter than 256 entries
    const int lane = threadIdx.x & 31;
    u32* hitc = keys + L::TS;
    u32* filt = hitc + L::TS / 2;
    u32* wbuf = filt + L::FW;
    const u32 lt_mask = (1u << lane) - 1;
    const uint4* headp4 = reinterpret_cast<const uint4*>(headp);
    const u64 x = tl.x;
    const Desc<OffT> dxd = ld_desc<CG>(vdesc + x);
    const u32 dx = dxd.d;
    const u64 fx1 = ld_in<CG>(fo + x + 1);
    const u64 a = ld_in<CG>(fo + x) + (u64)tl.y * seg;
    const u64 b = a + seg < fx1 ? a + seg : fx1;
    u32 lg, fl;
    chunk_sizes(dx, 31 - __clz((u32)L::TS), 31 - __clz((u32)(L::FW * 32)), &lg, &fl);
    const u32 size = 1u << lg, fwords = (1u << fl) >> 5;
    for (u32 i = lane; i < size; i += 32) keys[i] = EMPTY_KEY;
    for (u32 i = lane; i < size / 2; i += 32) hitc[i] = 0;
    for (u32 i = lane; i < fwords; i += 32) filt[i] = 0;
    __syncwarp();
    for (u32 q = lane; q < dx; q += 32) {
        const u32 w = ld_in<CG>(headp + list_start(dxd) + q);
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
            y = ld_in<CG>(head + e);
            vy = ld_desc<CG>(vdesc + y);
            const u32 dy = vy.d;
            if (dy > 0 && key_less(dy, y, dx, x)) {
                if (dy <= (u32)LONG_LIST) {
                    const u32 hits = lane_stream_short<OffT, CG>(headp4, vy, keys, hitc, lg, filt, fl);
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
            u32 hits = warp_stream_list<U, CG>(headp + ys, yd, keys, hitc, lg, filt, fl, wbuf, lane, lt_mask);
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

template <int BLOCK, typename OffT>
__global__ void __launch_bounds__(BLOCK)
    k_count_medium(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                   const Desc<OffT>* __restrict__ vdesc, const u32* __restrict__ headp,
                   const uint2* __restrict__ mtiles, u32 seg, u64* __restrict__ cnt,
                   u64* __restrict__ partials, Control* ctl) {
    using L = MediumLayout<BLOCK>;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ u64 s_red[L::NW];
    (void)n;
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32* keys = reinterpret_cast<u32*>(smem) + warp * L::PER_WARP;
    const u64 ntiles = *(volatile unsigned long long*)&ctl->medium_tiles;
    u64 local_total = 0;
    u32 dup = 0;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(&ctl->medium_next, 1ull);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        if (t >= ntiles) break;
        medium_tile<BLOCK, OffT>(keys, mtiles[t], fo, head, vdesc, headp, seg, cnt, local_total, dup);
    }
    if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
    const u64 bt = block_sum_u64<BLOCK>(local_total, s_red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bt;
}

// Sum of the per-block partial totals (a u64 tree reduction in one block), without the slots
// [skip0, skip1) of blocks that were not launched.  After a device error (invalid input, a
// bounded wait that ran out) the partials are incomplete or stale, so the total is written as 0.
__global__ void __launch_bounds__(1024) k_final(const u64* __restrict__ partials, u32 np, u32 skip0, u32 skip1,
                                                u64* total, const Control* ctl) {
    __shared__ u64 s_red[32];
    if (*(volatile const u32*)&ctl->err & DEV_ERR_MASK) {
        if (threadIdx.x == 0) *total = 0;
        return;
    }
    u64 s = 0;
    for (u32 i = threadIdx.x; i < np; i += 1024)
        if (i < skip0 || i >= skip1) s += partials[i];
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

// ---- the serving engine ----------------------------------------------------------------

constexpr int ENGINE_SD = SMALL_D;  // the small-owner layout for any small_outdegree bound
using EngineSmallL = SmallWarpLayout<ENGINE_SD, u32>;
using EngineMediumL = MediumLayout<ENGINE_BLOCK>;
using EngineLargeL = LargeLayout<ENGINE_BLOCK, LARGE_CAP, u32>;
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t ENGINE_SMEM =
    cmax(cmax(EngineSmallL::bytes(ENGINE_BLOCK / 32), EngineMediumL::bytes), EngineLargeL::bytes);
static_assert(SMALL_BLOCK == ENGINE_BLOCK && MEDIUM_BLOCK == ENGINE_BLOCK && LARGE_BLOCK == ENGINE_BLOCK,
              "the engine runs every kind of unit with one block shape");

// The claim cursor of a job holds the publication's tag (low 24 bits of its sequence number) in
// its top 24 bits and the next unit in its low 40 bits.  Units are claimed by compare-and-swap
// against a cursor whose tag matches the sequence number read before and after it, so a block
// can never take a unit of a later publication of the same slot, nor read a half-written record.
constexpr int ENGINE_TAG_SHIFT = 40;
constexpr unsigned long long ENGINE_COUNT_MASK = (1ull << ENGINE_TAG_SHIFT) - 1;
__device__ __forceinline__ unsigned long long engine_tag(unsigned long long seq) { return seq & 0xFFFFFFull; }

__global__ void k_publish(EngineJob* job, unsigned long long seq, const u64* fo, const u32* head, u64 n,
                          const void* vdesc, const u32* headp, const uint2* mtiles, const uint2* ltiles, u64* cnt,
                          Control* ctl, u32 small_d, u32 seg, unsigned long long* done_word) {
    if (threadIdx.x != 0) return;
    volatile EngineJob* vj = job;
    vj->seq = 0;  // unpublished while the record changes
    __threadfence();
    const bool bad = (*(volatile u32*)&ctl->err & DEV_ERR_MASK) != 0;
    const unsigned long long nbatch = (n + 31) / 32;
    const unsigned long long us = bad ? 0 : (nbatch + ENGINE_UNIT_ITEMS - 1) / ENGINE_UNIT_ITEMS;
    const unsigned long long um =
        bad ? 0 : (*(volatile unsigned long long*)&ctl->medium_tiles + ENGINE_UNIT_ITEMS - 1) / ENGINE_UNIT_ITEMS;
    const unsigned long long ul = bad ? 0 : *(volatile unsigned long long*)&ctl->large_tiles;
    if (us + um + ul == 0) {  // nothing for the engine: done at once
        __threadfence_system();
        *(volatile unsigned long long*)done_word = seq;
        return;
    }
    vj->fo = fo;
    vj->head = head;
    vj->n = n;
    vj->vdesc = vdesc;
    vj->headp = headp;
    vj->mtiles = mtiles;
    vj->ltiles = ltiles;
    vj->cnt = cnt;
    vj->ctl = ctl;
    vj->small_d = small_d;
    vj->seg = seg;
    vj->units_small = us;
    vj->units_medium = um;
    vj->units = us + um + ul;
    vj->done = 0;
    __threadfence();
    vj->next = engine_tag(seq) << ENGINE_TAG_SHIFT;
    __threadfence();
    vj->seq = seq;
}

__global__ void __launch_bounds__(ENGINE_BLOCK, 4) k_engine(EngineJob* jobs, u32 njobs, unsigned long long* done_words,
                                                         unsigned* stop, u32 idle_polls) {
    constexpr int BLOCK = ENGINE_BLOCK;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_job;
    __shared__ unsigned long long s_unit;
    __shared__ EngineJob s_jb;  // the claimed job's record, read at L2 by thread 0
    __shared__ u32 s_jb_slot;
    __shared__ unsigned s_stop;
    __shared__ int s_work;  // some published job was unfinished in the last scan
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    (void)lane;
    // the large-owner tiles' bulk-copy barrier: outside the dynamic region, which the small- and
    // medium-owner units overwrite between large tiles, since its phase persists across units
    __shared__ __align__(8) unsigned long long s_bar_engine;
    unsigned long long* s_bar = &s_bar_engine;
    if (threadIdx.x == 0) {
        mbar_init(s_bar, 1);
        s_jb.seq = 0;
        s_jb_slot = 0xFFFFFFFFu;
    }
    fence_proxy_async_smem();
    __syncthreads();
    u32 phase = 0;
    bool inflight = false;
    u32 idle = 0, start = blockIdx.x % (njobs ? njobs : 1);
    while (true) {
        if (threadIdx.x == 0) {
            s_job = -1;
            s_work = 0;
            // a launch leaves as a whole: once any block has set the stop word (or the host has),
            // no block claims another unit
            s_stop = *(volatile const unsigned*)stop;
            for (u32 k = 0; k < njobs && s_job < 0 && !s_stop; ++k) {
                const u32 j = (start + k) % njobs;
                volatile EngineJob* vj = jobs + j;
                for (int attempt = 0; attempt < 4; ++attempt) {
                    const unsigned long long s1 = vj->seq;
                    if (s1 == 0) break;
                    s_work = 1;  // a published job is not finished
                    __threadfence();
                    const unsigned long long cur = vj->next;
                    const unsigned long long units = vj->units;
                    __threadfence();
                    if (vj->seq != s1 || (cur >> ENGINE_TAG_SHIFT) != engine_tag(s1)) break;
                    if ((cur & ENGINE_COUNT_MASK) >= units) break;
                    if (atomicCAS(const_cast<unsigned long long*>(&vj->next), cur, cur + 1) != cur) continue;
                    // unit (cur & mask) of publication s1: its record stays as it is until the job
                    // is done, which needs this unit
                    s_job = (int)j;
                    s_unit = cur & ENGINE_COUNT_MASK;
                    start = j + 1;  // the next scan begins at the following job: no job is favoured
                    if (s_jb.seq == s1 && s_jb_slot == j) break;  // this block holds the record already
                    s_jb_slot = j;
                    s_jb.fo = vj->fo;
                    s_jb.head = vj->head;
                    s_jb.n = vj->n;
                    s_jb.vdesc = vj->vdesc;
                    s_jb.headp = vj->headp;
                    s_jb.mtiles = vj->mtiles;
                    s_jb.ltiles = vj->ltiles;
                    s_jb.cnt = vj->cnt;
                    s_jb.ctl = vj->ctl;
                    s_jb.small_d = vj->small_d;
                    s_jb.seg = vj->seg;
                    s_jb.units_small = vj->units_small;
                    s_jb.units_medium = vj->units_medium;
                    s_jb.units = units;
                    s_jb.seq = s1;
                    break;
                }
            }
        }
        __syncthreads();
        const int j = s_job;
        if (j < 0) {
            // Only scans that found every published job finished count towards leaving: while a
            // job's last units run on other blocks, this block stays for the jobs published next.
            // The first block to leave sets the stop word, and the others follow at their next
            // scan: a launch that shrank to a few blocks would serve a job published meanwhile at
            // a trickle, and the host relaunches the engine only once the launch has ended.
            if (s_work) idle = 0;
            if (s_stop) break;  // the same decision in every thread
            if (++idle > idle_polls) {
                if (threadIdx.x == 0) {
                    *(volatile unsigned*)stop = 1u;
                    __threadfence();
                }
                break;
            }
            __nanosleep(2000);
            __syncthreads();  // every thread has read s_job before thread 0 writes it again
            continue;
        }
        idle = 0;
        const EngineJob* jb = &s_jb;
        const unsigned long long u = s_unit;
        Control* ctl = jb->ctl;
        const auto* vd = reinterpret_cast<const Desc<u32>*>(jb->vdesc);
        u64 unused_total = 0;
        u32 dup = 0;
        bool timed_out = false;
        if (u < jb->units_small) {
            const u64 nb = (jb->n + 31) / 32;
            for (u32 r = 0; r < ENGINE_REPS; ++r) {
                const u64 bi = (u * (ENGINE_BLOCK / 32) + warp) * ENGINE_REPS + r;
                if (bi < nb)
                    small_batch<ENGINE_SD, u32, true>(reinterpret_cast<u32*>(smem) + warp * EngineSmallL::PER_WARP, bi,
                                                      jb->fo, jb->head, jb->n, vd, jb->headp, jb->small_d, jb->cnt,
                                                      unused_total, dup);
            }
        } else if (u < jb->units_small + jb->units_medium) {
            const u64 nt = *(volatile unsigned long long*)&ctl->medium_tiles;
            for (u32 r = 0; r < ENGINE_REPS; ++r) {
                const u64 t = ((u - jb->units_small) * (ENGINE_BLOCK / 32) + warp) * ENGINE_REPS + r;
                if (t < nt)
                    medium_tile<BLOCK, u32, true>(reinterpret_cast<u32*>(smem) + warp * EngineMediumL::PER_WARP,
                                                  __ldcg(jb->mtiles + t), jb->fo, jb->head, vd, jb->headp, jb->seg,
                                                  jb->cnt, unused_total, dup);
            }
        } else {
            const u64 t = u - jb->units_small - jb->units_medium;
            timed_out = large_tile<BLOCK, LARGE_CAP, u32, true>(smem, s_bar, __ldcg(jb->ltiles + t), jb->fo, jb->head,
                                                                jb->n, vd, jb->headp,
                                                          jb->seg, jb->cnt, COPY_WAIT_POLLS, phase, inflight,
                                                          unused_total, dup);
        }
        if (dup) atomicOr(&ctl->err, DEV_ERR_DUPLICATE);
        if (timed_out && threadIdx.x == 0)
            atomicOr(&ctl->err, DEV_ERR_TIMEOUT | (inflight ? DEV_ERR_COPY_INFLIGHT : 0u));
        __syncthreads();  // the unit's counts are all issued
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned long long d = atomicAdd(&jobs[j].done, 1ull) + 1;
            if (d == jb->units) {
                *(volatile unsigned long long*)&jobs[j].seq = 0;
                __threadfence_system();
                *(volatile unsigned long long*)(done_words + j) = jb->seq;
            }
        }
        // a copy that may still be landing in shared memory: this block stops taking units
        if (inflight) break;
    }
}

void launch_publish(EngineJob* job, unsigned long long seq, const u64* fo, const u32* head, u64 n,
                    const void* vdesc, const u32* headp, const uint2* mtiles, const uint2* ltiles, u64* cnt,
                    Control* ctl, u32 small_d, u32 seg, unsigned long long* done_word, cudaStream_t st) {
    k_publish<<<1, 32, 0, st>>>(job, seq, fo, head, n, vdesc, headp, mtiles, ltiles, cnt, ctl, small_d, seg, done_word);
}

size_t engine_smem_bytes() { return ENGINE_SMEM; }

int engine_grid(int num_sms) {
    static int occ = -1;
    if (occ < 0) {
        cudaFuncSetAttribute(k_engine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENGINE_SMEM);
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_engine, ENGINE_BLOCK, ENGINE_SMEM);
        occ = o > 0 ? o : 1;
    }
    // leave room on every SM for the preparation kernels of the batches being published: the
    // engine's blocks stay resident while any published job is unfinished, so with one block
    // slot per SM left the next batches' orientation starved (6.4K against 0.6-2.5K graphs/s at
    // saturation with two slots left against one)
    return num_sms * (occ > 2 ? occ - 2 : 1);
}

void launch_engine(EngineJob* jobs, u32 njobs, unsigned long long* done_words, unsigned* stop, u32 idle_polls,
                   int grid, cudaStream_t st) {
    k_engine<<<grid, ENGINE_BLOCK, ENGINE_SMEM, st>>>(jobs, njobs, done_words, stop, idle_polls);
}

// ---- launchers ------------------------------------------------------------------------

namespace {
template <typename OffT>
using LargeL = LargeLayout<LARGE_BLOCK, LARGE_CAP, OffT>;
using MediumL = MediumLayout<MEDIUM_BLOCK>;

template <int SD, typename OffT>
int occupancy_small() {
    static int occ = -1;
    if (occ < 0) {
        auto kern = k_count_small<SMALL_BLOCK, SD, OffT>;
        const size_t bytes = SmallWarpLayout<SD, OffT>::bytes(SMALL_BLOCK / 32);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        int o = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, SMALL_BLOCK, bytes);
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
int count_grid_small(int num_sms, u32 small_d) {
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
// Blocks the small-owner kernel is launched with: enough for one vertex batch per warp, at most
// its resident grid (a small graph does not start hundreds of warps that find no batch).
int small_grid_launched(u64 n, int cap) {
    const u64 need = ((n + 31) / 32 + SMALL_BLOCK / 32 - 1) / (SMALL_BLOCK / 32);
    return (int)(need < 1 ? 1 : (need < (u64)cap ? need : (u64)cap));
}

template <typename OffT>
int count_grid_auto(int num_sms, u32 small_d) {
    return count_grid_small<OffT>(num_sms, small_d) + count_grid_medium<OffT>(num_sms) +
           count_grid_large<OffT>(num_sms);
}

template <typename OffT>
cudaError_t launch_count_auto(const u64* fo, const u32* head, u64 n, u64 nnz, const void* vdesc, const u32* headp,
                              const uint2* mtiles, const uint2* ltiles, u32 small_d, u32 seg, u64* cnt, u64* partials,
                              Control* ctl, int num_sms, cudaStream_t st, cudaEvent_t after_small,
                              cudaEvent_t after_large, u32 copy_wait_polls) {
    (void)nnz;
    const int cap = count_grid_small<OffT>(num_sms, small_d);
    const int gs = small_grid_launched(n, cap);
    const int gm = count_grid_medium<OffT>(num_sms);
    const int gl = count_grid_large<OffT>(num_sms);
    const auto* vd = reinterpret_cast<const Desc<OffT>*>(vdesc);
    if (small_d <= (u32)SMALL_D_LOW)
        k_count_small<SMALL_BLOCK, SMALL_D_LOW, OffT>
            <<<gs, SMALL_BLOCK, SmallWarpLayout<SMALL_D_LOW, OffT>::bytes(SMALL_BLOCK / 32), st>>>(
                fo, head, n, vd, headp, small_d, cnt, partials, ctl);
    else
        k_count_small<SMALL_BLOCK, SMALL_D, OffT>
            <<<gs, SMALL_BLOCK, SmallWarpLayout<SMALL_D, OffT>::bytes(SMALL_BLOCK / 32), st>>>(
                fo, head, n, vd, headp, small_d, cnt, partials, ctl);
    if (after_small) cudaEventRecord(after_small, st);
    k_count_medium<MEDIUM_BLOCK, OffT>
        <<<gm, MEDIUM_BLOCK, MediumL::bytes, st>>>(fo, head, n, vd, headp, mtiles, seg, cnt, partials + cap, ctl);
    k_count_large<LARGE_BLOCK, LARGE_CAP, OffT>
        <<<gl, LARGE_BLOCK, LargeL<OffT>::bytes, st>>>(fo, head, n, vd, headp, ltiles, seg, cnt, partials + cap + gm,
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
    k_final<<<1, 1024, 0, st>>>(partials, np, 0, 0, total, ctl);
}

template <typename OffT>
void launch_final_auto(const u64* partials, u64 n, u32 small_d, int num_sms, u64* total, Control* ctl,
                       cudaStream_t st) {
    const int cap = count_grid_small<OffT>(num_sms, small_d);
    k_final<<<1, 1024, 0, st>>>(partials, (u32)count_grid_auto<OffT>(num_sms, small_d), (u32)small_grid_launched(n, cap),
                                (u32)cap, total, ctl);
}

template <typename OffT>
void launch_stats(const u64* fo, const u32* head, u64 n, const void* vdesc, const u32* headp, u32 medium_d,
                  Control* ctl, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    k_stats<OffT><<<num_sms * 8, 256, 0, st>>>(fo, head, n, reinterpret_cast<const Desc<OffT>*>(vdesc), headp,
                                               medium_d, ctl);
}

template void launch_final_auto<u32>(const u64*, u64, u32, int, u64*, Control*, cudaStream_t);
template void launch_final_auto<u64>(const u64*, u64, u32, int, u64*, Control*, cudaStream_t);
template int count_grid_small<u32>(int, u32);
template int count_grid_small<u64>(int, u32);
template int count_grid_large<u32>(int);
template int count_grid_large<u64>(int);
template int count_grid_medium<u32>(int);
template int count_grid_medium<u64>(int);
template int count_grid_auto<u32>(int, u32);
template int count_grid_auto<u64>(int, u32);
template cudaError_t launch_count_auto<u32>(const u64*, const u32*, u64, u64, const void*, const u32*, const uint2*,
                                            const uint2*, u32, u32, u64*, u64*, Control*, int, cudaStream_t,
                                            cudaEvent_t, cudaEvent_t, u32);
template cudaError_t launch_count_auto<u64>(const u64*, const u32*, u64, u64, const void*, const u32*, const uint2*,
                                            const uint2*, u32, u32, u64*, u64*, Control*, int, cudaStream_t,
                                            cudaEvent_t, cudaEvent_t, u32);
template void launch_stats<u32>(const u64*, const u32*, u64, const void*, const u32*, u32, Control*, int,
                                cudaStream_t);
template void launch_stats<u64>(const u64*, const u32*, u64, const void*, const u32*, u32, Control*, int,
                                cudaStream_t);

}  // namespace ktri
