// Sorted-list strategies: the reference's own intersection methods on the device.
//
//   sort_neighborhoods (distributed_graph.h:578-593): every out-list is sorted by id.  A warp
//     sorts lists of up to 32 entries in registers, a block sorts lists of up to SORT_SMEM
//     entries in shared memory, and longer lists are sorted by a block in global scratch
//     (bitonic networks throughout).  Lists found already sorted are left alone.
//   run_local (cetric_edge_iterator.h:889-1066 / :230-298) with intersection()
//     (intersection.h:41-79): one warp per tail vertex v walks its oriented edges (v,u) and
//     intersects N+(v) with N+(u):
//       merge         (intersection.h:82-96)  chunked warp merge: 32-entry chunks of both
//                     lists, shuffle binary search inside the chunk, advance the chunk with
//                     the smaller last entry;
//       binary-search (intersection.h:99-117) lanes take entries of the shorter list and
//                     binary-search the longer one;
//       binary        (intersection.h:120-192) the divide-and-conquer with an explicit task
//                     stack and a merge below the cutoff, one lane per oriented edge;
//       hybrid        (intersection.h:66-77) binary search when |S| * floor(log2 |L|) <
//                     scale * (|S| + |L|), else merge.
// Per-vertex counts: each hit w of edge (v,u) adds one to w; u gets the edge's hit count and
// v the sum over its edges.
#include "ktri_device.cuh"
#include "ktri_kernels.h"

namespace ktri {

constexpr int SORT_SMEM = 8192;
constexpr int SORT_BLOCK = 512;
constexpr int BIN_STACK = 96;

// ---- sorting ----------------------------------------------------------------------------

template <typename OffT>
__global__ void k_sort_warp(u64 n, const Desc<OffT>* __restrict__ vdesc, u32* __restrict__ headp, u32* mid_list,
                            u32* big_list, Control* ctl) {
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31;
    const u64 gw = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = gw; v < n; v += nwarps) {
        const Desc<OffT> d = load_desc(vdesc + v);
        if (d.d <= 1) continue;
        if (d.d > 32) {
            if (lane == 0) {
                if (d.d <= (u32)SORT_SMEM) mid_list[atomicAdd(&ctl->sort_mid, 1ull)] = (u32)v;
                else big_list[atomicAdd(&ctl->sort_big, 1ull)] = (u32)v;
            }
            continue;
        }
        u32* p = headp + list_start(d);
        u32 x = lane < (int)d.d ? p[lane] : EMPTY_KEY;
        const u32 nx = __shfl_down_sync(0xFFFFFFFFu, x, 1);
        const bool bad = lane + 1 < (int)d.d && nx < x;
        if (!__any_sync(0xFFFFFFFFu, bad)) continue;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const u32 o = __shfl_xor_sync(0xFFFFFFFFu, x, j);
                const bool asc = (lane & k) == 0;
                const bool lower = (lane & j) == 0;
                x = (lower == asc) ? min(x, o) : max(x, o);
            }
        }
        if (lane < (int)d.d) p[lane] = x;
    }
}

template <int BLOCK>
__device__ void bitonic_block(u32* s, u32 P) {
    for (u32 k = 2; k <= P; k <<= 1) {
        for (u32 j = k >> 1; j > 0; j >>= 1) {
            for (u32 i = threadIdx.x; i < P; i += BLOCK) {
                const u32 ixj = i ^ j;
                if (ixj > i) {
                    const u32 a = s[i], b = s[ixj];
                    const bool asc = (i & k) == 0;
                    if ((a > b) == asc) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

template <typename OffT>
__global__ void __launch_bounds__(SORT_BLOCK) k_sort_block(const Desc<OffT>* __restrict__ vdesc, u32* headp,
                                                           const u32* mid_list, Control* ctl) {
    __shared__ u32 s[SORT_SMEM];
    __shared__ int s_bad;
    const u64 cnt = *(volatile unsigned long long*)&ctl->sort_mid;
    for (u64 i = blockIdx.x; i < cnt; i += gridDim.x) {
        const Desc<OffT> d = load_desc(vdesc + mid_list[i]);
        u32* p = headp + list_start(d);
        u32 P = 1;
        while (P < d.d) P <<= 1;
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        for (u32 k = threadIdx.x; k < P; k += SORT_BLOCK) {
            s[k] = k < d.d ? p[k] : EMPTY_KEY;
            if (k + 1 < d.d && p[k + 1] < p[k]) s_bad = 1;
        }
        __syncthreads();
        if (s_bad) {
            bitonic_block<SORT_BLOCK>(s, P);
            for (u32 k = threadIdx.x; k < d.d; k += SORT_BLOCK) p[k] = s[k];
        }
        __syncthreads();
    }
}

template <typename OffT>
__global__ void __launch_bounds__(SORT_BLOCK) k_sort_global(const Desc<OffT>* __restrict__ vdesc, u32* headp,
                                                            const u32* big_list, u32* scratch, u64 scratch_per_block,
                                                            Control* ctl) {
    const u64 cnt = *(volatile unsigned long long*)&ctl->sort_big;
    u32* s = scratch + (u64)blockIdx.x * scratch_per_block;
    for (u64 i = blockIdx.x; i < cnt; i += gridDim.x) {
        const Desc<OffT> d = load_desc(vdesc + big_list[i]);
        u32* p = headp + list_start(d);
        u32 P = 1;
        while (P < d.d) P <<= 1;
        if (P > scratch_per_block) {  // cannot happen: out-degree <= sqrt(nnz)
            if (threadIdx.x == 0) atomicOr(&ctl->err, DEV_ERR_DEGREE);
            continue;
        }
        for (u32 k = threadIdx.x; k < P; k += SORT_BLOCK) s[k] = k < d.d ? p[k] : EMPTY_KEY;
        __syncthreads();
        bitonic_block<SORT_BLOCK>(s, P);
        for (u32 k = threadIdx.x; k < d.d; k += SORT_BLOCK) p[k] = s[k];
        __syncthreads();
    }
}

// ---- warp-level intersections of sorted lists ------------------------------------------

// Lower bound of key in a sorted global list.
__device__ __forceinline__ u32 lower_bound_g(const u32* a, u32 n, u32 key) {
    u32 lo = 0, hi = n;
    while (lo < hi) {
        const u32 mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Chunked warp merge.  on_hit(w, rank) is called by the lane holding w, where rank is the
// position of w among this call's hits (hits are discovered in increasing order).
template <class OnHit>
__device__ u32 warp_merge(const u32* A, u32 na, const u32* B, u32 nb, OnHit on_hit) {
    const int lane = threadIdx.x & 31;
    u32 ia = 0, ib = 0, found = 0;
    while (ia < na && ib < nb) {
        const u32 a = ia + lane < na ? __ldg(A + ia + lane) : EMPTY_KEY;
        const u32 b = ib + lane < nb ? __ldg(B + ib + lane) : EMPTY_KEY;
        const u32 ca = na - ia < 32 ? na - ia : 32, cb = nb - ib < 32 ? nb - ib : 32;
        const u32 amax = __shfl_sync(0xFFFFFFFFu, a, ca - 1);
        const u32 bmax = __shfl_sync(0xFFFFFFFFu, b, cb - 1);
        // search a among the b chunk (shuffle binary search over 32 sorted lanes; pads are EMPTY_KEY)
        u32 lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const u32 probe = __shfl_sync(0xFFFFFFFFu, b, lo + step - 1);
            if (probe < a) lo += step;
        }
        const u32 at = __shfl_sync(0xFFFFFFFFu, b, lo);
        const bool hit = (u32)lane < ca && at == a;
        const u32 ball = __ballot_sync(0xFFFFFFFFu, hit);
        if (hit) on_hit(a, found + __popc(ball & ((1u << lane) - 1)));
        found += __popc(ball);
        if (amax < bmax) ia += ca;
        else if (bmax < amax) ib += cb;
        else {
            ia += ca;
            ib += cb;
        }
    }
    return found;
}

// Lanes take entries of the shorter list and binary-search the longer one.
template <class OnHit>
__device__ u32 warp_bsearch(const u32* A, u32 na, const u32* B, u32 nb, OnHit on_hit) {
    const int lane = threadIdx.x & 31;
    const u32* S = na <= nb ? A : B;
    const u32* Lg = na <= nb ? B : A;
    const u32 ns = na <= nb ? na : nb, nl = na <= nb ? nb : na;
    u32 found = 0;
    for (u32 base = 0; base < ns; base += 32) {
        bool hit = false;
        u32 s = 0;
        if (base + lane < ns) {
            s = __ldg(S + base + lane);
            const u32 p = lower_bound_g(Lg, nl, s);
            hit = p < nl && __ldg(Lg + p) == s;
        }
        const u32 ball = __ballot_sync(0xFFFFFFFFu, hit);
        if (hit) on_hit(s, found + __popc(ball & ((1u << lane) - 1)));
        found += __popc(ball);
    }
    return found;
}

// floor(log2 x) for x > 0, cetric::log2 (util.h:136-150)
__device__ __forceinline__ u32 ilog2_floor(u32 x) { return 31 - __clz(x); }

__device__ __forceinline__ bool hybrid_use_bsearch(u32 na, u32 nb, double scale) {
    u32 d1 = na, d2 = nb;
    if (d2 < d1) {
        const u32 t = d1;
        d1 = d2;
        d2 = t;
    }
    if (d2 == 0) return false;
    return (double)((u64)d1 * ilog2_floor(d2)) < scale * (double)((u64)d1 + d2);
}

// One lane: binary_intersection with an explicit stack (intersection.h:120-192).
template <class OnHit>
__device__ u32 lane_binary(const u32* A, u32 na, const u32* B, u32 nb, u64 cutoff, OnHit on_hit, bool* overflow) {
    u32 st[BIN_STACK][4];
    int top = 0;
    u32 found = 0;
    st[top][0] = 0; st[top][1] = na; st[top][2] = 0; st[top][3] = nb; ++top;
    while (top > 0) {
        --top;
        const u32 f1 = st[top][0], l1 = st[top][1], f2 = st[top][2], l2 = st[top][3];
        const u32 d1 = l1 - f1, d2 = l2 - f2;
        if (d1 <= cutoff && d2 <= cutoff) {
            u32 i = f1, j = f2;
            while (i != l1 && j != l2) {
                const u32 a = __ldg(A + i), b = __ldg(B + j);
                if (a < b) ++i;
                else if (b < a) ++j;
                else {
                    on_hit(a, found++);
                    ++i;
                    ++j;
                }
            }
            continue;
        }
        if (d1 == 0 || d2 == 0) continue;
        u32 p1, p2;
        bool push_lo, push_hi;
        if (d1 <= d2) {
            p1 = f1 + d1 / 2;
            const u32 a = __ldg(A + p1);
            p2 = f2 + lower_bound_g(B + f2, d2, a);
            push_lo = !(p1 == l1 && p2 == l2);
            const u32 lo_l1 = p1, lo_l2 = p2;
            if (p2 != l2 && !(a < __ldg(B + p2))) {
                on_hit(a, found++);
                ++p1;
                ++p2;
            }
            push_hi = !(p1 == f1 && p2 == f2);
            if (top + 2 > BIN_STACK) { *overflow = true; return found; }
            if (push_lo) { st[top][0] = f1; st[top][1] = lo_l1; st[top][2] = f2; st[top][3] = lo_l2; ++top; }
            if (push_hi) { st[top][0] = p1; st[top][1] = l1; st[top][2] = p2; st[top][3] = l2; ++top; }
        } else {
            p2 = f2 + d2 / 2;
            const u32 b = __ldg(B + p2);
            p1 = f1 + lower_bound_g(A + f1, d1, b);
            push_lo = !(p2 == l2 && p1 == l1);
            const u32 lo_l1 = p1, lo_l2 = p2;
            if (p1 != l1 && !(b < __ldg(A + p1))) {
                on_hit(b, found++);
                ++p1;
                ++p2;
            }
            push_hi = !(p2 == f2 && p1 == f1);
            if (top + 2 > BIN_STACK) { *overflow = true; return found; }
            if (push_lo) { st[top][0] = f1; st[top][1] = lo_l1; st[top][2] = f2; st[top][3] = lo_l2; ++top; }
            if (push_hi) { st[top][0] = p1; st[top][1] = l1; st[top][2] = p2; st[top][3] = l2; ++top; }
        }
    }
    return found;
}

// ---- per-edge counting over sorted out-lists -------------------------------------------

constexpr int EDGE_BLOCK = 256;
constexpr u32 EDGE_CHUNK = 32;  // tail vertices per grab of the dynamic cursor

template <typename OffT>
__global__ void __launch_bounds__(EDGE_BLOCK) k_count_edges(u64 n, const Desc<OffT>* __restrict__ vdesc,
                                                            const u32* __restrict__ headp, int method, u64 cutoff,
                                                            double hybrid_scale, u64* __restrict__ cnt,
                                                            u64* __restrict__ partials, Control* ctl,
                                                            TriangleSink sink) {
    __shared__ u64 s_red[EDGE_BLOCK / 32];
    if (ctl->err & DEV_ERR_MASK) return;
    const int lane = threadIdx.x & 31;
    u64 local = 0;
    bool overflow = false;
    while (true) {
        u64 base = 0;
        if (lane == 0) base = atomicAdd(&ctl->edge_next, (u64)EDGE_CHUNK);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        const u64 end = base + EDGE_CHUNK < n ? base + EDGE_CHUNK : n;
        for (u64 v = base; v < end; ++v) {
            const Desc<OffT> dv = load_desc(vdesc + v);
            const u32* A = headp + list_start(dv);
            u64 tv = 0;
            if (method == KTRI_METHOD_BINARY) {
                for (u32 k0 = 0; k0 < dv.d; k0 += 32) {
                    u32 c = 0, u = 0;
                    if (k0 + lane < dv.d) {
                        u = __ldg(A + k0 + lane);
                        auto hit_w = [&](u32 w, u32) {
                            atomicAdd(&cnt[w], 1ull);
                            sink.emit((u32)v, u, w);
                        };
                        const Desc<OffT> du = load_desc(vdesc + u);
                        c = lane_binary(A, dv.d, headp + list_start(du), du.d, cutoff, hit_w, &overflow);
                        if (c) atomicAdd(&cnt[u], (u64)c);
                    }
                    tv += c;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) tv += __shfl_down_sync(0xFFFFFFFFu, tv, o);
                tv = __shfl_sync(0xFFFFFFFFu, tv, 0);
            } else {
                for (u32 k = 0; k < dv.d; ++k) {
                    const u32 u = __ldg(A + k);
                    auto hit_w = [&](u32 w, u32) {
                        atomicAdd(&cnt[w], 1ull);
                        sink.emit((u32)v, u, w);
                    };
                    const Desc<OffT> du = load_desc(vdesc + u);
                    const u32* B = headp + list_start(du);
                    u32 c;
                    const bool bs = method == KTRI_METHOD_BINARY_SEARCH ||
                                    (method == KTRI_METHOD_HYBRID && hybrid_use_bsearch(dv.d, du.d, hybrid_scale));
                    if (bs) c = warp_bsearch(A, dv.d, B, du.d, hit_w);
                    else c = warp_merge(A, dv.d, B, du.d, hit_w);
                    if (lane == 0 && c) atomicAdd(&cnt[u], (u64)c);
                    tv += c;
                }
            }
            if (lane == 0 && tv) atomicAdd(&cnt[v], tv);
            if (lane == 0) local += tv;
        }
    }
    if (overflow) atomicOr(&ctl->err, DEV_ERR_DEGREE);
    const u64 bt = block_sum_u64<EDGE_BLOCK>(local, s_red);
    if (threadIdx.x == 0) partials[blockIdx.x] = bt;
}

// ---- export of the oriented CSR ----------------------------------------------------------

template <typename OffT>
__global__ void k_outdeg(u64 n, const Desc<OffT>* __restrict__ vdesc, u64* out) {
    for (u64 v = (u64)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (u64)gridDim.x * blockDim.x)
        out[v] = load_desc(vdesc + v).d;
}

template <typename OffT>
__global__ void k_export(u64 n, const Desc<OffT>* __restrict__ vdesc, const u32* __restrict__ headp,
                         const u64* __restrict__ out_fo, u32* __restrict__ out_head) {
    const int lane = threadIdx.x & 31;
    const u64 gw = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = gw; v < n; v += nwarps) {
        const Desc<OffT> d = load_desc(vdesc + v);
        const u64 o = out_fo[v];
        for (u32 k = lane; k < d.d; k += 32) out_head[o + k] = headp[list_start(d) + k];
    }
}

// ---- batched pair intersection (known-answer tests) ----------------------------------------

constexpr int PAIR_BLOCK = 128;
constexpr u32 PAIR_TABLE = 2048;  // slots of the per-warp hash table (keys of up to 1024 entries per chunk)

__global__ void __launch_bounds__(PAIR_BLOCK) k_intersect_pairs(int method, const u32* __restrict__ av,
                                                                const u64* __restrict__ ao,
                                                                const u32* __restrict__ bv,
                                                                const u64* __restrict__ bo, u64 npairs, u64 cutoff,
                                                                double hybrid_scale, u64* __restrict__ counts,
                                                                u32* __restrict__ members, int* err) {
    __shared__ u32 s_tab[PAIR_BLOCK / 32][PAIR_TABLE];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const u64 gw = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    u32* tab = s_tab[wib];
    for (u64 p = gw; p < npairs; p += nwarps) {
        const u32* A = av + ao[p];
        const u32* B = bv + bo[p];
        const u32 na = (u32)(ao[p + 1] - ao[p]), nb = (u32)(bo[p + 1] - bo[p]);
        u32* out = members ? members + ao[p] : nullptr;
        auto rec = [&](u32 w, u32 rank) {
            if (out) out[rank] = w;
        };
        u32 c = 0;
        if (method == KTRI_METHOD_MERGE) {
            c = warp_merge(A, na, B, nb, rec);
        } else if (method == KTRI_METHOD_BINARY_SEARCH) {
            c = warp_bsearch(A, na, B, nb, rec);
        } else if (method == KTRI_METHOD_HYBRID) {
            c = hybrid_use_bsearch(na, nb, hybrid_scale) ? warp_bsearch(A, na, B, nb, rec)
                                                         : warp_merge(A, na, B, nb, rec);
        } else if (method == KTRI_METHOD_BINARY) {
            u32 r = 0;
            bool overflow = false;
            if (lane == 0) r = lane_binary(A, na, B, nb, cutoff, rec, &overflow);
            if (overflow) atomicOr(reinterpret_cast<unsigned*>(err), 1u);
            c = __shfl_sync(0xFFFFFFFFu, r, 0);
        } else {
            // owner-side table: the longer list in a shared-memory hash (in chunks), the
            // shorter one streamed through it; members are emitted in the shorter list's order
            const bool a_short = na <= nb;
            const u32* S = a_short ? A : B;
            const u32* Lg = a_short ? B : A;
            const u32 ns = a_short ? na : nb, nl = a_short ? nb : na;
            // hit flags of the streamed list are gathered per 32-entry window over all chunks
            for (u32 base = 0; base < ns; base += 32) {
                const u32 s = base + lane < ns ? __ldg(S + base + lane) : EMPTY_KEY;
                bool hit = false;
                for (u32 c0 = 0; c0 < nl; c0 += PAIR_TABLE / 2) {
                    const u32 klen = nl - c0 < PAIR_TABLE / 2 ? nl - c0 : PAIR_TABLE / 2;
                    u32 lg = ceil_log2(2 * klen);
                    if (lg < 1) lg = 1;
                    for (u32 t = lane; t < (1u << lg); t += 32) tab[t] = EMPTY_KEY;
                    __syncwarp();
                    for (u32 q = lane; q < klen; q += 32) table_insert(tab, lg, __ldg(Lg + c0 + q));
                    __syncwarp();
                    if (base + lane < ns && table_find(tab, lg, s) != NONE) hit = true;
                    __syncwarp();
                }
                const u32 ball = __ballot_sync(0xFFFFFFFFu, hit);
                if (hit) rec(s, c + __popc(ball & ((1u << lane) - 1)));
                c += __popc(ball);
            }
        }
        if (lane == 0) counts[p] = c;
    }
}

// ---- launchers ------------------------------------------------------------------------

template <typename OffT>
void launch_sort_lists(u64 n, const void* vdesc, u32* headp, u32* mid_list, u32* big_list, u32* scratch,
                       u64 scratch_per_block, int big_grid, Control* ctl, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    const auto* vd = reinterpret_cast<const Desc<OffT>*>(vdesc);
    k_sort_warp<OffT><<<num_sms * 8, 256, 0, st>>>(n, vd, headp, mid_list, big_list, ctl);
    k_sort_block<OffT><<<num_sms * 4, SORT_BLOCK, 0, st>>>(vd, headp, mid_list, ctl);
    k_sort_global<OffT><<<big_grid, SORT_BLOCK, 0, st>>>(vd, headp, big_list, scratch, scratch_per_block, ctl);
}

int count_grid_edges(int num_sms) { return num_sms * 8; }

template <typename OffT>
void launch_count_edges(u64 n, const void* vdesc, const u32* headp, int method, u64 cutoff, double hybrid_scale,
                        u64* cnt, u64* partials, int grid, Control* ctl, TriangleSink sink, cudaStream_t st) {
    k_count_edges<OffT><<<grid, EDGE_BLOCK, 0, st>>>(n, reinterpret_cast<const Desc<OffT>*>(vdesc), headp, method,
                                                     cutoff, hybrid_scale, cnt, partials, ctl, sink);
}

template <typename OffT>
void launch_outdeg(u64 n, const void* vdesc, u64* out, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    k_outdeg<OffT><<<num_sms * 4, 256, 0, st>>>(n, reinterpret_cast<const Desc<OffT>*>(vdesc), out);
}

template <typename OffT>
void launch_export(u64 n, const void* vdesc, const u32* headp, const u64* out_fo, u32* out_head, int num_sms,
                   cudaStream_t st) {
    if (n == 0) return;
    k_export<OffT><<<num_sms * 8, 256, 0, st>>>(n, reinterpret_cast<const Desc<OffT>*>(vdesc), headp, out_fo,
                                                out_head);
}

void launch_intersect_pairs(int method, const u32* a_vals, const u64* a_off, const u32* b_vals, const u64* b_off,
                            u64 npairs, u64 cutoff, double hybrid_scale, u64* counts, u32* members, int* err,
                            cudaStream_t st) {
    if (npairs == 0) return;
    u64 blocks = (npairs + (PAIR_BLOCK / 32) - 1) / (PAIR_BLOCK / 32);
    if (blocks > 4096) blocks = 4096;
    k_intersect_pairs<<<(unsigned)blocks, PAIR_BLOCK, 0, st>>>(method, a_vals, a_off, b_vals, b_off, npairs, cutoff,
                                                               hybrid_scale, counts, members, err);
}

#define KTRI_INST(OffT)                                                                                             \
    template void launch_sort_lists<OffT>(u64, const void*, u32*, u32*, u32*, u32*, u64, int, Control*, int,       \
                                          cudaStream_t);                                                            \
    template void launch_count_edges<OffT>(u64, const void*, const u32*, int, u64, double, u64*, u64*, int,         \
                                           Control*, TriangleSink, cudaStream_t);                                   \
    template void launch_outdeg<OffT>(u64, const void*, u64*, int, cudaStream_t);                                  \
    template void launch_export<OffT>(u64, const void*, const u32*, const u64*, u32*, int, cudaStream_t);
KTRI_INST(u32)
KTRI_INST(u64)
#undef KTRI_INST

}  // namespace ktri
