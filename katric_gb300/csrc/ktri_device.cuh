// Device helpers shared by the orientation and counting kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ktri_internal.h"

namespace ktri {

using u32 = uint32_t;
using u64 = unsigned long long;

constexpr u32 EMPTY_KEY = 0xFFFFFFFFu;
constexpr u32 NONE = 0xFFFFFFFFu;
constexpr u32 DEV_ERR_MASK = 0xFFu;

// Out-lists are stored gapped: vertex x's list starts at align4(first_out[x] + 3x), so
// every list begins on a 16-byte boundary and can be streamed with uint4 loads.  The
// region of x has room for deg(x) + 3 entries, so lists never overlap; the array holds
// nnz + 3n + 8 entries (a uint4 read past the end of the last list stays inside it).
__host__ __device__ __forceinline__ u64 oriented_start(u64 fo_x, u64 x) { return (fo_x + 3 * x + 3) & ~3ull; }
__host__ __device__ __forceinline__ u64 oriented_capacity(u64 n, u64 nnz) { return nnz + 3 * n + 8; }

// Per-vertex descriptor of the oriented out-list: start in the gapped array and length.
// Every list of the gapped array starts on a 16-byte boundary, so the 32-bit descriptor holds
// the start in 16-byte groups (4 entries) and addresses gapped arrays of up to 2^34 entries;
// the 64-bit descriptor holds the start in entries.  list_start / list_group / set_list_start
// hide the difference.
template <typename OffT>
struct Desc;
template <>
struct __align__(8) Desc<u32> {
    u32 start;  // in 16-byte groups
    u32 d;
};
template <>
struct __align__(16) Desc<u64> {
    u64 start;  // in entries
    u32 d;
    u32 pad;
};
__host__ __device__ __forceinline__ u64 list_start(const Desc<u32>& d) { return (u64)d.start << 2; }
__host__ __device__ __forceinline__ u64 list_start(const Desc<u64>& d) { return d.start; }
// the start as an index of 16-byte groups (lists in the gapped array only)
__host__ __device__ __forceinline__ u64 list_group(const Desc<u32>& d) { return d.start; }
__host__ __device__ __forceinline__ u64 list_group(const Desc<u64>& d) { return d.start >> 2; }
// s must be a multiple of 4 for the 32-bit descriptor
__host__ __device__ __forceinline__ void set_list_start(Desc<u32>& d, u64 s) { d.start = (u32)(s >> 2); }
__host__ __device__ __forceinline__ void set_list_start(Desc<u64>& d, u64 s) { d.start = s; }
// Largest gapped array (entries) the 32-bit descriptor addresses.
constexpr u64 NARROW_CAPACITY = 1ull << 34;

template <typename OffT>
__device__ __forceinline__ Desc<OffT> load_desc(const Desc<OffT>* p) {
    return __ldg(p);
}
template <>
__device__ __forceinline__ Desc<u32> load_desc<u32>(const Desc<u32>* p) {
    uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    return Desc<u32>{v.x, v.y};
}
template <>
__device__ __forceinline__ Desc<u64> load_desc<u64>(const Desc<u64>* p) {
    uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    return Desc<u64>{(u64)v.x | ((u64)v.y << 32), v.z, 0};
}

// Total order of the orientation, node_ordering::degree_outward: (deg, id).
__device__ __forceinline__ bool key_less(u64 da, u64 a, u64 db, u64 b) { return da < db || (da == db && a < b); }

// Exclusive block-wide scan of one u32 per thread.  s_warp holds BLOCK/32 entries.
// Contains __syncthreads(); every thread of the block must call it.
template <int BLOCK>
__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32* s_warp, u32* total) {
    constexpr int NW = BLOCK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        u32 w = lane < NW ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            u32 y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NW) s_warp[lane] = w;
    }
    __syncthreads();
    u32 base = warp ? s_warp[warp - 1] : 0;
    *total = s_warp[NW - 1];
    __syncthreads();
    return base + x - v;
}

// Block-wide sum of u64 (result valid in thread 0).  s_red holds BLOCK/32 entries.
template <int BLOCK>
__device__ __forceinline__ u64 block_sum_u64(u64 v, u64* s_red) {
    constexpr int NW = BLOCK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    u64 r = 0;
    if (warp == 0) {
        r = lane < NW ? s_red[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o);
    }
    __syncthreads();
    return r;
}

// Multiplicative hash into a power-of-two table of 2^lg slots (lg >= 1).
__device__ __forceinline__ u32 hash_slot(u32 w, u32 lg) { return (w * 0x9E3779B1u) >> (32 - lg); }

// Insert key w into the open-addressing table keys[0, 2^lg) (linear probing).
// Returns false when the key was already present.
__device__ __forceinline__ bool table_insert(u32* keys, u32 lg, u32 w) {
    const u32 mask = (1u << lg) - 1;
    u32 h = hash_slot(w, lg);
    for (u32 p = 0; p <= mask; ++p) {
        u32 s = (h + p) & mask;
        u32 prev = atomicCAS(&keys[s], EMPTY_KEY, w);
        if (prev == EMPTY_KEY) return true;
        if (prev == w) return false;
    }
    return true;  // unreachable: tables are at most half full
}

// Look key w up; returns the slot or NONE.
__device__ __forceinline__ u32 table_find(const u32* keys, u32 lg, u32 w) {
    const u32 mask = (1u << lg) - 1;
    u32 h = hash_slot(w, lg);
    for (u32 p = 0; p <= mask; ++p) {
        u32 s = (h + p) & mask;
        u32 k = keys[s];
        if (k == w) return s;
        if (k == EMPTY_KEY) return NONE;
    }
    return NONE;
}

// Bucketized open addressing for the counting tables: 2^lg slots (lg >= 2) in buckets of
// four.  A key hashes to a bucket; inserts fill a bucket's slots in order (slot i is taken
// only after slots 0..i-1), so a bucket whose last slot is empty ends every lookup.  A lookup
// reads one bucket (16 bytes) per step; at the load factors used here almost every lookup
// ends in its first bucket, which keeps the lanes of a warp in step.
__device__ __forceinline__ u32 bucket_home(u32 w, u32 lg) {
    return lg > 2 ? ((w * 0x9E3779B1u) >> (34 - lg)) : 0u;
}

// Returns false when w was already present.
__device__ __forceinline__ bool bucket_insert(u32* keys, u32 lg, u32 w) {
    const u32 nb_mask = (1u << (lg - 2)) - 1;
    u32 b = bucket_home(w, lg);
    for (u32 it = 0; it <= nb_mask; ++it) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const u32 prev = atomicCAS(&keys[4 * b + i], EMPTY_KEY, w);
            if (prev == EMPTY_KEY) return true;
            if (prev == w) return false;
        }
        b = (b + 1) & nb_mask;
    }
    return true;  // unreachable: tables are at most half full
}

// Count a lookup of w: on a hit, add one to the slot's hit counter and return 1.
__device__ __forceinline__ u32 bucket_probe(const u32* keys, u32* hits, u32 lg, u32 w) {
    const u32 nb_mask = (1u << (lg - 2)) - 1;
    u32 b = bucket_home(w, lg);
    for (u32 it = 0; it <= nb_mask; ++it) {
        const uint4 q = *reinterpret_cast<const uint4*>(keys + 4 * b);
        const bool m0 = q.x == w, m1 = q.y == w, m2 = q.z == w, m3 = q.w == w;
        if (m0 | m1 | m2 | m3) {
            const u32 i = m0 ? 0u : (m1 ? 1u : (m2 ? 2u : 3u));
            atomicAdd(&hits[4 * b + i], 1u);
            return 1u;
        }
        if (q.w == EMPTY_KEY) return 0u;
        b = (b + 1) & nb_mask;
    }
    return 0u;
}

__host__ __device__ __forceinline__ u32 ceil_log2(u32 v) {
    u32 lg = 0;
    while ((1u << lg) < v) ++lg;
    return lg;
}

}  // namespace ktri
