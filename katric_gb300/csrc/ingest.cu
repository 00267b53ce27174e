// Device side of ingest.
//  - The reference's binary format stores ids as u64 (graph-io's .head file); the engine's
//    lists hold u32.  Ids that do not fit become 0xFFFFFFFF, which the orientation kernel
//    reports as out of range.
//  - Copies between host and device memory done by the GPU's own 16-byte loads and stores over
//    the chip-to-chip link, for host buffers the device can address (pinned, registered, or
//    pageable where the platform translates host page tables for the GPU).  On GB300 they run
//    at the link's rate, as the copy engines do, but without the copy engines' recurring slow
//    windows (copies up to ten times slower for about 0.1 s, about twice a second).
#include "ktri_device.cuh"
#include "ktri_kernels.h"

namespace ktri {

namespace {

__global__ void k_narrow_ids(const u64* __restrict__ src, u64 count, u32* __restrict__ dst) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const u64 x = src[i];
        dst[i] = x > 0xFFFFFFFFull ? 0xFFFFFFFFu : (u32)x;
    }
}

// n16 16-byte words, four in flight per thread; the first `tail` threads of block 0 then copy
// the bytes after them.
__global__ void k_copy16(const uint4* __restrict__ src, uint4* __restrict__ dst, u64 n16, u32 tail) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n16; i += stride) dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < tail)
        reinterpret_cast<unsigned char*>(dst + n16)[threadIdx.x] =
            reinterpret_cast<const unsigned char*>(src + n16)[threadIdx.x];
}

}  // namespace

bool copy_by_kernel_ok(const void* src, const void* dst) {
    return ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
}

bool launch_copy(const void* src, void* dst, u64 bytes, int num_sms, cudaStream_t st) {
    if (bytes == 0) return true;
    if (!copy_by_kernel_ok(src, dst)) {
        // unaligned ends: one byte per thread, for short copies only
        if (bytes > 256) return false;
        k_copy16<<<1, 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), 0, (u32)bytes);
        return true;
    }
    const u64 n16 = bytes / 16;
    u64 blocks = (n16 + 255) / 256;
    // four blocks per SM (each with 16 KB of loads in flight) keep the link busy and leave room
    // for kernels that run beside the copy
    const u64 cap = (u64)num_sms * 4;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    k_copy16<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16,
                                               (u32)(bytes % 16));
    return true;
}

void launch_narrow_ids(const u64* src, u64 count, u32* dst, int num_sms, cudaStream_t st) {
    if (count == 0) return;
    u64 blocks = (count + 255) / 256;
    const u64 cap = (u64)num_sms * 16;
    if (blocks > cap) blocks = cap;
    k_narrow_ids<<<(unsigned)blocks, 256, 0, st>>>(src, count, dst);
}

}  // namespace ktri
