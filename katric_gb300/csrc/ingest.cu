// Device side of file ingest: the reference's binary format stores ids as u64
// (graph-io's .head file); the engine's lists hold u32.  Ids that do not fit become
// 0xFFFFFFFF, which the orientation kernel reports as out of range.
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

}  // namespace

void launch_narrow_ids(const u64* src, u64 count, u32* dst, int num_sms, cudaStream_t st) {
    if (count == 0) return;
    u64 blocks = (count + 255) / 256;
    const u64 cap = (u64)num_sms * 16;
    if (blocks > cap) blocks = cap;
    k_narrow_ids<<<(unsigned)blocks, 256, 0, st>>>(src, count, dst);
}

}  // namespace ktri
