// Symmetrisation of oriented out-lists into the undirected CSR of their edges.
//
// KaTric's local phase (CetricEdgeIterator::run_local, cetric_edge_iterator.h:230-298, and
// the variant with ghosts, :301-388) walks out-lists the caller has already oriented: out_adj
// of the rank's vertices and ghost_adj of its ghosts.  The triangles it finds are the
// triangles whose three edges appear in those lists.  That set does not depend on the
// orientation, so the lists are turned back into an undirected CSR here and counted by the
// ordinary pipeline, under its own (degree, id) orientation.
//
// Vertex v's undirected list is its out-list (in the given order) followed by its in-list
// (in arrival order).  Entries that are out of range or self-loops are copied into the out
// part as they are, so the pipeline's validation reports them; they get no in-list entry.
#include "ktri_device.cuh"
#include "ktri_kernels.h"

namespace ktri {

namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_IPT = 8;
constexpr u64 SCAN_CHUNK = (u64)SCAN_BLOCK * SCAN_IPT;

// deg[v] = |out(v)| + number of valid entries naming v (deg has n + 1 zeroed entries).
__global__ void k_dag_degrees(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n, u64* deg) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = warp; v < n; v += nwarps) {
        const u64 a = fo[v], b = fo[v + 1];
        if (lane == 0 && b > a) atomicAdd(&deg[v], b - a);
        for (u64 e = a + lane; e < b; e += 32) {
            const u32 u = head[e];
            if (u < n && u != v) atomicAdd(&deg[u], 1ull);
        }
    }
}

// In-place exclusive scan of x[0..len), pass 1: every chunk scanned locally, its sum to sums.
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_chunks(u64* x, u64 len, u64* sums) {
    __shared__ u64 s_warp[SCAN_BLOCK / 32];
    const u64 c0 = (u64)blockIdx.x * SCAN_CHUNK + (u64)threadIdx.x * SCAN_IPT;
    u64 v[SCAN_IPT], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        v[k] = c0 + k < len ? x[c0 + k] : 0ull;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u64 incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u64 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    u64 wbase = 0, total = 0;
#pragma unroll
    for (int w = 0; w < SCAN_BLOCK / 32; ++w) {
        if (w < warp) wbase += s_warp[w];
        total += s_warp[w];
    }
    u64 run = wbase + incl - t;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        if (c0 + k < len) x[c0 + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Pass 2: exclusive scan of the chunk sums in one block (any number of chunks).
__global__ void __launch_bounds__(1024) k_scan_sums(u64* sums, u64 nchunks) {
    __shared__ u64 s_warp[32];
    __shared__ u64 s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (u64 base = 0; base < nchunks; base += 1024) {
        const u64 i = base + threadIdx.x;
        const u64 t = i < nchunks ? sums[i] : 0ull;
        u64 incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u64 y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        u64 wbase = 0, total = 0;
        for (int w = 0; w < 32; ++w) {
            if (w < warp) wbase += s_warp[w];
            total += s_warp[w];
        }
        const u64 carry = s_carry;
        if (i < nchunks) sums[i] = carry + wbase + incl - t;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + total;
        __syncthreads();
    }
}

// Pass 3: add each chunk's offset.
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_add(u64* x, u64 len, const u64* sums) {
    const u64 off = sums[blockIdx.x];
    const u64 c0 = (u64)blockIdx.x * SCAN_CHUNK;
    for (u64 k = threadIdx.x; k < SCAN_CHUNK; k += SCAN_BLOCK)
        if (c0 + k < len) x[c0 + k] += off;
}

// Undirected lists: v's out-list copied to the front of its range, v appended to the in part
// of every valid out-neighbour u (cursor[u] counts u's in-entries so far).
__global__ void k_dag_scatter(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                              const u64* __restrict__ fs, u32* __restrict__ hs, u32* cursor) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = warp; v < n; v += nwarps) {
        const u64 a = fo[v], b = fo[v + 1], s = fs[v];
        for (u64 e = a + lane; e < b; e += 32) {
            const u32 u = head[e];
            hs[s + (e - a)] = u;
            if (u < n && u != v) {
                const u32 pos = atomicAdd(&cursor[u], 1u);
                hs[fs[u] + (fo[u + 1] - fo[u]) + pos] = (u32)v;
            }
        }
    }
}

}  // namespace

u64 dag_scan_chunks(u64 n) { return (n + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK; }

void launch_dag_symmetrize(const u64* fo, const u32* head, u64 n, u64* fs, u32* hs, u32* cursor, u64* sums,
                           int num_sms, cudaStream_t st) {
    if (n == 0) return;
    cudaMemsetAsync(fs, 0, sizeof(u64) * (n + 1), st);
    cudaMemsetAsync(cursor, 0, sizeof(u32) * n, st);
    const u64 warps_needed = n;
    u64 blocks = (warps_needed * 32 + 255) / 256;
    const u64 cap = (u64)num_sms * 16;
    if (blocks > cap) blocks = cap;
    k_dag_degrees<<<(unsigned)blocks, 256, 0, st>>>(fo, head, n, fs);
    const u64 nch = dag_scan_chunks(n);
    k_scan_chunks<<<(unsigned)nch, SCAN_BLOCK, 0, st>>>(fs, n + 1, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(sums, nch);
    k_scan_add<<<(unsigned)nch, SCAN_BLOCK, 0, st>>>(fs, n + 1, sums);
    k_dag_scatter<<<(unsigned)blocks, 256, 0, st>>>(fo, head, n, fs, hs, cursor);
}

}  // namespace ktri
