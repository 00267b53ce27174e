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
#include "ktri.h"
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

// Contraction, pass 1: per local vertex the number of ghosts in its out-list (the edges that
// survive), whether it survives, and the longest surviving list.
__global__ void k_contract_count(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n, u64 n_local,
                                 u64* __restrict__ cnt, u64* __restrict__ keep, unsigned long long* maxlen) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = warp; v < n_local; v += nwarps) {
        u64 c = 0;
        for (u64 e = fo[v] + lane; e < fo[v + 1]; e += 32) {
            const u32 u = head[e];
            c += (u >= n_local && u < n) ? 1u : 0u;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
        if (lane == 0) {
            cnt[v] = c;
            keep[v] = c ? 1ull : 0ull;
            if (c) atomicMax(maxlen, c);
        }
    }
}

// Contraction, pass 2: the surviving vertices renumbered in order, their ghost lists copied
// in list order, and one descriptor per surviving list (for the id sort).
__global__ void k_contract_scatter(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n, u64 n_local,
                                   const u64* __restrict__ cnt_scan, const u64* __restrict__ keep_scan,
                                   u32* __restrict__ kept, u64* __restrict__ out_fo, u32* __restrict__ out_head,
                                   Desc<u64>* __restrict__ desc) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    if (warp == 0 && lane == 0) out_fo[keep_scan[n_local]] = cnt_scan[n_local];
    for (u64 v = warp; v < n_local; v += nwarps) {
        const u64 base = cnt_scan[v], c = cnt_scan[v + 1] - base;
        if (c == 0) continue;
        const u64 k = keep_scan[v];
        if (lane == 0) {
            kept[k] = (u32)v;
            out_fo[k] = base;
            Desc<u64> d;
            d.start = base;
            d.d = (u32)c;
            d.pad = 0;
            desc[k] = d;
        }
        u64 at = base;
        for (u64 e0 = fo[v]; e0 < fo[v + 1]; e0 += 32) {
            const u64 e = e0 + lane;
            const u32 u = e < fo[v + 1] ? head[e] : 0xFFFFFFFFu;
            const bool g = u >= n_local && u < n;
            const u32 ball = __ballot_sync(0xFFFFFFFFu, g);
            if (g) out_head[at + __popc(ball & ((1u << lane) - 1))] = u;
            at += __popc(ball);
        }
    }
}

// Per-vertex cost of the reference's load-balancing cost functions (cost_function.h:287-345),
// one warp per vertex; deg = undirected degree, dplus = out-degree in (degree, id) order.
__global__ void k_vertex_cost(const u64* __restrict__ fo, const u32* __restrict__ head, u64 n,
                              const u32* __restrict__ deg, const u32* __restrict__ dplus, int fn, u64* __restrict__ cost) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 v = warp; v < n; v += nwarps) {
        const u64 dv = deg[v], ov = dplus[v];
        u64 c = 0;
        if (fn == KTRI_COST_DPD || fn == KTRI_COST_IDPD) {
            const bool higher = fn == KTRI_COST_DPD;
            for (u64 e = fo[v] + lane; e < fo[v + 1]; e += 32) {
                const u32 u = head[e];
                if (u >= n) continue;
                const bool above = key_less(dv, v, deg[u], u);  // (deg u, u) > (deg v, v)
                if (above == higher) c += ov + dplus[u];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
        } else {
            c = fn == KTRI_COST_N ? 1 : fn == KTRI_COST_D ? dv : fn == KTRI_COST_DH ? ov : fn == KTRI_COST_DDH ? dv * ov : ov * ov;
        }
        if (lane == 0) cost[v] = c;
    }
}

// boundaries[i] = first vertex whose cost prefix reaches i / parts of the total (prefix holds
// the exclusive prefix sums, prefix[n] = total); boundaries[parts] = n.
__global__ void k_cost_boundaries(const u64* __restrict__ prefix, u64 n, u32 parts, u64* __restrict__ boundaries) {
    const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > parts) return;
    if (i == parts) {
        boundaries[i] = n;
        return;
    }
    const u64 total = prefix[n];
    const u64 target = (u64)(((unsigned __int128)total * i + parts - 1) / parts);
    u64 lo = 0, hi = n;  // smallest v with prefix[v] >= target
    while (lo < hi) {
        const u64 mid = (lo + hi) >> 1;
        if (prefix[mid] >= target) hi = mid;
        else lo = mid + 1;
    }
    boundaries[i] = lo;
}

}  // namespace

u64 dag_scan_chunks(u64 n) { return (n + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK; }

void launch_cost_partition(const u64* fo, const u32* head, u64 n, const u32* deg, const u32* dplus, int fn, u32 parts,
                           u64* cost, u64* sums, u64* boundaries, int num_sms, cudaStream_t st) {
    if (n == 0) return;
    u64 blocks = (n * 32 + 255) / 256;
    const u64 cap = (u64)num_sms * 16;
    if (blocks > cap) blocks = cap;
    cudaMemsetAsync(cost + n, 0, sizeof(u64), st);
    k_vertex_cost<<<(unsigned)blocks, 256, 0, st>>>(fo, head, n, deg, dplus, fn, cost);
    launch_scan_u64(cost, n + 1, sums, st);
    k_cost_boundaries<<<(unsigned)((parts + 1 + 255) / 256), 256, 0, st>>>(cost, n, parts, boundaries);
}

void launch_scan_u64(u64* x, u64 len, u64* sums, cudaStream_t st) {
    if (len == 0) return;
    const u64 nch = (len + SCAN_CHUNK - 1) / SCAN_CHUNK;
    k_scan_chunks<<<(unsigned)nch, SCAN_BLOCK, 0, st>>>(x, len, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(sums, nch);
    k_scan_add<<<(unsigned)nch, SCAN_BLOCK, 0, st>>>(x, len, sums);
}

void launch_contract(const u64* fo, const u32* head, u64 n, u64 n_local, u64* cnt, u64* keep, u64* sums,
                     unsigned long long* maxlen, u32* kept, u64* out_fo, u32* out_head, void* desc, int num_sms,
                     cudaStream_t st) {
    if (n_local == 0) return;
    u64 blocks = (n_local * 32 + 255) / 256;
    const u64 cap = (u64)num_sms * 16;
    if (blocks > cap) blocks = cap;
    cudaMemsetAsync(cnt + n_local, 0, sizeof(u64), st);
    cudaMemsetAsync(keep + n_local, 0, sizeof(u64), st);
    cudaMemsetAsync(maxlen, 0, sizeof(u64), st);
    k_contract_count<<<(unsigned)blocks, 256, 0, st>>>(fo, head, n, n_local, cnt, keep, maxlen);
    launch_scan_u64(cnt, n_local + 1, sums, st);
    launch_scan_u64(keep, n_local + 1, sums, st);
    k_contract_scatter<<<(unsigned)blocks, 256, 0, st>>>(fo, head, n, n_local, cnt, keep, kept, out_fo, out_head,
                                                       reinterpret_cast<Desc<u64>*>(desc));
}

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
