// Serving: a request loop that counts many graphs with continuous batching.
//
// Requests (one graph each) are queued by ktri_server_submit.  A worker thread forms a batch
// from the waiting requests under a device-memory budget, packs the graphs as one disjoint
// union (host staging -> device, ids rebased on the device), counts the whole batch with one
// ktri_count_batch_device call on one of `slots` contexts (each with its own stream), and
// reads back totals and per-vertex counts.  While one batch runs, the next one is formed from
// the requests that arrived meanwhile and launched on a free slot, so the work of batches
// overlaps on the GPU.  Graphs stay resident (CSR and counts on the device, keyed by the
// caller's graph key) until the memory budget needs their room; a repeated request for a
// resident graph is answered from the resident counts without counting again, and one for a
// graph that is still queued or counting waits for that count instead of starting another.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ktri.h"
#include "ktri_device.cuh"
#include "ktri_internal.h"
#include "ktri_kernels.h"

using ktri::u32;
using ktri::u64;

namespace {

// Where the device reads pageable host memory (ATS/HMM over NVLink-C2C on Grace + Blackwell),
// a batch is gathered straight from the callers' arrays: no host-side packing pass.
struct GraphSrc {
    const u64* fo;  // the caller's first_out (n + 1 entries), host memory
    const u32* head;
    u64* pv_out;    // where the per-vertex counts go (host memory), or null
};

// The warp's 256 consecutive union elements at base: lane handles base + lane + 32 j, so each
// load instruction of the warp reads 128 consecutive bytes.  first[g] is the union offset of
// graph g (first[k] = total); g starts at the warp's first element's graph.
__device__ __forceinline__ u64 warp_graph_of(const u64* first, u64 k, u64 x) {
    u64 lo = 0, hi = k;  // first[lo] <= x < first[hi]
    while (hi - lo > 1) {
        const u64 mid = (lo + hi) >> 1;
        if (first[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Rebase a packed union: graph g's offsets were copied relative to its own start and its
// ids relative to its own first vertex.  The whole grid walks the union (a warp takes 256
// consecutive elements and finds their graph by binary search), so a large graph is spread
// over all SMs instead of one block.
__global__ void k_rebase(u64* __restrict__ fo, u32* __restrict__ head, const u64* __restrict__ vf,
                         const u64* __restrict__ ef, u64 k, u64 n, u64 nnz) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 base = warp * 256; base < nnz; base += nwarps * 256) {
        u64 g = 0;
        if (lane == 0) g = warp_graph_of(ef, k, base);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
#pragma unroll 4
        for (int j = 0; j < 8; ++j) {
            const u64 e = base + lane + 32 * j;
            if (e >= nnz) break;
            while (e >= ef[g + 1]) ++g;
            head[e] += (u32)vf[g];
        }
    }
    for (u64 base = warp * 256; base < n; base += nwarps * 256) {
        u64 g = 0;
        if (lane == 0) g = warp_graph_of(vf, k, base);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
#pragma unroll 4
        for (int j = 0; j < 8; ++j) {
            const u64 v = base + lane + 32 * j;
            if (v >= n) break;
            while (v >= vf[g + 1]) ++g;
            fo[v + 1] += ef[g];
        }
    }
}

// One word written by one thread (the engine's stop word, from a stream of its own).
__global__ void k_set_word(unsigned* p, unsigned v) { *(volatile unsigned*)p = v; }

__global__ void k_gather(const GraphSrc* __restrict__ src, const u64* __restrict__ vf, const u64* __restrict__ ef,
                         u64 k, u64 n, u64 nnz, u64* __restrict__ dfo, u32* __restrict__ dhead) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    if (warp == 0 && lane == 0) dfo[0] = 0;
    for (u64 base = warp * 256; base < nnz; base += nwarps * 256) {
        u64 g = 0;
        if (lane == 0) g = warp_graph_of(ef, k, base);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
#pragma unroll 4
        for (int j = 0; j < 8; ++j) {
            const u64 e = base + lane + 32 * j;
            if (e >= nnz) break;
            while (e >= ef[g + 1]) ++g;
            dhead[e] = src[g].head[e - ef[g]] + (u32)vf[g];
        }
    }
    for (u64 base = warp * 256; base < n; base += nwarps * 256) {
        u64 g = 0;
        if (lane == 0) g = warp_graph_of(vf, k, base);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
#pragma unroll 4
        for (int j = 0; j < 8; ++j) {
            const u64 v = base + lane + 32 * j;
            if (v >= n) break;
            while (v >= vf[g + 1]) ++g;
            dfo[v + 1] = src[g].fo[v - vf[g] + 1] + ef[g];
        }
    }
}

// Per-vertex counts of the union written into each wanting request's host buffer.
__global__ void k_scatter_pv(const GraphSrc* __restrict__ src, const u64* __restrict__ vf, u64 k, u64 n,
                             const u64* __restrict__ pv) {
    const int lane = threadIdx.x & 31;
    const u64 warp = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 base = warp * 256; base < n; base += nwarps * 256) {
        u64 g = 0;
        if (lane == 0) g = warp_graph_of(vf, k, base);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
#pragma unroll 4
        for (int j = 0; j < 8; ++j) {
            const u64 v = base + lane + 32 * j;
            if (v >= n) break;
            while (v >= vf[g + 1]) ++g;
            u64* out = src[g].pv_out;
            if (out) out[v - vf[g]] = pv[v];
        }
    }
}

// The caller's own CSR of one graph of a rebased union (the inverse of k_rebase for it).
__global__ void k_unbase(u64* __restrict__ dfo, u32* __restrict__ dhead, const u64* __restrict__ sfo,
                         const u32* __restrict__ shead, u64 n, u64 nnz, u64 vb, u64 eb) {
    const u64 stride = (u64)gridDim.x * blockDim.x;
    const u64 i0 = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    for (u64 i = i0; i <= n; i += stride) dfo[i] = sfo[vb + i] - eb;
    for (u64 i = i0; i < nnz; i += stride) dhead[i] = shead[eb + i] - (u32)vb;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id = 0, key = 0;
    std::vector<uint64_t> fo;  // the copied CSR (empty when borrowed)
    std::vector<uint32_t> head;
    const uint64_t* bfo = nullptr;  // the caller's CSR, read in place (borrowed or copied)
    const uint32_t* bhead = nullptr;
    uint64_t n = 0, nnz = 0;
    bool want_pv = false;
    double t_submit = 0, t_done = 0;
    bool done = false;
    int status = KTRI_OK;
    uint64_t total = 0;
    std::shared_ptr<std::vector<uint64_t>> pv;  // per-vertex counts (shared with the followers)
    std::vector<Request*> followers;  // later requests for the same key, answered with this one
    bool follower_pv = false;         // a follower wants the per-vertex counts
    bool pv_written = false;          // the batch wrote the per-vertex counts into pv directly
    bool pv_wanted = false;           // want_pv or follower_pv when the batch was formed (under the lock)
};

struct Resident {  // a graph kept on the device with its counts
    uint64_t key = 0, n = 0, nnz = 0, total = 0;
    void* mem = nullptr;  // [fo u64 n+1][head u32 nnz][pv u64 n]
    size_t bytes = 0;
    std::list<uint64_t>::iterator lru;
    // the per-vertex counts on the host as well (read-only, shared with every request that a
    // cache hit answers), while the server's host copies stay within a quarter of the budget
    std::shared_ptr<std::vector<uint64_t>> pv_host;
};

struct Slot {
    ktri_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr;  // the batch's first copy is enqueued (timing event)
    cudaEvent_t done = nullptr;   // the batch's last read-back is finished (timing event)
    cudaEvent_t cache_done = nullptr;  // resident copies out of this slot's buffers are finished
    bool busy = false;
    std::vector<Request*> reqs;
    // device union buffers (grow-only)
    void* dev = nullptr;
    size_t dev_bytes = 0;
    // pinned host staging (grow-only)
    void* host = nullptr;
    size_t host_bytes = 0;
    u64 n_total = 0, nnz_total = 0;
    size_t off_fo = 0, off_head = 0, off_vf = 0, off_ef = 0, off_tot = 0, off_pv = 0, off_src = 0;
    size_t h_tot = 0, h_pv = 0;
    bool direct = false;  // this batch was gathered from host memory by the device
    // engine mode: the batch's counting phase is job (slot index) with this sequence number; the
    // slot waits for the engine while counting is set, then reads back
    unsigned long long seq = 0;
    bool counting = false;
    ktri::Control* ctl = nullptr;
    double t_published = 0;
};

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct ktri_server {
    int device = 0;
    bool pageable = false;  // the device reads pageable host memory
    ktri_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;  // requests to count, in arrival order
    std::deque<Request*> hits;     // requests for keys resident at submit: answered from them
    std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    std::vector<Slot> slots;
    cudaStream_t aux = nullptr;  // cache copies
    // resident graphs
    std::unordered_map<uint64_t, Resident> resident;
    std::unordered_map<uint64_t, Request*> leaders;  // key -> the queued or counting request for it
    std::list<uint64_t> lru;  // front = most recent
    size_t resident_bytes = 0;
    size_t host_pv_bytes = 0;  // host bytes of the resident graphs' pv_host
    ktri_server_stats st{};
    int fatal = KTRI_OK;
    double alloc_s_acc = 0;  // seconds spent in grow() by the worker, moved into st.alloc_us under the lock
    // the engine: one persistent counting kernel that drains the slots' published jobs
    bool engine = false;
    ktri::EngineJob* jobs = nullptr;         // device, one per slot
    unsigned long long* done_host = nullptr;  // host-mapped completion words, one per slot
    unsigned long long* done_dev = nullptr;   // their device address
    unsigned* stop_dev = nullptr;             // device word: nonzero tells the engine to leave
    cudaStream_t control_stream = nullptr;    // highest priority: sets stop_dev while the engine runs
    cudaStream_t engine_stream = nullptr;
    cudaEvent_t engine_done = nullptr;        // recorded after each engine launch
    bool engine_launched = false;
    unsigned long long seq_next = 1;
    int engine_grid = 0;
    uint64_t engine_launches = 0;
};

namespace {

// Device bytes a batch of (n_total, nnz_total, k graphs) needs in a slot: union buffers plus
// the counting workspace.
size_t batch_bytes(u64 n, u64 nnz, u64 k) {
    return al(8 * (n + 1)) + al(4 * (nnz + 1)) + 2 * al(8 * (k + 1)) + al(8 * k) + al(8 * (n + 1)) +
           (size_t)ktri_workspace_bytes(n, nnz, KTRI_METHOD_AUTO);
}

// Drop one resident graph (called with s->mu held).
void drop_resident(ktri_server* s, std::unordered_map<uint64_t, Resident>::iterator it) {
    cudaFreeAsync(it->second.mem, s->aux);
    s->resident_bytes -= it->second.bytes;
    if (it->second.pv_host) s->host_pv_bytes -= 8 * it->second.n;
    s->lru.erase(it->second.lru);
    s->resident.erase(it);
    s->st.evictions++;
}

// Evict least-recently-used resident graphs until `need` more bytes fit the budget.
// Called with s->mu held.
bool make_room(ktri_server* s, size_t need, size_t inflight) {
    while (s->resident_bytes + inflight + need > s->opts.memory_budget && !s->lru.empty()) {
        auto it = s->resident.find(s->lru.back());
        if (it != s->resident.end()) drop_resident(s, it);
        else s->lru.pop_back();
    }
    return s->resident_bytes + inflight + need <= s->opts.memory_budget;
}

void finish(ktri_server* s, Request* r, int status) {
    r->status = status;
    r->t_done = now_s();
    r->done = true;
    s->st.completed++;
    if (r->key) {
        auto it = s->leaders.find(r->key);
        if (it != s->leaders.end() && it->second == r) s->leaders.erase(it);
    }
    for (Request* f : r->followers) {
        f->total = r->total;
        if (f->want_pv && status == KTRI_OK) f->pv = r->pv;
        f->status = status;
        f->t_done = r->t_done;
        f->done = true;
        s->st.completed++;
    }
    r->followers.clear();
}

// Answer a request for a resident graph from its resident counts.
// Host copies of resident counts are kept while they total at most a quarter of the budget.
bool host_pv_room(const ktri_server* s, u64 n) { return s->host_pv_bytes + 8 * n <= s->opts.memory_budget / 4; }

void serve_resident(ktri_server* s, Request* r, Resident& res) {
    r->total = res.total;
    if (r->want_pv && res.n) {
        if (res.pv_host) {
            r->pv = res.pv_host;  // no copy under the lock: the request shares the host counts
        } else {
            r->pv = std::make_shared<std::vector<uint64_t>>(res.n);
            const char* base = static_cast<const char*>(res.mem);
            const size_t off_pv = al(8 * (res.n + 1)) + al(4 * (res.nnz + 1));
            cudaMemcpyAsync(r->pv->data(), base + off_pv, 8 * res.n, cudaMemcpyDeviceToHost, s->aux);
            cudaStreamSynchronize(s->aux);
            if (host_pv_room(s, res.n)) {
                res.pv_host = r->pv;
                s->host_pv_bytes += 8 * res.n;
            }
        }
    }
    s->lru.erase(res.lru);
    s->lru.push_front(res.key);
    res.lru = s->lru.begin();
    s->st.cache_hits++;
}

// Keep a counted graph resident (CSR + counts on the device), room permitting.  The copy is
// taken on the device from the slot's union, on the auxiliary stream, which the slot's next
// batch waits for (cache_done) before it overwrites the union.
void keep_resident(ktri_server* s, Request* r, const Slot& sl, u64 vbase, u64 ebase, size_t inflight) {
    if (!r->key) return;
    // a key names one graph: a graph of another size counted under a resident key replaces it
    auto old = s->resident.find(r->key);
    if (old != s->resident.end()) {
        if (old->second.n == r->n && old->second.nnz == r->nnz) return;
        drop_resident(s, old);
    }
    const size_t bytes = al(8 * (r->n + 1)) + al(4 * (r->nnz + 1)) + al(8 * (r->n + 1));
    if (bytes > s->opts.memory_budget / 4) return;
    if (!make_room(s, bytes, inflight)) return;
    void* mem = nullptr;
    if (cudaMallocAsync(&mem, bytes, s->aux) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    char* b = static_cast<char*>(mem);
    const char* d = static_cast<const char*>(sl.dev);
    // the slot's union holds rebased ids; the resident copy keeps the caller's own CSR
    const u64 items = std::max<u64>(r->n + 1, r->nnz);
    const unsigned blocks = (unsigned)std::min<u64>((items + 255) / 256, 2048);
    k_unbase<<<blocks, 256, 0, s->aux>>>(reinterpret_cast<u64*>(b), reinterpret_cast<u32*>(b + al(8 * (r->n + 1))),
                                         reinterpret_cast<const u64*>(d + sl.off_fo),
                                         reinterpret_cast<const u32*>(d + sl.off_head), r->n, r->nnz, vbase, ebase);
    if (r->n)
        cudaMemcpyAsync(b + al(8 * (r->n + 1)) + al(4 * (r->nnz + 1)), d + sl.off_pv + 8 * vbase, 8 * r->n,
                        cudaMemcpyDeviceToDevice, s->aux);
    Resident res;
    res.key = r->key;
    res.n = r->n;
    res.nnz = r->nnz;
    res.total = r->total;
    res.mem = mem;
    res.bytes = bytes;
    if (r->pv && r->pv->size() == r->n && r->n && host_pv_room(s, r->n)) {
        res.pv_host = r->pv;
        s->host_pv_bytes += 8 * r->n;
    }
    s->lru.push_front(r->key);
    res.lru = s->lru.begin();
    s->resident_bytes += bytes;
    s->resident.emplace(r->key, res);
}

int grow(ktri_server* s, void** p, size_t* have, size_t need, bool host) {
    if (need <= *have) return KTRI_OK;
    const double t0 = now_s();
    struct Charge {
        ktri_server* s;
        double t0;
        ~Charge() { s->alloc_s_acc += now_s() - t0; }
    } charge{s, t0};
    if (*p) {
        cudaDeviceSynchronize();  // nothing may still read the old buffer
        if (host) cudaFreeHost(*p);
        else cudaFree(*p);
        *p = nullptr;
        *have = 0;
    }
    const size_t want = need + need / 4;
    cudaError_t e = host ? cudaHostAlloc(p, want, cudaHostAllocDefault) : cudaMalloc(p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return KTRI_ERR_OUT_OF_MEMORY;
    }
    *have = want;
    return KTRI_OK;
}

// Offsets of a batch of k graphs (n vertices, nnz entries) in a slot's device buffer and in
// its pinned host staging.
struct SlotLayout {
    size_t fo = 0, head = 0, vf = 0, ef = 0, tot = 0, pv = 0, src = 0, dev_bytes = 0;
    size_t h_fo = 0, h_head = 0, h_vf = 0, h_ef = 0, h_src = 0, h_tot = 0, h_pv = 0, host_bytes = 0;
};

SlotLayout slot_layout(u64 n, u64 nnz, u64 k, bool direct) {
    SlotLayout L;
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t at = off;
        off = al(off + b);
        return at;
    };
    L.fo = take(8 * (n + 1));
    L.head = take(4 * (nnz + 1));
    L.vf = take(8 * (k + 1));
    L.ef = take(8 * (k + 1));
    L.tot = take(8 * k);
    L.pv = take(8 * (n + 1));
    L.src = take(sizeof(GraphSrc) * (k + 1));
    L.dev_bytes = off;
    // host staging: [fo][head] (staged batches only), [vf][ef][sources], then read-back [tot][pv]
    size_t hoff = 0;
    auto htake = [&](size_t b) {
        size_t at = hoff;
        hoff = al(hoff + b);
        return at;
    };
    L.h_fo = direct ? 0 : htake(8 * (n + 1));
    L.h_head = direct ? 0 : htake(4 * (nnz + 1));
    L.h_vf = htake(8 * (k + 1));
    L.h_ef = htake(8 * (k + 1));
    L.h_src = htake(sizeof(GraphSrc) * (k + 1));
    L.h_tot = htake(8 * k);
    L.h_pv = direct ? 0 : htake(8 * (n + 1));
    L.host_bytes = hoff;
    return L;
}

// Scans with every published job finished (about 2 us each) before the engine leaves; it leaves
// as a whole (the first block to go sets the stop word).
constexpr unsigned ENGINE_IDLE_POLLS = 100;

size_t slot_index(const ktri_server* s, const Slot& sl) { return (size_t)(&sl - s->slots.data()); }

// Launch the engine unless one is running.  A job published while the running engine was
// already leaving is picked up by the next launch, which the worker loop makes as soon as it
// sees the previous one done and a slot still waiting.
int ensure_engine(ktri_server* s) {
    if (s->engine_launched) {
        const cudaError_t q = cudaEventQuery(s->engine_done);
        if (q == cudaErrorNotReady) return KTRI_OK;
        if (q != cudaSuccess) return KTRI_ERR_CUDA;
    }
    k_set_word<<<1, 1, 0, s->engine_stream>>>(s->stop_dev, 0u);  // before the launch, in stream order
    ktri::launch_engine(s->jobs, (u32)s->slots.size(), s->done_dev, s->stop_dev, ENGINE_IDLE_POLLS, s->engine_grid,
                        s->engine_stream);
    cudaEventRecord(s->engine_done, s->engine_stream);
    s->engine_launched = true;
    s->st.engine_launches++;
    return cudaGetLastError() == cudaSuccess ? KTRI_OK : KTRI_ERR_CUDA;
}

// Tell a running engine to leave, wait for it, and free its resources (the worker has ended).
void release_engine(ktri_server* s) {
    if (s->engine_launched && s->stop_dev) {
        k_set_word<<<1, 1, 0, s->control_stream>>>(s->stop_dev, 1u);
        cudaStreamSynchronize(s->engine_stream);
    }
    if (s->engine_done) cudaEventDestroy(s->engine_done);
    if (s->engine_stream) cudaStreamDestroy(s->engine_stream);
    if (s->control_stream) cudaStreamDestroy(s->control_stream);
    if (s->stop_dev) cudaFree(s->stop_dev);
    if (s->jobs) cudaFree(s->jobs);
    if (s->done_host) cudaFreeHost(s->done_host);
    s->engine_done = nullptr;
    s->engine_stream = nullptr;
    s->jobs = nullptr;
    s->stop_dev = nullptr;
    s->control_stream = nullptr;
    s->done_host = nullptr;
    s->engine_launched = false;
}

// Copy between a slot's pinned staging (device-addressable) and its device buffers on st, by a
// kernel: on Grace + Blackwell the copy engines have recurring slow windows that the SMs' own
// loads and stores over the chip-to-chip link do not.  The copy engines take what a kernel
// cannot (unaligned ends beyond 256 bytes).
void copy_staging(const Slot& sl, void* dst, const void* src, size_t bytes, bool to_device, cudaStream_t st) {
    if (bytes == 0) return;
    if (!ktri::launch_copy(src, dst, bytes, ktri::ctx_num_sms(sl.ctx), st))
        cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, st);
}

// Read-back of a counted batch on its slot's stream: totals, per-vertex counts (into pinned
// staging, or straight into the callers' memory), then the slot's done event.
int enqueue_readback(ktri_server* s, Slot& sl) {
    (void)s;
    char* d = static_cast<char*>(sl.dev);
    char* h = static_cast<char*>(sl.host);
    cudaStream_t st = sl.stream;
    const u64 k = sl.reqs.size(), n = sl.n_total;
    copy_staging(sl, h + sl.h_tot, d + sl.off_tot, 8 * k, false, st);
    if (sl.direct) {
        const u64 warps = (n + 255) / 256;
        const unsigned blocks = (unsigned)std::max<u64>(1, std::min<u64>((warps + 7) / 8, 152 * 16));
        k_scatter_pv<<<blocks, 256, 0, st>>>(reinterpret_cast<const GraphSrc*>(d + sl.off_src),
                                             reinterpret_cast<const u64*>(d + sl.off_vf), k, n,
                                             reinterpret_cast<const u64*>(d + sl.off_pv));
    } else {
        copy_staging(sl, h + sl.h_pv, d + sl.off_pv, 8 * n, false, st);
    }
    cudaEventRecord(sl.done, st);
    return cudaGetLastError() == cudaSuccess ? KTRI_OK : KTRI_ERR_CUDA;
}

// The engine has counted this slot's batch: per-graph totals from the per-vertex counts, then
// the read-back.
int finish_engine_batch(ktri_server* s, Slot& sl) {
    char* d = static_cast<char*>(sl.dev);
    ktri::launch_graph_totals(reinterpret_cast<const u64*>(d + sl.off_pv), reinterpret_cast<const u64*>(d + sl.off_vf),
                              sl.reqs.size(), sl.n_total, reinterpret_cast<u64*>(d + sl.off_tot), sl.ctl,
                              ktri::ctx_num_sms(sl.ctx), sl.stream);
    return enqueue_readback(s, sl);
}

// Pack the slot's requests and launch their count.  Called without the lock.
int launch_batch(ktri_server* s, Slot& sl) {
    const u64 k = sl.reqs.size();
    u64 n = 0, nnz = 0;
    for (Request* r : sl.reqs) {
        n += r->n;
        nnz += r->nnz;
    }
    sl.n_total = n;
    sl.nnz_total = nnz;
    sl.direct = s->pageable && s->opts.direct_host_access;
    const SlotLayout L = slot_layout(n, nnz, k, sl.direct);
    sl.off_fo = L.fo;
    sl.off_head = L.head;
    sl.off_vf = L.vf;
    sl.off_ef = L.ef;
    sl.off_tot = L.tot;
    sl.off_pv = L.pv;
    sl.off_src = L.src;
    int rc = grow(s, &sl.dev, &sl.dev_bytes, L.dev_bytes, false);
    if (rc) return rc;
    const size_t h_fo = L.h_fo, h_head = L.h_head, h_vf = L.h_vf, h_ef = L.h_ef, h_src = L.h_src;
    sl.h_tot = L.h_tot;
    sl.h_pv = L.h_pv;
    rc = grow(s, &sl.host, &sl.host_bytes, L.host_bytes, true);
    if (rc) return rc;
    char* h = static_cast<char*>(sl.host);
    u64* hvf = reinterpret_cast<u64*>(h + h_vf);
    u64* hef = reinterpret_cast<u64*>(h + h_ef);
    auto* hsrc = reinterpret_cast<GraphSrc*>(h + h_src);
    u64 vb = 0, eb = 0;
    for (u64 i = 0; i < k; ++i) {
        Request* r = sl.reqs[i];
        hvf[i] = vb;
        hef[i] = eb;
        vb += r->n;
        eb += r->nnz;
        r->pv_written = false;
        if (sl.direct) {
            if (r->pv_wanted && r->n) {
                r->pv = std::make_shared<std::vector<uint64_t>>(r->n);
                r->pv_written = true;
            }
            hsrc[i].fo = reinterpret_cast<const u64*>(r->bfo);
            hsrc[i].head = r->bhead;
            hsrc[i].pv_out = r->pv_written ? reinterpret_cast<u64*>(r->pv->data()) : nullptr;
        }
    }
    hvf[k] = vb;
    hef[k] = eb;
    char* d = static_cast<char*>(sl.dev);
    cudaStream_t st = sl.stream;
    cudaStreamWaitEvent(st, sl.cache_done, 0);  // earlier resident copies read these buffers
    cudaEventRecord(sl.start, st);
    auto* dfo = reinterpret_cast<u64*>(d + sl.off_fo);
    auto* dhead = reinterpret_cast<u32*>(d + sl.off_head);
    auto* dvf = reinterpret_cast<u64*>(d + sl.off_vf);
    auto* def = reinterpret_cast<u64*>(d + sl.off_ef);
    auto* dsrc = reinterpret_cast<GraphSrc*>(d + sl.off_src);
    copy_staging(sl, dvf, hvf, 8 * (k + 1), true, st);
    copy_staging(sl, def, hef, 8 * (k + 1), true, st);
    if (sl.direct) {
        copy_staging(sl, dsrc, hsrc, sizeof(GraphSrc) * k, true, st);
        const u64 warps = (std::max<u64>(n, nnz) + 255) / 256;
        const unsigned blocks = (unsigned)std::max<u64>(1, std::min<u64>((warps + 7) / 8, 152 * 16));
        k_gather<<<blocks, 256, 0, st>>>(dsrc, dvf, def, k, n, nnz, dfo, dhead);
    } else {
        u64* hfo = reinterpret_cast<u64*>(h + h_fo);
        u32* hhead = reinterpret_cast<u32*>(h + h_head);
        hfo[0] = 0;
        // pack the graphs into pinned staging in parallel, in pieces of at most 4 MiB so that a
        // large graph is copied by many threads (one host thread copies only ~13 GB/s); ids
        // are rebased on the device.  (Copying large graphs straight from the callers' pageable
        // arrays with the copy engines measured slower on Grace + Blackwell: the worker thread
        // blocks in each copy.)
        struct Piece {
            char* dst;
            const char* src;
            size_t bytes;
        };
        std::vector<Piece> pieces;
        constexpr size_t PIECE = 4u << 20;
        auto add = [&](void* dst, const void* src, size_t bytes) {
            for (size_t o = 0; o < bytes; o += PIECE)
                pieces.push_back({static_cast<char*>(dst) + o, static_cast<const char*>(src) + o,
                                  std::min(PIECE, bytes - o)});
        };
        for (u64 i = 0; i < k; ++i) {
            const Request* r = sl.reqs[i];
            add(hfo + hvf[i] + 1, r->bfo + 1, 8 * r->n);
            if (r->nnz) add(hhead + hef[i], r->bhead, 4 * r->nnz);
        }
#pragma omp parallel for schedule(dynamic, 1) if (pieces.size() > 1 && nnz > (1u << 16))
        for (int64_t p = 0; p < (int64_t)pieces.size(); ++p)
            std::memcpy(pieces[(size_t)p].dst, pieces[(size_t)p].src, pieces[(size_t)p].bytes);
        copy_staging(sl, dfo, hfo, 8 * (n + 1), true, st);
        copy_staging(sl, dhead, hhead, 4 * nnz, true, st);
        const u64 warps = (std::max<u64>(n, nnz) + 255) / 256;
        const unsigned blocks = (unsigned)std::max<u64>(1, std::min<u64>((warps + 7) / 8, 152 * 16));
        k_rebase<<<blocks, 256, 0, st>>>(dfo, dhead, dvf, def, k, n, nnz);
    }
    if (cudaGetLastError() != cudaSuccess) return KTRI_ERR_CUDA;
    if (s->engine && n > 0) {
        // prepare on this slot and publish to the engine; the read-back follows its completion
        const size_t j = slot_index(s, sl);
        sl.seq = s->seq_next++;
        rc = ktri::engine_prepare_batch(sl.ctx, reinterpret_cast<const uint64_t*>(dfo), dhead, n, nnz,
                                        reinterpret_cast<uint64_t*>(d + sl.off_pv), st, s->jobs + j, sl.seq,
                                        s->done_dev + j, &sl.ctl);
        if (rc == KTRI_OK) {
            sl.counting = true;
            sl.t_published = now_s();
            return ensure_engine(s);
        }
        if (rc != KTRI_ERR_UNSUPPORTED) return rc;
        // a batch beyond the engine's 32-bit descriptors: its own launch sequence below
    }
    ktri_opts o{};
    o.struct_size = sizeof(ktri_opts);
    o.intersection_method = KTRI_METHOD_AUTO;
    rc = ktri_count_batch_device(sl.ctx, reinterpret_cast<const uint64_t*>(dfo), dhead, n, nnz,
                                 reinterpret_cast<const uint64_t*>(dvf), k, reinterpret_cast<uint64_t*>(d + sl.off_tot),
                                 reinterpret_cast<uint64_t*>(d + sl.off_pv), &o, st);
    if (rc) return rc;
    return enqueue_readback(s, sl);
}

// Harvest a finished slot (called with the lock held).
void harvest(ktri_server* s, Slot& sl) {
    const double t0 = now_s();
    float dev_ms = 0;
    if (cudaEventElapsedTime(&dev_ms, sl.start, sl.done) == cudaSuccess) s->st.device_us += (u64)(dev_ms * 1e3);
    cudaGetLastError();
    int rc = ktri_ctx_check(sl.ctx);
    const char* h = static_cast<const char*>(sl.host);
    const u64* tot = reinterpret_cast<const u64*>(h + sl.h_tot);
    const u64* pv = reinterpret_cast<const u64*>(h + sl.h_pv);
    size_t inflight = 0;
    for (const Slot& o : s->slots) inflight += o.dev_bytes;
    const int64_t k = (int64_t)sl.reqs.size();
    if (rc == KTRI_OK && !sl.direct) {
        // per-vertex counts out of the pinned read-back, one request per host thread
        std::vector<u64> vfirst((size_t)k);
        u64 v = 0, pv_bytes = 0;
        for (int64_t i = 0; i < k; ++i) {
            vfirst[(size_t)i] = v;
            v += sl.reqs[(size_t)i]->n;
            if (sl.reqs[(size_t)i]->want_pv || sl.reqs[(size_t)i]->follower_pv) pv_bytes += 8 * sl.reqs[(size_t)i]->n;
        }
#pragma omp parallel for schedule(dynamic, 1) if (k > 1 && pv_bytes > (4u << 20))
        for (int64_t i = 0; i < k; ++i) {
            Request* r = sl.reqs[(size_t)i];
            if (r->want_pv || r->follower_pv)
                r->pv = std::make_shared<std::vector<uint64_t>>(pv + vfirst[(size_t)i], pv + vfirst[(size_t)i] + r->n);
        }
    }
    u64 vb = 0, eb = 0;
    for (int64_t i = 0; i < k; ++i) {
        Request* r = sl.reqs[(size_t)i];
        if (rc == KTRI_OK) {
            r->total = tot[i];
            // a follower that asked for counts after a direct batch started: read them back now
            if (sl.direct && (r->want_pv || r->follower_pv) && !r->pv_written && r->n) {
                r->pv = std::make_shared<std::vector<uint64_t>>(r->n);
                cudaMemcpy(r->pv->data(), static_cast<const char*>(sl.dev) + sl.off_pv + 8 * vb, 8 * r->n,
                           cudaMemcpyDeviceToHost);
            }
            keep_resident(s, r, sl, vb, eb, inflight);
        }
        vb += r->n;
        eb += r->nnz;
        finish(s, r, rc);
        r->fo.clear();
        r->fo.shrink_to_fit();
        r->head.clear();
        r->head.shrink_to_fit();
    }
    cudaEventRecord(sl.cache_done, s->aux);
    sl.reqs.clear();
    sl.busy = false;
    s->st.harvest_us += (u64)((now_s() - t0) * 1e6);
}

void worker_main(ktri_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->mu);
    while (true) {
        // batches the engine has counted: read them back
        bool any_counting = false;
        for (Slot& sl : s->slots) {
            if (!(sl.busy && sl.counting)) continue;
            const size_t j = slot_index(s, sl);
            if (*(volatile unsigned long long*)(s->done_host + j) == sl.seq) {
                sl.counting = false;
                if (finish_engine_batch(s, sl) != KTRI_OK) {
                    for (Request* r : sl.reqs) finish(s, r, KTRI_ERR_CUDA);
                    sl.reqs.clear();
                    sl.busy = false;
                    s->cv_done.notify_all();
                }
            } else {
                any_counting = true;
            }
        }
        // a published job needs a running engine (one that was leaving as it was published
        // is followed by a new launch)
        if (any_counting && ensure_engine(s) != KTRI_OK) {
            // the engine could not run: its batches fail (a device error is sticky, so the
            // buffers are not reused by anything that could still run)
            for (Slot& sl : s->slots) {
                if (!(sl.busy && sl.counting)) continue;
                for (Request* r : sl.reqs) finish(s, r, KTRI_ERR_CUDA);
                sl.reqs.clear();
                sl.counting = false;
                sl.busy = false;
            }
            s->cv_done.notify_all();
        }
        // finished batches
        bool any_busy = false;
        for (Slot& sl : s->slots) {
            if (sl.busy && !sl.counting && cudaEventQuery(sl.done) == cudaSuccess) {
                harvest(s, sl);
                s->cv_done.notify_all();
            }
            any_busy |= sl.busy;
        }
        if (s->stop && s->pending.empty() && s->hits.empty() && !any_busy) break;
        // requests for keys that were resident when submitted are answered at once (a graph of
        // another size under the key, or a key evicted since, is counted if its CSR came along)
        while (!s->hits.empty()) {
            Request* r = s->hits.front();
            s->hits.pop_front();
            auto res = s->resident.find(r->key);
            if (res != s->resident.end() && r->n == res->second.n && (!r->bfo || r->nnz == res->second.nnz)) {
                r->nnz = res->second.nnz;
                serve_resident(s, r, res->second);
                finish(s, r, KTRI_OK);
            } else if (r->bfo) {
                s->pending.push_back(r);
                continue;
            } else {  // a repeat by key of a graph that is no longer resident, or of another size
                finish(s, r, KTRI_ERR_INVALID_ARGUMENT);
            }
            s->cv_done.notify_all();
        }
        // admit a batch into a free slot
        Slot* free_slot = nullptr;
        for (Slot& sl : s->slots)
            if (!sl.busy) {
                free_slot = &sl;
                break;
            }
        if (free_slot && !s->pending.empty()) {
            std::vector<Request*> batch;
            u64 n = 0, nnz = 0;
            size_t inflight = 0;
            for (const Slot& o : s->slots)
                if (&o != free_slot) inflight += o.dev_bytes;
            while (!s->pending.empty() && batch.size() < s->opts.max_batch_graphs) {
                Request* r = s->pending.front();
                const u64 n2 = n + r->n, nnz2 = nnz + r->nnz;
                if (!batch.empty() && (nnz2 > s->opts.max_batch_nnz || n2 > 0x7FFFFFFFull)) break;
                if (!batch.empty() && batch_bytes(n2, nnz2, batch.size() + 1) + inflight + s->resident_bytes >
                                          s->opts.memory_budget)
                    break;
                batch.push_back(r);
                s->pending.pop_front();
                n = n2;
                nnz = nnz2;
            }
            const size_t need = batch_bytes(n, nnz, batch.size());
            make_room(s, need > free_slot->dev_bytes ? need - free_slot->dev_bytes : 0, inflight + free_slot->dev_bytes);
            if (need + inflight > s->opts.memory_budget || n > 0xFFFFFFFFull) {
                for (Request* r : batch) finish(s, r, KTRI_ERR_OUT_OF_MEMORY);
                s->cv_done.notify_all();
            } else {
                for (Request* r : batch) r->pv_wanted = r->want_pv || r->follower_pv;
                free_slot->reqs = batch;
                free_slot->busy = true;
                s->st.batches++;
                s->st.batched_graphs += batch.size();
                lock.unlock();
                const double t0 = now_s();
                const int rc = launch_batch(s, *free_slot);
                const double t1 = now_s();
                lock.lock();
                s->st.pack_us += (u64)((t1 - t0) * 1e6);
                s->st.alloc_us += (u64)(s->alloc_s_acc * 1e6);
                s->alloc_s_acc = 0;
                if (rc) {
                    cudaStreamSynchronize(free_slot->stream);
                    for (Request* r : free_slot->reqs) finish(s, r, rc);
                    free_slot->reqs.clear();
                    free_slot->busy = false;
                    s->cv_done.notify_all();
                }
                u64 busy = 0;
                for (const Slot& o : s->slots) busy += o.busy;
                s->st.peak_inflight_batches = std::max<u64>(s->st.peak_inflight_batches, busy);
            }
            continue;
        }
        // nothing to start: wait briefly for new requests or a finishing batch
        s->cv_work.wait_for(lock, std::chrono::microseconds(any_busy ? 50 : 2000));
    }
}

// first_out[0..n] is non-decreasing.  Blocks of offsets are tested without early exits (a loop
// the compiler vectorises), the blocks of a large graph by several threads: a submit checks
// every offset of its graph, which for the largest graphs of a stream costs more than the rest
// of the request.
bool offsets_nondecreasing(const uint64_t* fo, uint64_t n) {
    constexpr uint64_t BLK = uint64_t(1) << 14;
    const int64_t blocks = (int64_t)((n + BLK - 1) / BLK);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad) if (n >= (uint64_t(1) << 18))
    for (int64_t b = 0; b < blocks; ++b) {
        const uint64_t v0 = (uint64_t)b * BLK, v1 = std::min(n, v0 + BLK);
        int acc = 0;
        for (uint64_t v = v0; v < v1; ++v) acc |= fo[v + 1] < fo[v] ? 1 : 0;
        bad |= acc;
    }
    return bad == 0;
}

// Copy of a request's per-vertex counts into the caller's buffer, in 4 MiB pieces by several
// threads for a large graph.
void copy_counts(uint64_t* dst, const uint64_t* src, uint64_t n) {
    constexpr size_t PIECE = size_t(4) << 20;
    const size_t bytes = 8 * n;
    const int64_t pieces = (int64_t)((bytes + PIECE - 1) / PIECE);
#pragma omp parallel for schedule(static) if (pieces > 1)
    for (int64_t p = 0; p < pieces; ++p) {
        const size_t o = (size_t)p * PIECE;
        std::memcpy(reinterpret_cast<char*>(dst) + o, reinterpret_cast<const char*>(src) + o, std::min(PIECE, bytes - o));
    }
}

}  // namespace

extern "C" {

int ktri_server_create(int device, const ktri_server_opts* opts, ktri_server** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
        cudaGetLastError();
        return KTRI_ERR_NO_DEVICE;
    }
    ktri_server* s = new (std::nothrow) ktri_server();
    if (!s) return KTRI_ERR_OUT_OF_MEMORY;
    s->device = device;
    s->opts.struct_size = sizeof(ktri_server_opts);
    s->opts.slots = 2;
    s->opts.memory_budget = 120ull << 30;
    s->opts.max_batch_nnz = 1ull << 28;
    s->opts.max_batch_graphs = 4096;
    if (opts && opts->struct_size) {
        if (opts->slots) s->opts.slots = opts->slots;
        if (opts->memory_budget) s->opts.memory_budget = opts->memory_budget;
        if (opts->max_batch_nnz) s->opts.max_batch_nnz = opts->max_batch_nnz;
        if (opts->max_batch_graphs) s->opts.max_batch_graphs = opts->max_batch_graphs;
        s->opts.direct_host_access = opts->direct_host_access;
        s->opts.engine = opts->engine;
    }
    s->engine = s->opts.engine == 1;
    if (s->opts.slots > 8) s->opts.slots = 8;
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    s->pageable = pageable == 1;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    s->slots.resize(s->opts.slots);
    int rc = KTRI_OK;
    for (Slot& sl : s->slots) {
        rc = ktri_ctx_create(device, &sl.ctx);
        if (rc) break;
        cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        cudaEventCreate(&sl.start);
        cudaEventCreate(&sl.done);
        cudaEventCreateWithFlags(&sl.cache_done, cudaEventDisableTiming);
    }
    cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking);
    if (rc == KTRI_OK && s->engine) {
        // job records (zero: nothing published), the host-mapped completion words, the stop word
        // and the highest-priority stream that sets it while the engine runs
        void* hp = nullptr;
        int least_prio = 0, greatest_prio = 0;
        if (cudaMalloc(&s->jobs, sizeof(ktri::EngineJob) * s->slots.size()) != cudaSuccess ||
            cudaMalloc(&s->stop_dev, sizeof(unsigned)) != cudaSuccess ||
            cudaHostAlloc(&hp, sizeof(unsigned long long) * s->slots.size(), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->done_dev), hp, 0) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s->engine_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio) != cudaSuccess ||
            cudaStreamCreateWithPriority(&s->control_stream, cudaStreamNonBlocking, greatest_prio) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->engine_done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            rc = KTRI_ERR_CUDA;
        } else {
            s->done_host = static_cast<unsigned long long*>(hp);
            std::memset(s->done_host, 0, sizeof(unsigned long long) * s->slots.size());
            cudaMemset(s->jobs, 0, sizeof(ktri::EngineJob) * s->slots.size());
            cudaMemset(s->stop_dev, 0, sizeof(unsigned));
            s->engine_grid = ktri::engine_grid(ktri::ctx_num_sms(s->slots[0].ctx));
            if (cudaDeviceSynchronize() != cudaSuccess) rc = KTRI_ERR_CUDA;
        }
    }
    if (rc == KTRI_OK) {
        // Reserve every slot's union buffer and pinned staging for a full batch (max_batch_nnz
        // entries over max_batch_nnz / 8 vertices) when all slots together take at most a
        // quarter of the memory budget: the first large batches then find their buffers ready
        // instead of growing them (a device synchronisation and a pinned allocation each) while
        // requests wait.  Batches with more vertices still grow them.
        const u64 nnz_r = s->opts.max_batch_nnz, n_r = nnz_r / 8;
        const SlotLayout R = slot_layout(n_r, nnz_r, s->opts.max_batch_graphs, s->pageable && s->opts.direct_host_access);
        if ((R.dev_bytes + R.dev_bytes / 4) * s->slots.size() <= s->opts.memory_budget / 4) {
            for (Slot& sl : s->slots)
                if (grow(s, &sl.dev, &sl.dev_bytes, R.dev_bytes, false) != KTRI_OK ||
                    grow(s, &sl.host, &sl.host_bytes, R.host_bytes, true) != KTRI_OK)
                    break;  // not fatal: batches grow the buffers as they need them
        }
        s->alloc_s_acc = 0;  // set-up time is not the requests' allocation time
    }
    cudaSetDevice(prev);
    if (rc) {
        for (Slot& sl : s->slots)
            if (sl.ctx) ktri_ctx_destroy(sl.ctx);
        release_engine(s);
        delete s;
        return rc;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return KTRI_OK;
}

int ktri_server_submit(ktri_server* s, uint64_t graph_key, const uint64_t* first_out, const uint32_t* head,
                       uint64_t n, uint64_t nnz, uint32_t flags, uint64_t* request_id) {
    if (!s || !request_id) return KTRI_ERR_INVALID_ARGUMENT;
    auto r = std::make_unique<Request>();
    r->key = graph_key;
    r->want_pv = (flags & KTRI_SUBMIT_PER_VERTEX) != 0;
    if (first_out) {
        if (n > 0x7FFFFFFFull) return KTRI_ERR_UNSUPPORTED;
        if (first_out[0] != 0 || first_out[n] != nnz || (nnz && !head)) return KTRI_ERR_INVALID_CSR;
        if (!offsets_nondecreasing(first_out, n)) return KTRI_ERR_INVALID_CSR;
        r->n = n;
        r->nnz = nnz;
        if (flags & KTRI_SUBMIT_BORROW) {
            r->bfo = first_out;
            r->bhead = head;
        } else {
            r->fo.assign(first_out, first_out + n + 1);
            r->head.assign(head, head + nnz);
            r->bfo = r->fo.data();
            r->bhead = r->head.data();
        }
    } else if (!graph_key) {
        return KTRI_ERR_INVALID_ARGUMENT;  // a repeat by key needs a key
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return KTRI_ERR_INVALID_ARGUMENT;
    const bool resident = graph_key && s->resident.count(graph_key);
    auto lead = graph_key && !resident ? s->leaders.find(graph_key) : s->leaders.end();
    // a request for a key that is queued or counting joins that count (same graph size only)
    // (a repeat without a CSR may name the vertex count it expects in n: 0 takes any)
    if (lead != s->leaders.end() && (!first_out ? (n == 0 || lead->second->n == n)
                                                : (lead->second->n == n && lead->second->nnz == nnz))) {
        Request* l = lead->second;
        r->n = l->n;
        r->nnz = l->nnz;
        r->fo.clear();
        r->head.clear();
        r->bfo = nullptr;
        r->bhead = nullptr;
        r->id = s->next_id++;
        r->t_submit = now_s();
        *request_id = r->id;
        l->follower_pv |= r->want_pv;
        l->followers.push_back(r.get());
        s->requests.emplace(r->id, std::move(r));
        s->st.submitted++;
        s->st.coalesced++;
        return KTRI_OK;
    }
    if (!first_out && !resident) return KTRI_ERR_INVALID_ARGUMENT;
    if (!first_out) {
        const Resident& res = s->resident.at(graph_key);
        r->n = n ? n : res.n;  // checked against the resident graph when the worker answers
        r->nnz = res.nnz;
    }
    r->id = s->next_id++;
    r->t_submit = now_s();
    *request_id = r->id;
    if (graph_key && !resident && lead == s->leaders.end()) s->leaders[graph_key] = r.get();
    (resident ? s->hits : s->pending).push_back(r.get());
    s->requests.emplace(r->id, std::move(r));
    s->st.submitted++;
    s->cv_work.notify_one();
    return KTRI_OK;
}

int ktri_server_wait(ktri_server* s, uint64_t request_id, uint64_t* total, uint64_t* per_vertex_out,
                     double* latency_s) {
    if (!s) return KTRI_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        auto it = s->requests.find(request_id);
        if (it == s->requests.end()) return KTRI_ERR_INVALID_ARGUMENT;
        Request* p = it->second.get();
        s->cv_done.wait(lock, [&] { return p->done; });
        r = std::move(it->second);
        s->requests.erase(it);
    }
    // The worker finished with the request before marking it done (under the lock), so its
    // counts are read back without holding the lock: large copies do not stall the worker.
    const int status = r->status;
    if (status == KTRI_OK) {
        if (total) *total = r->total;
        if (per_vertex_out && r->want_pv && r->n) {
            if (r->pv) copy_counts(per_vertex_out, r->pv->data(), r->n);
            else std::memset(per_vertex_out, 0, 8 * r->n);
        }
    }
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    return status;
}

int ktri_server_get_stats(ktri_server* s, ktri_server_stats* out) {
    if (!s || !out) return KTRI_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->st;
    out->resident_graphs = s->resident.size();
    out->resident_bytes = s->resident_bytes;
    return KTRI_OK;
}

int ktri_server_destroy(ktri_server* s) {
    if (!s) return KTRI_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    release_engine(s);
    for (auto& kv : s->resident) cudaFreeAsync(kv.second.mem, s->aux);
    cudaStreamSynchronize(s->aux);
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.ctx) ktri_ctx_destroy(sl.ctx);  // before the stream it last ran on goes away
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.start) cudaEventDestroy(sl.start);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.cache_done) cudaEventDestroy(sl.cache_done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (s->aux) cudaStreamDestroy(s->aux);
    cudaSetDevice(prev);
    delete s;
    return KTRI_OK;
}

}  // extern "C"
