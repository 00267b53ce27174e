// C ABI: contexts, workspace management and the counting entry points.
#include <cuda.h>
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "ktri.h"
#include "ktri_device.cuh"
#include "ktri_internal.h"
#include "ktri_kernels.h"

using ktri::Control;
using ktri::u32;
using ktri::u64;

struct ktri_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;  // stream of the host-buffer entry points
    int pageable_access = 0;        // kernels may address pageable host memory
    void* readback = nullptr;       // grow-only pinned staging of large read-backs into pageable memory
    size_t readback_bytes = 0;
    void* ws = nullptr;             // grow-only device workspace
    size_t ws_bytes = 0;
    uint64_t budget = 0;
    std::string last_error;
    ktri_run_stats stats{};
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // host-buffer calls: a second stream for the chunked head copy, one event per chunk, and
    // events around the whole copy-in (ev_io[0..1]) and the read-back (ev_io[2..3])
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> chunk_ev;
    cudaEvent_t ev_io[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t ev_free = nullptr;  // marks earlier work on the stream before the chunked copies
    bool have_io = false;
    cudaStream_t last_stream = nullptr;
    Control* ctl = nullptr;
    bool pending = false;      // a device call whose status has not been read yet
    bool have_events = false;
    int32_t last_method = KTRI_METHOD_AUTO;
    bool last_collect = false;
};

namespace {

constexpr size_t ALIGN = 256;
inline size_t align_up(size_t x) { return (x + ALIGN - 1) & ~(ALIGN - 1); }

struct Layout {
    size_t ctl = 0, deg = 0, dplus = 0, tile_i0 = 0, vdesc = 0, headp = 0, ltiles = 0, thist = 0, tkeys = 0,
           spanning = 0,
           partials = 0, cnt = 0,
           total = 0, mid = 0, big = 0, scratch = 0, in_fo = 0, in_head = 0, bytes = 0;
    bool wide = false;
    u64 scratch_per_block = 0;
    int big_grid = 0;
    u32 npartials = 0;
};

u64 isqrt_ceil(u64 x) {
    u64 r = (u64)std::sqrt((double)x);
    while (r * r < x) ++r;
    while (r > 0 && (r - 1) * (r - 1) >= x) --r;
    return r;
}

// Workspace of one count.  num_sms = 0 sizes the grids for the largest supported part.
Layout make_layout(u64 n, u64 nnz, int32_t method, int num_sms, bool with_inputs, bool internal_cnt,
                   bool force_wide = false, u32 small_d = (u32)ktri::SMALL_D_LOW, u32 seg = ktri::LARGE_SEG) {
    Layout L;
    const u64 cap = ktri::oriented_capacity(n, nnz);
    L.wide = force_wide || cap > ktri::NARROW_CAPACITY;
    const int sms = num_sms > 0 ? num_sms : 160;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes);
        return at;
    };
    L.ctl = take(sizeof(Control));
    L.deg = take(sizeof(u32) * (n + 1));
    L.dplus = take(sizeof(u32) * (n + 1));
    L.vdesc = take((L.wide ? 16 : 8) * (n + 1));
    L.headp = take(sizeof(u32) * cap);
    L.spanning = take(sizeof(u32) * ktri::spanning_capacity(n, nnz));
    L.tile_i0 = take(sizeof(u32) * (ktri::base_tiles(n, nnz) + 2));
    u32 grid = 0;
    if (method == KTRI_METHOD_AUTO) {
        // medium- and large-owner tiles, and both reordered
        L.ltiles = take(sizeof(uint2) * 4 * ktri::large_tile_capacity(n, nnz, small_d, seg));
        L.thist = take(sizeof(u32) * ktri::tile_order_scratch_words());
        L.tkeys = take(sizeof(u32) * ktri::large_tile_capacity(n, nnz, small_d, seg));
        grid = (u32)(sms * 48);  // bound on the small + medium + large persistent grids (occupancy <= 16 each)
    } else {
        L.mid = take(sizeof(u32) * (n + 1));
        L.big = take(sizeof(u32) * (n + 1));
        u64 maxd = isqrt_ceil(nnz) + 1;
        u64 P = 1;
        while (P < maxd) P <<= 1;
        L.scratch_per_block = P;
        L.big_grid = sms;
        L.scratch = take(sizeof(u32) * P * (u64)sms);
        grid = (u32)ktri::count_grid_edges(sms);
    }
    L.npartials = grid;
    L.partials = take(sizeof(u64) * grid);
    if (internal_cnt) L.cnt = take(sizeof(u64) * (n + 1));
    L.total = take(sizeof(u64));
    if (with_inputs) {
        L.in_fo = take(sizeof(u64) * (n + 1));
        L.in_head = take(sizeof(u32) * (nnz + 1));
    }
    L.bytes = off;
    return L;
}

int set_error(ktri_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_fail(ktri_ctx* ctx, cudaError_t e, const char* what) {
    return set_error(ctx, e == cudaErrorMemoryAllocation ? KTRI_ERR_OUT_OF_MEMORY : KTRI_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

#define KTRI_CK(ctx, call)                                       \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

ktri::Options resolve(const ktri_opts* o) {
    ktri::Options r;
    if (!o || o->struct_size == 0) return r;
    r.method = o->intersection_method;
    if (o->small_outdegree) r.small_outdegree = o->small_outdegree;
    r.collect_stats = o->collect_stats != 0;
    if (o->binary_intersection_cutoff) r.binary_cutoff = o->binary_intersection_cutoff;
    if (o->hybrid_cutoff_scale > 0) r.hybrid_scale = o->hybrid_cutoff_scale;
    r.force_wide = o->force_wide_offsets != 0;
    if (o->medium_outdegree) r.medium_outdegree = o->medium_outdegree;
    if (o->segment) r.segment = o->segment;
    r.copy_wait_polls = o->copy_wait_polls;
    r.tile_order = o->tile_order;
    return r;
}

// Pieces of head copied at a time by the host-buffer entry points (graphs with at least two
// pieces of adjacency are copied in pieces, overlapping the orientation).
constexpr u64 HEAD_CHUNK_BYTES = u64(64) << 20;

int ensure_chunk_events(ktri_ctx* ctx, size_t count) {
    if (!ctx->copy_stream) {
        // the pieces of head are copied by kernels that run beside the orientation of the pieces
        // already in: the copy stream's blocks are dispatched first, so the copy keeps the link busy
        int least = 0, greatest = 0;
        KTRI_CK(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        KTRI_CK(ctx, cudaStreamCreateWithPriority(&ctx->copy_stream, cudaStreamNonBlocking, greatest));
    }
    while (ctx->chunk_ev.size() < count) {
        cudaEvent_t e = nullptr;
        KTRI_CK(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->chunk_ev.push_back(e);
    }
    return KTRI_OK;
}

int ensure_ws(ktri_ctx* ctx, size_t bytes) {
    if (ctx->budget && bytes > ctx->budget)
        return set_error(ctx, KTRI_ERR_OUT_OF_MEMORY,
                         "workspace of " + std::to_string(bytes) + " bytes exceeds the memory budget of " +
                             std::to_string(ctx->budget));
    if (bytes <= ctx->ws_bytes) return KTRI_OK;
    if (ctx->ws) {
        KTRI_CK(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->ws);  // waits for the work still using the old workspace
        ctx->ws = nullptr;
        ctx->ws_bytes = 0;
    }
    size_t grow = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&ctx->ws, grow);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&ctx->ws, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ctx->ws = nullptr;
            return cuda_fail(ctx, e, "cudaMalloc(workspace)");
        }
        grow = bytes;
    }
    ctx->ws_bytes = grow;
    return KTRI_OK;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// head arriving in pieces: chunk c holds adjacency slots [ends[c-1], ends[c]) and is on the
// device once events[c] has completed.  Orientation tiles run as soon as their slots are in.
struct HeadChunks {
    int count = 0;
    const u64* ends = nullptr;
    const cudaEvent_t* events = nullptr;
};

// Where a prepared batch goes instead of the counting kernels: an engine job slot.
struct EnginePublish {
    ktri::EngineJob* job = nullptr;
    unsigned long long seq = 0;
    unsigned long long* done_word = nullptr;  // device address of the host-mapped completion word
};

// The address under which the device reads or writes a caller's host buffer, or nullptr when
// only the copy engines reach it: pinned and registered memory through its device pointer,
// pageable memory directly where the platform lets kernels address it.
const void* device_view(const ktri_ctx* ctx, const void* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if (a.type == cudaMemoryTypeUnregistered && ctx->pageable_access) return host;
    return nullptr;
}

// Host -> device (to_device) or device -> host copy of a caller's buffer on stream st: by a
// kernel where the device can address the host side and both ends are 16-byte aligned (or the
// copy is at most 256 bytes), otherwise by the copy engines.  The kernel copies avoid the copy
// engines' recurring slow windows on this platform.
cudaError_t copy_host(ktri_ctx* ctx, void* dst, const void* src, size_t bytes, bool to_device, cudaStream_t st) {
    if (bytes == 0) return cudaSuccess;
    const void* view = device_view(ctx, to_device ? src : dst);
    if (view) {
        const void* from = to_device ? view : src;
        void* to = to_device ? dst : const_cast<void*>(view);
        if (ktri::launch_copy(from, to, bytes, ctx->num_sms, st)) return cudaGetLastError();
    }
    return cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, st);
}

// A read-back of at least this many bytes into pageable host memory goes through the
// context's pinned staging: written there by a kernel, then copied into the caller's buffer by
// host threads after the call's synchronisation.  Written straight into pageable memory that
// the caller has not touched yet, every 64 KiB page faults through the host's page tables
// (RMAT-24's 134 MB of per-vertex counts: 40 ms against 0.8 ms into touched pages).
constexpr size_t READBACK_STAGE_BYTES = size_t(1) << 20;

// Enqueue the device -> host copy of `bytes` from src to the caller's dst on st.  Returns
// true when the copy went to the pinned staging and must be finished by finish_readback
// after the stream has been synchronised.
bool start_readback(ktri_ctx* ctx, void* dst, const void* src, size_t bytes, cudaStream_t st, cudaError_t* err) {
    *err = cudaSuccess;
    if (bytes >= READBACK_STAGE_BYTES) {
        cudaPointerAttributes a{};
        const bool pageable = cudaPointerGetAttributes(&a, dst) == cudaSuccess && a.type == cudaMemoryTypeUnregistered;
        cudaGetLastError();
        if (pageable) {
            if (ctx->readback_bytes < bytes) {
                if (ctx->readback) cudaFreeHost(ctx->readback);  // waits for the copies still using it
                ctx->readback = nullptr;
                ctx->readback_bytes = 0;
                if (cudaHostAlloc(&ctx->readback, bytes, cudaHostAllocDefault) == cudaSuccess) {
                    ctx->readback_bytes = bytes;
                } else {
                    ctx->readback = nullptr;
                    cudaGetLastError();
                }
            }
            if (ctx->readback && ktri::launch_copy(src, ctx->readback, bytes, ctx->num_sms, st)) {
                *err = cudaGetLastError();
                return true;
            }
        }
    }
    *err = copy_host(ctx, dst, src, bytes, false, st);
    return false;
}

// Copy a staged read-back into the caller's buffer, in pieces on host threads.
void finish_readback(const ktri_ctx* ctx, void* dst, size_t bytes) {
    constexpr size_t PIECE = size_t(4) << 20;
    const int64_t pieces = (int64_t)((bytes + PIECE - 1) / PIECE);
    const char* src = static_cast<const char*>(ctx->readback);
#pragma omp parallel for schedule(static) if (pieces > 1)
    for (int64_t p = 0; p < pieces; ++p) {
        const size_t o = (size_t)p * PIECE;
        std::memcpy(static_cast<char*>(dst) + o, src + o, std::min(PIECE, bytes - o));
    }
}

// Polls of the large-owner kernel's first bulk-copy wait for an option value.
u32 first_wait_polls(uint32_t opt) {
    return opt == 0 ? ktri::COPY_WAIT_POLLS : (opt == KTRI_COPY_WAIT_NONE ? 0u : opt);
}

// The launch sequence of one count on the workspace at base.  ctx may be NULL (the
// no-allocation entry point): errors then carry no message and no events are recorded.
template <typename OffT>
int enqueue_pipeline(ktri_ctx* ctx, int sms, char* base, const Layout& L, const u64* fo, const u32* head, u64 n,
                     u64 nnz, u64* d_total, u64* cnt, const ktri::Options& opt, cudaStream_t st, bool sort_all,
                     bool events, ktri::TriangleSink sink = ktri::TriangleSink{}, const HeadChunks* chunks = nullptr,
                     const EnginePublish* publish = nullptr) {
    events = events && ctx;
    auto* ctl = reinterpret_cast<Control*>(base + L.ctl);
    auto* deg = reinterpret_cast<u32*>(base + L.deg);
    auto* dplus = reinterpret_cast<u32*>(base + L.dplus);
    void* vdesc = base + L.vdesc;
    auto* headp = reinterpret_cast<u32*>(base + L.headp);
    auto* spanning = reinterpret_cast<u32*>(base + L.spanning);
    auto* partials = reinterpret_cast<u64*>(base + L.partials);
    auto* tile_i0 = reinterpret_cast<u32*>(base + L.tile_i0);

    // an error a caller's own failed runtime call left in this thread must not be taken for a
    // failed launch of ours below (errors of kernels that faulted are sticky and stay visible)
    (void)cudaGetLastError();
    KTRI_CK(ctx, cudaMemsetAsync(ctl, 0, sizeof(Control), st));
    if (events) KTRI_CK(ctx, cudaEventRecord(ctx->ev[0], st));
    const bool autom = opt.method == KTRI_METHOD_AUTO && !sort_all;
    ktri::launch_prep(fo, n, nnz, deg, dplus, cnt, tile_i0, ctl, sms, st);
    if (!chunks) {
        ktri::launch_orient(fo, head, n, nnz, deg, tile_i0, headp, dplus, spanning, ctl, st);
    } else {
        // tile t reads slots below (t + 1) * ORIENT_TILE + 1: launch each tile once its slots are in
        u64 done = 0;
        for (int c = 0; c < chunks->count; ++c) {
            KTRI_CK(ctx, cudaStreamWaitEvent(st, chunks->events[c], 0));
            const u64 upto = c + 1 == chunks->count ? ktri::orient_tiles(n, nnz)
                                                    : (chunks->ends[c] - 1) / ktri::ORIENT_TILE;
            if (upto > done) {
                ktri::launch_orient(fo, head, n, nnz, deg, tile_i0, headp, dplus, spanning, ctl, st, done, upto);
                done = upto;
            }
        }
    }
    auto* mtiles = autom ? reinterpret_cast<uint2*>(base + L.ltiles) : nullptr;
    const u64 tcap = ktri::large_tile_capacity(n, nnz, opt.small_outdegree, opt.segment);
    auto* ltiles = autom ? mtiles + tcap : nullptr;
    ktri::launch_desc<OffT>(fo, n, dplus, vdesc, mtiles, ltiles, autom ? opt.small_outdegree : 0xFFFFFFFFu,
                            opt.medium_outdegree, opt.segment,
                            autom ? ktri::SMALL_WARP_DEG : 0xFFFFFFFFu, ctl, sms, st);
    // Tile orders (large tiles by the vertex range they stream, for L2 reuse; medium tiles
    // longest owner first, so the warps' last tiles are short).  Below 2^20 adjacency entries
    // everything fits L2 and the few tiles are not worth the four extra launches.
    const bool order = autom && nnz >= (1ull << 20);
    uint2* lrun = ltiles;
    uint2* mrun = mtiles;
    if (order) {
        lrun = ltiles + tcap;
        mrun = lrun + tcap;
        const bool by_cost = opt.tile_order == KTRI_TILE_ORDER_COST;
        auto* keys = reinterpret_cast<u32*>(base + L.tkeys);
        ktri::launch_order_tiles(fo, head, dplus, n, ltiles, &ctl->large_tiles, opt.segment,
                                 by_cost ? ktri::TILE_BY_COST : ktri::TILE_BY_VERTEX, keys,
                                 reinterpret_cast<u32*>(base + L.thist), lrun, ctl, sms, st);
        ktri::launch_order_tiles(fo, head, dplus, n, mtiles, &ctl->medium_tiles, opt.segment,
                                 by_cost ? ktri::TILE_BY_COST : ktri::TILE_BY_DEGREE, keys,
                                 reinterpret_cast<u32*>(base + L.thist), mrun, ctl, sms, st);
    }
    if (!autom) {
        ktri::launch_sort_lists<OffT>(n, vdesc, headp, reinterpret_cast<u32*>(base + L.mid),
                                      reinterpret_cast<u32*>(base + L.big), reinterpret_cast<u32*>(base + L.scratch),
                                      L.scratch_per_block, L.big_grid, ctl, sms, st);
    }
    if (events) KTRI_CK(ctx, cudaEventRecord(ctx->ev[1], st));
    if (opt.collect_stats)
        ktri::launch_stats<OffT>(fo, head, n, vdesc, headp, autom ? opt.medium_outdegree : 0xFFFFFFFFu, ctl, sms, st);
    if (events) KTRI_CK(ctx, cudaEventRecord(ctx->ev[2], st));
    if (sort_all) {
        // orientation export only: no counting
    } else if (autom && publish) {
        // the counting phase runs in the serving engine: publish the prepared batch as a job
        ktri::launch_publish(publish->job, publish->seq, fo, head, n, vdesc, headp, mrun, lrun, cnt, ctl,
                             opt.small_outdegree, opt.segment, publish->done_word, st);
    } else if (autom) {
        KTRI_CK(ctx, ktri::launch_count_auto<OffT>(fo, head, n, nnz, vdesc, headp, mrun, lrun, opt.small_outdegree,
                                                   opt.segment, cnt, partials, ctl, sms, st,
                                                   events ? ctx->ev[4] : nullptr, events ? ctx->ev[5] : nullptr,
                                                   first_wait_polls(opt.copy_wait_polls)));
        ktri::launch_final_auto<OffT>(partials, n, opt.small_outdegree, sms, d_total, ctl, st);
    } else {
        const int grid = ktri::count_grid_edges(sms);
        ktri::launch_count_edges<OffT>(n, vdesc, headp, opt.method, opt.binary_cutoff, opt.hybrid_scale, cnt, partials,
                                       grid, ctl, sink, st);
        ktri::launch_final(partials, (u32)grid, d_total, ctl, st);
    }
    if (events) KTRI_CK(ctx, cudaEventRecord(ctx->ev[3], st));
    KTRI_CK(ctx, cudaGetLastError());
    return KTRI_OK;
}

// Enqueue a count on the context's workspace and remember it for ktri_ctx_check / stats.
template <typename OffT>
int run_pipeline(ktri_ctx* ctx, const Layout& L, const u64* fo, const u32* head, u64 n, u64 nnz, u64* d_total,
                 u64* cnt, const ktri::Options& opt, cudaStream_t st, bool sort_all,
                 ktri::TriangleSink sink = ktri::TriangleSink{}, const HeadChunks* chunks = nullptr) {
    char* base = static_cast<char*>(ctx->ws);
    const int rc = enqueue_pipeline<OffT>(ctx, ctx->num_sms, base, L, fo, head, n, nnz, d_total, cnt, opt, st, sort_all,
                                          true, sink, chunks);
    if (rc) return rc;
    ctx->ctl = reinterpret_cast<Control*>(base + L.ctl);
    ctx->last_stream = st;
    ctx->pending = true;
    ctx->have_events = true;
    ctx->last_method = opt.method;
    ctx->last_collect = opt.collect_stats;
    ctx->have_io = false;
    ctx->stats = ktri_run_stats{};
    ctx->stats.n = n;
    ctx->stats.nnz = nnz;
    ctx->stats.method = (u32)opt.method;
    return KTRI_OK;
}

int check_common(ktri_ctx* ctx, const void* fo, const void* head, u64 n, u64 nnz, const void* total,
                 const ktri::Options& opt) {
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    if (!total) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "total output pointer is NULL");
    if (n > 0xFFFFFFFFull) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "n must be below 2^32 (u32 vertex ids)");
    if (n && !fo) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "first_out is NULL");
    if (nnz && !head) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "head is NULL");
    if (n == 0 && nnz != 0) return set_error(ctx, KTRI_ERR_INVALID_CSR, "nnz > 0 with n == 0");
    if (opt.method < KTRI_METHOD_AUTO || opt.method > KTRI_METHOD_HYBRID)
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "unknown intersection method");
    if (opt.small_outdegree < 1 || opt.small_outdegree > (u32)ktri::SMALL_D)
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "small_outdegree must be in 1..48");
    if (opt.medium_outdegree < opt.small_outdegree || opt.medium_outdegree > (u32)ktri::MEDIUM_D)
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "medium_outdegree must be in small_outdegree..256");
    if (opt.segment < ktri::MIN_SEG || opt.segment > ktri::LARGE_SEG || (opt.segment & (opt.segment - 1)))
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "segment must be a power of two in 64..1024");
    return KTRI_OK;
}

int device_status(ktri_ctx* ctx) {
    if (!ctx->pending) return KTRI_OK;
    // The context's own stream also carries the host entry points' read-backs; a caller's
    // stream is waited for through the end-of-call event (the stream may be gone by now).
    if (ctx->last_stream == ctx->stream) KTRI_CK(ctx, cudaStreamSynchronize(ctx->stream));
    else KTRI_CK(ctx, cudaEventSynchronize(ctx->ev[3]));
    Control h;
    KTRI_CK(ctx, cudaMemcpy(&h, ctx->ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    ctx->pending = false;
    ctx->stats.input_sorted = (h.err & ktri::DEV_FLAG_UNSORTED) ? 0 : 1;
    if (ctx->last_collect) {
        ctx->stats.wedge_checks = h.stat_wedge;
        ctx->stats.intersection_size_local = h.stat_isz;
        ctx->stats.streamed_entries = h.stat_streamed;
        ctx->stats.oriented_edges = h.stat_oriented;
        ctx->stats.streamed_chunked = h.stat_chunked;
    }
    if (ctx->have_events) {
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&b, ctx->ev[2], ctx->ev[3]);
        cudaEventElapsedTime(&c, ctx->ev[0], ctx->ev[3]);
        ctx->stats.ms_orient = a;
        ctx->stats.ms_count = b;
        ctx->stats.ms_total = c;
        if (ctx->last_method == KTRI_METHOD_AUTO) {
            float s1 = 0, s2 = 0;
            cudaEventElapsedTime(&s1, ctx->ev[2], ctx->ev[4]);
            cudaEventElapsedTime(&s2, ctx->ev[4], ctx->ev[5]);
            ctx->stats.ms_count_small = s1;
            ctx->stats.ms_count_large = s2;
        }
    }
    if (ctx->have_io) {
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, ctx->ev_io[0], ctx->ev_io[1]);
        cudaEventElapsedTime(&b, ctx->ev_io[2], ctx->ev_io[3]);
        cudaEventElapsedTime(&c, ctx->ev_io[0], ctx->ev_io[3]);
        ctx->stats.ms_h2d = a;
        ctx->stats.ms_d2h = b;
        ctx->stats.ms_call = c;
    }
    const u32 e = h.err & ktri::DEV_ERR_MASK;
    if (e & ktri::DEV_ERR_COPY_INFLIGHT)
        return set_error(ctx, KTRI_ERR_TIMEOUT, "a bulk copy into shared memory did not complete in time, not even "
                                                "after a second wait: it may still have been in flight when its block "
                                                "left, so treat the device state as suspect");
    if (e & ktri::DEV_ERR_TIMEOUT)
        return set_error(ctx, KTRI_ERR_TIMEOUT, "a bulk copy into shared memory did not complete in time");
    if (e & ktri::DEV_ERR_DEGREE)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out is not a valid offset array (non-monotone, "
                                                    "first_out[0] != 0, first_out[n] != nnz, or a degree >= 2^32)");
    if (e & ktri::DEV_ERR_ID_RANGE) return set_error(ctx, KTRI_ERR_INVALID_CSR, "adjacency entry >= n");
    if (e & ktri::DEV_ERR_SELF_LOOP) return set_error(ctx, KTRI_ERR_INVALID_CSR, "self-loop in the adjacency");
    if (e & ktri::DEV_ERR_DUPLICATE) return set_error(ctx, KTRI_ERR_INVALID_CSR, "duplicate adjacency entry");
    return KTRI_OK;
}

std::mutex g_default_mu;
std::map<int, ktri_ctx*> g_default;

// ---- counting without allocation --------------------------------------------------------
// Scratch of ktri_count_csr_device_noalloc: a fixed array in device memory that every GPU
// which loads this library holds until the process exits.  All calls on a device share it.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch.  The array lives in this library's module, which the
// CUDA runtime loads once per context, so the address is looked up (cudaGetSymbolAddress, with
// the device current) once per device and context and cached under the context's unique id.
// A new context on the same device (after cudaDeviceReset, or a driver-API caller that makes
// its own context current) gets a fresh lookup instead of a stale address.
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
struct NoallocSlot {
    unsigned long long ctx_id = 0;  // 0: no cached address
    void* ptr = nullptr;
};
NoallocSlot g_noalloc_slot[NOALLOC_MAX_DEVICES];

// Unique id of the calling thread's current CUDA context, through the driver entry points the
// runtime hands out (no link against the driver library); 0 when it cannot be read.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int noalloc_scratch(int device, void** out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return KTRI_ERR_NO_DEVICE;
    const unsigned long long id = current_context_id();
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSlot& slot = g_noalloc_slot[device];
    if (id == 0 || slot.ctx_id != id || !slot.ptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return KTRI_ERR_CUDA;
        }
        slot.ptr = p;
        // the lookup makes the device's context current if nothing had yet: key the address
        // by the context it belongs to (0, never matched, when the id cannot be read)
        slot.ctx_id = current_context_id();
    }
    *out = slot.ptr;
    return KTRI_OK;
}

// The AUTO pipeline of ktri_count_csr_device (the same launch sequence, default options) on
// the fixed scratch array.  enqueue_pipeline zeroes the control block; k_prep zeroes the
// out-degrees and per-vertex counts; every other region is fully written before it is read.
template <typename OffT>
int run_noalloc(char* base, const Layout& L, const u64* fo, const u32* head, u64 n, u64 nnz, u64* d_total, u64* cnt,
                int sms, cudaStream_t st) {
    const ktri::Options opt;  // AUTO, default owner bins and segment (the layout is sized for them)
    if (enqueue_pipeline<OffT>(nullptr, sms, base, L, fo, head, n, nnz, d_total, cnt, opt, st, false, false) !=
        KTRI_OK)
        return KTRI_ERR_CUDA;
    auto* ctl = reinterpret_cast<Control*>(base + L.ctl);
    u32 herr = 0;
    if (cudaMemcpyAsync(&herr, &ctl->err, sizeof(u32), cudaMemcpyDeviceToHost, st) != cudaSuccess) return KTRI_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return KTRI_ERR_CUDA;
    if (herr & ktri::DEV_ERR_TIMEOUT) return KTRI_ERR_TIMEOUT;
    return (herr & ktri::DEV_ERR_MASK) ? KTRI_ERR_INVALID_CSR : KTRI_OK;
}

}  // namespace

int ktri::ctx_device(const ktri_ctx* ctx) { return ctx->device; }

int ktri::ctx_num_sms(const ktri_ctx* ctx) { return ctx->num_sms; }

int ktri::engine_prepare_batch(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                               uint64_t nnz_total, uint64_t* d_per_vertex, void* stream, ktri::EngineJob* job,
                               unsigned long long seq, unsigned long long* done_word, ktri::Control** ctl_out) {
    ktri::Options opt;  // AUTO with the default bins and segment
    int rc = check_common(ctx, d_first_out, d_head, n_total, nnz_total, d_per_vertex, opt);
    if (rc) return rc;
    if (!d_per_vertex || !job || !done_word || n_total == 0) return KTRI_ERR_INVALID_ARGUMENT;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    const Layout L = make_layout(n_total, nnz_total, opt.method, ctx->num_sms, false, false, false,
                                 opt.small_outdegree, opt.segment);
    if (L.wide) return KTRI_ERR_UNSUPPORTED;  // the engine's jobs use 32-bit descriptors
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* base = static_cast<char*>(ctx->ws);
    EnginePublish pub;
    pub.job = job;
    pub.seq = seq;
    pub.done_word = done_word;
    rc = enqueue_pipeline<u32>(ctx, ctx->num_sms, base, L, reinterpret_cast<const u64*>(d_first_out), d_head, n_total,
                               nnz_total, reinterpret_cast<u64*>(base + L.total), reinterpret_cast<u64*>(d_per_vertex),
                               opt, st, false, false, ktri::TriangleSink{}, nullptr, &pub);
    if (rc) return rc;
    ctx->ctl = reinterpret_cast<Control*>(base + L.ctl);
    ctx->last_stream = st;
    ctx->pending = true;
    ctx->have_events = false;
    ctx->have_io = false;
    ctx->last_method = opt.method;
    ctx->last_collect = false;
    ctx->stats = ktri_run_stats{};
    ctx->stats.n = n_total;
    ctx->stats.nnz = nnz_total;
    *ctl_out = ctx->ctl;
    return KTRI_OK;
}

extern "C" {

const char* ktri_version(void) { return "katric_gb300 1.0 (sm_103a)"; }

int ktri_ctx_create(int device, ktri_ctx** out) {
    if (!out) return KTRI_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return KTRI_ERR_NO_DEVICE;
    }
    if (device < 0) cudaGetDevice(&device);
    if (device >= ndev) return KTRI_ERR_NO_DEVICE;
    ktri_ctx* ctx = new (std::nothrow) ktri_ctx();
    if (!ctx) return KTRI_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    DeviceGuard g(device);
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        ctx->pageable_access = 0;
        cudaGetLastError();
    }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return KTRI_ERR_CUDA;
    }
    for (auto& e : ctx->ev) cudaEventCreate(&e);
    for (auto& e : ctx->ev_io) cudaEventCreate(&e);
    cudaEventCreateWithFlags(&ctx->ev_free, cudaEventDisableTiming);
    *out = ctx;
    return KTRI_OK;
}

int ktri_ctx_destroy(ktri_ctx* ctx) {
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    {
        // The caller's streams are not touched here (one may already be destroyed); freeing the
        // workspace waits for the work still using it.
        DeviceGuard g(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        if (ctx->ws) cudaFree(ctx->ws);
        if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
        if (ctx->readback) cudaFreeHost(ctx->readback);
        for (auto& e : ctx->ev)
            if (e) cudaEventDestroy(e);
        for (auto& e : ctx->ev_io)
            if (e) cudaEventDestroy(e);
        for (auto e : ctx->chunk_ev) cudaEventDestroy(e);
        if (ctx->ev_free) cudaEventDestroy(ctx->ev_free);
        if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return KTRI_OK;
}

int ktri_ctx_set_memory_budget(ktri_ctx* ctx, uint64_t bytes) {
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    ctx->budget = bytes;
    return KTRI_OK;
}

uint64_t ktri_workspace_bytes(uint64_t n, uint64_t nnz, int32_t method) {
    return make_layout(n, nnz, method, 0, false, true).bytes;
}

const char* ktri_last_error(const ktri_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int ktri_ctx_stats(ktri_ctx* ctx, ktri_run_stats* out) {
    if (!ctx || !out) return KTRI_ERR_INVALID_ARGUMENT;
    DeviceGuard g(ctx->device);
    int rc = device_status(ctx);
    *out = ctx->stats;
    return rc;
}

int ktri_ctx_check(ktri_ctx* ctx) {
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    DeviceGuard g(ctx->device);
    return device_status(ctx);
}

int ktri_count_csr_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n,
                          uint64_t nnz, uint64_t* d_total, uint64_t* d_per_vertex, const ktri_opts* opts,
                          void* stream) {
    const ktri::Options opt = resolve(opts);
    int rc = check_common(ctx, d_first_out, d_head, n, nnz, d_total, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) {
        rc = device_status(ctx);
        (void)rc;  // the previous call's status was not collected; the new call proceeds
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        KTRI_CK(ctx, cudaMemsetAsync(d_total, 0, sizeof(u64), st));
        ctx->pending = false;
        ctx->stats = ktri_run_stats{};
        return KTRI_OK;
    }
    const Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, false, d_per_vertex == nullptr,
                                 opt.force_wide, opt.small_outdegree, opt.segment);
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    u64* cnt = d_per_vertex ? reinterpret_cast<u64*>(d_per_vertex)
                            : reinterpret_cast<u64*>(static_cast<char*>(ctx->ws) + L.cnt);
    auto* fo = reinterpret_cast<const u64*>(d_first_out);
    auto* tot = reinterpret_cast<u64*>(d_total);
    if (L.wide) return run_pipeline<u64>(ctx, L, fo, d_head, n, nnz, tot, cnt, opt, st, false);
    return run_pipeline<u32>(ctx, L, fo, d_head, n, nnz, tot, cnt, opt, st, false);
}

int ktri_count_csr_device_noalloc(const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n, uint64_t nnz,
                                  uint64_t* d_total, uint64_t* d_per_vertex, void* stream) {
    if (!d_total || !d_per_vertex || (n && !d_first_out) || (nnz && !d_head)) return KTRI_ERR_INVALID_ARGUMENT;
    if (n == 0 && nnz != 0) return KTRI_ERR_INVALID_CSR;
    if (n > 0x7FFFFFFFull) return KTRI_ERR_UNSUPPORTED;
    // the workspace must fit the fixed scratch array: checked before anything is launched
    // (the same layout ktri_workspace_bytes reports; its per-vertex count region goes unused)
    const Layout L = make_layout(n, nnz, KTRI_METHOD_AUTO, 0, false, true);
    if (L.bytes > NOALLOC_SCRATCH_BYTES) return KTRI_ERR_UNSUPPORTED;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return KTRI_ERR_NO_DEVICE;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        if (cudaMemsetAsync(d_total, 0, sizeof(u64), st) != cudaSuccess) return KTRI_ERR_CUDA;
        return cudaStreamSynchronize(st) == cudaSuccess ? KTRI_OK : KTRI_ERR_CUDA;
    }
    void* scratch = nullptr;
    int rc = noalloc_scratch(dev, &scratch);
    if (rc) return rc;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return KTRI_ERR_CUDA;
    if (sms > 160) return KTRI_ERR_UNSUPPORTED;  // the layout's partial-sum array is sized for 160 SMs
    char* base = static_cast<char*>(scratch);
    auto* fo = reinterpret_cast<const u64*>(d_first_out);
    auto* tot = reinterpret_cast<u64*>(d_total);
    auto* cnt = reinterpret_cast<u64*>(d_per_vertex);
    if (L.wide) return run_noalloc<u64>(base, L, fo, d_head, n, nnz, tot, cnt, sms, st);
    return run_noalloc<u32>(base, L, fo, d_head, n, nnz, tot, cnt, sms, st);
}

int ktri_count_csr_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                       uint64_t* total_out, uint64_t* per_vertex_out, const ktri_opts* opts) {
    const auto t_entry = std::chrono::steady_clock::now();
    const ktri::Options opt = resolve(opts);
    int rc = check_common(ctx, first_out, head, n, nnz, total_out, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    if (n == 0) {
        *total_out = 0;
        return KTRI_OK;
    }
    if (first_out[0] != 0 || first_out[n] != nnz)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz");
    const Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, true, true,
                                 opt.force_wide, opt.small_outdegree, opt.segment);
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, cudaEventRecord(ctx->ev_io[0], st));
    KTRI_CK(ctx, copy_host(ctx, d_fo, first_out, sizeof(u64) * (n + 1), true, st));
    // head in pieces on the copy stream; the orientation tiles of each piece start on the
    // counting stream as soon as it has landed, so the copy hides the orientation
    HeadChunks chunks;
    std::vector<u64> ends;
    const u64 head_bytes = sizeof(u32) * nnz;
    if (head_bytes >= 2 * HEAD_CHUNK_BYTES) {
        const u64 per = HEAD_CHUNK_BYTES / sizeof(u32);
        for (u64 e = per; e < nnz; e += per) ends.push_back(e);
        ends.push_back(nnz);
        rc = ensure_chunk_events(ctx, ends.size());
        if (rc) return rc;
        // the copies overwrite the workspace's input region: they wait for earlier work on st
        KTRI_CK(ctx, cudaEventRecord(ctx->ev_free, st));
        KTRI_CK(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_free, 0));
        u64 b = 0;
        for (size_t c = 0; c < ends.size(); ++c) {
            KTRI_CK(ctx, copy_host(ctx, d_head + b, head + b, sizeof(u32) * (ends[c] - b), true, ctx->copy_stream));
            KTRI_CK(ctx, cudaEventRecord(ctx->chunk_ev[c], ctx->copy_stream));
            b = ends[c];
        }
        KTRI_CK(ctx, cudaEventRecord(ctx->ev_io[1], ctx->copy_stream));
        chunks.count = (int)ends.size();
        chunks.ends = ends.data();
        chunks.events = ctx->chunk_ev.data();
    } else {
        if (nnz) KTRI_CK(ctx, copy_host(ctx, d_head, head, head_bytes, true, st));
        KTRI_CK(ctx, cudaEventRecord(ctx->ev_io[1], st));
    }
    rc = L.wide ? run_pipeline<u64>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false, {},
                                    chunks.count ? &chunks : nullptr)
                : run_pipeline<u32>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false, {},
                                    chunks.count ? &chunks : nullptr);
    if (rc) return rc;
    KTRI_CK(ctx, cudaEventRecord(ctx->ev_io[2], st));
    KTRI_CK(ctx, copy_host(ctx, total_out, d_total, sizeof(u64), false, st));
    bool staged = false;
    if (per_vertex_out) {
        cudaError_t e = cudaSuccess;
        staged = start_readback(ctx, per_vertex_out, d_cnt, sizeof(u64) * n, st, &e);
        KTRI_CK(ctx, e);
    }
    KTRI_CK(ctx, cudaEventRecord(ctx->ev_io[3], st));
    ctx->have_io = true;
    const auto t_enqueued = std::chrono::steady_clock::now();
    rc = device_status(ctx);
    if (rc == KTRI_OK) ctx->stats.triangles = *total_out;
    if (rc == KTRI_OK && staged) finish_readback(ctx, per_vertex_out, sizeof(u64) * n);
    const auto t_done = std::chrono::steady_clock::now();
    ctx->stats.host_ms_enqueue = std::chrono::duration<float, std::milli>(t_enqueued - t_entry).count();
    ctx->stats.host_ms_call = std::chrono::duration<float, std::milli>(t_done - t_entry).count();
    return rc;
}

int ktri_count_csr(const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz, uint64_t* total_out,
                   uint64_t* per_vertex_out, const ktri_opts* opts) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return KTRI_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_default_mu);
    ktri_ctx*& ctx = g_default[dev];
    if (!ctx) {
        int rc = ktri_ctx_create(dev, &ctx);
        if (rc) {
            ctx = nullptr;
            return rc;
        }
    }
    return ktri_count_csr_ctx(ctx, first_out, head, n, nnz, total_out, per_vertex_out, opts);
}

// ---- file ingest ---------------------------------------------------------------------------

int ktri_binary_file_shape(const char* stem, uint64_t* n_out, uint64_t* nnz_out) {
    if (!stem || !n_out || !nnz_out) return KTRI_ERR_INVALID_ARGUMENT;
    struct stat a, b;
    const std::string s(stem);
    if (stat((s + ".first_out").c_str(), &a) != 0 || stat((s + ".head").c_str(), &b) != 0) return KTRI_ERR_IO;
    if (a.st_size < 8 || a.st_size % 8 || b.st_size % 8) return KTRI_ERR_INVALID_CSR;
    *n_out = (uint64_t)a.st_size / 8 - 1;
    *nnz_out = (uint64_t)b.st_size / 8;
    return KTRI_OK;
}

int ktri_count_binary_file(ktri_ctx* ctx, const char* stem, uint64_t* total_out, uint64_t* per_vertex_out,
                           const ktri_opts* opts, uint64_t chunk_bytes) {
    const ktri::Options opt = resolve(opts);
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    if (!stem || !total_out) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "stem and total_out are required");
    uint64_t n = 0, nnz = 0;
    int rc = ktri_binary_file_shape(stem, &n, &nnz);
    if (rc) return set_error(ctx, rc, std::string("cannot read ") + stem + ".first_out / .head");
    const u64 dummy = 0;
    rc = check_common(ctx, &dummy, &dummy, n, nnz, total_out, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    if (chunk_bytes == 0) chunk_bytes = 64ull << 20;
    chunk_bytes = std::max<u64>(8, chunk_bytes & ~7ull);
    const std::string s(stem);
    const int ffo = open((s + ".first_out").c_str(), O_RDONLY);
    const int fhd = open((s + ".head").c_str(), O_RDONLY);
    void* pinned[2] = {nullptr, nullptr};
    cudaEvent_t freed[2] = {nullptr, nullptr};
    auto cleanup = [&](int code) {
        if (ffo >= 0) close(ffo);
        if (fhd >= 0) close(fhd);
        for (int i = 0; i < 2; ++i) {
            if (freed[i]) {
                cudaEventSynchronize(freed[i]);
                cudaEventDestroy(freed[i]);
            }
            if (pinned[i]) cudaFreeHost(pinned[i]);
        }
        return code;
    };
    if (ffo < 0 || fhd < 0) return cleanup(set_error(ctx, KTRI_ERR_IO, "cannot open the graph files"));
    if (n == 0) {
        *total_out = 0;
        return cleanup(nnz ? set_error(ctx, KTRI_ERR_INVALID_CSR, "edges without vertices") : KTRI_OK);
    }
    Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, true, true, opt.force_wide, opt.small_outdegree,
                           opt.segment);
    // two device staging chunks for u64 ids follow the count's workspace
    const size_t x_stage = L.bytes;
    L.bytes = align_up(x_stage + 2 * chunk_bytes);
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return cleanup(rc);
    for (int i = 0; i < 2; ++i) {
        if (cudaHostAlloc(&pinned[i], chunk_bytes, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&freed[i], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return cleanup(set_error(ctx, KTRI_ERR_OUT_OF_MEMORY, "pinned staging buffers"));
        }
    }
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    char* stage = base + x_stage;
    cudaStream_t st = ctx->stream;
    // file -> pinned chunk (read on the host) -> device, two chunks in flight: the read of one
    // chunk overlaps the copy (and id narrowing) of the other
    int slot = 0;
    u64 fo_first = 1, fo_last = 0;
    auto pump = [&](int fd, u64 bytes, char* dst, bool narrow) -> int {
        for (u64 off = 0; off < bytes; off += chunk_bytes) {
            const u64 len = std::min<u64>(chunk_bytes, bytes - off);
            KTRI_CK(ctx, cudaEventSynchronize(freed[slot]));
            u64 got = 0;
            while (got < len) {
                const ssize_t r = pread(fd, static_cast<char*>(pinned[slot]) + got, len - got, (off_t)(off + got));
                if (r <= 0) return set_error(ctx, KTRI_ERR_IO, "short read of the graph files");
                got += (u64)r;
            }
            if (!narrow) {
                if (off == 0) fo_first = *static_cast<const u64*>(pinned[slot]);
                if (off + len == bytes)
                    fo_last = *reinterpret_cast<const u64*>(static_cast<const char*>(pinned[slot]) + len - 8);
                KTRI_CK(ctx, copy_host(ctx, dst + off, pinned[slot], len, true, st));
            } else {
                char* sdev = stage + (size_t)slot * chunk_bytes;
                KTRI_CK(ctx, copy_host(ctx, sdev, pinned[slot], len, true, st));
                ktri::launch_narrow_ids(reinterpret_cast<const u64*>(sdev), len / 8,
                                        reinterpret_cast<u32*>(dst) + off / 8, ctx->num_sms, st);
            }
            KTRI_CK(ctx, cudaEventRecord(freed[slot], st));
            slot ^= 1;
        }
        return KTRI_OK;
    };
    rc = pump(ffo, 8 * (n + 1), reinterpret_cast<char*>(d_fo), false);
    if (rc) return cleanup(rc);
    if (fo_first != 0 || fo_last != nnz)
        return cleanup(set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz"));
    rc = pump(fhd, 8 * nnz, reinterpret_cast<char*>(d_head), true);
    if (rc) return cleanup(rc);
    KTRI_CK(ctx, cudaGetLastError());
    rc = L.wide ? run_pipeline<u64>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false)
                : run_pipeline<u32>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false);
    if (rc) return cleanup(rc);
    KTRI_CK(ctx, copy_host(ctx, total_out, d_total, sizeof(u64), false, st));
    bool staged = false;
    if (per_vertex_out) {
        cudaError_t e = cudaSuccess;
        staged = start_readback(ctx, per_vertex_out, d_cnt, sizeof(u64) * n, st, &e);
        KTRI_CK(ctx, e);
    }
    rc = device_status(ctx);
    if (rc == KTRI_OK) ctx->stats.triangles = *total_out;
    if (rc == KTRI_OK && staged) finish_readback(ctx, per_vertex_out, sizeof(u64) * n);
    return cleanup(rc);
}

// ---- contraction after the local phase -------------------------------------------------------

int ktri_contract_dag_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t n_local,
                          uint64_t m, uint32_t* kept_out, uint64_t* out_first_out, uint32_t* out_head,
                          uint64_t* kept_count, uint64_t* edge_count) {
    if (!ctx) return KTRI_ERR_INVALID_ARGUMENT;
    if (!first_out || (m && !head) || !kept_count || !edge_count || !out_first_out || (n_local && !kept_out) ||
        (m && !out_head))
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "NULL input or output pointer");
    if (n_local > n) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "n_local > n");
    if (n > 0xFFFFFFFFull) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "n must be below 2^32 (u32 vertex ids)");
    if (first_out[0] != 0 || first_out[n] != m)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal m");
    u64 maxdeg = 0;
    for (u64 v = 0; v < n; ++v) {
        if (first_out[v + 1] < first_out[v]) return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out is not monotone");
        if (v < n_local) maxdeg = std::max<u64>(maxdeg, first_out[v + 1] - first_out[v]);
    }
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    *kept_count = 0;
    *edge_count = 0;
    out_first_out[0] = 0;
    if (n_local == 0) return KTRI_OK;
    // lists longer than the block sort's shared memory are sorted through global scratch of
    // the next power of two, as many at a time as 256 MiB allows
    u64 P = 1;
    while (P < maxdeg) P <<= 1;
    const int big_grid = P <= 8192 ? 1 : (int)std::max<u64>(1, std::min<u64>(ctx->num_sms, (256ull << 20) / (4 * P)));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes);
        return at;
    };
    const size_t x_ctl = take(sizeof(Control)), x_fo = take(8 * (n + 1)), x_head = take(4 * (m + 1)),
                 x_cnt = take(8 * (n_local + 1)), x_keep = take(8 * (n_local + 1)),
                 x_sums = take(8 * (ktri::dag_scan_chunks(n_local) + 1)), x_max = take(8), x_kept = take(4 * n_local),
                 x_ofo = take(8 * (n_local + 1)), x_ohead = take(4 * (m + 1)), x_desc = take(16 * n_local),
                 x_mid = take(4 * n_local), x_big = take(4 * n_local),
                 x_scr = take(P <= 8192 ? 4 : 4 * P * (u64)big_grid);
    int rc = ensure_ws(ctx, off);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* ctl = reinterpret_cast<Control*>(base + x_ctl);
    auto* d_fo = reinterpret_cast<u64*>(base + x_fo);
    auto* d_head = reinterpret_cast<u32*>(base + x_head);
    auto* d_cnt = reinterpret_cast<u64*>(base + x_cnt);
    auto* d_keep = reinterpret_cast<u64*>(base + x_keep);
    auto* d_ofo = reinterpret_cast<u64*>(base + x_ofo);
    auto* d_ohead = reinterpret_cast<u32*>(base + x_ohead);
    auto* d_kept = reinterpret_cast<u32*>(base + x_kept);
    auto* d_max = reinterpret_cast<unsigned long long*>(base + x_max);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, cudaMemsetAsync(ctl, 0, sizeof(Control), st));
    KTRI_CK(ctx, cudaMemsetAsync(base + x_desc, 0, 16 * n_local, st));
    KTRI_CK(ctx, cudaMemcpyAsync(d_fo, first_out, 8 * (n + 1), cudaMemcpyHostToDevice, st));
    if (m) KTRI_CK(ctx, cudaMemcpyAsync(d_head, head, 4 * m, cudaMemcpyHostToDevice, st));
    ktri::launch_contract(d_fo, d_head, n, n_local, d_cnt, d_keep, reinterpret_cast<u64*>(base + x_sums), d_max,
                          d_kept, d_ofo, d_ohead, base + x_desc, ctx->num_sms, st);
    // sorted by id, as preprocessing_global does after compact (cetric.h:916-930)
    ktri::launch_sort_lists<u64>(n_local, base + x_desc, d_ohead, reinterpret_cast<u32*>(base + x_mid),
                                 reinterpret_cast<u32*>(base + x_big), reinterpret_cast<u32*>(base + x_scr), P, big_grid,
                                 ctl, ctx->num_sms, st);
    KTRI_CK(ctx, cudaGetLastError());
    u64 ke[2] = {0, 0};
    KTRI_CK(ctx, cudaMemcpyAsync(&ke[0], d_keep + n_local, 8, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaMemcpyAsync(&ke[1], d_cnt + n_local, 8, cudaMemcpyDeviceToHost, st));
    u32 err = 0;
    KTRI_CK(ctx, cudaMemcpyAsync(&err, &ctl->err, 4, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaStreamSynchronize(st));
    if (err & ktri::DEV_ERR_MASK) return set_error(ctx, KTRI_ERR_CUDA, "list sort found a list above its scratch");
    const u64 K = ke[0], E = ke[1];
    if (K) KTRI_CK(ctx, cudaMemcpyAsync(kept_out, d_kept, 4 * K, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaMemcpyAsync(out_first_out, d_ofo, 8 * (K + 1), cudaMemcpyDeviceToHost, st));
    if (E) KTRI_CK(ctx, cudaMemcpyAsync(out_head, d_ohead, 4 * E, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaStreamSynchronize(st));
    *kept_count = K;
    *edge_count = E;
    return KTRI_OK;
}

// ---- load-balancing cost functions -------------------------------------------------------------

int ktri_partition_cost(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                        int32_t cost_function, uint32_t parts, uint64_t* boundaries_out, uint64_t* costs_out,
                        uint64_t* total_cost_out) {
    ktri::Options opt;
    opt.method = KTRI_METHOD_MERGE;
    int rc = check_common(ctx, first_out, head, n, nnz, total_cost_out, opt);
    if (rc) return rc;
    if (!boundaries_out || parts == 0) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "need parts >= 1 boundaries");
    if (cost_function < KTRI_COST_N || cost_function > KTRI_COST_IDPD)
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "unknown cost function");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    *total_cost_out = 0;
    if (n == 0) {
        for (u32 i = 0; i <= parts; ++i) boundaries_out[i] = 0;
        return KTRI_OK;
    }
    if (first_out[0] != 0 || first_out[n] != nnz)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz");
    Layout L = make_layout(n, nnz, KTRI_METHOD_MERGE, ctx->num_sms, true, true);
    const size_t x_cost = L.bytes, x_sums = align_up(x_cost + 8 * (n + 1)),
                 x_bnd = align_up(x_sums + 8 * (ktri::dag_scan_chunks(n) + 1));
    L.bytes = align_up(x_bnd + 8 * ((u64)parts + 1));
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_cost = reinterpret_cast<u64*>(base + x_cost);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, cudaMemcpyAsync(d_fo, first_out, 8 * (n + 1), cudaMemcpyHostToDevice, st));
    if (nnz) KTRI_CK(ctx, cudaMemcpyAsync(d_head, head, 4 * nnz, cudaMemcpyHostToDevice, st));
    // degrees and out-degrees come from the orientation stage of the pipeline
    rc = L.wide ? run_pipeline<u64>(ctx, L, d_fo, d_head, n, nnz, reinterpret_cast<u64*>(base + L.total),
                                    reinterpret_cast<u64*>(base + L.cnt), opt, st, true)
                : run_pipeline<u32>(ctx, L, d_fo, d_head, n, nnz, reinterpret_cast<u64*>(base + L.total),
                                    reinterpret_cast<u64*>(base + L.cnt), opt, st, true);
    if (rc) return rc;
    ktri::launch_cost_partition(d_fo, d_head, n, reinterpret_cast<const u32*>(base + L.deg),
                                reinterpret_cast<const u32*>(base + L.dplus), cost_function, parts, d_cost,
                                reinterpret_cast<u64*>(base + x_sums), reinterpret_cast<u64*>(base + x_bnd),
                                ctx->num_sms, st);
    KTRI_CK(ctx, cudaGetLastError());
    std::vector<u64> prefix(costs_out ? n + 1 : 0);
    if (costs_out) KTRI_CK(ctx, cudaMemcpyAsync(prefix.data(), d_cost, 8 * (n + 1), cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaMemcpyAsync(total_cost_out, d_cost + n, 8, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaMemcpyAsync(boundaries_out, base + x_bnd, 8 * ((u64)parts + 1), cudaMemcpyDeviceToHost, st));
    rc = device_status(ctx);
    if (rc) return rc;
    if (costs_out)
        for (u64 v = 0; v < n; ++v) costs_out[v] = prefix[v + 1] - prefix[v];
    return KTRI_OK;
}

// ---- triangle listing (checking) -----------------------------------------------------------

int ktri_list_triangles(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                        uint32_t* triples_out, uint64_t capacity, uint64_t* count_out) {
    ktri::Options opt;
    opt.method = KTRI_METHOD_MERGE;
    int rc = check_common(ctx, first_out, head, n, nnz, count_out, opt);
    if (rc) return rc;
    if (capacity && !triples_out) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "triples_out is NULL");
    if (capacity > (1ull << 40)) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "capacity above 2^40 triangles");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    *count_out = 0;
    if (n == 0) return KTRI_OK;
    if (first_out[0] != 0 || first_out[n] != nnz)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz");
    Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, true, true);
    const size_t x_tri = L.bytes, x_pos = align_up(x_tri + sizeof(u32) * 3 * capacity);
    L.bytes = align_up(x_pos + sizeof(u64));
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    ktri::TriangleSink sink;
    sink.triples = reinterpret_cast<u32*>(base + x_tri);
    sink.cap = capacity;
    sink.pos = reinterpret_cast<unsigned long long*>(base + x_pos);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, cudaMemsetAsync(sink.pos, 0, sizeof(u64), st));
    KTRI_CK(ctx, cudaMemcpyAsync(d_fo, first_out, sizeof(u64) * (n + 1), cudaMemcpyHostToDevice, st));
    if (nnz) KTRI_CK(ctx, cudaMemcpyAsync(d_head, head, sizeof(u32) * nnz, cudaMemcpyHostToDevice, st));
    rc = L.wide ? run_pipeline<u64>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false, sink)
                : run_pipeline<u32>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, false, sink);
    if (rc) return rc;
    u64 total = 0;
    KTRI_CK(ctx, cudaMemcpyAsync(&total, d_total, sizeof(u64), cudaMemcpyDeviceToHost, st));
    rc = device_status(ctx);
    if (rc) return rc;
    const u64 got = total < capacity ? total : capacity;
    if (got) KTRI_CK(ctx, cudaMemcpy(triples_out, sink.triples, sizeof(u32) * 3 * got, cudaMemcpyDeviceToHost));
    *count_out = total;
    ctx->stats.triangles = total;
    return total > capacity ? set_error(ctx, KTRI_ERR_OUT_OF_MEMORY, "more triangles than the output capacity")
                            : KTRI_OK;
}

// ---- oriented lists (the katric local phase) ---------------------------------------------

int ktri_count_dag_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n, uint64_t m,
                          uint64_t* d_total, uint64_t* d_per_vertex, const ktri_opts* opts, void* stream) {
    const ktri::Options opt = resolve(opts);
    int rc = check_common(ctx, d_first_out, d_head, n, m, d_total, opt);
    if (rc) return rc;
    if (m > (1ull << 62)) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "too many edges");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        KTRI_CK(ctx, cudaMemsetAsync(d_total, 0, sizeof(u64), st));
        ctx->pending = false;
        ctx->stats = ktri_run_stats{};
        return KTRI_OK;
    }
    const u64 nnz = 2 * m;
    const Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, true, d_per_vertex == nullptr, opt.force_wide,
                                 opt.small_outdegree, opt.segment);
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* fs = reinterpret_cast<u64*>(base + L.in_fo);
    auto* hs = reinterpret_cast<u32*>(base + L.in_head);
    // the out-list and descriptor regions are free until orientation starts: in-list cursors
    // and scan sums live there meanwhile
    auto* cursor = reinterpret_cast<u32*>(base + L.deg);
    auto* sums = reinterpret_cast<u64*>(base + L.headp);
    ktri::launch_dag_symmetrize(reinterpret_cast<const u64*>(d_first_out), d_head, n, fs, hs, cursor, sums,
                                ctx->num_sms, st);
    KTRI_CK(ctx, cudaGetLastError());
    u64* cnt = d_per_vertex ? reinterpret_cast<u64*>(d_per_vertex) : reinterpret_cast<u64*>(base + L.cnt);
    auto* tot = reinterpret_cast<u64*>(d_total);
    return L.wide ? run_pipeline<u64>(ctx, L, fs, hs, n, nnz, tot, cnt, opt, st, false)
                  : run_pipeline<u32>(ctx, L, fs, hs, n, nnz, tot, cnt, opt, st, false);
}

int ktri_count_dag_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t m,
                       uint64_t* total_out, uint64_t* per_vertex_out, const ktri_opts* opts) {
    const ktri::Options opt = resolve(opts);
    int rc = check_common(ctx, first_out, head, n, m, total_out, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    if (n == 0) {
        *total_out = 0;
        return KTRI_OK;
    }
    if (first_out[0] != 0 || first_out[n] != m)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal m");
    for (u64 v = 0; v < n; ++v)
        if (first_out[v + 1] < first_out[v])
            return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out is not monotone");
    if (m > (1ull << 62)) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "too many edges");
    const u64 nnz = 2 * m;
    Layout L = make_layout(n, nnz, opt.method, ctx->num_sms, true, true, opt.force_wide, opt.small_outdegree,
                           opt.segment);
    // the caller's lists and the scan sums follow the count's workspace
    const size_t x_fo = L.bytes, x_head = align_up(x_fo + sizeof(u64) * (n + 1)),
                 x_sums = align_up(x_head + sizeof(u32) * m);
    L.bytes = align_up(x_sums + sizeof(u64) * (ktri::dag_scan_chunks(n) + 1));
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* dfo = reinterpret_cast<u64*>(base + x_fo);
    auto* dhead = reinterpret_cast<u32*>(base + x_head);
    auto* sums = reinterpret_cast<u64*>(base + x_sums);
    auto* fs = reinterpret_cast<u64*>(base + L.in_fo);
    auto* hs = reinterpret_cast<u32*>(base + L.in_head);
    auto* cursor = reinterpret_cast<u32*>(base + L.deg);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, copy_host(ctx, dfo, first_out, sizeof(u64) * (n + 1), true, st));
    if (m) KTRI_CK(ctx, copy_host(ctx, dhead, head, sizeof(u32) * m, true, st));
    ktri::launch_dag_symmetrize(dfo, dhead, n, fs, hs, cursor, sums, ctx->num_sms, st);
    KTRI_CK(ctx, cudaGetLastError());
    rc = L.wide ? run_pipeline<u64>(ctx, L, fs, hs, n, nnz, d_total, d_cnt, opt, st, false)
                : run_pipeline<u32>(ctx, L, fs, hs, n, nnz, d_total, d_cnt, opt, st, false);
    if (rc) return rc;
    KTRI_CK(ctx, copy_host(ctx, total_out, d_total, sizeof(u64), false, st));
    bool staged = false;
    if (per_vertex_out) {
        cudaError_t e = cudaSuccess;
        staged = start_readback(ctx, per_vertex_out, d_cnt, sizeof(u64) * n, st, &e);
        KTRI_CK(ctx, e);
    }
    rc = device_status(ctx);
    if (rc == KTRI_OK) ctx->stats.triangles = *total_out;
    if (rc == KTRI_OK && staged) finish_readback(ctx, per_vertex_out, sizeof(u64) * n);
    return rc;
}

// ---- batches of graphs ----------------------------------------------------------------

}  // extern "C"

namespace {

int check_batch(ktri_ctx* ctx, const void* fo, const void* head, u64 n, u64 nnz, const void* graph_first,
                u64 num_graphs, const void* totals, const ktri::Options& opt) {
    int rc = check_common(ctx, fo, head, n, nnz, totals, opt);
    if (rc) return rc;
    if (num_graphs && !graph_first) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "graph_first is NULL");
    return KTRI_OK;
}

template <typename OffT>
int enqueue_batch(ktri_ctx* ctx, char* base, const Layout& L, const u64* fo, const u32* head, u64 n, u64 nnz,
                  const u64* graph_first, u64 num_graphs, u64* totals, u64* cnt, const ktri::Options& opt,
                  cudaStream_t st, bool events) {
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    int rc = enqueue_pipeline<OffT>(ctx, ctx->num_sms, base, L, fo, head, n, nnz, d_total, cnt, opt, st, false,
                                    events);
    if (rc) return rc;
    ktri::launch_graph_totals(cnt, graph_first, num_graphs, n, totals, reinterpret_cast<Control*>(base + L.ctl),
                              ctx->num_sms, st);
    if (events) KTRI_CK(ctx, cudaEventRecord(ctx->ev[3], st));  // the call ends after the totals
    KTRI_CK(ctx, cudaGetLastError());
    return KTRI_OK;
}

void note_pending(ktri_ctx* ctx, const Layout& L, char* base, cudaStream_t st, u64 n, u64 nnz,
                  const ktri::Options& opt) {
    ctx->ctl = reinterpret_cast<Control*>(base + L.ctl);
    ctx->last_stream = st;
    ctx->pending = true;
    ctx->have_events = true;
    ctx->last_method = opt.method;
    ctx->last_collect = opt.collect_stats;
    ctx->stats = ktri_run_stats{};
    ctx->stats.n = n;
    ctx->stats.nnz = nnz;
    ctx->stats.method = (u32)opt.method;
}

}  // namespace

extern "C" {

int ktri_count_batch_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                            uint64_t nnz_total, const uint64_t* d_graph_first, uint64_t num_graphs, uint64_t* d_totals,
                            uint64_t* d_per_vertex, const ktri_opts* opts, void* stream) {
    const ktri::Options opt = resolve(opts);
    int rc = check_batch(ctx, d_first_out, d_head, n_total, nnz_total, d_graph_first, num_graphs, d_totals, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n_total == 0) {
        if (num_graphs) KTRI_CK(ctx, cudaMemsetAsync(d_totals, 0, sizeof(u64) * num_graphs, st));
        ctx->pending = false;
        return KTRI_OK;
    }
    const Layout L = make_layout(n_total, nnz_total, opt.method, ctx->num_sms, false, true,
                                 opt.force_wide, opt.small_outdegree, opt.segment);
    rc = ensure_ws(ctx, L.bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    u64* cnt = d_per_vertex ? reinterpret_cast<u64*>(d_per_vertex) : reinterpret_cast<u64*>(base + L.cnt);
    auto* fo = reinterpret_cast<const u64*>(d_first_out);
    auto* gf = reinterpret_cast<const u64*>(d_graph_first);
    auto* tot = reinterpret_cast<u64*>(d_totals);
    rc = L.wide ? enqueue_batch<u64>(ctx, base, L, fo, d_head, n_total, nnz_total, gf, num_graphs, tot, cnt, opt, st,
                                     true)
                : enqueue_batch<u32>(ctx, base, L, fo, d_head, n_total, nnz_total, gf, num_graphs, tot, cnt, opt, st,
                                     true);
    if (rc) return rc;
    note_pending(ctx, L, base, st, n_total, nnz_total, opt);
    return KTRI_OK;
}

int ktri_count_batch_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n_total,
                         uint64_t nnz_total, const uint64_t* graph_first, uint64_t num_graphs, uint64_t* totals_out,
                         uint64_t* per_vertex_out, const ktri_opts* opts) {
    const ktri::Options opt = resolve(opts);
    int rc = check_batch(ctx, first_out, head, n_total, nnz_total, graph_first, num_graphs, totals_out, opt);
    if (rc) return rc;
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    for (u64 i = 0; i < num_graphs; ++i)
        if (graph_first[i + 1] < graph_first[i] || graph_first[i + 1] > n_total)
            return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "graph_first must be non-decreasing and end within n");
    if (num_graphs && (graph_first[0] != 0 || graph_first[num_graphs] != n_total))
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "graph_first must run from 0 to n_total");
    if (n_total == 0) {
        for (u64 i = 0; i < num_graphs; ++i) totals_out[i] = 0;
        return KTRI_OK;
    }
    if (first_out[0] != 0 || first_out[n_total] != nnz_total)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz");
    const Layout L = make_layout(n_total, nnz_total, opt.method, ctx->num_sms, true, true,
                                 opt.force_wide, opt.small_outdegree, opt.segment);
    const size_t off_gf = L.bytes, off_tot = align_up(off_gf + sizeof(u64) * (num_graphs + 1));
    const size_t total_bytes = align_up(off_tot + sizeof(u64) * (num_graphs + 1));
    rc = ensure_ws(ctx, total_bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_gf = reinterpret_cast<u64*>(base + off_gf);
    auto* d_tot = reinterpret_cast<u64*>(base + off_tot);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, copy_host(ctx, d_fo, first_out, sizeof(u64) * (n_total + 1), true, st));
    if (nnz_total) KTRI_CK(ctx, copy_host(ctx, d_head, head, sizeof(u32) * nnz_total, true, st));
    KTRI_CK(ctx, copy_host(ctx, d_gf, graph_first, sizeof(u64) * (num_graphs + 1), true, st));
    rc = L.wide ? enqueue_batch<u64>(ctx, base, L, d_fo, d_head, n_total, nnz_total, d_gf, num_graphs, d_tot, d_cnt,
                                     opt, st, true)
                : enqueue_batch<u32>(ctx, base, L, d_fo, d_head, n_total, nnz_total, d_gf, num_graphs, d_tot, d_cnt,
                                     opt, st, true);
    if (rc) return rc;
    note_pending(ctx, L, base, st, n_total, nnz_total, opt);
    if (num_graphs) KTRI_CK(ctx, copy_host(ctx, totals_out, d_tot, sizeof(u64) * num_graphs, false, st));
    bool staged = false;
    if (per_vertex_out) {
        cudaError_t e = cudaSuccess;
        staged = start_readback(ctx, per_vertex_out, d_cnt, sizeof(u64) * n_total, st, &e);
        KTRI_CK(ctx, e);
    }
    rc = device_status(ctx);
    if (rc == KTRI_OK && staged) finish_readback(ctx, per_vertex_out, sizeof(u64) * n_total);
    return rc;
}

// ---- captured plans ----------------------------------------------------------------------

}  // extern "C"

struct ktri_plan {
    ktri_ctx* ctx = nullptr;  // launch and check report errors through it
    int device = 0;           // destroy needs only this, so it is safe after the context is gone
    void* ws = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Control* ctl = nullptr;
    cudaStream_t last = nullptr;
    bool launched = false;
};

extern "C" {

int ktri_plan_create_batch(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                           uint64_t nnz_total, const uint64_t* d_graph_first, uint64_t num_graphs,
                           uint64_t* d_totals, uint64_t* d_per_vertex, const ktri_opts* opts, ktri_plan** out) {
    if (!out) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    const ktri::Options opt = resolve(opts);
    int rc = check_batch(ctx, d_first_out, d_head, n_total, nnz_total, d_graph_first, num_graphs, d_totals, opt);
    if (rc) return rc;
    if (n_total == 0) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "a plan needs at least one vertex");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    const Layout L = make_layout(n_total, nnz_total, opt.method, ctx->num_sms, false, true,
                                 opt.force_wide, opt.small_outdegree, opt.segment);
    if (ctx->budget && L.bytes > ctx->budget)
        return set_error(ctx, KTRI_ERR_OUT_OF_MEMORY, "plan workspace exceeds the memory budget");
    ktri_plan* p = new (std::nothrow) ktri_plan();
    if (!p) return KTRI_ERR_OUT_OF_MEMORY;
    p->ctx = ctx;
    p->device = ctx->device;
    cudaError_t e = cudaMalloc(&p->ws, L.bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return cuda_fail(ctx, e, "cudaMalloc(plan workspace)");
    }
    // occupancy queries happen once, outside the capture
    for (u32 sd : {(u32)ktri::SMALL_D_LOW, (u32)ktri::SMALL_D}) {
        (void)ktri::count_grid_auto<u32>(ctx->num_sms, sd);
        (void)ktri::count_grid_auto<u64>(ctx->num_sms, sd);
    }
    cudaStream_t cs = nullptr;
    cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    char* base = static_cast<char*>(p->ws);
    u64* cnt = d_per_vertex ? reinterpret_cast<u64*>(d_per_vertex) : reinterpret_cast<u64*>(base + L.cnt);
    auto* fo = reinterpret_cast<const u64*>(d_first_out);
    auto* gf = reinterpret_cast<const u64*>(d_graph_first);
    auto* tot = reinterpret_cast<u64*>(d_totals);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        rc = L.wide ? enqueue_batch<u64>(ctx, base, L, fo, d_head, n_total, nnz_total, gf, num_graphs, tot, cnt, opt, cs,
                                         false)
                    : enqueue_batch<u32>(ctx, base, L, fo, d_head, n_total, nnz_total, gf, num_graphs, tot, cnt, opt, cs,
                                         false);
        cudaGraph_t graph = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (rc == KTRI_OK && e2 != cudaSuccess) rc = cuda_fail(ctx, e2, "cudaStreamEndCapture");
        p->graph = graph;
        if (rc == KTRI_OK) {
            const cudaError_t e3 = cudaGraphInstantiate(&p->exec, graph, 0);
            if (e3 != cudaSuccess) rc = cuda_fail(ctx, e3, "cudaGraphInstantiate");
        }
    } else {
        rc = cuda_fail(ctx, e, "cudaStreamBeginCapture");
    }
    cudaStreamDestroy(cs);
    if (rc) {
        if (p->exec) cudaGraphExecDestroy(p->exec);
        if (p->graph) cudaGraphDestroy(p->graph);
        cudaFree(p->ws);
        delete p;
        return rc;
    }
    p->ctl = reinterpret_cast<Control*>(base + L.ctl);
    *out = p;
    return KTRI_OK;
}

int ktri_plan_launch(ktri_plan* plan, void* stream) {
    if (!plan) return KTRI_ERR_INVALID_ARGUMENT;
    DeviceGuard g(plan->ctx->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    KTRI_CK(plan->ctx, cudaGraphLaunch(plan->exec, st));
    plan->last = st;
    plan->launched = true;
    return KTRI_OK;
}

int ktri_plan_check(ktri_plan* plan) {
    if (!plan) return KTRI_ERR_INVALID_ARGUMENT;
    if (!plan->launched) return KTRI_OK;
    DeviceGuard g(plan->ctx->device);
    ktri_ctx* ctx = plan->ctx;
    KTRI_CK(ctx, cudaStreamSynchronize(plan->last));
    u32 err = 0;
    KTRI_CK(ctx, cudaMemcpy(&err, &plan->ctl->err, sizeof(u32), cudaMemcpyDeviceToHost));
    if (err & ktri::DEV_ERR_TIMEOUT)
        return set_error(ctx, KTRI_ERR_TIMEOUT, "a bulk copy into shared memory did not complete in time");
    if (err & ktri::DEV_ERR_MASK) return set_error(ctx, KTRI_ERR_INVALID_CSR, "invalid CSR found on the device");
    return KTRI_OK;
}

int ktri_plan_destroy(ktri_plan* plan) {
    if (!plan) return KTRI_ERR_INVALID_ARGUMENT;
    {
        DeviceGuard g(plan->device);
        if (plan->launched) cudaStreamSynchronize(plan->last);
        if (plan->exec) cudaGraphExecDestroy(plan->exec);
        if (plan->graph) cudaGraphDestroy(plan->graph);
        if (plan->ws) cudaFree(plan->ws);
    }
    delete plan;
    return KTRI_OK;
}

int ktri_orient_csr(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                    uint64_t* out_first_out, uint32_t* out_head) {
    if (!ctx || !out_first_out || (n && !first_out) || (nnz && (!head || !out_head)))
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "null pointer");
    if (n > 0xFFFFFFFFull) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "n must be below 2^32");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    out_first_out[0] = 0;
    if (n == 0) return KTRI_OK;
    if (first_out[0] != 0 || first_out[n] != nnz)
        return set_error(ctx, KTRI_ERR_INVALID_CSR, "first_out[0] must be 0 and first_out[n] must equal nnz");
    ktri::Options opt;
    opt.method = KTRI_METHOD_MERGE;
    Layout L = make_layout(n, nnz, KTRI_METHOD_MERGE, ctx->num_sms, true, true);
    // room for the exported CSR: out offsets (u64[n+1]) and out heads (u32[nnz/2])
    const size_t off_ofo = L.bytes, off_oh = align_up(off_ofo + sizeof(u64) * (n + 1));
    const size_t total_bytes = align_up(off_oh + sizeof(u32) * (nnz / 2 + 1));
    int rc = ensure_ws(ctx, total_bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    auto* d_fo = reinterpret_cast<u64*>(base + L.in_fo);
    auto* d_head = reinterpret_cast<u32*>(base + L.in_head);
    auto* d_total = reinterpret_cast<u64*>(base + L.total);
    auto* d_cnt = reinterpret_cast<u64*>(base + L.cnt);
    auto* d_ofo = reinterpret_cast<u64*>(base + off_ofo);
    auto* d_oh = reinterpret_cast<u32*>(base + off_oh);
    cudaStream_t st = ctx->stream;
    KTRI_CK(ctx, cudaMemcpyAsync(d_fo, first_out, sizeof(u64) * (n + 1), cudaMemcpyHostToDevice, st));
    if (nnz) KTRI_CK(ctx, cudaMemcpyAsync(d_head, head, sizeof(u32) * nnz, cudaMemcpyHostToDevice, st));
    rc = L.wide ? run_pipeline<u64>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, true)
                : run_pipeline<u32>(ctx, L, d_fo, d_head, n, nnz, d_total, d_cnt, opt, st, true);
    if (rc) return rc;
    if (L.wide) ktri::launch_outdeg<u64>(n, base + L.vdesc, d_cnt, ctx->num_sms, st);
    else ktri::launch_outdeg<u32>(n, base + L.vdesc, d_cnt, ctx->num_sms, st);
    std::vector<u64> outdeg(n);
    KTRI_CK(ctx, cudaMemcpyAsync(outdeg.data(), d_cnt, sizeof(u64) * n, cudaMemcpyDeviceToHost, st));
    rc = device_status(ctx);
    if (rc) return rc;
    for (u64 v = 0; v < n; ++v) out_first_out[v + 1] = out_first_out[v] + outdeg[v];
    if (out_first_out[n] > nnz / 2 + 1) return set_error(ctx, KTRI_ERR_INVALID_CSR, "graph is not symmetric");
    KTRI_CK(ctx, cudaMemcpyAsync(d_ofo, out_first_out, sizeof(u64) * (n + 1), cudaMemcpyHostToDevice, st));
    if (L.wide) ktri::launch_export<u64>(n, base + L.vdesc, reinterpret_cast<u32*>(base + L.headp), d_ofo, d_oh,
                                         ctx->num_sms, st);
    else ktri::launch_export<u32>(n, base + L.vdesc, reinterpret_cast<u32*>(base + L.headp), d_ofo, d_oh,
                                  ctx->num_sms, st);
    if (out_first_out[n])
        KTRI_CK(ctx, cudaMemcpyAsync(out_head, d_oh, sizeof(u32) * out_first_out[n], cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaStreamSynchronize(st));
    KTRI_CK(ctx, cudaGetLastError());
    return KTRI_OK;
}

int ktri_intersect_pairs(ktri_ctx* ctx, int32_t method, const uint32_t* a_vals, const uint64_t* a_off,
                         const uint32_t* b_vals, const uint64_t* b_off, uint64_t npairs, uint64_t* counts_out,
                         uint32_t* members_out) {
    if (!ctx || !a_off || !b_off || !counts_out) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "null pointer");
    if (method < KTRI_METHOD_AUTO || method > KTRI_METHOD_HYBRID)
        return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "unknown intersection method");
    if (npairs == 0) return KTRI_OK;
    const u64 na = a_off[npairs], nb = b_off[npairs];
    for (u64 i = 0; i < npairs; ++i) {
        if (a_off[i + 1] < a_off[i] || b_off[i + 1] < b_off[i] || a_off[i + 1] - a_off[i] > 0xFFFFFFFFull ||
            b_off[i + 1] - b_off[i] > 0xFFFFFFFFull)
            return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "offsets must be non-decreasing");
    }
    if ((na && !a_vals) || (nb && !b_vals)) return set_error(ctx, KTRI_ERR_INVALID_ARGUMENT, "null list values");
    DeviceGuard g(ctx->device);
    if (ctx->pending) device_status(ctx);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = align_up(off + bytes);
        return at;
    };
    const size_t o_av = take(4 * (na + 1)), o_bv = take(4 * (nb + 1)), o_ao = take(8 * (npairs + 1)),
                 o_bo = take(8 * (npairs + 1)), o_c = take(8 * npairs), o_m = take(4 * (na + 1)), o_e = take(4);
    int rc = ensure_ws(ctx, off);
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->ws);
    cudaStream_t st = ctx->stream;
    if (na) KTRI_CK(ctx, cudaMemcpyAsync(base + o_av, a_vals, 4 * na, cudaMemcpyHostToDevice, st));
    if (nb) KTRI_CK(ctx, cudaMemcpyAsync(base + o_bv, b_vals, 4 * nb, cudaMemcpyHostToDevice, st));
    KTRI_CK(ctx, cudaMemcpyAsync(base + o_ao, a_off, 8 * (npairs + 1), cudaMemcpyHostToDevice, st));
    KTRI_CK(ctx, cudaMemcpyAsync(base + o_bo, b_off, 8 * (npairs + 1), cudaMemcpyHostToDevice, st));
    KTRI_CK(ctx, cudaMemsetAsync(base + o_e, 0, 4, st));
    ktri::launch_intersect_pairs(method, reinterpret_cast<u32*>(base + o_av), reinterpret_cast<u64*>(base + o_ao),
                                 reinterpret_cast<u32*>(base + o_bv), reinterpret_cast<u64*>(base + o_bo), npairs,
                                 1000, 1.0, reinterpret_cast<u64*>(base + o_c),
                                 members_out ? reinterpret_cast<u32*>(base + o_m) : nullptr,
                                 reinterpret_cast<int*>(base + o_e), st);
    KTRI_CK(ctx, cudaGetLastError());
    KTRI_CK(ctx, cudaMemcpyAsync(counts_out, base + o_c, 8 * npairs, cudaMemcpyDeviceToHost, st));
    if (members_out && na) KTRI_CK(ctx, cudaMemcpyAsync(members_out, base + o_m, 4 * na, cudaMemcpyDeviceToHost, st));
    int herr = 0;
    KTRI_CK(ctx, cudaMemcpyAsync(&herr, base + o_e, 4, cudaMemcpyDeviceToHost, st));
    KTRI_CK(ctx, cudaStreamSynchronize(st));
    if (herr) return set_error(ctx, KTRI_ERR_UNSUPPORTED, "binary intersection stack overflow");
    return KTRI_OK;
}

}  // extern "C"
