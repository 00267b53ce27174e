/*
 * ktri.h — C ABI of the katric_gb300 exact local triangle-counting engine (sm_103a).
 *
 * The engine replaces the local counting phase of KaTric (degree-based orientation,
 * per-vertex id sort, edge-iterator set intersection) with CUDA kernels on one GPU.
 * Input: an undirected simple graph in CSR form, u64 first_out[n+1] and u32 head[nnz],
 * both directions of every edge stored, no self-loops, no duplicate entries, adjacency
 * lists in any order.  Output: the u64 triangle total and, optionally, u64 per-vertex
 * counts (each triangle {v,u,w} adds one to v, u and w).
 *
 * Every function returns an int status: KTRI_OK (0) or a negative KTRI_ERR_* code.
 * No C++ exception crosses this boundary.  Reference paths below are relative to the
 * KaTric source tree.
 */
#ifndef KTRI_H
#define KTRI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KTRI_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------------------ */
#define KTRI_OK 0
#define KTRI_ERR_INVALID_ARGUMENT (-1) /* null pointer, size mismatch, bad option */
#define KTRI_ERR_INVALID_CSR (-2)      /* id >= n, self-loop, non-monotone first_out, duplicate */
#define KTRI_ERR_OUT_OF_MEMORY (-3)    /* device or host allocation failed, or over the memory budget */
#define KTRI_ERR_CUDA (-4)             /* a CUDA runtime call failed; see ktri_last_error */
#define KTRI_ERR_TIMEOUT (-5)          /* a bounded device-side wait gave up */
#define KTRI_ERR_UNSUPPORTED (-6)      /* valid input outside what the library handles */
#define KTRI_ERR_IO (-7)               /* file could not be read or written, or is malformed */
#define KTRI_ERR_NO_DEVICE (-8)        /* no CUDA device, or the requested one does not exist */

/* ---- options ------------------------------------------------------------------------- */
/* Intersection strategy, mirroring Config::intersection_method (include/cetric/config.h:172,
 * selected by shmetric's --intersection-method, apps/parse_parameters.h:156-158).
 * KTRI_METHOD_AUTO is the GPU default: owner-side shared-memory hash tables that stream the
 * shorter out-list of every edge.  The other four run the reference's strategies on
 * id-sorted out-lists, one warp per oriented edge.  All five give identical counts. */
#define KTRI_METHOD_AUTO 0
#define KTRI_METHOD_MERGE 1         /* merge_intersection, include/cetric/counters/intersection.h:82-96 */
#define KTRI_METHOD_BINARY_SEARCH 2 /* binary_search_intersection, intersection.h:99-117 */
#define KTRI_METHOD_BINARY 3        /* binary_intersection, intersection.h:120-192 */
#define KTRI_METHOD_HYBRID 4        /* hybrid rule, intersection.h:66-77 */

typedef struct ktri_opts {
    uint32_t struct_size;          /* sizeof(ktri_opts); 0 is read as "all defaults" */
    int32_t intersection_method;   /* KTRI_METHOD_* */
    uint32_t small_outdegree;      /* owners with out-degree <= this use the tile kernel: 1..48 (0 = default 32;
                                      bounds above 32 pay off on graphs of average degree above ~40) */
    uint32_t collect_stats;        /* 1: also compute wedge_checks / intersection work counters */
    uint64_t binary_intersection_cutoff; /* Config::binary_intersection_cutoff (config.h:173), default 1000 */
    double hybrid_cutoff_scale;    /* Config::hybrid_cutoff_scale (config.h:174), default 1.0 */
    uint32_t force_wide_offsets;   /* 1: 64-bit out-list offsets even where 32 bits suffice (the path
                                      graphs with nnz + 3n > 2^32 take; exposed for testing) */
    uint32_t medium_outdegree;     /* owners above small_outdegree and at most this use the warp-per-tile
                                      kernel, larger ones the block-per-tile kernel: small_outdegree..256
                                      (0 = default 256) */
    uint32_t segment;              /* adjacency slots per owner tile of those two kernels: a power of two
                                      in 64..1024 (0 = default 1024) */
    uint32_t copy_wait_polls;      /* bound on the polls of the large-owner kernel's first wait for each
                                      bulk copy into shared memory (0 = default 2^22).  A wait that runs
                                      out makes the call fail with KTRI_ERR_TIMEOUT and a total of 0.
                                      KTRI_COPY_WAIT_NONE gives up at once (tests of that path). */
    uint32_t tile_order;           /* order in which the medium- and large-owner kernels take their tiles:
                                      0 (default) large tiles by the first vertex they stream (tiles that run
                                      together read nearby out-lists), medium tiles longest owner first;
                                      KTRI_TILE_ORDER_COST both by the entries each tile streams, heaviest first
                                      (the reference's DPD edge cost, cost_function.h:287-376, per tile) */
    uint32_t reserved[3];
} ktri_opts;

#define KTRI_TILE_ORDER_COST 1u

#define KTRI_COPY_WAIT_NONE 0xFFFFFFFFu

/* Counters of the last run on a context, named after the reference's Statistics fields
 * (include/cetric/statistics.h:193-199) where one exists. */
typedef struct ktri_run_stats {
    uint64_t triangles;               /* stats.local.local_triangles */
    uint64_t n;                       /* vertices */
    uint64_t nnz;                     /* stored adjacency entries (2m) */
    uint64_t oriented_edges;          /* m: out-list entries after orientation */
    uint64_t wedge_checks;            /* sum over oriented (v,u) of |N+(u)| (collect_stats) */
    uint64_t intersection_size_local; /* sum over oriented (v,u) of |N+(v)|+|N+(u)| (collect_stats) */
    uint64_t streamed_entries;        /* out-list entries the AUTO kernels stream (collect_stats) */
    uint32_t input_sorted;            /* 1 when every input adjacency list was strictly increasing */
    uint32_t method;                  /* strategy that ran */
    float ms_orient;                  /* device time of orientation (+ sort when one ran) */
    float ms_count;                   /* device time of intersection + reduction */
    float ms_total;                   /* device time of the whole call */
    float ms_count_small;             /* AUTO: device time of the small-owner tile kernel */
    float ms_count_large;             /* AUTO: device time of the large-owner vertex kernel */
    float ms_h2d;                     /* host-buffer calls: device time from the first input copy until the
                                         last piece of head has landed (orientation overlaps it) */
    float ms_d2h;                     /* host-buffer calls: device time of the read-back of the results */
    float ms_call;                    /* host-buffer calls: device time of the whole call, copies included */
    float host_ms_enqueue;            /* host-buffer calls: host time from entry until every copy and launch
                                         was enqueued (includes waiting where a copy to pageable memory blocks) */
    float host_ms_call;               /* host-buffer calls: host time of the whole call */
    uint64_t streamed_chunked;        /* entries the AUTO kernels stream, counted once per owner-table chunk
                                         that streams them (collect_stats); above streamed_entries only when
                                         some owner has more than 2048 out-neighbours */
} ktri_run_stats;

typedef struct ktri_ctx ktri_ctx;

/* ---- context ---------------------------------------------------------------------------- */
/* A context binds one CUDA device, owns a grow-only device workspace (oriented CSR, tables,
 * counters) and a pinned host staging buffer.  Calls on one context are serialised by the
 * caller; different contexts may be used from different threads. */
int ktri_ctx_create(int device, ktri_ctx** out);
int ktri_ctx_destroy(ktri_ctx* ctx);
/* Cap on the workspace this context may hold (bytes; 0 = no cap).  Over-budget calls fail
 * with KTRI_ERR_OUT_OF_MEMORY before launching anything. */
int ktri_ctx_set_memory_budget(ktri_ctx* ctx, uint64_t bytes);
/* Device bytes a count of a graph with n vertices and nnz entries needs in the workspace. */
uint64_t ktri_workspace_bytes(uint64_t n, uint64_t nnz, int32_t intersection_method);
const char* ktri_last_error(const ktri_ctx* ctx);
int ktri_ctx_stats(ktri_ctx* ctx, ktri_run_stats* out); /* synchronises the context's last stream */
const char* ktri_version(void);

/* ---- counting ----------------------------------------------------------------------------- */
/* Replaces: size_t cetric::run_shmem(DistributedGraph<>&, Statistics&, const Config&)
 *   (include/cetric/counters/shared_memory_cetric.h:105, called from apps/shmetric.cpp:140)
 * together with the preprocessing it runs (shared_memory_cetric.h:72-103: orient by
 * degree_outward, distributed_graph.h:148-163 and :538-566; sort_neighborhoods, :578-593)
 * and CetricEdgeIterator::run_local (include/cetric/counters/cetric_edge_iterator.h:173-227).
 * Host buffers in and out; copies to and from the device are part of the call; synchronous.
 * Where the device can address a host buffer (pinned or registered memory, or pageable memory
 * on platforms that let kernels address it, as Grace + Blackwell does) and its address is
 * 16-byte aligned, the copy is done by the GPU's own loads and stores; otherwise by the copy
 * engines.  A read-back of 1 MiB or more into pageable memory is staged in the context's pinned
 * buffer and copied by host threads after the call's synchronisation.  Pinned, 16-byte-aligned
 * buffers give the fastest calls.
 * per_vertex_out may be NULL; otherwise it receives n counts.  opts may be NULL.
 * Uses an internal context on the current CUDA device. */
int ktri_count_csr(const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz, uint64_t* total_out,
                   uint64_t* per_vertex_out, const ktri_opts* opts);

/* Same as ktri_count_csr on an explicit context (reuses its workspace and staging). */
int ktri_count_csr_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                       uint64_t* total_out, uint64_t* per_vertex_out, const ktri_opts* opts);

/* Device-resident variant, asynchronous on `stream` (a cudaStream_t, NULL = legacy default).
 * d_first_out, d_head: device CSR.  d_total: device u64.  d_per_vertex: device u64[n] or NULL.
 * Invalid-CSR conditions found on the device are reported by ktri_ctx_check. */
int ktri_count_csr_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n,
                          uint64_t nnz, uint64_t* d_total, uint64_t* d_per_vertex, const ktri_opts* opts,
                          void* stream);
/* Synchronise the context's last stream and report device-side CSR errors of the last call. */
int ktri_ctx_check(ktri_ctx* ctx);

/* No counterpart in the reference: a count that allocates no memory.  For callers that
 * cannot call cudaMalloc, such as a host runtime that owns all device memory through its
 * own pool (where an allocation outside the pool breaks its accounting and can synchronise
 * the device), or a latency-bound loop that must not pay for an allocation.  Same inputs and
 * outputs as ktri_count_csr_device with the AUTO method (d_per_vertex is required here), and
 * no context: the workspace is a fixed 64 MiB array in device memory, held by every GPU that
 * loads this library until the process exits.  A graph fits when
 * ktri_workspace_bytes(n, nnz, KTRI_METHOD_AUTO) <= 64 MiB (about 600 000 vertices with 16
 * adjacency entries each); larger graphs return KTRI_ERR_UNSUPPORTED before anything is
 * launched.
 * The first call on a device looks up the array's device address (with that device current;
 * again whenever the calling thread's CUDA context has changed, e.g. after cudaDeviceReset);
 * make that first call before any stream capture.  All calls on a
 * device share the one array and leave the last call's contents in it; calls whose work
 * overlaps on the GPU race on it, so serialise them.  Runs on `stream` and returns when that
 * work is done, with KTRI_ERR_INVALID_CSR for invalid input found on the device. */
int ktri_count_csr_device_noalloc(const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n, uint64_t nnz,
                                  uint64_t* d_total, uint64_t* d_per_vertex, void* stream);

/* ---- batches of graphs ---------------------------------------------------------------------
 * No counterpart in the reference (KaTric counts one graph per run).  Many independent graphs
 * are packed as one disjoint-union CSR: graph g owns the vertices [graph_first[g],
 * graph_first[g+1]) and its adjacency entries name only those vertices.  One launch sequence
 * counts every graph (the merge-path and owner tiles of all graphs share one device work
 * queue); totals[g] receives graph g's triangle count and per_vertex (optional) the union's
 * per-vertex counts.  ktri_batch_pack / ktri_batch_generate build such a union on the host. */
int ktri_count_batch_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                            uint64_t nnz_total, const uint64_t* d_graph_first, uint64_t num_graphs, uint64_t* d_totals,
                            uint64_t* d_per_vertex, const ktri_opts* opts, void* stream);
int ktri_count_batch_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n_total,
                         uint64_t nnz_total, const uint64_t* graph_first, uint64_t num_graphs, uint64_t* totals_out,
                         uint64_t* per_vertex_out, const ktri_opts* opts);

/* A captured plan: the launch sequence of one batch count recorded once as a CUDA graph and
 * replayed by ktri_plan_launch (one graph launch instead of one launch per kernel).  The plan
 * owns its workspace and is bound to the device buffers given here; refill those buffers with
 * another batch of the same n_total / nnz_total / num_graphs and launch again.
 * ktri_plan_check synchronises the last launch and reports invalid input found on the device.
 * Launch and check need the plan's context alive; destroy does not. */
typedef struct ktri_plan ktri_plan;
int ktri_plan_create_batch(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n_total,
                           uint64_t nnz_total, const uint64_t* d_graph_first, uint64_t num_graphs,
                           uint64_t* d_totals, uint64_t* d_per_vertex, const ktri_opts* opts, ktri_plan** out);
int ktri_plan_launch(ktri_plan* plan, void* stream);
int ktri_plan_check(ktri_plan* plan);
int ktri_plan_destroy(ktri_plan* plan);

/* ---- file ingest ---------------------------------------------------------------------------
 * The reference's binary graph format (shmetric --input-format binary, read by graph-io:
 * <stem>.first_out u64[n+1] and <stem>.head u64[nnz]) counted straight from the files: the
 * files are read in chunks of chunk_bytes (0 = 64 MiB) into two pinned buffers while the other
 * buffer's chunk is copied to the device, so the disk or page-cache read overlaps the transfer.
 * ktri_binary_file_shape reports n and nnz from the file sizes (to size per_vertex_out). */
int ktri_binary_file_shape(const char* stem, uint64_t* n_out, uint64_t* nnz_out);
int ktri_count_binary_file(ktri_ctx* ctx, const char* stem, uint64_t* total_out, uint64_t* per_vertex_out,
                           const ktri_opts* opts, uint64_t chunk_bytes);

/* ---- triangle listing ----------------------------------------------------------------------
 * The check run_shmem performs in debug builds (shared_memory_cetric.h:151-167: collect every
 * emitted triangle, sort, look for duplicates) needs the triangles themselves.
 * ktri_list_triangles writes up to `capacity` triangles as id triples (x < y < z, in no
 * particular order) and the total count; with more triangles than capacity it fills the
 * buffer, sets *count_out and returns KTRI_ERR_OUT_OF_MEMORY.  It runs the merge strategy. */
int ktri_list_triangles(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                        uint32_t* triples_out, uint64_t capacity, uint64_t* count_out);

/* ---- oriented lists: the katric local phase -----------------------------------------------
 * Replaces CetricEdgeIterator::run_local on one rank's graph (cetric_edge_iterator.h:173-227,
 * called from cetric.h:431,450 and :827,847), which walks lists the caller has already
 * oriented: out_adj of the local vertices and, in the variant with ghosts (:301-388), ghost_adj
 * of the ghosts.  Give every vertex (local and ghost, numbered 0..n-1) its list; m is the total
 * length.  The count is that of the triangles whose three edges appear in the lists, which is
 * what run_local finds, whatever orientation the caller used.  Every edge must appear in exactly
 * one of its endpoints' lists; lists may be in any order.  Out-of-range ids and self-loops are
 * reported as KTRI_ERR_INVALID_CSR; an edge listed at both endpoints is reported as a duplicate
 * where a shared-memory table meets it (not guaranteed).  Per-vertex counts are indexed like
 * the lists (ghosts included). */
int ktri_count_dag_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t m,
                       uint64_t* total_out, uint64_t* per_vertex_out, const ktri_opts* opts);
int ktri_count_dag_device(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n, uint64_t m,
                          uint64_t* d_total, uint64_t* d_per_vertex, const ktri_opts* opts, void* stream);

/* ---- contraction after the local phase ---------------------------------------------------
 * CeTriC-X contracts each rank's graph once its local phase is done (cetric.h:872-930):
 * remove_internal_edges keeps, per local vertex, only its out-edges to other ranks and drops
 * its in-edges (distributed_graph.h:680-764); compact drops the vertices left without edges and
 * renumbers the rest (:979-1056); the lists are then sorted by id.  ktri_contract_dag_ctx does
 * this on the device for lists numbered as ktri_count_dag's input: vertices 0..n_local-1 are
 * the rank's own, n_local..n-1 its ghosts.  Outputs (caller-sized: kept_out n_local entries,
 * out_first_out n_local + 1, out_head m): kept_out[k] = the list index of the k-th surviving
 * vertex, out_first_out / out_head its ghost out-neighbours sorted by id, *kept_count and
 * *edge_count the sizes. */
int ktri_contract_dag_ctx(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t n_local,
                          uint64_t m, uint32_t* kept_out, uint64_t* out_first_out, uint32_t* out_head,
                          uint64_t* kept_count, uint64_t* edge_count);

/* ---- load-balancing cost functions -------------------------------------------------------
 * The reference balances work across ranks by a per-vertex cost (cost_function.h:287-376,
 * chosen with --cost-function): N (1), D (degree), DH (out-degree), DDH (degree x out-degree),
 * DH2 (out-degree^2), DPD (sum over higher neighbours u of d+(v) + d+(u), the edge iterator's
 * merge work), IDPD (the same over lower neighbours).  Orientation is (degree, id).
 * ktri_partition_cost computes the costs on the device and cuts the vertex range into `parts`
 * ranges of about equal total cost: boundaries_out[0] = 0 <= ... <= boundaries_out[parts] = n.
 * costs_out (n entries) is optional. */
#define KTRI_COST_N 0
#define KTRI_COST_D 1
#define KTRI_COST_DH 2
#define KTRI_COST_DDH 3
#define KTRI_COST_DH2 4
#define KTRI_COST_DPD 5
#define KTRI_COST_IDPD 6
int ktri_partition_cost(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                        int32_t cost_function, uint32_t parts, uint64_t* boundaries_out, uint64_t* costs_out,
                        uint64_t* total_cost_out);

/* ---- autotuning ---------------------------------------------------------------------------
 * No counterpart in the reference (its strategy is a command-line choice, --intersection-method,
 * apps/parse_parameters.h:156-158).  ktri_autotune times candidate configurations of one count
 * of the given device input (one graph when d_graph_first is NULL, else a packed batch):
 * intersection strategy, small_outdegree, medium_outdegree and segment, and writes the fastest
 * into *opts (other fields are kept).  With a cache_path the choice is looked up first and, when
 * timed, appended as one JSON line keyed by the input's shape class (compute capability, SM
 * count, floor log2 of graphs, n, nnz and the largest degree).  The call synchronises `stream`. */
typedef struct ktri_tuning {
    uint32_t struct_size;
    int32_t intersection_method; /* the chosen configuration */
    uint32_t small_outdegree, medium_outdegree, segment;
    uint32_t from_cache;         /* 1: read from the cache file, nothing timed */
    uint32_t candidates;         /* configurations timed */
    uint32_t tile_order;         /* the chosen ktri_opts.tile_order */
    double ms;                   /* device time of one count with the chosen configuration */
    double default_ms;           /* the same with the library defaults (0 when read from the cache) */
    char signature[96];          /* the shape class */
} ktri_tuning;
int ktri_autotune(ktri_ctx* ctx, const uint64_t* d_first_out, const uint32_t* d_head, uint64_t n, uint64_t nnz,
                  const uint64_t* d_graph_first, uint64_t num_graphs, const char* cache_path, ktri_opts* opts,
                  ktri_tuning* out, void* stream);

/* ---- serving ------------------------------------------------------------------------------
 * No counterpart in the reference.  A request loop with continuous batching: requests (one
 * graph each) queue up; a worker thread packs the waiting ones into a batch under the device
 * memory budget and counts it on one of `slots` contexts, while batches already on the GPU
 * keep running (their work overlaps).  Counted graphs stay resident (CSR and counts on the
 * device, keyed by graph_key) until the budget needs their room; a request for a resident
 * key is answered from the resident counts (the per-vertex counts are also kept in host
 * memory, up to a quarter of memory_budget in all, so a repeat needs no device copy).  A key
 * names one graph: a graph of another n or nnz submitted under a resident key is counted and
 * replaces the resident one.  submit checks first_out (0 first, nnz last, non-decreasing:
 * KTRI_ERR_INVALID_CSR otherwise) and copies the caller's CSR, or with KTRI_SUBMIT_BORROW
 * reads it in place (the caller keeps it alive and unchanged until wait returns).  first_out
 * may be NULL to repeat a key that is resident, queued or counting, with n = 0 (any size) or
 * the vertex count that the caller's per-vertex buffer holds: a repeat whose key's graph has
 * another n fails with KTRI_ERR_INVALID_ARGUMENT instead of writing past that buffer.  A
 * request whose key is queued or counting (same n and nnz) joins that count instead of
 * starting another.  wait blocks until the request is done and reports its latency (submit
 * to completion). */
#define KTRI_SUBMIT_PER_VERTEX 1u /* return per-vertex counts */
#define KTRI_SUBMIT_BORROW 2u     /* read the caller's CSR in place instead of copying it */
typedef struct ktri_server ktri_server;
typedef struct ktri_server_opts {
    uint32_t struct_size;        /* sizeof(ktri_server_opts); 0 = defaults */
    uint32_t slots;              /* batches in flight at once (default 2) */
    uint64_t memory_budget;      /* device bytes for resident graphs and batches (default 120 GiB) */
    uint64_t max_batch_nnz;      /* adjacency entries per batch (default 2^28) */
    uint32_t max_batch_graphs;   /* graphs per batch (default 4096) */
    uint32_t direct_host_access; /* 1: where the device reads pageable host memory (Grace + Blackwell), kernels
                                    gather the callers' graphs and write per-vertex counts straight into host
                                    memory; 0 (default): batches go through pinned host staging.  Direct access
                                    lowers latency at low load, but the driver may migrate the touched pages to
                                    the GPU, which slows the callers' later host accesses */
    uint32_t engine;             /* 1: one persistent counting kernel (the engine) runs across batches; each batch
                                    is prepared on its slot (orientation, owner tiles) and published to the
                                    running engine as a job, so arrivals fold into the kernel that is already
                                    counting.  0 (default): one counting launch sequence per batch */
    uint32_t reserved[5];
} ktri_server_opts;
typedef struct ktri_server_stats {
    uint64_t submitted, completed, batches, batched_graphs, cache_hits, evictions, resident_graphs, resident_bytes,
        peak_inflight_batches;
    uint64_t coalesced; /* requests answered by the count of an earlier queued request with their key */
    uint64_t pack_us;    /* worker time spent packing batches and enqueueing their copies and counts */
    uint64_t alloc_us;   /* of pack_us: time spent growing the slots' device and pinned host buffers */
    uint64_t harvest_us; /* worker time spent reading back results and keeping graphs resident */
    uint64_t device_us;  /* device time of the batches (first copy to last read-back), summed */
    uint64_t engine_launches; /* launches of the persistent counting kernel (engine mode): it leaves when idle
                                 and is launched again by the next published batch */
    uint64_t reserved[1];
} ktri_server_stats;
int ktri_server_create(int device, const ktri_server_opts* opts, ktri_server** out);
int ktri_server_submit(ktri_server* s, uint64_t graph_key, const uint64_t* first_out, const uint32_t* head,
                       uint64_t n, uint64_t nnz, uint32_t flags, uint64_t* request_id);
int ktri_server_wait(ktri_server* s, uint64_t request_id, uint64_t* total, uint64_t* per_vertex_out,
                     double* latency_s);
int ktri_server_get_stats(ktri_server* s, ktri_server_stats* out);
int ktri_server_destroy(ktri_server* s);

/* Oriented, id-sorted out-lists (the state of DistributedGraph after preprocessing,
 * shared_memory_cetric.h:72-103, restricted to out_adj, distributed_graph.h:512-514) as a
 * compact CSR: out_first_out[n+1] and out_head[nnz/2].  Host buffers; synchronous. */
int ktri_orient_csr(ktri_ctx* ctx, const uint64_t* first_out, const uint32_t* head, uint64_t n, uint64_t nnz,
                    uint64_t* out_first_out, uint32_t* out_head);

/* Batched set intersection of sorted u32 lists on the device, one pair per entry:
 * pair i intersects a_vals[a_off[i]..a_off[i+1]) with b_vals[b_off[i]..b_off[i+1]) using
 * the given strategy (cetric::intersection, intersection.h:41-79).  counts_out[i] gets the
 * intersection size; if members_out is non-NULL it must hold a_off[npairs] entries and
 * pair i writes its members, in increasing order, from members_out[a_off[i]].  Host buffers. */
int ktri_intersect_pairs(ktri_ctx* ctx, int32_t method, const uint32_t* a_vals, const uint64_t* a_off,
                         const uint32_t* b_vals, const uint64_t* b_off, uint64_t npairs, uint64_t* counts_out,
                         uint32_t* members_out);

/* ---- graphs on the host: generators and file formats ------------------------------------- */
/* Replaces graphio::read_graph (apps/shmetric.cpp:119) and the KaGen generators behind
 * --gen (apps/parse_parameters.h:72-73) for the inputs this engine is measured on. */
typedef struct ktri_graph ktri_graph;
int ktri_graph_from_csr(uint64_t n, const uint64_t* first_out, const uint32_t* head, ktri_graph** out);
int ktri_graph_gnm(uint64_t n, uint64_t m, uint64_t seed, ktri_graph** out);
int ktri_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                    ktri_graph** out);
int ktri_graph_rmat_n(uint64_t n, uint64_t samples, double a, double b, double c, uint64_t seed, ktri_graph** out);
int ktri_graph_rgg2d(uint64_t n, double avg_degree, uint64_t seed, ktri_graph** out);
/* Disjoint union of graphs (graph_first needs num_graphs + 1 entries). */
int ktri_batch_pack(uint64_t num_graphs, const ktri_graph* const* graphs, ktri_graph** out, uint64_t* graph_first);
/* The batched workload: num_graphs graphs with n = round(2^U(log2_n_min, log2_n_max)),
 * average degree U(deg_min, deg_max), generator i mod 3 = G(n,m) / RMAT(0.57,0.19,0.19) / 2D
 * RGG, graph i seeded with seed + i; returned packed as one union. */
int ktri_batch_generate(uint64_t num_graphs, double log2_n_min, double log2_n_max, double deg_min, double deg_max,
                        uint64_t seed, ktri_graph** out, uint64_t* graph_first);
int ktri_graph_read_metis(const char* path, ktri_graph** out);
int ktri_graph_read_binary(const char* stem, ktri_graph** out);
int ktri_graph_write_binary(const ktri_graph* g, const char* stem);
int ktri_graph_write_metis(const ktri_graph* g, const char* path);
/* Many graphs from explicit specs in parallel: kinds[i] 0 = G(n,m) (m = round(n d / 2)),
 * 1 = RMAT (0.57, 0.19, 0.19) with round(n d / 2) draws, 2 = 2D RGG; outs[i] receives graph i. */
int ktri_graphs_generate(uint64_t count, const uint32_t* kinds, const uint64_t* ns, const double* degrees,
                         const uint64_t* seeds, ktri_graph** outs);
uint64_t ktri_graph_n(const ktri_graph* g);
uint64_t ktri_graph_nnz(const ktri_graph* g);
const uint64_t* ktri_graph_first_out(const ktri_graph* g);
const uint32_t* ktri_graph_head(const ktri_graph* g);
void ktri_graph_free(ktri_graph* g);

#ifdef __cplusplus
}
#endif
#endif /* KTRI_H */
