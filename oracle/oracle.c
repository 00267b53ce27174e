/*
 * TEST INFRASTRUCTURE ONLY — the CPU oracle for exact local triangle counting.
 *
 * This file restates, in plain C, the algorithm of KaTric's shared-memory local
 * counting path so that the CUDA product path can be checked against it.  It is
 * never linked into the product library: only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference leg load it.
 *
 * Restated reference functions (paths relative to the KaTric source tree):
 *   - node_ordering::degree_outward      include/cetric/datastructures/distributed/distributed_graph.h:148-163
 *   - DistributedGraph::orient            include/cetric/datastructures/distributed/distributed_graph.h:538-566
 *   - DistributedGraph::sort_neighborhoods include/cetric/datastructures/distributed/distributed_graph.h:578-593
 *   - preprocessing                       include/cetric/counters/shared_memory_cetric.h:72-103
 *   - run_shmem (emit + combine)          include/cetric/counters/shared_memory_cetric.h:105-170
 *   - run_local_sequential                include/cetric/counters/cetric_edge_iterator.h:230-298
 *   - run_local_parallel (node-parallel)  include/cetric/counters/cetric_edge_iterator.h:889-1066
 *   - intersection dispatch + hybrid      include/cetric/counters/intersection.h:41-79
 *   - merge_intersection                  include/cetric/counters/intersection.h:82-96
 *   - binary_search_intersection          include/cetric/counters/intersection.h:99-117
 *   - binary_intersection (explicit stack) include/cetric/counters/intersection.h:120-192
 *   - cetric::log2 (integer floor)        include/cetric/util.h:136-150
 *
 * Per-vertex counts have no counterpart in the reference (it only emits
 * Triangle{v,u,w} to a callback, shared_memory_cetric.h:131-142).  They are
 * defined here as: for every emitted triangle {v,u,w}, add one to v, u and w.
 *
 * Ids are u32 (the reference packs a 16-bit rank into a u64, graph_definitions.h:48-161;
 * on one rank the rank bits are constant and .id() is the plain id).  Offsets are u64.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORC_MERGE = 0, ORC_BINARY_SEARCH = 1, ORC_BINARY = 2, ORC_HYBRID = 3 };

typedef struct {
    uint64_t triangles;               /* total, stats.local.local_triangles */
    uint64_t wedge_checks;            /* sum over oriented edges (v,u) of |N+(u)|, cetric_edge_iterator.h:279 */
    uint64_t intersection_size_local; /* sum of |N+(v)| + |N+(u)|, cetric_edge_iterator.h:280-281 */
    uint64_t skipped_nodes;           /* pseudo2core skips */
    double orientation_s;             /* phase timers, shared_memory_cetric.h:74-102 */
    double sorting_s;
    double local_phase_s;
} orc_stats;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---- intersection strategies (intersection.h) ----------------------------------- */

typedef struct {
    uint64_t* cnt;      /* per-vertex counts or NULL */
    uint32_t v, u;      /* the oriented edge whose intersection is being taken */
    uint64_t hits;      /* triangles found by this intersection */
    uint32_t* out;      /* optional: write intersected values (known-answer tests) */
    uint64_t out_len;
    int atomic;         /* per-vertex adds must be atomic (OpenMP mode) */
} emit_t;

static inline void add_count(uint64_t* c, uint32_t x, int atomic) {
    if (atomic) {
#pragma omp atomic
        c[x] += 1;
    } else {
        c[x] += 1;
    }
}

static inline void on_intersection(emit_t* e, uint32_t w) {
    e->hits++;
    if (e->out) e->out[e->out_len++] = w;
    if (e->cnt) {
        add_count(e->cnt, e->v, e->atomic);
        add_count(e->cnt, e->u, e->atomic);
        add_count(e->cnt, w, e->atomic);
    }
}

/* merge_intersection, intersection.h:82-96 */
static void merge_isect(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb, emit_t* e) {
    uint64_t i = 0, j = 0;
    while (i != na && j != nb) {
        if (a[i] < b[j]) {
            ++i;
        } else if (b[j] < a[i]) {
            ++j;
        } else {
            on_intersection(e, a[i]);
            ++i;
            ++j;
        }
    }
}

/* std::binary_search over a sorted range */
static int bsearch_u32(const uint32_t* a, uint64_t n, uint32_t key) {
    uint64_t lo = 0, hi = n; /* first index with a[idx] >= key */
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo < n && !(key < a[lo]);
}

/* std::lower_bound */
static uint64_t lower_bound_u32(const uint32_t* a, uint64_t n, uint32_t key) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* binary_search_intersection, intersection.h:99-117: probe the shorter list into the longer */
static void bsearch_isect(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb, emit_t* e) {
    if (na <= nb) {
        for (uint64_t i = 0; i < na; ++i)
            if (bsearch_u32(b, nb, a[i])) on_intersection(e, a[i]);
    } else {
        for (uint64_t j = 0; j < nb; ++j)
            if (bsearch_u32(a, na, b[j])) on_intersection(e, b[j]);
    }
}

/* binary_intersection with an explicit task stack, intersection.h:120-192 */
typedef struct { uint64_t f1, l1, f2, l2; } isect_task;

static void binary_isect(const uint32_t* A, uint64_t na, const uint32_t* B, uint64_t nb, uint64_t cutoff, emit_t* e) {
    uint64_t cap = 64, top = 0;
    isect_task* st = (isect_task*)malloc(cap * sizeof(isect_task));
    st[top++] = (isect_task){0, na, 0, nb};
    while (top) {
        isect_task t = st[--top];
        uint64_t d1 = t.l1 - t.f1, d2 = t.l2 - t.f2;
        if (d1 <= cutoff && d2 <= cutoff) {
            merge_isect(A + t.f1, d1, B + t.f2, d2, e);
            continue;
        }
        if (d1 == 0 || d2 == 0) continue;
        isect_task lo, hi;
        int push_lo, push_hi, hit = 0;
        uint64_t p1, p2; /* absolute indices */
        if (d1 <= d2) {
            p1 = t.f1 + d1 / 2;
            p2 = t.f2 + lower_bound_u32(B + t.f2, d2, A[p1]);
            push_lo = !(p1 == t.l1 && p2 == t.l2);
            lo = (isect_task){t.f1, p1, t.f2, p2};
            if (p2 != t.l2 && !(A[p1] < B[p2])) {
                hit = 1;
                on_intersection(e, A[p1]);
                p1++;
                p2++;
            }
            push_hi = !(p1 == t.f1 && p2 == t.f2);
            hi = (isect_task){p1, t.l1, p2, t.l2};
        } else {
            p2 = t.f2 + d2 / 2;
            p1 = t.f1 + lower_bound_u32(A + t.f1, d1, B[p2]);
            push_lo = !(p2 == t.l2 && p1 == t.l1);
            lo = (isect_task){t.f1, p1, t.f2, p2};
            if (p1 != t.l1 && !(B[p2] < A[p1])) {
                hit = 1;
                on_intersection(e, B[p2]);
                p1++;
                p2++;
            }
            push_hi = !(p2 == t.f2 && p1 == t.f1);
            hi = (isect_task){p1, t.l1, p2, t.l2};
        }
        (void)hit;
        if (top + 2 > cap) {
            cap *= 2;
            st = (isect_task*)realloc(st, cap * sizeof(isect_task));
        }
        if (push_lo) st[top++] = lo;
        if (push_hi) st[top++] = hi;
    }
    free(st);
}

/* cetric::log2, util.h:136-150: floor(log2(x)) for x > 0 */
static uint64_t ilog2_u64(uint64_t x) {
    uint64_t r = 0;
    while (x >>= 1) ++r;
    return r;
}

/* intersection dispatch incl. hybrid rule, intersection.h:41-79 */
static void intersect(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb, int method,
                      uint64_t cutoff, double hybrid_scale, emit_t* e) {
    switch (method) {
        case ORC_MERGE: merge_isect(a, na, b, nb, e); break;
        case ORC_BINARY_SEARCH: bsearch_isect(a, na, b, nb, e); break;
        case ORC_BINARY: binary_isect(a, na, b, nb, cutoff, e); break;
        default: {
            uint64_t d1 = na, d2 = nb;
            if (d2 < d1) { uint64_t t = d1; d1 = d2; d2 = t; }
            /* d2 == 0 implies an empty result; the reference would call log2(0) there */
            if (d2 > 0 && (double)(d1 * ilog2_u64(d2)) < hybrid_scale * (double)(d1 + d2))
                bsearch_isect(a, na, b, nb, e);
            else
                merge_isect(a, na, b, nb, e);
        }
    }
}

/* Known-answer hook: intersect two sorted lists with one method and write the result. */
uint64_t orc_intersect(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb, int method,
                       uint64_t cutoff, double hybrid_scale, uint32_t* out) {
    emit_t e;
    memset(&e, 0, sizeof e);
    e.out = out;
    intersect(a, na, b, nb, method, cutoff, hybrid_scale, &e);
    return e.hits;
}

/* ---- orientation and sorting (distributed_graph.h) -------------------------------- */

/* degree_outward: u is an out-neighbour of v iff (deg(v), v) < (deg(u), u), distributed_graph.h:148-163 */
static inline int is_outgoing(uint64_t dv, uint32_t v, uint64_t du, uint32_t u) {
    return dv < du || (dv == du && v < u);
}

/* DistributedGraph::orient, distributed_graph.h:538-566: in-place two-pointer partition of the
 * adjacency of v into [in-neighbours | out-neighbours]; returns the split offset. */
static uint64_t orient_vertex(uint32_t* head, const uint64_t* fo, uint32_t v) {
    uint64_t dv = fo[v + 1] - fo[v];
    int64_t left = (int64_t)fo[v];
    int64_t right = (int64_t)fo[v] + (int64_t)dv - 1;
#define DEG(x) (fo[(x) + 1] - fo[(x)])
    while (left <= right) {
        while (left <= right && !is_outgoing(dv, v, DEG(head[left]), head[left])) left++;
        while (right >= (int64_t)fo[v] && is_outgoing(dv, v, DEG(head[right]), head[right])) right--;
        if (left <= right) {
            uint32_t t = head[left];
            head[left] = head[right];
            head[right] = t;
        }
    }
#undef DEG
    return (uint64_t)left - fo[v];
}

static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return (x > y) - (x < y);
}

/* sort_neighborhoods by id, distributed_graph.h:578-593: sort the in part and the out part separately */
static void sort_vertex(uint32_t* head, const uint64_t* fo, const uint64_t* offset, uint32_t v) {
    uint64_t b = fo[v], in_end = fo[v] + offset[v], out_end = fo[v + 1];
    qsort(head + b, in_end - b, sizeof(uint32_t), cmp_u32);
    qsort(head + in_end, out_end - in_end, sizeof(uint32_t), cmp_u32);
}

/* preprocessing, shared_memory_cetric.h:72-103, on a caller-provided mutable copy of head.
 * offset[v] receives the in/out split (first_out_offset_). */
void orc_preprocess(uint64_t n, const uint64_t* fo, uint32_t* head, uint64_t* offset, int num_threads,
                    orc_stats* st) {
    double t0 = now_s();
#ifdef _OPENMP
    if (num_threads > 1) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(num_threads)
        for (int64_t v = 0; v < (int64_t)n; ++v) offset[v] = orient_vertex(head, fo, (uint32_t)v);
    } else
#endif
    {
        for (uint64_t v = 0; v < n; ++v) offset[v] = orient_vertex(head, fo, (uint32_t)v);
    }
    double t1 = now_s();
#ifdef _OPENMP
    if (num_threads > 1) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(num_threads)
        for (int64_t v = 0; v < (int64_t)n; ++v) sort_vertex(head, fo, offset, (uint32_t)v);
    } else
#endif
    {
        for (uint64_t v = 0; v < n; ++v) sort_vertex(head, fo, offset, (uint32_t)v);
    }
    double t2 = now_s();
    if (st) {
        st->orientation_s = t1 - t0;
        st->sorting_s = t2 - t1;
    }
}

/* Edge iterator over a preprocessed graph: run_local_sequential (cetric_edge_iterator.h:230-298)
 * when num_threads <= 1, else the node-parallel run_local_parallel (:889-1066).  On one rank
 * NodeOrdering = id_outward(0) differs from the orientation order, so the offset is 0
 * (:275-277); every oriented edge (v,u) intersects N+(v) with N+(u). */
void orc_local_phase(uint64_t n, const uint64_t* fo, const uint32_t* head, const uint64_t* offset, int method,
                     uint64_t cutoff, double hybrid_scale, int pseudo2core, int num_threads, uint64_t* per_vertex,
                     orc_stats* st) {
    double t0 = now_s();
    uint64_t tri = 0, wedges = 0, isz = 0, skipped = 0;
    if (per_vertex) memset(per_vertex, 0, n * sizeof(uint64_t));
    int par = 0;
#ifdef _OPENMP
    par = num_threads > 1;
#endif
#pragma omp parallel for schedule(dynamic, 64) num_threads(num_threads) reduction(+ : tri, wedges, isz, skipped) if (par)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint32_t v = (uint32_t)vi;
        const uint32_t* nv = head + fo[v] + offset[v];
        uint64_t dv = fo[v + 1] - fo[v] - offset[v];
        if (pseudo2core && dv < 2) {
            skipped++;
            continue;
        }
        for (uint64_t k = 0; k < dv; ++k) {
            uint32_t u = nv[k];
            const uint32_t* nu = head + fo[u] + offset[u];
            uint64_t du = fo[u + 1] - fo[u] - offset[u];
            wedges += du;
            isz += dv + du;
            emit_t e;
            memset(&e, 0, sizeof e);
            e.cnt = per_vertex;
            e.v = v;
            e.u = u;
            e.atomic = par;
            intersect(nv, dv, nu, du, method, cutoff, hybrid_scale, &e);
            tri += e.hits;
        }
    }
    if (st) {
        st->triangles = tri;
        st->wedge_checks = wedges;
        st->intersection_size_local = isz;
        st->skipped_nodes = skipped;
        st->local_phase_s = now_s() - t0;
    }
}

/* run_shmem, shared_memory_cetric.h:105-170: preprocessing + local phase on a mutable copy.
 * work_head must hold a copy of head (it is permuted in place, as the reference permutes G).
 * Returns the triangle count. */
uint64_t orc_run_shmem(uint64_t n, const uint64_t* fo, uint32_t* work_head, int method, uint64_t cutoff,
                       double hybrid_scale, int pseudo2core, int num_threads, uint64_t* per_vertex, orc_stats* st) {
    uint64_t* offset = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
    orc_stats local;
    memset(&local, 0, sizeof local);
    orc_preprocess(n, fo, work_head, offset, num_threads, &local);
    orc_local_phase(n, fo, work_head, offset, method, cutoff, hybrid_scale, pseudo2core, num_threads, per_vertex,
                    &local);
    free(offset);
    if (st) *st = local;
    return local.triangles;
}

/* Oriented CSR (out-lists only, sorted by id) for orientation tests: out_fo has n+1 entries,
 * out_head has room for nnz/2 entries.  Uses the same orient + sort as preprocessing. */
uint64_t orc_oriented_csr(uint64_t n, const uint64_t* fo, const uint32_t* head, uint64_t* out_fo, uint32_t* out_head) {
    uint64_t nnz = fo[n];
    uint32_t* work = (uint32_t*)malloc((nnz ? nnz : 1) * sizeof(uint32_t));
    uint64_t* offset = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
    memcpy(work, head, nnz * sizeof(uint32_t));
    orc_preprocess(n, fo, work, offset, 1, NULL);
    uint64_t pos = 0;
    out_fo[0] = 0;
    for (uint64_t v = 0; v < n; ++v) {
        uint64_t b = fo[v] + offset[v], e = fo[v + 1];
        memcpy(out_head + pos, work + b, (e - b) * sizeof(uint32_t));
        pos += e - b;
        out_fo[v + 1] = pos;
    }
    free(work);
    free(offset);
    return pos;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Slice of a vertex set by a hash of the id: vertex v belongs to slice hash(v) mod slices. */
static inline uint64_t slice_of(uint32_t v, uint64_t slices) {
    uint64_t h = (uint64_t)v * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    return h % slices;
}

/* One timed piece of a full run_shmem count, for the CPU baseline: the vertices of one hash
 * slice have their lists copied back from the input, oriented and id-sorted (the per-vertex
 * work of preprocessing, shared_memory_cetric.h:72-103), then the node-parallel local phase
 * (cetric_edge_iterator.h:889-1066, merge or the configured strategy) runs over the same
 * vertices as tails.  work_head/offset must hold a fully preprocessed graph (orc_preprocess)
 * so that the out-lists of the other slices are in place; re-orienting a slice reproduces the
 * same lists.  Running the slices 0..slices-1 once each does the work of exactly one count.
 * Returns the triangles whose tail vertex is in the slice; *adj_out receives the slice's
 * degree sum (twice its share of the undirected edges; the slices' sums add up to nnz). */
uint64_t orc_count_slice(uint64_t n, const uint64_t* fo, const uint32_t* head, uint32_t* work_head, uint64_t* offset,
                         uint64_t slice, uint64_t slices, int method, int num_threads, uint64_t* adj_out,
                         orc_stats* st) {
    if (slices == 0) slices = 1;
    double t0 = now_s();
    uint64_t deg2 = 0;
#pragma omp parallel for schedule(dynamic, 256) num_threads(num_threads) reduction(+ : deg2)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint32_t v = (uint32_t)vi;
        if (slice_of(v, slices) != slice) continue;
        uint64_t b = fo[v], e = fo[v + 1];
        memcpy(work_head + b, head + b, (e - b) * sizeof(uint32_t));
        offset[v] = orient_vertex(work_head, fo, v);
        deg2 += e - b;
    }
    double t1 = now_s();
#pragma omp parallel for schedule(dynamic, 256) num_threads(num_threads)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint32_t v = (uint32_t)vi;
        if (slice_of(v, slices) != slice) continue;
        sort_vertex(work_head, fo, offset, v);
    }
    double t2 = now_s();
    uint64_t tri = 0, wedges = 0, isz = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(num_threads) reduction(+ : tri, wedges, isz)
    for (int64_t vi = 0; vi < (int64_t)n; ++vi) {
        uint32_t v = (uint32_t)vi;
        if (slice_of(v, slices) != slice) continue;
        const uint32_t* nv = work_head + fo[v] + offset[v];
        uint64_t dv = fo[v + 1] - fo[v] - offset[v];
        for (uint64_t k = 0; k < dv; ++k) {
            uint32_t u = nv[k];
            const uint32_t* nu = work_head + fo[u] + offset[u];
            uint64_t du = fo[u + 1] - fo[u] - offset[u];
            wedges += du;
            isz += dv + du;
            emit_t em;
            memset(&em, 0, sizeof em);
            intersect(nv, dv, nu, du, method, 1000, 1.0, &em);
            tri += em.hits;
        }
    }
    double t3 = now_s();
    if (adj_out) *adj_out = deg2;
    if (st) {
        memset(st, 0, sizeof *st);
        st->triangles = tri;
        st->wedge_checks = wedges;
        st->intersection_size_local = isz;
        st->orientation_s = t1 - t0;
        st->sorting_s = t2 - t1;
        st->local_phase_s = t3 - t2;
    }
    return tri;
}
