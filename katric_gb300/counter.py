"""Host mirror of KaTric's shared-memory counting interface, backed by the CUDA engine.

  run_shmem(G, stats, conf) -> int        cetric::run_shmem (include/cetric/counters/shared_memory_cetric.h:105)
  preprocessing(G, conf) -> (fo, head)    cetric::preprocessing (shared_memory_cetric.h:72-103): oriented,
                                          id-sorted out-lists
  intersection(a, b, conf) -> list        cetric::intersection (include/cetric/counters/intersection.h:41-79)
  Config                                  the hot-path knobs of cetric::Config (include/cetric/config.h:140-200)
  Statistics                              the counters run_shmem fills (include/cetric/statistics.h:193-217)

All counting runs on the GPU through libktri.so; nothing here computes triangles on the CPU.
Errors raise KtriError (the reference asserts or throws; the C ABI returns status codes).
"""
from __future__ import annotations

import ctypes
import dataclasses
import weakref
from typing import Optional

import numpy as np

from . import _native
from .graph import Batch, Graph

METHOD_BY_NAME = {
    "auto": _native.METHOD_AUTO,
    "merge": _native.METHOD_MERGE,
    "binary-search": _native.METHOD_BINARY_SEARCH,
    "binary_search": _native.METHOD_BINARY_SEARCH,
    "binary": _native.METHOD_BINARY,
    "hybrid": _native.METHOD_HYBRID,
}


@dataclasses.dataclass
class Config:
    """Hot-path fields of cetric::Config with the reference's defaults (config.h:140-200).

    intersection_method: "auto" (GPU default: owner-side shared-memory hash), or one of the
    reference's "merge" (its default), "binary-search", "binary", "hybrid".  Counts are
    identical for all five.  num_threads, pseudo2core, grainsize and the partitioning
    switches steer CPU threading in the reference; they are accepted and recorded, and do
    not change results.
    """
    intersection_method: str = "auto"
    binary_intersection_cutoff: int = 1000
    hybrid_cutoff_scale: float = 1.0
    num_threads: int = 1
    pseudo2core: bool = False
    edge_partitioning: bool = False
    local_degree_of_parallelism: int = 1
    high_degree_threshold_scale: float = 1.0
    iterations: int = 1
    per_vertex: bool = True
    collect_stats: bool = False
    device: int = 0
    force_wide_offsets: bool = False
    small_outdegree: int = 0    # owner bins of the "auto" kernels (0 = library default; see ktri_opts)
    medium_outdegree: int = 0
    segment: int = 0
    copy_wait_polls: int = 0    # bound on the large-owner kernel's first bulk-copy wait (0 = default;
                                # COPY_WAIT_NONE gives up at once, for tests of the timeout path)
    tile_order: int = 0         # 0: tiles by locality (default); 1: by streamed work, heaviest first

    def opts(self) -> _native.Opts:
        o = _native.Opts()
        o.struct_size = ctypes.sizeof(_native.Opts)
        try:
            o.intersection_method = METHOD_BY_NAME[self.intersection_method.lower()]
        except KeyError:
            raise ValueError(f"unknown intersection method {self.intersection_method!r}") from None
        o.small_outdegree = self.small_outdegree
        o.medium_outdegree = self.medium_outdegree
        o.segment = self.segment
        o.collect_stats = 1 if self.collect_stats else 0
        o.binary_intersection_cutoff = self.binary_intersection_cutoff
        o.hybrid_cutoff_scale = self.hybrid_cutoff_scale
        o.force_wide_offsets = 1 if self.force_wide_offsets else 0
        o.copy_wait_polls = self.copy_wait_polls
        o.tile_order = self.tile_order
        return o


@dataclasses.dataclass
class LocalStatistics:
    local_triangles: int = 0
    wedge_checks: int = 0
    intersection_size_local: int = 0
    oriented_edges: int = 0
    streamed_entries: int = 0
    input_sorted: bool = True
    local_phase_time: float = 0.0   # seconds, device time of intersection + reduction
    preprocessing_time: float = 0.0  # seconds, device time of orientation (+ sort)
    wedges: int = 0


@dataclasses.dataclass
class Statistics:
    """Filled by run_shmem: counted_triangles, per-vertex counts and phase timers."""
    local: LocalStatistics = dataclasses.field(default_factory=LocalStatistics)
    counted_triangles: int = 0
    per_vertex: Optional[np.ndarray] = None
    global_wall_time: float = 0.0


class TriangleCounter:
    """One library context on one GPU: owns the device workspace across calls."""

    def __init__(self, device: int = 0, memory_budget: int = 0):
        self._L = _native.load()
        h = ctypes.c_void_p()
        _native.check(self._L.ktri_ctx_create(device, ctypes.byref(h)))
        self._ctx = h
        self.device = device
        self._plans = weakref.WeakSet()  # plans bound to this context, closed before it
        if memory_budget:
            self.set_memory_budget(memory_budget)

    def close(self) -> None:
        for plan in list(getattr(self, "_plans", ())):
            plan.close()
        if getattr(self, "_ctx", None) is not None:
            self._L.ktri_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._ctx

    def set_memory_budget(self, nbytes: int) -> None:
        _native.check(self._L.ktri_ctx_set_memory_budget(self._ctx, nbytes), self._ctx)

    def _check(self, rc: int) -> None:
        _native.check(rc, self._ctx)

    def count(self, first_out, head, conf: Config | None = None, per_vertex: bool = True):
        """Host CSR in, (total, per-vertex counts or None) out; copies are part of the call."""
        conf = conf or Config()
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, nnz = len(fo) - 1, len(hd)
        total = ctypes.c_uint64(0)
        pv = np.zeros(max(n, 1), dtype=np.uint64) if per_vertex else None
        opts = conf.opts()
        self._check(self._L.ktri_count_csr_ctx(self._ctx, fo.ctypes.data, hd.ctypes.data if nnz else None, n, nnz,
                                               ctypes.byref(total), pv.ctypes.data if pv is not None else None,
                                               ctypes.byref(opts)))
        return int(total.value), (pv[:n] if pv is not None else None)

    def count_device(self, first_out_ptr: int, head_ptr: int, n: int, nnz: int, total_ptr: int,
                     per_vertex_ptr: int | None = None, conf: Config | None = None, stream: int = 0) -> None:
        """Device CSR in, device outputs; asynchronous on `stream` (a cudaStream_t as int)."""
        conf = conf or Config()
        opts = conf.opts()
        self._check(self._L.ktri_count_csr_device(self._ctx, first_out_ptr, head_ptr, n, nnz, total_ptr,
                                                  per_vertex_ptr, ctypes.byref(opts), stream or None))

    def count_binary_file(self, stem: str, conf: Config | None = None, per_vertex: bool = True,
                          chunk_bytes: int = 0):
        """Count <stem>.first_out / <stem>.head (the reference's binary format) straight from the
        files; reads overlap the host-to-device copies.  Returns (total, per-vertex or None)."""
        conf = conf or Config()
        n, nnz = ctypes.c_uint64(0), ctypes.c_uint64(0)
        path = str(stem).encode()
        _native.check(self._L.ktri_binary_file_shape(path, ctypes.byref(n), ctypes.byref(nnz)))
        total = ctypes.c_uint64(0)
        pv = np.zeros(max(1, n.value), dtype=np.uint64) if per_vertex else None
        opts = conf.opts()
        self._check(self._L.ktri_count_binary_file(self._ctx, path, ctypes.byref(total),
                                                   pv.ctypes.data if pv is not None else None, ctypes.byref(opts),
                                                   chunk_bytes))
        return int(total.value), (pv[: n.value] if pv is not None else None)

    def list_triangles(self, first_out, head, capacity: int | None = None) -> np.ndarray:
        """All triangles as a (count, 3) u32 array of ids x < y < z (unordered rows): the
        debug check of run_shmem (shared_memory_cetric.h:151-167).  With capacity=None the
        count is taken first."""
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, nnz = len(fo) - 1, len(hd)
        if capacity is None:
            capacity = self.count(fo, hd, Config(intersection_method="merge"), per_vertex=False)[0]
        out = np.zeros((max(1, capacity), 3), dtype=np.uint32)
        count = ctypes.c_uint64(0)
        self._check(self._L.ktri_list_triangles(self._ctx, fo.ctypes.data, hd.ctypes.data if nnz else None, n, nnz,
                                                out.ctypes.data, capacity, ctypes.byref(count)))
        return out[: int(count.value)]

    def count_dag(self, first_out, head, conf: Config | None = None, per_vertex: bool = True):
        """CetricEdgeIterator::run_local on lists the caller oriented (out_adj of local vertices,
        ghost_adj of ghosts): the triangles whose three edges appear in the lists.
        Returns (total, per-vertex counts or None)."""
        conf = conf or Config()
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, m = len(fo) - 1, len(hd)
        total = ctypes.c_uint64(0)
        pv = np.zeros(max(n, 1), dtype=np.uint64) if per_vertex else None
        opts = conf.opts()
        self._check(self._L.ktri_count_dag_ctx(self._ctx, fo.ctypes.data, hd.ctypes.data if m else None, n, m,
                                               ctypes.byref(total), pv.ctypes.data if pv is not None else None,
                                               ctypes.byref(opts)))
        return int(total.value), (pv[:n] if pv is not None else None)

    def contract_dag(self, first_out, head, n_local: int):
        """The contraction that follows the local phase (remove_internal_edges + compact +
        id sort, cetric.h:872-930) on lists numbered like count_dag's input (vertices
        0..n_local-1 local, the rest ghosts).  Returns (kept, first_out, head): the surviving
        local vertices and their ghost out-neighbours sorted by id."""
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, m = len(fo) - 1, len(hd)
        kept = np.zeros(max(1, n_local), dtype=np.uint32)
        ofo = np.zeros(n_local + 1, dtype=np.uint64)
        oh = np.zeros(max(1, m), dtype=np.uint32)
        k, e = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(self._L.ktri_contract_dag_ctx(self._ctx, fo.ctypes.data, hd.ctypes.data if m else None, n, n_local,
                                                  m, kept.ctypes.data, ofo.ctypes.data, oh.ctypes.data,
                                                  ctypes.byref(k), ctypes.byref(e)))
        return kept[: k.value].copy(), ofo[: k.value + 1].copy(), oh[: e.value].copy()

    COST_FUNCTIONS = {"N": 0, "D": 1, "DH": 2, "DDH": 3, "DH2": 4, "DPD": 5, "IDPD": 6}

    def partition_cost(self, first_out, head, cost_function: str = "DPD", parts: int = 1, costs: bool = False):
        """The reference's load-balancing cost functions (cost_function.h:287-376) on the device:
        (boundaries of `parts` vertex ranges of about equal cost, total cost, per-vertex costs
        or None)."""
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, nnz = len(fo) - 1, len(hd)
        bnd = np.zeros(parts + 1, dtype=np.uint64)
        cst = np.zeros(max(1, n), dtype=np.uint64) if costs else None
        total = ctypes.c_uint64(0)
        self._check(self._L.ktri_partition_cost(self._ctx, fo.ctypes.data, hd.ctypes.data if nnz else None, n, nnz,
                                                self.COST_FUNCTIONS[cost_function], parts, bnd.ctypes.data,
                                                cst.ctypes.data if cst is not None else None, ctypes.byref(total)))
        return bnd, int(total.value), (cst[:n] if cst is not None else None)

    def count_dag_device(self, first_out_ptr: int, head_ptr: int, n: int, m: int, total_ptr: int,
                         per_vertex_ptr: int | None = None, conf: Config | None = None, stream: int = 0) -> None:
        conf = conf or Config()
        opts = conf.opts()
        self._check(self._L.ktri_count_dag_device(self._ctx, first_out_ptr, head_ptr, n, m, total_ptr,
                                                  per_vertex_ptr, ctypes.byref(opts), stream or None))

    def check(self) -> None:
        self._check(self._L.ktri_ctx_check(self._ctx))

    def stats(self) -> _native.RunStats:
        st = _native.RunStats()
        self._check(self._L.ktri_ctx_stats(self._ctx, ctypes.byref(st)))
        return st

    def count_batch(self, batch: Batch, conf: Config | None = None, per_vertex: bool = True):
        """Host batch in, (per-graph totals, union per-vertex counts or None) out; one launch sequence."""
        conf = conf or Config()
        fo, hd, gf = batch.union.first_out, batch.union.head, batch.graph_first
        n, nnz, k = batch.union.n, batch.union.nnz, batch.num_graphs
        totals = np.zeros(max(1, k), dtype=np.uint64)
        pv = np.zeros(max(1, n), dtype=np.uint64) if per_vertex else None
        opts = conf.opts()
        self._check(self._L.ktri_count_batch_ctx(self._ctx, fo.ctypes.data, hd.ctypes.data if nnz else None, n, nnz,
                                                 gf.ctypes.data, k, totals.ctypes.data,
                                                 pv.ctypes.data if pv is not None else None, ctypes.byref(opts)))
        return totals[:k], (pv[:n] if pv is not None else None)

    def count_batch_device(self, first_out_ptr: int, head_ptr: int, n_total: int, nnz_total: int,
                           graph_first_ptr: int, num_graphs: int, totals_ptr: int, per_vertex_ptr: int | None = None,
                           conf: Config | None = None, stream: int = 0) -> None:
        conf = conf or Config()
        opts = conf.opts()
        self._check(self._L.ktri_count_batch_device(self._ctx, first_out_ptr, head_ptr, n_total, nnz_total,
                                                    graph_first_ptr, num_graphs, totals_ptr, per_vertex_ptr,
                                                    ctypes.byref(opts), stream or None))

    def plan_batch(self, first_out_ptr: int, head_ptr: int, n_total: int, nnz_total: int, graph_first_ptr: int,
                   num_graphs: int, totals_ptr: int, per_vertex_ptr: int | None = None,
                   conf: Config | None = None) -> "Plan":
        """Capture one batch count as a CUDA graph bound to these device buffers."""
        conf = conf or Config()
        opts = conf.opts()
        h = ctypes.c_void_p()
        self._check(self._L.ktri_plan_create_batch(self._ctx, first_out_ptr, head_ptr, n_total, nnz_total,
                                                   graph_first_ptr, num_graphs, totals_ptr, per_vertex_ptr,
                                                   ctypes.byref(opts), ctypes.byref(h)))
        plan = Plan(self, h)
        self._plans.add(plan)
        return plan

    def autotune(self, first_out_ptr: int, head_ptr: int, n: int, nnz: int, graph_first_ptr: int | None = None,
                 num_graphs: int = 0, cache_path: str | None = None, conf: Config | None = None,
                 stream: int = 0) -> tuple[Config, dict]:
        """Time candidate configurations of one count of this device input (a packed batch when
        graph_first_ptr is given) and return (conf with the fastest strategy, owner bins and
        segment, details).  With cache_path the choice is read from / appended to that JSON-lines
        file, keyed by the input's shape class."""
        conf = conf or Config()
        opts = conf.opts()
        res = _native.Tuning()
        res.struct_size = ctypes.sizeof(_native.Tuning)
        path = cache_path.encode() if cache_path else None
        self._check(self._L.ktri_autotune(self._ctx, first_out_ptr, head_ptr, n, nnz, graph_first_ptr,
                                          num_graphs if graph_first_ptr else 0, path, ctypes.byref(opts),
                                          ctypes.byref(res), stream or None))
        name = {v: k for k, v in METHOD_BY_NAME.items() if "_" not in k}[res.intersection_method]
        tuned = dataclasses.replace(conf, intersection_method=name, small_outdegree=res.small_outdegree,
                                    medium_outdegree=res.medium_outdegree, segment=res.segment,
                                    tile_order=res.tile_order)
        info = {"from_cache": bool(res.from_cache), "candidates": int(res.candidates), "ms": float(res.ms),
                "default_ms": float(res.default_ms), "signature": res.signature.decode()}
        return tuned, info

    def orient(self, first_out, head):
        """Oriented, id-sorted out-lists as a compact CSR (u64 offsets, u32 ids)."""
        fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        hd = np.ascontiguousarray(head, dtype=np.uint32)
        n, nnz = len(fo) - 1, len(hd)
        ofo = np.zeros(n + 1, dtype=np.uint64)
        oh = np.zeros(max(1, nnz // 2 + 1), dtype=np.uint32)
        self._check(self._L.ktri_orient_csr(self._ctx, fo.ctypes.data, hd.ctypes.data if nnz else None, n, nnz,
                                            ofo.ctypes.data, oh.ctypes.data))
        return ofo, oh[: int(ofo[-1])].copy()

    def intersect_pairs(self, pairs, method: str = "merge", members: bool = True):
        """Intersect each (a, b) pair of sorted u32 lists on the device.

        Returns a list of intersections (lists) when members is true, else the sizes."""
        a_lists = [np.ascontiguousarray(a, dtype=np.uint32) for a, _ in pairs]
        b_lists = [np.ascontiguousarray(b, dtype=np.uint32) for _, b in pairs]
        a_off = np.zeros(len(pairs) + 1, dtype=np.uint64)
        b_off = np.zeros(len(pairs) + 1, dtype=np.uint64)
        a_off[1:] = np.cumsum([len(a) for a in a_lists]) if pairs else []
        b_off[1:] = np.cumsum([len(b) for b in b_lists]) if pairs else []
        av = np.concatenate(a_lists) if a_lists and a_off[-1] else np.zeros(1, np.uint32)
        bv = np.concatenate(b_lists) if b_lists and b_off[-1] else np.zeros(1, np.uint32)
        counts = np.zeros(max(1, len(pairs)), dtype=np.uint64)
        mem = np.zeros(max(1, int(a_off[-1])), dtype=np.uint32) if members else None
        self._check(self._L.ktri_intersect_pairs(self._ctx, METHOD_BY_NAME[method], av.ctypes.data,
                                                 a_off.ctypes.data, bv.ctypes.data, b_off.ctypes.data, len(pairs),
                                                 counts.ctypes.data, mem.ctypes.data if mem is not None else None))
        if not members:
            return [int(c) for c in counts[: len(pairs)]]
        return [[int(x) for x in mem[int(a_off[i]): int(a_off[i]) + int(counts[i])]] for i in range(len(pairs))]


class Plan:
    """A captured batch count (CUDA graph); launch() replays it on a stream."""

    def __init__(self, counter: TriangleCounter, handle):
        self._counter = counter
        self._h = handle

    def launch(self, stream: int = 0) -> None:
        self._counter._check(self._counter._L.ktri_plan_launch(self._h, stream or None))

    def check(self) -> None:
        self._counter._check(self._counter._L.ktri_plan_check(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._counter._L.ktri_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default: dict[int, TriangleCounter] = {}


def default_counter(device: int = 0) -> TriangleCounter:
    if device not in _default:
        _default[device] = TriangleCounter(device)
    return _default[device]


def run_shmem(G: Graph, stats: Statistics, conf: Config) -> int:
    """cetric::run_shmem: orientation + sort + local phase on G; returns the triangle count.

    Unlike the reference, G is not modified (the engine orients a device copy); the
    per-vertex counts are left in stats.per_vertex."""
    ctr = default_counter(conf.device)
    c2 = dataclasses.replace(conf, collect_stats=conf.collect_stats)
    total, pv = ctr.count(G.first_out, G.head, c2, per_vertex=conf.per_vertex)
    st = ctr.stats()
    stats.counted_triangles = total
    stats.per_vertex = pv
    stats.local.local_triangles = total
    stats.local.wedge_checks = int(st.wedge_checks)
    stats.local.intersection_size_local = int(st.intersection_size_local)
    stats.local.oriented_edges = int(st.oriented_edges)
    stats.local.streamed_entries = int(st.streamed_entries)
    stats.local.input_sorted = bool(st.input_sorted)
    stats.local.preprocessing_time = st.ms_orient / 1e3
    stats.local.local_phase_time = st.ms_count / 1e3
    stats.global_wall_time = st.ms_total / 1e3
    return total


def preprocessing(G: Graph, conf: Config | None = None):
    """Oriented out-lists after orient(degree_outward) + sort_neighborhoods(id), as a compact CSR."""
    return default_counter((conf or Config()).device).orient(G.first_out, G.head)


def intersection(a, b, conf: Config | None = None) -> list[int]:
    """cetric::intersection of two sorted lists with conf.intersection_method, on the device."""
    conf = conf or Config(intersection_method="merge")
    return default_counter(conf.device).intersect_pairs([(a, b)], method=conf.intersection_method)[0]
