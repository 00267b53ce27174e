"""ctypes binding of libktri.so (the C ABI declared in include/ktri.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_INVALID_CSR = -2
ERR_OUT_OF_MEMORY = -3
ERR_CUDA = -4
ERR_TIMEOUT = -5
ERR_UNSUPPORTED = -6
ERR_IO = -7
ERR_NO_DEVICE = -8

METHOD_AUTO, METHOD_MERGE, METHOD_BINARY_SEARCH, METHOD_BINARY, METHOD_HYBRID = 0, 1, 2, 3, 4
COPY_WAIT_NONE = 0xFFFFFFFF  # KTRI_COPY_WAIT_NONE
TILE_ORDER_COST = 1  # KTRI_TILE_ORDER_COST

ERROR_NAMES = {
    ERR_INVALID_ARGUMENT: "invalid argument",
    ERR_INVALID_CSR: "invalid CSR",
    ERR_OUT_OF_MEMORY: "out of memory",
    ERR_CUDA: "CUDA error",
    ERR_TIMEOUT: "timeout",
    ERR_UNSUPPORTED: "unsupported",
    ERR_IO: "I/O error",
    ERR_NO_DEVICE: "no CUDA device",
}


class KtriError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        self.code = code
        super().__init__(f"{ERROR_NAMES.get(code, 'error')} ({code}){': ' + msg if msg else ''}")


class Opts(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("intersection_method", ctypes.c_int32),
        ("small_outdegree", ctypes.c_uint32),
        ("collect_stats", ctypes.c_uint32),
        ("binary_intersection_cutoff", ctypes.c_uint64),
        ("hybrid_cutoff_scale", ctypes.c_double),
        ("force_wide_offsets", ctypes.c_uint32),
        ("medium_outdegree", ctypes.c_uint32),
        ("segment", ctypes.c_uint32),
        ("copy_wait_polls", ctypes.c_uint32),
        ("tile_order", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 3),
    ]


class ServerOpts(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("slots", ctypes.c_uint32),
        ("memory_budget", ctypes.c_uint64),
        ("max_batch_nnz", ctypes.c_uint64),
        ("max_batch_graphs", ctypes.c_uint32),
        ("direct_host_access", ctypes.c_uint32),
        ("engine", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 5),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("submitted", "completed", "batches", "batched_graphs", "cache_hits",
                                              "evictions", "resident_graphs", "resident_bytes",
                                              "peak_inflight_batches", "coalesced", "pack_us", "alloc_us",
                                              "harvest_us", "device_us", "engine_launches")] + \
        [("reserved", ctypes.c_uint64 * 1)]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("intersection_method", ctypes.c_int32),
        ("small_outdegree", ctypes.c_uint32),
        ("medium_outdegree", ctypes.c_uint32),
        ("segment", ctypes.c_uint32),
        ("from_cache", ctypes.c_uint32),
        ("candidates", ctypes.c_uint32),
        ("tile_order", ctypes.c_uint32),
        ("ms", ctypes.c_double),
        ("default_ms", ctypes.c_double),
        ("signature", ctypes.c_char * 96),
    ]


class RunStats(ctypes.Structure):
    _fields_ = [
        ("triangles", ctypes.c_uint64),
        ("n", ctypes.c_uint64),
        ("nnz", ctypes.c_uint64),
        ("oriented_edges", ctypes.c_uint64),
        ("wedge_checks", ctypes.c_uint64),
        ("intersection_size_local", ctypes.c_uint64),
        ("streamed_entries", ctypes.c_uint64),
        ("input_sorted", ctypes.c_uint32),
        ("method", ctypes.c_uint32),
        ("ms_orient", ctypes.c_float),
        ("ms_count", ctypes.c_float),
        ("ms_total", ctypes.c_float),
        ("ms_count_small", ctypes.c_float),
        ("ms_count_large", ctypes.c_float),
        ("ms_h2d", ctypes.c_float),
        ("ms_d2h", ctypes.c_float),
        ("ms_call", ctypes.c_float),
        ("host_ms_enqueue", ctypes.c_float),
        ("host_ms_call", ctypes.c_float),
        ("streamed_chunked", ctypes.c_uint64),
    ]


# every symbol include/ktri.h declares, with (restype, argtypes)
P, U32, U64, I32, D, CP = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double, \
    ctypes.c_char_p
PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "ktri_ctx_create": (ctypes.c_int, [ctypes.c_int, PP]),
    "ktri_ctx_destroy": (ctypes.c_int, [P]),
    "ktri_ctx_set_memory_budget": (ctypes.c_int, [P, U64]),
    "ktri_workspace_bytes": (U64, [U64, U64, I32]),
    "ktri_last_error": (CP, [P]),
    "ktri_ctx_stats": (ctypes.c_int, [P, ctypes.POINTER(RunStats)]),
    "ktri_version": (CP, []),
    "ktri_count_csr": (ctypes.c_int, [P, P, U64, U64, P, P, ctypes.POINTER(Opts)]),
    "ktri_count_csr_ctx": (ctypes.c_int, [P, P, P, U64, U64, P, P, ctypes.POINTER(Opts)]),
    "ktri_count_csr_device": (ctypes.c_int, [P, P, P, U64, U64, P, P, ctypes.POINTER(Opts), P]),
    "ktri_ctx_check": (ctypes.c_int, [P]),
    "ktri_count_csr_device_noalloc": (ctypes.c_int, [P, P, U64, U64, P, P, P]),
    "ktri_count_batch_device": (ctypes.c_int, [P, P, P, U64, U64, P, U64, P, P, ctypes.POINTER(Opts), P]),
    "ktri_count_batch_ctx": (ctypes.c_int, [P, P, P, U64, U64, P, U64, P, P, ctypes.POINTER(Opts)]),
    "ktri_plan_create_batch": (ctypes.c_int, [P, P, P, U64, U64, P, U64, P, P, ctypes.POINTER(Opts), PP]),
    "ktri_plan_launch": (ctypes.c_int, [P, P]),
    "ktri_plan_check": (ctypes.c_int, [P]),
    "ktri_plan_destroy": (ctypes.c_int, [P]),
    "ktri_binary_file_shape": (ctypes.c_int, [CP, ctypes.POINTER(U64), ctypes.POINTER(U64)]),
    "ktri_count_binary_file": (ctypes.c_int, [P, CP, ctypes.POINTER(U64), P, ctypes.POINTER(Opts), U64]),
    "ktri_list_triangles": (ctypes.c_int, [P, P, P, U64, U64, P, U64, ctypes.POINTER(U64)]),
    "ktri_count_dag_ctx": (ctypes.c_int, [P, P, P, U64, U64, P, P, ctypes.POINTER(Opts)]),
    "ktri_count_dag_device": (ctypes.c_int, [P, P, P, U64, U64, P, P, ctypes.POINTER(Opts), P]),
    "ktri_contract_dag_ctx": (ctypes.c_int, [P, P, P, U64, U64, U64, P, P, P, ctypes.POINTER(U64),
                                             ctypes.POINTER(U64)]),
    "ktri_partition_cost": (ctypes.c_int, [P, P, P, U64, U64, I32, U32, P, P, ctypes.POINTER(U64)]),
    "ktri_autotune": (ctypes.c_int, [P, P, P, U64, U64, P, U64, CP, ctypes.POINTER(Opts), ctypes.POINTER(Tuning), P]),
    "ktri_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ServerOpts), PP]),
    "ktri_server_submit": (ctypes.c_int, [P, U64, P, P, U64, U64, U32, ctypes.POINTER(U64)]),
    "ktri_server_wait": (ctypes.c_int, [P, U64, ctypes.POINTER(U64), P, ctypes.POINTER(ctypes.c_double)]),
    "ktri_server_get_stats": (ctypes.c_int, [P, ctypes.POINTER(ServerStats)]),
    "ktri_server_destroy": (ctypes.c_int, [P]),
    "ktri_orient_csr": (ctypes.c_int, [P, P, P, U64, U64, P, P]),
    "ktri_intersect_pairs": (ctypes.c_int, [P, I32, P, P, P, P, U64, P, P]),
    "ktri_graph_from_csr": (ctypes.c_int, [U64, P, P, PP]),
    "ktri_graph_gnm": (ctypes.c_int, [U64, U64, U64, PP]),
    "ktri_graph_rmat": (ctypes.c_int, [U32, U32, D, D, D, U64, PP]),
    "ktri_graph_rmat_n": (ctypes.c_int, [U64, U64, D, D, D, U64, PP]),
    "ktri_graph_rgg2d": (ctypes.c_int, [U64, D, U64, PP]),
    "ktri_batch_pack": (ctypes.c_int, [U64, P, PP, P]),
    "ktri_batch_generate": (ctypes.c_int, [U64, D, D, D, D, U64, PP, P]),
    "ktri_graphs_generate": (ctypes.c_int, [U64, P, P, P, P, P]),
    "ktri_graph_read_metis": (ctypes.c_int, [CP, PP]),
    "ktri_graph_read_binary": (ctypes.c_int, [CP, PP]),
    "ktri_graph_write_binary": (ctypes.c_int, [P, CP]),
    "ktri_graph_write_metis": (ctypes.c_int, [P, CP]),
    "ktri_graph_n": (U64, [P]),
    "ktri_graph_nnz": (U64, [P]),
    "ktri_graph_first_out": (P, [P]),
    "ktri_graph_head": (P, [P]),
    "ktri_graph_free": (None, [P]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libktri.so (building it first when it is missing or stale and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        try:
            _build.build()
        except RuntimeError:
            if not os.path.exists(_build.LIB):
                raise
    if not os.path.exists(_build.LIB):
        raise KtriError(ERR_NO_DEVICE, f"{_build.LIB} is missing: build it with katric_gb300.build.build()")
    L = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int, ctx=None) -> None:
    if rc != OK:
        msg = ""
        if ctx is not None:
            raw = load().ktri_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise KtriError(rc, msg)
