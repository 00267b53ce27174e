"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle (oracle.c).

The oracle restates KaTric's shared-memory local counting path (orientation by
(degree, id), per-vertex id sort, node-parallel edge iterator with the four
intersection strategies).  Only tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg use it, always as the reference the GPU results are
compared with or as the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")

MERGE, BINARY_SEARCH, BINARY, HYBRID = 0, 1, 2, 3
METHODS = {"merge": MERGE, "binary-search": BINARY_SEARCH, "binary": BINARY, "hybrid": HYBRID}


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("triangles", ctypes.c_uint64),
        ("wedge_checks", ctypes.c_uint64),
        ("intersection_size_local", ctypes.c_uint64),
        ("skipped_nodes", ctypes.c_uint64),
        ("orientation_s", ctypes.c_double),
        ("sorting_s", ctypes.c_double),
        ("local_phase_s", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with make (gcc + OpenMP)."""
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", _HERE, "-B", "liboracle.so"], check=True, stdout=subprocess.DEVNULL)
    return _LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        U64 = ctypes.c_uint64
        L.orc_intersect.restype = U64
        L.orc_intersect.argtypes = [P, U64, P, U64, ctypes.c_int, U64, ctypes.c_double, P]
        L.orc_run_shmem.restype = U64
        L.orc_run_shmem.argtypes = [U64, P, P, ctypes.c_int, U64, ctypes.c_double, ctypes.c_int, ctypes.c_int, P,
                                    ctypes.POINTER(OrcStats)]
        L.orc_oriented_csr.restype = U64
        L.orc_oriented_csr.argtypes = [U64, P, P, P, P]
        L.orc_preprocess.restype = None
        L.orc_preprocess.argtypes = [U64, P, P, P, ctypes.c_int, ctypes.POINTER(OrcStats)]
        L.orc_count_slice.restype = U64
        L.orc_count_slice.argtypes = [U64, P, P, P, P, U64, U64, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(U64), ctypes.POINTER(OrcStats)]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_max_threads.argtypes = []
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def intersect(a, b, method: str = "merge", cutoff: int = 1000, hybrid_scale: float = 1.0) -> list[int]:
    """Intersect two sorted u32 lists with one of the reference's strategies."""
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    out = np.zeros(max(1, min(len(a), len(b))), dtype=np.uint32)
    k = lib().orc_intersect(_ptr(a), len(a), _ptr(b), len(b), METHODS[method], cutoff, hybrid_scale, _ptr(out))
    return [int(x) for x in out[:k]]


def count(first_out, head, method: str = "merge", num_threads: int = 1, per_vertex: bool = True,
          pseudo2core: bool = False, cutoff: int = 1000, hybrid_scale: float = 1.0):
    """Run the restated run_shmem on a copy of (first_out, head).

    Returns (total, per_vertex_counts or None, stats dict)."""
    fo = np.ascontiguousarray(first_out, dtype=np.uint64)
    work = np.array(head, dtype=np.uint32, copy=True)
    n = len(fo) - 1
    pv = np.zeros(max(n, 1), dtype=np.uint64) if per_vertex else None
    st = OrcStats()
    total = lib().orc_run_shmem(n, _ptr(fo), _ptr(work), METHODS[method], cutoff, hybrid_scale, int(pseudo2core),
                                int(num_threads), _ptr(pv) if pv is not None else None, ctypes.byref(st))
    stats = {k: getattr(st, k) for k, _ in OrcStats._fields_}
    return int(total), (pv[:n] if pv is not None else None), stats


class SlicedCount:
    """A full run_shmem count cut into pieces for timing: vertex v belongs to slice
    hash(v) mod slices; piece s orients and id-sorts the lists of slice s (copied back from the
    input) and runs the node-parallel local phase over slice s's tail vertices.  Pieces
    0..slices-1 together do exactly the work of one count, and their triangles add up to the
    total.  Construction preprocesses the whole graph once (outside any timing), so each piece
    finds the other slices' out-lists in place."""

    def __init__(self, first_out, head, slices: int, method: str = "merge", num_threads: int = 1):
        self.fo = np.ascontiguousarray(first_out, dtype=np.uint64)
        self.head = np.ascontiguousarray(head, dtype=np.uint32)
        self.n = len(self.fo) - 1
        self.work = np.array(self.head, dtype=np.uint32, copy=True)
        self.offset = np.zeros(max(self.n, 1), dtype=np.uint64)
        self.slices = int(slices)
        self.method = METHODS[method]
        self.threads = int(num_threads)
        lib().orc_preprocess(self.n, _ptr(self.fo), _ptr(self.work), _ptr(self.offset), self.threads, None)

    def run(self, s: int):
        """Piece s: returns (triangles with their tail in slice s, adjacency entries of slice s,
        stats dict with the piece's orientation, sorting and local-phase seconds)."""
        st = OrcStats()
        adj = ctypes.c_uint64(0)
        t = lib().orc_count_slice(self.n, _ptr(self.fo), _ptr(self.head), _ptr(self.work), _ptr(self.offset),
                                  int(s) % self.slices, self.slices, self.method, self.threads, ctypes.byref(adj),
                                  ctypes.byref(st))
        return int(t), int(adj.value), {k: getattr(st, k) for k, _ in OrcStats._fields_}


def oriented_csr(first_out, head):
    """Out-lists after orient + sort_neighborhoods, as a compact CSR (u64 offsets, u32 ids)."""
    fo = np.ascontiguousarray(first_out, dtype=np.uint64)
    hd = np.ascontiguousarray(head, dtype=np.uint32)
    n = len(fo) - 1
    ofo = np.zeros(n + 1, dtype=np.uint64)
    oh = np.zeros(max(1, len(hd)), dtype=np.uint32)
    m = lib().orc_oriented_csr(n, _ptr(fo), _ptr(hd), _ptr(ofo), _ptr(oh))
    return ofo, oh[:m].copy()


def max_threads() -> int:
    return int(lib().orc_max_threads())
