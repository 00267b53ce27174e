"""TEST INFRASTRUCTURE ONLY: the seeded graph generators, loaded without the CUDA library.

libgraphgen.so is the counting library's host generator source (G(n,m), RMAT, 2D RGG in
Morton order; katric_gb300/csrc/graph_host.cpp) compiled on its own with g++ by this folder's
Makefile.  The CPU baseline (bench.py --impl reference) builds its input graph through it, so
that the reference arm loads no part of the GPU product.  The same seed gives the same CSR
bytes as the library's generators (both arms print a SHA-256 of the CSR to show it).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgraphgen.so")
_SRC = os.path.join(os.path.dirname(_HERE), "katric_gb300", "csrc", "graph_host.cpp")

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        subprocess.run(["make", "-C", _HERE, "-B", "libgraphgen.so"], check=True, stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P, U64, U32, D = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double
        PP = ctypes.POINTER(ctypes.c_void_p)
        L.ktri_graph_rmat.argtypes = [U32, U32, D, D, D, U64, PP]
        L.ktri_graph_rgg2d.argtypes = [U64, D, U64, PP]
        L.ktri_graph_gnm.argtypes = [U64, U64, U64, PP]
        for f in (L.ktri_graph_rmat, L.ktri_graph_rgg2d, L.ktri_graph_gnm):
            f.restype = ctypes.c_int
        L.ktri_graph_n.argtypes = [P]
        L.ktri_graph_n.restype = U64
        L.ktri_graph_nnz.argtypes = [P]
        L.ktri_graph_nnz.restype = U64
        L.ktri_graph_first_out.argtypes = [P]
        L.ktri_graph_first_out.restype = P
        L.ktri_graph_head.argtypes = [P]
        L.ktri_graph_head.restype = P
        L.ktri_graph_free.argtypes = [P]
        L.ktri_graph_free.restype = None
        _lib = L
    return _lib


def _take(fn, *args):
    """Run a generator; copy its CSR into numpy arrays and free the native graph."""
    L = lib()
    h = ctypes.c_void_p()
    rc = fn(*args, ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"graph generator failed with status {rc}")
    try:
        n, nnz = int(L.ktri_graph_n(h)), int(L.ktri_graph_nnz(h))
        fo = np.ctypeslib.as_array((ctypes.c_uint64 * (n + 1)).from_address(L.ktri_graph_first_out(h))).copy()
        hd = (np.ctypeslib.as_array((ctypes.c_uint32 * nnz).from_address(L.ktri_graph_head(h))).copy()
              if nnz else np.zeros(0, dtype=np.uint32))
    finally:
        L.ktri_graph_free(h)
    return fo, hd


def rmat(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int):
    return _take(lib().ktri_graph_rmat, scale, edge_factor, a, b, c, seed)


def rgg2d(n: int, avg_degree: float, seed: int):
    return _take(lib().ktri_graph_rgg2d, n, avg_degree, seed)


def gnm(n: int, m: int, seed: int):
    return _take(lib().ktri_graph_gnm, n, m, seed)
