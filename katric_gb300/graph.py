"""Host graphs: CSR containers, seeded generators and the reference's file formats.

A Graph holds an undirected simple graph as CSR (u64 first_out[n+1], u32 head[nnz]), the
layout the counting entry points take.  Generators and readers run in libktri.so's host
code (C++ with OpenMP), so the same seed gives the same graph on every host.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


class _NativeGraph:
    """Owns one ktri_graph; every numpy view of its arrays holds a reference to it."""

    def __init__(self, handle):
        self.handle = handle

    def __del__(self):
        if self.handle is not None:
            try:
                _native.load(build_if_missing=False).ktri_graph_free(self.handle)
            except Exception:
                pass
            self.handle = None


def _view(owner: _NativeGraph, ptr: int, ctype, count: int, dtype) -> np.ndarray:
    if count == 0:
        return np.zeros(0, dtype=dtype)
    buf = (ctype * count).from_address(ptr)
    buf._owner = owner  # the array's base keeps the native graph alive
    return np.ctypeslib.as_array(buf)


class Graph:
    """CSR graph on the host.  first_out: u64[n+1], head: u32[nnz]."""

    def __init__(self, first_out, head, *, _owner=None):
        self.first_out = np.ascontiguousarray(first_out, dtype=np.uint64)
        self.head = np.ascontiguousarray(head, dtype=np.uint32)
        self._owner = _owner  # native graph behind the arrays, if they are views of one
        if len(self.first_out) == 0:
            raise ValueError("first_out needs n+1 entries")

    @property
    def n(self) -> int:
        return len(self.first_out) - 1

    @property
    def nnz(self) -> int:
        return len(self.head)

    @property
    def m(self) -> int:
        """Undirected edges (each stored twice)."""
        return self.nnz // 2

    def degree(self) -> np.ndarray:
        return np.diff(self.first_out)

    def wedges(self) -> int:
        """sum over v of deg(v) choose 2 (apps/shmetric.cpp:120-129)."""
        d = self.degree().astype(np.uint64)
        return int(np.sum(d * (d - 1) // 2, dtype=np.uint64)) if len(d) else 0

    # ---- construction -------------------------------------------------------------------
    @staticmethod
    def _from_handle(h) -> "Graph":
        L = _native.load()
        owner = _NativeGraph(h)
        n = L.ktri_graph_n(h)
        nnz = L.ktri_graph_nnz(h)
        fo = _view(owner, L.ktri_graph_first_out(h), ctypes.c_uint64, n + 1, np.uint64)
        hd = _view(owner, L.ktri_graph_head(h), ctypes.c_uint32, nnz, np.uint32)
        return Graph(fo, hd, _owner=owner)

    @staticmethod
    def _call(fn, *args) -> "Graph":
        h = ctypes.c_void_p()
        _native.check(fn(*args, ctypes.byref(h)))
        return Graph._from_handle(h)

    @classmethod
    def gnm(cls, n: int, m: int, seed: int = 1) -> "Graph":
        """G(n,m): m distinct undirected edges uniformly at random, no self-loops."""
        return cls._call(_native.load().ktri_graph_gnm, n, m, seed)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 2) -> "Graph":
        """RMAT with 2^scale vertices and edge_factor*2^scale samples; symmetrised, deduplicated, no loops."""
        return cls._call(_native.load().ktri_graph_rmat, scale, edge_factor, a, b, c, seed)

    @classmethod
    def rgg2d(cls, n: int, avg_degree: float = 32.0, seed: int = 3) -> "Graph":
        """2D random geometric graph in the unit square, ids in Morton order of the points."""
        return cls._call(_native.load().ktri_graph_rgg2d, n, avg_degree, seed)

    @classmethod
    def read_metis(cls, path: str) -> "Graph":
        return cls._call(_native.load().ktri_graph_read_metis, path.encode())

    @classmethod
    def read_binary(cls, stem: str) -> "Graph":
        """<stem>.first_out (u64[n+1]) + <stem>.head (u64[nnz]), the reference's binary input format."""
        return cls._call(_native.load().ktri_graph_read_binary, stem.encode())

    @classmethod
    def read(cls, path: str, input_format: str = "metis") -> "Graph":
        """graphio::read_graph(file, format) equivalent (apps/shmetric.cpp:119)."""
        fmt = input_format.lower()
        if fmt == "metis":
            return cls.read_metis(path)
        if fmt == "binary":
            return cls.read_binary(path)
        raise ValueError(f"unknown input format {input_format!r} (metis or binary)")

    def _native_handle(self):
        """A native graph with this graph's content (the backing one, or a copy)."""
        if self._owner is not None:
            return self._owner.handle
        h = ctypes.c_void_p()
        L = _native.load()
        _native.check(L.ktri_graph_from_csr(self.n, self.first_out.ctypes.data,
                                            self.head.ctypes.data if self.nnz else None, ctypes.byref(h)))
        self._owner = _NativeGraph(h)
        return h

    def write_binary(self, stem: str) -> None:
        _native.check(_native.load().ktri_graph_write_binary(self._native_handle(), stem.encode()))

    def write_metis(self, path: str) -> None:
        _native.check(_native.load().ktri_graph_write_metis(self._native_handle(), path.encode()))


def generate_many(kinds, ns, degrees, seeds) -> list[Graph]:
    """Graphs from explicit specs, generated in parallel on the host (one thread per graph).
    kinds: 0 = G(n,m) with m = round(n d / 2), 1 = RMAT with round(n d / 2) draws, 2 = 2D RGG."""
    k = len(kinds)
    kinds = np.ascontiguousarray(kinds, dtype=np.uint32)
    ns = np.ascontiguousarray(ns, dtype=np.uint64)
    degrees = np.ascontiguousarray(degrees, dtype=np.float64)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    outs = (ctypes.c_void_p * max(1, k))()
    _native.check(_native.load().ktri_graphs_generate(k, kinds.ctypes.data, ns.ctypes.data, degrees.ctypes.data,
                                                      seeds.ctypes.data, outs))
    return [Graph._from_handle(ctypes.c_void_p(outs[i])) for i in range(k)]


def generate(name: str, seed: int | None = None, **kw) -> Graph:
    """Named generator (the subset of --gen the engine is measured on): gnm, rmat, rgg2d."""
    name = name.lower()
    if name in ("gnm", "gnm_undirected"):
        return Graph.gnm(kw["n"], kw["m"], 1 if seed is None else seed)
    if name == "rmat":
        return Graph.rmat(kw["scale"], kw.get("edge_factor", 16), kw.get("a", 0.57), kw.get("b", 0.19),
                          kw.get("c", 0.19), 2 if seed is None else seed)
    if name in ("rgg2d", "rgg_2d"):
        return Graph.rgg2d(kw["n"], kw.get("avg_degree", 32.0), 3 if seed is None else seed)
    raise ValueError(f"unknown generator {name!r}")


class Batch:
    """Independent graphs packed as one disjoint-union CSR.

    Graph g owns the union's vertices [graph_first[g], graph_first[g+1]); the union is what
    the batched entry points count in one launch sequence."""

    def __init__(self, union: Graph, graph_first):
        self.union = union
        self.graph_first = np.ascontiguousarray(graph_first, dtype=np.uint64)

    @property
    def num_graphs(self) -> int:
        return len(self.graph_first) - 1

    def graph(self, g: int) -> Graph:
        """Graph g with its own 0-based ids."""
        a, b = int(self.graph_first[g]), int(self.graph_first[g + 1])
        fo = self.union.first_out[a:b + 1]
        hd = self.union.head[int(fo[0]):int(fo[-1])]
        return Graph(fo - fo[0], (hd.astype(np.int64) - a).astype(np.uint32))

    @classmethod
    def pack(cls, graphs) -> "Batch":
        L = _native.load()
        handles = (ctypes.c_void_p * max(1, len(graphs)))(*[g._native_handle() for g in graphs])
        gf = np.zeros(len(graphs) + 1, dtype=np.uint64)
        h = ctypes.c_void_p()
        _native.check(L.ktri_batch_pack(len(graphs), handles, ctypes.byref(h), gf.ctypes.data))
        return cls(Graph._from_handle(h), gf)

    @classmethod
    def generate(cls, num_graphs: int = 8192, log2_n_min: float = 8.0, log2_n_max: float = 17.0,
                 deg_min: float = 4.0, deg_max: float = 64.0, seed: int = 4) -> "Batch":
        """The batched workload: n log-uniform, average degree uniform, generators G(n,m) / RMAT /
        2D RGG by index mod 3, graph i seeded with seed + i."""
        L = _native.load()
        gf = np.zeros(num_graphs + 1, dtype=np.uint64)
        h = ctypes.c_void_p()
        _native.check(L.ktri_batch_generate(num_graphs, log2_n_min, log2_n_max, deg_min, deg_max, seed,
                                            ctypes.byref(h), gf.ctypes.data))
        return cls(Graph._from_handle(h), gf)
