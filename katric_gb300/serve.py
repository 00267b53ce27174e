"""Serving: the continuous-batching request loop of libktri.so (ktri_server_*).

    with Server(memory_budget=120 << 30) as srv:
        rid = srv.submit(graph, key=17)          # copies the CSR; key makes the graph resident
        total, per_vertex, latency = srv.wait(rid)
        rid = srv.submit(None, key=17)           # repeat of a resident graph: no CSR needed
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _native
from .graph import Graph


class Server:
    def __init__(self, device: int = 0, slots: int = 2, memory_budget: int = 120 << 30,
                 max_batch_nnz: int = 1 << 28, max_batch_graphs: int = 4096, direct_host_access: bool = False,
                 engine: bool = False):
        self._L = _native.load()
        o = _native.ServerOpts()
        o.struct_size = ctypes.sizeof(_native.ServerOpts)
        o.slots = slots
        o.memory_budget = memory_budget
        o.max_batch_nnz = max_batch_nnz
        o.max_batch_graphs = max_batch_graphs
        o.direct_host_access = 1 if direct_host_access else 0
        o.engine = 1 if engine else 0
        h = ctypes.c_void_p()
        _native.check(self._L.ktri_server_create(device, ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._meta: dict[int, tuple[int, bool]] = {}
        self._mu = threading.Lock()
        self._sizes: dict[int, int] = {}  # key -> n of the graph last submitted under it

    def submit(self, graph: Graph | None, key: int = 0, per_vertex: bool = True, borrow: bool = False) -> int:
        """Queue a count.  borrow=True reads the graph's arrays in place: the Server keeps a
        reference to the graph until wait() returns for this request."""
        rid = ctypes.c_uint64(0)
        flags = (1 if per_vertex else 0) | (2 if borrow else 0)
        if graph is None:
            if not key:
                raise ValueError("a repeat needs the key of a resident graph")
            n = self._sizes.get(key, 0)
            if per_vertex and not n and key not in self._sizes:
                raise ValueError("a repeat with per-vertex counts needs a key this Server was given a graph for")
            # n: the vertex count the counts buffer is sized for; the server refuses the request
            # (KTRI_ERR_INVALID_ARGUMENT) if the graph resident under the key has another (n = 0
            # would take any size, so a graph without vertices is repeated without counts)
            rc = self._L.ktri_server_submit(self._h, key, None, None, n, 0, flags & 1 if n else 0,
                                            ctypes.byref(rid))
        else:
            rc = self._L.ktri_server_submit(self._h, key, graph.first_out.ctypes.data,
                                            graph.head.ctypes.data if graph.nnz else None, graph.n, graph.nnz,
                                            flags, ctypes.byref(rid))
            n = graph.n
        _native.check(rc)
        with self._mu:
            self._meta[rid.value] = (n, per_vertex, graph if borrow else None)
            if graph is not None and key:
                self._sizes[key] = graph.n
        return rid.value

    def wait(self, rid: int):
        """(total, per-vertex counts or None, latency in seconds)."""
        with self._mu:
            n, want, _keep = self._meta.pop(rid)
        total = ctypes.c_uint64(0)
        lat = ctypes.c_double(0)
        pv = np.empty(max(1, n), dtype=np.uint64) if want else None
        rc = self._L.ktri_server_wait(self._h, rid, ctypes.byref(total), pv.ctypes.data if pv is not None else None,
                                      ctypes.byref(lat))
        _native.check(rc)
        return int(total.value), (pv[:n] if pv is not None else None), float(lat.value)

    def stats(self) -> dict:
        st = _native.ServerStats()
        _native.check(self._L.ktri_server_get_stats(self._h, ctypes.byref(st)))
        return {k: int(getattr(st, k)) for k, _ in _native.ServerStats._fields_ if k != "reserved"}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._L.ktri_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
