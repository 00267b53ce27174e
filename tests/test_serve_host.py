"""The Server wrapper's request bookkeeping on CPU, against a stand-in for libktri.so: a repeat
without a CSR names the vertex count its counts buffer is sized for, a graph without vertices is
repeated without counts, and a repeat with counts of a key the wrapper never saw is refused
before it reaches the library."""
import ctypes
import threading

import numpy as np
import pytest

from katric_gb300 import Graph, serve


class FakeLib:
    def __init__(self):
        self.calls = []
        self.next_id = 1

    def ktri_server_submit(self, h, key, fo, head, n, nnz, flags, rid_ref):
        self.calls.append((key, fo is not None, n, nnz, flags))
        ctypes.cast(rid_ref, ctypes.POINTER(ctypes.c_uint64)).contents.value = self.next_id
        self.next_id += 1
        return 0


def make_server():
    srv = serve.Server.__new__(serve.Server)  # no device: only the wrapper's own state
    srv._L = FakeLib()
    srv._h = None
    srv._meta = {}
    srv._mu = threading.Lock()
    srv._sizes = {}
    return srv


def test_repeats_name_the_size_they_expect():
    srv = make_server()
    g = Graph(np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32))
    empty = Graph(np.zeros(1, np.uint64), np.zeros(0, np.uint32))
    srv.submit(g, key=7)
    srv.submit(empty, key=8)
    srv.submit(None, key=7)
    srv.submit(None, key=7, per_vertex=False)
    srv.submit(None, key=8)
    calls = srv._L.calls
    assert calls[0] == (7, True, 2, 2, 1)
    assert calls[2] == (7, False, 2, 0, 1)  # the size of the graph last given under the key
    assert calls[3] == (7, False, 2, 0, 0)
    assert calls[4] == (8, False, 0, 0, 0)  # n = 0 would take any size: no counts asked for
    assert srv._meta[5][0] == 0
    srv._L.calls.clear()
    with pytest.raises(ValueError):
        srv.submit(None, key=99)  # counts of a key this wrapper was never given a graph for
    with pytest.raises(ValueError):
        srv.submit(None, key=0)
    assert srv._L.calls == []
    srv.submit(None, key=99, per_vertex=False)  # a total only: any size will do
    assert srv._L.calls == [(99, False, 0, 0, 0)]
