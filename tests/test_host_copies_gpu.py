"""Host-buffer counts through each way the library moves host memory (needs a GB300).

ktri_count_csr_ctx copies its inputs and outputs by kernels where the device can address the
host buffer and both ends are 16-byte aligned, and by the copy engines otherwise.  Here the same
graph (large enough that head is copied in 64 MiB pieces) is counted from pinned buffers (their
device address), from pageable numpy arrays (addressed directly where the platform allows, else
copied by the copy engines), and from views shifted by 4 or 8 bytes (the copy engines); every
result must equal the oracle's, total and per vertex."""
import ctypes
import os

import numpy as np
import pytest

from katric_gb300 import Graph, _native

pytestmark = pytest.mark.gpu


def _shifted(arr, shift_bytes):
    """A copy of arr whose data starts shift_bytes past a 16-byte boundary."""
    raw = np.zeros(arr.nbytes + 64, dtype=np.uint8)
    base = (-raw.ctypes.data) % 16
    view = raw[base + shift_bytes: base + shift_bytes + arr.nbytes].view(arr.dtype)
    view[:] = arr
    assert view.ctypes.data % 16 == shift_bytes
    return view


def _count(counter, fo_ptr, hd_ptr, n, nnz, pv_ptr):
    L = _native.load()
    tot = ctypes.c_uint64(0)
    opts = _native.Opts()
    opts.struct_size = ctypes.sizeof(_native.Opts)
    rc = L.ktri_count_csr_ctx(counter.handle, fo_ptr, hd_ptr, n, nnz, ctypes.byref(tot), pv_ptr, ctypes.byref(opts))
    assert rc == _native.OK, L.ktri_last_error(counter.handle)
    return tot.value


@pytest.fixture(scope="module")
def graph_and_truth(oracle):
    g = Graph.rmat(21, 16, seed=7)
    assert 4 * g.nnz >= 2 * (64 << 20)  # head goes in pieces
    total, pv, _ = oracle.count(g.first_out, g.head, num_threads=os.cpu_count() or 4)
    return g, total, pv


def test_pinned_buffers(counter, graph_and_truth):
    torch = pytest.importorskip("torch")
    g, total, pv = graph_and_truth
    fo = torch.from_numpy(g.first_out.view(np.int64)).pin_memory()
    hd = torch.from_numpy(g.head.view(np.int32)).pin_memory()
    out = torch.full((g.n,), -1, dtype=torch.int64).pin_memory()
    for _ in range(2):
        assert _count(counter, fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, out.data_ptr()) == total
        assert np.array_equal(out.numpy().view(np.uint64), pv)


def test_pageable_buffers(counter, graph_and_truth):
    g, total, pv = graph_and_truth
    fo = np.ascontiguousarray(g.first_out)
    hd = np.ascontiguousarray(g.head)
    out = np.full(g.n, 7, dtype=np.uint64)
    assert _count(counter, fo.ctypes.data, hd.ctypes.data, g.n, g.nnz, out.ctypes.data) == total
    assert np.array_equal(out, pv)


@pytest.mark.parametrize("shift", [4, 8])
def test_unaligned_buffers_take_the_copy_engines(counter, graph_and_truth, shift):
    g, total, pv = graph_and_truth
    fo = _shifted(np.ascontiguousarray(g.first_out), 8)
    hd = _shifted(np.ascontiguousarray(g.head), shift)
    out = _shifted(np.zeros(g.n, dtype=np.uint64), 8)
    assert _count(counter, fo.ctypes.data, hd.ctypes.data, g.n, g.nnz, out.ctypes.data) == total
    assert np.array_equal(out, pv)
