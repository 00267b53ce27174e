"""ktri_count_csr_device_noalloc: the count that allocates no device memory (needs a GB300).

Some callers cannot call cudaMalloc: a host runtime that owns all device memory through its
own pool, or a latency-bound loop that must not pay for an allocation.  This entry point
runs the same counting kernels on a fixed scratch array inside the library.  The test calls
it through the C ABI twice in a row (the second call reuses the scratch the first one left
behind) and checks total and per-vertex counts against ktri_count_csr_device, bit for bit
(the tolerance of every count test here), then checks that a graph whose workspace exceeds
the 64 MiB scratch is refused.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from katric_gb300 import Config, Graph, TriangleCounter, _native

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20


def _dev(arr, torch):
    return torch.from_numpy(arr.view(np.int64 if arr.dtype == np.uint64 else np.int32).copy()).cuda()


def _reference_counts(g, torch):
    with TriangleCounter(0) as ctr:
        fo, hd = _dev(g.first_out, torch), _dev(g.head, torch)
        tot = torch.zeros(1, dtype=torch.int64, device="cuda")
        pv = torch.zeros(g.n, dtype=torch.int64, device="cuda")
        ctr.count_device(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, tot.data_ptr(), pv.data_ptr(), Config())
        ctr.check()
        return int(tot.item()), pv.cpu().numpy().view(np.uint64).copy()


@pytest.mark.parametrize("kind", ["gnm14", "rmat14", "rgg14"])
def test_noalloc_matches_device_entry_point(kind):
    torch = pytest.importorskip("torch")
    if kind == "gnm14":
        g = Graph.gnm(1 << 14, 1 << 17, seed=1)
    elif kind == "rmat14":
        g = Graph.rmat(14, 16, seed=2)
    else:
        g = Graph.rgg2d(1 << 14, 32.0, seed=3)
    L = _native.load()
    assert L.ktri_workspace_bytes(g.n, g.nnz, _native.METHOD_AUTO) <= SCRATCH_BYTES
    total, pv = _reference_counts(g, torch)
    fo, hd = _dev(g.first_out, torch), _dev(g.head, torch)
    stream = torch.cuda.Stream()
    for _ in range(2):
        tot = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        out = torch.full((g.n,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        rc = L.ktri_count_csr_device_noalloc(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, tot.data_ptr(),
                                             out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == _native.OK
        assert int(tot.item()) == total
        assert np.array_equal(out.cpu().numpy().view(np.uint64), pv)


def test_noalloc_near_the_limit_against_the_oracle(oracle):
    """RMAT scale 18 (7.6e6 adjacency entries, a 45 MiB workspace): big enough that the tile
    orders run, with owners above out-degree 256 (the large-owner kernel and its bulk copies),
    checked against the CPU oracle, twice in a row."""
    torch = pytest.importorskip("torch")
    g = Graph.rmat(18, 16, seed=2)
    L = _native.load()
    ws = L.ktri_workspace_bytes(g.n, g.nnz, _native.METHOD_AUTO)
    assert SCRATCH_BYTES // 2 < ws <= SCRATCH_BYTES and g.nnz >= 1 << 20
    ofo, _ = oracle.oriented_csr(g.first_out, g.head)
    assert int(np.diff(ofo).max()) > 256  # some owner runs in the large-owner kernel
    total, pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    fo, hd = _dev(g.first_out, torch), _dev(g.head, torch)
    for _ in range(2):
        tot = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        out = torch.full((g.n,), -1, dtype=torch.int64, device="cuda")
        rc = L.ktri_count_csr_device_noalloc(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, tot.data_ptr(),
                                             out.data_ptr(), None)
        assert rc == _native.OK
        assert int(tot.item()) == total
        assert np.array_equal(out.cpu().numpy().view(np.uint64), pv)


def test_noalloc_refuses_graphs_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    L = _native.load()
    n = 1 << 21  # an edgeless graph whose workspace (about 72 MiB) exceeds the 64 MiB scratch
    assert L.ktri_workspace_bytes(n, 0, _native.METHOD_AUTO) > SCRATCH_BYTES
    fo = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    hd = torch.zeros(1, dtype=torch.int32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    out = torch.zeros(n, dtype=torch.int64, device="cuda")
    rc = L.ktri_count_csr_device_noalloc(fo.data_ptr(), hd.data_ptr(), n, 0, tot.data_ptr(), out.data_ptr(), None)
    assert rc == _native.ERR_UNSUPPORTED
