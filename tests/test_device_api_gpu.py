"""The device-resident entry point (ktri_count_csr_device) on torch-allocated buffers and
streams, and size-independent properties at large sizes (needs a GB300)."""
import os

import numpy as np
import pytest

from katric_gb300 import Config, Graph, TriangleCounter

pytestmark = pytest.mark.gpu


def _dev(arr, torch):
    """Copy a u64/u32 numpy array to the GPU as int64/int32 with the same bits."""
    return torch.from_numpy(arr.view(np.int64 if arr.dtype == np.uint64 else np.int32).copy()).cuda()


def test_device_entry_point_on_a_stream(counter, oracle):
    torch = pytest.importorskip("torch")
    g = Graph.rmat(14, 16, seed=3)
    total, pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    fo = _dev(g.first_out, torch)
    hd = _dev(g.head, torch)
    out_t = torch.zeros(1, dtype=torch.int64, device="cuda")
    out_pv = torch.zeros(g.n, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    for _ in range(2):  # two calls in a row reuse the workspace
        out_t.zero_()
        counter.count_device(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, out_t.data_ptr(), out_pv.data_ptr(),
                             Config(), stream=s.cuda_stream)
        counter.check()
        assert int(out_t.item()) == total
        assert np.array_equal(out_pv.cpu().numpy().view(np.uint64), pv)
    # no per-vertex buffer: the library uses its own
    counter.count_device(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, out_t.data_ptr(), None, Config(),
                         stream=s.cuda_stream)
    counter.check()
    assert int(out_t.item()) == total


def _relabel(g: Graph, perm: np.ndarray):
    """Graph with vertex v renamed perm[v] (lists re-sorted)."""
    n = g.n
    fo = g.first_out.astype(np.int64)
    src = np.repeat(np.arange(n), np.diff(fo))
    s2, h2 = perm[src], perm[g.head.astype(np.int64)]
    order = np.lexsort((h2, s2))
    s2, h2 = s2[order], h2[order]
    nfo = np.zeros(n + 1, dtype=np.uint64)
    nfo[1:] = np.cumsum(np.bincount(s2, minlength=n))
    return nfo, h2.astype(np.uint32)


@pytest.mark.parametrize("kind", ["rmat20", "rgg20"])
def test_properties_large(counter, kind):
    """Checks that need no oracle: 3 * total == sum of per-vertex counts; the AUTO and merge
    kernels (independent algorithms) agree bit for bit; totals and per-vertex counts are
    invariant under relabelling the vertices."""
    g = Graph.rmat(20, 16, seed=2) if kind == "rmat20" else Graph.rgg2d(1 << 20, 32.0, seed=3)
    t, pv = counter.count(g.first_out, g.head, Config(intersection_method="auto"))
    assert int(pv.sum()) == 3 * t
    t2, pv2 = counter.count(g.first_out, g.head, Config(intersection_method="merge"))
    assert t2 == t and np.array_equal(pv, pv2)
    perm = np.random.default_rng(4).permutation(g.n)
    fo3, hd3 = _relabel(g, perm)
    t3, pv3 = counter.count(fo3, hd3)
    assert t3 == t
    assert np.array_equal(pv3[perm], pv)


def test_memory_budget(counter):
    g = Graph.gnm(1 << 12, 1 << 14, seed=1)
    with TriangleCounter(0, memory_budget=1 << 16) as small:
        from katric_gb300 import KtriError, _native
        with pytest.raises(KtriError) as e:
            small.count(g.first_out, g.head)
        assert e.value.code == _native.ERR_OUT_OF_MEMORY
        small.set_memory_budget(0)
        assert small.count(g.first_out, g.head)[0] == counter.count(g.first_out, g.head)[0]


def test_host_path_copies_head_in_pieces(counter, oracle):
    """Host buffers of more than two 64 MiB pieces of adjacency: head is copied in pieces on a
    second stream and the orientation tiles of each piece start as soon as it lands.  Counts
    must equal the oracle's, and the call reports its copy / read-back split."""
    g = Graph.rmat(21, 16, seed=5)
    assert 4 * g.nnz >= 2 * (64 << 20)
    total, pv, _ = oracle.count(g.first_out, g.head, num_threads=os.cpu_count() or 4)
    for _ in range(2):
        t, p = counter.count(g.first_out, g.head, Config())
        assert t == total and np.array_equal(p, pv)
        st = counter.stats()
        assert 0 < st.ms_h2d <= st.ms_call and 0 < st.ms_d2h <= st.ms_call
    t, p = counter.count(g.first_out, g.head, Config(intersection_method="merge"))
    assert t == total and np.array_equal(p, pv)
