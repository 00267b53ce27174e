"""Host graph ingest: generators, formats and the C ABI's exported symbols (no GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from katric_gb300 import Graph, _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def assert_simple_undirected(g: Graph):
    fo, hd = g.first_out.astype(np.int64), g.head.astype(np.int64)
    n = g.n
    assert fo[0] == 0 and fo[-1] == len(hd)
    assert (np.diff(fo) >= 0).all()
    src = np.repeat(np.arange(n), np.diff(fo))
    assert (hd < n).all()
    assert (src != hd).all()
    for v in range(min(n, 2000)):
        lst = hd[fo[v]:fo[v + 1]]
        assert (np.diff(lst) > 0).all()  # sorted, no duplicates
    fwd = set(zip(src.tolist(), hd.tolist()))
    assert all((b, a) in fwd for a, b in list(fwd)[:20000])


def test_gnm_exact_size_and_determinism():
    g = Graph.gnm(1 << 10, 5000, seed=11)
    assert g.n == 1 << 10 and g.m == 5000
    assert_simple_undirected(g)
    g2 = Graph.gnm(1 << 10, 5000, seed=11)
    assert (g.head == g2.head).all() and (g.first_out == g2.first_out).all()
    g3 = Graph.gnm(1 << 10, 5000, seed=12)
    assert not np.array_equal(g.head, g3.head)


def test_rmat_shape():
    g = Graph.rmat(12, 16, seed=2)
    assert g.n == 1 << 12
    assert 0 < g.m <= 16 << 12
    assert_simple_undirected(g)
    deg = g.degree()
    assert deg[0] == deg.max()  # (0.57, ...) puts the heaviest vertex at id 0
    g2 = Graph.rmat(12, 16, seed=2)
    assert np.array_equal(g.head, g2.head)


def test_rgg_shape_and_locality():
    g = Graph.rgg2d(1 << 14, 32.0, seed=3)
    assert g.n == 1 << 14
    assert 28 < g.degree().mean() < 36
    assert_simple_undirected(g)
    # Morton order keeps neighbours close in id space
    src = np.repeat(np.arange(g.n), np.diff(g.first_out.astype(np.int64)))
    gap = np.abs(src - g.head.astype(np.int64))
    assert np.median(gap) < g.n / 32


def test_metis_and_binary_round_trip(tmp_path, golden):
    ex, _ = golden
    for e in ex["graphs"]:
        p = tmp_path / f"{e['name']}.metis"
        with open(p, "w") as f:
            fo, hd = e["first_out"], e["head"]
            f.write(f"{e['n']} {len(hd) // 2}\n")
            for v in range(e["n"]):
                f.write(" ".join(str(x + 1) for x in hd[fo[v]:fo[v + 1]]) + "\n")
        g = Graph.read(str(p), "metis")
        assert g.first_out.tolist() == e["first_out"]
        assert g.head.tolist() == e["head"]  # adjacency order is preserved
        stem = str(tmp_path / e["name"])
        g.write_binary(stem)
        assert np.fromfile(stem + ".first_out", dtype="<u8").tolist() == e["first_out"]
        assert np.fromfile(stem + ".head", dtype="<u8").tolist() == e["head"]
        g2 = Graph.read(stem, "binary")
        assert g2.head.tolist() == e["head"]
        g.write_metis(str(tmp_path / "again.metis"))
        g3 = Graph.read_metis(str(tmp_path / "again.metis"))
        assert g3.head.tolist() == e["head"]


def test_reference_binary_fixture(tmp_path, golden):
    """The reference's own binary files (u64 heads) decode to the METIS adjacency."""
    ex, _ = golden
    e = next(g for g in ex["graphs"] if g["name"] == "hiv")
    stem = str(tmp_path / "hiv")
    np.array(e["binary_first_out"], dtype="<u8").tofile(stem + ".first_out")
    np.array(e["binary_head"], dtype="<u8").tofile(stem + ".head")
    g = Graph.read_binary(stem)
    assert g.n == e["n"] and g.nnz == len(e["head"])


def test_bad_files(tmp_path):
    p = tmp_path / "bad.metis"
    p.write_text("3 2\n2 9\n1\n\n")
    with pytest.raises(_native.KtriError):
        Graph.read_metis(str(p))
    with pytest.raises(_native.KtriError):
        Graph.read_binary(str(tmp_path / "missing"))


def test_generator_argument_errors():
    with pytest.raises(_native.KtriError):
        Graph.gnm(4, 100)
    with pytest.raises(_native.KtriError):
        Graph.rmat(0)


def test_abi_exports_every_declared_symbol():
    with open(os.path.join(ROOT, "include", "ktri.h")) as f:
        src = f.read()
    declared = set(re.findall(r"\b(ktri_[a-z0-9_]+)\s*\(", src))
    assert len(declared) >= 25
    L = _native.load()
    for name in declared:
        assert hasattr(L, name), name
    assert set(_native.SIGNATURES) == declared


def test_no_device_is_an_error_not_a_fallback():
    """Without a GPU the counting entry points fail with a status code (no CPU path)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = _native.load()
    h = ctypes.c_void_p()
    assert L.ktri_ctx_create(0, ctypes.byref(h)) == _native.ERR_NO_DEVICE
    total = ctypes.c_uint64(0)
    fo = np.array([0, 1, 2], dtype=np.uint64)
    hd = np.array([1, 0], dtype=np.uint32)
    rc = L.ktri_count_csr(fo.ctypes.data, hd.ctypes.data, 2, 2, ctypes.byref(total), None, None)
    assert rc in (_native.ERR_NO_DEVICE, _native.ERR_CUDA)
