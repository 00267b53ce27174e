"""Batched workload generation and packing on the host (no GPU)."""
import ctypes

import numpy as np

from katric_gb300 import Batch, Graph, _native


def test_batch_generate_deterministic_and_well_formed():
    b = Batch.generate(48, 6, 11, 4, 32, seed=7)
    b2 = Batch.generate(48, 6, 11, 4, 32, seed=7)
    assert np.array_equal(b.union.head, b2.union.head)
    assert np.array_equal(b.graph_first, b2.graph_first)
    assert b.num_graphs == 48 and int(b.graph_first[-1]) == b.union.n
    ns = np.diff(b.graph_first.astype(np.int64))
    assert ns.min() >= 2 ** 6 - 1 and ns.max() <= 2 ** 11 + 1
    fo = b.union.first_out.astype(np.int64)
    for g in range(b.num_graphs):
        a, e = int(b.graph_first[g]), int(b.graph_first[g + 1])
        heads = b.union.head[fo[a]:fo[e]].astype(np.int64)
        assert heads.size == 0 or (heads.min() >= a and heads.max() < e)  # edges stay inside their graph


def test_batch_pack_round_trip():
    b = Batch.generate(20, 5, 9, 4, 24, seed=3)
    graphs = [b.graph(i) for i in range(b.num_graphs)]
    bb = Batch.pack(graphs)
    assert np.array_equal(bb.union.head, b.union.head)
    assert np.array_equal(bb.union.first_out, b.union.first_out)
    assert np.array_equal(bb.graph_first, b.graph_first)


def test_batch_mix_of_generators():
    b = Batch.generate(9, 8, 8, 16, 16, seed=11)  # all graphs n = 256, degree 16
    for i in range(9):
        g = b.graph(i)
        assert g.n == 256
        if i % 3 == 0:  # G(n, m) has exactly round(n d / 2) edges
            assert g.m == 256 * 16 // 2
        if i % 3 == 1:
            ref = Graph.rmat(8, 8, seed=11 + i)  # same draws: n d / 2 = 8 n samples
            assert np.array_equal(g.head, ref.head)


def test_rmat_n_matches_power_of_two_rmat():
    L = _native.load()
    h = ctypes.c_void_p()
    assert L.ktri_graph_rmat_n(1 << 12, 16 << 12, 0.57, 0.19, 0.19, 2, ctypes.byref(h)) == 0
    g = Graph._from_handle(h)
    assert np.array_equal(g.head, Graph.rmat(12, 16, seed=2).head)
    h2 = ctypes.c_void_p()
    assert L.ktri_graph_rmat_n(3000, 40000, 0.57, 0.19, 0.19, 5, ctypes.byref(h2)) == 0
    g2 = Graph._from_handle(h2)
    assert g2.n == 3000 and int(g2.head.max()) < 3000
