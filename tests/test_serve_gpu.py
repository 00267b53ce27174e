"""Serving with continuous batching (needs a GB300): every result is the same alone and in
the mix, repeats are answered from resident graphs, the memory budget is honoured, and with
the engine batches published while the persistent counting kernel runs are counted by that
same kernel."""
import ctypes
import threading
import time

import numpy as np
import pytest

from katric_gb300 import Batch, Graph, KtriError, Server, TriangleCounter, _native

pytestmark = pytest.mark.gpu


def graph_mix(count, seed):
    b = Batch.generate(count, 6, 14, 4, 48, seed=seed)
    return [b.graph(i) for i in range(b.num_graphs)]


@pytest.mark.parametrize("direct,engine", [(False, False), (True, False), (False, True), (True, True)])
def test_results_alone_equal_results_in_the_mix(direct, engine):
    # besides the mix: a larger RMAT graph, an edgeless graph and a graph without vertices
    graphs = graph_mix(90, seed=31) + [Graph.rmat(15, 16, seed=3), Graph(np.zeros(5, np.uint64),
                                                                          np.zeros(0, np.uint32)),
                                       Graph(np.zeros(1, np.uint64), np.zeros(0, np.uint32))]
    with TriangleCounter(0) as ctr:
        alone = [ctr.count(g.first_out, g.head) for g in graphs]
    # direct=True: on Grace + Blackwell the device gathers the graphs from host memory itself
    with Server(slots=2, max_batch_nnz=1 << 18, direct_host_access=direct, engine=engine) as srv:
        rids = [None] * len(graphs)

        def client(lo, hi):
            for i in range(lo, hi):
                rids[i] = srv.submit(graphs[i], key=1000 + i, borrow=(i % 2 == 0))

        per = (len(graphs) + 3) // 4
        threads = [threading.Thread(target=client, args=(k * per, min(len(graphs), (k + 1) * per))) for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for i, g in enumerate(graphs):
            total, pv, lat = srv.wait(rids[i])
            assert total == alone[i][0], i
            assert np.array_equal(pv, alone[i][1]), i
            assert lat >= 0
        st = srv.stats()
        assert st["completed"] == len(graphs)
        assert st["batches"] >= 2 and st["batched_graphs"] == len(graphs)
        assert st["batches"] < len(graphs)  # requests were batched together
        # repeats of resident graphs by key: answered from the resident counts
        reps = [srv.submit(None, key=1000 + i) for i in range(0, len(graphs), 7)]
        for j, rid in zip(range(0, len(graphs), 7), reps):
            total, pv, _ = srv.wait(rid)
            assert total == alone[j][0] and np.array_equal(pv, alone[j][1])
        assert srv.stats()["cache_hits"] == len(reps)


def test_memory_budget_evicts_and_refuses():
    graphs = graph_mix(30, seed=5)
    with TriangleCounter(0) as ctr:
        alone = [ctr.count(g.first_out, g.head)[0] for g in graphs]
    big = Graph.rmat(16, 16, seed=1)
    budget = 96 << 20
    with Server(slots=1, memory_budget=budget, max_batch_nnz=1 << 16) as srv:
        for rnd in range(2):  # the second round re-submits with CSRs: evicted graphs are counted again
            rids = [srv.submit(g, key=1 + i) for i, g in enumerate(graphs)]
            for i, rid in enumerate(rids):
                assert srv.wait(rid)[0] == alone[i]
        st = srv.stats()
        assert st["resident_bytes"] <= budget
        rid = srv.submit(Graph.rmat(20, 16, seed=2), key=0, per_vertex=False)
        with pytest.raises(KtriError) as e:  # its batch alone needs more than the budget
            srv.wait(rid)
        assert e.value.code == _native.ERR_OUT_OF_MEMORY
        rid = srv.submit(big, key=0)
        with TriangleCounter(0) as ctr:
            assert srv.wait(rid)[0] == ctr.count(big.first_out, big.head)[0]


@pytest.mark.parametrize("direct", [False, True])
def test_repeats_while_queued_join_the_count(direct):
    """A request for a key that is still queued or counting is answered by that count; later
    repeats are answered from the resident copy taken on the device from the batch union."""
    big = Graph.rmat(17, 16, seed=9)
    small = graph_mix(12, seed=77)
    with TriangleCounter(0) as ctr:
        want_big = ctr.count(big.first_out, big.head)
        want_small = [ctr.count(g.first_out, g.head) for g in small]
    with Server(slots=1, direct_host_access=direct) as srv:
        first = srv.submit(big, key=5)
        again = [srv.submit(big, key=5, borrow=True), srv.submit(None, key=5),
                 srv.submit(big, key=5, per_vertex=False)]
        mix = [srv.submit(g, key=100 + i) for i, g in enumerate(small)]
        total, pv, _ = srv.wait(first)
        assert total == want_big[0] and np.array_equal(pv, want_big[1])
        for rid, wants_pv in zip(again, (True, True, False)):
            total, pv, _ = srv.wait(rid)
            assert total == want_big[0]
            assert (pv is None) if not wants_pv else np.array_equal(pv, want_big[1])
        for rid, w in zip(mix, want_small):
            total, pv, _ = srv.wait(rid)
            assert total == w[0] and np.array_equal(pv, w[1])
        st = srv.stats()
        assert st["coalesced"] + st["cache_hits"] == 3
        assert st["batched_graphs"] == 1 + len(small)
        later = [srv.submit(None, key=5)] + [srv.submit(None, key=100 + i) for i in range(len(small))]
        for rid, w in zip(later, [want_big] + want_small):
            total, pv, _ = srv.wait(rid)
            assert total == w[0] and np.array_equal(pv, w[1])


def test_submit_checks_offsets_and_repeats_share_the_host_counts():
    """A submit refuses a graph whose offsets decrease, for a graph large enough that several
    threads check its offsets and for a small one.  A graph counted without per-vertex counts
    answers its first repeat that wants them from the device copy and later repeats from the
    host copy kept with it.  A key names one graph: a graph of another size under a resident
    key is counted and replaces it.  Every answer equals the plain count."""
    g = Graph.rmat(18, 8, seed=5)
    small, other = graph_mix(4, seed=3)[1:3]
    with TriangleCounter(0) as ctr:
        want = ctr.count(g.first_out, g.head)
        want_other = ctr.count(other.first_out, other.head)
    with Server(slots=2) as srv:
        for base in (g, small):
            bad = base.first_out.copy()
            k = base.n // 2
            bad[k] = bad[k + 1] + 1  # one offset above its successor; first and last stay valid
            with pytest.raises(KtriError) as e:
                srv.submit(Graph(bad, base.head), key=0)
            assert e.value.code == _native.ERR_INVALID_CSR
        total, pv, _ = srv.wait(srv.submit(g, key=9, per_vertex=False))
        assert total == want[0] and pv is None
        for _ in range(3):
            total, pv, _ = srv.wait(srv.submit(None, key=9))
            assert total == want[0] and np.array_equal(pv, want[1])
            pv[:] = 0  # the caller's copy: later answers do not see it
        assert srv.stats()["cache_hits"] == 3
        # a graph of another size under the same key is counted (not answered from the resident
        # graph) and replaces it: a repeat by key then answers for the new graph
        assert other.n != g.n
        for _ in range(2):
            total, pv, _ = srv.wait(srv.submit(other, key=9))
            assert total == want_other[0] and np.array_equal(pv, want_other[1])
        total, pv, _ = srv.wait(srv.submit(None, key=9))
        assert total == want_other[0] and np.array_equal(pv, want_other[1])
        assert srv.stats()["cache_hits"] == 5
        # a repeat without a CSR that names another vertex count than the resident graph's is
        # refused (its counts buffer would be too small), one that names none takes any size
        L = _native.load()
        for expect_n, want_rc in ((g.n, _native.ERR_INVALID_ARGUMENT), (0, 0)):
            rid = ctypes.c_uint64(0)
            _native.check(L.ktri_server_submit(srv._h, 9, None, None, expect_n, 0, 0, ctypes.byref(rid)))
            total = ctypes.c_uint64(0)
            assert L.ktri_server_wait(srv._h, rid.value, ctypes.byref(total), None, None) == want_rc
            assert want_rc or total.value == want_other[0]


def test_engine_folds_arrivals_into_the_running_kernel():
    """Requests that arrive while the engine counts are prepared on a free slot and published
    to the running engine: many batches, fewer engine launches, every result exact.  After the
    stream dries up the engine leaves, and the next request launches it again."""
    graphs = graph_mix(240, seed=13) + [Graph.rmat(16, 16, seed=s) for s in range(3)]
    with TriangleCounter(0) as ctr:
        alone = [ctr.count(g.first_out, g.head) for g in graphs]
    with Server(slots=2, max_batch_nnz=1 << 17, engine=True) as srv:
        rids = [srv.submit(g, key=0, borrow=True) for g in graphs]
        for i, rid in enumerate(rids):
            total, pv, _ = srv.wait(rid)
            assert total == alone[i][0] and np.array_equal(pv, alone[i][1]), i
        st = srv.stats()
        assert st["batches"] >= 6
        assert 1 <= st["engine_launches"] < st["batches"]
        time.sleep(0.05)  # idle: the engine leaves
        launches = st["engine_launches"]
        rid = srv.submit(graphs[-1], key=0)
        total, pv, _ = srv.wait(rid)
        assert total == alone[-1][0] and np.array_equal(pv, alone[-1][1])
        assert srv.stats()["engine_launches"] == launches + 1


def test_engine_mixes_large_owner_tiles_with_small_units():
    """The engine's blocks take small-owner, medium and large-owner units of different jobs in
    turn; a graph with large owners (out-degree above 256: bulk copies into shared memory) counted
    among many small graphs must come out exact, per vertex."""
    big = Graph.rmat(18, 16, seed=2)
    graphs = graph_mix(120, seed=21)
    mixed = graphs[:60] + [big] + graphs[60:] + [big]
    with TriangleCounter(0) as ctr:
        alone = [ctr.count(g.first_out, g.head) for g in mixed]
    with Server(slots=2, max_batch_nnz=1 << 16, engine=True) as srv:
        for rnd in range(2):
            rids = [srv.submit(g, key=0, borrow=True) for g in mixed]
            for i, rid in enumerate(rids):
                total, pv, _ = srv.wait(rid)
                assert total == alone[i][0] and np.array_equal(pv, alone[i][1]), (rnd, i)
