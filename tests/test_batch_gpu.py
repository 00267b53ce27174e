"""Batched counting on the GPU (needs a GB300): one launch sequence over many graphs, exact
per-graph totals and per-vertex counts against the oracle graph by graph, and captured plans
(CUDA graphs) replayed on refilled buffers."""
import numpy as np
import pytest

from katric_gb300 import Batch, Config, Graph

pytestmark = pytest.mark.gpu


def oracle_batch(oracle, b: Batch):
    totals, pvs = [], []
    for i in range(b.num_graphs):
        g = b.graph(i)
        t, pv, _ = oracle.count(g.first_out, g.head, num_threads=4)
        totals.append(t)
        pvs.append(pv)
    return np.array(totals, dtype=np.uint64), np.concatenate(pvs)


@pytest.mark.parametrize("method,wide", [("auto", False), ("merge", False), ("auto", True)])
def test_batch_parity(counter, oracle, method, wide):
    b = Batch.generate(60, 5, 12, 4, 40, seed=21)
    et, epv = oracle_batch(oracle, b)
    totals, pv = counter.count_batch(b, Config(intersection_method=method, force_wide_offsets=wide))
    assert np.array_equal(totals, et)
    assert np.array_equal(pv, epv)


def test_batch_with_empty_and_tiny_graphs(counter, oracle):
    graphs = [Graph(np.zeros(4, np.uint64), np.zeros(0, np.uint32)),
              Graph.gnm(3, 3, seed=1), Graph.rmat(10, 16, seed=3),
              Graph(np.zeros(2, np.uint64), np.zeros(0, np.uint32)), Graph.rgg2d(500, 20.0, seed=2)]
    b = Batch.pack(graphs)
    et, epv = oracle_batch(oracle, b)
    totals, pv = counter.count_batch(b)
    assert np.array_equal(totals, et) and totals[1] == 1
    assert np.array_equal(pv, epv)


def _dev(arr, torch):
    return torch.from_numpy(arr.view(np.int64 if arr.dtype == np.uint64 else np.int32).copy()).cuda()


def _permuted(b: Batch, seed: int) -> Batch:
    """Same graph sizes, every graph relabelled by its own permutation."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(b.num_graphs):
        g = b.graph(i)
        perm = rng.permutation(g.n)
        fo = g.first_out.astype(np.int64)
        src = np.repeat(np.arange(g.n), np.diff(fo))
        s2, h2 = perm[src], perm[g.head.astype(np.int64)]
        order = np.lexsort((h2, s2))
        nfo = np.zeros(g.n + 1, dtype=np.uint64)
        nfo[1:] = np.cumsum(np.bincount(s2[order], minlength=g.n))
        out.append(Graph(nfo, h2[order].astype(np.uint32)))
    return Batch.pack(out)


def test_plan_capture_and_replay(counter, oracle):
    torch = pytest.importorskip("torch")
    b = Batch.generate(40, 6, 12, 4, 40, seed=5)
    et, epv = oracle_batch(oracle, b)
    fo, hd, gf = _dev(b.union.first_out, torch), _dev(b.union.head, torch), _dev(b.graph_first, torch)
    tot = torch.zeros(b.num_graphs, dtype=torch.int64, device="cuda")
    pv = torch.zeros(b.union.n, dtype=torch.int64, device="cuda")
    plan = counter.plan_batch(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(), b.num_graphs,
                              tot.data_ptr(), pv.data_ptr())
    s = torch.cuda.Stream()
    for _ in range(2):
        tot.zero_()
        torch.cuda.synchronize()
        plan.launch(s.cuda_stream)
        plan.check()
        assert np.array_equal(tot.cpu().numpy().view(np.uint64), et)
        assert np.array_equal(pv.cpu().numpy().view(np.uint64), epv)
    # refill the bound buffers with another batch of the same shape and replay
    b2 = _permuted(b, 9)
    assert b2.union.nnz == b.union.nnz and np.array_equal(b2.graph_first, b.graph_first)
    et2, epv2 = oracle_batch(oracle, b2)
    hd.copy_(_dev(b2.union.head, torch))
    fo.copy_(_dev(b2.union.first_out, torch))
    torch.cuda.synchronize()
    plan.launch(s.cuda_stream)
    plan.check()
    assert np.array_equal(tot.cpu().numpy().view(np.uint64), et2) and np.array_equal(et2, et)
    assert np.array_equal(pv.cpu().numpy().view(np.uint64), epv2)
    plan.close()


def test_batch_device_entry_point(counter, oracle):
    torch = pytest.importorskip("torch")
    b = Batch.generate(25, 5, 11, 4, 32, seed=8)
    et, _ = oracle_batch(oracle, b)
    fo, hd, gf = _dev(b.union.first_out, torch), _dev(b.union.head, torch), _dev(b.graph_first, torch)
    tot = torch.zeros(b.num_graphs, dtype=torch.int64, device="cuda")
    counter.count_batch_device(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(), b.num_graphs,
                               tot.data_ptr(), None)
    counter.check()
    assert np.array_equal(tot.cpu().numpy().view(np.uint64), et)


def test_autotune_persists_and_plans_exactly(counter, oracle, tmp_path):
    """The autotuner times strategies, bins and segments on the batch, persists the choice as a
    JSON line, reads it back for an input of the same shape class, and the plan it configures
    counts exactly."""
    import json
    torch = pytest.importorskip("torch")
    b = Batch.generate(48, 6, 13, 4, 48, seed=17)
    et, epv = oracle_batch(oracle, b)
    fo, hd, gf = _dev(b.union.first_out, torch), _dev(b.union.head, torch), _dev(b.graph_first, torch)
    cache = tmp_path / "tune.jsonl"
    conf, info = counter.autotune(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(),
                                  b.num_graphs, cache_path=str(cache))
    assert not info["from_cache"] and info["candidates"] >= 5 and info["ms"] <= info["default_ms"]
    lines = cache.read_text().splitlines()
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["signature"] == info["signature"] and rec["segment"] == conf.segment
    assert rec["small_outdegree"] == conf.small_outdegree and rec["medium_outdegree"] == conf.medium_outdegree
    conf2, info2 = counter.autotune(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(),
                                    b.num_graphs, cache_path=str(cache))
    assert info2["from_cache"] and info2["candidates"] == 0 and conf2 == conf
    tot = torch.zeros(b.num_graphs, dtype=torch.int64, device="cuda")
    pv = torch.zeros(b.union.n, dtype=torch.int64, device="cuda")
    plan = counter.plan_batch(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(), b.num_graphs,
                              tot.data_ptr(), pv.data_ptr(), conf)
    plan.launch()
    plan.check()
    assert np.array_equal(tot.cpu().numpy().view(np.uint64), et)
    assert np.array_equal(pv.cpu().numpy().view(np.uint64), epv)
    plan.close()
    # a single graph (no graph_first) tunes too
    g = Graph.rmat(13, 16, seed=6)
    gfo, ghd = _dev(g.first_out, torch), _dev(g.head, torch)
    conf3, info3 = counter.autotune(gfo.data_ptr(), ghd.data_ptr(), g.n, g.nnz)
    assert info3["candidates"] >= 5
    t, p = counter.count(g.first_out, g.head, conf3)
    assert t == oracle.count(g.first_out, g.head, num_threads=4)[0]


def test_plan_destroyed_after_its_context():
    """A plan may be destroyed after the context it was made on (a garbage-collected plan in a
    host language can outlive an explicitly closed context): destroy touches only the plan, and
    leaves no error behind for the next call on another context."""
    import ctypes

    import numpy as np
    import torch

    from katric_gb300 import Batch, Config, TriangleCounter, _native
    L = _native.load()
    b = Batch.generate(8, 6.0, 9.0, 4.0, 16.0, seed=11)
    fo = torch.from_numpy(b.union.first_out.view(np.int64)).cuda()
    hd = torch.from_numpy(b.union.head.view(np.int32)).cuda()
    gf = torch.from_numpy(b.graph_first.view(np.int64)).cuda()
    tot = torch.zeros(b.num_graphs, dtype=torch.int64, device="cuda")
    ctx = ctypes.c_void_p()
    assert L.ktri_ctx_create(0, ctypes.byref(ctx)) == _native.OK
    plan = ctypes.c_void_p()
    opts = Config().opts()
    assert L.ktri_plan_create_batch(ctx, fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(),
                                    b.num_graphs, tot.data_ptr(), None, ctypes.byref(opts),
                                    ctypes.byref(plan)) == _native.OK
    assert L.ktri_plan_launch(plan, None) == _native.OK
    assert L.ktri_plan_check(plan) == _native.OK
    expect = tot.clone()
    assert L.ktri_ctx_destroy(ctx) == _native.OK
    assert L.ktri_plan_destroy(plan) == _native.OK
    with TriangleCounter(0) as ctr:
        out = torch.zeros_like(tot)
        ctr.count_batch_device(fo.data_ptr(), hd.data_ptr(), b.union.n, b.union.nnz, gf.data_ptr(), b.num_graphs,
                               out.data_ptr(), None, Config())
        ctr.check()
        assert torch.equal(out, expect)
