"""Full-size workloads (the headline shapes) checked against the oracle on a GB300.

tests/golden/fullsize.json holds full, unsampled oracle runs of RMAT scale 24 (seed 2), the
2D RGG with n = 2^24 (seed 3) and the 8192-graph batch (seed 4), made by
tests/golden/make_fullsize.py: SHA-256 digests of the CSR bytes, the exact totals, and
SHA-256 digests of the per-vertex counts (per-graph totals for the batch).  Each test
regenerates the graph, proves it is byte-identical to the one the oracle counted, counts it on
the GPU and compares total and per-vertex digest -- bit-exact parity at full size.  RGG-24 is
also counted by the oracle inline (a few seconds on the host).  Two kernel splits (different
owner bins and tile segments, so different kernels handle each edge) must agree as well."""
import hashlib
import json
import os

import numpy as np
import pytest

from katric_gb300 import Batch, Config, Graph, TriangleCounter

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fullsize.json")


def _fixture(name):
    with open(FIXTURE) as f:
        return json.load(f)[name]


def _sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).view(np.uint8).data)
    return h.hexdigest()


@pytest.mark.parametrize("workload", ["rmat24", "rgg24"])
def test_full_size_against_oracle(workload, oracle):
    torch = pytest.importorskip("torch")
    fx = _fixture(workload)
    g = Graph.rmat(24, 16, seed=2) if workload == "rmat24" else Graph.rgg2d(1 << 24, 32.0, seed=3)
    assert (g.n, g.nnz) == (fx["n"], fx["nnz"])
    assert _sha(g.first_out) == fx["first_out_sha256"] and _sha(g.head) == fx["head_sha256"], \
        "the generator produced other bytes than the graph the oracle counted"
    fo = torch.from_numpy(g.first_out.view(np.int64)).cuda()
    hd = torch.from_numpy(g.head.view(np.int32)).cuda()
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    with TriangleCounter(0) as ctr:
        for conf in (Config(), Config(small_outdegree=8, medium_outdegree=64, segment=256)):
            pv = torch.zeros(g.n, dtype=torch.int64, device="cuda")
            ctr.count_device(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, tot.data_ptr(), pv.data_ptr(), conf)
            ctr.check()
            p = pv.cpu().numpy().view(np.uint64)
            assert int(tot.item()) == fx["total"]
            assert _sha(p.astype("<u8")) == fx["per_vertex_sha256"]
            assert all(int(p[int(v)]) == c for v, c in fx["spot"].items())
            del pv
    if workload == "rgg24":
        total, opv, _ = oracle.count(g.first_out, g.head, num_threads=os.cpu_count() or 4)
        assert total == fx["total"] and np.array_equal(opv, p)


def test_batch8192_against_oracle():
    """The 8192-graph batched workload: the captured plan's per-graph totals and the union's
    per-vertex counts against the oracle's graph-by-graph run."""
    torch = pytest.importorskip("torch")
    fx = _fixture("batch8192")
    b = Batch.generate(8192, 8.0, 17.0, 4.0, 64.0, 4)
    assert (b.num_graphs, b.union.n, b.union.nnz) == (fx["graphs"], fx["n_total"], fx["nnz_total"])
    assert _sha(b.union.first_out) == fx["first_out_sha256"] and _sha(b.union.head) == fx["head_sha256"]
    assert _sha(b.graph_first.astype("<u8")) == fx["graph_first_sha256"]
    dev = torch.device("cuda")
    fo = torch.from_numpy(b.union.first_out.view(np.int64)).to(dev)
    hd = torch.from_numpy(b.union.head.view(np.int32)).to(dev)
    gf = torch.from_numpy(b.graph_first.view(np.int64)).to(dev)
    n, nnz, k = b.union.n, b.union.nnz, b.num_graphs
    del b
    tot = torch.zeros(k, dtype=torch.int64, device=dev)
    pv = torch.zeros(n, dtype=torch.int64, device=dev)
    with TriangleCounter(0) as ctr:
        plan = ctr.plan_batch(fo.data_ptr(), hd.data_ptr(), n, nnz, gf.data_ptr(), k, tot.data_ptr(), pv.data_ptr(),
                              Config(small_outdegree=48))
        plan.launch()
        plan.check()
        totals = tot.cpu().numpy().view(np.uint64).astype("<u8")
        assert int(totals.sum()) == fx["totals_sum"]
        assert [int(x) for x in totals[:16]] == fx["totals_first16"]
        assert _sha(totals) == fx["totals_sha256"]
        assert _sha(pv.cpu().numpy().view(np.uint64).astype("<u8")) == fx["per_vertex_sha256"]
        plan.close()


def test_list_starts_beyond_2_32_entries():
    """A graph whose gapped out-list array exceeds 2^32 entries (1.45e9 vertices, nearly all
    isolated) still uses 32-bit descriptors, which hold list starts in 16-byte groups: a
    triangle on the first three vertices and a K_300 on the last 300 (owners of out-degree up
    to 299, so the large-owner kernel reads lists beyond entry 2^32) count exactly, and the
    same as with 64-bit descriptors forced."""
    torch = pytest.importorskip("torch")
    n, k = 1_450_000_000, 300
    assert n * 3 + 8 > 1 << 32
    dev = torch.device("cuda")
    fo = torch.full((n + 1,), 6, dtype=torch.int64, device=dev)
    fo[0], fo[1], fo[2] = 0, 2, 4
    fo[n - k:] = 6 + (k - 1) * torch.arange(k + 1, dtype=torch.int64, device=dev)
    ids = torch.arange(n - k, n, dtype=torch.int64, device=dev)
    clique = ids.repeat(k, 1)[~torch.eye(k, dtype=torch.bool, device=dev)]  # row v: the others, ascending
    head = torch.cat([torch.tensor([1, 2, 0, 2, 0, 1], dtype=torch.int64, device=dev), clique]).to(torch.int32)
    nnz = head.numel()
    assert int(fo[n].item()) == nnz
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    expect = 1 + k * (k - 1) * (k - 2) // 6
    with TriangleCounter(0) as ctr:
        for wide in (False, True):
            pv = torch.zeros(n, dtype=torch.int64, device=dev)
            ctr.count_device(fo.data_ptr(), head.data_ptr(), n, nnz, tot.data_ptr(), pv.data_ptr(),
                             Config(force_wide_offsets=wide))
            ctr.check()
            assert int(tot.item()) == expect
            assert pv[:3].tolist() == [1, 1, 1]
            assert torch.all(pv[n - k:] == (k - 1) * (k - 2) // 2)
            assert int(pv.sum().item()) == 3 * expect
            del pv
