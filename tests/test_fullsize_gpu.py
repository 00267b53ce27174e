"""Full-size workloads (RMAT scale 24 and RGG n = 2^24, the headline shapes) checked through
size-independent properties on a GB300: every triangle is counted once at each of its three
vertices (sum of per-vertex counts = 3 x total), and two independent kernel splits (different
owner bins and tile segments, so different kernels handle each edge) give the same exact
total and per-vertex counts.  The totals asserted here are those of a full run of the oracle
on the same graphs (16 host cores: 53.8 s for RMAT-24, 3.5 s for RGG-24), whose per-vertex
counts also matched the GPU's exactly; the oracle is too slow to rerun inside the test."""
import numpy as np
import pytest

from katric_gb300 import Config, Graph, TriangleCounter

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload", ["rmat24", "rgg24"])
def test_full_size_invariants(workload):
    torch = pytest.importorskip("torch")
    g = Graph.rmat(24, 16, seed=2) if workload == "rmat24" else Graph.rgg2d(1 << 24, 32.0, seed=3)
    fo = torch.from_numpy(g.first_out.view(np.int64)).cuda()
    hd = torch.from_numpy(g.head.view(np.int32)).cuda()
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    with TriangleCounter(0) as ctr:
        results = []
        for conf in (Config(), Config(small_outdegree=8, medium_outdegree=64, segment=256)):
            pv = torch.zeros(g.n, dtype=torch.int64, device="cuda")
            ctr.count_device(fo.data_ptr(), hd.data_ptr(), g.n, g.nnz, tot.data_ptr(), pv.data_ptr(), conf)
            ctr.check()
            results.append((int(tot.item()), pv))
        (t0, pv0), (t1, pv1) = results
        assert t0 == t1 and torch.equal(pv0, pv1)
        assert int(pv0.sum().item()) == 3 * t0
        assert t0 == {"rmat24": 10284079224, "rgg24": 1677814828}[workload]


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
