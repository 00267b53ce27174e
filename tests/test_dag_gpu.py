"""The katric local phase on lists the caller oriented (needs a GB300): ktri_count_dag counts
the triangles whose three edges appear in the given out-lists, whatever the orientation, with
ghosts as ordinary list owners (CetricEdgeIterator::run_local, cetric_edge_iterator.h:230-388).
The bar is bit-exactness against the oracle on the undirected graph of the same edges."""
import numpy as np
import pytest

from katric_gb300 import Graph, KtriError, _native

pytestmark = pytest.mark.gpu


def undirected_csr(n, src, dst):
    s = np.concatenate([src, dst]).astype(np.int64)
    d = np.concatenate([dst, src]).astype(np.int64)
    order = np.lexsort((d, s))
    fo = np.zeros(n + 1, dtype=np.uint64)
    fo[1:] = np.cumsum(np.bincount(s[order], minlength=n))
    return fo, d[order].astype(np.uint32)


def oriented_lists(n, src, dst, rank, seed):
    """Out-lists of the edges (src[i], dst[i]) oriented from lower to higher rank, shuffled."""
    fwd = rank[src] < rank[dst]
    a = np.where(fwd, src, dst).astype(np.int64)
    b = np.where(fwd, dst, src).astype(np.int64)
    order = np.argsort(a, kind="stable")
    a, b = a[order], b[order]
    fo = np.zeros(n + 1, dtype=np.uint64)
    fo[1:] = np.cumsum(np.bincount(a, minlength=n))
    rng = np.random.default_rng(seed)
    hd = b.astype(np.uint32)
    for v in range(n):
        rng.shuffle(hd[int(fo[v]):int(fo[v + 1])])
    return fo, hd


def edges_of(g: Graph):
    fo = g.first_out.astype(np.int64)
    src = np.repeat(np.arange(g.n), np.diff(fo))
    dst = g.head.astype(np.int64)
    keep = src < dst
    return src[keep], dst[keep]


@pytest.mark.parametrize("gen", ["rmat", "gnm", "rgg"])
def test_any_orientation_counts_the_graph(counter, oracle, gen):
    g = {"rmat": lambda: Graph.rmat(12, 16, seed=7), "gnm": lambda: Graph.gnm(3000, 40000, seed=8),
         "rgg": lambda: Graph.rgg2d(4000, 24.0, seed=9)}[gen]()
    src, dst = edges_of(g)
    want_t, want_pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    rng = np.random.default_rng(3)
    for rank in (rng.permutation(g.n), np.arange(g.n), np.arange(g.n)[::-1].copy()):
        fo, hd = oriented_lists(g.n, src, dst, rank, seed=4)
        t, pv = counter.count_dag(fo, hd)
        assert t == want_t
        assert np.array_equal(pv, want_pv)


def test_rank_local_phase_with_ghosts(counter, oracle):
    """Two ranks own halves of the vertices.  Rank r's lists: out_adj of its vertices (to local
    vertices or ghosts) and ghost_adj of its ghosts (to local vertices), oriented by (degree, id)
    as degree_outward does.  The local phase finds the triangles with at most one ghost."""
    g = Graph.rmat(11, 16, seed=12)
    src, dst = edges_of(g)
    deg = np.diff(g.first_out.astype(np.int64))
    key = deg * (1 << 32) + np.arange(g.n)
    owner = (np.arange(g.n) >= g.n // 2).astype(np.int64)
    for r in (0, 1):
        keep = (owner[src] == r) | (owner[dst] == r)  # edges with a local endpoint
        s, d = src[keep], dst[keep]
        verts = np.unique(np.concatenate([s, d]))
        local_id = np.full(g.n, -1, dtype=np.int64)
        local_id[verts] = np.arange(len(verts))
        ls, ld = local_id[s], local_id[d]
        nr = len(verts)
        fo, hd = oriented_lists(nr, ls, ld, np.argsort(np.argsort(key[verts])), seed=r)
        t, pv = counter.count_dag(fo, hd)
        ufo, uhd = undirected_csr(nr, ls, ld)
        want_t, want_pv, _ = oracle.count(ufo, uhd, num_threads=8)
        assert t == want_t and np.array_equal(pv, want_pv)


def test_dag_device_entry_point(counter, oracle):
    torch = pytest.importorskip("torch")
    g = Graph.rmat(13, 16, seed=5)
    src, dst = edges_of(g)
    fo, hd = oriented_lists(g.n, src, dst, np.random.default_rng(1).permutation(g.n), seed=2)
    dfo = torch.from_numpy(fo.view(np.int64).copy()).cuda()
    dhd = torch.from_numpy(hd.view(np.int32).copy()).cuda()
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    pv = torch.zeros(g.n, dtype=torch.int64, device="cuda")
    counter.count_dag_device(dfo.data_ptr(), dhd.data_ptr(), g.n, len(hd), tot.data_ptr(), pv.data_ptr())
    counter.check()
    want_t, want_pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    assert int(tot.item()) == want_t
    assert np.array_equal(pv.cpu().numpy().view(np.uint64), want_pv)


def test_dag_edge_cases_and_errors(counter):
    # empty, edgeless, one triangle given in one orientation
    assert counter.count_dag(np.zeros(1, np.uint64), np.zeros(0, np.uint32))[0] == 0
    assert counter.count_dag(np.zeros(6, np.uint64), np.zeros(0, np.uint32))[0] == 0
    t, pv = counter.count_dag(np.array([0, 2, 3, 3], np.uint64), np.array([2, 1, 2], np.uint32))
    assert t == 1 and list(pv) == [1, 1, 1]
    for fo, hd in [(np.array([0, 1, 1], np.uint64), np.array([5], np.uint32)),   # id out of range
                   (np.array([0, 1, 1], np.uint64), np.array([0], np.uint32))]:  # self-loop
        with pytest.raises(KtriError) as e:
            counter.count_dag(fo, hd)
        assert e.value.code == _native.ERR_INVALID_CSR
    t, _ = counter.count_dag(np.array([0, 2, 3, 3], np.uint64), np.array([2, 1, 2], np.uint32))
    assert t == 1  # the context stays usable after an error


def rank_lists(g: Graph, r: int, ranks: int, seed: int):
    """Rank r's oriented lists with its own vertices numbered first: (fo, head, n_local)."""
    src, dst = edges_of(g)
    owner = (np.arange(g.n) * ranks) // g.n
    keep = (owner[src] == r) | (owner[dst] == r)
    s, d = src[keep], dst[keep]
    local = np.flatnonzero(owner == r)
    ghosts = np.setdiff1d(np.unique(np.concatenate([s, d])), local)
    order = np.concatenate([local, ghosts])
    idx = np.full(g.n, -1, dtype=np.int64)
    idx[order] = np.arange(len(order))
    deg = np.diff(g.first_out.astype(np.int64))
    key = deg * (1 << 32) + np.arange(g.n)
    fo, hd = oriented_lists(len(order), idx[s], idx[d], np.argsort(np.argsort(key[order])), seed=seed)
    return fo, hd, len(local)


@pytest.mark.parametrize("ranks", [2, 4])
def test_contraction_after_local_phase(counter, ranks):
    """remove_internal_edges + compact + id sort (cetric.h:872-930): every local vertex keeps
    its ghost out-neighbours, sorted; vertices left without any are dropped."""
    g = Graph.rmat(12, 16, seed=21)
    for r in range(ranks):
        fo, hd, nl = rank_lists(g, r, ranks, seed=r)
        kept, cfo, chd = counter.contract_dag(fo, hd, nl)
        want_kept, want_lists = [], []
        f = fo.astype(np.int64)
        for v in range(nl):
            gl = np.sort(hd[f[v]:f[v + 1]][hd[f[v]:f[v + 1]] >= nl])
            if len(gl):
                want_kept.append(v)
                want_lists.append(gl)
        assert list(kept) == want_kept
        assert cfo[0] == 0 and len(cfo) == len(want_kept) + 1
        assert np.array_equal(np.diff(cfo.astype(np.int64)), [len(x) for x in want_lists])
        assert np.array_equal(chd, np.concatenate(want_lists) if want_lists else np.zeros(0, np.uint32))


def test_contraction_edge_cases(counter):
    kept, cfo, chd = counter.contract_dag(np.array([0, 1, 1], np.uint64), np.array([1], np.uint32), 2)
    assert len(kept) == 0 and list(cfo) == [0] and len(chd) == 0       # no ghosts: nothing survives
    kept, cfo, chd = counter.contract_dag(np.array([0, 0, 0], np.uint64), np.zeros(0, np.uint32), 0)
    assert len(kept) == 0 and list(cfo) == [0]
    # a hub with a long ghost list (sorted through global scratch) next to short ones
    nl, ng = 3, 20000
    rng = np.random.default_rng(2)
    lists = [rng.permutation(np.arange(nl, nl + ng)).astype(np.uint32), np.array([nl + 5, 1], np.uint32),
             np.zeros(0, np.uint32)]
    fo = np.zeros(nl + ng + 1, np.uint64)
    fo[1:nl + 1] = np.cumsum([len(x) for x in lists])
    fo[nl + 1:] = fo[nl]
    kept, cfo, chd = counter.contract_dag(fo, np.concatenate(lists), nl)
    assert list(kept) == [0, 1] and list(cfo) == [0, ng, ng + 1]
    assert np.array_equal(chd[:ng], np.arange(nl, nl + ng)) and chd[ng] == nl + 5
