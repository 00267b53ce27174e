"""Orientation on graphs whose lists are spread across long runs of isolated vertices (needs a
GB300).

Merge-path tiles cut the sequence of vertex ends and adjacency slots evenly, so runs of isolated
vertices give tiles of vertex ends only (no slots: nothing to orient) and tiles whose first list
began many tiles earlier; a graph that ends in such a run has a last tile without slots.  Counts
and out-lists must equal the oracle's."""
import numpy as np
import pytest

from katric_gb300 import Config, Graph

pytestmark = pytest.mark.gpu


def _csr(n, edges):
    e = np.array(edges, dtype=np.int64)
    e = e[e[:, 0] != e[:, 1]]
    both = np.concatenate([e, e[:, ::-1]])
    both = np.unique(both, axis=0)
    fo = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(fo, both[:, 0] + 1, 1)
    fo = np.cumsum(fo).astype(np.uint64)
    return Graph(fo, both[:, 1].astype(np.uint32))


def _sparse_over_isolated(n, seed):
    rng = np.random.default_rng(seed)
    edges = []
    hubs = rng.choice(n - 1, size=24, replace=False)
    for h in hubs:  # stars whose leaves lie far apart: lists of one entry between long gaps
        leaves = rng.choice(n, size=int(rng.integers(50, 700)), replace=False)
        edges += [(int(h), int(v)) for v in leaves]
    spaced = np.arange(0, n, n // 45)[:45]  # a clique of far-apart vertices
    edges += [(int(a), int(b)) for i, a in enumerate(spaced) for b in spaced[i + 1:]]
    dense = np.arange(n // 2, n // 2 + 600)  # one dense region in the middle
    edges += [(int(a), int(b)) for a, b in rng.choice(dense, size=(20000, 2))]
    edges += [(int(a), int(b)) for a, b in rng.integers(0, n, size=(3000, 2))]
    return _csr(n, edges)


@pytest.mark.parametrize("n,seed", [(200_000, 1), (1_000_000, 2)])
def test_long_windows_against_the_oracle(counter, oracle, n, seed):
    g = _sparse_over_isolated(n, seed)
    isolated = int((np.diff(g.first_out) == 0).sum())
    assert isolated > n // 2  # most of the merge path is vertex ends
    total, pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    for method in ("auto", "merge"):
        t, p = counter.count(g.first_out, g.head, Config(intersection_method=method))
        assert t == total, method
        assert np.array_equal(p, pv), method
    ofo, oh = counter.orient(g.first_out, g.head)
    efo, eh = oracle.oriented_csr(g.first_out, g.head)
    assert np.array_equal(ofo, efo)
    assert np.array_equal(oh, eh)
