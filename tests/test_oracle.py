"""The CPU oracle pinned against the reference's own golden vectors (no GPU).

Pins: the ten hand-written intersection triples (tests/intersection_test.cpp:41-50, each run
both ways round, merge/binary-search exact order, binary unordered, :56-93), the random
intersection check against a set-intersection oracle (:96-172), the example totals
(examples/examples.yaml: triangle=1, metis-sample=4, hiv=45) and the orientation invariant
(tests/orientation_test.cpp:98-120: out-edges union in-edges equals the adjacency).
"""
import random

import numpy as np
import pytest

METHODS = ["merge", "binary-search", "binary", "hybrid"]


@pytest.mark.parametrize("method", METHODS)
def test_intersection_kat(oracle, golden, method):
    _, kat = golden
    assert len(kat["triples"]) == 10
    for a, b, expected in kat["triples"]:
        for x, y in ((a, b), (b, a)):
            got = oracle.intersect(x, y, method)
            if method == "binary":
                assert sorted(got) == expected
            else:
                assert got == expected


@pytest.mark.parametrize("method", METHODS)
def test_intersection_random(oracle, method):
    rng = random.Random(7)
    for _ in range(100):
        sizes = [rng.randint(0, 1000) for _ in range(2)]
        lists = [sorted(set(rng.randint(1, 100) for _ in range(s))) for s in sizes]
        for v2_empty in (False, True):
            a, b = lists[0], ([] if v2_empty else lists[1])
            for x, y in ((a, b), (b, a)):
                expected = sorted(set(x) & set(y))
                got = oracle.intersect(x, y, method, cutoff=rng.choice([0, 3, 1000]))
                assert sorted(got) == expected
                if method != "binary":
                    assert got == expected


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("threads", [1, 4])
def test_example_totals(oracle, golden, method, threads):
    ex, _ = golden
    for g in ex["graphs"]:
        total, pv, st = oracle.count(g["first_out"], g["head"], method=method, num_threads=threads)
        assert total == g["triangles"], g["name"]
        assert int(pv.sum()) == 3 * total
        assert st["triangles"] == total


def test_binary_format_matches_metis(golden):
    ex, _ = golden
    seen = 0
    for g in ex["graphs"]:
        if "binary_head" not in g:
            continue
        seen += 1
        fo, hd = g["first_out"], g["head"]
        bfo, bhd = g["binary_first_out"], g["binary_head"]
        assert bfo == fo
        for v in range(g["n"]):
            assert sorted(bhd[bfo[v]:bfo[v + 1]]) == sorted(hd[fo[v]:fo[v + 1]])
    assert seen == 2


def test_orientation_invariant(oracle, golden):
    ex, _ = golden
    for g in ex["graphs"]:
        fo = np.array(g["first_out"], dtype=np.uint64)
        hd = np.array(g["head"], dtype=np.uint32)
        ofo, oh = oracle.oriented_csr(fo, hd)
        n = len(fo) - 1
        deg = np.diff(fo)
        assert int(ofo[-1]) * 2 == len(hd)
        inn = [[] for _ in range(n)]
        for v in range(n):
            outs = oh[ofo[v]:ofo[v + 1]].tolist()
            assert outs == sorted(outs)
            for u in outs:
                assert (deg[v], v) < (deg[u], u)
                inn[u].append(v)
        for v in range(n):
            adj = sorted(hd[fo[v]:fo[v + 1]].tolist())
            assert sorted(oh[ofo[v]:ofo[v + 1]].tolist() + inn[v]) == adj


def test_per_vertex_brute_force(oracle):
    """Per-vertex definition: +1 to each corner of every triangle (checked by enumeration)."""
    rng = np.random.default_rng(5)
    n = 40
    A = rng.random((n, n)) < 0.25
    A = np.triu(A, 1)
    A = A | A.T
    fo = np.zeros(n + 1, dtype=np.uint64)
    heads = []
    for v in range(n):
        nb = np.nonzero(A[v])[0].tolist()
        rng.shuffle(nb)  # unsorted input lists are allowed
        heads += nb
        fo[v + 1] = len(heads)
    expected = np.zeros(n, dtype=np.uint64)
    total = 0
    for a in range(n):
        for b in range(a + 1, n):
            if not A[a, b]:
                continue
            for c in range(b + 1, n):
                if A[a, c] and A[b, c]:
                    total += 1
                    expected[[a, b, c]] += 1
    for method in METHODS:
        t, pv, _ = oracle.count(fo, heads, method=method, num_threads=2)
        assert t == total
        assert (pv == expected).all()


def test_work_counters_match_their_definition(oracle):
    """The oracle's work counters, which give the roofline's algorithmic bytes, recomputed from
    the (degree, id) orientation in numpy: wedge_checks = sum over oriented edges (v,u) of
    |N+(u)| and intersection_size_local = sum of |N+(v)| + |N+(u)|
    (cetric_edge_iterator.h:279-281).  A sample stride of 1 counts the whole graph."""
    rng = np.random.default_rng(11)
    n, m = 300, 2500
    edges = set()
    while len(edges) < m:
        a, b = (int(x) for x in rng.integers(0, n, 2))
        if a != b:
            edges.add((min(a, b), max(a, b)))
    adj = [[] for _ in range(n)]
    for a, b in edges:
        adj[a].append(b)
        adj[b].append(a)
    fo = np.zeros(n + 1, dtype=np.uint64)
    fo[1:] = np.cumsum([len(a) for a in adj])
    head = np.array([u for a in adj for u in a], dtype=np.uint32)
    deg = np.array([len(a) for a in adj])
    key = lambda v: (deg[v], v)  # degree_outward, distributed_graph.h:148-163
    dplus = np.array([sum(1 for u in adj[v] if key(v) < key(u)) for v in range(n)])
    wedges = isz = 0
    for v in range(n):
        for u in adj[v]:
            if key(v) < key(u):
                wedges += int(dplus[u])
                isz += int(dplus[v] + dplus[u])
    for method in METHODS:
        t, _, st = oracle.count(fo, head, method=method, num_threads=2)
        assert st["wedge_checks"] == wedges and st["intersection_size_local"] == isz, method
        sc = oracle.SlicedCount(fo, head, 3, method=method, num_threads=2)
        parts = [sc.run(s) for s in range(3)]
        assert sum(p[0] for p in parts) == t and sum(p[1] for p in parts) == len(head), method
        assert sum(p[2]["wedge_checks"] for p in parts) == wedges, method
