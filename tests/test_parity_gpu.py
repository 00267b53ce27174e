"""Parity of the CUDA path with the CPU oracle, through the C ABI (needs a GB300).

Bar: bit-exact u64 totals and per-vertex counts for every intersection method, on the
reference's example graphs, on the small G(n,m) workload (n=2^14, m=2^17, seed 1) and on
seeded RMAT / RGG graphs at sizes the oracle finishes in seconds; unsorted input lists;
edge cases (empty, edgeless, single triangle, star, cliques whose out-lists need chunked
tables); invalid CSR reported as KTRI_ERR_INVALID_CSR.
"""
import ctypes

import numpy as np
import pytest

from katric_gb300 import Config, Graph, KtriError, _native

pytestmark = pytest.mark.gpu

GPU_METHODS = ["auto", "merge", "binary-search", "binary", "hybrid"]


def check_parity(counter, oracle, fo, hd, methods=GPU_METHODS, threads=8):
    total, pv, _ = oracle.count(fo, hd, method="merge", num_threads=threads)
    for m in methods:
        t, p = counter.count(fo, hd, Config(intersection_method=m))
        assert t == total, (m, t, total)
        assert np.array_equal(p, pv), m
    return total


def csr_from_edges(n, edges, shuffle_seed=None):
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    src = np.concatenate([e[:, 0], e[:, 1]])
    dst = np.concatenate([e[:, 1], e[:, 0]])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    fo = np.zeros(n + 1, dtype=np.uint64)
    fo[1:] = np.cumsum(np.bincount(src, minlength=n))
    hd = dst.astype(np.uint32)
    if shuffle_seed is not None:
        rng = np.random.default_rng(shuffle_seed)
        for v in range(n):
            rng.shuffle(hd[int(fo[v]):int(fo[v + 1])])
    return fo, hd


def test_examples(counter, oracle, golden):
    ex, _ = golden
    for g in ex["graphs"]:
        t = check_parity(counter, oracle, g["first_out"], g["head"])
        assert t == g["triangles"], g["name"]


def test_gnm_small_workload(counter, oracle):
    g = Graph.gnm(1 << 14, 1 << 17, seed=1)
    check_parity(counter, oracle, g.first_out, g.head)


@pytest.mark.parametrize("scale", [10, 14, 16])
def test_rmat(counter, oracle, scale):
    g = Graph.rmat(scale, 16, seed=2)
    check_parity(counter, oracle, g.first_out, g.head)


@pytest.mark.parametrize("n", [1 << 12, 1 << 16])
def test_rgg(counter, oracle, n):
    g = Graph.rgg2d(n, 32.0, seed=3)
    check_parity(counter, oracle, g.first_out, g.head)


@pytest.mark.parametrize("method", ["auto", "merge"])
def test_wide_offsets(counter, oracle, method):
    """64-bit out-list offsets (the path of unions with nnz + 3n > 2^32), forced on small graphs."""
    for g in (Graph.rmat(14, 16, seed=2), Graph.rgg2d(1 << 14, 32.0, seed=3), Graph.gnm(1 << 14, 1 << 17, seed=1)):
        total, pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
        t, p = counter.count(g.first_out, g.head, Config(intersection_method=method, force_wide_offsets=True))
        assert t == total and np.array_equal(p, pv)


def test_unsorted_lists(counter, oracle):
    g = Graph.rmat(13, 16, seed=5)
    fo = g.first_out
    hd = g.head.copy()
    rng = np.random.default_rng(1)
    for v in range(g.n):
        a, b = int(fo[v]), int(fo[v + 1])
        rng.shuffle(hd[a:b])
    check_parity(counter, oracle, fo, hd)
    assert counter.stats().input_sorted == 0


def test_empty_and_edgeless(counter):
    t, p = counter.count(np.zeros(1, np.uint64), np.zeros(0, np.uint32))
    assert t == 0 and len(p) == 0
    t, p = counter.count(np.zeros(6, np.uint64), np.zeros(0, np.uint32))
    assert t == 0 and (p == 0).all() and len(p) == 5


def test_single_triangle_and_star(counter, oracle):
    fo, hd = csr_from_edges(4, [(0, 1), (1, 2), (0, 2)])
    assert check_parity(counter, oracle, fo, hd) == 1
    star = [(0, i) for i in range(1, 3000)] + [(1, 2), (5, 6)]
    fo, hd = csr_from_edges(3000, star)
    assert check_parity(counter, oracle, fo, hd) == 2


@pytest.mark.parametrize("k", [40, 700])
def test_cliques(counter, oracle, k):
    """Cliques: every vertex has the same degree, so ties in (degree, id) decide the orientation."""
    edges = [(a, b) for a in range(k) for b in range(a + 1, k)]
    fo, hd = csr_from_edges(k + 3, edges + [(k, k + 1)], shuffle_seed=3)
    t = check_parity(counter, oracle, fo, hd)
    assert t == k * (k - 1) * (k - 2) // 6


def test_big_clique_chunked_tables(counter):
    """K_4200: out-degrees up to 4199 exceed one shared-memory table chunk (4096 keys).
    Checked against the closed form (the oracle would take minutes)."""
    k = 4200
    a, b = np.triu_indices(k, 1)
    fo, hd = csr_from_edges(k + 3, list(zip(a.tolist(), b.tolist())) + [(k, k + 1)])
    t, pv = counter.count(fo, hd, Config(intersection_method="auto"))
    assert t == k * (k - 1) * (k - 2) // 6
    assert (pv[:k] == (k - 1) * (k - 2) // 2).all() and (pv[k:] == 0).all()


def test_many_components_mixed(counter, oracle):
    """Disjoint union of a hub-heavy RMAT, an RGG and cliques: tiles mix small and large owners."""
    parts = [Graph.rmat(11, 16, seed=9), Graph.rgg2d(3000, 24.0, seed=4), Graph.gnm(500, 20000, seed=8)]
    fo = [0]
    hd = []
    off = 0
    for g in parts:
        f = g.first_out.astype(np.int64)
        for v in range(g.n):
            hd.extend((g.head[f[v]:f[v + 1]].astype(np.int64) + off).tolist())
            fo.append(len(hd))
        off += g.n
    check_parity(counter, oracle, np.array(fo, np.uint64), np.array(hd, np.uint32))


@pytest.mark.parametrize("small,medium,segment", [(1, 1, 64), (8, 64, 128), (16, 256, 256), (32, 32, 512),
                                                   (32, 128, 1024), (4, 200, 64), (48, 48, 1024), (40, 256, 256)])
def test_bin_thresholds_and_segments(counter, oracle, small, medium, segment):
    """Every owner-bin split and tile segment gives the same counts (the autotuner's space)."""
    graphs = [Graph.rmat(14, 16, seed=4), Graph.rgg2d(1 << 13, 24.0, seed=5)]
    fo, hd = csr_from_edges(300, [(i, j) for i in range(300) for j in range(i + 1, 300)
                                  if (i * 7 + j * 3) % 5 != 0])
    for g_fo, g_hd in [(g.first_out, g.head) for g in graphs] + [(fo, hd)]:
        total, pv, _ = oracle.count(g_fo, g_hd, method="merge", num_threads=8)
        t, p = counter.count(g_fo, g_hd, Config(small_outdegree=small, medium_outdegree=medium, segment=segment))
        assert t == total and np.array_equal(p, pv), (small, medium, segment)


@pytest.mark.parametrize("bad", [dict(small_outdegree=49), dict(small_outdegree=16, medium_outdegree=8),
                                 dict(medium_outdegree=257), dict(segment=100), dict(segment=32),
                                 dict(segment=2048)])
def test_bad_bin_options(counter, bad):
    g = Graph.gnm(1 << 10, 1 << 13, seed=3)
    with pytest.raises(KtriError) as e:
        counter.count(g.first_out, g.head, Config(**bad))
    assert e.value.code == _native.ERR_INVALID_ARGUMENT


def test_invalid_csr(counter):
    fo = np.array([0, 2, 3, 4], dtype=np.uint64)
    with pytest.raises(KtriError) as e:  # self-loop 0-0
        counter.count(fo, np.array([0, 1, 0, 0], dtype=np.uint32))
    assert e.value.code == _native.ERR_INVALID_CSR
    with pytest.raises(KtriError) as e:  # id out of range
        counter.count(fo, np.array([1, 7, 0, 0], dtype=np.uint32))
    assert e.value.code == _native.ERR_INVALID_CSR
    with pytest.raises(KtriError) as e:  # non-monotone offsets
        counter.count(np.array([0, 3, 1, 4], dtype=np.uint64), np.array([1, 2, 0, 0], dtype=np.uint32))
    assert e.value.code == _native.ERR_INVALID_CSR
    with pytest.raises(KtriError) as e:  # duplicate entry in a sorted list
        counter.count(np.array([0, 2, 3, 4], dtype=np.uint64), np.array([1, 1, 0, 0], dtype=np.uint32))
    assert e.value.code == _native.ERR_INVALID_CSR
    # the context stays usable after errors
    f2, h2 = csr_from_edges(3, [(0, 1), (1, 2), (0, 2)])
    assert counter.count(f2, h2)[0] == 1


def test_stats_match_reference_counters(counter, oracle):
    g = Graph.rmat(12, 16, seed=2)
    total, _, st = oracle.count(g.first_out, g.head, num_threads=4)
    t, _ = counter.count(g.first_out, g.head, Config(collect_stats=True))
    rs = counter.stats()
    assert t == total
    assert rs.wedge_checks == st["wedge_checks"]
    assert rs.intersection_size_local == st["intersection_size_local"]
    assert rs.oriented_edges * 2 == g.nnz
    assert rs.streamed_entries <= rs.wedge_checks


def test_orientation_export(counter, oracle, golden):
    ex, _ = golden
    graphs = [(g["first_out"], g["head"]) for g in ex["graphs"]]
    big = Graph.rmat(12, 16, seed=6)
    graphs.append((big.first_out, big.head))
    for fo, hd in graphs:
        ofo, oh = counter.orient(fo, hd)
        efo, eh = oracle.oriented_csr(fo, hd)
        assert np.array_equal(ofo, efo)
        assert np.array_equal(oh, eh)


@pytest.mark.parametrize("method", GPU_METHODS)
def test_intersection_kat_gpu(counter, golden, method):
    _, kat = golden
    pairs = []
    expect = []
    for a, b, e in kat["triples"]:
        pairs += [(a, b), (b, a)]
        expect += [e, e]
    got = counter.intersect_pairs(pairs, method=method)
    for g, e in zip(got, expect):
        assert (sorted(g) if method in ("binary", "auto") else g) == e


@pytest.mark.parametrize("method", GPU_METHODS)
def test_intersection_random_gpu(counter, method):
    rng = np.random.default_rng(11)
    pairs = []
    for _ in range(200):
        na, nb = rng.integers(0, 1500, size=2)
        hi = int(rng.choice([100, 5000, 1 << 30]))
        a = np.unique(rng.integers(1, hi, size=na)).astype(np.uint32)
        b = np.unique(rng.integers(1, hi, size=nb)).astype(np.uint32)
        pairs.append((a, b))
    got = counter.intersect_pairs(pairs, method=method)
    for (a, b), g in zip(pairs, got):
        assert sorted(g) == np.intersect1d(a, b).tolist()


@pytest.mark.parametrize("gen", ["rmat", "gnm", "clique"])
def test_list_triangles_no_duplicates(counter, oracle, gen):
    """The debug check of run_shmem (shared_memory_cetric.h:151-167): every emitted triangle,
    sorted, has no duplicate; here also every row is a triangle and the rows number the total."""
    if gen == "clique":
        fo, hd = csr_from_edges(40, [(i, j) for i in range(40) for j in range(i + 1, 40)])
    else:
        g = Graph.rmat(10, 16, seed=3) if gen == "rmat" else Graph.gnm(2000, 12000, seed=4)
        fo, hd = g.first_out, g.head
    total = oracle.count(fo, hd, num_threads=4)[0]
    tri = counter.list_triangles(fo, hd)
    assert len(tri) == total
    assert np.all(tri[:, 0] < tri[:, 1]) and np.all(tri[:, 1] < tri[:, 2])
    keys = (tri[:, 0].astype(np.uint64) << np.uint64(42)) | (tri[:, 1].astype(np.uint64) << np.uint64(21)) | \
        tri[:, 2].astype(np.uint64)
    assert len(np.unique(keys)) == len(keys)
    n = len(fo) - 1
    adj = set()
    f = fo.astype(np.int64)
    for v in range(n):
        for u in hd[f[v]:f[v + 1]]:
            adj.add((v, int(u)))
    for x, y, z in tri[:2000].tolist():
        assert (x, y) in adj and (y, z) in adj and (x, z) in adj
    with pytest.raises(KtriError) as e:
        counter.list_triangles(fo, hd, capacity=max(0, total - 1))
    assert e.value.code == _native.ERR_OUT_OF_MEMORY


@pytest.mark.parametrize("chunk", [0, 4096, 8 * 1000 + 8])
def test_count_binary_file_overlapped_ingest(counter, oracle, tmp_path, chunk):
    """Counting straight from the reference's binary format (u64 .first_out / .head), the file
    read in chunks overlapping the host-to-device copies."""
    g = Graph.rmat(13, 16, seed=11)
    stem = str(tmp_path / "g")
    g.write_binary(stem)
    want_t, want_pv, _ = oracle.count(g.first_out, g.head, num_threads=8)
    t, pv = counter.count_binary_file(stem, chunk_bytes=chunk)
    assert t == want_t and np.array_equal(pv, want_pv)


def test_count_binary_file_errors(counter, tmp_path):
    with pytest.raises(KtriError) as e:
        counter.count_binary_file(str(tmp_path / "missing"))
    assert e.value.code == _native.ERR_IO
    stem = str(tmp_path / "bad")
    np.array([0, 2, 3, 3], np.uint64).tofile(stem + ".first_out")
    np.array([1, 7, 0], np.uint64).tofile(stem + ".head")  # id 7 >= n
    with pytest.raises(KtriError) as e:
        counter.count_binary_file(stem)
    assert e.value.code == _native.ERR_INVALID_CSR
    np.array([0, 2, 3, 4], np.uint64).tofile(stem + ".first_out")  # first_out[n] != nnz
    with pytest.raises(KtriError) as e:
        counter.count_binary_file(stem)
    assert e.value.code == _native.ERR_INVALID_CSR


@pytest.mark.parametrize("fn", ["N", "D", "DH", "DDH", "DH2", "DPD", "IDPD"])
def test_cost_functions_and_partition(counter, fn):
    """The reference's load-balancing costs (cost_function.h:287-376), computed on the device,
    against numpy; the cut points split the cost prefix evenly."""
    g = Graph.rmat(12, 16, seed=8)
    fo = g.first_out.astype(np.int64)
    n = g.n
    deg = np.diff(fo)
    src = np.repeat(np.arange(n), deg)
    dst = g.head.astype(np.int64)
    key = deg * (1 << 32) + np.arange(n)
    up = key[dst] > key[src]
    dplus = np.bincount(src[up], minlength=n)
    if fn in ("DPD", "IDPD"):
        sel = up if fn == "DPD" else ~up
        want = np.bincount(src[sel], weights=(dplus[src] + dplus[dst])[sel], minlength=n).astype(np.int64)
    else:
        want = {"N": np.ones(n, np.int64), "D": deg, "DH": dplus, "DDH": deg * dplus, "DH2": dplus * dplus}[fn]
    parts = 7
    bnd, total, cost = counter.partition_cost(g.first_out, g.head, fn, parts, costs=True)
    assert np.array_equal(cost.astype(np.int64), want) and total == int(want.sum())
    prefix = np.concatenate([[0], np.cumsum(want)])
    assert bnd[0] == 0 and bnd[-1] == n and np.all(np.diff(bnd.astype(np.int64)) >= 0)
    for i in range(1, parts):
        b = int(bnd[i])
        target = -(-total * i // parts)
        assert prefix[b] >= target and (b == 0 or prefix[b - 1] < target)
