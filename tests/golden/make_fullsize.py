"""Pin the full-size workloads to the oracle: writes fullsize.json next to this script.

Usage: python tests/golden/make_fullsize.py [--threads T] [--only rmat24,rgg24,batch8192]

For each workload this generates the graph with the seeded generators (host code, the same
bytes on every machine), runs the FULL oracle count (no sampling: orientation, id sort and
the node-parallel merge local phase of the reference's run_shmem, restated in oracle/oracle.c)
and records:
  - n, nnz and SHA-256 digests of the CSR bytes (u64 first_out, u32 head, little-endian), so a
    test can prove it regenerated identical input before comparing counts;
  - the exact u64 total and a SHA-256 of the u64 per-vertex count array, plus its sum, its
    maximum and the counts of a few named vertices (readable spot values);
  - for the batch: the per-graph totals (their SHA-256, their sum and the first 16) and a
    SHA-256 of the union's per-vertex counts.  The batch is counted graph by graph (every
    graph on its own 0-based ids), as the reference would count each request.

The workloads:
  rmat24    RMAT scale 24, edge factor 16, (0.57, 0.19, 0.19, 0.05), seed 2
  rgg24     2D random geometric graph, n = 2^24, average degree 32, seed 3 (Morton order)
  batch8192 8192 graphs, n log-uniform in [2^8, 2^17], degree U(4, 64), G(n,m) / RMAT / RGG by
            index mod 3, graph i seeded with 4 + i

The GPU tests (tests/test_fullsize_gpu.py, tests/test_batch_gpu.py) read the JSON; nothing at
test time runs this script.  A full RMAT-24 oracle run takes about 160 s on 8 x86 cores.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "fullsize.json")


def sha256(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).view(np.uint8).data)
    return h.hexdigest()


def spot_vertices(n: int, deg: np.ndarray) -> list[int]:
    """A few fixed vertices plus the two of largest degree."""
    fixed = [0, 1, 2, 3, n // 3, n // 2, n - 2, n - 1]
    top = [int(v) for v in np.argsort(deg, kind="stable")[-2:]]
    return sorted(set(v for v in fixed + top if 0 <= v < n))


def pin_single(name: str, g, threads: int) -> dict:
    from oracle import oracle as O
    t0 = time.perf_counter()
    total, pv, st = O.count(g.first_out, g.head, method="merge", num_threads=threads)
    secs = time.perf_counter() - t0
    deg = np.diff(g.first_out)
    vs = spot_vertices(g.n, deg)
    return {
        "n": g.n, "nnz": g.nnz,
        "first_out_sha256": sha256(g.first_out), "head_sha256": sha256(g.head),
        "csr_sha256": sha256(g.first_out, g.head),
        "total": int(total),
        "per_vertex_sha256": sha256(pv.astype("<u8")),
        "per_vertex_sum": int(pv.sum(dtype=np.uint64)), "per_vertex_max": int(pv.max()),
        "spot": {str(v): int(pv[v]) for v in vs},
        "wedge_checks": int(st["wedge_checks"]),
        "oracle": {"method": "merge", "threads": threads, "seconds": round(secs, 1)},
    }


def pin_batch(b, threads: int) -> dict:
    from oracle import oracle as O
    k = b.num_graphs
    gf = b.graph_first.astype(np.int64)
    ufo = b.union.first_out
    totals = np.zeros(k, dtype=np.uint64)
    pv_union = np.zeros(b.union.n, dtype=np.uint64)
    t0 = time.perf_counter()
    for g in range(k):
        a, e = int(gf[g]), int(gf[g + 1])
        fo = ufo[a:e + 1] - ufo[a]
        hd = (b.union.head[int(ufo[a]):int(ufo[e])].astype(np.int64) - a).astype(np.uint32)
        t, pv, _ = O.count(fo, hd, method="merge", num_threads=threads)
        totals[g] = t
        pv_union[a:e] = pv
    secs = time.perf_counter() - t0
    return {
        "graphs": k, "n_total": b.union.n, "nnz_total": b.union.nnz,
        "graph_first_sha256": sha256(b.graph_first.astype("<u8")),
        "first_out_sha256": sha256(b.union.first_out), "head_sha256": sha256(b.union.head),
        "totals_sha256": sha256(totals.astype("<u8")), "totals_sum": int(totals.sum(dtype=np.uint64)),
        "totals_first16": [int(x) for x in totals[:16]],
        "per_vertex_sha256": sha256(pv_union.astype("<u8")),
        "oracle": {"method": "merge", "threads": threads, "seconds": round(secs, 1), "per_graph": True},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--only", default="rmat24,rgg24,batch8192")
    args = ap.parse_args()
    from katric_gb300 import Batch, Graph
    doc = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            doc = json.load(f)
    doc["about"] = ("Full oracle runs (tests/golden/make_fullsize.py) of the full-size workloads: CSR digests, "
                    "exact totals and per-vertex digests.")
    for name in args.only.split(","):
        t0 = time.perf_counter()
        if name == "rmat24":
            g = Graph.rmat(24, 16, 0.57, 0.19, 0.19, 2)
            entry = pin_single(name, g, args.threads)
            entry["generator"] = {"kind": "rmat", "scale": 24, "edge_factor": 16, "abcd": [0.57, 0.19, 0.19, 0.05],
                                  "seed": 2}
        elif name == "rgg24":
            g = Graph.rgg2d(1 << 24, 32.0, 3)
            entry = pin_single(name, g, args.threads)
            entry["generator"] = {"kind": "rgg2d", "n": 1 << 24, "avg_degree": 32.0, "seed": 3}
        elif name == "batch8192":
            b = Batch.generate(8192, 8.0, 17.0, 4.0, 64.0, 4)
            entry = pin_batch(b, args.threads)
            entry["generator"] = {"kind": "batch", "graphs": 8192, "log2_n": [8.0, 17.0], "degree": [4.0, 64.0],
                                  "seed": 4}
            del b
        else:
            raise SystemExit(f"unknown workload {name}")
        doc[name] = entry
        print(f"{name}: total {entry.get('total', entry.get('totals_sum'))} in {time.perf_counter() - t0:.0f} s",
              flush=True)
        with open(OUT, "w") as f:
            json.dump(doc, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main()
