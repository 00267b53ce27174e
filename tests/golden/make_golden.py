"""Regenerate the golden fixtures in this folder from a KaTric source tree.

Usage: python tests/golden/make_golden.py /path/to/katric

Reads, as text or raw bytes, only the reference's own test inputs:
  - examples/examples.yaml                      expected totals per example graph
  - examples/{triangle,metis-sample,hiv}.metis  METIS adjacency (1-based, header "n m [fmt]")
  - examples/{metis-sample,hiv}.{first_out,head} raw little-endian u64 CSR (binary input format)
  - tests/intersection_test.cpp                 the ten hand-written intersection triples

Writes examples.json and intersection_kat.json next to this script.  Nothing at
test time reads the reference tree; the tests read these JSON files.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_metis(path: str):
    """METIS text -> (first_out u64 list, head u32 list), 0-based, adjacency order kept."""
    with open(path) as f:
        lines = [ln.strip() for ln in f if not ln.lstrip().startswith("%")]
    header = lines[0].split()
    n, m = int(header[0]), int(header[1])
    first_out = [0]
    head = []
    for v in range(n):
        toks = lines[1 + v].split() if 1 + v < len(lines) else []
        head.extend(int(t) - 1 for t in toks)
        first_out.append(len(head))
    assert len(head) == 2 * m, (path, len(head), m)
    return first_out, head


def read_binary(stem: str):
    fo = np.fromfile(stem + ".first_out", dtype="<u8")
    hd = np.fromfile(stem + ".head", dtype="<u8")
    return fo.tolist(), hd.tolist()


def parse_yaml_totals(path: str):
    totals = {}
    name = None
    with open(path) as f:
        for ln in f:
            m = re.match(r"\s*-\s*name:\s*(\S+)", ln)
            if m:
                name = m.group(1)
            m = re.match(r"\s*triangles:\s*(\d+)", ln)
            if m and name:
                totals[name] = int(m.group(1))
    return totals


def parse_intersection_triples(path: str):
    src = open(path).read()
    triples = []
    for m in re.finditer(r"make_input\(\{([^}]*)\},\s*\{([^}]*)\},\s*\{([^}]*)\}\)", src):
        lists = [[int(x) for x in g.replace(" ", "").split(",") if x] for g in m.groups()]
        triples.append(lists)
    return triples


def main(ref: str) -> None:
    ex = os.path.join(ref, "examples")
    totals = parse_yaml_totals(os.path.join(ex, "examples.yaml"))
    graphs = []
    for name in ["triangle", "metis-sample", "hiv"]:
        fo, hd = read_metis(os.path.join(ex, name + ".metis"))
        entry = {"name": name, "n": len(fo) - 1, "first_out": fo, "head": hd, "triangles": totals[name],
                 "source": f"examples/{name}.metis, examples/examples.yaml"}
        stem = os.path.join(ex, name)
        if os.path.exists(stem + ".first_out"):
            bfo, bhd = read_binary(stem)
            entry["binary_first_out"] = bfo
            entry["binary_head"] = bhd
        graphs.append(entry)
    with open(os.path.join(HERE, "examples.json"), "w") as f:
        json.dump({"graphs": graphs, "missing": {"com-amazon": totals.get("com-amazon")}}, f, indent=1)

    triples = parse_intersection_triples(os.path.join(ref, "tests", "intersection_test.cpp"))
    assert len(triples) == 10, len(triples)
    with open(os.path.join(HERE, "intersection_kat.json"), "w") as f:
        json.dump({"source": "tests/intersection_test.cpp:41-50", "triples": triples}, f, indent=1)
    print(f"wrote {len(graphs)} graphs and {len(triples)} intersection triples")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/katric")
    main(sys.argv[1])
