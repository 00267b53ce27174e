"""bench.py on CPU: the reference arm prints one JSON line that keeps the bench contract (metric,
unit, cpu_baseline, a host-only e2e) and counts exactly the oracle's triangles on the graph whose
CSR digest it reports; the workload config labels the L2 regime by the graph's size."""
import json
import os
import subprocess
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _reference_line(workload: str, steps: int) -> dict:
    env = dict(os.environ)
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        env.pop(k, None)
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          workload, "--steps", str(steps), "--warmup", "1"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line_counts_the_oracle_total(oracle):
    import bench
    from oracle import graphgen
    line = _reference_line("gnm14", 4)
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "edges/s" and line["higher_is_better"] is True
    assert line["steps"] == 4 and line["warmup"] == 3  # warm-up raised to the minimum of three
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["unit"] == "edges/s"
    assert cb["cores"] >= 1 and "4 hash slices" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "edges/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    fo, hd = graphgen.gnm(1 << 14, 1 << 17, 1)
    total, _, _ = oracle.count(fo, hd, per_vertex=False)
    assert line["triangles"] == total
    cfg = line["config"]
    assert cfg["workload"] == "gnm14" and cfg["csr_sha256"] == bench.csr_sha256(fo, hd)
    assert cfg["n"] == len(fo) - 1 and cfg["nnz"] == len(hd) and cfg["m_undirected"] == len(hd) // 2


def test_partial_slice_coverage_reports_no_total(oracle, monkeypatch, capsys):
    """More hash slices than timed steps cover only part of the vertices: the line then claims
    no triangle total and says so in its sample."""
    import bench
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    bench.run_reference_arm(types.SimpleNamespace(workload="gnm14", steps=2, warmup=3, ref_slices=4))
    part = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert "triangles" not in part and "partial coverage" in part["cpu_baseline"]["sample"]
    assert part["value"] > 0


def test_l2_label_follows_the_csr_size():
    import bench
    small = bench.workload_config("gnm14", 1 << 14, 1 << 18, "x")
    assert small["l2"].startswith("inputs smaller than L2")
    big = bench.workload_config("rmat24", 1 << 24, 520766974, "x")
    assert big["l2"].startswith("inputs larger than L2")
    assert np.isclose(float(big["l2"].split("CSR ")[1].split(" GB")[0]), (8 * ((1 << 24) + 1) + 4 * 520766974) / 1e9,
                      atol=0.01)
