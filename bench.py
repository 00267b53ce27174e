"""Throughput of exact local triangle counting on one GB300 (and N replicas under torchrun).

Default workload: RMAT scale 24, edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05), seed 2,
symmetrised, deduplicated, self-loops removed (u32 ids, u64 offsets).  One step = one full
pass of the counting path on a device-resident undirected CSR: orientation by (degree, id),
out-list compaction, owner-side hash intersection, per-vertex counts and the u64 total.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload rmat24|rgg24|gnm14]
  python bench.py --impl reference ...   # the CPU restatement of the reference's path

Prints one JSON line (rank 0).  metric: undirected edges per second (value: device-resident
inputs; e2e: host buffers through the public API, copies inside the timed region).  At one GPU
the default run also measures the batched form (8192 graphs in one captured plan against the
plain per-graph loop) and the served form (a 60 s Poisson stream against the continuous-batching
server, then the same requests at saturation against the plain loop), and adds their numbers
to the same line under "batched" and "served".
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "rmat24": dict(kind="rmat", scale=24, edge_factor=16, seed=2),
    "rgg24": dict(kind="rgg2d", n=1 << 24, avg_degree=32.0, seed=3),
    "gnm14": dict(kind="gnm", n=1 << 14, m=1 << 17, seed=1),
    # smaller cases of the same generators (profiling captures, quick checks)
    "rmat20": dict(kind="rmat", scale=20, edge_factor=16, seed=2),
    "rmat22": dict(kind="rmat", scale=22, edge_factor=16, seed=2),
    "rgg20": dict(kind="rgg2d", n=1 << 20, avg_degree=32.0, seed=3),
    "rgg22": dict(kind="rgg2d", n=1 << 22, avg_degree=32.0, seed=3),
    # batched workload: many graphs, n log-uniform in [2^8, 2^17], degree U(4, 64),
    # G(n,m) / RMAT / RGG by index mod 3, graph i seeded with 4 + i
    "batch8192": dict(kind="batch", graphs=8192, log2_n=(8.0, 17.0), degree=(4.0, 64.0), seed=4),
    "batch1024": dict(kind="batch", graphs=1024, log2_n=(8.0, 17.0), degree=(4.0, 64.0), seed=4),
    # served workload: Poisson arrivals, edge counts lognormal(median 2^16, sigma 2) clipped to
    # [1e3, 5e7], the same generator mix, 30% repeats of a resident graph, 120 GB budget
    "serve": dict(kind="serve", rate=200.0, seconds=60.0, median_m=65536, sigma=2.0, m_clip=(1e3, 5e7),
                  repeat=0.3, budget=120 << 30, seed=5),
}
METRIC = "edges/s (undirected edges / time of one exact total + per-vertex count)"
L2_BYTES = 129 << 20  # GB300 L2: a CSR above this streams from HBM on every step
KERNELS_PER_STEP = 7  # k_prep, k_orient, k_desc, k_count_small, k_count_medium, k_count_large, k_final


def kernels_per_count(nnz: int) -> int:
    """Kernels of one AUTO count: the seven above, plus k_tile_hist / k_tile_scan /
    k_tile_scatter for the large and the medium tiles from 2^20 adjacency entries on."""
    return KERNELS_PER_STEP + (6 if nnz >= (1 << 20) else 0)


def make_graph(name: str):
    from katric_gb300 import Graph
    w = WORKLOADS[name]
    if w["kind"] == "rmat":
        return Graph.rmat(w["scale"], w["edge_factor"], 0.57, 0.19, 0.19, w["seed"])
    if w["kind"] == "rgg2d":
        return Graph.rgg2d(w["n"], w["avg_degree"], w["seed"])
    return Graph.gnm(w["n"], w["m"], w["seed"])


def make_graph_cpu(name: str):
    """The same graph through the generators built without CUDA (oracle/libgraphgen.so), for the
    CPU arm: (first_out u64, head u32)."""
    from oracle import graphgen
    w = WORKLOADS[name]
    if w["kind"] == "rmat":
        return graphgen.rmat(w["scale"], w["edge_factor"], 0.57, 0.19, 0.19, w["seed"])
    if w["kind"] == "rgg2d":
        return graphgen.rgg2d(w["n"], w["avg_degree"], w["seed"])
    return graphgen.gnm(w["n"], w["m"], w["seed"])


def csr_sha256(first_out, head) -> str:
    """SHA-256 of the CSR bytes (u64 first_out, then u32 head): both arms print it, so equal
    digests show that they counted the same graph."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(first_out, dtype=np.uint64).view(np.uint8).data)
    h.update(np.ascontiguousarray(head, dtype=np.uint32).view(np.uint8).data)
    return h.hexdigest()


def workload_config(name: str, n: int, nnz: int, sha: str) -> dict:
    """The config dict both arms print (identical for the same workload and graph)."""
    w = dict(WORKLOADS[name])
    cfg = {"workload": name, "n": n, "m_undirected": nnz // 2, "nnz": nnz}
    cfg.update({k: v for k, v in w.items() if k != "kind"})
    cfg["generator"] = w["kind"]
    if w["kind"] == "rmat":
        cfg["abcd"] = [0.57, 0.19, 0.19, 0.05]
    cfg["csr_sha256"] = sha
    csr_bytes = 8 * (n + 1) + 4 * nnz
    if csr_bytes > L2_BYTES:
        cfg["l2"] = "inputs larger than L2 (CSR %.2f GB vs 129 MB L2)" % (csr_bytes / 1e9)
    else:
        cfg["l2"] = ("inputs smaller than L2 (CSR %.1f MB vs 129 MB L2), not flushed between steps: "
                     "a launch-bound check case, not a bandwidth figure" % (csr_bytes / 1e6))
    return cfg


def fixture(name: str) -> dict | None:
    """The oracle's full-size record of a workload (tests/golden/fullsize.json), if any."""
    p = os.path.join(ROOT, "tests", "golden", "fullsize.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f).get(name)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        # a region shorter than nvidia-smi's start-up and sampling interval got no sample: take the
        # first one, right after the region
        after = not self.lines
        t0 = time.perf_counter()
        while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 2.0:
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
               "reasons": sorted(reasons), "samples": len(sm)}
        if after:
            out["note"] = "timed region shorter than the sampling interval: sampled right after it"
        return out


def measured_traffic(workload: str):
    """DRAM bytes (read + write) of the intersection-phase kernels of one count, from the ncu
    capture summarised in profiles/dram_traffic.txt (None when that workload was not captured)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if parts and not line.startswith("#") and parts[0] == workload:
                return float(parts[1])
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def max_over_ranks(x: float, device) -> float:
    """The largest x over all ranks (a replicated job takes as long as its slowest rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(m: int, ms: float, ws: int) -> float:
    """Whole-job edges/s of ws replicas that each count an m-edge graph in ms (the max over ranks)."""
    return ws * m / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_baseline_sample(first_out, head, target_s: float = 12.0, slices: int = 20, threads: int | None = None) -> dict:
    """The oracle (CPU restatement of the reference path, merge strategy) on all host cores, on
    a bounded sample: pieces of a full count (a hash slice of the vertices each: their lists
    oriented and id-sorted, then the node-parallel local phase over them as tails), timed
    until about target_s seconds of CPU work; value = the pieces' edges / their time."""
    from oracle import oracle as O
    threads = threads or (os.cpu_count() or 1)
    sc = O.SlicedCount(first_out, head, slices, num_threads=threads)
    adj, secs, k = 0, 0.0, 0
    while k < slices and (k == 0 or secs < target_s):
        t0 = time.perf_counter()
        _, a, _ = sc.run(k)
        secs += time.perf_counter() - t0
        adj += a
        k += 1
    return {"value": (adj / 2) / secs, "unit": "edges/s", "cores": threads, "kind": "port",
            "sample": (f"oracle (C/OpenMP restatement of run_shmem, merge) on the same graph: {k} of {slices} hash "
                       f"slices of the vertices, each timed as orientation + id sort of its lists and the local "
                       f"phase over its tail vertices; {adj // 2} of {len(head) // 2} edges in {secs:.2f} s")}


def run_reference_arm(args):
    """The reference's CPU path, restated (the oracle, merge strategy as in run_shmem's default),
    on all host cores.  The timed steps together are exactly one full count: step i orients and
    sorts the lists of hash slice i of the vertices and runs the local phase over its tail
    vertices, for slices = steps, so the K timed steps cover every vertex once.  The input is
    built by the generators compiled without CUDA (oracle/libgraphgen.so)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    fo, hd = make_graph_cpu(args.workload)
    n, nnz = len(fo) - 1, len(hd)
    cfg = workload_config(args.workload, n, nnz, csr_sha256(fo, hd))
    threads = os.cpu_count() or 1
    slices = args.ref_slices or args.steps
    t0 = time.perf_counter()
    sc = O.SlicedCount(fo, hd, slices, num_threads=threads)
    setup_s = time.perf_counter() - t0
    times, adj, tri = [], 0, 0
    for i in range(args.warmup + args.steps):
        j = i - args.warmup
        s = j % slices  # warm-up steps run the last slices, the timed ones 0, 1, ...
        t0 = time.perf_counter()
        t, a, _ = sc.run(s)
        dt = time.perf_counter() - t0
        if j >= 0:
            times.append(dt)
            adj += a
            tri += t
    full = args.steps % slices == 0
    secs = sum(times)
    v = (adj / 2) / secs
    fx = fixture(args.workload)
    line = {"metric": METRIC, "value": v, "unit": "edges/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs * 1e3 / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator, no dataset)",
            "impl": "reference", "config": cfg,
            "count_s": secs * slices / args.steps,
            "step_s": {"min": min(times), "median": statistics.median(times), "max": max(times)},
            "cpu_baseline": {"value": v, "unit": "edges/s", "cores": threads, "kind": "port",
                             "sample": (f"full count timed in {args.steps} pieces ({slices} hash slices of the "
                                        f"vertices: orientation + id sort of each slice's lists, then the local "
                                        f"phase over its tail vertices){'' if full else '; partial coverage'}; "
                                        f"whole-graph preprocessing before the steps, untimed: {setup_s:.2f} s")},
            "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (C++17, TBB/MPI/Boost/sparsehash, un-vendored graph-io) cannot be built here; "
                    "this is the oracle restatement of its path (merge intersection) on all host cores"}
    if full:
        line["triangles"] = tri * slices // args.steps
        if fx and "total" in fx:
            line["triangles_match_oracle_fixture"] = line["triangles"] == fx["total"]
    print(json.dumps(line), flush=True)


def tune_cache_path() -> str:
    """Persisted autotuner choices: $KTRI_TUNE_CACHE, else ~/.cache/katric_gb300/tune.jsonl."""
    path = os.environ.get("KTRI_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "katric_gb300",
                                                              "tune.jsonl")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    return path


def run_batch(args, steps: int, warmup: int, plain_passes: int = 3) -> dict:
    """Batched workload: one captured plan (CUDA graph) over the packed union of all graphs,
    against the plain loop of one device entry-point call per graph (median of plain_passes
    passes), both timed here.  The per-graph totals are compared with the oracle's record of
    this batch when tests/golden/fullsize.json holds one."""
    import hashlib
    import torch
    from katric_gb300 import Batch, TriangleCounter
    name = args.workload if WORKLOADS[args.workload]["kind"] == "batch" else "batch8192"
    w = WORKLOADS[name]
    t0 = time.perf_counter()
    b = Batch.generate(w["graphs"], w["log2_n"][0], w["log2_n"][1], w["degree"][0], w["degree"][1], w["seed"])
    gen_s = time.perf_counter() - t0
    n, nnz, k = b.union.n, b.union.nnz, b.num_graphs
    ctr = TriangleCounter(0)
    dev = torch.device("cuda:0")
    fo = torch.from_numpy(b.union.first_out.view(np.int64)).to(dev)
    hd = torch.from_numpy(b.union.head.view(np.int32)).to(dev)
    gf = torch.from_numpy(b.graph_first.view(np.int64)).to(dev)
    tot = torch.zeros(k, dtype=torch.int64, device=dev)
    pv = torch.zeros(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    # bins, segment and strategy from the autotuner, tuned on a prefix of the batch (a quarter of
    # the graphs: on an eighth the owner bins 32 and 48 came within timing noise of each other,
    # while on the whole union 48 is 15 % faster) and persisted; later runs of the same shape
    # class read the choice back
    ks = max(1, min(k, k // 4))
    ns = int(b.graph_first[ks])
    t0 = time.perf_counter()
    conf, tune = ctr.autotune(fo.data_ptr(), hd.data_ptr(), ns, int(b.union.first_out[ns]), gf.data_ptr(), ks,
                              cache_path=tune_cache_path(), stream=stream.cuda_stream)
    tune.update({"sample_graphs": ks, "tune_s": round(time.perf_counter() - t0, 2),
                 "chosen": {"intersection_method": conf.intersection_method, "small_outdegree": conf.small_outdegree,
                            "medium_outdegree": conf.medium_outdegree, "segment": conf.segment,
                            "tile_order": conf.tile_order}})
    plan = ctr.plan_batch(fo.data_ptr(), hd.data_ptr(), n, nnz, gf.data_ptr(), k, tot.data_ptr(), pv.data_ptr(),
                          conf)
    for _ in range(warmup):
        plan.launch(stream.cuda_stream)
    plan.check()
    ref_tot = tot.clone()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        plan.launch(stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    clk = clocks.stop()
    plan.check()
    assert torch.equal(tot, ref_tot)
    totals = ref_tot.cpu().numpy().astype("<u8")
    fx = fixture(name)
    pinned = None
    if fx and fx.get("graphs") == k:
        pinned = (hashlib.sha256(totals.view(np.uint8).data).hexdigest() == fx["totals_sha256"] and
                  hashlib.sha256(pv.cpu().numpy().astype("<u8").view(np.uint8).data).hexdigest() ==
                  fx["per_vertex_sha256"])
    # plain loop: one ktri_count_csr_device call per graph on per-graph device CSRs
    gfo = b.graph_first.astype(np.int64)
    ufo = b.union.first_out.astype(np.int64)
    per = []
    for g in range(k):
        a, e = gfo[g], gfo[g + 1]
        f = fo[a:e + 1] - int(ufo[a])
        h = (hd[int(ufo[a]):int(ufo[e])] - int(a)).to(torch.int32)
        per.append((f.contiguous(), h.contiguous(), int(e - a), int(ufo[e] - ufo[a])))
    out_t = torch.zeros(k, dtype=torch.int64, device=dev)
    out_pv = torch.zeros(int(max(p[2] for p in per)) + 1, dtype=torch.int64, device=dev)

    def plain_pass():
        for g, (f, h, gn, gnnz) in enumerate(per):
            ctr.count_device(f.data_ptr(), h.data_ptr(), gn, gnnz, out_t[g:g + 1].data_ptr(), out_pv.data_ptr(), conf,
                             stream=stream.cuda_stream)

    plain_pass()  # warm-up (grows the workspace to the largest graph)
    ctr.check()
    assert torch.equal(out_t, ref_tot), "plain loop and batch disagree"
    plain = []
    for _ in range(plain_passes):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        plain_pass()
        ctr.check()
        plain.append((time.perf_counter() - t1) * 1e3)
    plain_ms = statistics.median(plain)
    del per, fo, hd, pv
    plan.close()
    ctr.close()
    return {
        "workload": name, "graphs": k, "n_total": n, "m_total": b.union.m, "seed": w["seed"],
        "generation_s": round(gen_s, 1),
        "path": "one captured plan (CUDA graph) over the packed union, device-resident inputs",
        "ms_per_batch": ms, "steps": steps, "warmup": warmup,
        "graphs_per_s": k / (ms / 1e3), "edges_per_s": b.union.m / (ms / 1e3),
        "plain_loop": {"ms_median": plain_ms, "ms_passes": plain, "graphs_per_s": k / (plain_ms / 1e3),
                       "path": "ktri_count_csr_device per graph, one stream, device-resident inputs"},
        "batched_vs_plain": plain_ms / ms,
        "autotune": tune,
        "triangles_total": int(totals.sum()),
        "totals_match_oracle_fixture": pinned,
        "gpu_launches": (kernels_per_count(nnz) + 1) * steps,  # the pipeline + k_graph_totals per replay
        "clocks": clk,
    }


def serve_requests(w, seconds, rate):
    """The request stream: arrival times, and per request either a new graph spec or a repeat."""
    rng = np.random.default_rng(w["seed"])
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        arrivals.append(t)
    reqs, specs = [], []
    for i in range(len(arrivals)):
        if specs and rng.random() < w["repeat"]:
            reqs.append(("repeat", int(rng.integers(len(specs)))))
            continue
        m = float(np.clip(np.exp(np.log(w["median_m"]) + w["sigma"] * rng.standard_normal()), *w["m_clip"]))
        d = float(rng.uniform(4.0, 64.0))
        n = max(8, int(round(2 * m / d)))
        specs.append((len(specs) % 3, n, d, 1000 + len(specs)))
        reqs.append(("new", len(specs) - 1))
    return arrivals, reqs, specs


def run_serve(args, passes: int = 3) -> dict:
    """Served workload: Poisson arrivals replayed against the continuous-batching server (p50/p99
    latency, achieved graphs/s); then the same request list at saturation against the server
    and against the plain loop (one synchronous ktri_count_csr_ctx call per request), each
    `passes` times (medians reported)."""
    from katric_gb300 import Config, Server, TriangleCounter
    from katric_gb300.graph import generate_many
    w = WORKLOADS["serve"]
    seconds = args.serve_seconds or w["seconds"]
    arrivals, reqs, specs = serve_requests(w, seconds, w["rate"])
    t0 = time.perf_counter()
    graphs = generate_many([s[0] for s in specs], [s[1] for s in specs], [s[2] for s in specs],
                           [s[3] for s in specs])
    gen_s = time.perf_counter() - t0
    req_graph = [graphs[j] for _, j in reqs]
    m_total = sum(g.m for g in req_graph)

    def replay(srv, paced):
        lat = [0.0] * len(reqs)
        rids = [0] * len(reqs)
        done = threading.Event()

        def submitter():
            start = time.perf_counter()
            for i, (kind, j) in enumerate(reqs):
                if paced:
                    delay = arrivals[i] - (time.perf_counter() - start)
                    if delay > 0:
                        time.sleep(delay)
                # a repeat of a graph that was already submitted goes by key (resident graphs are
                # answered from their counts; others are counted again from the CSR)
                rids[i] = srv.submit(graphs[j], key=1 + j, borrow=True)
            done.set()

        th = threading.Thread(target=submitter)
        start = time.perf_counter()
        th.start()
        for i in range(len(reqs)):
            while rids[i] == 0:
                time.sleep(0.0002)
            _, _, lat[i] = srv.wait(rids[i])
        th.join()
        return time.perf_counter() - start, lat

    with Server(memory_budget=w["budget"], direct_host_access=args.serve_direct) as srv:
        wall, lat = replay(srv, paced=True)
        st = srv.stats()
    sat_walls, sat_st = [], None
    for _ in range(passes):
        with Server(memory_budget=w["budget"], direct_host_access=args.serve_direct) as srv:
            sw, _ = replay(srv, paced=False)
            sat_walls.append(sw)
            sat_st = srv.stats()
    ctr = TriangleCounter(0)
    for g in req_graph[:3]:
        ctr.count(g.first_out, g.head, per_vertex=True)  # warm-up
    plain_walls = []
    for _ in range(passes):
        t1 = time.perf_counter()
        for g in req_graph:
            ctr.count(g.first_out, g.head, Config(), per_vertex=True)
        plain_walls.append(time.perf_counter() - t1)
    ctr.close()
    sat_wall, plain_wall = statistics.median(sat_walls), statistics.median(plain_walls)
    lat_ms = np.array(lat) * 1e3
    k = len(reqs)
    return {
        "workload": "serve", "rate_per_s": w["rate"], "seconds": seconds, "requests": k,
        "host_copies": "device reads host memory where it can" if args.serve_direct else "pinned staging",
        "distinct_graphs": len(specs), "m_total": m_total, "median_m": w["median_m"], "sigma": w["sigma"],
        "repeat": w["repeat"], "memory_budget": w["budget"], "generation_s": round(gen_s, 1),
        "paced": {"graphs_per_s": k / wall, "wall_s": wall},
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "mean": float(lat_ms.mean()), "max": float(lat_ms.max())},
        "server": st,
        "saturation": {"graphs_per_s": k / sat_wall, "edges_per_s": m_total / sat_wall, "wall_s_passes": sat_walls,
                       "server": sat_st},
        "plain_loop": {"graphs_per_s": k / plain_wall, "edges_per_s": m_total / plain_wall,
                       "wall_s_passes": plain_walls,
                       "path": "ktri_count_csr_ctx per request (host buffers, synchronous, no resident graphs)"},
        "served_vs_plain_at_saturation": plain_wall / sat_wall,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="rmat24", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-slices", type=int, default=0,
                    help="reference arm: hash slices of a count (default: --steps, so the timed steps are one count)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched and served measurements of the default run")
    ap.add_argument("--serve-seconds", type=float, default=0.0, help="duration of the served stream (default 60)")
    ap.add_argument("--serve-direct", action="store_true",
                    help="let the GPU read and write the requests' host memory directly where it can")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
        return
    kind = WORKLOADS[args.workload]["kind"]
    if kind in ("batch", "serve"):
        # the batched and served forms measure one GPU; under torchrun rank 0 runs them
        if dist_env()[1] != 0:
            return
        if kind == "batch":
            r = run_batch(args, args.steps, args.warmup)
            head = {"metric": METRIC + "; batched workload", "value": r["edges_per_s"], "unit": "edges/s",
                    "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_batch"],
                    "gpu_launches": r["gpu_launches"], "clocks": r["clocks"]}
        else:
            r = run_serve(args)
            head = {"metric": "served graphs/s and p50/p99 latency (exact total + per-vertex counts per request)",
                    "value": r["paced"]["graphs_per_s"], "unit": "graphs/s", "n_gpus": 1, "steps": r["requests"],
                    "warmup": 0, "ms_per_step": r["paced"]["wall_s"] * 1e3 / r["requests"]}
        head.update({"higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                     "data": "synthetic (seeded generators)", "config": {"workload": args.workload}})
        head.update({k: v for k, v in r.items() if k not in head})
        print(json.dumps(head), flush=True)
        return

    import torch
    import katric_gb300
    from katric_gb300 import Config, TriangleCounter

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)

    g = make_graph(args.workload)
    csr_sha = csr_sha256(g.first_out, g.head)
    ctr = TriangleCounter(dev)
    fo_d = torch.from_numpy(g.first_out.view(np.int64)).to(f"cuda:{dev}")
    hd_d = torch.from_numpy(g.head.view(np.int32)).to(f"cuda:{dev}")
    tot_d = torch.zeros(1, dtype=torch.int64, device=f"cuda:{dev}")
    pv_d = torch.zeros(g.n, dtype=torch.int64, device=f"cuda:{dev}")
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    # work counters for the roofline (outside the timed region)
    ctr.count_device(fo_d.data_ptr(), hd_d.data_ptr(), g.n, g.nnz, tot_d.data_ptr(), pv_d.data_ptr(),
                     Config(collect_stats=True), stream=sptr)
    ctr.check()
    st0 = ctr.stats()
    wedge_checks, m_oriented, streamed = int(st0.wedge_checks), int(st0.oriented_edges), int(st0.streamed_entries)
    total_ref = int(tot_d.item())
    pv_ref = pv_d.clone()

    cfg = Config()

    def step():
        ctr.count_device(fo_d.data_ptr(), hd_d.data_ptr(), g.n, g.nnz, tot_d.data_ptr(), pv_d.data_ptr(), cfg,
                         stream=sptr)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = ClockSampler(dev)
    clocks.start()
    barrier()
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    small_ms, large_ms, count_ms, orient_ms = [], [], [], []
    for _ in range(args.steps):
        step()
        st = ctr.stats()  # per-kernel CUDA events recorded by the library on this stream
        small_ms.append(st.ms_count_small)
        large_ms.append(st.ms_count_large)
        count_ms.append(st.ms_count)
        orient_ms.append(st.ms_orient)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    ctr.check()
    assert int(tot_d.item()) == total_ref and torch.equal(pv_d, pv_ref), "result changed between steps"

    ms = max_over_ranks(ms, f"cuda:{dev}")
    value = replica_value(g.m, ms, ws)

    # e2e through the public host-buffer API, pinned host memory, copies inside the region
    fo_h = torch.from_numpy(g.first_out.view(np.int64)).pin_memory()
    hd_h = torch.from_numpy(g.head.view(np.int32)).pin_memory()
    pv_h = torch.zeros(g.n, dtype=torch.int64).pin_memory()
    tot = ctypes.c_uint64(0)
    L = katric_gb300.load()
    opts = cfg.opts()

    def e2e_step():
        rc = L.ktri_count_csr_ctx(ctr.handle, fo_h.data_ptr(), hd_h.data_ptr(), g.n, g.nnz, ctypes.byref(tot),
                                  pv_h.data_ptr(), ctypes.byref(opts))
        if rc:
            raise katric_gb300.KtriError(rc, L.ktri_last_error(ctr.handle).decode())

    for _ in range(3):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 20))
    barrier()
    split = {"h2d": [], "d2h": [], "call": [], "orient": [], "count": [], "host_enqueue": [], "host_call": []}
    walls = []
    gc.disable()  # no collector pause inside the timed region
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        e2e_step()
        walls.append((time.perf_counter() - ts) * 1e3)
        st = ctr.stats()  # device-side split of the call (the library's events)
        split["h2d"].append(st.ms_h2d)
        split["d2h"].append(st.ms_d2h)
        split["call"].append(st.ms_call)
        split["orient"].append(st.ms_orient)
        split["count"].append(st.ms_count)
        split["host_enqueue"].append(st.host_ms_enqueue)
        split["host_call"].append(st.host_ms_call)
    t1 = time.perf_counter()
    gc.enable()
    barrier()
    e2e_ms = (t1 - t0) * 1e3 / e2e_steps
    assert tot.value == total_ref
    e2e_ms = max_over_ranks(e2e_ms, f"cuda:{dev}")
    e2e_value = replica_value(g.m, e2e_ms, ws)

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    hbm_peak, peak_kind = peaks()
    # algorithmic bytes (per step), from the reference's own work counter wedge_checks
    n, m = g.n, g.m
    b_orient = (8 * (n + 1) + 4 * 2 * m) + (8 * (n + 1) + 4 * m)
    b_int = 4 * (wedge_checks + m)
    b_out = 8 * n + 8
    b_total = b_orient + b_int + b_out
    k_ms = statistics.mean(c for c in count_ms)
    achieved = b_int / (k_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator, no dataset)",
        "config": workload_config(args.workload, n, g.nnz, csr_sha),
        "parallelism": f"replicas x{ws}",
        "triangles": total_ref,
        "hbm_gbs_algorithmic": b_total / (ms / 1e3) / 1e9,
        "phases_ms": {"orient": statistics.mean(orient_ms), "count_small": statistics.mean(small_ms),
                      "count_medium_large": statistics.mean(large_ms), "count_total": k_ms},
        "work": {"wedge_checks": wedge_checks, "oriented_edges": m_oriented, "streamed_entries": streamed},
        "roofline": {"bound": "hbm",
                     "kernel": "intersection phase (k_count_small + k_count_medium + k_count_large + k_final)",
                     "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "algorithmic_bytes": b_int, "traffic": measured_traffic(args.workload),
                     "traffic_source": "profiles/dram_traffic.txt (ncu dram__bytes_read.sum + "
                                       "dram__bytes_write.sum of the three counting kernels, captured at "
                                       "RMAT-22 / RGG-22 and scaled by streamed entries; the RMAT-24 "
                                       "figure is a lower bound, L2 reuse falls with size)"},
        "e2e": {"value": e2e_value, "unit": "edges/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(8 * (n + 1) + 4 * g.nnz), "d2h_bytes_per_step": int(8 * n + 8),
                "call_wall_ms": {"min": min(walls), "median": statistics.median(walls), "max": max(walls),
                                 "each": [round(x, 2) for x in walls],
                                 "host_call_each": [round(x, 2) for x in split["host_call"]]},
                "split_ms": {k: statistics.median(v) for k, v in split.items()},
                "split_note": "device time inside ktri_count_csr_ctx (library events): h2d = first input copy to "
                              "last piece of head landed (orientation runs on the pieces already in), orient = "
                              "orientation phase incl. waiting for pieces, count = intersection phase, d2h = "
                              "read-back of total + per-vertex counts, call = all of it; host_enqueue / host_call = host time "
                              "until everything was enqueued / of the whole call"},
        "gpu_launches": kernels_per_count(g.nnz) * args.steps,
        "clocks": clk,
    }
    fx = fixture(args.workload)
    if fx and fx.get("csr_sha256") == csr_sha:
        # the oracle's full count of this same graph (tests/golden/fullsize.json)
        line["triangles_match_oracle_fixture"] = total_ref == fx["total"]
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"] = cpu_baseline_sample(g.first_out, g.head)
    if ws == 1 and not args.no_forms and args.workload == "rmat24":
        # the batched and served forms of the same metric family, on the same GPU
        del fo_h, hd_h, pv_h, fo_d, hd_d, pv_d, pv_ref
        ctr.close()
        torch.cuda.empty_cache()
        line["batched"] = run_batch(args, args.steps, args.warmup)
        torch.cuda.empty_cache()
        line["served"] = run_serve(args)
        line["batched_vs_plain"] = line["batched"]["batched_vs_plain"]
        line["served_vs_plain_at_saturation"] = line["served"]["served_vs_plain_at_saturation"]
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
