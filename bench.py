"""Throughput of exact local triangle counting on one GB300 (and N replicas under torchrun).

Default workload: RMAT scale 24, edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05), seed 2,
symmetrised, deduplicated, self-loops removed (u32 ids, u64 offsets).  One step = one full
pass of the counting path on a device-resident undirected CSR: orientation by (degree, id),
out-list compaction, owner-side hash intersection, per-vertex counts and the u64 total.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload rmat24|rgg24|gnm14]
  python bench.py --impl reference ...   # the CPU restatement of the reference's path

Prints one JSON line (rank 0).  metric: undirected edges per second (value: device-resident
inputs; e2e: host buffers through the public API, copies inside the timed region).
"""
from __future__ import annotations

import argparse
import ctypes
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


def workload_config(name: str, g) -> dict:
    w = dict(WORKLOADS[name])
    cfg = {"workload": name, "n": g.n, "m_undirected": g.m, "nnz": g.nnz}
    cfg.update({k: v for k, v in w.items() if k != "kind"})
    cfg["generator"] = w["kind"]
    if w["kind"] == "rmat":
        cfg["abcd"] = [0.57, 0.19, 0.19, 0.05]
    return cfg


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


def cpu_baseline_sample(g, target_s: float = 15.0, threads: int | None = None) -> dict:
    """The oracle (CPU restatement of the reference path) on all host cores, on a bounded
    sample: full preprocessing, local phase over a 1/stride sample of tail vertices."""
    from oracle import oracle as O
    threads = threads or (os.cpu_count() or 1)
    stride = 1
    probe_stride = 4096
    _, st = O.count_sampled(g.first_out, g.head, probe_stride, num_threads=threads)
    est_full = st["local_phase_s"] * probe_stride
    if est_full > target_s:
        stride = int(min(probe_stride, max(1, round(est_full / target_s))))
    _, st = O.count_sampled(g.first_out, g.head, stride, num_threads=threads)
    pre = st["orientation_s"] + st["sorting_s"]
    local_est = st["local_phase_s"] * stride
    t = pre + local_est
    return {"value": g.m / t, "unit": "edges/s", "cores": threads, "kind": "port",
            "sample": (f"oracle (C/OpenMP restatement of run_shmem) on the same graph: full orientation+sort "
                       f"({pre:.2f} s), merge local phase over a 1/{stride} hash sample of tail vertices "
                       f"({st['local_phase_s']:.2f} s, scaled x{stride}); estimated full time {t:.2f} s"),
            "est_seconds": t}


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    g = make_graph(args.workload)
    threads = os.cpu_count() or 1
    times = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline_sample(g, target_s=args.ref_step_seconds, threads=threads)
        if i >= args.warmup:
            times.append(cb["est_seconds"])
    t = statistics.median(times)
    v = g.m / t
    line = {"metric": METRIC, "value": v, "unit": "edges/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator)", "impl": "reference",
            "config": workload_config(args.workload, g),
            "cpu_baseline": {"value": v, "unit": "edges/s", "cores": threads, "kind": "port",
                             "sample": cb["sample"]},
            "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (C++17, TBB/MPI/Boost/sparsehash, un-vendored graph-io) cannot be built here; "
                    "this is the oracle restatement of its path on all host cores"}
    print(json.dumps(line), flush=True)


def tune_cache_path() -> str:
    """Persisted autotuner choices: $KTRI_TUNE_CACHE, else ~/.cache/katric_gb300/tune.jsonl."""
    path = os.environ.get("KTRI_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "katric_gb300",
                                                              "tune.jsonl")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    return path


def run_batch(args):
    """Batched workload: one captured plan (CUDA graph) over the packed union of all graphs,
    against the plain loop of one device entry-point call per graph, both timed here."""
    import torch
    from katric_gb300 import Batch, Config, TriangleCounter
    w = WORKLOADS[args.workload]
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
    # bins, segment and strategy from the autotuner, tuned on a prefix of the batch (about an
    # eighth of the graphs) and persisted; later runs of the same shape class read the choice back
    ks = max(1, min(k, k // 8))
    ns = int(b.graph_first[ks])
    t0 = time.perf_counter()
    conf, tune = ctr.autotune(fo.data_ptr(), hd.data_ptr(), ns, int(b.union.first_out[ns]), gf.data_ptr(), ks,
                              cache_path=tune_cache_path(), stream=stream.cuda_stream)
    tune.update({"sample_graphs": ks, "tune_s": round(time.perf_counter() - t0, 2),
                 "chosen": {"intersection_method": conf.intersection_method, "small_outdegree": conf.small_outdegree,
                            "medium_outdegree": conf.medium_outdegree, "segment": conf.segment}})
    plan = ctr.plan_batch(fo.data_ptr(), hd.data_ptr(), n, nnz, gf.data_ptr(), k, tot.data_ptr(), pv.data_ptr(),
                          conf)
    for _ in range(args.warmup):
        plan.launch(stream.cuda_stream)
    plan.check()
    ref_tot = tot.clone()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        plan.launch(stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    plan.check()
    assert torch.equal(tot, ref_tot)
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
    cfg = conf

    def plain_pass():
        for g, (f, h, gn, gnnz) in enumerate(per):
            ctr.count_device(f.data_ptr(), h.data_ptr(), gn, gnnz, out_t[g:g + 1].data_ptr(), out_pv.data_ptr(), cfg,
                             stream=stream.cuda_stream)

    plain_pass()  # warm-up (grows the workspace to the largest graph)
    ctr.check()
    assert torch.equal(out_t, ref_tot), "plain loop and batch disagree"
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    plain_pass()
    ctr.check()
    plain_ms = (time.perf_counter() - t1) * 1e3
    line = {
        "metric": METRIC + "; batched workload", "value": b.union.m / (ms / 1e3), "unit": "edges/s",
        "graphs_per_s": k / (ms / 1e3), "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded generators)",
        "config": {"workload": args.workload, "graphs": k, "n_total": n, "m_total": b.union.m, "seed": w["seed"],
                   "log2_n": list(w["log2_n"]), "degree": list(w["degree"]), "generation_s": round(gen_s, 2),
                   "path": "one captured plan (CUDA graph) over the packed union"},
        "plain_loop": {"ms": plain_ms, "graphs_per_s": k / (plain_ms / 1e3), "edges_per_s": b.union.m / (plain_ms / 1e3),
                       "path": "ktri_count_csr_device per graph, one stream, device-resident inputs"},
        "batched_vs_plain": plain_ms / ms,
        "autotune": tune,
        "triangles_total": int(ref_tot.sum().item()),
        "gpu_launches": (kernels_per_count(nnz) + 1) * args.steps,  # the pipeline + k_graph_totals per replay
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


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


def run_serve(args):
    """Served workload: Poisson arrivals replayed against the continuous-batching server (p50/p99
    latency, achieved graphs/s); then the same request list at saturation against the server
    and against the plain loop (one synchronous ktri_count_csr_ctx call per request)."""
    import threading
    import katric_gb300
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
    with Server(memory_budget=w["budget"], direct_host_access=args.serve_direct) as srv:
        sat_wall, _ = replay(srv, paced=False)
        sat_st = srv.stats()
    ctr = TriangleCounter(0)
    for g in req_graph[:3]:
        ctr.count(g.first_out, g.head, per_vertex=True)  # warm-up
    t1 = time.perf_counter()
    for g in req_graph:
        ctr.count(g.first_out, g.head, Config(), per_vertex=True)
    plain_wall = time.perf_counter() - t1
    lat_ms = np.array(lat) * 1e3
    k = len(reqs)
    line = {
        "metric": "served graphs/s and p50/p99 latency (exact total + per-vertex counts per request)",
        "value": k / wall, "unit": "graphs/s", "n_gpus": 1, "steps": k, "warmup": 0,
        "ms_per_step": wall * 1e3 / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded generators)",
        "config": {"workload": "serve", "rate_per_s": w["rate"], "seconds": seconds, "requests": k,
                   "host_copies": "device reads host memory where it can" if args.serve_direct else "pinned staging",
                   "distinct_graphs": len(specs), "m_total": m_total, "median_m": w["median_m"], "sigma": w["sigma"],
                   "repeat": w["repeat"], "memory_budget": w["budget"], "generation_s": round(gen_s, 1)},
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "mean": float(lat_ms.mean()), "max": float(lat_ms.max())},
        "server": st,
        "saturation": {"graphs_per_s": k / sat_wall, "edges_per_s": m_total / sat_wall, "server": sat_st},
        "plain_loop": {"graphs_per_s": k / plain_wall, "edges_per_s": m_total / plain_wall,
                       "path": "ktri_count_csr_ctx per request (host buffers, synchronous, no resident graphs)"},
        "served_vs_plain_at_saturation": plain_wall / sat_wall,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="rmat24", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--serve-seconds", type=float, default=0.0, help="duration of the served stream (default 60)")
    ap.add_argument("--serve-direct", action="store_true",
                    help="let the GPU read and write the requests' host memory directly where it can")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if WORKLOADS[args.workload]["kind"] in ("batch", "serve"):
        # the batched and served forms measure one GPU; under torchrun rank 0 runs them
        if dist_env()[1] != 0:
            return
        (run_batch if WORKLOADS[args.workload]["kind"] == "batch" else run_serve)(args)
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

    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t1 = time.perf_counter()
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
        "config": dict(workload_config(args.workload, g), parallelism=f"replicas x{ws}",
                       l2="inputs larger than L2 (CSR %.2f GB vs 129 MB L2)" % ((8 * (n + 1) + 4 * g.nnz) / 1e9)),
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
                                       "dram__bytes_write.sum of the three counting kernels, one capture)"},
        "e2e": {"value": e2e_value, "unit": "edges/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(8 * (n + 1) + 4 * g.nnz), "d2h_bytes_per_step": int(8 * n + 8)},
        "gpu_launches": kernels_per_count(g.nnz) * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu_baseline and ws == 1:
        cb = cpu_baseline_sample(g)
        cb.pop("est_seconds", None)
        line["cpu_baseline"] = cb
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
