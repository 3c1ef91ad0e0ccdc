#!/usr/bin/env python
"""Benchmarks of the GB300 out-of-memory graph engine.

Default workload (`serving`, the headline metric "served queries/s + p50/p99
latency vs plain per-query path"): four resident weighted R-MAT graphs
(scales 22, 24, 26, 27; edge factor 16, a,b,c,d = .57/.19/.19/.05,
symmetrised, deduplicated, no self-loops, seeded vertex permutation (seed 1),
uint32 weights uniform in [1, 64] (seed 2)) under a 24 GiB device budget;
400 requests with Poisson arrivals at 2000/s (seed 4), 60 % BFS / 30 % SSSP /
10 % PageRank (5 iterations), graph chosen by Zipf(1.1).  One step = one
pass of the mix through og_server; `value` = served queries/s with results
left on the device, `e2e` = the same with every result read into page-locked
host memory; the plain per-query path and the CPU baseline are in the line.
The graphs are synthetic (no datasets offline).

--workload sssp-oom: one out-of-memory SSSP query per step on R-MAT 27 with
an 8 GiB budget, advisek 0.8, 32 seeded sources (seed 3).  Other workloads:
cc-oom, bfs-batch, bfs-resident, pr-precision (see run_* below).

--impl reference times the reference's CPU path on the host cores (the
oracle's restatement; the reference's GPU path needs a SYCL compiler this
image lacks), on graphs the oracle builds on the CPU: the engine is not
loaded.  The reference ships no CPU SSSP; its stand-in is a serial Dijkstra.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from onegraph_gb300 import replicas  # noqa: E402

GIB = 1 << 30


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=None,
                    help="default per workload: 27 (sssp-oom, bfs-batch), 26 (pr-precision), 20 (bfs-resident)")
    ap.add_argument("--budget-gib", type=float, default=None,
                    help="default per workload: 8 GiB, 6 GiB for pr-precision")
    ap.add_argument("--advisek", type=float, default=0.8)
    ap.add_argument("--sources", type=int, default=32)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="serving",
                    choices=["serving", "sssp-oom", "sssp-batch", "cc-oom", "bfs-batch", "bfs-resident",
                             "pr-precision", "replace"],
                    help="serving (default: the served-queries/s headline), or another measured configuration")
    ap.add_argument("--tune", type=int, default=1, help="bfs-batch: run the autotuner first")
    ap.add_argument("--serving-scales", default="22,24,26,27")
    ap.add_argument("--serving-budget-gib", type=float, default=24.0)
    ap.add_argument("--serving-slots", default=None,
                    help="serving: SSSP sources per multi-source pass for each graph (comma list, one per "
                         "--serving-scales entry); default per scale: 16 (22, 24), 8 (26), 4 (27)")
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--rate", type=float, default=2000.0)
    ap.add_argument("--serving-legs", default="all", choices=["all", "served"],
                    help="serving: 'served' runs only the warm-up and the timed passes (for launch lists)")
    ap.add_argument("--configs", default="all",
                    help="serving at N=1: after the serving measurement, run the other measured "
                         "configurations (resident BFS, out-of-memory SSSP and CC, PageRank precision, "
                         "batched BFS) each in its own process and embed their lines under 'configs' "
                         "('all', 'none', or a comma list of workload names)")
    ap.add_argument("--bfs-direction", default="auto", choices=["auto", "top-down"],
                    help="bfs-resident: direction of the timed plain queries (top-down: every level "
                         "from the frontier, the relax kernel on every edge)")
    ap.add_argument("--sssp-sources", type=int, default=8,
                    help="sssp-batch: sources per multi-source pass (1..32)")
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--delta", type=float, default=None,
                    help="SSSP near/far split width (default: the engine's, (wmin + wmax) / 16; "
                         "0: plain frontier relaxation as in the reference)")
    ap.add_argument("--direct", type=int, default=1,
                    help="1: relax the dynamic region straight from page-locked host memory "
                         "(fastest); 0: gather into double-buffered device staging first")
    a = ap.parse_args()
    if a.scale is None:
        a.scale = {"pr-precision": 26, "bfs-resident": 20}.get(a.workload, 27)
    if a.workload == "serving":
        a.steps = max(1, a.steps)
    if a.serving_slots:
        SERVING_SLOTS.update(zip((int(x) for x in a.serving_scales.split(",")),
                                 (int(x) for x in a.serving_slots.split(","))))
    if a.budget_gib is None:
        a.budget_gib = 6.0 if a.workload == "pr-precision" else 8.0
    return a


def dist_env():
    return replicas.rank_info()


def pick_sources(deg: np.ndarray, n: int, seed: int = 3) -> list[int]:
    rng = np.random.default_rng(seed)
    out, seen = [], set()
    while len(out) < n:
        for s in rng.integers(0, deg.size, 4 * n).tolist():
            if deg[s] > 0 and s not in seen:
                seen.add(s)
                out.append(int(s))
                if len(out) == n:
                    break
    return out


def make_graph(scale: int):
    import onegraph_gb300 as og
    t0 = time.time()
    try:
        g = og.Graph.rmat(scale, 16, seed=1, weight_seed=2, weighted=True, on_gpu=True)
    except og.OGError:
        g = og.Graph.rmat(scale, 16, seed=1, weight_seed=2, weighted=True)
    return g, time.time() - t0


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="og_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names[1:], f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


LINK_PEAKS: dict = {}


def h2d_peak_gbs() -> float:
    """Host-link ceiling for the rooflines: the highest of three probes over a
    2 GiB page-locked buffer (og_link_probe, best of 3 each): SM loads of the
    buffer (how the direct-mode kernels read host records), one DMA copy, and
    two DMA copies at once.  All three are kept in LINK_PEAKS."""
    import torch
    import onegraph_gb300 as og
    src = torch.empty(2 * GIB, dtype=torch.uint8, pin_memory=True)
    LINK_PEAKS.clear()
    for mode, name in ((0, "sm_read_gbs"), (1, "dma_copy_gbs"), (2, "dma_copy_2streams_gbs")):
        LINK_PEAKS[name] = og.link_probe(src, mode, 3)
    del src
    torch.cuda.empty_cache()
    return max(LINK_PEAKS.values())


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def reached_edges(deg: np.ndarray, dist: np.ndarray) -> int:
    return int(deg[dist != 0xFFFFFFFF].sum(dtype=np.int64))


def cpu_dijkstra_sample(g, srcs, deg, target_s, threads, per_query_edges):
    """Bounded serial Dijkstra runs (one per thread); returns queries/s
    extrapolated from edges scanned per second to each query's edge count."""
    import oracle
    V = g.V
    offp, edp = getattr(g, "_off_p", None) or g.off_p, getattr(g, "_edges_p", None) or g.edges_p

    def one(i, max_edges):
        s = srcs[i % len(srcs)]
        out = np.empty(V, np.uint32)
        t = time.perf_counter()
        scanned = oracle.sssp_dijkstra_bounded_raw(V, offp, edp, s, max_edges, out)
        return scanned, time.perf_counter() - t, s

    # calibrate the per-thread edge budget
    sc, dt, _ = one(0, 20_000_000)
    rate = sc / max(dt, 1e-6)
    max_edges = max(int(rate * target_s), 1)
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        t0 = time.perf_counter()
        res = list(ex.map(lambda i: one(i, max_edges), range(threads)))
        wall = time.perf_counter() - t0
    qps = 0.0
    for scanned, dt, s in res:
        qps += 1.0 / (dt * per_query_edges(s) / max(scanned, 1))
    return {"value": qps, "cores": threads, "wall_s": wall, "edges_per_thread": max_edges,
            "rate_edges_per_s_1core": rate}


def oracle_graph(scale: int):
    """The benchmark graph built on the CPU by the oracle (the reference arm
    must not load the engine); bit-identical to make_graph's."""
    import oracle
    t0 = time.time()
    g = oracle.RmatGraph(scale, 16, seed=1, weight_seed=2, weighted=True)
    return g, time.time() - t0


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores (the oracle's restatement
    of it; the reference's GPU path needs a SYCL compiler this image lacks),
    on this arm's workload and config.  Loads nothing from onegraph_gb300."""
    if rank != 0:
        return
    if args.workload == "serving":
        return run_reference_serving(args, world)
    g, gen_s = oracle_graph(args.scale)
    deg = g.degrees()
    srcs = pick_sources(deg, args.sources)
    threads = os.cpu_count() or 1
    E = g.E

    def per_query_edges(_s):
        return E  # symmetric R-MAT: the giant component holds essentially every edge

    samples = []
    for step in range(args.warmup + args.steps):
        r = cpu_dijkstra_sample(g, srcs[step % len(srcs):] + srcs, deg,
                                max(2.0, args.cpu_seconds / 3), threads, per_query_edges)
        if step >= args.warmup:
            samples.append(r)
    val = statistics.median(s["value"] for s in samples)
    wall = sum(s["wall_s"] for s in samples)
    line = {
        "impl": "reference", "metric": "queries/s", "value": val, "unit": "queries/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / len(samples) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config_dict(args, g),
        "cpu_baseline": {"value": val, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": "serial binary-heap Dijkstra (the reference ships no CPU SSSP), "
                                   "one bounded run per host thread, %d edges each, extrapolated "
                                   "to E=%d edges per query" % (samples[0]["edges_per_thread"], E)},
        "e2e": {"value": val, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": gen_s,
    }
    print(json.dumps(line), flush=True)


def run_reference_serving(args, world):
    scales = [int(x) for x in args.serving_scales.split(",")]
    graphs, gen_s = [], 0.0
    for sc in scales:
        g, t = oracle_graph(sc)
        graphs.append(g)
        gen_s += t
    n = args.requests
    arrivals, gsel, algos, srcs = serving_requests([g.degrees() for g in graphs], n, args.rate)
    views = [(g.V, g.E, g.off_p, g.edges_p) for g in graphs]
    threads = os.cpu_count() or 1
    target = max(1.0, args.cpu_seconds / 6)
    samples = []
    for step in range(args.warmup + args.steps):
        r = cpu_serving_estimate(views, gsel, algos, srcs, target, threads)
        if step >= args.warmup:
            samples.append(r)
    val = statistics.median(s["value"] for s in samples)
    wall = sum(s["wall_s"] for s in samples)
    line = {
        "impl": "reference", "metric": "served queries/s", "value": val, "unit": "queries/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / len(samples) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/f32", "data": "synthetic",
        "config": serving_config(args, scales, [(g.V, g.E) for g in graphs], algos),
        "cpu_baseline": {"value": val, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": "per step, one bounded sample (~%.1f s) of every (graph, algorithm) class of "
                                   "the %d-request mix, all classes at once on the host threads: runCPUBFS, "
                                   "serial Dijkstra (no CPU SSSP in the reference), pr_cal pull iterations; "
                                   "extrapolated to E (BFS, SSSP) or 5E (PR5) edges per request, requests "
                                   "spread over %d threads" % (target, n, threads)},
        "e2e": {"value": val, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": gen_s,
    }
    print(json.dumps(line), flush=True)


def packed_bits(V: int, wmin: int = 1, wmax: int = 64) -> int:
    """Bits of one packed edge record: column bits(V - 1) + weight bits(wmax - wmin)."""
    return int(V - 1).bit_length() + int(wmax - wmin).bit_length()


def config_dict(args, g):
    delta = args.delta if args.delta is not None else max(1, (1 + 64) // 16)  # the engine's default
    return {"workload": "oom-sssp-rmat%d-%gGiB-%dsrc" % (args.scale, args.budget_gib, args.sources),
            "graph": "R-MAT scale %d ef16 a,b,c=.57,.19,.19 symmetric dedup weights U[1,64]" % args.scale,
            "V": g.V, "E": g.E, "budget_bytes": int(args.budget_gib * GIB), "advisek": args.advisek,
            "sources": args.sources, "seeds": {"graph": 1, "weights": 2, "sources": 3},
            "l2": "inputs larger than L2 (packed graph %.1f GB)" % (g.E * packed_bits(g.V) / 8e9),
            "dynamic_mode": "direct" if args.direct else "staged", "sssp_delta": float(delta)}


def run_ours(args, rank, world, local):
    import torch
    import onegraph_gb300 as og

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    g, gen_s = make_graph(args.scale)
    deg = g.degrees()
    srcs = pick_sources(deg, args.sources)
    # replicas: each rank serves its own slice of the source list
    srcs = replicas.slice_queries(srcs, rank, world)
    t0 = time.time()
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=args.advisek,
                    direct=bool(args.direct), device=local)
    engine_s = time.time() - t0
    if args.delta is not None:
        eng.set_param(og.PARAM_SSSP_DELTA, args.delta)
    args.delta = eng.get_param(og.PARAM_SSSP_DELTA)
    plan = eng.plan

    def barrier():
        replicas.barrier(world)

    # Large page-locked allocations (the end-to-end result buffer, the copy
    # probe's 2 GiB) are made before the warm-up: queries run right after such
    # an allocation were at times twice as slow.
    host = torch.empty(g.V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    h2d = h2d_peak_gbs()
    for i in range(args.warmup):
        eng.sssp(srcs[i % len(srcs)], out=False)
    # device-resident timing
    sampler = ClockSampler(local)
    sampler.start()
    stream = torch.cuda.current_stream()
    stats = []
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(args.steps):
        eng.sssp(srcs[(args.warmup + k) % len(srcs)], out=False)
        stats.append(dict(eng.stats))
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    t_dev = replicas.max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    value = replicas.whole_job_rate(args.steps, world, t_dev)
    # end-to-end through the C ABI into a page-locked host buffer
    torch.cuda.synchronize()
    barrier()
    e0 = time.perf_counter()
    for k in range(args.steps):
        eng.sssp(srcs[(args.warmup + k) % len(srcs)], out=host)
    e2e_s = time.perf_counter() - e0
    e2e_stats = dict(eng.stats)
    # per-query edges of the reached component (from the last e2e result)
    comp_edges = reached_edges(deg, host)
    lat = sorted(s["ms_total"] for s in stats)
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(round(0.99 * (len(lat) - 1))))]
    launches = sum(s["launches"] for s in stats)
    peaks = measured_peaks()
    # Kernel-level timing of the dominant kernel: the same queries again with
    # the relax timer on, so that every relax launch of the device-driven
    # rounds is bracketed by two stamp kernels reading the GPU's global timer
    # (og_stats.ms_relax); the timed queries above run without them.  The
    # host-driven loop is timed beside it with CUDA events around each round's
    # relax launch, for comparison: those intervals also hold any host delay
    # between the start event and the launch.
    eng.set_param(og.PARAM_RELAX_TIMER, 1)
    # one untimed query first: a mode switch recaptures the round graphs, and
    # the first replay pays for loading kernels used for the first time
    eng.sssp(srcs[0], out=False)
    tstats = []
    for k in range(min(args.steps, 8)):
        eng.sssp(srcs[(args.warmup + k) % len(srcs)], out=False)
        tstats.append(dict(eng.stats))
    eng.set_param(og.PARAM_RELAX_TIMER, 0)
    relax_dev_ms = statistics.mean(s["ms_relax"] for s in tstats)
    link_dev = statistics.mean(s["link_bytes"] for s in tstats)
    static_dev = statistics.mean(s["edges_static"] for s in tstats)
    eng.set_param(og.PARAM_LEVEL_LOOP, og.LOOP_HOST)
    eng.sssp(srcs[0], out=False)  # untimed, as above
    kstats = []
    for k in range(min(4, len(srcs))):
        eng.sssp(srcs[k], out=False)
        kstats.append(dict(eng.stats))
    eng.set_param(og.PARAM_LEVEL_LOOP, og.LOOP_AUTO)
    st_edges = sum(s["edges_static"] for s in kstats)
    st_verts = sum(s["static_vertices"] for s in kstats)
    dyn_bytes = sum(s["link_bytes"] for s in kstats)
    relax_ms = sum(s["ms_dynamic"] + s["ms_static"] for s in kstats)
    # algorithmic bytes: per edge one packed record (plan edge_bits: 27 column +
    # 6 weight bits at scale 27) and the target distance (4 B); 20 B per vertex
    eb = plan["edge_bits"] / 8
    kname = ("k_lbs_pair_dev<SrcP<true>,SrcP<true>,MinOp<true>> (device-driven rounds: static + dynamic "
             "tiles of a round)" if args.direct else "k_gather<SrcP<true>,DstW<u8>> + staged relax")
    link_gbs = link_dev / (relax_dev_ms / 1e3) / 1e9 if relax_dev_ms else 0.0
    static_gbs = (eb + 4) * static_dev / (relax_dev_ms / 1e3) / 1e9 if relax_dev_ms else 0.0
    host_link_gbs = dyn_bytes / (relax_ms / 1e3) / 1e9 if relax_ms else 0.0
    host_static_gbs = ((eb + 4) * st_edges + 20 * st_verts) / (relax_ms / 1e3) / 1e9 if relax_ms else 0.0
    rounds_dev = statistics.mean(s["iterations"] for s in tstats)
    roof_link = {"bound": "host-link", "kernel": kname, "achieved": link_gbs, "peak": h2d, "unit": "GB/s",
                 "frac": link_gbs / h2d if h2d else None,
                 "traffic": link_dev / max(rounds_dev, 1) * SSSP_RELAX_LINK_TRAFFIC_RATIO,
                 "traffic_note": "host-link bytes per relax launch: this query's algorithmic link bytes per round "
                                 "x %.3f, the sysmem-sector / algorithmic ratio ncu measured for the same relax's "
                                 "largest dynamic launch on R-MAT 22 under a 256 MiB budget"
                                 % SSSP_RELAX_LINK_TRAFFIC_RATIO,
                 "peak_source": "highest of the link probes measured in this run (og_link_probe)", "link_probes": dict(LINK_PEAKS),
                 "timing": "globaltimer stamps around every relax launch of %d device-driven queries "
                           "(the timed queries' sources, timer on)" % len(tstats)}
    roof_static = {"bound": "hbm", "kernel": kname + ", its HBM side", "achieved": static_gbs,
                   "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": static_gbs / peaks["hbm_gbs"],
                   "traffic": None, "peak_source": peaks["source"],
                   "note": "static records + target distances over the same kernel time"}
    roof_host = {"kernel": "k_lbs_pair<SrcP<true>,SrcP<true>,MinOp<true>> (host-driven rounds)",
                 "link_gbs": host_link_gbs, "link_frac": host_link_gbs / h2d if h2d else None,
                 "static_hbm_gbs": host_static_gbs,
                 "timing": "CUDA events around the relax launches of %d host-driven queries" % len(kstats)}
    dominant = roof_link
    if rank != 0:
        return
    cpu = None
    try:
        cpu = cpu_dijkstra_sample(g, srcs, deg, args.cpu_seconds, 1, lambda s: comp_edges)
        cpu = {"value": cpu["value"], "unit": "queries/s", "cores": 1, "kind": "port",
               "sample": "serial Dijkstra (oracle port; the reference has no CPU SSSP) bounded at "
                         "%d edges (~%.0f s), extrapolated to the %d edges of the reached component"
                         % (cpu["edges_per_thread"], args.cpu_seconds, comp_edges)}
    except Exception as ex:  # the baseline is reported, never required
        cpu = {"value": None, "unit": "queries/s", "cores": 1, "kind": "port", "sample": "failed: %s" % ex}
    line = {
        "metric": "queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": config_dict(args, g),
        "gteps": comp_edges * args.steps * world / t_dev / 1e9,
        "gteps_traversed": sum(s["edges_static"] + s["edges_dynamic"] for s in stats) / t_dev / 1e9,
        "p50_ms": p50, ("p99_ms" if len(lat) >= 100 else "latency_max_ms"): p99,
        "latency_samples": len(lat),
        "e2e": {"value": args.steps / e2e_s, "unit": "queries/s", "h2d_bytes_per_step":
                int(4 + e2e_stats["link_bytes"]), "d2h_bytes_per_step": 4 * g.V},
        "roofline": dominant, "roofline_static": roof_static, "roofline_link": roof_link,
        "roofline_host_loop": roof_host,
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
        "plan": {k: plan[k] for k in ("static_vertices", "static_edges", "dynamic_edges",
                                      "chunk_edges", "advisek", "edge_bits")},
        "per_query": {"iterations": statistics.mean(s["iterations"] for s in stats),
                      "ms_rounds": statistics.mean(s["ms_dynamic"] for s in stats),
                      "ms_relax": relax_dev_ms,
                      "ms_rounds_with_timer": statistics.mean(s["ms_dynamic"] for s in tstats),
                      "link_gb": statistics.mean(s["link_bytes"] for s in stats) / 1e9,
                      "host_loop_ms_relax": relax_ms / len(kstats),
                      "host_loop_ms_compact": statistics.mean(s["ms_compact"] for s in kstats)},
        "setup_s": {"generate": gen_s, "engine": engine_s},
    }
    print(json.dumps(line), flush=True)
    eng.close()


def run_sssp_batch(args, rank, world, local):
    """Multi-source SSSP: one step is one og_sssp_batch pass of --sssp-sources
    seeded sources (seed 3) on the weighted R-MAT graph, against the plain
    per-query og_sssp on an engine with the same budget and no batch state;
    per-source distances are checked equal to the plain path's."""
    import torch
    import onegraph_gb300 as og
    torch.cuda.set_device(local)
    g, gen_s = make_graph(args.scale)
    k = max(1, min(32, args.sssp_sources))
    srcs = np.array(pick_sources(g.degrees(), max(k, 32)), np.uint32)
    budget = int(args.budget_gib * GIB)
    eng = og.Engine(g, budget=budget, advisek=args.advisek, direct=True, sssp_batch=k, device=local)
    batches = [srcs[(i * k) % len(srcs):][:k] for i in range(4)]
    batches = [b if b.size == k else srcs[:k] for b in batches]
    for i in range(args.warmup):
        eng.sssp_batch(batches[i % 4], out=False)
    sampler = ClockSampler(local)
    sampler.start()
    stats = []

    def one(i):
        _, ck = eng.sssp_batch(batches[i % 4], out=False)
        stats.append(dict(eng.stats))
        return ck
    t, cks = timed(one, args.steps)
    clocks = sampler.stop()
    value = k * args.steps / t
    plan = eng.plan
    eng.close()
    plain = og.Engine(g, budget=budget, advisek=args.advisek, direct=True, device=local)
    plain.sssp(int(srcs[0]), out=False)
    exact = True
    pst = []

    def p1(i):
        plain.sssp(int(batches[0][i]), out=False)
        pst.append(dict(plain.stats))
        return plain.checksum(og.ALGO_SSSP)
    tp, pck = timed(p1, k)
    for i in range(k):
        exact &= tuple(int(x) for x in cks[0][i]) == pck[i]
    plain_plan = plain.plan
    plain.close()
    link = sum(x["link_bytes"] for x in stats) / len(stats)
    kms = sum(x["ms_dynamic"] for x in stats) / len(stats)
    peak = h2d_peak_gbs()
    ach = link / (kms / 1e3) / 1e9 if kms else 0.0
    line = {
        "metric": "queries/s", "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": dict(config_dict(args, g), workload="sssp-batch-rmat%d-%gGiB-%dsrc" % (args.scale,
                                                                                       args.budget_gib, k)),
        "plain_queries_per_s": k / tp, "speedup_vs_plain": value / (k / tp), "bit_exact_vs_single_source": exact,
        "per_pass": {"rounds": stats[0]["iterations"], "link_gb": link / 1e9, "ms_relax": kms,
                     "ms_compact": sum(x["ms_compact"] for x in stats) / len(stats)},
        "plain_per_query": {"link_gb": sum(x["link_bytes"] for x in pst) / len(pst) / 1e9},
        "plan": {"static_edges": plan["static_edges"], "plain_static_edges": plain_plan["static_edges"]},
        "roofline": {"bound": "host-link", "kernel": "k_sb_relax_pair (multi-source SSSP relax)", "achieved": ach,
                     "peak": peak, "unit": "GB/s", "frac": ach / peak if peak else None, "traffic": None,
                     "peak_source": "highest of the link probes measured in this run (og_link_probe)",
                     "link_probes": dict(LINK_PEAKS)},
        "clocks": clocks, "gpu_launches": sum(x["launches"] for x in stats), "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def timed(fn, steps):
    """Device-bracketed wall time of `steps` calls (every call synchronises)."""
    import torch
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s = torch.cuda.current_stream()
    ev0.record(s)
    out = [fn(k) for k in range(steps)]
    ev1.record(s)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3, out


def run_bfs_batch(args, rank, world, local):
    """Batched BFS: 256 seeded sources as four 64-source batches on the
    out-of-memory scale-27 graph, against the plain per-query BFS path."""
    import torch
    import onegraph_gb300 as og
    torch.cuda.set_device(local)
    g, gen_s = make_graph(args.scale)
    deg = g.degrees()
    srcs = np.array(pick_sources(deg, 256), np.uint32)
    # page-locked result buffers for the end-to-end legs (43 GB at R-MAT 27)
    # and the link probe come first, before the engine page-locks the graph
    # and before any query: large page-locked allocations between queries
    # have slowed the queries after them
    host32 = og.pinned_empty((64, g.V), np.uint32)
    host8 = og.pinned_empty((64, g.V), np.uint8)
    h2d = h2d_peak_gbs()
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=args.advisek, batch=True,
                    direct=True, device=local)
    tune = eng.bfs_batch_tune(srcs[:64], reps=1) if args.tune else None
    batches = [srcs[64 * i:64 * (i + 1)] for i in range(4)]
    for i in range(args.warmup):
        eng.bfs_batch(batches[i % 4], out=False)
    sampler = ClockSampler(local)
    sampler.start()
    stats = []

    def one(k):
        _, ck = eng.bfs_batch(batches[k % 4], out=False)
        stats.append(dict(eng.stats))
        return ck
    t, cks = timed(one, args.steps)
    clocks = sampler.stop()
    value = 64 * args.steps / t
    # plain per-query path on the same engine and sources
    nplain = 4

    def plain(k):
        eng.bfs(int(srcs[k]), out=False)
        return dict(eng.stats)
    tp, pst = timed(plain, nplain)
    plain_qps = nplain / tp
    # bit-exactness: the batch's per-source (reached, depth sum) vs single runs
    exact = True
    for k in range(nplain):
        dd = eng.bfs(int(srcs[k]))
        reached = dd != g.V + 1
        want = (int(reached.sum()), int(dd[reached].sum(dtype=np.uint64)))
        got = tuple(int(x) for x in cks[0][k])
        exact &= (want == got)
    # end to end: every depth into page-locked host memory (the first call
    # allocates the kept device depth matrix and is not timed)
    eng.bfs_batch(batches[0], out=host32)
    eng.bfs_batch_u8(batches[0], out=host8)
    ne2e = max(2, min(args.steps, 4))
    e2e_t, _ = timed(lambda k: eng.bfs_batch(batches[k % 4], out=host32)[1], ne2e)
    e2e8_t, cl = timed(lambda k: eng.bfs_batch_u8(batches[k % 4], out=host8)[1], ne2e)
    # the plain path end to end: one source's depths into page-locked memory
    host1 = og.pinned_empty(g.V, np.uint32)
    tpe, _ = timed(lambda k: eng.bfs(int(srcs[k]), out=host1), nplain)
    # the same batches with every level top-down (the bottom-up levels off)
    eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
    eng.bfs_batch(batches[0], out=False)  # captures the top-down graph
    std = []

    def td(k):
        _, ck = eng.bfs_batch(batches[k % 4], out=False)
        std.append(dict(eng.stats))
        return ck
    ttd, tcks = timed(td, 2)
    eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_AUTO)
    exact &= all(np.array_equal(tcks[k], cks[k]) for k in range(min(2, len(cks))))
    link = sum(x["link_bytes"] for x in stats) / len(stats)
    kms = sum(x["ms_static"] for x in stats) / len(stats)
    line = {
        "metric": "queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64-mask",
        "data": "synthetic",
        "config": dict(config_dict(args, g), workload="bfs-batch-rmat%d-%gGiB-4x64src" % (
            args.scale, args.budget_gib)),
        "plain_queries_per_s": plain_qps, "speedup_vs_plain": value / plain_qps,
        "bit_exact_vs_single_source": exact,
        "gteps": sum(x["edges_static"] + x["edges_dynamic"] for x in stats) / t / 1e9,
        "per_batch": {"levels": stats[0]["iterations"], "ms_kernel": kms,
                      "link_gb": link / 1e9, "link_gbs": link / (kms / 1e3) / 1e9 if kms else None,
                      "graph_replay": bool(stats[-1]["chunks"]),
                      "edges_examined": stats[0]["edges_static"] + stats[0]["edges_dynamic"]},
        "top_down_only": {"queries_per_s": 128 / ttd,
                          "ms_kernel": sum(x["ms_static"] for x in std) / len(std),
                          "link_gb": sum(x["link_bytes"] for x in std) / len(std) / 1e9,
                          "edges_examined": std[0]["edges_static"] + std[0]["edges_dynamic"]},
        "e2e": {"value": 64 * ne2e / e2e_t, "unit": "queries/s",
                "h2d_bytes_per_step": int(256 + link), "d2h_bytes_per_step": 64 * 4 * g.V,
                "note": "u32 depths of every source into page-locked host memory"},
        "e2e_u8": {"value": 64 * ne2e / e2e8_t, "unit": "queries/s", "d2h_bytes_per_step": 64 * g.V,
                   "clamped_entries": int(sum(cl)),
                   "note": "og_bfs_batch_u8: byte depths (0 unreached, 255 for depth >= 255)"},
        "plain_e2e_queries_per_s": nplain / tpe,
        "e2e_speedup_vs_plain_e2e": (64 * ne2e / e2e_t) / (nplain / tpe),
        "e2e_u8_speedup_vs_plain_e2e": (64 * ne2e / e2e8_t) / (nplain / tpe),
        "roofline": {"bound": "host-link", "kernel": "k_batch_persistent (one launch per 64-source batch)",
                     "achieved": link / (kms / 1e3) / 1e9 if kms else 0.0, "peak": h2d, "unit": "GB/s",
                     "frac": link / (kms / 1e3) / 1e9 / h2d if kms and h2d else None, "traffic": None,
                     "peak_source": "highest of the link probes measured in this run (og_link_probe)",
                     "link_probes": dict(LINK_PEAKS), "bytes_per_launch": link,
                     "note": "packed records read over the host link per batch over the kernel's CUDA-event "
                             "time; bottom-up levels read a few records per vertex at random, so the kernel is "
                             "bound by the link's request rate and grid barriers rather than its bandwidth"},
        "tune": tune, "clocks": clocks,
        "gpu_launches": sum(x["launches"] for x in stats),
        "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


def run_pr_precision(args, rank, world, local):
    """PageRank precision study: R-MAT scale 26, directed, in-edge CSR +
    out-degrees, 6 GiB budget; FP32 ranks with FP32 pull sums and the FP64 L1
    delta reduced on the GPU, stopped at L1 < 1e-6 (normalised ranks),
    against the multi-threaded FP64 host oracle; the reference's delta form
    (og_pr, per-vertex 1e-3) is timed beside it, and so is the push form
    (og_pr_l1_push over the out-edge CSR from og_graph_transpose, same budget),
    with its own errors against the same oracle."""
    import torch
    import onegraph_gb300 as og
    import oracle
    torch.cuda.set_device(local)
    t0 = time.time()
    try:
        g = og.Graph.rmat(args.scale, 16, seed=1, pagerank=True, symmetric=False, on_gpu=True)
    except og.OGError:
        g = og.Graph.rmat(args.scale, 16, seed=1, pagerank=True, symmetric=False)
    gen_s = time.time() - t0
    h2d = h2d_peak_gbs()
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=args.advisek,
                    direct=bool(args.direct), device=local)
    eng.pr_l1(0.85, 1e-6, 3, out=False)  # warm-up
    sampler = ClockSampler(local)
    sampler.start()
    t, outs = timed(lambda k: eng.pr_l1(0.85, 1e-6, 500), 1)
    clocks = sampler.stop()
    st = dict(eng.stats)
    rank32 = outs[0].astype(np.float64)
    t1, _ = timed(lambda k: eng.pr(0.001, 0, out=False), 1)
    st_delta = dict(eng.stats)
    eng.close()
    c0 = time.time()
    gt = g.transpose()
    tr_s = time.time() - c0
    peng = og.Engine(gt, budget=int(args.budget_gib * GIB), advisek=args.advisek,
                     direct=bool(args.direct), pagerank=True, device=local)
    peng.pr_l1_push(0.85, 1e-6, 3, out=False)  # warm-up
    tpush, pouts = timed(lambda k: peng.pr_l1_push(0.85, 1e-6, 500), 1)
    st_push = dict(peng.stats)
    push64 = pouts[0].astype(np.float64)
    peng.close()
    threads = os.cpu_count() or 1
    ref = np.empty(g.V)
    c0 = time.perf_counter()
    it_ref, l1_ref = oracle.pr_l1_mt_raw(g.V, g._off_p, g._edges_p, g._outdeg_p, 0.85, 1e-6, 500,
                                         threads, ref)
    cpu_s = time.perf_counter() - c0
    err = np.abs(rank32 - ref)
    perr = np.abs(push64 - ref)
    iters = max(st["iterations"], 1)
    piters = max(st_push["iterations"], 1)
    # The pull launches (both regions interleaved) per iteration: HBM side =
    # the algorithmic bytes of an iteration, V (16 + 4 + 4) + 8 E (offset
    # pair, rank write, contribution write; column + contribution per edge),
    # over their CUDA-event time; at 6 GiB most records are static, so HBM is
    # the bound.  Link side = packed dynamic records per iteration.
    peaks = measured_peaks()
    kms = st["ms_dynamic"] / iters
    hbm_gbs = (24 * g.V + 8 * g.E) / (kms / 1e3) / 1e9 if kms else 0.0
    roof_hbm = {"bound": "hbm", "kernel": "k_pr_pull_pair<SrcP<false>,SrcP<false>> (every iteration of the run)",
                "achieved": hbm_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": hbm_gbs / peaks["hbm_gbs"], "traffic": None, "peak_source": peaks["source"],
                "bytes_per_launch": 24 * g.V + 8 * g.E, "kernel_ms_per_iter": kms,
                "note": "algorithmic bytes V (16 + 4 + 4) + 8 E per iteration over the pull launches' time"}
    link_gbs = st["link_bytes"] / (st["ms_dynamic"] / 1e3) / 1e9 if st["ms_dynamic"] else 0.0
    roof = {"bound": "host-link", "kernel": "k_pr_pull_pair<SrcP<false>,SrcP<false>> (every iteration of the run)",
            "achieved": link_gbs, "peak": h2d, "unit": "GB/s", "frac": link_gbs / h2d if h2d else None,
            "traffic": st["link_bytes"] / iters * PR_PULL_LINK_TRAFFIC_RATIO,
            "traffic_note": "host-link bytes per launch: algorithmic bytes x %.3f, the sysmem-sector / "
                            "algorithmic ratio ncu measured for the same kernel on R-MAT 22 under a 256 MiB "
                            "budget" % PR_PULL_LINK_TRAFFIC_RATIO,
            "peak_source": "highest of the link probes measured in this run (og_link_probe)",
            "link_probes": dict(LINK_PEAKS), "link_gb_per_iter": st["link_bytes"] / iters / 1e9,
            "kernel_ms_per_iter": st["ms_dynamic"] / iters}
    line = {
        "metric": "pagerank iterations/s", "value": iters / t, "unit": "iterations/s",
        "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": t * 1e3 / iters,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 L1 reduction)", "data": "synthetic",
        "config": {"workload": "pr-precision-rmat%d-directed-%gGiB" % (args.scale, args.budget_gib),
                   "V": g.V, "E": g.E, "damping": 0.85, "tol_l1": 1e-6, "budget_bytes": int(args.budget_gib * GIB),
                   "advisek": args.advisek, "dynamic_mode": "direct" if args.direct else "staged"},
        "iterations": st["iterations"], "residual_l1": st["residual"], "ms_total": t * 1e3,
        "max_abs_err": float(err.max()), "l1_err": float(err.sum()),
        "max_rel_err": float((err / ref).max()),
        "oracle": {"iterations": it_ref, "residual_l1": l1_ref, "seconds": cpu_s, "threads": threads},
        "link_gb_per_iter": st["link_bytes"] / iters / 1e9,
        "delta_form": {"rounds": st_delta["iterations"], "ms": t1 * 1e3},
        "push": {"iterations_per_s": piters / tpush, "iterations": st_push["iterations"],
                 "ms_per_iter": tpush * 1e3 / piters, "residual_l1": st_push["residual"],
                 "max_abs_err": float(perr.max()), "l1_err": float(perr.sum()),
                 "max_rel_err": float((perr / ref).max()),
                 "max_abs_diff_vs_pull": float(np.abs(push64 - rank32).max()),
                 "link_gb_per_iter": st_push["link_bytes"] / piters / 1e9,
                 "transpose_s": tr_s},
        "cpu_baseline": {"value": it_ref / cpu_s, "unit": "iterations/s", "cores": threads, "kind": "port",
                         "sample": "FP64 pull PageRank oracle, full run to L1 < 1e-6"},
        "roofline": roof_hbm, "roofline_link": roof, "gpu_launches": st["launches"],
        "clocks": clocks, "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_bfs_resident(args, rank, world, local):
    """Single-source BFS on a fully resident graph (advisek 1.0): R-MAT scale
    20, symmetric, u32 CSR, source = highest-degree vertex; bit-exact against
    the runCPUBFS restatement.  Plain path (og_bfs) and the persistent
    one-launch path (og_bfs_batch with one source, CUDA-graph replay)."""
    import torch
    import onegraph_gb300 as og
    import oracle
    torch.cuda.set_device(local)
    t0 = time.time()
    try:
        g = og.Graph.rmat(args.scale, 16, seed=1, on_gpu=True)
    except og.OGError:
        g = og.Graph.rmat(args.scale, 16, seed=1)
    gen_s = time.time() - t0
    deg = g.degrees()
    src = int(np.argmax(deg))
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=1.0, batch=True, device=local)
    if args.bfs_direction == "top-down":
        eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
    for _ in range(args.warmup):
        eng.bfs(src, out=False)
        eng.bfs_batch([src], out=False)
    sampler = ClockSampler(local)
    sampler.start()
    stats = []

    def plain(k):
        eng.bfs(src, out=False)
        stats.append(dict(eng.stats))
    t, _ = timed(plain, args.steps)
    tb, _ = timed(lambda k: eng.bfs_batch([src], out=False), args.steps)
    clocks = sampler.stop()
    d = eng.bfs(src)
    want, _ = oracle.bfs(np.array(g.offsets), np.array(g.columns), src)
    exact = bool((oracle.normalise_bfs(d, g.V) == want).all())
    reached = d != g.V + 1
    comp_edges = int(deg[reached].sum(dtype=np.int64))
    # kernel time of all levels: top-down levels count as static-region time,
    # bottom-up levels as dynamic-region time
    k_ms = sum(x["ms_static"] + x["ms_dynamic"] for x in stats)
    examined = sum(x["edges_static"] + x["edges_dynamic"] for x in stats)
    fverts = sum(x["frontier_sum"] for x in stats)
    peaks = measured_peaks()
    # per examined edge: one packed column record (edge_bits) + the 4 B probe of
    # the target's visited word (top-down) or the neighbour's frontier word
    # (bottom-up); 20 B per frontier vertex
    eb = eng.plan["edge_bits"] / 8
    gbs = ((eb + 4) * examined + 20 * fverts) / (k_ms / 1e3) / 1e9 if k_ms else 0.0
    # the same query with every level top-down: every edge of the component
    # is read once, so this leg shows the kernels' bandwidth on the resident
    # region (direction optimisation reads a small fraction of the edges)
    eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
    eng.bfs(src, out=False)
    tstats = []

    def topdown(k):
        eng.bfs(src, out=False)
        tstats.append(dict(eng.stats))
    ttd, _ = timed(topdown, args.steps)
    td_ms = sum(x["ms_static"] + x["ms_dynamic"] for x in tstats)
    td_ex = sum(x["edges_static"] + x["edges_dynamic"] for x in tstats)
    td_fv = sum(x["frontier_sum"] for x in tstats)
    td_gbs = ((eb + 4) * td_ex + 20 * td_fv) / (td_ms / 1e3) / 1e9 if td_ms else 0.0
    # the relax kernel alone: the same top-down queries with the engine's stamp
    # timer around every relax launch (og_stats.ms_relax)
    eng.set_param(og.PARAM_RELAX_TIMER, 1)
    eng.bfs(src, out=False)
    rstats = []
    for _ in range(args.steps):
        eng.bfs(src, out=False)
        rstats.append(dict(eng.stats))
    eng.set_param(og.PARAM_RELAX_TIMER, 0)
    eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_AUTO if args.bfs_direction == "auto" else og.BFS_TOP_DOWN)
    rx_ms = sum(x["ms_relax"] for x in rstats)
    rx_ex = sum(x["edges_static"] + x["edges_dynamic"] for x in rstats)
    rx_fv = sum(x["frontier_sum"] for x in rstats)
    rx_gbs = ((eb + 4) * rx_ex + 20 * rx_fv) / (rx_ms / 1e3) / 1e9 if rx_ms else 0.0
    c0 = time.perf_counter()
    oracle.bfs(np.array(g.offsets), np.array(g.columns), src)
    cpu_s = time.perf_counter() - c0
    line = {
        "metric": "GTEPS", "value": comp_edges * args.steps / t / 1e9, "unit": "GTEPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "bfs-resident-rmat%d" % args.scale, "V": g.V, "E": g.E, "source": src,
                   "advisek": 1.0, "l2": "graph %.0f MB" % (g.E * 4 / 1e6)},
        "persistent_ms_per_query": tb / args.steps * 1e3,
        "persistent_gteps": comp_edges * args.steps / tb / 1e9,
        "top_down_only": {"ms_per_query": ttd / args.steps * 1e3,
                          "gteps": comp_edges * args.steps / ttd / 1e9,
                          "edges_examined_per_query": td_ex / args.steps,
                          "achieved_gbs": td_gbs, "frac": td_gbs / peaks["hbm_gbs"],
                          "graph_vs_l2": "packed records %.0f MB, L2 129 MB" % (g.E * eb / 1e6),
                          "relax_kernel": {"kernel": "k_lbs_pair_dev<SrcP<false>,SrcP<false>,BfsOp>",
                                           "ms_per_query": rx_ms / args.steps, "achieved_gbs": rx_gbs,
                                           "frac": rx_gbs / peaks["hbm_gbs"],
                                           "timing": "globaltimer stamps around every relax launch"}},
        "direction": args.bfs_direction,
        "bit_exact_vs_runCPUBFS": exact, "levels": stats[0]["iterations"],
        "edges_examined_per_query": examined / args.steps,
        "roofline": {"bound": "hbm", "kernel": "device-driven level loop (compaction, top-down k_lbs_pair_dev, "
                                               "k_bfs_bottom_up, control): all kernels of a query",
                     "achieved": gbs,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
                     "traffic": None, "peak_source": peaks["source"]},
        "cpu_baseline": {"value": comp_edges / cpu_s / 1e9, "unit": "GTEPS", "cores": 1, "kind": "port",
                         "sample": "runCPUBFS restatement, one full query"},
        "gpu_launches": sum(x["launches"] for x in stats), "clocks": clocks, "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


def run_replace(args, rank, world, local):
    """Static-region replacement (OG_CFG_REPLACE: half of the static region's
    bytes as fragment slots that the policy refills between rounds) against
    the same engine without it, on the out-of-memory R-MAT 27 graph (8 GiB,
    advisek 0.8, direct), both with host-driven rounds: near/far SSSP from
    the seeded sources, label-propagation CC, top-down BFS.  A step is one
    SSSP query; the other algorithms' figures sit beside it."""
    import torch
    import onegraph_gb300 as og
    torch.cuda.set_device(local)
    g, gen_s = make_graph(args.scale)
    srcs = pick_sources(g.degrees(), args.sources)
    budget = int(args.budget_gib * GIB)
    out, checks = {}, {}
    clocks = None
    for mode in ("plain", "replace"):
        eng = og.Engine(g, budget=budget, advisek=args.advisek, direct=True, replace=mode == "replace",
                        device=local)
        eng.set_param(og.PARAM_LEVEL_LOOP, og.LOOP_HOST)
        eng.set_param(og.PARAM_CC_METHOD, og.CC_LABEL_PROPAGATION)
        for i in range(args.warmup):
            eng.sssp(srcs[i % len(srcs)], out=False)
        sampler = ClockSampler(local)
        sampler.start()
        r = {}
        for algo, name, n in ((og.ALGO_SSSP, "sssp", args.steps), (og.ALGO_CC, "cc_label_propagation", 2),
                              (og.ALGO_BFS, "bfs_top_down", args.steps)):
            if algo == og.ALGO_BFS:
                eng.set_param(og.PARAM_BFS_DIRECTION, og.BFS_TOP_DOWN)
            f0 = eng.fragment_stats() if mode == "replace" else None
            st, cks = [], []

            def one(k):
                if algo == og.ALGO_SSSP:
                    eng.sssp(srcs[(args.warmup + k) % len(srcs)], out=False)
                elif algo == og.ALGO_CC:
                    eng.cc(out=False)
                else:
                    eng.bfs(srcs[(args.warmup + k) % len(srcs)], out=False)
                st.append(dict(eng.stats))
                cks.append(eng.checksum(algo))
            t, _ = timed(one, n)
            r[name] = {"ms_per_query": t / n * 1e3, "link_gb_per_query": sum(x["link_bytes"] for x in st) / n / 1e9,
                       "rounds": statistics.mean(x["iterations"] for x in st)}
            if f0 is not None:
                f1 = eng.fragment_stats()
                dh = f1["records_host"] - f0["records_host"]
                ds = f1["records_slots"] - f0["records_slots"]
                r[name].update({"records_from_slots_frac": ds / max(ds + dh, 1),
                                "swaps_per_query": (f1["swaps"] - f0["swaps"]) / n,
                                "swap_gb_per_query": (f1["swap_bytes"] - f0["swap_bytes"]) / n / 1e9})
            checks.setdefault(name, []).append(cks)
        c = sampler.stop()
        clocks = clocks or c
        r["plan"] = {k: eng.plan[k] for k in ("static_vertices", "static_edges", "dynamic_edges", "edge_bits")}
        if mode == "replace":
            r["fragments"] = eng.fragment_stats()
        out[mode] = r
        eng.close()
    exact = all(a == b for a, b in checks.values())
    sp, rp = out["plain"]["sssp"], out["replace"]["sssp"]
    line = {
        "metric": "queries/s", "value": 1e3 / rp["ms_per_query"], "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": rp["ms_per_query"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": dict(config_dict(args, g), workload="replace-rmat%d-%gGiB" % (args.scale, args.budget_gib),
                       level_loop="host"),
        "plain_queries_per_s": 1e3 / sp["ms_per_query"], "results_identical": exact,
        "replace": out["replace"], "plain": out["plain"], "clocks": clocks, "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_cc_oom(args, rank, world, local):
    """Connected components out of memory: the R-MAT 27 graph of the SSSP
    workload (columns only), 8 GiB budget, advisek 0.8, direct dynamic region.
    One step = one full CC (labels reset to the vertex ids, label propagation
    to the fixed point)."""
    import torch
    import onegraph_gb300 as og
    import oracle
    torch.cuda.set_device(local)
    g, gen_s = make_graph(args.scale)
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=args.advisek,
                    direct=bool(args.direct), device=local)
    # page-locked result buffer and link probe before the warm-up (a large
    # page-locked allocation between queries slows the queries after it)
    host = torch.empty(g.V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    h2d = h2d_peak_gbs()
    for _ in range(args.warmup):
        eng.cc(out=False)
    sampler = ClockSampler(local)
    sampler.start()
    stats = []

    def one(k):
        eng.cc(out=False)
        stats.append(dict(eng.stats))
    t, _ = timed(one, args.steps)
    clocks = sampler.stop()
    check = eng.checksum(og.ALGO_CC)
    method = {og.CC_AUTO: "auto", og.CC_LABEL_PROPAGATION: "label propagation",
              og.CC_UNION_FIND: "union-find"}[int(eng.get_param(og.PARAM_CC_METHOD))]
    if method == "auto":
        method = "union-find" if g.symmetric() else "label propagation"
    # the other method on the same engine: timing and the same components
    other = og.CC_LABEL_PROPAGATION if method == "union-find" else og.CC_AUTO
    eng.set_param(og.PARAM_CC_METHOD, other)
    eng.cc(out=False)
    t_other, _ = timed(lambda k: eng.cc(out=False), 1)
    other_stats = dict(eng.stats)
    same = eng.checksum(og.ALGO_CC) == check
    eng.set_param(og.PARAM_CC_METHOD, og.CC_AUTO)
    eng.cc(out=False)
    e0 = time.perf_counter()
    for _ in range(args.steps):
        eng.cc(out=host)
    e2e_s = time.perf_counter() - e0
    visits = statistics.mean(x["edges_static"] + x["edges_dynamic"] for x in stats)
    # edge visits of label propagation (the reference's algorithm): the CPU
    # baseline's work
    lp_stats = other_stats if method == "union-find" else stats[0]
    lp_visits = lp_stats["edges_static"] + lp_stats["edges_dynamic"]
    dyn_ms = sum(x["ms_dynamic"] for x in stats)
    dyn_bytes = sum(x["link_bytes"] for x in stats)
    link_gbs = dyn_bytes / (dyn_ms / 1e3) / 1e9 if dyn_ms else 0.0
    # CPU: the serial label propagation's first round over the same graph,
    # bounded, as an edge-visit rate; the full run is extrapolated by the edge
    # visits of the GPU run (the same frontier-synchronous propagation)
    lab = np.empty(g.V, np.uint32)
    c0 = time.perf_counter()
    n0 = oracle.cc_round_bounded_raw(g.V, g._off_p, g._edges_p, 2, 20_000_000, lab)
    rate = n0 / (time.perf_counter() - c0)
    budget_edges = int(rate * args.cpu_seconds)
    c0 = time.perf_counter()
    n1 = oracle.cc_round_bounded_raw(g.V, g._off_p, g._edges_p, 2, budget_edges, lab)
    rate = n1 / (time.perf_counter() - c0)
    plan = eng.plan
    line = {
        "metric": "CC runs/s", "value": args.steps * world / t, "unit": "runs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": "oom-cc-rmat%d-%gGiB" % (args.scale, args.budget_gib), "V": g.V, "E": g.E,
                   "budget_bytes": int(args.budget_gib * GIB), "advisek": args.advisek,
                   "dynamic_mode": "direct" if args.direct else "staged",
                   "l2": "inputs larger than L2 (packed graph %.1f GB)" % (g.E * plan["edge_bits"] / 8e9)},
        "gteps": g.E / (t / args.steps) / 1e9, "rounds": stats[0]["iterations"],
        "components_checksum": check, "cc_method": method,
        "other_method": {"method": "label propagation" if method == "union-find" else "union-find",
                         "ms_per_run": t_other * 1e3, "link_gb": other_stats["link_bytes"] / 1e9,
                         "same_components": same},
        "e2e": {"value": args.steps / e2e_s, "unit": "runs/s", "h2d_bytes_per_step":
                int(statistics.mean(x["link_bytes"] for x in stats)), "d2h_bytes_per_step": 4 * g.V},
        "roofline": {"bound": "host-link",
                     "kernel": "k_uf_sample (one record per vertex, random 32-byte sectors over the link)"
                     if method == "union-find" else "k_lbs_pair<SrcP<false>,MinOp<false>> over host-mapped records",
                     "achieved": link_gbs, "peak": h2d, "unit": "GB/s", "frac": link_gbs / h2d if h2d else None,
                     "traffic": None, "peak_source": "highest of the link probes measured in this run (og_link_probe)", "link_probes": dict(LINK_PEAKS),
                     "note": "algorithmic bytes = packed records read; union-find reads one record per "
                             "sampled vertex, a full 32-byte sector each, so it is bound by the link's "
                             "request rate rather than its bandwidth" if method == "union-find" else ""},
        "cpu_baseline": {"value": rate / lp_visits, "unit": "runs/s", "cores": 1, "kind": "port",
                         "sample": "first round of the serial label propagation (CC/serial restatement) "
                                   "bounded at %d edges (~%.0f s, %.2f G edge visits/s), extrapolated to "
                                   "the %.2f G edge visits of label propagation on the GPU (the same "
                                   "frontier-synchronous propagation)" % (n1, args.cpu_seconds, rate / 1e9,
                                                                          lp_visits / 1e9)},
        "per_run": {"edge_visits": visits, "link_gb": statistics.mean(x["link_bytes"] for x in stats) / 1e9,
                    "ms_static": statistics.mean(x["ms_static"] for x in stats),
                    "ms_dynamic": statistics.mean(x["ms_dynamic"] for x in stats),
                    "ms_compact": statistics.mean(x["ms_compact"] for x in stats)},
        "plan": {k: plan[k] for k in ("static_vertices", "static_edges", "dynamic_edges", "edge_bits")},
        "gpu_launches": sum(x["launches"] for x in stats), "clocks": clocks, "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


# Serving mix: per graph scale, the device budget (GiB) of its resident state
# and first query context, and the sources of one multi-source SSSP pass.
# The four budgets hold 22.5 of the 24 GiB; the rest admits extra contexts.
SERVING_GRAPHS = {22: (1.0, 16), 24: (3.75, 16), 26: (6.75, 8), 27: (12.2, 4)}


SERVING_SLOTS: dict = {}  # --serving-slots overrides by scale


def serving_graph(sc: int):
    """(budget GiB, SSSP sources per pass) of a serving graph; smaller test
    graphs get 1 GiB and 8 sources."""
    b, k = SERVING_GRAPHS.get(sc, (1.0, 8))
    return b, SERVING_SLOTS.get(sc, k)
# direct mode keeps no staging buffers, so the whole edge share is static
SERVING_ADVISEK = 1.0
ALGO_BFS, ALGO_SSSP, ALGO_PR = 0, 1, 3  # og_algo values (the reference arm loads no engine)
# host-link sectors read by one PageRank pull launch over its algorithmic link
# bytes, measured with ncu on R-MAT 22 directed under a 256 MiB budget:
# 2,025,677 sectors of 32 B for 64.2 MB of records per iteration
PR_PULL_LINK_TRAFFIC_RATIO = 1.010
# the same for the single-source SSSP relax's largest dynamic launch on R-MAT
# 22 weighted, 256 MiB: 96.6 MB of sysmem sectors for 94.8 MB of records
SSSP_RELAX_LINK_TRAFFIC_RATIO = 1.019


def serving_requests(degrees, n, rate, seed=4):
    """The request mix: Poisson arrivals at `rate`/s, graph by Zipf(1.1) with
    the smallest graph most popular, 60 % BFS / 30 % SSSP / 10 % PageRank
    (5 iterations), sources uniform over each graph's vertices with edges."""
    rng = np.random.default_rng(seed)
    z = np.array([1.0 / (k + 1) ** 1.1 for k in range(len(degrees))])
    z /= z.sum()
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    gsel = rng.choice(len(degrees), n, p=z)
    u = rng.random(n)
    algos = np.where(u < 0.6, ALGO_BFS, np.where(u < 0.9, ALGO_SSSP, ALGO_PR))
    nz = [np.nonzero(d)[0] for d in degrees]
    srcs = [int(nz[gi][rng.integers(0, nz[gi].size)]) for gi in gsel]
    return arrivals, gsel, algos, srcs


def serving_config(args, scales, VE, gsel_algos):
    algos = gsel_algos
    return {"workload": "serving-rmat%s-%gGiB" % ("-".join(map(str, scales)), args.serving_budget_gib),
            "graphs": {str(sc): {"V": V, "E": E, "budget_bytes": int(serving_graph(sc)[0] * GIB),
                                 "sssp_sources_per_pass": serving_graph(sc)[1]}
                       for sc, (V, E) in zip(scales, VE)},
            "graph": "R-MAT ef16 a,b,c=.57,.19,.19 symmetric dedup weights U[1,64], seeds graph 1 weights 2",
            "budget_bytes": int(args.serving_budget_gib * GIB), "advisek": SERVING_ADVISEK,
            "arrivals": "Poisson %g/s, seed 4" % args.rate, "requests_per_pass": args.requests,
            "mix": {"bfs": int((algos == ALGO_BFS).sum()), "sssp": int((algos == ALGO_SSSP).sum()),
                    "pr5": int((algos == ALGO_PR).sum())},
            "zipf": "1.1, smallest graph most popular", "workers": args.workers,
            "l2": "inputs larger than L2 (R-MAT 26/27 packed records 8.4 / 17.4 GB)"}


def cpu_serving_estimate(views, gsel, algos, srcs, target_s, threads):
    """Served queries/s of the reference's CPU paths on the host cores for the
    request mix.  views[g] = (V, E, offsets pointer, {dst, w} pairs pointer).
    Every (graph, algorithm) class of the mix gets one bounded sample of its
    CPU algorithm, all classes at once on the host threads (so the samples
    share memory bandwidth as concurrent requests would): runCPUBFS for BFS,
    serial Dijkstra for SSSP (the reference ships no CPU SSSP), pr_cal pull
    iterations for PageRank.  Each class's edges/s extrapolate to its
    per-request edges (E for BFS and SSSP, 5 E for five PageRank iterations);
    requests are independent, so the mix's CPU time is their sum spread over
    the threads."""
    import oracle
    classes = sorted(set(zip(gsel.tolist(), algos.tolist())))
    first = {}
    for i, c in enumerate(zip(gsel.tolist(), algos.tolist())):
        first.setdefault(c, srcs[i])

    def sample(c, max_edges):
        gi, a = c
        V, E, offp, edp = views[gi]
        t = time.perf_counter()
        if a == ALGO_BFS:
            out = np.empty(V, np.uint32)
            n = oracle.bfs_bounded_raw(V, offp, edp, 2, first[c], max_edges, out)
        elif a == ALGO_SSSP:
            out = np.empty(V, np.uint32)
            n = oracle.sssp_dijkstra_bounded_raw(V, offp, edp, first[c], max_edges, out)
        else:
            out = np.empty(V, np.float64)
            n = oracle.pr_pull_bounded_raw(V, offp, edp, 2, max_edges, out)
        return max(n, 1), time.perf_counter() - t

    # calibration: a short sample of each class on its own
    rate0 = {c: (lambda r: r[0] / max(r[1], 1e-6))(sample(c, 2_000_000)) for c in classes}
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        t0 = time.perf_counter()
        res = dict(zip(classes, ex.map(lambda c: sample(c, max(int(rate0[c] * target_s), 1)), classes)))
        wall = time.perf_counter() - t0
    rate = {c: res[c][0] / res[c][1] for c in classes}
    total_s = 0.0
    for c in zip(gsel.tolist(), algos.tolist()):
        work = views[c[0]][1] * (5 if c[1] == ALGO_PR else 1)
        total_s += work / rate[c]
    n = len(gsel)
    return {"value": n / (total_s / threads), "cores": threads, "wall_s": wall,
            "rates_edges_per_s": {"g%d/a%d" % c: r for c, r in rate.items()}}


def serve_pass(srv, arrivals, gsel, algos, srcs, outs=None):
    """Submits the mix at its arrival times (client thread) and collects every
    response; returns (responses by request, span in ms from the first
    submission to the last response, server clock)."""
    import threading
    n = len(gsel)
    t0 = time.perf_counter()
    err = []

    def client():
        try:
            for i in range(n):
                dt = arrivals[i] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                srv.submit(int(gsel[i]), int(algos[i]), srcs[i], iterations=5,
                           out=None if outs is None else outs[i], user=i)
        except Exception as ex:  # reported below
            err.append(ex)
    th = threading.Thread(target=client)
    th.start()
    resp = {}
    while len(resp) < n and (th.is_alive() or len(resp) < srv.stats()["submitted"]):
        for r in srv.poll(1024, wait_ms=200):
            resp[r["user"]] = r
    th.join()
    if err:
        raise err[0]
    span = max(r["t_done_ms"] for r in resp.values()) - min(r["t_submit_ms"] for r in resp.values())
    return resp, span


def run_serving(args, rank, world, local):
    """Serving mix: four resident weighted R-MAT graphs (scales 22/24/26/27)
    under a 24 GiB budget, Poisson arrivals at 2000 requests/s (seed 4),
    60 % BFS / 30 % SSSP / 10 % PageRank (5 iterations), graph by Zipf(1.1)
    with the smallest graph most popular.  A step is one pass of the 400
    requests through og_server (continuous batching: multi-source SSSP passes
    that requests join in flight, fused BFS passes, shared PageRank).  Then
    the same requests end to end (every result into page-locked host memory),
    and one at a time through the plain per-query path (og_bfs / og_sssp /
    og_pr_l1 on an engine per graph with the same budget and no batch state)."""
    import torch
    import onegraph_gb300 as og
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    scales = [int(x) for x in args.serving_scales.split(",")]
    graphs, gen_s = [], 0.0
    for sc in scales:
        g, t = make_graph(sc)
        graphs.append(g)
        gen_s += t
    n = args.requests
    arrivals, gsel, algos, srcs = serving_requests([g.degrees() for g in graphs], n, args.rate)
    budgets = [int(serving_graph(sc)[0] * GIB) for sc in scales]
    slots = [serving_graph(sc)[1] for sc in scales]
    # page-locked result buffers of the end-to-end passes (one per request),
    # allocated before any query: large page-locked allocations made between
    # queries have slowed the queries after them
    words = [graphs[gi].V for gi in gsel]
    pool = og.pinned_empty(int(sum(words)), np.uint32)
    outs, o = [], 0
    for i, w in enumerate(words):
        v = pool[o:o + w]
        outs.append(v.view(np.float32) if algos[i] == ALGO_PR else v.view(np.uint32))
        o += w
    h2d = h2d_peak_gbs()
    srv = og.Server(budget=int(args.serving_budget_gib * GIB), workers=args.workers, max_batch=64,
                    device=local)
    for g, b, k in zip(graphs, budgets, slots):
        srv.add_graph(g, budget=b, advisek=SERVING_ADVISEK, direct=True, pagerank=True, sssp_batch=k)
    # warm-up: every (graph, algorithm) once per warm-up step
    for w in range(args.warmup):
        for gi, g in enumerate(graphs):
            for a in (ALGO_BFS, ALGO_SSSP, ALGO_PR):
                srv.submit(gi, a, srcs[int(np.nonzero(gsel == gi)[0][0])], iterations=5, user=1 << 40)
        srv.drain()
        srv.poll(1 << 16, wait_ms=0)
    st0 = srv.stats()
    sampler = ClockSampler(local)
    sampler.start()
    lat, spans, ref_resp = [], [], None
    replicas.barrier(world)
    for k in range(args.steps):
        resp, span = serve_pass(srv, arrivals, gsel, algos, srcs)
        spans.append(span)
        lat.extend(resp[i]["t_done_ms"] - resp[i]["t_submit_ms"] for i in range(n))
        if ref_resp is None:
            ref_resp = resp
        elif any(resp[i]["checksum"] != ref_resp[i]["checksum"] for i in range(n)):
            raise RuntimeError("a served result changed between passes")
    replicas.barrier(world)
    clocks = sampler.stop()
    st1 = srv.stats()
    t_srv = replicas.max_over_ranks(sum(spans) / 1e3, world)
    value = replicas.whole_job_rate(args.steps * n, world, t_srv)
    if args.serving_legs == "served":
        srv.close()
        if rank == 0:
            print(json.dumps({"metric": "served queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "legs": "served passes only",
                              "gpu_launches": st1["launches"] - st0["launches"], "clocks": clocks}), flush=True)
        return
    # end to end: the same passes with every result in page-locked host memory
    e2e_passes = max(1, min(args.steps, 3))
    e2e_spans = []
    for k in range(e2e_passes):
        resp, span = serve_pass(srv, arrivals, gsel, algos, srcs, outs=outs)
        e2e_spans.append(span)
        bad = [i for i in range(n) if resp[i]["checksum"] != ref_resp[i]["checksum"] or resp[i]["status"]]
        if bad:
            raise RuntimeError("end-to-end results differ from the device-resident pass: %s" % bad[:5])
    e2e_qps = replicas.whole_job_rate(e2e_passes * n, world, replicas.max_over_ranks(sum(e2e_spans) / 1e3, world))
    srv.close()
    batch_of = {i: ref_resp[i]["batch"] for i in range(n)}
    run_ms = {i: ref_resp[i]["t_done_ms"] - ref_resp[i]["t_start_ms"] for i in range(n)}
    # plain per-query path: an engine per graph with the same budget and no
    # batch state, requests one after another in arrival order
    engines = [og.Engine(g, budget=b, advisek=SERVING_ADVISEK, direct=True, pagerank=True, device=local)
               for g, b in zip(graphs, budgets)]
    for gi, e in enumerate(engines):  # warm-up
        s0 = srcs[int(np.nonzero(gsel == gi)[0][0])]
        e.bfs(s0, out=False)
        e.sssp(s0, out=False)
        e.pr_l1(0.85, 0.0, 5, out=False)
    mism = 0
    pr_dev = 0.0
    plain_lat, plain_svc = [], []
    p0 = time.perf_counter()
    for i in range(n):
        e, a = engines[gsel[i]], int(algos[i])
        q0 = time.perf_counter()
        if a == ALGO_BFS:
            e.bfs(srcs[i], out=False)
        elif a == ALGO_SSSP:
            e.sssp(srcs[i], out=False)
        else:
            e.pr_l1(0.85, 0.0, 5, out=False)
        now = time.perf_counter()
        plain_svc.append((now - q0) * 1e3)
        plain_lat.append(max(0.0, (now - p0) - arrivals[i]) * 1e3)
        ck = e.checksum(a)
        if a == ALGO_PR:
            # FP32 pull sums are deterministic for a given plan; the plain
            # engines (no batch state) plan a larger static region, so their
            # tiles and summation order differ: equal to FP32 rounding
            fp = [float(np.array([x], np.uint64).view(np.float64)[0]) for x in (ck[1], ref_resp[i]["checksum"][1])]
            pr_dev = max(pr_dev, abs(fp[0] - fp[1]) / max(abs(fp[1]), 1e-30))
            mism += ck[0] != ref_resp[i]["checksum"][0] or pr_dev > 1e-5
        else:
            mism += ck != ref_resp[i]["checksum"]
    plain_wall = time.perf_counter() - p0
    for e in engines:
        e.close()
    plain_qps = n / plain_wall
    plain_svc = np.array(plain_svc)
    lat = np.array(lat)
    names = {ALGO_BFS: "bfs", ALGO_SSSP: "sssp", ALGO_PR: "pr5"}
    breakdown = {}
    for gi, sc in enumerate(scales):
        for a, nm in names.items():
            idx = [i for i in range(n) if gsel[i] == gi and algos[i] == a]
            if idx:
                breakdown["rmat%d/%s" % (sc, nm)] = {
                    "requests": len(idx), "plain_service_ms_mean": float(plain_svc[idx].mean()),
                    "plain_service_ms_total": float(plain_svc[idx].sum()),
                    "served_batch_mean": float(np.mean([batch_of[i] for i in idx])),
                    "served_run_ms_mean": float(np.mean([run_ms[i] for i in idx]))}
    # the dominant kernels measured alone on the R-MAT 27 graph's configuration
    roof = serving_rooflines(og, graphs[-1], budgets[-1], slots[-1], srcs, gsel, algos, len(graphs) - 1, h2d,
                             local)
    cpu = None
    if rank == 0 and world == 1:
        try:
            views = [(g.V, g.E, g._off_p, g._edges_p) for g in graphs]
            threads = os.cpu_count() or 1
            c = cpu_serving_estimate(views, gsel, algos, srcs, max(2.0, args.cpu_seconds / 3), threads)
            cpu = {"value": c["value"], "unit": "queries/s", "cores": threads, "kind": "port",
                   "sample": "one bounded sample (~%.0f s) per (graph, algorithm) class of the mix, all classes "
                             "at once: runCPUBFS, serial Dijkstra (no CPU SSSP in the reference), pr_cal pull "
                             "iterations; extrapolated to E (BFS, SSSP) or 5E (PR5) edges per request"
                             % max(2.0, args.cpu_seconds / 3), "rates_edges_per_s": c["rates_edges_per_s"]}
        except Exception as ex:
            cpu = {"value": None, "unit": "queries/s", "cores": 0, "kind": "port", "sample": "failed: %s" % ex}
    d2h = float(np.mean([4 * graphs[gi].V for gi in gsel]))
    line = {
        "metric": "served queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(spans) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32/f32",
        "data": "synthetic", "config": serving_config(args, scales, [(g.V, g.E) for g in graphs], algos),
        "step": "one pass of the %d-request mix through og_server" % n,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "latency_samples": int(lat.size),
        "plain_queries_per_s": plain_qps, "plain_p50_ms": float(np.percentile(plain_lat, 50)),
        "plain_p99_ms": float(np.percentile(plain_lat, 99)),
        "speedup_vs_plain": value / plain_qps, "results_identical_to_plain": mism == 0,
        "results_note": "BFS depths and SSSP distances bit-identical ({reached, sum} per request); PageRank "
                        "sum of FP32 ranks within 1e-5 relative (max seen %.2e): the plain engines plan a "
                        "different static region, so their pull tiles differ" % pr_dev,
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step":
                int(d2h * n), "passes": e2e_passes,
                "note": "a step is one pass of the mix; every request's V results read into page-locked host "
                        "memory, the request (graph, algorithm, source) sent from the host"},
        "roofline": roof["dominant"], "rooflines": roof["all"],
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": st1["launches"] - st0["launches"],
        "server": {k: st1[k] - st0.get(k, 0) if k != "used_bytes" else st1[k] for k in st1},
        "breakdown": breakdown, "setup_s": {"generate": gen_s},
    }
    if rank == 0 and world == 1 and args.configs != "none":
        # release this process's page-locked buffers and graphs first: every
        # configuration builds its own inputs in its own process
        pool = outs = None
        for g in graphs:
            g.close()
        graphs = []
        import gc
        gc.collect()
        torch.cuda.empty_cache()
        line["configs"] = run_config_legs(args)
    if rank == 0:
        print(json.dumps(line), flush=True)


# The other measured configurations, run after the serving measurement of the
# default line (one process each, so that each starts from an empty device):
# (key, bench.py arguments).  Graph, budget, sources and seeds are each
# workload's defaults: R-MAT 20 resident BFS from the highest-degree vertex;
# R-MAT 27 weighted, 8 GiB, advisek 0.8, 32 seeded SSSP sources; the same
# graph's CC; R-MAT 26 directed PageRank to L1 < 1e-6 under 6 GiB; 256 BFS
# sources as four 64-source batches on the R-MAT 27 graph.
CONFIG_LEGS = (
    ("bfs-resident", ["--workload", "bfs-resident", "--steps", "20"]),
    ("sssp-oom", ["--workload", "sssp-oom", "--steps", "8", "--cpu-seconds", "4"]),
    ("cc-oom", ["--workload", "cc-oom", "--steps", "4", "--cpu-seconds", "4"]),
    ("pr-precision", ["--workload", "pr-precision"]),
    ("bfs-batch", ["--workload", "bfs-batch", "--steps", "4"]),
)
CONFIG_LEGS_DEADLINE_S = 900.0


def run_config_legs(args) -> dict:
    """Runs the CONFIG_LEGS selected by --configs, each as `python bench.py
    --workload ...` with this run's warm-up count, and returns their JSON
    lines by workload.  A leg that fails or runs out of the shared deadline is
    recorded with its reason instead of a line."""
    want = None if args.configs == "all" else set(args.configs.split(","))
    out = {}
    t_end = time.time() + CONFIG_LEGS_DEADLINE_S
    for key, argv in CONFIG_LEGS:
        if want is not None and key not in want:
            continue
        left = t_end - time.time()
        if left < 60:
            out[key] = {"error": "not run: the configurations' %.0f s deadline was reached" % CONFIG_LEGS_DEADLINE_S}
            continue
        cmd = [sys.executable, os.path.abspath(__file__), *argv, "--warmup", str(max(3, args.warmup)),
               "--configs", "none"]
        t0 = time.time()
        try:
            p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=left)
            lines = [x for x in p.stdout.splitlines() if x.startswith("{")]
            if p.returncode == 0 and lines:
                out[key] = json.loads(lines[-1])
            else:
                out[key] = {"error": "exit %d: %s" % (p.returncode, (p.stderr or p.stdout)[-400:])}
        except subprocess.TimeoutExpired:
            out[key] = {"error": "killed after %.0f s (deadline)" % left}
        except Exception as ex:  # a leg never takes the headline line down
            out[key] = {"error": repr(ex)[:400]}
        out[key]["wall_s"] = time.time() - t0
    return out


def serving_rooflines(og, g, budget, slots, srcs, gsel, algos, gi, h2d, local):
    """Link-side rooflines of the serving mix's dominant kernels on the
    largest graph, in the server's engine configuration: the multi-source
    SSSP relax (k_sb_relax_pair) over one pass of `slots` sources, and the
    PageRank pull (k_pr_pull_pair) over five iterations.  Achieved = packed
    records read over the host link (og_stats.link_bytes) / the kernels'
    CUDA-event time on the engine's stream (og_stats.ms_dynamic); peak = the
    pinned host-to-device copy measured in this run."""
    e = og.Engine(g, budget=budget, advisek=SERVING_ADVISEK, direct=True, pagerank=True, batch=True,
                  sssp_batch=slots, device=local)
    idx = [i for i in range(len(gsel)) if gsel[i] == gi and algos[i] == ALGO_SSSP][:slots]
    ss = [srcs[i] for i in idx] or [srcs[0]]
    e.sssp_batch(ss, out=False)  # untimed first pass
    e.sssp_batch(ss, out=False)
    sb = dict(e.stats)
    e.pr_l1(0.85, 0.0, 5, out=False)
    e.pr_l1(0.85, 0.0, 5, out=False)
    pr = dict(e.stats)
    e.close()

    def roof(kernel, st, unit_note, traffic_ratio=None):
        ach = st["link_bytes"] / (st["ms_dynamic"] / 1e3) / 1e9 if st["ms_dynamic"] else 0.0
        per_launch = st["link_bytes"] / max(st["iterations"], 1)
        return {"bound": "host-link", "kernel": kernel, "achieved": ach, "peak": h2d, "unit": "GB/s",
                "frac": ach / h2d if h2d else None,
                "traffic": per_launch * traffic_ratio if traffic_ratio else None,
                "traffic_note": ("host-link bytes per launch: this launch's algorithmic bytes x %.3f, the "
                                 "sysmem-sector / algorithmic ratio ncu measured for the same kernel on R-MAT 22 "
                                 "under a 256 MiB budget" % traffic_ratio)
                if traffic_ratio else None,
                "peak_source": "highest of the link probes measured in this run (og_link_probe)", "link_probes": dict(LINK_PEAKS), "bytes_per_launch_note": unit_note,
                "link_gb": st["link_bytes"] / 1e9, "kernel_ms": st["ms_dynamic"]}
    a = roof("k_sb_relax_pair<SrcP<true>,SrcP<true>,%d> (multi-source SSSP relax, R-MAT %d pass of %d sources)"
             % (4 if slots <= 4 else 8, 27, len(ss)), sb, "packed 33-bit records of the dynamic region")
    b = roof("k_pr_pull_pair<SrcP<false>,SrcP<false>> (PageRank pull, R-MAT 27, 5 iterations)", pr,
             "packed records of the dynamic region per iteration", PR_PULL_LINK_TRAFFIC_RATIO)
    dom = a if sb["ms_dynamic"] >= pr["ms_dynamic"] else b
    return {"dominant": dom, "all": [a, b]}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "bfs-batch":
        run_bfs_batch(args, rank, world, local)
    elif args.workload == "serving":
        run_serving(args, rank, world, local)
    elif args.workload == "pr-precision":
        run_pr_precision(args, rank, world, local)
    elif args.workload == "bfs-resident":
        run_bfs_resident(args, rank, world, local)
    elif args.workload == "cc-oom":
        run_cc_oom(args, rank, world, local)
    elif args.workload == "sssp-batch":
        run_sssp_batch(args, rank, world, local)
    elif args.workload == "replace":
        run_replace(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
