#!/usr/bin/env python
"""Benchmark of the out-of-memory SSSP path on one GB300.

Workload (the reference's out-of-memory configuration): R-MAT scale 27,
edge factor 16, a,b,c,d = .57/.19/.19/.05, symmetrised, deduplicated, no
self-loops, seeded vertex permutation (seed 1), uint32 weights uniform in
[1, 64] (seed 2); device budget 8 GiB, advisek 0.8; SSSP from 32 seeded random
sources (seed 3) with edges.  The graph is synthetic (no datasets offline).

One step = one SSSP query (the next source, cycling over the 32) through the
engine: static prefix relaxed from HBM, the dynamic region gathered from
page-locked host memory every round.  `value` = queries/s with the result left
in device memory; `e2e` = queries/s through the C ABI writing the distances
into a page-locked host buffer (D2H of 4V bytes per query inside the timing).

--impl reference times the reference's CPU path on the host cores: the
reference ships no CPU SSSP, so its stand-in is the oracle's serial Dijkstra
(one query per host thread, bounded samples, extrapolated per query).
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

GIB = 1 << 30


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=27)
    ap.add_argument("--budget-gib", type=float, default=8.0)
    ap.add_argument("--advisek", type=float, default=0.8)
    ap.add_argument("--sources", type=int, default=32)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="sssp-oom",
                    choices=["sssp-oom", "bfs-batch", "bfs-resident", "pr-precision", "serving"],
                    help="sssp-oom (default headline), or another measured configuration")
    ap.add_argument("--tune", type=int, default=1, help="bfs-batch: run the autotuner first")
    ap.add_argument("--direct", type=int, default=1,
                    help="1: relax the dynamic region straight from page-locked host memory "
                         "(fastest); 0: gather into double-buffered device staging first")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def h2d_peak_gbs() -> float:
    """Page-locked host -> device copy bandwidth (best of 5, 2 GiB)."""
    import torch
    n = 2 * GIB
    src = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    dst = torch.empty(n, dtype=torch.uint8, device="cuda")
    best = 0.0
    s = torch.cuda.current_stream()
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        dst.copy_(src, non_blocking=True)
        b.record(s)
        b.synchronize()
        best = max(best, n / (a.elapsed_time(b) / 1e3) / 1e9)
    del src, dst
    torch.cuda.empty_cache()
    return best


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
    offp, edp = g._off_p, g._edges_p

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


def run_reference(args, rank, world):
    if rank != 0:
        return
    import onegraph_gb300 as og  # graph synthesis only; the timed path is the CPU oracle
    g, gen_s = make_graph(args.scale)
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


def config_dict(args, g):
    return {"workload": "oom-sssp-rmat%d-%gGiB-%dsrc" % (args.scale, args.budget_gib, args.sources),
            "graph": "R-MAT scale %d ef16 a,b,c=.57,.19,.19 symmetric dedup weights U[1,64]" % args.scale,
            "V": g.V, "E": g.E, "budget_bytes": int(args.budget_gib * GIB), "advisek": args.advisek,
            "sources": args.sources, "seeds": {"graph": 1, "weights": 2, "sources": 3},
            "l2": "inputs larger than L2 (graph %.1f GB)" % (g.E * 8 / 1e9),
            "dynamic_mode": "direct" if args.direct else "staged"}


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
    srcs = srcs[rank::world] if world > 1 else srcs
    t0 = time.time()
    eng = og.Engine(g, budget=int(args.budget_gib * GIB), advisek=args.advisek,
                    direct=bool(args.direct), device=local)
    engine_s = time.time() - t0
    plan = eng.plan

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

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
    t_dev = ev0.elapsed_time(ev1) / 1e3
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_dev], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_dev = float(t.item())
    value = args.steps * world / t_dev
    # end-to-end through the C ABI into a page-locked host buffer
    host = torch.empty(g.V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
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
    st_edges = sum(s["edges_static"] for s in stats)
    st_verts = sum(s["static_vertices"] for s in stats)
    st_ms = sum(s["ms_static"] for s in stats)
    dyn_bytes = sum(s["link_bytes"] for s in stats)
    dyn_ms = sum(s["ms_dynamic"] for s in stats)
    launches = sum(s["launches"] for s in stats)
    peaks = measured_peaks()
    h2d = h2d_peak_gbs()
    # algorithmic bytes: 12 B per edge ({dst,w} 8 B + dist 4 B), 20 B per vertex
    static_gbs = (12 * st_edges + 20 * st_verts) / (st_ms / 1e3) / 1e9 if st_ms else 0.0
    link_gbs = dyn_bytes / (dyn_ms / 1e3) / 1e9 if dyn_ms else 0.0
    roof_static = {"bound": "hbm", "kernel": "k_lbs<uint2,MinOp<true>> (static region relax)",
                   "achieved": static_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                   "frac": static_gbs / peaks["hbm_gbs"], "traffic": None,
                   "peak_source": peaks["source"]}
    roof_link = {"bound": "host-link", "kernel": "k_lbs<uint2,GatherOp> + dynamic relax",
                 "achieved": link_gbs, "peak": h2d, "unit": "GB/s", "frac": link_gbs / h2d if h2d else None,
                 "traffic": None, "peak_source": "measured pinned H2D copy in this run"}
    dominant = roof_link if dyn_ms > st_ms else roof_static
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
        "gteps_traversed": (st_edges + sum(s["edges_dynamic"] for s in stats)) / t_dev / 1e9,
        "p50_ms": p50, "p99_ms": p99,
        "e2e": {"value": args.steps / e2e_s, "unit": "queries/s", "h2d_bytes_per_step":
                int(4 + e2e_stats["link_bytes"]), "d2h_bytes_per_step": 4 * g.V},
        "roofline": dominant, "roofline_static": roof_static, "roofline_link": roof_link,
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
        "plan": {k: plan[k] for k in ("static_vertices", "static_edges", "dynamic_edges",
                                      "chunk_edges", "advisek")},
        "per_query": {"iterations": statistics.mean(s["iterations"] for s in stats),
                      "chunks": statistics.mean(s["chunks"] for s in stats),
                      "ms_static": st_ms / len(stats), "ms_dynamic": dyn_ms / len(stats),
                      "ms_compact": sum(s["ms_compact"] for s in stats) / len(stats),
                      "link_gb": dyn_bytes / len(stats) / 1e9},
        "setup_s": {"generate": gen_s, "engine": engine_s},
    }
    print(json.dumps(line), flush=True)
    eng.close()


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
    e2e_t, _ = timed(lambda k: eng.bfs_batch(batches[k % 4], out=None)[0], 1)
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
                      "graph_replay": bool(stats[-1]["chunks"])},
        "e2e": {"value": 64 / e2e_t, "unit": "queries/s",
                "h2d_bytes_per_step": int(256 + link), "d2h_bytes_per_step": 64 * 4 * g.V},
        "tune": tune, "clocks": clocks,
        "gpu_launches": sum(x["launches"] for x in stats),
        "setup_s": {"generate": gen_s},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "bfs-batch":
        run_bfs_batch(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
