#!/usr/bin/env python
"""Sliding-window GPMA+ benchmark on GB300 (edge updates/s, BFS GTEPS).

Workload (the reference demo, gpma_bfs_demo.cu:32-116, on its social-graph
configuration): a seeded Chung-Lu graph with 1,632,803 nodes and 30,622,564
directed edges (power law, exponent 2.3, largest expected degree 9,000; a
synthetic stand-in for the unavailable pokec file) is shuffled, its first
half loaded, a BFS run from node 0, then slide steps each insert the next
153,112 edges and delete the oldest 153,112 in one batch; a BFS from node 0
follows. One step = one slide update. The schedule wraps around the edge
list when warm-up + timed steps exceed its 100 slides.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpma|reference]

value  - updates/s over K steps with batches resident in HBM, device time
         from CUDA events on the launching stream; L2 flushed before every
         step (outside the timed span).
e2e    - the same through the C ABI from pinned host buffers: the batch
         upload and the read-back of the update status are inside the span.
--impl reference - the reference algorithm on the host cores (the C
         restatement in oracle/, OpenMP on all cores), same workload/metric;
         it loads only oracle/ libraries (graph generator included).
Several GPUs run independent replicas (the path does not shard); value sums
the ranks' updates over the slowest rank's time.

The printed line carries the headline figures of every configuration as
top-level scalars (bfs, batched, served, large_graph); the full sub-reports
go to --report (default bench_report.json next to this file).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "edge updates/s + BFS GTEPS on 1 GB300, batched vs plain GPMA; p99 query latency"
UNIT = "edge updates/s"
GRAPH = "social"
DATA = ("synthetic: seeded Chung-Lu power-law graph with pokec's shape (1,632,803 nodes, 30,622,564 edges, "
        "exponent 2.3, max expected degree 9,000, seed 2), shuffled")
L2_FLUSH_BYTES = 256 << 20
# the social configuration's generator parameters (gpma_bfs_gb300.workloads.GRAPHS["social"])
SOCIAL = dict(n=1632803, m=30622564, exponent=2.3, max_degree=9000, seed=2)


def workload_config(n, m, step):
    return {"workload": f"social sliding window: {n:,} nodes, {m:,} edges, half-load then slides of "
                        f"{step:,} inserts + {step:,} deletes; timed: the last steps of the 100-slide demo "
                        f"(e2e: the slides after it)",
            "graph": GRAPH, "nodes": n, "edges": m, "batch": 2 * step, "bfs_source": 0,
            "l2": "flushed (256 MiB write) before every timed step", "parallelism": "replicas"}


DEMO_SLIDES = 100  # slides between the demo's two searches (gpma_bfs_demo.cu:85-112)


def schedule(keys, num_slide=DEMO_SLIDES):
    """Slide i: insert keys[half + i*step ..], delete keys[i*step ..] (cyclic)."""
    m = len(keys)
    half = m // 2
    step = half // num_slide

    def slide(i):
        ins_idx = (half + i * step + np.arange(step)) % m
        del_idx = (i * step + np.arange(step)) % m
        k = np.concatenate([keys[ins_idx], keys[del_idx]])
        v = np.concatenate([np.ones(step, np.uint8), np.zeros(step, np.uint8)])
        return k, v

    return half, step, slide


def peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if d.get("hbm_gbs"):
            return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6.8 TB/s"


def profiled_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from a committed ncu summary, if any."""
    f = ROOT / "profiles" / f"{kernel}.social.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            return float(line.split(":", 1)[1].split()[0])
    return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        else:
            self.lines = []

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "0x1", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's figure; every rank calls it (NCCL on the GPUs, gloo
    with device="cpu")."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, time_s: float, world: int) -> float:
    """Whole-job throughput of N replicas: all ranks' units over the slowest
    rank's time (time_s already reduced with max_over_ranks)."""
    return units_per_rank * world / time_s


def bfs_counts(g, levels):
    """(edges traversed, algorithmic bytes) of a BFS: the live out-edges of the
    reached nodes (GTEPS numerator), and the HBM model 9 B x slots of every
    reached row + 8 B x reached nodes (their row_offset pair) + 4 B x nodes
    (level array) + 2 x nodes/8 B x levels (frontier bitmaps)."""
    keys, vals, ro = g.export_layout()
    valid = ((keys & np.uint64(0xFFFFFFFF)) != np.uint64(0xFFFFFFFF)) & (vals != 0)
    csum = np.concatenate([[0], np.cumsum(valid, dtype=np.int64)])
    ro = ro.astype(np.int64)
    per_row = csum[ro[1:]] - csum[ro[:-1]]
    reached = levels != 0
    n = len(levels)
    slots = int((ro[1:] - ro[:-1])[reached].sum())
    model = 9.0 * slots + 8.0 * int(reached.sum()) + 4.0 * n + 2.0 * (n / 8.0) * int(levels.max())
    return int(per_row[reached].sum()), model


class _DeviceArray:
    """A zero-copy view of library-owned device memory for torch.as_tensor."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


def live_out_degrees(G, g):
    """Live out-degree of every row, on the device (torch), read straight from
    the graph's arrays: for graphs too large to export."""
    import torch

    kp, vp, _ = g.device_arrays()
    size = g.get_size()
    keys = torch.as_tensor(_DeviceArray(kp, size, "<i8"), device="cuda")
    vals = torch.as_tensor(_DeviceArray(vp, size, "|u1"), device="cuda")
    src = keys >> 32
    ok = (vals != 0) & ((keys & 0xFFFFFFFF) != 0xFFFFFFFF) & (keys >= 0) & (src < g.row_num)
    deg = torch.bincount(src[ok], minlength=g.row_num)
    del keys, vals, src, ok
    return deg


def run_gpu(args):
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph

    t0 = time.time()
    n, src, dst = make_graph(GRAPH)
    keys = G.edges_to_keys(src, dst)
    m = len(keys)
    half, step, slide = schedule(keys)
    gen_s = time.time() - t0
    stream = torch.cuda.current_stream()
    g = G.GPMA(n, stream)
    G.update_gpma(g, keys[:half], np.ones(half, np.uint8), stream)
    g.set_profiling(True)

    def timed_bfs(repeats):
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        times = []
        reached = 0
        for _ in range(repeats):
            g.reset_profile()
            _, reached = G.gpma_bfs(g, n, m, 0, out, stream)
            times.append(g.profile()["bfs_ms"])
        levels = out.cpu().numpy().view(np.uint32)
        edges, model = bfs_counts(g, levels)
        ms = statistics.median(times)
        return {"reached": int(reached), "edges_traversed": edges, "ms": ms, "gteps": edges / (ms * 1e-3) / 1e9,
                "levels": int(levels.max()), "model_bytes": model}

    tuning = {}
    if not args.no_autotune:
        import gpma_bfs_gb300.autotune as T

        tuning["bfs"] = T.autotune({"bfs": T.bfs_probe(g, 0, torch.empty(n, dtype=torch.int32, device="cuda"))})["bfs"]
    bfs_before = timed_bfs(args.bfs_repeats)

    # the demo's 100 slides with the LAST K timed: deletes leave tombstones
    # until their window is redispatched, so a slide costs more as the window
    # ages (kernel ~0.13 ms over slides 0-19, ~0.17 ms over 40-59); the early
    # slides, and the W warm-up steps before the timed ones, run untimed
    total = max(DEMO_SLIDES, args.warmup + args.steps)
    first = total - args.steps
    for i in range(first - args.warmup):
        k, v = slide(i)
        G.update_gpma(g, k, v, stream)
    dk, dv = [], []
    for i in range(first - args.warmup, total):
        k, v = slide(i)
        dk.append(torch.from_numpy(k.view(np.int64)).cuda())
        dv.append(torch.from_numpy(v).cuda())
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for i in range(args.warmup):
        G.update_gpma(g, dk[i], dv[i], stream)

    st0 = g.stats()
    g.reset_profile()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for j in range(args.steps):
            flush.fill_(j & 0xFF)
            a, b = ev[j]
            a.record(stream)
            G.update_gpma(g, dk[args.warmup + j], dv[args.warmup + j], stream)
            b.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    prof = g.profile()
    st1 = g.stats()
    time_s = max_over_ranks(sum(step_ms) / 1e3, world)
    batch = 2 * step
    updates = batch * args.steps * world
    value = replica_value(batch * args.steps, time_s, world)
    accepted_slots = (st1["accepted_slots"] - st0["accepted_slots"]) / args.steps

    # roofline of the dominant kernel (the persistent update kernel):
    # algorithmic bytes per launch = 18 B x batch (read the batch, write it sorted)
    #                              + 18 B x slots of redispatched windows (read + write)
    upd_ms = prof["update_kernel_ms"] / max(1, prof["update_kernels"])
    upd_bytes = 18.0 * batch + 18.0 * accepted_slots
    peak, peak_src = peak_hbm()
    achieved = upd_bytes / (upd_ms * 1e-3) / 1e9
    traffic = profiled_traffic("update_kernel")
    step_bytes = 18.0 * batch + 18.0 * accepted_slots

    # BFS after the slides (the demo's second BFS)
    bfs_after = timed_bfs(args.bfs_repeats)
    analytics = run_analytics(G, g, n, stream)

    # e2e: next K slides through the C ABI from pinned host buffers
    hk, hv = [], []
    for i in range(total, total + args.steps):
        k, v = slide(i)
        hk.append(torch.from_numpy(k.view(np.int64)).pin_memory())
        hv.append(torch.from_numpy(v).pin_memory())
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for j in range(args.steps):
        flush.fill_(j & 0xFF)
        a, b = e2e_ev[j]
        a.record(stream)
        G.update_gpma(g, hk[j], hv[j], stream)
        b.record(stream)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(sum(a.elapsed_time(b) for a, b in e2e_ev) / 1e3, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(n, keys, half, slide, args.cpu_sample_steps, first)
    g.close()
    del dk, dv, hk, hv
    steps_report = run_steps(args, G, n, keys, half, slide, stream, flush)
    del keys
    batched = None
    if args.batched_graphs > 0:
        batched = run_batched(args, stream)
    served = None
    if args.served_seconds > 0:
        served = run_served(args, stream)
    large = None
    if args.large_graph and rank == 0:
        large = run_sweep(args, sizes=(100_000, 1_000_000, 10_000_000), ratios=((1, 1),), reps=2, bfs_sources=4)

    if rank == 0:
        bfs_roof = {"bound": "hbm", "kernel": "bfs_kernel", "unit": "GB/s", "peak": peak,
                    "bytes_per_launch": bfs_after["model_bytes"], "launch_ms": bfs_after["ms"],
                    "achieved": bfs_after["model_bytes"] / (bfs_after["ms"] * 1e-3) / 1e9,
                    "traffic": profiled_traffic("bfs_kernel")}
        bfs_roof["frac"] = bfs_roof["achieved"] / peak
        roofline = {"bound": "hbm", "kernel": "update_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_launch": upd_bytes,
                    "launch_ms": upd_ms, "peak_source": peak_src, "step_bytes": step_bytes,
                    "step_frac": step_bytes / (1e-3 * time_s * 1e3 / args.steps) / 1e9 / peak}
        phases = {"update_kernel": prof["update_kernel_ms"] / args.steps,
                  "in_kernel_sort": prof["sort_ms"] / args.steps,
                  "in_kernel_locate": prof["locate_ms"] / args.steps,
                  "in_kernel_group": prof["group_ms"] / args.steps,
                  "in_kernel_levels": prof["levels_ms"] / args.steps,
                  "root_rebuild": prof["rebuild_ms"] / args.steps}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * time_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": DATA,
            "config": workload_config(n, m, step),
            "roofline": roofline,
            "e2e": {"value": updates / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 9 * batch,
                    "d2h_bytes_per_step": 64},
            "gpu_launches": prof["kernel_launches"],
            "clocks": clk.summary(),
            "phases_ms_per_step": phases,
            "bfs": {"unit": "GTEPS", "gteps": bfs_after["gteps"], "gteps_before": bfs_before["gteps"],
                    "ms": bfs_after["ms"], "reached": bfs_after["reached"], "levels": bfs_after["levels"],
                    "roofline": bfs_roof},
        }
        if cpu:
            line["cpu_baseline"] = cpu
        line["update_bfs_step_ms"] = {"eager": steps_report["eager_ms"], "graph": steps_report["graph_ms"],
                                      "identical": steps_report["identical_levels"]}
        if batched:
            bu, bb = batched["update"], batched["bfs"]
            line["batched"] = {
                "graphs": batched["graphs"], "updates_per_step": batched["updates_per_step"],
                "updates_per_s": bu["batched_updates_per_s"], "plain_updates_per_s": bu["plain_updates_per_s"],
                "speedup_vs_plain": bu["speedup"], "roofline_frac": bu["roofline"]["frac"],
                "update_kernel_ms": bu["phases_ms_per_step"]["update_kernel_ms"],
                "bfs_gteps": bb["batched_gteps"], "plain_bfs_gteps": bb["plain_gteps"], "bfs_speedup": bb["speedup"],
                "identical_layouts": bu["identical_layouts"],
                "step_ms": {"eager": batched["update_bfs_steps"]["eager_ms"],
                            "graph": batched["update_bfs_steps"]["graph_ms"],
                            "identical": batched["update_bfs_steps"]["identical"]}}
            many = batched.get("recorded_steps")
            if many:
                line["batched"]["recorded_steps"] = {
                    "steps": many["steps"], "graph_launches": many["graph_launches"],
                    "graph_ms_per_step": many["graph_ms_per_step"], "eager_ms_per_step": many["eager_ms_per_step"],
                    "updates_per_s": many["updates_per_s"], "identical": many["identical"]}
        if served:
            light, sat = served["phases"][0], served["phases"][-1]

            def lat(ph, who):
                return {f"{k}_{q[:3]}_ms": (ph[who][f"{k}_latency"] or {}).get(q) for k in ("update", "bfs")
                        for q in ("p50_ms", "p99_ms")}

            line["served"] = {
                "graphs": served["graphs"], "requests": served["requests"], "failed": served["failed"],
                "identical_results": served["identical_results"], "lanes": served["lanes"],
                "max_inflight_rounds": served["server_stats"]["max_inflight_rounds"],
                "light_load": {"rate_per_s": light["rate_per_s"], "served": lat(light, "served"),
                               "plain": lat(light, "plain")},
                "saturation": {"rate_per_s": sat["rate_per_s"], "speedup_sustained": sat["speedup_sustained"],
                               "requests_per_s": sat["served"]["requests_per_s"],
                               "plain_requests_per_s": sat["plain"]["requests_per_s"],
                               "served": lat(sat, "served"), "plain": lat(sat, "plain")}}
        if large:
            line["large_graph"] = {
                "workload": large["config"]["workload"],
                "updates_per_s": {str(r["batch"]): r["edge_updates_per_s"] for r in large["updates"]},
                "kernel_hbm_frac": {str(r["batch"]): r["hbm_frac"] for r in large["updates"]},
                "bfs_gteps": large["bfs"]["gteps"], "multi_source_gteps": large["bfs"]["multi_gteps"],
                "load_edges_per_s": large["load"]["edges_per_s"]}
        report = dict(line)
        report.update({"roofline": roofline, "autotune": tuning or None, "analytics": analytics,
                       "bfs_detail": {"before": bfs_before, "after": bfs_after},
                       "levels_per_step": (st1["levels_visited"] - st0["levels_visited"]) / args.steps,
                       "setup_s": {"generate": gen_s}, "update_bfs_steps": steps_report,
                       "batched_detail": batched, "served_detail": served, "large_graph_detail": large})
        if args.report:
            Path(args.report).write_text(json.dumps(report, indent=1))
            line["report"] = str(args.report)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_steps(args, G, n, keys, half, slide, stream, flush):
    """The demo's loop body -- update_gpma of a slide batch, then BFS from
    node 0 -- on two copies of the half-loaded graph: one call after the other
    (eager) and as a recorded step replayed as one CUDA graph launch. Batches
    come from pinned host memory, levels stay on the device; every step's
    levels are compared between the two."""
    import torch

    ga, gb = G.GPMA(n, stream), G.GPMA(n, stream)
    ones = np.ones(half, np.uint8)
    G.update_gpma(ga, keys[:half], ones, stream)
    G.update_gpma(gb, keys[:half], ones, stream)
    step = G.Step(gb)
    total = args.warmup + args.steps
    hk, hv = [], []
    for i in range(total):
        k, v = slide(i)
        hk.append(torch.from_numpy(k.view(np.int64)).pin_memory())
        hv.append(torch.from_numpy(v).pin_memory())
    la = torch.empty(n, dtype=torch.int32, device="cuda")
    lb = torch.empty(n, dtype=torch.int32, device="cuda")
    same = True
    times = {"eager": [], "graph": []}
    for i in range(total):
        for name in ("eager", "graph"):
            flush.fill_(i & 0xFF)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if name == "eager":
                G.update_gpma(ga, hk[i], hv[i], stream)
                G.gpma_bfs(ga, n, 0, 0, la, stream)
            else:
                step.run(hk[i], hv[i], 0, lb, stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                times[name].append(time.perf_counter() - t0)
        same = same and bool(torch.equal(la, lb))
    st = step.stats()
    step.close()
    ga.close()
    gb.close()
    eager_ms = 1e3 * statistics.median(times["eager"])
    graph_ms = 1e3 * statistics.median(times["graph"])
    return {"workload": "slide batch from pinned host memory + BFS from node 0 per step, wall clock per step "
                        "(median), L2 flushed before each step",
            "steps": args.steps, "eager_ms": eager_ms, "graph_ms": graph_ms, "speedup": eager_ms / graph_ms,
            "identical_levels": same, "graph_builds": st["builds"], "param_updates": st["param_updates"],
            "host_runs": st["host_runs"], "graph_launches": st["graph_launches"]}


def run_analytics(G, g, n, stream):
    """PageRank (20 iterations, damping 0.85) and weakly connected components
    on the graph as the slides left it; both sweep every slot per iteration."""
    import torch

    geo = g.geometry()
    ranks = torch.empty(n, dtype=torch.float32, device="cuda")
    labels = torch.empty(n, dtype=torch.int32, device="cuda")
    G.pagerank(g, 0.85, 2, out=ranks, stream=stream)  # warm-up
    a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    _, iters = G.pagerank(g, 0.85, 20, out=ranks, stream=stream)
    c.record(stream)
    torch.cuda.synchronize()
    pr_ms = a.elapsed_time(c)
    a.record(stream)
    _, comps, rounds = G.components(g, labels, stream=stream)
    c.record(stream)
    torch.cuda.synchronize()
    cc_ms = a.elapsed_time(c)
    peak, _ = peak_hbm()
    sweep = 9.0 * geo["size"]  # keys + values read once per iteration
    per_iter = sweep + 16.0 * n  # + degree, rank, contribution, accumulator traffic per node
    return {"pagerank": {"iterations": iters, "ms": pr_ms, "ms_per_iteration": pr_ms / iters,
                         "hbm_frac": per_iter * iters / (pr_ms * 1e-3) / 1e9 / peak,
                         "note": "call time (CUDA events) incl. the initial ranks upload and the result copy; bytes = 9 B/slot + 16 B/node per iteration"},
            "components": {"components": comps, "rounds": rounds, "ms": cc_ms,
                           "hbm_frac": sweep * (rounds + 1) / (cc_ms * 1e-3) / 1e9 / peak}}


def run_batched(args, stream):
    """Batched configuration: many independent R-MAT graphs (edge counts
    log-uniform in [10k, 2M], ~edges/16 nodes), each updated every step by a
    sliding-window batch of log-uniform [100, 200k] keys (half inserts, half
    deletes), all graphs in ONE launch per step; then 64-source BFS on every
    graph in one launch. The plain drop-in (one gpma_update / gpma_bfs_multi
    per graph, same device-resident batches) is timed on the same stream."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    t0 = time.time()
    specs = batched_graphs(args.batched_graphs, seed=4)
    gen_s = time.time() - t0
    rng = np.random.default_rng(44)
    graphs_b = [G.GPMA(nn) for nn, _ in specs]  # batched form
    graphs_p = [G.GPMA(nn) for nn, _ in specs]  # plain drop-in, same stream of updates
    streams = [SlidingStream(kk) for _, kk in specs]
    streams_p = [SlidingStream(kk) for _, kk in specs]
    b = G.Batch()
    k = len(specs)
    loads = [s.load() for s in streams]
    off = np.concatenate([[0], np.cumsum([len(x[0]) for x in loads])]).astype(np.uint64)
    b.update_packed(graphs_b, np.concatenate([x[0] for x in loads]), np.concatenate([x[1] for x in loads]), off,
                    stream)
    for gp, sp in zip(graphs_p, streams_p):
        G.update_gpma(gp, *sp.load(), stream=stream)
    total_steps = args.warmup + args.batched_steps
    staged = []
    for _ in range(total_steps):
        sizes = np.exp(rng.uniform(np.log(100), np.log(200_000), k)).astype(np.int64)
        parts = [s.step(int(z)) for s, z in zip(streams, sizes)]
        for sp, z in zip(streams_p, sizes):
            sp.step(int(z))  # keep the plain copy's window in step (same batches)
        o = np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64)
        staged.append((torch.from_numpy(np.concatenate([p[0] for p in parts]).view(np.int64)).cuda(),
                       torch.from_numpy(np.concatenate([p[1] for p in parts])).cuda(), o))
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def timed(fn):
        flush.fill_(1)
        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        c.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(c)

    bt, pt, nupd = [], [], 0
    b.set_profiling(True)
    slots0 = 0
    for j, (dk, dv, o) in enumerate(staged):
        if j == args.warmup:
            b.reset_profile()
            slots0 = sum(x.stats()["accepted_slots"] for x in graphs_p)
        tb = timed(lambda: b.update_packed(graphs_b, dk, dv, o, stream))

        def plain():
            for i, gp in enumerate(graphs_p):
                lo, hi = int(o[i]), int(o[i + 1])
                G.update_gpma(gp, dk[lo:hi], dv[lo:hi], stream)

        tp = timed(plain)
        if j >= args.warmup:
            bt.append(tb)
            pt.append(tp)
            nupd += int(o[-1])
    # the two copies must agree (same batches, same algorithm)
    same = all(np.array_equal(x.export_layout()[0], y.export_layout()[0]) for x, y in zip(graphs_b, graphs_p))
    # phases of the batched launch (in-kernel stamps) and its roofline: the
    # plain copies ran the same windows, so their stats give the accepted slots
    prof = b.profile()
    steps_t = max(1, len(bt))
    slots = sum(x.stats()["accepted_slots"] for x in graphs_p) - slots0
    upd_bytes = 18.0 * nupd + 18.0 * slots
    peak, peak_src = peak_hbm()
    kern_s = prof["update_kernel_ms"] * 1e-3
    b_roof = {"bound": "hbm", "kernel": "update_kernel (256 graphs per launch)",
              "achieved": upd_bytes / kern_s / 1e9 if kern_s else None, "peak": peak, "unit": "GB/s",
              "frac": upd_bytes / kern_s / 1e9 / peak if kern_s else None,
              "algorithmic_bytes_per_launch": upd_bytes / steps_t, "peak_source": peak_src}
    b_phases = {k: prof[k] / steps_t for k in ("update_kernel_ms", "sort_ms", "locate_ms", "group_ms", "levels_ms",
                                               "rebuild_ms")}
    # 64-source BFS on every graph
    sources = []
    for (nn, kk) in specs:
        cand = np.unique((kk >> np.uint64(32)).astype(np.uint32))
        sources.append(rng.choice(cand, min(64, len(cand)), replace=False).astype(np.uint32))
    b.set_profiling(True)
    tuned = None
    if not args.no_autotune:
        import gpma_bfs_gb300.autotune as T

        tuned = T.autotune({"ms": T.ms_probe(b, graphs_b, sources)})["ms"]
    b.bfs_multi(graphs_b, sources)  # warm-up
    b.reset_profile()
    tbb = timed(lambda: b.bfs_multi(graphs_b, sources, stream=stream))
    edges_b = b.profile()["bfs_edges"]

    # the plain call writes 64 level arrays per graph: keep them on the device
    lv = torch.empty(64 * max(nn for nn, _ in specs), dtype=torch.int32, device="cuda")

    def plain_bfs():
        for gp, srcs in zip(graphs_p, sources):
            G.gpma_bfs_multi(gp, srcs, lv[: len(srcs) * gp.row_num].view(len(srcs), gp.row_num), stream=stream)

    plain_bfs()
    tpb = timed(plain_bfs)

    # recorded steps: each step's packed update of every graph and its 64-source
    # BFS, as the two eager calls on the batched copy and as one CUDA graph launch
    # (gpma_batch_step) on the plain copy, which holds the same layouts now
    b2 = G.Batch()
    rec = b2.step(graphs_p)
    te, tr, same_reached = [], [], True
    for j in range(args.warmup + args.batched_steps):
        sizes = np.exp(rng.uniform(np.log(100), np.log(200_000), k)).astype(np.int64)
        parts = [s.step(int(z)) for s, z in zip(streams, sizes)]
        for sp, z in zip(streams_p, sizes):
            sp.step(int(z))
        o = np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64)
        dk = torch.from_numpy(np.concatenate([p[0] for p in parts]).view(np.int64)).cuda()
        dv = torch.from_numpy(np.concatenate([p[1] for p in parts])).cuda()
        got = {}

        def eager():
            b.update_packed(graphs_b, dk, dv, o, stream)
            got["e"] = b.bfs_multi(graphs_b, sources, stream=stream)[1]

        def recorded():
            got["r"] = rec.run(dk, dv, o, sources, stream=stream)

        t_e, t_r = timed(eager), timed(recorded)
        same_reached = same_reached and all(np.array_equal(x, y) for x, y in zip(got["e"], got["r"]))
        if j >= args.warmup:
            te.append(t_e)
            tr.append(t_r)
    same_steps = same_reached and all(
        np.array_equal(x.export_layout()[0], y.export_layout()[0]) for x, y in zip(graphs_b, graphs_p))
    rec_stats = rec.stats()
    rec.close()

    # the same for S steps recorded in ONE graph launch (gpma_batch_step_run_many)
    # against S pairs of eager calls; the batches are device-resident up front
    S = args.graph_steps
    many = None
    if S > 1:
        ks, vs, offs = [], [], []
        for _ in range(S):
            sizes = np.exp(rng.uniform(np.log(100), np.log(200_000), k)).astype(np.int64)
            parts = [s.step(int(z)) for s, z in zip(streams, sizes)]
            for sp, z in zip(streams_p, sizes):
                sp.step(int(z))
            offs.append(np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64))
            ks.append(torch.from_numpy(np.concatenate([p[0] for p in parts]).view(np.int64)).cuda())
            vs.append(torch.from_numpy(np.concatenate([p[1] for p in parts])).cuda())
        rec_many = b2.step(graphs_p)
        got_e = []

        def eager_many():
            for t in range(S):
                b.update_packed(graphs_b, ks[t], vs[t], offs[t], stream)
                got_e.append(b.bfs_multi(graphs_b, sources, stream=stream)[1])

        got_r = {}

        def recorded_many():
            got_r["r"] = rec_many.run_many(ks, vs, offs, sources, stream=stream)

        t_em, t_rm = timed(eager_many), timed(recorded_many)
        same_many = all(all(np.array_equal(x, y) for x, y in zip(got_e[t], got_r["r"][t])) for t in range(S)) and all(
            np.array_equal(x.export_layout()[0], y.export_layout()[0]) for x, y in zip(graphs_b, graphs_p))
        ms_stats = rec_many.stats()
        rec_many.close()
        n_many = int(sum(int(o[-1]) for o in offs))
        many = {"steps": S, "graph_ms_per_step": t_rm / S, "eager_ms_per_step": t_em / S,
                "updates_per_s": n_many / (t_rm * 1e-3), "identical": same_many,
                "graph_launches": ms_stats["graph_launches"], "graph_builds": ms_stats["builds"],
                "host_runs": ms_stats["host_runs"]}
        del ks, vs
    b2.close()
    b.close()
    total_edges = int(sum(len(kk) for _, kk in specs))
    for x in graphs_b + graphs_p:
        x.close()
    sb, sp_ = sum(bt) / 1e3, sum(pt) / 1e3
    return {
        "workload": f"{k} R-MAT graphs, edges log-uniform [10k, 2M] (~edges/16 nodes), sliding-window batches "
                    f"log-uniform [100, 200k] keys per graph per step (1:1 insert:delete), 64-source BFS per graph",
        "graphs": k, "edges_total": total_edges, "half_loaded": int(off[-1]), "steps": len(bt),
        "updates_per_step": nupd / max(1, len(bt)),
        "update": {"batched_updates_per_s": nupd / sb, "batched_ms_per_step": 1e3 * sb / len(bt),
                   "plain_updates_per_s": nupd / sp_, "plain_ms_per_step": 1e3 * sp_ / len(pt),
                   "speedup": sp_ / sb, "identical_layouts": same,
                   "phases_ms_per_step": b_phases, "roofline": b_roof},
        "bfs": {"sources_per_graph": 64, "edges_traversed": edges_b, "autotune": tuned,
                "batched_ms": tbb, "batched_gteps": edges_b / (tbb * 1e-3) / 1e9,
                "plain_ms": tpb, "plain_gteps": edges_b / (tpb * 1e-3) / 1e9, "speedup": tpb / tbb},
        "update_bfs_steps": {"eager_ms": statistics.median(te), "graph_ms": statistics.median(tr),
                             "identical": same_steps, "graph_launches": rec_stats["graph_launches"],
                             "graph_builds": rec_stats["builds"], "host_runs": rec_stats["host_runs"]},
        "recorded_steps": many,
        "setup_s": {"generate": gen_s},
    }


def run_served(args, stream):
    """Served configuration: 32 R-MAT graphs drawn as in the batched one plus
    two R-MAT graphs of scale 22 (edge factor 16), first halves resident;
    Poisson arrivals, 70% update batches (log-uniform 1k-1M keys, sliding
    window, 1:1 insert:delete) and 30% BFS queries (1-64 sources from nodes
    with out-edges), each on a uniformly drawn graph; HBM admission budget
    120 GB. The server runs its native serving loop in real time with
    `served_lanes` rounds in flight (continuous batching: a round starts as
    soon as a request has arrived and a lane is free); the trace's arrivals
    are seconds on the server's clock. The plain drop-in serves the same trace
    one request at a time (gpma_update / gpma_bfs_multi per request, FIFO) on
    its own copy of the graphs, each request starting at max(its arrival, the
    previous one's completion) and taking its measured wall time.
    Latency = completion - arrival."""
    import torch

    import gpma_bfs_gb300 as G
    import gpma_bfs_gb300.serving as S
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    t0 = time.time()
    specs = batched_graphs(32, seed=5)
    for i in range(2):
        src, dst = G.gen_rmat(args.served_big_scale, 16, seed=5_000 + i)
        specs.append((1 << args.served_big_scale, G.edges_to_keys(src, dst)))
        del src, dst
    gen_s = time.time() - t0
    phases = [(args.served_rate, args.served_seconds)]
    if args.served_burst_seconds > 0:
        phases.append((args.served_burst_rate, args.served_burst_seconds))
    trace = S.make_trace(specs, phases, seed=5)

    # ---- served form ----------------------------------------------------------
    srv = G.Server(hbm_budget_bytes=120 << 30, max_round_keys=1 << 24, max_queued_keys=1 << 40, stream=stream,
                   lanes=args.served_lanes, input_ring_bytes=4 << 30)
    gids = [srv.add_graph(nn, len(kk)) for nn, kk in specs]
    streams = [SlidingStream(kk) for _, kk in specs]
    t0 = time.time()
    for gid, s in zip(gids, streams):
        G.update_gpma(srv.graph(gid), *s.load(), stream=stream)
    torch.cuda.synchronize()
    load_s = time.time() - t0
    w0 = time.perf_counter()
    out = S.replay_served_live(srv, gids, streams, trace)
    served_wall = time.perf_counter() - w0
    layouts_s = [srv.graph(gid).export_layout()[0] for gid in gids]
    committed = srv.committed_bytes()
    stats = out["stats"]
    srv.close()
    del streams

    # ---- plain drop-in, one request at a time ------------------------------------
    plain, pstreams = S.plain_graphs(specs, stream)
    lv = torch.empty(64 * max(nn for nn, _ in specs), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    done_p, busy_p, reach_p = S.replay_plain(plain, pstreams, trace, stream, lv, torch.cuda.synchronize)
    same_reach = all(np.array_equal(a, b) for a, b, k in zip(out["reach"], reach_p, trace.kind) if k == 1)
    same_layout = all(np.array_equal(x.export_layout()[0], y) for x, y in zip(plain, layouts_s))
    for g in plain:
        g.close()

    # per phase: sustained rates over the phase's makespan, latency per type
    res = []
    for p, (rate, seconds) in enumerate(phases):
        sel = trace.phase == p
        upd = sel & (trace.kind == 0)
        keys = int(out["keys"][upd].sum())
        t_start = trace.phase_start[p]
        span_s = float(out["done"][sel].max() - t_start) if sel.any() else 0.0
        span_p = float(done_p[sel].max() - t_start) if sel.any() else 0.0
        busy_pl = float(busy_p[sel].sum())

        def rates(span):
            return {"requests_per_s": int(sel.sum()) / span if span else None,
                    "edge_updates_per_s": keys / span if span else None}

        res.append({
            "rate_per_s": rate, "seconds": seconds, "requests": int(sel.sum()), "updates": int(upd.sum()),
            "bfs_queries": int((sel & (trace.kind == 1)).sum()), "update_keys": keys,
            "served": {"rounds": int(len(np.unique(out["round"][sel]))), "makespan_s": span_s, **rates(span_s),
                       "update_latency": S.latency_summary(trace, out["done"], p, 0),
                       "bfs_latency": S.latency_summary(trace, out["done"], p, 1)},
            "plain": {"busy_s": busy_pl, "makespan_s": span_p, "utilisation": busy_pl / seconds, **rates(span_p),
                      "update_latency": S.latency_summary(trace, done_p, p, 0),
                      "bfs_latency": S.latency_summary(trace, done_p, p, 1)},
            "speedup_sustained": span_p / span_s if span_s else None,
        })
    # the light phase's slowest served requests (kind, keys or sources, latency, wait before its round)
    light = np.nonzero(trace.phase == 0)[0]
    lat = out["done"][light] - trace.arrival[light]
    slow = [{"kind": "update" if trace.kind[i] == 0 else "bfs", "graph": int(trace.graph[i]),
             "size": int(out["keys"][i]) if trace.kind[i] == 0 else int(len(trace.sources[i])),
             "arrival_s": float(trace.arrival[i]), "latency_ms": 1e3 * float(out["done"][i] - trace.arrival[i]),
             "wait_ms": 1e3 * float(out["start"][i] - trace.arrival[i]), "plain_ms": 1e3 * float(busy_p[i])}
            for i in light[np.argsort(-lat)[:12]]]
    return {
        "slowest_light": slow,
        "workload": f"32 R-MAT graphs (edges log-uniform [10k, 2M]) + 2 R-MAT scale {args.served_big_scale} "
                    f"(edge factor 16); Poisson arrivals, 70% updates (log-uniform 1k-1M keys, 1:1 "
                    f"insert:delete), 30% BFS (1-64 sources), uniform graph choice; HBM budget 120 GB; "
                    f"native serving loop, {args.served_lanes} lanes, real time; phases "
                    + ", ".join(f"{r:g}/s for {s:g} s" for r, s in phases),
        "graphs": len(specs), "edges_total": int(sum(len(kk) for _, kk in specs)), "requests": len(trace),
        "failed": int((~out["ok"]).sum()), "committed_bytes": int(committed),
        "lanes": args.served_lanes, "server_stats": stats,
        "phases": res,
        "identical_results": bool(same_reach and same_layout),
        "driver_wall_s": served_wall,
        "setup_s": {"generate": gen_s, "load": load_s},
    }


SWEEP_SIZES = (1_000, 10_000, 100_000, 1_000_000, 10_000_000)
SWEEP_RATIOS = ((1, 0), (1, 1), (0, 1))


def run_sweep(args, sizes=SWEEP_SIZES, ratios=SWEEP_RATIOS, reps=None, bfs_sources=16):
    """Large single graph + batch sweep: R-MAT scale `sweep_scale` (edge factor
    `sweep_edge_factor`, a/b/c = .57/.19/.19, seed 3, deduplicated, shuffled)
    loaded except for a reserve of fresh edges; then, per insert:delete ratio
    (1:0, 1:1, 0:1) and batch size (1k ... 10M), `sweep_reps` batches of fresh
    inserts and uniformly drawn existing edges to delete, each timed alone
    (device-resident batch, L2 flushed, CUDA events); then BFS from 16 random
    non-isolated sources (one search each, and all 16 as lanes of one
    multi-source search). The default bench run takes a subset: batches of
    100k, 1M and 10M keys at 1:1, two each, BFS from 4 sources."""
    import torch

    import gpma_bfs_gb300 as G

    stream = torch.cuda.current_stream()
    t0 = time.time()
    src, dst = G.gen_rmat(args.sweep_scale, args.sweep_edge_factor, seed=3)
    n = 1 << args.sweep_scale
    keys = G.edges_to_keys(src, dst)
    del src, dst
    m = len(keys)
    gen_s = time.time() - t0
    reps = reps or args.sweep_reps
    # batch sizes the graph can feed (fresh inserts and distinct deletes)
    sizes = [s for s in sizes if 2 * reps * s <= m // 4]
    reserve = sum(reps * s * i // (i + d) for s in sizes for i, d in ratios) + 1
    loaded = keys[: m - reserve]
    fresh = keys[m - reserve:]
    rng = np.random.default_rng(3)
    del_order = rng.permutation(len(loaded))  # deletes: uniformly drawn, each live edge at most once
    g = G.GPMA(n, stream)
    t0 = time.time()
    chunk = 1 << 26
    for i in range(0, len(loaded), chunk):
        part = torch.from_numpy(loaded[i:i + chunk].view(np.int64)).cuda()
        G.update_gpma(g, part, torch.ones(len(part), dtype=torch.uint8, device="cuda"), stream)
        del part
    torch.cuda.synchronize()
    load_s = time.time() - t0
    geo = g.geometry()
    live = len(loaded) + n + 2
    g.set_profiling(True)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    fi = di = 0
    rows = []
    peak, _ = peak_hbm()
    for ins, dels in ratios:
        for size in sizes:
            times, kern, slots = [], [], []
            for _ in range(reps):
                ni = size * ins // (ins + dels)
                nd = size - ni
                k = np.concatenate([fresh[fi:fi + ni], loaded[del_order[di:di + nd]]])
                v = np.concatenate([np.ones(ni, np.uint8), np.zeros(nd, np.uint8)])
                fi += ni
                di += nd
                live += ni - nd
                dk = torch.from_numpy(k.view(np.int64)).cuda()
                dv = torch.from_numpy(v).cuda()
                flush.fill_(1)
                s0 = g.stats()["accepted_slots"]
                g.reset_profile()
                a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                G.update_gpma(g, dk, dv, stream)
                c.record(stream)
                torch.cuda.synchronize()
                times.append(a.elapsed_time(c))
                p = g.profile()
                kern.append(p["update_kernel_ms"] + p["rebuild_ms"])
                slots.append(g.stats()["accepted_slots"] - s0)
            ms = statistics.median(times)
            kms = statistics.median(kern)
            bytes_ = 18.0 * size + 18.0 * statistics.median(slots)
            rows.append({"ratio": f"{ins}:{dels}", "batch": size, "ms": ms, "edge_updates_per_s": size / (ms * 1e-3),
                         "kernel_ms": kms, "hbm_frac": bytes_ / (kms * 1e-3) / 1e9 / peak if kms else None})
    # BFS from random non-isolated sources (live out-degree per row, once, on the device)
    deg = live_out_degrees(G, g)
    cand = torch.nonzero(deg > 0).flatten().cpu().numpy()
    sources = rng.choice(cand, bfs_sources, replace=False).astype(np.uint32)
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    single = []
    for s in sources:
        g.reset_profile()
        G.gpma_bfs(g, n, live, int(s), out, stream)
        hit = out != 0
        single.append((g.profile()["bfs_ms"], int(deg[hit].sum()), int(hit.sum())))
    g.reset_profile()
    lvm = torch.empty(len(sources) * n, dtype=torch.int32, device="cuda")
    G.gpma_bfs_multi(g, sources, lvm.view(len(sources), n), stream=stream)
    pm = g.profile()
    del deg, lvm
    bfs_ms = statistics.median(x[0] for x in single)
    edges = statistics.median(x[1] for x in single)
    g.close()
    return {
        "metric": "edge updates/s and BFS GTEPS, large single graph", "impl": "gpma",
        "config": {"workload": f"R-MAT scale {args.sweep_scale}, edge factor {args.sweep_edge_factor}, "
                               f"{m:,} edges after dedup, {len(loaded):,} loaded, batches of "
                               + "/".join(f"{z:,}" for z in sizes) + " keys at "
                               + " / ".join(f"{i}:{d}" for i, d in ratios)
                               + f", {reps} each, BFS from {len(sources)} random non-isolated sources",
                   "l2": "flushed before every timed update"},
        "geometry": geo, "density_after_load": (len(loaded) + n + 2) / geo["size"],
        "load": {"edges": len(loaded), "seconds": load_s, "edges_per_s": len(loaded) / load_s},
        "updates": rows,
        "bfs": {"single_source_median_ms": bfs_ms, "median_edges": edges,
                "gteps": edges / (bfs_ms * 1e-3) / 1e9,
                "reached": [x[2] for x in single],
                "multi_ms": pm["bfs_ms"], "multi_gteps": pm["bfs_edges"] / (pm["bfs_ms"] * 1e-3) / 1e9},
        "setup_s": {"generate": gen_s},
    }


def run_profile_case(args):
    """Small cases for ncu captures (one JSON line each, not a bench line):
    `bulk`: R-MAT scale --profile-scale (edge factor 32) loaded in 64M-key
    batches, then one batch of 10M fresh inserts (the >= 5M bulk rebuild);
    `batched`: the batched configuration's 256 graphs loaded, then four
    packed sliding-window steps."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    torch.cuda.set_device(0)
    out = {"case": args.profile_case}
    if args.profile_case == "bulk":
        src, dst = G.gen_rmat(args.profile_scale, 32, seed=3)
        keys = G.edges_to_keys(src, dst)
        del src, dst
        fresh, loaded = keys[len(keys) - 10_000_000:], keys[: len(keys) - 10_000_000]
        g = G.GPMA(1 << args.profile_scale)
        for i in range(0, len(loaded), 1 << 26):
            part = torch.from_numpy(loaded[i:i + (1 << 26)].view(np.int64)).cuda()
            G.update_gpma(g, part, torch.ones(len(part), dtype=torch.uint8, device="cuda"))
        dk = torch.from_numpy(fresh.view(np.int64)).cuda()
        dv = torch.ones(len(fresh), dtype=torch.uint8, device="cuda")
        g.set_profiling(True)
        g.reset_profile()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        G.update_gpma(g, dk, dv)
        b.record()
        torch.cuda.synchronize()
        p = g.profile()
        out.update(loaded=len(loaded), geometry=g.geometry(), batch_ms=a.elapsed_time(b),
                   update_kernel_ms=p["update_kernel_ms"], rebuild_ms=p["rebuild_ms"])
        g.close()
    else:
        specs = batched_graphs(256, seed=4)
        graphs = [G.GPMA(nn) for nn, _ in specs]
        streams = [SlidingStream(kk) for _, kk in specs]
        b = G.Batch()
        loads = [s.load() for s in streams]
        off = np.concatenate([[0], np.cumsum([len(x[0]) for x in loads])]).astype(np.uint64)
        b.update_packed(graphs, np.concatenate([x[0] for x in loads]), np.concatenate([x[1] for x in loads]), off)
        rng = np.random.default_rng(44)
        b.set_profiling(True)
        steps = []
        for _ in range(4):
            sizes = np.exp(rng.uniform(np.log(100), np.log(200_000), len(specs))).astype(np.int64)
            parts = [s.step(int(z)) for s, z in zip(streams, sizes)]
            o = np.concatenate([[0], np.cumsum([len(q[0]) for q in parts])]).astype(np.uint64)
            dk = torch.from_numpy(np.concatenate([q[0] for q in parts]).view(np.int64)).cuda()
            dv = torch.from_numpy(np.concatenate([q[1] for q in parts])).cuda()
            b.reset_profile()
            b.update_packed(graphs, dk, dv, o)
            steps.append({"keys": int(o[-1]), **{k: v for k, v in b.profile().items() if k.endswith("_ms")}})
        out["steps"] = steps
        b.close()
        for x in graphs:
            x.close()
    print(json.dumps(out), flush=True)


def cpu_baseline(n, keys, half, slide, steps, first=0):
    """The oracle restatement on all host cores: load and slides [0, first)
    untimed, then `steps` slides timed (the GPU arm's timed slides start at
    `first` too)."""
    from oracle.oracle import OracleGPMA, build

    build()
    cores = os.cpu_count() or 1
    o = OracleGPMA(n, threads=cores)
    o.update(keys[:half], np.ones(half, np.uint8))
    for i in range(first):
        o.update(*slide(i))
    t = 0.0
    batch = 0
    for i in range(first, first + steps):
        k, v = slide(i)
        t0 = time.perf_counter()
        o.update(k, v)
        t += time.perf_counter() - t0
        batch = len(k)
    # the next slides on one core (the reference's own CPU baseline program is single-threaded)
    o.set_threads(1)
    one_steps = min(steps, 3)
    t1 = 0.0
    for i in range(first + steps, first + steps + one_steps):
        k, v = slide(i)
        t0 = time.perf_counter()
        o.update(k, v)
        t1 += time.perf_counter() - t0
    o.close()
    return {"value": steps * batch / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} slide updates of {batch:,} keys (slides {first}..{first + steps - 1}) after an "
                      f"untimed load of {half:,} edges and the earlier slides (same graph), OpenMP on {cores} threads",
            "single_core": {"value": one_steps * batch / t1, "unit": UNIT, "cores": 1,
                            "sample": f"the next {one_steps} slide updates on one thread"}}


def run_reference(args):
    """The reference algorithm (the oracle's restatement of GPMA<CPU>) on all
    host cores. Loads only oracle/ libraries: the graph comes from the same
    generator source built into oracle/_build/libgraphgen.so."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    from oracle.oracle import OracleGPMA, build, gen_chung_lu

    build()
    n = SOCIAL["n"]
    src, dst = gen_chung_lu(**SOCIAL)
    keys = (src.astype(np.uint64) << np.uint64(32)) + dst.astype(np.uint64)
    del src, dst
    half, step, slide = schedule(keys)
    cores = os.cpu_count() or 1
    o = OracleGPMA(n, threads=cores)
    o.update(keys[:half], np.ones(half, np.uint8))
    # the GPU arm's timed slides: the last K of the 100-slide demo
    total = max(DEMO_SLIDES, args.warmup + args.steps)
    first = total - args.steps
    for i in range(first):
        o.update(*slide(i))
    t = 0.0
    for j in range(args.steps):
        k, v = slide(first + j)
        t0 = time.perf_counter()
        o.update(k, v)
        t += time.perf_counter() - t0
    value = 2 * step * args.steps / t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": DATA, "config": workload_config(n, len(keys), step), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} timed slide updates of {2 * step:,} keys (slides {first}.."
                                   f"{total - 1}) after an untimed load of {half:,} edges and the earlier slides"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gpma", "reference"], default="gpma")
    ap.add_argument("--bfs-repeats", type=int, default=3)
    ap.add_argument("--cpu-sample-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the built-in tuning (no sweep before timing)")
    ap.add_argument("--batched-graphs", type=int, default=256, help="graphs of the batched configuration (0: skip)")
    ap.add_argument("--batched-steps", type=int, default=5)
    ap.add_argument("--graph-steps", type=int, default=50,
                    help="batched steps recorded in one CUDA graph launch, against as many eager steps (0/1: skip)")
    ap.add_argument("--served-seconds", type=float, default=30.0,
                    help="seconds of served traffic at the light rate, in real time (0: skip the served configuration)")
    ap.add_argument("--served-rate", type=float, default=20.0, help="served request arrivals per second (light load)")
    ap.add_argument("--served-lanes", type=int, default=2, help="rounds the server keeps in flight")
    ap.add_argument("--served-big-scale", type=int, default=22, help="R-MAT scale of the two large served graphs")
    ap.add_argument("--served-burst-rate", type=float, default=20000.0,
                    help="arrivals per second of the saturating phase that follows")
    ap.add_argument("--served-burst-seconds", type=float, default=0.25)
    ap.add_argument("--sweep", action="store_true",
                    help="only the large-graph batch sweep (R-MAT scale 24, edge factor 32): its own JSON line")
    ap.add_argument("--sweep-scale", type=int, default=24)
    ap.add_argument("--sweep-edge-factor", type=int, default=32)
    ap.add_argument("--sweep-reps", type=int, default=3)
    ap.add_argument("--no-large-graph", dest="large_graph", action="store_false",
                    help="skip the large-graph subset (R-MAT scale 24: 100k/1M/10M batches at 1:1, BFS) of the "
                         "default run")
    ap.add_argument("--profile-case", choices=["bulk", "batched"],
                    help="only a small case for ncu captures (its own JSON line, not a bench line)")
    ap.add_argument("--profile-scale", type=int, default=21, help="R-MAT scale of the bulk profile case")
    ap.add_argument("--report", default=str(ROOT / "bench_report.json"),
                    help="file for the full sub-reports ('' for none)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.profile_case:
        run_profile_case(args)
    elif args.sweep:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(run_sweep(args)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
