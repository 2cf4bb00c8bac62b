"""Served-form traffic: request traces and their replay.

``make_trace`` draws Poisson arrivals of update batches and BFS queries over
resident graphs, in phases of (rate, seconds). ``replay_served`` feeds a trace
to a ``Server`` (continuous batching: every request that has arrived by the
current virtual time is submitted, then one round runs and the clock advances
by its measured wall time; an idle server jumps to the next arrival).
``replay_plain`` serves the same trace one request at a time through the
plain drop-in calls (``update_gpma`` / ``gpma_bfs_multi``), FIFO, on its own
graphs, with the same clock rule. Both return per-request completion times
and BFS reach, so results and latencies can be compared request by request.
``replay_served_live`` replays a trace in real time through the server's
native serving loop (worker threads per lane on the server's clock).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import ERR_BUSY, GPMA, GPMAError, Server, gpma_bfs_multi, update_gpma
from .workloads import SlidingStream


@dataclass
class Trace:
    arrival: np.ndarray      # float64 seconds, non-decreasing
    kind: np.ndarray         # 0 update, 1 BFS
    graph: np.ndarray        # graph index
    size: np.ndarray         # update: requested batch size (inserts + deletes)
    sources: list            # BFS: uint32 source arrays (None for updates)
    phase: np.ndarray        # phase index of each request
    phase_start: list        # virtual start of each phase

    def __len__(self):
        return len(self.arrival)


def make_trace(specs, phases, seed=5, update_share=0.7, min_batch=1_000, max_batch=1_000_000, max_sources=64):
    """Phases of Poisson arrivals (rate per second, seconds), back to back.
    Each request picks a graph uniformly; updates have log-uniform sizes in
    [min_batch, max_batch], searches 1..max_sources distinct sources among the
    graph's nodes with out-edges."""
    rng = np.random.default_rng(seed)
    cands = [np.unique((k >> np.uint64(32)).astype(np.uint32)) for _, k in specs]
    arr, ph, starts, t0 = [], [], [], 0.0
    for p, (rate, seconds) in enumerate(phases):
        c = int(rng.poisson(rate * seconds))
        arr.append(t0 + np.sort(rng.uniform(0.0, seconds, c)))
        ph.append(np.full(c, p, np.int32))
        starts.append(t0)
        t0 += seconds
    arrival = np.concatenate(arr) if arr else np.zeros(0)
    count = len(arrival)
    kind = (rng.random(count) >= update_share).astype(np.int8)
    graph = rng.integers(0, len(specs), count)
    size = np.exp(rng.uniform(np.log(min_batch), np.log(max_batch), count)).astype(np.int64)
    nsrc = rng.integers(1, max_sources + 1, count)
    sources = [rng.choice(cands[g], min(int(nsrc[i]), len(cands[g])), replace=False).astype(np.uint32)
               if kind[i] else None for i, g in enumerate(graph)]
    return Trace(arrival, kind, graph, size, sources, np.concatenate(ph) if ph else np.zeros(0, np.int32), starts)


def replay_served(srv: Server, gids, streams, trace: Trace):
    """dict of per-request arrays (done time, ok, update keys, BFS reach) and
    the rounds (each with the trace indices of its requests)."""
    n = len(trace)
    ids = []
    rounds = []
    now, j = 0.0, 0
    held = None  # a request the server refused as busy: retried after the next round
    while j < n or srv.queued()[0]:
        while j < n and trace.arrival[j] <= now:
            g = int(trace.graph[j])
            try:
                if trace.kind[j] == 0:
                    k, v = held if held is not None else streams[g].step(int(trace.size[j]))
                    ids.append(srv.submit_update(gids[g], k, v, float(trace.arrival[j])))
                else:
                    ids.append(srv.submit_bfs(gids[g], trace.sources[j], float(trace.arrival[j])))
            except GPMAError as e:
                if e.status != ERR_BUSY or srv.queued()[0] == 0:
                    raise  # not busy, or larger than the whole queue: never admissible
                held = (k, v) if trace.kind[j] == 0 else None
                break  # admission control: wait for a round to free queue slots
            held = None
            j += 1
        r = srv.run_round(now)
        if r["updates"] + r["bfs_requests"] + r["failed"]:
            r["ids"] = srv.last_round()
            rounds.append(r)
            now += r["seconds"]
        elif j < n:
            now = max(now, float(trace.arrival[j]))
    infos = [srv.poll(i, release=True) for i in ids]
    index = {i: x for x, i in enumerate(ids)}
    for r in rounds:
        r["requests"] = [index[i] for i in r.pop("ids")]
    return {"done": np.array([x["done"] for x in infos]), "ok": np.array([x["state"] == 1 for x in infos]),
            "keys": np.array([x["keys"] for x in infos], np.int64), "reach": [x["reached"] for x in infos],
            "rounds": rounds}


def replay_served_live(srv: Server, gids, streams, trace: Trace, timeout: float = 600.0):
    """The trace in real time through the server's native serving loop:
    every request is submitted in arrival order with its arrival on the
    server's clock, ahead of time -- as many as the queue limits take before
    the loop starts (clock 0), the rest while it runs (ERR_BUSY holds the
    submitter back) -- and runs once the clock has passed its arrival, in a
    round of whichever lane is free. Returns per-request arrays as
    replay_served does, plus the server's round totals."""
    n = len(trace)
    ids = []
    started = False
    try:
        j = 0
        held = None
        while j < n:
            g = int(trace.graph[j])
            try:
                if trace.kind[j] == 0:
                    k, v = held if held is not None else streams[g].step(int(trace.size[j]))
                    ids.append(srv.submit_update(gids[g], k, v, float(trace.arrival[j])))
                else:
                    ids.append(srv.submit_bfs(gids[g], trace.sources[j], float(trace.arrival[j])))
            except GPMAError as e:
                if e.status != ERR_BUSY:
                    raise
                held = (k, v) if trace.kind[j] == 0 else None
                if not started:
                    srv.start()
                    started = True
                time.sleep(0.0005)  # the queue is full: rounds free its slots
                continue
            held = None
            j += 1
        if not started:
            srv.start()
            started = True
        srv.drain(timeout)
    finally:
        if started:
            srv.stop()
    infos = [srv.poll(i, release=True) for i in ids]
    return {"done": np.array([x["done"] for x in infos]), "start": np.array([x["start"] for x in infos]),
            "ok": np.array([x["state"] == 1 for x in infos]), "round": np.array([x["round"] for x in infos]),
            "keys": np.array([x["keys"] for x in infos], np.int64), "reach": [x["reached"] for x in infos],
            "stats": srv.stats()}


def replay_plain(graphs: list[GPMA], streams, trace: Trace, stream=None, level_buffer=None, sync=None):
    """One request at a time, FIFO. level_buffer: device int32 tensor of at
    least 64 x max(row_num) entries for the search levels (host arrays are
    used when omitted); sync: callable that waits for the stream."""
    n = len(trace)
    done = np.zeros(n)
    busy = np.zeros(n)
    reach = [None] * n
    now = 0.0
    for j in range(n):
        now = max(now, float(trace.arrival[j]))
        g = int(trace.graph[j])
        if trace.kind[j] == 0:
            k, v = streams[g].step(int(trace.size[j]))
            a = time.perf_counter()
            update_gpma(graphs[g], k, v, stream)
            if sync:
                sync()
        else:
            s = trace.sources[j]
            out = None
            if level_buffer is not None:
                rows = graphs[g].row_num
                out = level_buffer[: len(s) * rows].view(len(s), rows)
            a = time.perf_counter()
            _, reach[j] = gpma_bfs_multi(graphs[g], s, out, stream=stream)
        dt = time.perf_counter() - a
        busy[j] = dt
        now += dt
        done[j] = now
    return done, busy, reach


def latency_summary(trace: Trace, done: np.ndarray, phase: int, kind: int):
    sel = (trace.phase == phase) & (trace.kind == kind)
    lat = (done - trace.arrival)[sel]
    if not len(lat):
        return None
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "count": int(len(lat))}


def plain_graphs(specs, stream=None):
    """Fresh plain-API copies of the graphs with their first halves loaded,
    and their sliding streams."""
    graphs, streams = [], []
    for n, k in specs:
        g = GPMA(n, stream)
        s = SlidingStream(k)
        update_gpma(g, *s.load(), stream)
        graphs.append(g)
        streams.append(s)
    return graphs, streams
