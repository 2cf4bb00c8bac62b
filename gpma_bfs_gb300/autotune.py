"""Autotuner for the launch shapes and switch points (``gpma_set_tuning``).

The PMA geometry (segment length, tree height, array size) is fixed by the
reference's sizing rules and is not tuned: changing it would change the
layout. What is tuned only changes speed: grid shapes (CTAs per SM) of the
persistent kernels and the frontier size at which a BFS level switches from
walking frontier rows to sweeping the whole slot array.

A probe is a callable that runs one operation and returns
``(milliseconds, digest)``: its device time and a digest of its result. For
every group of parameters the tuner times each candidate (median of
``repeats`` runs), rejects any candidate whose digest differs from the
current setting's (the switch must never change results), and keeps the
fastest. Groups are tuned one after another, each with the others' best.
"""
from __future__ import annotations

import hashlib
import json
import statistics
from dataclasses import dataclass, field

import numpy as np

from . import GPMA, Batch, get_tuning, gpma_bfs, set_tuning

SPACE = {
    "bfs": {"bfs_blocks_per_sm": (4, 8), "bfs_dense_div": (0, 2, 3, 4, 6, 8)},
    "ms": {"ms_blocks_per_sm": (4, 8), "ms_dense_div": (0, 2, 3, 4, 8, 16)},
    "update": {"update_blocks_per_sm": (2, 3)},
}


def digest(*arrays) -> str:
    h = hashlib.sha1()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@dataclass
class GroupResult:
    group: str
    best: dict
    best_ms: float
    default_ms: float
    trials: list = field(default_factory=list)  # (setting, median ms, digest ok)


def _grid(space: dict):
    keys = list(space)
    combos = [{}]
    for k in keys:
        combos = [dict(c, **{k: v}) for c in combos for v in space[k]]
    return combos


def tune_group(group: str, probe, repeats: int = 3, space: dict | None = None) -> GroupResult:
    """Tunes one parameter group with `probe`; leaves the best setting in force."""
    space = space or SPACE[group]
    base = get_tuning()
    ref_ms, ref_digest = [], None
    for _ in range(repeats):
        ms, d = probe()
        ref_ms.append(ms)
        ref_digest = ref_digest or d
        if d != ref_digest:
            raise RuntimeError(f"{group}: the probe is not deterministic at the current setting")
    default_ms = statistics.median(ref_ms)
    best, best_ms = {k: base[k] for k in space}, default_ms
    trials = []
    try:
        for cand in _grid(space):
            set_tuning(**dict(base, **cand))
            times, ok = [], True
            for _ in range(repeats):
                ms, d = probe()
                times.append(ms)
                ok &= d == ref_digest
            med = statistics.median(times)
            trials.append((cand, med, ok))
            if ok and med < best_ms:
                best, best_ms = cand, med
    finally:
        set_tuning(**dict(base, **best))
    bad = [c for c, _, ok in trials if not ok]
    if bad:
        raise RuntimeError(f"{group}: settings changed the result: {bad}")
    return GroupResult(group, best, best_ms, default_ms, trials)


def bfs_probe(g: GPMA, source: int, levels_out=None):
    """Single-source BFS on `g` from `source`, timed with the library's events."""
    g.set_profiling(True)

    def probe():
        g.reset_profile()
        lv, reached = gpma_bfs(g, g.row_num, 0, source, levels_out)
        host = lv.cpu().numpy() if hasattr(lv, "cpu") else lv
        return g.profile()["bfs_ms"], digest(host, np.array([reached], np.uint64))

    return probe


def ms_probe(batch: Batch, graphs, sources):
    """Multi-source BFS over `graphs` (up to 64 sources each) in one launch."""
    batch.set_profiling(True)

    def probe():
        batch.reset_profile()
        _, reached = batch.bfs_multi(graphs, sources)
        p = batch.profile()
        return p["bfs_ms"], digest(np.concatenate(reached), np.array([p["bfs_edges"]], np.uint64))

    return probe


def update_probe(make_graph, keys, values):
    """One update of a fresh graph from `make_graph()` (so every run starts
    from the same state); the digest is the resulting layout."""

    def probe():
        g = make_graph()
        g.set_profiling(True)
        g.reset_profile()
        from . import update_gpma

        update_gpma(g, keys, values)
        ms = g.profile()["update_kernel_ms"]
        d = digest(*g.export_layout())
        g.close()
        return ms, d

    return probe


def autotune(probes: dict, repeats: int = 3) -> dict:
    """Tunes every group that has a probe ({"bfs": probe, "ms": probe,
    "update": probe}); returns a report and leaves the best tuning in force."""
    report = {}
    for group in ("bfs", "ms", "update"):
        if group in probes:
            r = tune_group(group, probes[group], repeats)
            report[group] = {"best": r.best, "best_ms": r.best_ms, "default_ms": r.default_ms,
                             "candidates": len(r.trials)}
    report["tuning"] = get_tuning()
    return report


def save(path: str, report: dict) -> None:
    with open(path, "w") as f:
        json.dump(report, f, indent=1)


def load(path: str) -> dict:
    """Applies a saved report's tuning; returns it."""
    with open(path) as f:
        report = json.load(f)
    set_tuning(**report["tuning"])
    return report
