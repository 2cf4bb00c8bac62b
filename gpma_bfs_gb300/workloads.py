"""Workloads of the reference demo on seeded synthetic graphs.

``sliding_window`` is the schedule of gpma_bfs_demo.cu:50-112: load the first
half of the (shuffled) edge list, BFS, then ``num_slide`` steps that each
insert the next ``half // num_slide`` edges (value 1) and delete the oldest
as many (value 0) in one batch [inserts ++ deletes], then BFS again.

The reference's dataset (pokec) is not available offline; ``GRAPHS`` holds
the synthetic stand-ins with the shapes the benchmarks are quoted on.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import edges_to_keys, gen_chung_lu, gen_rmat

# name -> generator parameters
GRAPHS = {
    # R-MAT scale 16 (65,536 nodes), edge factor 16, a/b/c/d = .57/.19/.19/.05
    "rmat16": dict(kind="rmat", scale=16, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1),
    # social-network shape: 1,632,803 nodes, 30,622,564 directed edges,
    # Chung-Lu out/in exponent 2.3, largest expected degree 9,000
    "social": dict(kind="chung_lu", n=1632803, m=30622564, exponent=2.3, max_degree=9000, seed=2),
}


def make_graph(name: str | dict):
    """(node count, src, dst) of a named (or explicitly parameterised) graph."""
    p = GRAPHS[name] if isinstance(name, str) else name
    if p["kind"] == "rmat":
        src, dst = gen_rmat(p["scale"], p["edge_factor"], p.get("a", 0.57), p.get("b", 0.19), p.get("c", 0.19),
                            p["seed"])
        return 1 << p["scale"], src, dst
    if p["kind"] == "chung_lu":
        src, dst = gen_chung_lu(p["n"], p["m"], p.get("exponent", 2.3), p.get("max_degree", 9000), p["seed"])
        return p["n"], src, dst
    raise ValueError(p["kind"])


def batched_graphs(count: int = 256, seed: int = 4, min_edges: int = 10_000, max_edges: int = 2_000_000):
    """Independent R-MAT graphs with edge counts log-uniform in [min, max] and
    about edges/16 nodes (the batched configuration). Returns a list of
    (node count, shuffled keys)."""
    rng = np.random.default_rng(seed)
    out = []
    for i, e in enumerate(np.exp(rng.uniform(np.log(min_edges), np.log(max_edges), count))):
        scale = int(np.clip(np.round(np.log2(e / 16)), 4, 24))
        ef = max(1, int(round(e / (1 << scale))))
        src, dst = gen_rmat(scale, ef, seed=seed * 100_000 + i)
        out.append((1 << scale, edges_to_keys(src, dst)))
    return out


class SlidingStream:
    """Per-graph sliding window over a cyclic edge list: the first half is the
    initial load; each step inserts the next b/2 edges and deletes the oldest
    b/2 (gpma_bfs_demo.cu:85-104 with a per-step batch size)."""

    def __init__(self, keys: np.ndarray):
        self.keys = keys
        self.m = len(keys)
        self.ins = self.m // 2
        self.dels = 0
        self._cyc = None  # keys twice over: any cyclic window of <= m keys is one slice

    def load(self):
        return self.keys[: self.m // 2], np.ones(self.m // 2, np.uint8)

    def step(self, batch: int):
        h = max(1, min(batch // 2, self.m // 2))
        if self._cyc is None:
            self._cyc = np.concatenate([self.keys, self.keys])
        i, d = self.ins % self.m, self.dels % self.m
        self.ins += h
        self.dels += h
        vals = np.zeros(2 * h, np.uint8)
        vals[:h] = 1
        return np.concatenate([self._cyc[i:i + h], self._cyc[d:d + h]]), vals


@dataclass
class SlidingWindow:
    half: int
    step: int
    load_keys: np.ndarray
    load_values: np.ndarray
    slide_keys: list
    slide_values: list

    @property
    def num_slide(self) -> int:
        return len(self.slide_keys)


def sliding_window(src: np.ndarray, dst: np.ndarray, num_slide: int = 100) -> SlidingWindow:
    keys = edges_to_keys(src, dst)
    half = len(keys) // 2
    step = half // num_slide
    sk, sv = [], []
    for i in range(num_slide):
        ins = keys[half + i * step: half + (i + 1) * step]
        dels = keys[i * step: (i + 1) * step]
        sk.append(np.concatenate([ins, dels]))
        sv.append(np.concatenate([np.ones(step, np.uint8), np.zeros(step, np.uint8)]))
    return SlidingWindow(half, step, keys[:half].copy(), np.ones(half, np.uint8), sk, sv)
