"""Golden-vector cases: operation scripts replayed by the reference and by us.

Each case is (row_num, ops) with ops drawn from
    ("update", keys u64[], values u8[]), ("bfs", src), ("dump",)
Small cases store their ops inside the fixture; generated cases ("rmat*")
are rebuilt from their generator parameters and checked against the stored
input digest, so the fixtures stay small.
"""
from __future__ import annotations

import numpy as np

GUARD = np.uint64(0xFFFFFFFF)


def _keys(src, dst) -> np.ndarray:
    return (np.asarray(src, np.uint64) << np.uint64(32)) | np.asarray(dst, np.uint64)


def edge_cases():
    """Hand-written corner cases of the update semantics (gpma.cuh:188-220, 968-1050).
    Destinations stay below row_num: the reference BFS indexes its bitmap and
    level array with them unchecked."""
    n = 3037
    ops = []
    upd = lambda k, v: ops.append(("update", np.asarray(k, np.uint64), np.asarray(v, np.uint8)))
    upd([], [])                                             # empty batch
    upd(_keys([0, 0, 1, 5], [1, 2, 0, 36]), [1, 1, 1, 1])  # plain inserts
    ops.append(("bfs", 0))
    upd(_keys([3, 4], [4, 3]), [0, 0])                      # deletes of missing keys: dropped
    upd(_keys([0], [2]), [0])                               # delete -> tombstone
    ops.append(("dump",))
    upd(_keys([0], [2]), [1])                               # re-insert: revives the tombstone in place
    upd(_keys([1], [0]), [7])                               # modify the value of an existing key
    upd(_keys([2, 2], [9, 9]), [1, 1])                      # duplicate key within one batch, same value
    ops.append(("dump",))
    upd(_keys([2], [9]), [0])                               # deletes the first copy only
    rng = np.random.default_rng(123)
    s = rng.integers(0, n, 400)
    d = rng.integers(0, n - 1, 400)
    d = np.where(d >= s, d + 1, d)                          # no self-loops
    k = np.unique(_keys(s, d))
    upd(k, np.ones(len(k), np.uint8))                      # batch that forces root resizes
    ops.append(("bfs", 0))
    ops.append(("dump",))
    upd(k[::2], np.zeros(len(k[::2]), np.uint8))           # mass delete (tombstones)
    upd(k[:5], np.ones(5, np.uint8))                       # partly revives
    ops.append(("bfs", 5))
    ops.append(("dump",))
    upd(np.arange(0, 2000, dtype=np.uint64) + (np.uint64(36) << np.uint64(32)),
        np.ones(2000, np.uint8))                           # dense row: deep windows
    ops.append(("bfs", 36))
    ops.append(("dump",))
    big = np.arange(0, 3000, dtype=np.uint64) + (np.uint64(36) << np.uint64(32))
    upd(big, np.zeros(3000, np.uint8))                     # delete it again, then a small insert
    upd(_keys([10, 11], [12, 13]), [1, 1])                  # ... forcing a shrinking root resize
    ops.append(("bfs", 10))
    ops.append(("dump",))
    return n, ops


def random_case(seed: int):
    """Random mixed scripts: inserts, deletes of live and missing keys,
    revivals, modifications, duplicate keys with equal values."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 300))
    ops = []
    live: set[int] = set()
    ever: list[int] = []
    for step in range(int(rng.integers(20, 60))):
        size = int(rng.choice([0, 1, 3, 17, 64, 250, 1200]))
        ks, vs = [], []
        for _ in range(size):
            r = rng.random()
            if r < 0.55 or not ever:
                s = int(rng.integers(0, n))
                d = int(rng.integers(0, n))
                key = (s << 32) | d
                ks.append(key)
                vs.append(1 if rng.random() < 0.9 else int(rng.integers(2, 256)))
            elif r < 0.85:
                key = int(ever[int(rng.integers(0, len(ever)))])
                ks.append(key)
                vs.append(0)
            else:
                key = int(ever[int(rng.integers(0, len(ever)))])
                ks.append(key)
                vs.append(int(rng.integers(1, 256)))
        # one value per key within a batch (duplicates keep the same value)
        seen = {}
        for key, v in zip(ks, vs):
            seen.setdefault(key, v)
        if size and rng.random() < 0.3:
            dup = ks[: max(1, size // 10)]
            ks = ks + dup
        vs = [seen[k] for k in ks]
        ops.append(("update", np.asarray(ks, np.uint64), np.asarray(vs, np.uint8)))
        for key, v in zip(ks, vs):
            if v:
                live.add(key)
                ever.append(key)
            else:
                live.discard(key)
        if rng.random() < 0.2 and n > 0:
            ops.append(("bfs", int(rng.integers(0, n))))
        if rng.random() < 0.15:
            ops.append(("dump",))
    ops.append(("bfs", 0))
    ops.append(("dump",))
    return n, ops


def sliding_ops(n, src, dst, num_slide, bfs_src=0, dumps=()):
    keys = _keys(src, dst)
    half = len(keys) // 2
    step = half // num_slide
    ops = [("update", keys[:half], np.ones(half, np.uint8)), ("bfs", bfs_src)]
    if 0 in dumps:
        ops.append(("dump",))
    for i in range(num_slide):
        ins = keys[half + i * step: half + (i + 1) * step]
        dels = keys[i * step: (i + 1) * step]
        ops.append(("update", np.concatenate([ins, dels]),
                    np.concatenate([np.ones(step, np.uint8), np.zeros(step, np.uint8)])))
        if i + 1 in dumps:
            ops.append(("dump",))
    ops.append(("bfs", bfs_src))
    return ops


def bulk_ops(n, src, dst):
    """All edges in one batch (>= 5M insertions: the bulk rebuild, gpma.cuh:936-966),
    then three slides of deletions and re-insertions."""
    keys = _keys(src, dst)
    ops = [("update", keys, np.ones(len(keys), np.uint8)), ("bfs", 0)]
    step = 100000
    for i in range(3):
        dels = keys[i * step: (i + 1) * step]
        ops.append(("update", dels, np.zeros(len(dels), np.uint8)))
        ops.append(("update", dels[::2], np.ones(len(dels[::2]), np.uint8)))
    ops.append(("bfs", 0))
    return ops


# Generated cases: generator parameters (gpma_bfs_gb300.workloads.make_graph)
GENERATED = {
    "rmat8_slide": dict(graph=dict(kind="rmat", scale=8, edge_factor=8, seed=11), schedule="slide", num_slide=100,
                        dumps=(0, 50, 100), full=True),
    "rmat12_slide": dict(graph=dict(kind="rmat", scale=12, edge_factor=16, seed=7), schedule="slide",
                         num_slide=100, dumps=(100,), full=True),
    "rmat16_slide": dict(graph=dict(kind="rmat", scale=16, edge_factor=16, seed=1), schedule="slide",
                         num_slide=100, dumps=(), full=False),
    "rmat20_bulk": dict(graph=dict(kind="rmat", scale=20, edge_factor=8, seed=5), schedule="bulk", full=False),
}
SMALL = {"edge_cases": edge_cases, **{f"random_{s}": (lambda s=s: random_case(s)) for s in (1, 2, 3, 4, 5, 6)}}


def generated_ops(name):
    from gpma_bfs_gb300.workloads import make_graph

    spec = GENERATED[name]
    n, src, dst = make_graph(spec["graph"])
    if spec["schedule"] == "slide":
        ops = sliding_ops(n, src, dst, spec["num_slide"], dumps=spec.get("dumps", ()))
    else:
        ops = bulk_ops(n, src, dst)
    return n, ops, _keys(src, dst)
