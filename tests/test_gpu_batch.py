"""Many graphs per launch: each graph must end exactly as if updated alone."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def _graphs(rng, count):
    import gpma_bfs_gb300 as G

    out = []
    for i in range(count):
        scale = int(rng.integers(6, 13))
        src, dst = G.gen_rmat(scale, 8, seed=100 + i)
        out.append((1 << scale, G.edges_to_keys(src, dst)))
    return out


def _batch_for(rng, keys, live, n):
    size = int(np.exp(rng.uniform(np.log(10), np.log(3000))))
    ins = keys[rng.integers(0, len(keys), size)]
    dels = live[rng.integers(0, len(live), size // 2)] if len(live) else np.zeros(0, np.uint64)
    k = np.unique(np.concatenate([ins, dels]))
    is_ins = np.isin(k, ins) & ~np.isin(k, dels)
    v = is_ins.astype(np.uint8)
    return k, v


def test_batch_update_matches_individual_updates(built_lib):
    import gpma_bfs_gb300 as G

    rng = np.random.default_rng(5)
    specs = _graphs(rng, 14)
    gpus = [G.GPMA(n) for n, _ in specs]
    orcs = [OracleGPMA(n, threads=2) for n, _ in specs]
    live = [np.zeros(0, np.uint64) for _ in specs]
    b = G.Batch()
    for step in range(8):
        ks, vs = [], []
        for i, (n, keys) in enumerate(specs):
            if step == 3 and i % 5 == 0:
                k, v = np.zeros(0, np.uint64), np.zeros(0, np.uint8)  # empty batch
            elif step == 0 or (step == 5 and i % 4 == 1):
                k = keys[: len(keys) // 2]  # bulk load: deep windows and root resizes
                v = np.ones(len(k), np.uint8)
            else:
                k, v = _batch_for(rng, keys, live[i], n)
            ks.append(k)
            vs.append(v)
            orcs[i].update(k, v)
            lk = orcs[i].compact_keys()
            # deletable edges only: no row guards (reserved column) or sentinels
            live[i] = lk[(lk & np.uint64(0xFFFFFFFF)) < np.uint64(0xFFFFFFFE)]
        b.update(gpus, ks, vs)
        for i in range(len(specs)):
            gk, gv, gr = gpus[i].export_layout()
            ok, ov, orr = orcs[i].export_layout()
            ctx = f"step {step} graph {i}"
            assert gpus[i].geometry() == orcs[i].geometry(), ctx
            assert np.array_equal(gk, ok), ctx + ": keys"
            assert np.array_equal(gv, ov), ctx + ": values"
            assert np.array_equal(gr, orr), ctx + ": row_offset"
    b.close()


def test_batch_bfs_multi_matches_single_source(built_lib):
    import gpma_bfs_gb300 as G

    rng = np.random.default_rng(9)
    specs = _graphs(rng, 9)
    gpus, orcs, sources = [], [], []
    for n, keys in specs:
        g = G.GPMA(n)
        o = OracleGPMA(n, threads=2)
        G.update_gpma(g, keys, np.ones(len(keys), np.uint8))
        o.update(keys, np.ones(len(keys), np.uint8))
        gpus.append(g)
        orcs.append(o)
        sources.append(rng.choice(n, int(rng.integers(1, 65)), replace=False).astype(np.uint32))
    b = G.Batch()
    levels, reached = b.bfs_multi(gpus, sources, levels=True)
    for i in range(len(specs)):
        ol, orr = orcs[i].bfs_multi(sources[i])
        assert np.array_equal(reached[i], orr), f"graph {i}"
        assert np.array_equal(levels[i], ol), f"graph {i}"
    # traversed edges = sum over sources of live out-edges of reached nodes
    want = sum(orcs[i].traversed_edges(ol_row) for i in range(len(specs))
               for ol_row in orcs[i].bfs_multi(sources[i])[0])
    assert b.profile()["bfs_edges"] == want
    _, reached2 = b.bfs_multi(gpus, sources, levels=False)
    assert all(np.array_equal(a, c) for a, c in zip(reached, reached2))
    b.close()
