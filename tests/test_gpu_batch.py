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


def test_packed_update_any_graph_order(built_lib):
    """One packed buffer, graphs in arbitrary (not segment-sorted) order, keys
    on the host and on the device."""
    import torch

    import gpma_bfs_gb300 as G

    rng = np.random.default_rng(13)
    specs = _graphs(rng, 10)[::-1]
    gpus = [G.GPMA(n) for n, _ in specs]
    orcs = [OracleGPMA(n, threads=2) for n, _ in specs]
    b = G.Batch()
    for step in range(4):
        ks, vs = [], []
        for i, (n, keys) in enumerate(specs):
            if step == 0:
                k = keys[: len(keys) // 2]
                v = np.ones(len(k), np.uint8)
            else:
                lk = orcs[i].compact_keys()
                live = lk[(lk & np.uint64(0xFFFFFFFF)) < np.uint64(0xFFFFFFFE)]
                k, v = _batch_for(rng, keys, live, n)
            ks.append(k)
            vs.append(v)
            orcs[i].update(k, v)
        off = np.concatenate([[0], np.cumsum([len(k) for k in ks])]).astype(np.uint64)
        pk, pv = np.concatenate(ks), np.concatenate(vs)
        if step % 2:
            b.update_packed(gpus, torch.from_numpy(pk.view(np.int64)).cuda(), torch.from_numpy(pv).cuda(), off)
        else:
            b.update_packed(gpus, pk, pv, off)
        for i in range(len(specs)):
            gk, gv, gr = gpus[i].export_layout()
            ok, ov, orr = orcs[i].export_layout()
            assert np.array_equal(gk, ok) and np.array_equal(gv, ov) and np.array_equal(gr, orr), f"{step}/{i}"
    b.close()


def test_batched_sliding_windows_mixed_segment_lengths(built_lib):
    """Many graphs of different segment lengths in one launch, with sliding
    batches up to the whole edge list: every level then holds several runs of
    windows (warp, CTA and grid-wide widths side by side). Each graph must end
    exactly as the single-graph path leaves it, and as the oracle does."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    specs = batched_graphs(64, seed=7, min_edges=10_000, max_edges=400_000)
    rng = np.random.default_rng(71)
    gb = [G.GPMA(n) for n, _ in specs]
    gp = [G.GPMA(n) for n, _ in specs]
    sliding = [SlidingStream(k) for _, k in specs]
    history = [[s.load()] for s in sliding]
    off = np.concatenate([[0], np.cumsum([len(h[0][0]) for h in history])]).astype(np.uint64)
    b = G.Batch()
    b.update_packed(gb, np.concatenate([h[0][0] for h in history]), np.concatenate([h[0][1] for h in history]), off)
    for g, h in zip(gp, history):
        G.update_gpma(g, *h[0])
    for step in range(4):
        sizes = np.exp(rng.uniform(np.log(100), np.log(400_000), len(specs))).astype(np.int64)
        parts = [s.step(int(z)) for s, z in zip(sliding, sizes)]
        for h, p in zip(history, parts):
            h.append(p)
        o = np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64)
        dk = torch.from_numpy(np.concatenate([p[0] for p in parts]).view(np.int64)).cuda()
        dv = torch.from_numpy(np.concatenate([p[1] for p in parts])).cuda()
        b.update_packed(gb, dk, dv, o)
        for i, g in enumerate(gp):
            G.update_gpma(g, dk[int(o[i]):int(o[i + 1])], dv[int(o[i]):int(o[i + 1])])
        for i in range(len(specs)):
            x, y = gb[i].export_layout(), gp[i].export_layout()
            assert all(np.array_equal(p, q) for p, q in zip(x, y)), f"step {step} graph {i}"
            assert gb[i].validate() == 0 and gp[i].validate() == 0, f"step {step} graph {i}: segment heads"
    for i in rng.choice(len(specs), 4, replace=False):
        orc = OracleGPMA(specs[i][0], threads=4)
        for k, v in history[i]:
            orc.update(k, v)
        assert all(np.array_equal(p, q) for p, q in zip(gb[i].export_layout(), orc.export_layout())), f"graph {i}"
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
