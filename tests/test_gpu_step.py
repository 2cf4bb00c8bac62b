"""Recorded update+BFS steps (CUDA graph replay) give exactly what
update_gpma followed by gpma_bfs gives, step by step: levels, reachable
count and the whole layout, through root resizes, batch-size and source
changes, empty batches, host and device buffers, and a rejected batch."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def _same_layout(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a.export_layout(), b.export_layout()))


def test_step_matches_update_then_bfs(built_lib):
    import torch

    import gpma_bfs_gb300 as G

    scale = 12
    n = 1 << scale
    src, dst = G.gen_rmat(scale, 8, seed=31)
    keys = G.edges_to_keys(src, dst)
    rng = np.random.default_rng(5)
    keys = keys[rng.permutation(len(keys))]
    half = len(keys) // 2
    eager, graphed = G.GPMA(n), G.GPMA(n)
    o = OracleGPMA(n, threads=2)
    step = G.Step(graphed)
    ones = np.ones(half, np.uint8)
    # the first step grows the array from the guards alone: root resize on the host
    G.update_gpma(eager, keys[:half], ones)
    want, want_r = G.gpma_bfs(eager, n, 0, 0)
    got = np.zeros(n, np.uint32)
    r = step.run(keys[:half], ones, 0, got)
    o.update(keys[:half], ones)
    assert r == want_r and np.array_equal(got, want) and _same_layout(eager, graphed)
    assert step.stats()["host_runs"] >= 1
    # sliding window: batch sizes and sources vary, host and device buffers
    lo, hi = 0, half
    dev_levels = torch.zeros(n, dtype=torch.int32, device="cuda")
    for i in range(14):
        w = [300, 300, 301, 1200, 64, 0, 300][i % 7]
        ins, dele = keys[hi: hi + w], keys[lo: lo + w]
        lo, hi = lo + w, hi + w
        k = np.concatenate([ins, dele])
        v = np.concatenate([np.ones(len(ins), np.uint8), np.zeros(len(dele), np.uint8)])
        s0 = int(keys[hi - 1] >> np.uint64(32)) if i % 3 else 0
        G.update_gpma(eager, k, v)
        want, want_r = G.gpma_bfs(eager, n, 0, s0)
        o.update(k, v)
        if i % 2:
            kd = torch.from_numpy(k.view(np.int64)).cuda()
            vd = torch.from_numpy(v).cuda()
            r = step.run(kd, vd, s0, dev_levels)
            got = dev_levels.cpu().numpy().view(np.uint32)
        else:
            got = np.zeros(n, np.uint32)
            r = step.run(k, v, s0, got)
        assert r == want_r and np.array_equal(got, want), f"step {i}"
        assert _same_layout(eager, graphed), f"step {i}"
        ol, orr = o.bfs(s0)
        assert np.array_equal(got, ol) and r == orr, f"step {i} against the oracle"
    st = step.stats()
    assert st["runs"] == 15 and st["graph_launches"] >= 10 and st["param_updates"] > 0
    assert st["builds"] >= 1 and st["last_ms"] > 0
    # levels=None keeps them inside the library; the count still matches
    assert step.run(keys[:0], ones[:0], 0) == G.gpma_bfs(eager, n, 0, 0)[1]
    step.close()
    eager.close()
    graphed.close()


def test_step_rejected_batch_then_recovers(built_lib):
    import gpma_bfs_gb300 as G

    n = 1 << 10
    src, dst = G.gen_rmat(10, 8, seed=7)
    keys = G.edges_to_keys(src, dst)
    eager, graphed = G.GPMA(n), G.GPMA(n)
    ones = np.ones(len(keys), np.uint8)
    G.update_gpma(eager, keys, ones)
    with G.Step(graphed) as step:
        step.run(keys, ones, 0)
        bad = np.array([(3 << 32) | 0xFFFFFFFF], np.uint64)  # reserved column
        with pytest.raises(G.GPMAError):
            step.run(bad, np.ones(1, np.uint8), 0)
        k = keys[:50]
        G.update_gpma(eager, k, np.zeros(50, np.uint8))
        want, want_r = G.gpma_bfs(eager, n, 0, 1)
        got = np.zeros(n, np.uint32)
        assert step.run(k, np.zeros(50, np.uint8), 1, got) == want_r
        assert np.array_equal(got, want) and _same_layout(eager, graphed)
    eager.close()
    graphed.close()


def test_batch_step_matches_eager_calls(built_lib):
    """The batched form's recorded step equals update_packed + bfs_multi:
    every graph's layout and every source's reach, step by step, including a
    step with an empty part (eager fallback) and device-resident batches."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    specs = batched_graphs(24, seed=9, min_edges=5_000, max_edges=200_000)
    rng = np.random.default_rng(12)
    ge = [G.GPMA(n) for n, _ in specs]
    gr = [G.GPMA(n) for n, _ in specs]
    se = [SlidingStream(k) for _, k in specs]
    sr = [SlidingStream(k) for _, k in specs]
    be, br = G.Batch(), G.Batch()
    loads = [s.load() for s in se]
    for s in sr:
        s.load()
    off = np.concatenate([[0], np.cumsum([len(x[0]) for x in loads])]).astype(np.uint64)
    keys, vals = np.concatenate([x[0] for x in loads]), np.concatenate([x[1] for x in loads])
    be.update_packed(ge, keys, vals, off)
    br.update_packed(gr, keys, vals, off)
    sources = [rng.choice(n, 16, replace=False).astype(np.uint32) for n, _ in specs]
    step = br.step(gr)
    for j in range(8):
        sizes = np.exp(rng.uniform(np.log(50), np.log(40_000), len(specs))).astype(np.int64)
        parts = [s.step(int(z)) for s, z in zip(se, sizes)]
        for s, z in zip(sr, sizes):
            s.step(int(z))
        if j == 5:
            parts[3] = (parts[3][0][:0], parts[3][1][:0])  # an empty part: the step runs the eager calls
        o = np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64)
        k = np.concatenate([p[0] for p in parts])
        v = np.concatenate([p[1] for p in parts])
        if j % 2:
            k, v = torch.from_numpy(k.view(np.int64)).cuda(), torch.from_numpy(v).cuda()
        be.update_packed(ge, k, v, o)
        want = be.bfs_multi(ge, sources)[1]
        got = step.run(k, v, o, sources)
        assert all(np.array_equal(x, y) for x, y in zip(want, got)), f"step {j}: reach"
        for i in range(len(specs)):
            assert all(np.array_equal(x, y) for x, y in zip(ge[i].export_layout(), gr[i].export_layout())), \
                f"step {j} graph {i}"
            assert gr[i].validate() == 0
    st = step.stats()
    assert st["runs"] == 8 and st["host_runs"] >= 1 and st["graph_launches"] >= 6 and st["builds"] >= 1
    step.close()
    be.close()
    br.close()
    for g in ge + gr:
        g.close()


def _batched_pair(count, seed):
    """Two identical sets of graphs (eager and recorded) after the same load."""
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream, batched_graphs

    specs = batched_graphs(count, seed=seed, min_edges=5_000, max_edges=200_000)
    ge = [G.GPMA(n) for n, _ in specs]
    gr = [G.GPMA(n) for n, _ in specs]
    se = [SlidingStream(k) for _, k in specs]
    sr = [SlidingStream(k) for _, k in specs]
    be, br = G.Batch(), G.Batch()
    loads = [s.load() for s in se]
    for s in sr:
        s.load()
    off = np.concatenate([[0], np.cumsum([len(x[0]) for x in loads])]).astype(np.uint64)
    keys, vals = np.concatenate([x[0] for x in loads]), np.concatenate([x[1] for x in loads])
    be.update_packed(ge, keys, vals, off)
    br.update_packed(gr, keys, vals, off)
    return specs, ge, gr, se, be, br


def _packed_steps(rng, streams, steps, lo=50, hi=40_000):
    import torch

    ks, vs, offs = [], [], []
    for _ in range(steps):
        sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), len(streams))).astype(np.int64)
        parts = [s.step(int(z)) for s, z in zip(streams, sizes)]
        offs.append(np.concatenate([[0], np.cumsum([len(p[0]) for p in parts])]).astype(np.uint64))
        ks.append(torch.from_numpy(np.concatenate([p[0] for p in parts]).view(np.int64)).cuda())
        vs.append(torch.from_numpy(np.concatenate([p[1] for p in parts])).cuda())
    return ks, vs, offs


def _check_many(specs, ge, gr, be, got, ks, vs, offs, sources):
    for t in range(len(ks)):
        be.update_packed(ge, ks[t], vs[t], offs[t])
        want = be.bfs_multi(ge, sources)[1]
        assert all(np.array_equal(x, y) for x, y in zip(want, got[t])), f"step {t}: reach"
    for i in range(len(specs)):
        assert all(np.array_equal(x, y) for x, y in zip(ge[i].export_layout(), gr[i].export_layout())), f"graph {i}"
        assert gr[i].validate() == 0


def test_batch_steps_recorded_in_one_graph(built_lib):
    """Twelve steps of 20 graphs in one graph launch equal the per-step eager
    calls (every step's reach, the final layouts); the recording is replayed
    for the next twelve with its kernel arguments refreshed."""
    specs, ge, gr, se, be, br = _batched_pair(20, seed=31)
    rng = np.random.default_rng(32)
    sources = [rng.choice(n, 8, replace=False).astype(np.uint32) for n, _ in specs]
    step = br.step(gr)
    for call in range(2):
        ks, vs, offs = _packed_steps(rng, se, 12)
        got = step.run_many(ks, vs, offs, sources)
        _check_many(specs, ge, gr, be, got, ks, vs, offs, sources)
    st = step.stats()
    assert st["runs"] == 24 and st["graph_launches"] == 2 and st["host_runs"] == 0
    assert st["builds"] == 1 and st["param_updates"] > 0
    step.close()
    be.close()
    br.close()
    for g in ge + gr:
        g.close()


def test_batch_steps_recorded_stop_at_host_work(built_lib):
    """A step whose update needs host work (a burst of new edges grows one
    graph past its root) stops the recorded steps after it; that step and the
    rest finish through the per-step path with identical results."""
    import torch

    specs, ge, gr, se, be, br = _batched_pair(8, seed=41)
    rng = np.random.default_rng(42)
    sources = [rng.choice(n, 4, replace=False).astype(np.uint32) for n, _ in specs]
    step = br.step(gr)
    ks, vs, offs = _packed_steps(rng, se, 6)
    # step 2: graph 0 also receives a burst of new edges, more than its array holds
    n0 = specs[0][0]
    size0 = gr[0].geometry()["size"]
    extra = np.unique((rng.integers(0, n0, 2 * size0).astype(np.uint64) << np.uint64(32)) |
                      rng.integers(0, n0, 2 * size0).astype(np.uint64))
    k2 = ks[2].cpu().numpy().view(np.uint64)
    v2 = vs[2].cpu().numpy()
    o2 = offs[2]
    # none of the step's own keys again (a present key given two values in one
    # batch would be written twice in place, in no fixed order)
    extra = np.setdiff1d(extra, k2)
    cut = int(o2[1])
    k2 = np.concatenate([k2[:cut], extra, k2[cut:]])
    v2 = np.concatenate([v2[:cut], np.ones(len(extra), np.uint8), v2[cut:]])
    offs[2] = np.concatenate([[0], o2[1:] + np.uint64(len(extra))]).astype(np.uint64)
    ks[2] = torch.from_numpy(k2.view(np.int64)).cuda()
    vs[2] = torch.from_numpy(v2).cuda()
    got = step.run_many(ks, vs, offs, sources)
    _check_many(specs, ge, gr, be, got, ks, vs, offs, sources)
    st = step.stats()
    assert st["runs"] == 6 and st["host_runs"] >= 1 and st["graph_launches"] >= 1
    step.close()
    be.close()
    br.close()
    for g in ge + gr:
        g.close()
