"""Served form on the GPU: every request's result in the continuously batched
mix equals its result when the same requests are applied to that graph alone
(bit-exact: BFS reach per source, level arrays, final layouts), and the
graphs match the oracle."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def _trace(rng, specs, count, rate):
    """(arrival, graph, kind, payload) in arrival order; updates are sliding
    windows over each graph's edge list (1:1 insert:delete), searches 1..64
    sources, every fifth search keeping its level arrays."""
    from gpma_bfs_gb300.workloads import SlidingStream

    streams = [SlidingStream(k) for _, k in specs]
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        g = int(rng.integers(len(specs)))
        if rng.random() < 0.7:
            size = int(np.exp(rng.uniform(np.log(10), np.log(4000))))
            out.append((float(t[i]), g, 0, streams[g].step(size)))
        else:
            n = specs[g][0]
            k = int(rng.integers(1, 65))
            src = rng.choice(n, min(k, n), replace=False).astype(np.uint32)
            out.append((float(t[i]), g, 1, (src, i % 5 == 0)))
    return streams, out


def test_served_results_equal_alone(built_lib):
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream

    rng = np.random.default_rng(21)
    specs = []
    for i in range(12):
        scale = int(rng.integers(6, 12))
        src, dst = G.gen_rmat(scale, 8, seed=500 + i)
        specs.append((1 << scale, G.edges_to_keys(src, dst)))
    loads = [SlidingStream(k).load() for _, k in specs]
    _, trace = _trace(rng, specs, 400, rate=2000.0)

    srv = G.Server(max_round_keys=20_000, max_round_bfs_graphs=8)
    gids = [srv.add_graph(n, len(k)) for n, k in specs]
    for gid, (k, v) in zip(gids, loads):
        G.update_gpma(srv.graph(gid), k, v)

    # continuous batching in virtual time: submit what has arrived, run a round
    now, j, ids, rounds = 0.0, 0, [], []
    while j < len(trace) or srv.queued()[0]:
        while j < len(trace) and trace[j][0] <= now:
            t, g, kind, p = trace[j]
            if kind == 0:
                ids.append(srv.submit_update(gids[g], p[0], p[1], t))
            else:
                ids.append(srv.submit_bfs(gids[g], p[0], t, levels=p[1]))
            j += 1
        r = srv.run_round(now)
        if r["updates"] + r["bfs_requests"]:
            rounds.append(r)
            now += r["seconds"]
        elif j < len(trace):
            now = max(now, trace[j][0])
    assert all(r["failed"] == 0 for r in rounds)
    # the mix really mixed: several graphs per launch, searches behind updates
    assert max(r["updates"] for r in rounds) > 1
    assert max(r["bfs_graphs"] for r in rounds) > 1
    assert any(r["updates"] and r["bfs_requests"] for r in rounds)
    infos = [srv.poll(i) for i in ids]
    assert all(x["state"] == 1 and x["done"] >= x["arrival"] for x in infos)

    # the same requests, graph by graph, one plain call each
    alone = [G.GPMA(n) for n, _ in specs]
    for g, (k, v) in zip(alone, loads):
        G.update_gpma(g, k, v)
    for (t, g, kind, p), rid, info in zip(trace, ids, infos):
        if kind == 0:
            G.update_gpma(alone[g], p[0], p[1])
            continue
        lv, reached = G.gpma_bfs_multi(alone[g], p[0])
        assert np.array_equal(info["reached"], reached), f"request {rid} (graph {g})"
        got = srv.levels(rid)
        if p[1]:
            assert np.array_equal(got, lv), f"levels of request {rid}"
    for i, gid in enumerate(gids):
        a = srv.graph(gid).export_layout()
        b = alone[i].export_layout()
        assert all(np.array_equal(x, y) for x, y in zip(a, b)), f"graph {i}"
    # and the oracle agrees with the served graphs
    for i in (0, 7):
        o = OracleGPMA(specs[i][0], threads=2)
        o.update(*loads[i])
        for t, g, kind, p in trace:
            if g == i and kind == 0:
                o.update(*p)
        assert all(np.array_equal(x, y) for x, y in zip(srv.graph(gids[i]).export_layout(), o.export_layout()))
    for g in alone:
        g.close()
    srv.close()


def test_served_budget_rejects_growth(built_lib):
    """A batch whose worst-case growth cannot fit the HBM budget fails with
    ERR_BUDGET and leaves the graph untouched; the next request still runs."""
    import gpma_bfs_gb300 as G

    src, dst = G.gen_rmat(10, 8, seed=3)
    keys = G.edges_to_keys(src, dst)
    srv = G.Server(hbm_budget_bytes=8 << 20, max_round_keys=1 << 12)
    gid = srv.add_graph(1024, len(keys))
    G.update_gpma(srv.graph(gid), keys, np.ones(len(keys), np.uint8))
    before = srv.graph(gid).export_layout()
    big = np.arange(1, 400_001, dtype=np.uint64) << np.uint64(32)
    r1 = srv.submit_update(gid, big, np.ones(len(big), np.uint8), 0.0)
    r2 = srv.submit_bfs(gid, [int(src[0])], 0.0)
    srv.run_round(0.0)
    p = srv.poll(r1)
    assert p["state"] == 2 and p["status"] == G.ERR_BUDGET
    after = srv.graph(gid).export_layout()
    assert all(np.array_equal(x, y) for x, y in zip(before, after))
    assert srv.poll(r2)["state"] == 1
    srv.close()


def test_served_live_two_lanes_equal_alone(built_lib):
    """The native serving loop with two lanes in real time: rounds of
    different graphs are in flight at once (each lane its own stream and
    buffers), batches are uploaded from the pinned input ring or from host
    vectors, and still every search's reach and levels and every graph's
    final layout equal the same requests applied to each graph alone."""
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import SlidingStream

    rng = np.random.default_rng(22)
    specs = []
    for i in range(16):
        scale = int(rng.integers(8, 14))
        src, dst = G.gen_rmat(scale, 8, seed=700 + i)
        specs.append((1 << scale, G.edges_to_keys(src, dst)))
    loads = [SlidingStream(k).load() for _, k in specs]
    _, trace = _trace(rng, specs, 600, rate=3000.0)

    # a small pinned input ring: some batches are staged there (wrapping
    # around), the others stay in host vectors
    srv = G.Server(max_round_keys=20_000, max_round_bfs_graphs=8, lanes=2, input_ring_bytes=256 << 10)
    gids = [srv.add_graph(n, len(k)) for n, k in specs]
    for gid, (k, v) in zip(gids, loads):
        G.update_gpma(srv.graph(gid), k, v)
    import torch

    torch.cuda.synchronize()
    srv.start()
    ids = []
    for t, g, kind, p in trace:  # all submitted ahead; each runs once the clock passes its arrival
        if kind == 0:
            ids.append(srv.submit_update(gids[g], p[0], p[1], t))
        else:
            ids.append(srv.submit_bfs(gids[g], p[0], t, levels=p[1]))
    srv.drain(120.0)
    srv.stop()
    st = srv.stats()
    assert st["requests"] == len(trace)
    assert st["max_inflight_rounds"] == 2  # the lanes overlapped
    infos = [srv.poll(i) for i in ids]
    assert all(x["state"] == 1 and x["start"] >= x["arrival"] - 1e-9 for x in infos)

    alone = [G.GPMA(n) for n, _ in specs]
    for g, (k, v) in zip(alone, loads):
        G.update_gpma(g, k, v)
    for (t, g, kind, p), rid, info in zip(trace, ids, infos):
        if kind == 0:
            G.update_gpma(alone[g], p[0], p[1])
            continue
        lv, reached = G.gpma_bfs_multi(alone[g], p[0])
        assert np.array_equal(info["reached"], reached), f"request {rid} (graph {g})"
        if p[1]:
            assert np.array_equal(srv.levels(rid), lv), f"levels of request {rid}"
    for i, gid in enumerate(gids):
        a = srv.graph(gid).export_layout()
        b = alone[i].export_layout()
        assert all(np.array_equal(x, y) for x, y in zip(a, b)), f"graph {i}"
    for g in alone:
        g.close()
    srv.close()
