"""Served form: the scheduling and admission policy, in plan-only mode (no
device work), so it runs on a host without a GPU."""
import numpy as np
import pytest


@pytest.fixture
def G(built_lib):
    import gpma_bfs_gb300 as G

    return G


def _upd(n, inserts=True):
    keys = (np.arange(n, dtype=np.uint64) + np.uint64(1)) << np.uint64(32)
    return keys, np.full(n, 1 if inserts else 0, np.uint8)


def test_fifo_per_graph_one_update_per_round(G):
    s = G.Server(plan_only=True)
    g0, g1 = s.add_graph(100, 1000), s.add_graph(100, 1000)
    u1 = s.submit_update(g0, *_upd(10), arrival=0.0)
    b1 = s.submit_bfs(g0, [1, 2], arrival=0.1)
    u2 = s.submit_update(g0, *_upd(10), arrival=0.2)
    b2 = s.submit_bfs(g0, [3], arrival=0.3)
    b3 = s.submit_bfs(g1, [4], arrival=0.0)
    u3 = s.submit_update(g1, *_upd(5), arrival=0.05)
    r = s.run_round(1.0)
    assert (r["updates"], r["bfs_requests"], r["round"]) == (1, 2, 1)
    # updates first, then searches graph by graph: b1 sees u1 and not u2
    assert s.last_round() == [u1, b1, b3]
    r = s.run_round(1.0)
    # graphs in order of their queue head's arrival: g1 (0.05) before g0 (0.2)
    assert s.last_round() == [u3, u2, b2]
    assert (r["updates"], r["keys"], r["bfs_requests"]) == (2, 15, 1)
    assert s.run_round(1.0)["updates"] == 0 and s.last_round() == []
    for rid in (u1, b1, u2, b2, b3, u3):
        p = s.poll(rid)
        assert p["state"] == 1 and p["done"] == p["start"] == 1.0
    assert s.poll(u3)["round"] == 2 and s.poll(b3)["round"] == 1
    s.close()


def test_arrival_gating_and_virtual_time(G):
    s = G.Server(plan_only=True)
    g = s.add_graph(50, 100)
    u = s.submit_update(g, *_upd(4), arrival=1.0)
    b = s.submit_bfs(g, [0], arrival=2.0)
    assert s.run_round(0.5)["updates"] == 0  # nothing has arrived yet
    assert s.queued()[:2] == (2, 4) and s.queued()[2] == 1.0
    s.run_round(1.5)
    assert s.last_round() == [u]  # the search arrives later
    assert s.poll(b)["state"] == 0
    s.run_round(2.0)
    assert s.last_round() == [b]
    assert s.queued()[0] == 0 and s.queued()[2] == float("inf")
    info = s.poll(b, release=True)
    assert info["arrival"] == 2.0 and info["round"] == 2
    with pytest.raises(G.GPMAError):
        s.poll(b)  # released
    s.close()


def test_bfs_lanes_packed_up_to_64(G):
    s = G.Server(plan_only=True)
    g = s.add_graph(1000, 10)
    ids = [s.submit_bfs(g, np.arange(30) + i, arrival=0.0) for i in range(3)]
    r = s.run_round(0.0)
    assert (r["bfs_requests"], r["sources"], r["bfs_graphs"]) == (2, 60, 1)
    assert [s.poll(i)["lane"] for i in ids[:2]] == [0, 30]
    s.run_round(0.0)
    assert s.last_round() == [ids[2]] and s.poll(ids[2])["lane"] == 0
    with pytest.raises(G.GPMAError):
        s.submit_bfs(g, np.arange(65), arrival=0.0)
    with pytest.raises(G.GPMAError):
        s.submit_bfs(g, [1000], arrival=0.0)  # out of range
    s.close()


def test_round_key_cap_and_graph_cap(G):
    s = G.Server(plan_only=True, max_round_keys=1000, max_round_bfs_graphs=2)
    gs = [s.add_graph(10, 100) for _ in range(4)]
    a = s.submit_update(gs[0], *_upd(600), arrival=0.0)
    b = s.submit_update(gs[1], *_upd(600), arrival=0.0)
    c = s.submit_update(gs[2], *_upd(5000), arrival=0.0)  # larger than the cap: runs alone
    s.run_round(0.0)
    assert s.last_round() == [a]
    s.run_round(0.0)
    assert s.last_round() == [b]
    s.run_round(0.0)
    assert s.last_round() == [c]
    q = [s.submit_bfs(g, [1], arrival=0.0) for g in gs]
    s.run_round(0.0)
    assert s.last_round() == q[:2]
    s.run_round(0.0)
    assert s.last_round() == q[2:]
    s.close()


def test_queue_full_is_busy_until_a_round_runs(G):
    s = G.Server(plan_only=True, max_queued=3, max_queued_keys=100)
    g = s.add_graph(10, 10)
    for _ in range(3):
        s.submit_bfs(g, [0], arrival=0.0)
    with pytest.raises(G.GPMAError) as e:
        s.submit_bfs(g, [0], arrival=0.0)
    assert e.value.status == G.ERR_BUSY
    s.run_round(0.0)
    s.submit_update(g, *_upd(60), arrival=0.0)
    with pytest.raises(G.GPMAError) as e:
        s.submit_update(g, *_upd(60), arrival=0.0)  # 120 waiting keys > 100
    assert e.value.status == G.ERR_BUSY
    s.close()


def test_hbm_budget_admission(G):
    budget = 64 << 20
    s = G.Server(plan_only=True, hbm_budget_bytes=budget, max_round_keys=1 << 16)
    g = s.add_graph(1000, 100_000)
    base = s.committed_bytes()
    assert 0 < base <= budget
    with pytest.raises(G.GPMAError) as e:
        s.add_graph(1_000_000, 10_000_000)  # about 300 MB
    assert e.value.status == G.ERR_BUDGET
    assert s.committed_bytes() == base
    # deletes cannot grow the graph; 3M insertions cannot fit the budget at all
    d = s.submit_update(g, *_upd(1000, inserts=False), arrival=0.0)
    s.run_round(0.0)
    assert s.poll(d)["state"] == 1
    keys = np.zeros(1, np.uint64)
    big = s.submit_update(g, np.repeat(keys, 3_000_000), np.ones(3_000_000, np.uint8), arrival=0.0)
    r = s.run_round(0.0)
    assert r["failed"] == 1
    p = s.poll(big)
    assert p["state"] == 2 and p["status"] == G.ERR_BUDGET
    s.close()


def test_replay_keeps_per_graph_order(G):
    """The virtual-time driver over a plan-only server: every request runs
    once; per graph, requests run in arrival order, at most one update per
    round, and a search shares a round only with the update queued before it."""
    import gpma_bfs_gb300.serving as S
    from gpma_bfs_gb300.workloads import SlidingStream

    rng = np.random.default_rng(3)
    specs = []
    for i in range(6):
        n = 1 << int(rng.integers(6, 10))
        keys = np.unique(rng.integers(0, n, 4 * n).astype(np.uint64) << np.uint64(32)
                         | rng.integers(0, n, 4 * n).astype(np.uint64))
        specs.append((n, rng.permutation(keys)))
    trace = S.make_trace(specs, [(500.0, 1.0), (20000.0, 0.05)], seed=9, min_batch=10, max_batch=400)
    # plan-only rounds take no time: bucket the arrivals so that requests coincide
    trace.arrival = np.floor(trace.arrival * 100.0) / 100.0
    srv = G.Server(plan_only=True, max_round_keys=600)
    gids = [srv.add_graph(n, len(k)) for n, k in specs]
    out = S.replay_served(srv, gids, [SlidingStream(k) for _, k in specs], trace)
    assert out["ok"].all() and len(out["done"]) == len(trace)
    seen = sorted(i for r in out["rounds"] for i in r["requests"])
    assert seen == list(range(len(trace)))
    round_of = np.zeros(len(trace), np.int64)
    for k, r in enumerate(out["rounds"]):
        assert r["keys"] <= 600 or r["updates"] == 1
        for i in r["requests"]:
            round_of[i] = k
    for g in range(len(specs)):
        idx = np.nonzero(trace.graph == g)[0]  # arrival order
        assert np.all(np.diff(round_of[idx]) >= 0)
        for k in np.unique(round_of[idx]):
            mine = idx[round_of[idx] == k]
            kinds = trace.kind[mine]
            assert (kinds == 0).sum() <= 1
            if (kinds == 0).any():
                assert kinds[0] == 0  # the update is the first of the graph's requests in the round
    assert max(r["updates"] for r in out["rounds"]) > 1  # the burst batched several graphs
    srv.close()


def test_replay_waits_when_the_queue_is_full(G):
    """Admission control: with room for 4 requests the driver holds the rest
    back until rounds free slots; every request still runs, in order."""
    import gpma_bfs_gb300.serving as S
    from gpma_bfs_gb300.workloads import SlidingStream

    rng = np.random.default_rng(5)
    specs = [(1024, rng.permutation(np.arange(1, 600, dtype=np.uint64) << np.uint64(32) | np.uint64(7)))
             for _ in range(3)]
    trace = S.make_trace(specs, [(1000.0, 0.2)], seed=2, min_batch=4, max_batch=40)
    trace.arrival = np.zeros(len(trace))  # everything arrives at once
    srv = G.Server(plan_only=True, max_queued=4)
    gids = [srv.add_graph(n, len(k)) for n, k in specs]
    out = S.replay_served(srv, gids, [SlidingStream(k) for _, k in specs], trace)
    assert out["ok"].all()
    assert max(len(r["requests"]) for r in out["rounds"]) <= 4
    assert sorted(i for r in out["rounds"] for i in r["requests"]) == list(range(len(trace)))
    big = G.Server(plan_only=True, max_queued_keys=10)
    gid = big.add_graph(64, 10)
    with pytest.raises(G.GPMAError):
        big.submit_update(gid, *_upd(11), arrival=0.0)  # never admissible
    srv.close()
    big.close()


def test_cancel_withdraws_queued_requests_only(G):
    """A client that goes away: its queued request leaves the queue (keys no
    longer count), the graph's other requests keep their order, and a request
    that already ran cannot be cancelled."""
    s = G.Server(plan_only=True, max_queued_keys=25)
    g0, g1 = s.add_graph(100, 1000), s.add_graph(100, 1000)
    u1 = s.submit_update(g0, *_upd(10), arrival=0.0)
    u2 = s.submit_update(g0, *_upd(10), arrival=0.1)
    b1 = s.submit_bfs(g0, [1], arrival=0.2, levels=True)
    b2 = s.submit_bfs(g1, [2], arrival=0.0)
    with pytest.raises(G.GPMAError) as e:
        s.submit_update(g1, *_upd(10), arrival=0.3)  # 30 keys would wait: over max_queued_keys
    assert e.value.status == G.ERR_BUSY
    s.cancel(u2)
    assert s.queued()[:2] == (3, 10)
    u3 = s.submit_update(g1, *_upd(10), arrival=0.3)  # fits now
    s.cancel(b2)
    assert s.poll(u2)["state"] == 3 and s.poll(b2)["state"] == 3 and s.levels(b2) is None
    s.run_round(1.0)
    # u1 then the search behind it (u2 is gone); g1's head is now its update
    assert s.last_round() == [u1, u3, b1]
    assert s.poll(b1)["state"] == 1
    with pytest.raises(G.GPMAError):
        s.cancel(u1)  # already ran
    with pytest.raises(G.GPMAError):
        s.cancel(12345)  # unknown
    assert s.poll(u2, release=True)["state"] == 3
    with pytest.raises(G.GPMAError):
        s.poll(u2)  # released
    assert s.queued()[0] == 0 and s.run_round(2.0)["updates"] == 0
    s.close()


def test_cancelled_update_frees_the_graph_for_its_searches(G):
    """An update that must wait (the round's key limit is taken by an earlier
    graph) holds back the searches queued behind it; cancelled, it no longer
    does, and they run in the same round."""
    def scenario(cancel):
        s = G.Server(plan_only=True, max_round_keys=20)
        g0, g1 = s.add_graph(100, 1000), s.add_graph(100, 1000)
        first = s.submit_update(g1, *_upd(15), arrival=0.0)
        late = s.submit_update(g0, *_upd(10), arrival=0.1)
        b = s.submit_bfs(g0, [5], arrival=0.1)
        if cancel:
            s.cancel(late)
        s.run_round(1.0)
        ran = s.last_round()
        s.close()
        return ran, first, late, b

    ran, first, late, b = scenario(cancel=False)
    assert ran == [first]  # g0's update waits for the next round, its search with it
    ran, first, late, b = scenario(cancel=True)
    assert ran == [first, b]


def test_serving_loop_runs_requests_after_their_arrival(G):
    """The native serving loop (two lanes, plan-only): requests submitted
    ahead of their arrival run once the server's clock passes it, every one
    exactly once, per graph in arrival order with at most one update per
    round, and drain returns once nothing is queued or running."""
    import gpma_bfs_gb300.serving as S
    from gpma_bfs_gb300.workloads import SlidingStream

    rng = np.random.default_rng(11)
    specs = []
    for i in range(5):
        n = 1 << int(rng.integers(6, 9))
        keys = np.unique(rng.integers(0, n, 4 * n).astype(np.uint64) << np.uint64(32)
                         | rng.integers(0, n, 4 * n).astype(np.uint64))
        specs.append((n, rng.permutation(keys)))
    trace = S.make_trace(specs, [(2000.0, 0.1), (20000.0, 0.02)], seed=12, min_batch=10, max_batch=300)
    srv = G.Server(plan_only=True, lanes=2, max_round_keys=500)
    gids = [srv.add_graph(n, len(k)) for n, k in specs]
    out = S.replay_served_live(srv, gids, [SlidingStream(k) for _, k in specs], trace, timeout=30.0)
    assert out["ok"].all() and len(out["done"]) == len(trace)
    assert np.all(out["start"] >= trace.arrival - 1e-9)  # nothing ran before it arrived
    st = out["stats"]
    assert st["requests"] == len(trace) and st["rounds"] >= 1
    for g in range(len(specs)):
        idx = np.nonzero(trace.graph == g)[0]
        rounds = out["round"][idx]
        assert np.all(np.diff(rounds) >= 0)  # a graph's requests in arrival order
        for k in np.unique(rounds):
            assert (trace.kind[idx][rounds == k] == 0).sum() <= 1
    assert srv.queued()[0] == 0
    srv.close()


def test_serving_loop_start_stop_and_lane_limits(G):
    with pytest.raises(G.GPMAError):
        G.Server(plan_only=True, lanes=5)
    s = G.Server(plan_only=True, lanes=3)
    g = s.add_graph(16, 10)
    s.start()
    with pytest.raises(G.GPMAError):
        s.start()  # already running
    t = s.clock()
    rid = s.submit_bfs(g, [1], arrival=t + 0.05)
    assert s.poll(rid)["state"] == 0  # not yet arrived
    s.drain(10.0)
    p = s.poll(rid)
    assert p["state"] == 1 and p["start"] >= t + 0.05
    s.stop()
    s.stop()  # idempotent
    s.close()


def test_input_ring_takes_what_fits_and_reuses_space(G):
    """Queued batches go to the input ring while it has room (the rest stay in
    host vectors); completed and cancelled requests give their space back,
    also across the ring's wrap-around, and every request still runs once."""
    s = G.Server(plan_only=True, input_ring_bytes=4096, max_round_keys=1 << 20)
    g = [s.add_graph(64, 1000) for _ in range(3)]
    rng = np.random.default_rng(5)
    ids = []
    for step in range(40):
        for gi in g:
            n = int(rng.integers(1, 200))  # 9 B per key: up to 1.8 KB, so the ring fills and wraps
            ids.append(s.submit_update(gi, *_upd(n), arrival=float(step)))
        if step % 7 == 3:
            s.cancel(ids[-1])
        s.run_round(float(step))
    while s.queued()[0]:
        s.run_round(1e9)
    states = [s.poll(i)["state"] for i in ids]
    assert all(x in (1, 3) for x in states) and states.count(3) == 6
    s.close()
