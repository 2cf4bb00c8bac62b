"""Tuning changes speed, never results: BFS (single and multi-source) and
updates under every switch setting and grid shape equal the oracle."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu

SETTINGS = [
    dict(bfs_dense_div=0, ms_dense_div=0),                    # rows only
    dict(bfs_dense_div=1 << 30, ms_dense_div=1 << 30),        # every level sweeps all slots
    dict(bfs_dense_div=4, ms_dense_div=4),                    # a middle switch point
    dict(bfs_dense_div=16, ms_dense_div=2, bfs_blocks_per_sm=1, ms_blocks_per_sm=3, update_blocks_per_sm=1),
]


@pytest.fixture
def restore_tuning(built_lib):
    import gpma_bfs_gb300 as G

    old = G.get_tuning()
    yield G
    G.set_tuning(**old)


def _graphs():
    import gpma_bfs_gb300 as G

    out = []
    for scale, ef, seed in ((9, 8, 1), (12, 4, 2), (14, 16, 3)):
        src, dst = G.gen_rmat(scale, ef, seed=seed)
        out.append((1 << scale, G.edges_to_keys(src, dst)))
    return out


@pytest.mark.parametrize("setting", SETTINGS)
def test_bfs_results_independent_of_tuning(restore_tuning, setting):
    G = restore_tuning
    G.set_tuning(**setting)
    rng = np.random.default_rng(2)
    gs, orcs, srcs = [], [], []
    for n, keys in _graphs():
        half = len(keys) // 2
        g, o = G.GPMA(n), OracleGPMA(n, threads=4)
        for part in (keys[:half], keys[half: half + half // 3]):
            G.update_gpma(g, part, np.ones(len(part), np.uint8))
            o.update(part, np.ones(len(part), np.uint8))
        dels = keys[: half // 4]  # tombstones inside rows
        G.update_gpma(g, dels, np.zeros(len(dels), np.uint8))
        o.update(dels, np.zeros(len(dels), np.uint8))
        assert all(np.array_equal(x, y) for x, y in zip(g.export_layout(), o.export_layout()))
        start = int(keys[0] >> np.uint64(32))
        lv, reached = G.gpma_bfs(g, n, len(keys), start)
        ol, orr = o.bfs(start)
        assert np.array_equal(lv, ol) and reached == orr
        gs.append(g)
        orcs.append(o)
        srcs.append(rng.choice(n, 64, replace=False).astype(np.uint32))
    b = G.Batch()
    b.set_profiling(True)
    levels, reached = b.bfs_multi(gs, srcs, levels=True)
    want_edges = 0
    for i, o in enumerate(orcs):
        ol, orr = o.bfs_multi(srcs[i])
        assert np.array_equal(levels[i], ol) and np.array_equal(reached[i], orr), f"graph {i}"
        want_edges += sum(o.traversed_edges(row) for row in ol)
    assert b.profile()["bfs_edges"] == want_edges
    b.close()


def test_update_results_independent_of_grid(restore_tuning):
    G = restore_tuning
    n, keys = _graphs()[1]
    layouts = []
    for blocks in (1, 3, 0):  # the 128-register build at 1 CTA/SM, the 80-register build, automatic
        G.set_tuning(update_blocks_per_sm=blocks)
        g = G.GPMA(n)
        for i in range(0, len(keys), 7000):
            G.update_gpma(g, keys[i:i + 7000], np.ones(len(keys[i:i + 7000]), np.uint8))
        layouts.append(g.export_layout())
        g.close()
    assert all(all(np.array_equal(x, y) for x, y in zip(layouts[0], other)) for other in layouts[1:])


def test_set_tuning_rejects_bad_grid(restore_tuning):
    G = restore_tuning
    with pytest.raises(G.GPMAError):
        G.set_tuning(bfs_blocks_per_sm=33)
    with pytest.raises(ValueError):
        G.set_tuning(nonsense=1)
