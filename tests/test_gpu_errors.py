"""Error paths of the bounded device-side waits, run on the GPU without
hanging it.

Every grid barrier and look-back of the library gives up after a time limit
and the call returns GPMA_ERR_TIMEOUT. The test hooks make the first grid
barrier of an update (or BFS) launch wait for an arrival that never comes,
with a 50 ms limit: the call must return GPMA_ERR_TIMEOUT, leave the
structure unchanged, and the next calls must give the oracle's results bit
for bit (the stalled launch's leftover barrier, status and sort state are
cleared by the next launch).
"""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # GPMA_ERR_TIMEOUT


@pytest.fixture()
def hooks(built_lib):
    import gpma_bfs_gb300 as G

    yield G
    G.set_test_hooks(update_stall=0, bfs_stall=0, wait_limit_us=0, noalloc_chunk_cap=0)


def _same(g, o, ctx):
    gk, gv, gr = g.export_layout()
    ok, ov, orow = o.export_layout()
    assert g.geometry() == o.geometry(), ctx
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov) and np.array_equal(gr, orow), ctx
    assert g.validate() == 0, ctx


def test_stalled_update_barrier_times_out_and_the_next_update_is_exact(hooks):
    G = hooks
    from gpma_bfs_gb300.workloads import make_graph, sliding_window

    n, src, dst = make_graph(dict(kind="rmat", scale=12, edge_factor=16, seed=61))
    sw = sliding_window(src, dst, 100)
    g, o = G.GPMA(n), OracleGPMA(n, threads=4)
    G.update_gpma(g, sw.load_keys, sw.load_values)
    o.update(sw.load_keys, sw.load_values)
    _same(g, o, "load")

    G.set_test_hooks(update_stall=1, wait_limit_us=50_000)
    for i in range(2):  # twice: the second stalled launch starts from the first one's leftovers
        with pytest.raises(G.GPMAError) as e:
            G.update_gpma(g, sw.slide_keys[i], sw.slide_values[i])
        assert e.value.status == TIMEOUT
        assert b"gave up" in G.lib().gpma_last_error()
        _same(g, o, f"after stalled update {i}")  # nothing applied
    G.set_test_hooks(update_stall=0, wait_limit_us=0)

    for i in range(6):
        G.update_gpma(g, sw.slide_keys[i], sw.slide_values[i])
        o.update(sw.slide_keys[i], sw.slide_values[i])
        _same(g, o, f"slide {i} after the timeout")
    gl, gr = G.gpma_bfs(g, n, 0, 0)
    ol, orr = o.bfs(0)
    assert gr == orr and np.array_equal(gl, ol)
    g.close()
    o.close()


def test_stalled_bfs_barrier_times_out_and_the_next_bfs_is_exact(hooks):
    G = hooks
    from gpma_bfs_gb300.workloads import make_graph

    n, src, dst = make_graph(dict(kind="rmat", scale=12, edge_factor=16, seed=62))
    keys = G.edges_to_keys(src, dst)
    g, o = G.GPMA(n), OracleGPMA(n, threads=4)
    G.update_gpma(g, keys, np.ones(len(keys), np.uint8))
    o.update(keys, np.ones(len(keys), np.uint8))
    ol, orr = o.bfs(int(src[0]))
    G.set_test_hooks(bfs_stall=1, wait_limit_us=50_000)
    with pytest.raises(G.GPMAError) as e:
        G.gpma_bfs(g, n, 0, int(src[0]))
    assert e.value.status == TIMEOUT
    G.set_test_hooks(bfs_stall=0, wait_limit_us=0)
    gl, gr = G.gpma_bfs(g, n, 0, int(src[0]))
    assert gr == orr and np.array_equal(gl, ol)
    # and the update path is untouched by the BFS's failure
    more = keys[: len(keys) // 4]
    G.update_gpma(g, more, np.zeros(len(more), np.uint8))
    o.update(more, np.zeros(len(more), np.uint8))
    _same(g, o, "deletes after the BFS timeout")
    g.close()
    o.close()
