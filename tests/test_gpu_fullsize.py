"""The social-network sliding window at full size (1,632,803 nodes,
30,622,564 edges: the first half loaded in one bulk batch, then slides of
153,112 inserts + 153,112 deletes).

test_social_sliding_window_matches_oracle runs the whole schedule -- bulk
load, BFS from node 0, all 100 slides, BFS from node 0 -- through the CUDA
path and the oracle side by side and compares, after the load and after
every slide, the full key layout, the values (masked where the key is
empty), row_offset, geometry and density thresholds, and both BFS level
arrays and reach counts: bit-exact.

test_social_sliding_window_full_size checks properties that hold at any
size on the same configuration:

* the live edge set equals the window's edges exactly;
* layout invariants: live slots strictly ascending, row r's guard at
  row_offset[r + 1], every edge inside its source row's slot range, the
  cached segment heads consistent (validate);
* idempotence: re-applying the last slide (its inserts are now modifies of
  live keys, its deletes hit deleted keys) leaves the layout bit-identical;
* round trip: inserting fresh edges and deleting them again restores the
  live edge set;
* BFS levels and reach equal a level-synchronous BFS over the window's
  edges in numpy; the multi-source BFS's levels equal single-source BFS.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEY_NONE = np.uint64(0xFFFFFFFFFFFFFFFF)
KEY_MAX = np.uint64(0xFFFFFFFFFFFFFFFE)
LOW = np.uint64(0xFFFFFFFF)


def _edges_of(compact):
    """Sorted edge keys of a compacted key array (guards and sentinels removed)."""
    return compact[(compact != KEY_MAX) & ((compact & LOW) != LOW)]


def _numpy_bfs(n, edge_keys, s):
    """Levels (source 1, unreached 0) of a level-synchronous BFS over sorted edge keys."""
    src = (edge_keys >> np.uint64(32)).astype(np.int64)
    dst = (edge_keys & LOW).astype(np.int64)
    indptr = np.searchsorted(src, np.arange(n + 1, dtype=np.int64))
    levels = np.zeros(n, np.uint32)
    levels[s] = 1
    frontier = np.array([s], np.int64)
    level = 1
    while len(frontier):
        starts = indptr[frontier]
        lens = indptr[frontier + 1] - starts
        total = int(lens.sum())
        if total == 0:
            break
        first = np.cumsum(lens) - lens
        offs = np.repeat(starts - first, lens) + np.arange(total)
        mark = np.zeros(n, bool)
        mark[dst[offs]] = True
        frontier = np.flatnonzero(mark & (levels == 0))
        level += 1
        levels[frontier] = level
    return levels


def test_social_sliding_window_full_size(built_lib):
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph, sliding_window

    n, src, dst = make_graph("social")
    sw = sliding_window(src, dst, num_slide=100)
    keys = G.edges_to_keys(src, dst)
    half, step = sw.half, sw.step
    assert (n, len(keys), step) == (1_632_803, 30_622_564, 153_112)
    g = G.GPMA(n)
    G.update_gpma(g, sw.load_keys, sw.load_values)
    assert g.stats()["significant"] == 1  # >= 5M insertions: the bulk rebuild
    slides = 3
    for i in range(slides):
        G.update_gpma(g, sw.slide_keys[i], sw.slide_values[i])

    # the live edge set is exactly the window
    window = np.sort(keys[slides * step: half + slides * step])
    live = _edges_of(g.compact_keys())
    assert np.array_equal(live, window)

    # layout invariants
    assert g.validate() == 0
    lk, lv, ro = g.export_layout()
    assert len(lk) == g.get_size() and ro[0] == 0
    occupied = (lv != 0) & (lk != KEY_NONE)
    ok = lk[occupied & (lk != KEY_MAX)]
    assert np.all(ok[1:] > ok[:-1]), "live slots out of order"
    # the two KEY_MAX sentinels of the initial layout sort after everything
    sentinels = np.flatnonzero(occupied & (lk == KEY_MAX))
    assert len(sentinels) == 2 and sentinels.min() > np.flatnonzero(occupied & (lk != KEY_MAX)).max()
    rows = np.arange(n, dtype=np.uint64)
    assert np.array_equal(lk[ro[1:]], (rows << np.uint64(32)) | LOW), "a guard is not at row_offset[row + 1]"
    slots = np.flatnonzero(occupied & (lk != KEY_MAX) & ((lk & LOW) != LOW))
    esrc = (lk[slots] >> np.uint64(32)).astype(np.int64)
    # row r's slots are [row_offset[r], row_offset[r + 1]): row_offset[r] is
    # row r - 1's guard slot, or 0 for row 0, whose first edge may sit there
    assert np.all((ro[esrc] <= slots) & (slots < ro[esrc + 1])), "an edge outside its row's slot range"
    assert len(slots) == len(window)

    # idempotence: the last slide again changes nothing
    G.update_gpma(g, sw.slide_keys[slides - 1], sw.slide_values[slides - 1])
    lk2, lv2, ro2 = g.export_layout()
    assert np.array_equal(lk2, lk) and np.array_equal(lv2, lv) and np.array_equal(ro2, ro)
    del lk2, lv2, ro2

    # BFS from node 0 against numpy over the window's edges
    want = _numpy_bfs(n, window, 0)
    got, reached = G.gpma_bfs(g, n, len(window), 0)
    assert np.array_equal(got, want) and reached == int((want > 0).sum())

    # multi-source BFS: each lane equals the single-source BFS
    rng = np.random.default_rng(26)
    sources = rng.choice(n, 8, replace=False).astype(np.uint32)
    multi, mreached = G.gpma_bfs_multi(g, sources)
    for j, s in enumerate(sources):
        one, r = G.gpma_bfs(g, n, len(window), int(s))
        assert np.array_equal(multi[j], one) and mreached[j] == r, f"source {s}"

    # round trip: fresh edges in, then out again
    fresh = keys[half + slides * step: half + slides * step + 200_000]
    G.update_gpma(g, fresh, np.ones(len(fresh), np.uint8))
    assert len(_edges_of(g.compact_keys())) == len(window) + len(fresh)
    G.update_gpma(g, fresh, np.zeros(len(fresh), np.uint8))
    assert np.array_equal(_edges_of(g.compact_keys()), window)
    assert g.validate() == 0
    g.close()


def test_social_sliding_window_matches_oracle(built_lib):
    """Every step of the full social schedule, GPU against the oracle, bit for
    bit (gpma_bfs_demo.cu:85-112: load, BFS, 100 slides, BFS)."""
    import os

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph, sliding_window
    from oracle.oracle import OracleGPMA

    n, src, dst = make_graph("social")
    sw = sliding_window(src, dst, num_slide=100)
    del src, dst
    assert (n, sw.half, sw.step, sw.num_slide) == (1_632_803, 15_311_282, 153_112, 100)
    g = G.GPMA(n)
    o = OracleGPMA(n, threads=os.cpu_count() or 1)

    def compare(ctx):
        assert g.geometry() == o.geometry(), ctx + ": geometry"
        glo, ghi = g.thresholds()
        olo, ohi = o.thresholds()
        assert np.array_equal(glo, olo) and np.array_equal(ghi, ohi), ctx + ": density thresholds"
        gk, gv, gr = g.export_layout()
        ok, ov, orow = o.export_layout()
        assert np.array_equal(gk, ok), ctx + ": key layout"
        assert np.array_equal(gv, ov), ctx + ": values"
        assert np.array_equal(gr, orow), ctx + ": row_offset"

    def bfs(ctx):
        gl, gr = G.gpma_bfs(g, n, 0, 0)
        ol, orr = o.bfs(0)
        assert gr == orr and np.array_equal(gl, ol), ctx + ": BFS from node 0"
        return gr

    G.update_gpma(g, sw.load_keys, sw.load_values)
    o.update(sw.load_keys, sw.load_values)
    assert g.stats()["significant"] == 1  # >= 5M insertions: the bulk rebuild
    compare("after the bulk load")
    before = bfs("before the slides")
    for i in range(sw.num_slide):
        G.update_gpma(g, sw.slide_keys[i], sw.slide_values[i])
        o.update(sw.slide_keys[i], sw.slide_values[i])
        compare(f"slide {i}")
    after = bfs("after the slides")
    assert before > n // 2 and after > n // 2  # the giant component is reached
    assert g.validate() == 0
    g.close()
    o.close()
