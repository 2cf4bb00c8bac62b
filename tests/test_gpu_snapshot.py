"""Snapshot and resume: the loaded graph has exactly the saved layout, and
the same updates afterwards give the same layouts as without the resume."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def test_save_load_resume_is_layout_exact(built_lib, tmp_path):
    import gpma_bfs_gb300 as G

    src, dst = G.gen_rmat(12, 8, seed=11)
    n = 1 << 12
    keys = G.edges_to_keys(src, dst)
    g, o = G.GPMA(n), OracleGPMA(n, threads=2)
    first = keys[: len(keys) // 2]
    G.update_gpma(g, first, np.ones(len(first), np.uint8))
    o.update(first, np.ones(len(first), np.uint8))
    dels = first[::5]
    G.update_gpma(g, dels, np.zeros(len(dels), np.uint8))  # tombstones in the snapshot
    o.update(dels, np.zeros(len(dels), np.uint8))
    G.save(g, tmp_path / "g.snap")
    r = G.load(tmp_path / "g.snap")
    assert r.geometry() == g.geometry() and r.row_num == n
    assert all(np.array_equal(x, y) for x, y in zip(r.thresholds(), g.thresholds()))
    assert all(np.array_equal(x, y) for x, y in zip(r.export_layout(), g.export_layout()))
    assert r.validate() == 0
    rest = keys[len(keys) // 2:]
    for i in range(0, len(rest), 3000):
        k = rest[i:i + 3000]
        v = np.ones(len(k), np.uint8)
        for x in (g, r):
            G.update_gpma(x, k, v)
        o.update(k, v)
        assert all(np.array_equal(x, y) for x, y in zip(r.export_layout(), o.export_layout()))
    assert all(np.array_equal(x, y) for x, y in zip(r.export_layout(), g.export_layout()))
    lv, reached = G.gpma_bfs(r, n, len(keys), int(src[0]))
    ol, orr = o.bfs(int(src[0]))
    assert np.array_equal(lv, ol) and reached == orr
    r.close()
    g.close()
