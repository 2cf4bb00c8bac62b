"""The large-graph batch sweep's operations at a size the oracle checks in
seconds: an R-MAT graph loaded except for a reserve of fresh edges, then
batches of growing size at insert:delete ratios 1:0, 1:1 and 0:1 (deletes
drawn uniformly from live edges), bit-exact after every batch, then BFS from
random non-isolated sources."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def test_batch_sweep_ratios_match_oracle(built_lib):
    import gpma_bfs_gb300 as G

    src, dst = G.gen_rmat(13, 16, seed=3)
    n = 1 << 13
    keys = G.edges_to_keys(src, dst)
    sizes = [100, 1_000, 10_000]
    ratios = [(1, 0), (1, 1), (0, 1)]
    reserve = sum(s * i // (i + d) for s in sizes for i, d in ratios)
    loaded, fresh = keys[:-reserve], keys[-reserve:]
    rng = np.random.default_rng(3)
    order = rng.permutation(len(loaded))
    g, o = G.GPMA(n), OracleGPMA(n, threads=4)
    for part in (loaded[: len(loaded) // 2], loaded[len(loaded) // 2:]):
        G.update_gpma(g, part, np.ones(len(part), np.uint8))
        o.update(part, np.ones(len(part), np.uint8))
    fi = di = 0
    for ins, dels in ratios:
        for size in sizes:
            ni = size * ins // (ins + dels)
            nd = size - ni
            k = np.concatenate([fresh[fi:fi + ni], loaded[order[di:di + nd]]])
            v = np.concatenate([np.ones(ni, np.uint8), np.zeros(nd, np.uint8)])
            fi, di = fi + ni, di + nd
            G.update_gpma(g, k, v)
            o.update(k, v)
            ctx = f"ratio {ins}:{dels} batch {size}"
            assert g.geometry() == o.geometry(), ctx
            assert all(np.array_equal(x, y) for x, y in zip(g.export_layout(), o.export_layout())), ctx
    live = o.compact_keys()
    live = live[(live & np.uint64(0xFFFFFFFF)) < np.uint64(0xFFFFFFFE)]
    for s in rng.choice(np.unique(live >> np.uint64(32)), 4, replace=False):
        lv, reached = G.gpma_bfs(g, n, len(keys), int(s))
        ol, orr = o.bfs(int(s))
        assert np.array_equal(lv, ol) and reached == orr
    g.close()
