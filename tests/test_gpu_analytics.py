"""PageRank and weakly connected components over the gapped array, against
plain CPU computations on the graph's live edge set (taken from the oracle
after the same updates, tombstones included)."""
import numpy as np
import pytest

from oracle.oracle import OracleGPMA

pytestmark = pytest.mark.gpu


def _graph():
    import gpma_bfs_gb300 as G

    n = 1 << 12
    src, dst = G.gen_rmat(12, 6, seed=21)
    keys = G.edges_to_keys(src, dst)
    g, o = G.GPMA(n), OracleGPMA(n, threads=2)
    for k, v in ((keys, np.ones(len(keys), np.uint8)), (keys[::3], np.zeros(len(keys[::3]), np.uint8))):
        G.update_gpma(g, k, v)
        o.update(k, v)
    live = o.compact_keys()
    s, d = (live >> np.uint64(32)).astype(np.int64), (live & np.uint64(0xFFFFFFFF)).astype(np.int64)
    edge = (d != 0xFFFFFFFF) & (s < n) & (d < n)
    return G, g, n, s[edge], d[edge]


def test_components_equal_scipy(built_lib):
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    G, g, n, s, d = _graph()
    labels, count, rounds = G.components(g)
    a = sp.csr_matrix((np.ones(len(s)), (s, d)), shape=(n, n))
    ncomp, lab = csgraph.connected_components(a, directed=True, connection="weak")
    # canonical labels: the smallest node id of each component
    first = np.full(ncomp, n, np.int64)
    np.minimum.at(first, lab, np.arange(n))
    assert count == ncomp and rounds >= 1
    assert np.array_equal(labels, first[lab].astype(np.uint32))
    g.close()


def _pagerank_f64(n, s, d, damping, iterations):
    deg = np.bincount(s, minlength=n).astype(np.float64)
    r = np.full(n, 1.0 / n)
    for _ in range(iterations):
        contrib = np.where(deg > 0, r / np.maximum(deg, 1), 0.0)
        dangling = r[deg == 0].sum()
        acc = np.bincount(d, weights=contrib[s], minlength=n)
        r = (1 - damping) / n + damping * (acc + dangling / n)
    return r


def test_pagerank_matches_float64_power_iteration(built_lib):
    G, g, n, s, d = _graph()
    want = _pagerank_f64(n, s, d, 0.85, 30)
    got, iters = G.pagerank(g, 0.85, 30)
    assert iters == 30
    # float32 ranks with float atomics: within 2e-4 relative (+1e-8 absolute) of float64
    np.testing.assert_allclose(got, want, rtol=2e-4, atol=1e-8)
    assert abs(got.sum() - 1.0) < 1e-3
    # with a tolerance the iteration stops early and is still close to the fixed point
    conv, it2 = G.pagerank(g, 0.85, 500, tol=1e-7)
    assert it2 < 500
    np.testing.assert_allclose(conv, _pagerank_f64(n, s, d, 0.85, 200), rtol=1e-3, atol=1e-8)
    g.close()


def test_analytics_on_device_outputs_and_empty_edges(built_lib):
    import torch

    import gpma_bfs_gb300 as G

    g = G.GPMA(100)  # guards only: every node is isolated and dangling
    lab = torch.zeros(100, dtype=torch.int32, device="cuda")
    _, count, _ = G.components(g, lab)
    assert count == 100 and np.array_equal(lab.cpu().numpy(), np.arange(100))
    r = torch.zeros(100, dtype=torch.float32, device="cuda")
    G.pagerank(g, 0.85, 5, out=r)
    np.testing.assert_allclose(r.cpu().numpy(), np.full(100, 0.01), rtol=1e-5)
    g.close()
