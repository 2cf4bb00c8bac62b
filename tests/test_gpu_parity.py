"""CUDA path vs the reference (golden vectors) and vs the oracle, through the C ABI.

Bit-exact: integer/index work, so layout keys, values, row_offset,
thresholds, geometry and BFS levels must be identical after every operation.
"""
import numpy as np
import pytest

import cases
from oracle.oracle import OracleGPMA
from replay import GpuAdapter, load_case, record_after_update, replay_and_compare

pytestmark = pytest.mark.gpu

GOLDEN = list(cases.SMALL) + ["rmat8_slide", "rmat12_slide", "rmat16_slide", "rmat20_bulk"]


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


@pytest.mark.parametrize("name", GOLDEN)
def test_gpu_matches_reference_golden(name):
    n, ops, z = load_case(name)
    g = GpuAdapter(n)
    ui, bi, _ = replay_and_compare(g, ops, z)
    assert ui == len(z["rec_size"]) and bi == len(z["bfs_src"])
    g.close()


def _compare_full(gpu, orc, ctx):
    gk, gv, gr = gpu.export_layout()
    ok, ov, orow = orc.export_layout()
    assert gpu.geometry() == orc.geometry(), ctx
    assert np.array_equal(gk, ok), ctx + ": key layout"
    assert np.array_equal(gv, ov), ctx + ": values"
    assert np.array_equal(gr, orow), ctx + ": row_offset"
    assert gpu.g.validate() == 0, ctx + ": segment heads differ from the array"


@pytest.mark.parametrize("seed", range(100, 112))
def test_gpu_matches_oracle_random_scripts(seed):
    n, ops = cases.random_case(seed)
    gpu, orc = GpuAdapter(n), OracleGPMA(n, threads=4)
    for i, op in enumerate(ops):
        if op[0] == "update":
            gpu.update(op[1], op[2])
            orc.update(op[1], op[2])
            _compare_full(gpu, orc, f"seed {seed} op {i}")
        elif op[0] == "bfs":
            gl, gr = gpu.bfs(op[1])
            ol, orr = orc.bfs(op[1])
            assert gr == orr and np.array_equal(gl, ol), f"seed {seed} op {i}: bfs"
    gpu.close()


def test_wide_windows_in_level_loop():
    """Windows wider than one CTA (grid path) are rebalanced inside the level
    loop: a burst of insertions into one row of a large structure."""
    n = 1 << 15
    gpu, orc = GpuAdapter(n), OracleGPMA(n, threads=4)
    rng = np.random.default_rng(7)
    for burst in (3000, 9000, 30000):
        row = int(rng.integers(0, n))
        dst = rng.choice(n, burst, replace=False).astype(np.uint64)
        keys = (np.uint64(row) << np.uint64(32)) | dst
        vals = np.ones(burst, np.uint8)
        gpu.update(keys, vals)
        orc.update(keys, vals)
        _compare_full(gpu, orc, f"burst {burst}")
    st = gpu.g.stats()
    assert st["accepted_slots"] > 0
    # then delete most of it again (tombstones) and insert elsewhere
    keys = (np.uint64(5) << np.uint64(32)) | np.arange(4000, dtype=np.uint64)
    gpu.update(keys, np.ones(4000, np.uint8))
    orc.update(keys, np.ones(4000, np.uint8))
    gpu.update(keys[::3], np.zeros(len(keys[::3]), np.uint8))
    orc.update(keys[::3], np.zeros(len(keys[::3]), np.uint8))
    _compare_full(gpu, orc, "after deletes")
    for src in (0, 5, int(rng.integers(0, n))):
        gl, gr = gpu.bfs(src)
        ol, orr = orc.bfs(src)
        assert gr == orr and np.array_equal(gl, ol)
    gpu.close()


def test_sliding_window_rmat14_step_by_step():
    from gpma_bfs_gb300.workloads import make_graph, sliding_window

    n, src, dst = make_graph(dict(kind="rmat", scale=14, edge_factor=16, seed=21))
    sw = sliding_window(src, dst, 100)
    gpu, orc = GpuAdapter(n), OracleGPMA(n, threads=8)
    gpu.update(sw.load_keys, sw.load_values)
    orc.update(sw.load_keys, sw.load_values)
    _compare_full(gpu, orc, "load")
    for i in range(sw.num_slide):
        gpu.update(sw.slide_keys[i], sw.slide_values[i])
        orc.update(sw.slide_keys[i], sw.slide_values[i])
        if i % 10 == 9:
            _compare_full(gpu, orc, f"slide {i}")
    gl, gr = gpu.bfs(0)
    ol, orr = orc.bfs(0)
    assert gr == orr and np.array_equal(gl, ol)
    gpu.close()


def test_sliding_window_chung_lu_20k_every_slide():
    """The social configuration's power-law shape (hub rows of thousands of
    edges, deep windows) at 20,000 nodes and 300,000 edges: half-load, BFS
    from node 0, 100 slides, BFS again; the full layout is compared after
    every operation (the same graph the oracle is checked on against the
    reference binary)."""
    from gpma_bfs_gb300.workloads import make_graph, sliding_window

    n, src, dst = make_graph(dict(kind="chung_lu", n=20000, m=300000, exponent=2.3, max_degree=3000, seed=41))
    sw = sliding_window(src, dst, 100)
    gpu, orc = GpuAdapter(n), OracleGPMA(n, threads=8)
    gpu.update(sw.load_keys, sw.load_values)
    orc.update(sw.load_keys, sw.load_values)
    _compare_full(gpu, orc, "load")
    assert gpu.thresholds()[0].tolist() == orc.thresholds()[0].tolist()
    gl, gr = gpu.bfs(0)
    ol, orr = orc.bfs(0)
    assert gr == orr and np.array_equal(gl, ol), "bfs before the slides"
    for i in range(sw.num_slide):
        gpu.update(sw.slide_keys[i], sw.slide_values[i])
        orc.update(sw.slide_keys[i], sw.slide_values[i])
        _compare_full(gpu, orc, f"slide {i}")
        glo, ghi = gpu.thresholds()
        olo, ohi = orc.thresholds()
        assert np.array_equal(glo, olo) and np.array_equal(ghi, ohi), f"slide {i}: thresholds"
    gl, gr = gpu.bfs(0)
    ol, orr = orc.bfs(0)
    assert gr == orr and np.array_equal(gl, ol), "bfs after the slides"
    gpu.close()


def test_device_pointers_and_torch_tensors():
    import torch

    import gpma_bfs_gb300 as G

    n, ops, z = load_case("rmat8_slide")
    g = G.GPMA(n)
    o = OracleGPMA(n)
    for op in ops:
        if op[0] != "update":
            continue
        k = torch.from_numpy(op[1].view(np.int64)).cuda()
        v = torch.from_numpy(op[2]).cuda()
        G.update_gpma(g, k, v)
        o.update(op[1], op[2])
    gk, gv, gr = g.export_layout()
    ok, ov, orow = o.export_layout()
    assert np.array_equal(gk, ok) and np.array_equal(gr, orow)
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    _, reached = G.gpma_bfs(g, n, 0, 0, out)
    ol, orr = o.bfs(0)
    assert reached == orr
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ol)
    # compacted key set == the oracle's
    assert np.array_equal(g.compact_keys(), o.compact_keys())


def test_multi_source_bfs_matches_single():
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph

    n, src, dst = make_graph(dict(kind="rmat", scale=13, edge_factor=8, seed=4))
    keys = G.edges_to_keys(src, dst)
    g = G.GPMA(n)
    o = OracleGPMA(n, threads=8)
    G.update_gpma(g, keys, np.ones(len(keys), np.uint8))
    o.update(keys, np.ones(len(keys), np.uint8))
    rng = np.random.default_rng(3)
    for k in (1, 7, 64):
        srcs = rng.choice(n, k, replace=False).astype(np.uint32)
        lv, reached = G.gpma_bfs_multi(g, srcs)
        olv, orr = o.bfs_multi(srcs)
        assert np.array_equal(reached, orr)
        assert np.array_equal(lv, olv)


def test_errors_leave_structure_unchanged():
    import gpma_bfs_gb300 as G

    n = 100
    g = G.GPMA(n)
    keys = (np.arange(10, dtype=np.uint64) << np.uint64(32)) | np.uint64(3)
    G.update_gpma(g, keys, np.ones(10, np.uint8))
    before = g.export_layout()
    bad = np.array([(7 << 32) | 0xFFFFFFFF], np.uint64)  # reserved column (guard)
    with pytest.raises(G.GPMAError) as e:
        G.update_gpma(g, np.concatenate([keys, bad]), np.ones(11, np.uint8))
    assert e.value.status == 1
    after = g.export_layout()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    with pytest.raises(G.GPMAError):
        G.gpma_bfs(g, n, 0, n + 5)
    with pytest.raises(ValueError):
        G.update_gpma(g, keys, np.ones(9, np.uint8))
    with pytest.raises(G.GPMAError):
        G.gpma_bfs_multi(g, np.arange(65, dtype=np.uint32) % n)
    g.close()


def test_empty_graph_and_single_row():
    import gpma_bfs_gb300 as G

    for n in (0, 1, 2, 3):
        g = G.GPMA(n)
        o = OracleGPMA(n)
        assert g.geometry() == o.geometry()
        gk, gv, gr = g.export_layout()
        ok, ov, orow = o.export_layout()
        assert np.array_equal(gk, ok) and np.array_equal(gr, orow)
        if n:
            keys = np.array([0, (0 << 32) | (n - 1)], np.uint64)
            G.update_gpma(g, keys, np.ones(2, np.uint8))
            o.update(keys, np.ones(2, np.uint8))
            assert np.array_equal(g.export_layout()[0], o.export_layout()[0])
            gl, gr2 = G.gpma_bfs(g, n, 2, 0)
            ol, orr = o.bfs(0)
            assert gr2 == orr and np.array_equal(gl, ol)
        g.close()
