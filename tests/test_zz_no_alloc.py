"""gpma_bfs_noalloc: the BFS entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc while they run (a host-side
arena or fixed device budget owns every allocation, or allocation is
forbidden once serving starts). Its working set sits in one fixed array
inside the library, so the graph may have at most 2,097,152 nodes. The
result must equal gpma_bfs bit for bit; two calls in a row check that the
second call is not disturbed by what the first left in the shared array. A
graph whose long rows overflow a shortened chunk list takes the branch that
walks such rows in place, and the device's free memory is unchanged by the
calls (the allocating gpma_bfs on the same graph does take memory).

This file is collected last on purpose: it must pass both alone in a fresh
process and after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 21


def _noalloc(G, g, src, out_ptr):
    reached = ctypes.c_uint64()
    rc = G.lib().gpma_bfs_noalloc(g.handle, src, out_ptr, ctypes.byref(reached), None)
    return rc, reached.value


def test_noalloc_bfs_matches_allocating_bfs_twice(built_lib):
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph

    assert torch.cuda.is_available()
    n, src, dst = make_graph(dict(kind="rmat", scale=15, edge_factor=8, seed=31))
    g = G.GPMA(n)
    G.update_gpma(g, G.edges_to_keys(src, dst), np.ones(len(src), np.uint8))
    out = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    for source in (0, int(src[0])):
        rc, reached = _noalloc(G, g, source, out.data_ptr())
        assert rc == 0, G.lib().gpma_last_error()
        ref, ref_reached = G.gpma_bfs(g, n, len(src), source)
        assert reached == ref_reached
        assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
    g.close()


def test_noalloc_bfs_rejects_what_it_cannot_serve(built_lib):
    import torch

    import gpma_bfs_gb300 as G

    g = G.GPMA(100)
    host_levels = np.zeros(100, np.uint32)
    rc, _ = _noalloc(G, g, 0, host_levels.ctypes.data)
    assert rc == 1 and b"device memory" in G.lib().gpma_last_error()
    dev = torch.zeros(100, dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(G, g, 100, dev.data_ptr())
    assert rc == 1
    g.close()
    big = G.GPMA(MAX_ROWS + 1)
    dev = torch.zeros(MAX_ROWS + 1, dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(G, big, 0, dev.data_ptr())
    assert rc == 4 and b"2097152" in G.lib().gpma_last_error()
    big.close()


def test_noalloc_bfs_full_chunk_list_walks_rows_in_place(built_lib):
    """The fixed chunk list holds 65,536 long-row chunks; rows that find it
    full are walked by the warp that found them. A shortened list (test hook)
    makes that branch run on a small graph: same results, overflows counted."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph

    n, src, dst = make_graph(dict(kind="rmat", scale=15, edge_factor=16, seed=32))
    g = G.GPMA(n)
    G.update_gpma(g, G.edges_to_keys(src, dst), np.ones(len(src), np.uint8))
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    sources = (0, int(src[0]), int(src[len(src) // 2]))
    try:
        for cap in (4, 64):
            G.set_test_hooks(noalloc_chunk_cap=cap)
            for s in sources:
                rc, reached = _noalloc(G, g, s, out.data_ptr())
                assert rc == 0, G.lib().gpma_last_error()
                over = G.get_test_hooks()["noalloc_overflows"]
                ref, ref_reached = G.gpma_bfs(g, n, len(src), s)
                assert reached == ref_reached and np.array_equal(out.cpu().numpy().view(np.uint32), ref)
                if s == 0 and cap == 4:
                    assert over > 0, "the full-list branch did not run"
    finally:
        G.set_test_hooks(noalloc_chunk_cap=0)
    g.close()


def test_noalloc_bfs_takes_no_device_memory(built_lib):
    """After the library's first use on this device, gpma_bfs_noalloc calls on
    a fresh graph leave the device's free memory unchanged, while the
    allocating gpma_bfs on the same graph takes its per-graph buffers."""
    import torch

    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import make_graph

    warm = G.GPMA(64)
    w_out = torch.zeros(64, dtype=torch.int32, device="cuda")
    assert _noalloc(G, warm, 0, w_out.data_ptr())[0] == 0  # commits the module and its array on this device
    n = MAX_ROWS
    _, src, dst = make_graph(dict(kind="rmat", scale=21, edge_factor=2, seed=33))
    g = G.GPMA(n)
    G.update_gpma(g, G.edges_to_keys(src, dst), np.ones(len(src), np.uint8))
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for s in (0, int(src[0]), int(src[1])):
        rc, reached = _noalloc(G, g, s, out.data_ptr())
        assert rc == 0 and reached >= 1
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "gpma_bfs_noalloc changed the device's free memory"
    levels, _ = G.gpma_bfs(g, n, len(src), int(src[1]))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), levels)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] < free0 - (4 << 20), "the allocating BFS should take its buffers"
    g.close()
    warm.close()
