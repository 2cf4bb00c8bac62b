"""The bounds-checked build (libgpma_gb300_checked.so: every data-dependent
index range of the kernels checked before the access; it stands in for a
memory checker).

1. The same workload through the checked and the product library gives the
   same layouts, BFS levels and reach: root resizes, slides, the >= 5M-key
   bulk rebuild, the batched update and the multi-source BFS, with no check
   failing (any failure is an error status, which fails the run).
2. A corrupt row_offset entry (one past the array) is reported by the
   checked BFS as GPMA_ERR_DEVICE naming the row check, and nothing outside
   the array is touched: the failing row is skipped, the launch stops at its
   next grid barrier, and after the entry is restored the next BFS is exact.
The checked library runs in a child process (a process loads one library).
"""
import hashlib
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def workload_digest() -> str:
    """Digest of every layout, level array and reach of a fixed workload run
    through whichever library this process loaded."""
    import gpma_bfs_gb300 as G
    from gpma_bfs_gb300.workloads import batched_graphs, make_graph, sliding_window

    h = hashlib.sha256()

    def add(*arrays):
        for a in arrays:
            h.update(np.ascontiguousarray(a).tobytes())

    # one graph: load from the guards (root resizes), slides, BFS
    n, src, dst = make_graph(dict(kind="rmat", scale=14, edge_factor=16, seed=21))
    sw = sliding_window(src, dst, num_slide=40)
    g = G.GPMA(n)
    G.update_gpma(g, sw.load_keys, sw.load_values)
    for i in range(12):
        G.update_gpma(g, sw.slide_keys[i], sw.slide_values[i])
        if i % 4 == 3:
            add(*G.gpma_bfs(g, n, len(src), 0)[:1])
    add(*g.export_layout())
    levels, reached = G.gpma_bfs_multi(g, np.arange(0, 64 * 17, 17, dtype=np.uint32))
    add(levels, reached)
    assert g.validate() == 0
    g.close()
    # the bulk rebuild: one batch of >= 5M insertions
    n2, s2, d2 = make_graph(dict(kind="rmat", scale=20, edge_factor=8, seed=22))
    keys = G.edges_to_keys(s2, d2)
    assert len(keys) >= 5_000_000
    g2 = G.GPMA(n2)
    G.update_gpma(g2, keys, np.ones(len(keys), np.uint8))
    G.update_gpma(g2, keys[::3], np.zeros(len(keys[::3]), np.uint8))
    add(*g2.export_layout())
    add(*G.gpma_bfs(g2, n2, len(keys), 0)[:1])
    assert g2.validate() == 0
    g2.close()
    # batched: packed updates of several graphs, multi-source BFS of each
    specs = batched_graphs(12, seed=23, min_edges=5_000, max_edges=300_000)
    graphs = [G.GPMA(m) for m, _ in specs]
    b = G.Batch()
    for part, value in ((slice(0, None, 2), 1), (slice(0, None, 6), 0), (slice(1, None, 4), 1)):
        ks = [k[part] for _, k in specs]
        off = np.concatenate([[0], np.cumsum([len(k) for k in ks])]).astype(np.uint64)
        b.update_packed(graphs, np.concatenate(ks), np.full(int(off[-1]), value, np.uint8), off)
    rng = np.random.default_rng(24)
    sources = [rng.choice(m, 32, replace=False).astype(np.uint32) for m, _ in specs]
    outs, parts = b.bfs_multi(graphs, sources, levels=True)
    for gr, o, p in zip(graphs, outs, parts):
        add(*gr.export_layout(), o, p)
        assert gr.validate() == 0
        gr.close()
    b.close()
    return h.hexdigest()


def corrupt_row_check() -> str:
    """Runs in the checked library: BFS over a row_offset whose entry for
    row 0's end points one past the array, then again after restoring it."""
    import torch

    import gpma_bfs_gb300 as G

    n, src, dst = 1 << 12, *G.gen_rmat(12, 8, seed=25)
    keys = G.edges_to_keys(src, dst)
    g = G.GPMA(n)
    G.update_gpma(g, keys, np.ones(len(keys), np.uint8))
    want, want_r = G.gpma_bfs(g, n, len(keys), 0)
    _, _, ro_ptr = g.device_arrays()

    class View:  # row_offset as an int32 tensor (values stay below 2^31)
        __cuda_array_interface__ = {"shape": (n + 1,), "typestr": "<i4", "data": (ro_ptr, False), "version": 3}

    ro = torch.as_tensor(View(), device="cuda")
    torch.cuda.synchronize()
    saved = int(ro[1].item())
    ro[1] = g.get_size() + 1
    torch.cuda.synchronize()
    with pytest.raises(G.GPMAError) as e:
        G.gpma_bfs(g, n, len(keys), 0)
    assert e.value.status == 7 and "site 6" in str(e.value), str(e.value)
    ro[1] = saved
    torch.cuda.synchronize()
    got, got_r = G.gpma_bfs(g, n, len(keys), 0)
    assert got_r == want_r and np.array_equal(got, want)
    g.close()
    return "corrupt row reported"


def _run_checked(func: str) -> str:
    from gpma_bfs_gb300.build import build

    lib = build(checked=True)
    env = dict(os.environ, GPMA_GB300_LIB=str(lib))
    code = (f"import sys; sys.path[:0] = [{str(ROOT)!r}, {str(ROOT / 'tests')!r}]; "
            f"import gpma_bfs_gb300 as G, test_gpu_checked as t; "
            f"assert G.lib()._name.endswith('_checked.so'); print('RESULT', t.{func}())")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return next(line.split(" ", 1)[1] for line in r.stdout.splitlines() if line.startswith("RESULT "))


def test_checked_build_matches_product_build(built_lib):
    assert _run_checked("workload_digest") == workload_digest()


def test_checked_build_reports_corrupt_row_offset(built_lib):
    assert _run_checked("corrupt_row_check") == "corrupt row reported"
