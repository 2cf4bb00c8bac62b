"""Differential check of the C restatement (oracle/) against the reference run live.

The committed fixtures pin the oracle on fixed scripts. This file draws fresh
scripts (new seeds of the same generators: mixed inserts, deletes of live and
missing keys, revivals, modifications, duplicate keys, root resizes, R-MAT
sliding windows) and runs each through both the reference's own
GPMA<CPU> + update_gpma + CPU BFS (oracle/_ref/ref_driver, built from the
reference sources by `make -C oracle ref`) and the oracle; every layout,
row_offset, geometry, threshold set, compacted key set and BFS level array
must agree bit for bit. Where the reference binary has not been built (a
host without the reference sources) the tests skip.
"""
import numpy as np
import pytest

import cases
import make_golden
from oracle.oracle import OracleGPMA
from replay import replay_and_compare

needs_ref = pytest.mark.skipif(not make_golden.DRIVER.exists(), reason="reference binary oracle/_ref/ref_driver not built")


def _compare(n, ops):
    z = make_golden.records_to_arrays(n, ops, make_golden.run_reference(n, ops), store_ops=True)
    o = OracleGPMA(n, threads=4)
    ui, bi, _ = replay_and_compare(o, ops, z)
    assert ui == sum(1 for op in ops if op[0] == "update")
    assert bi == sum(1 for op in ops if op[0] == "bfs")


@needs_ref
@pytest.mark.parametrize("seed", range(100, 164))
def test_random_script_matches_reference(seed, built_lib):
    n, ops = cases.random_case(seed)
    _compare(n, ops)


@needs_ref
@pytest.mark.parametrize("scale,seed", [(10, 21), (10, 22), (11, 23), (12, 24)])
def test_rmat_slide_matches_reference(scale, seed, built_lib):
    """R-MAT sliding window (half-load, 40 slides, BFS before and after) with
    dumps of the whole layout along the way."""
    from gpma_bfs_gb300.workloads import make_graph

    n, src, dst = make_graph(dict(kind="rmat", scale=scale, edge_factor=16, seed=seed))
    ops = cases.sliding_ops(n, src, dst, 40, bfs_src=int(src[0]), dumps=(0, 20, 40))
    _compare(n, ops)


@needs_ref
def test_single_row_hub_matches_reference(built_lib):
    """Every edge in one row: the deepest windows, repeated root resizes up and down."""
    n = 64
    rng = np.random.default_rng(9)
    dst = rng.permutation(n)
    keys = (np.uint64(7) << np.uint64(32)) | dst.astype(np.uint64)
    ops = []
    for lo in range(0, n, 8):
        ops.append(("update", keys[lo:lo + 8], np.ones(8, np.uint8)))
        ops.append(("dump",))
    ops.append(("bfs", 7))
    for lo in range(0, n, 16):
        ops.append(("update", keys[lo:lo + 16], np.zeros(16, np.uint8)))
        ops.append(("dump",))
    ops.append(("bfs", 7))
    _compare(n, ops)


@needs_ref
def test_timed_update_op_applies_the_same_update(built_lib):
    """The driver's timed update (used to time the reference's CPU path) changes
    the structure exactly as the recorded update does."""
    n, ops = cases.random_case(200)
    timed = [("timed_update", op[1], op[2]) if op[0] == "update" else op for op in ops]
    recs = make_golden.run_reference(n, timed)
    assert sum(r["op"] == "timed_update" for r in recs) == sum(op[0] == "update" for op in ops)
    assert all(r["seconds"] >= 0 for r in recs if r["op"] == "timed_update")
    o = OracleGPMA(n, threads=2)
    dumps = iter(r for r in recs if r["op"] == "dump")
    for op in ops:
        if op[0] == "update":
            o.update(op[1], op[2])
        elif op[0] == "dump":
            r = next(dumps)
            keys, masked, ro = o.export_layout()
            assert np.array_equal(keys, r["keys"]) and np.array_equal(masked, r["values"])
            assert np.array_equal(ro, r["row_offset"])


@needs_ref
@pytest.mark.parametrize("spec", [dict(kind="chung_lu", n=20000, m=300000, exponent=2.3, max_degree=3000, seed=41),
                                  dict(kind="rmat", scale=14, edge_factor=16, seed=42)],
                         ids=["chung_lu_20k", "rmat14"])
def test_larger_slides_match_reference(spec, built_lib):
    """The social configuration's shape at a size the reference runs in
    seconds (power-law hubs: long rows, deep windows), and R-MAT scale 14:
    half-load (bulk of the first batch), 100 slides, BFS from a hub before
    and after, a whole-layout dump at the end."""
    from gpma_bfs_gb300.workloads import make_graph

    n, src, dst = make_graph(spec)
    ops = cases.sliding_ops(n, src, dst, 100, bfs_src=0, dumps=(100,))
    _compare(n, ops)
