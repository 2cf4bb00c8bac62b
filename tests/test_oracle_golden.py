"""Pins the C restatement (oracle/) to vectors produced by the reference itself.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py,
which runs the reference's own GPMA<CPU> / update_gpma / CPU BFS
(oracle/ref/ref_driver.cu built from the reference sources). Every update's
layout, values, row_offset, compacted key set, geometry and thresholds, and
every BFS level array must match bit for bit.
"""
import pytest

import cases
from oracle.oracle import OracleGPMA
from replay import load_case, replay_and_compare

CASES = list(cases.SMALL) + ["rmat8_slide", "rmat12_slide", "rmat16_slide"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name, built_lib):
    n, ops, z = load_case(name)
    o = OracleGPMA(n, threads=4)
    ui, bi, di = replay_and_compare(o, ops, z)
    assert ui == len(z["rec_size"]) and bi == len(z["bfs_src"])


@pytest.mark.slow
def test_oracle_bulk_rebuild_matches_reference(built_lib):
    """>= 5M insertions in one batch: significant_insert (gpma.cuh:936-966)."""
    n, ops, z = load_case("rmat20_bulk")
    o = OracleGPMA(n, threads=8)
    replay_and_compare(o, ops, z)
    assert o.stats()["significant"] == 1
