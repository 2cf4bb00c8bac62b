"""C ABI boundary and host logic (no GPU needed, no compute calls on a GPU)."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        for m in re.finditer(r"GPMA_API\s+[\w\s\*]+?\b(gpma_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for core in ("gpma_create", "gpma_destroy", "gpma_update", "gpma_bfs", "gpma_bfs_multi",
                 "gpma_export_layout", "gpma_get_geometry"):
        assert core in names


def test_header_is_plain_c99_and_links(tmp_path, built_lib):
    """An FFI or C caller includes the header with a C compiler: no C++ in it,
    no warnings under -pedantic, and every call resolves against the library."""
    calls = "\n".join(f"    (void)&{n};" for n in declared_symbols())
    src = tmp_path / "c_caller.c"
    src.write_text('#include "gpma_gb300.h"\n#include <string.h>\nint main(void) {\n'
                   f"{calls}\n"
                   "    return gpma_create(4, 0, 0) == GPMA_ERR_INVALID && strlen(gpma_last_error()) > 0 ? 0 : 1;\n}\n")
    exe = tmp_path / "c_caller"
    libdir = ROOT / "gpma_bfs_gb300"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{ROOT / 'include'}",
                        str(src), f"-L{libdir}", "-lgpma_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0


def _exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_library_exports_every_declared_symbol(built_lib):
    exported = _exported(ROOT / "gpma_bfs_gb300" / "libgpma_gb300.so")
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_symbols():
        assert getattr(built_lib, n) is not None


def test_checked_build_exports_the_same_entry_points(built_lib):
    """The bounds-checked variant is a drop-in for the product library."""
    from gpma_bfs_gb300.build import build

    checked = build(checked=True)
    assert checked.name == "libgpma_gb300_checked.so"
    assert _exported(checked) == _exported(ROOT / "gpma_bfs_gb300" / "libgpma_gb300.so")
    assert "GPMA_BOUNDS_CHECK=1" in (checked.parent / "_build_checked" / "options.txt").read_text()
    assert "GPMA_BOUNDS_CHECK=0" in (checked.parent / "_build" / "options.txt").read_text()
    ctypes.CDLL(str(checked))


def test_status_strings(built_lib):
    built_lib.gpma_status_string.restype = ctypes.c_char_p
    assert built_lib.gpma_status_string(0) == b"ok"
    assert built_lib.gpma_status_string(1) == b"invalid argument"
    assert b"sm_103a" in built_lib.gpma_version()


def test_null_arguments_rejected_without_gpu(built_lib):
    import gpma_bfs_gb300 as G

    assert built_lib.gpma_create(5, None, None) == 1
    assert built_lib.gpma_update(None, None, None, 0, None) == 1
    assert built_lib.gpma_bfs(None, 0, None, None, None) == 1
    assert b"null" in built_lib.gpma_last_error() or b"NULL" in built_lib.gpma_last_error()
    with pytest.raises(ValueError):
        G.update_gpma(object(), np.zeros(3, np.uint64), np.zeros(2, np.uint8))
    # recorded steps, the consistency check and the shard helpers validate
    # their arguments before any CUDA call
    L = G.lib()
    out = ctypes.c_void_p()
    assert L.gpma_step_create(None, ctypes.byref(out)) == 1
    assert L.gpma_step_run(None, None, None, 0, 0, None, None, None) == 1
    assert L.gpma_step_get_stats(None, None) == 1
    assert L.gpma_step_destroy(None) == 0
    assert L.gpma_batch_step_create(None, None, 0, ctypes.byref(out)) == 1
    assert L.gpma_batch_step_run(None, None, None, None, None, None, None, None) == 1
    assert L.gpma_batch_step_run_many(None, 2, None, None, None, None, None, None, None) == 1
    assert L.gpma_batch_step_destroy(None) == 0
    assert L.gpma_validate(None, None, None) == 1
    assert L.gpma_partition_rows(None, None, 0, 10, 0, 1, None, None, None) == 1
    assert L.gpma_shard_first_row(10, 3, 1) == 3 and L.gpma_shard_first_row(10, 0, 1) == 0


def test_rmat_generator_deterministic(built_lib):
    import gpma_bfs_gb300 as G

    s1, d1 = G.gen_rmat(12, 8, seed=9)
    s2, d2 = G.gen_rmat(12, 8, seed=9)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    k = G.edges_to_keys(s1, d1)
    assert len(np.unique(k)) == len(k), "duplicates survived"
    assert not np.any(s1 == d1), "self-loops survived"
    assert s1.max() < 4096 and d1.max() < 4096
    # R-MAT skew: quadrant a dominates, so low ids are heavy
    assert np.mean(s1 < 2048) > 0.7
    s3, _ = G.gen_rmat(12, 8, seed=10)
    assert not np.array_equal(s1, s3)


def test_chung_lu_generator(built_lib):
    import gpma_bfs_gb300 as G

    n, m = 20000, 150000
    s, d = G.gen_chung_lu(n, m, 2.3, 900, seed=4)
    assert len(s) == m
    k = G.edges_to_keys(s, d)
    assert len(np.unique(k)) == m and not np.any(s == d)
    deg = np.bincount(s, minlength=n)
    assert deg.argmax() == 0, "node 0 is the top out-hub"
    assert 400 < deg[0] <= 1100, deg[0]
    assert np.median(deg) < m / n, "power law: median below mean"


def test_text_format_round_trip(tmp_path, built_lib):
    import gpma_bfs_gb300 as G

    s, d = G.gen_rmat(8, 4, seed=2)
    p = tmp_path / "g.txt"
    G.write_edges_text(p, 256, s, d)
    first = p.read_text().splitlines()[0]
    assert first == f"256 {len(s)}"
    n, s2, d2 = G.read_edges_text(p)
    assert n == 256 and np.array_equal(s, s2) and np.array_equal(d, d2)


def test_sliding_window_schedule(built_lib):
    from gpma_bfs_gb300.workloads import sliding_window

    s = np.arange(1000, dtype=np.uint32)
    d = s + 1
    sw = sliding_window(s, d, num_slide=100)
    assert sw.half == 500 and sw.step == 5
    k, v = sw.slide_keys[3], sw.slide_values[3]
    # inserts first (next edges), then deletes (oldest edges): gpma_bfs_demo.cu:85-104
    assert list(k[:5] >> np.uint64(32)) == [515, 516, 517, 518, 519]
    assert list(k[5:] >> np.uint64(32)) == [15, 16, 17, 18, 19]
    assert list(v) == [1] * 5 + [0] * 5


def test_oracle_thresholds_follow_reference_formula():
    """recalculate_density (gpma.cuh:147-168) on a known geometry."""
    from oracle.oracle import OracleGPMA

    o = OracleGPMA(0)
    lo, hi = o.thresholds()
    # initial structure: 4 slots, segment 2, height 1
    assert o.geometry() == {"size": 4, "segment_length": 2, "tree_height": 1, "row_num": 0}
    assert list(lo) == [1, 2] and list(hi) == [1, 2]


def test_test_hooks_round_trip_and_reject_bad_values(built_lib):
    """The error-path test hooks are plain host settings: checked on the host,
    read back as set, and left at zero."""
    import gpma_bfs_gb300 as G

    assert G.get_test_hooks() == dict(update_stall=0, bfs_stall=0, wait_limit_us=0, noalloc_chunk_cap=0,
                                      noalloc_overflows=0)
    for bad in (dict(update_stall=2), dict(bfs_stall=3), dict(noalloc_chunk_cap=65537)):
        with pytest.raises(G.GPMAError):
            G.set_test_hooks(**bad)
    old = G.set_test_hooks(update_stall=1, wait_limit_us=50_000, noalloc_chunk_cap=16)
    try:
        now = G.get_test_hooks()
        assert (now["update_stall"], now["wait_limit_us"], now["noalloc_chunk_cap"]) == (1, 50_000, 16)
    finally:
        G.set_test_hooks(**old)
    assert G.get_test_hooks()["update_stall"] == 0


def test_update_sort_setting(built_lib):
    """The batch-sort switch is host state: 0 (buckets) and 1 (digit passes)
    are accepted, anything else is rejected and leaves the setting alone."""
    import gpma_bfs_gb300 as G

    old = G.get_tuning()
    try:
        assert old["update_sort"] == 0
        G.set_tuning(update_sort=1)
        assert G.get_tuning()["update_sort"] == 1
        with pytest.raises(G.GPMAError):
            G.set_tuning(update_sort=2)
        assert G.get_tuning()["update_sort"] == 1
    finally:
        G.set_tuning(**old)


def test_profile_reports_sort_fallbacks(built_lib):
    import gpma_bfs_gb300 as G

    assert "sort_fallbacks" in [n for n, _ in G._Profile._fields_]
