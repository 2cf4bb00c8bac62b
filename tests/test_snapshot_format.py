"""gpma_load's host-side checks of a snapshot file, without a GPU.

Snapshot format (capi.cu): "GPMASNP1", u32 version 1, row_num, size,
segment_length, tree_height, u32 0, u64 payload checksum; payload = keys
(size x u64), masked values (size x u8), row_offset ((row_num + 1) x u32),
little-endian. gpma_load checks the header, the checksum and the layout
(row_offset from 0, non-decreasing, inside the array, each row's guard at
row_offset[row + 1], live keys ascending) before it touches the GPU. Here
files are written in Python from layouts the reference itself produced (the
golden dumps) and from corrupted copies with a correct checksum: the good
ones get past the host checks (on a host without a GPU the load then fails
with a CUDA error, on a GPU host it succeeds), the corrupted ones are
refused with GPMA_ERR_IO.
"""
import numpy as np
import pytest

from replay import GOLDEN

ERR_CUDA, ERR_IO = 2, 6
KEY_NONE = np.uint64(0xFFFFFFFFFFFFFFFF)


def _checksum(payload: bytes) -> int:
    h = 0x243F6A8885A308D3
    for b in payload:
        h = ((h ^ b) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
        h ^= h >> 29
    return h


def _geometry(size: int):
    fls = lambda x: x.bit_length()
    seg = 1 << (fls(fls(size)) - 1)
    return seg, fls(size // seg) - 1


def _write(path, row_num, keys, vals, ro):
    size = len(keys)
    seg, height = _geometry(size)
    payload = (np.asarray(keys, "<u8").tobytes() + np.asarray(vals, np.uint8).tobytes()
               + np.asarray(ro, "<u4").tobytes())
    hdr = (b"GPMASNP1" + np.asarray([1, row_num, size, seg, height, 0], "<u4").tobytes()
           + np.asarray([_checksum(payload)], "<u8").tobytes())
    path.write_bytes(hdr + payload)


def _load_status(built_lib, path):
    import ctypes

    h = ctypes.c_void_p()
    st = built_lib.gpma_load(str(path).encode(), None, ctypes.byref(h))
    if st == 0:
        assert built_lib.gpma_destroy(h) == 0
    return st


def _reference_layouts():
    """(row_num, keys, masked values, row_offset) of every layout dump the reference wrote."""
    out = []
    for name in ("edge_cases", "random_1", "random_4", "rmat8_slide"):
        z = np.load(GOLDEN / f"{name}.npz")
        n = int(z["row_num"])
        ko = 0
        for i, size in enumerate(z["dump_size"]):
            size = int(size)
            keys, vals = z["dump_keys"][ko:ko + size], z["dump_vals"][ko:ko + size]
            ro = z["dump_ro"][i * (n + 1):(i + 1) * (n + 1)]
            out.append((f"{name}#{i}", n, keys, vals, ro))
            ko += size
    return out


LAYOUTS = _reference_layouts()


@pytest.mark.parametrize("case", range(len(LAYOUTS)), ids=[c[0] for c in LAYOUTS])
def test_reference_layouts_pass_the_host_checks(case, built_lib, tmp_path):
    _, n, keys, vals, ro = LAYOUTS[case]
    _write(tmp_path / "g.snap", n, keys, vals, ro)
    assert _load_status(built_lib, tmp_path / "g.snap") in (0, ERR_CUDA), built_lib.gpma_last_error()


def _corrupt(kind, n, keys, vals, ro):
    keys, vals, ro = keys.copy(), vals.copy(), ro.copy()
    if kind == "row_offset_past_end":
        ro[-1] = len(keys) + 7
    elif kind == "row_offset_decreasing":
        ro[1], ro[2] = ro[2], ro[1]
    elif kind == "row_offset_start":
        ro[0] = 1
    elif kind == "guard_moved":
        r = n // 2
        keys[ro[r + 1]] = KEY_NONE
    elif kind == "keys_out_of_order":
        live = np.flatnonzero((keys != KEY_NONE) & (vals != 0))
        i, j = live[1], live[-2]
        keys[i], keys[j] = keys[j], keys[i]
        vals[i], vals[j] = vals[j], vals[i]
    return keys, vals, ro


@pytest.mark.parametrize("kind", ["row_offset_past_end", "row_offset_decreasing", "row_offset_start", "guard_moved",
                                  "keys_out_of_order"])
def test_corrupt_layout_with_valid_checksum_is_refused(kind, built_lib, tmp_path):
    _, n, keys, vals, ro = next(c for c in LAYOUTS if c[0].startswith("rmat8_slide"))
    _write(tmp_path / "bad.snap", n, *_corrupt(kind, n, keys, vals, ro))
    assert _load_status(built_lib, tmp_path / "bad.snap") == ERR_IO
    assert b"not a valid layout" in built_lib.gpma_last_error()


def test_truncated_and_bad_checksum_refused(built_lib, tmp_path):
    _, n, keys, vals, ro = LAYOUTS[0]
    p = tmp_path / "g.snap"
    _write(p, n, keys, vals, ro)
    raw = p.read_bytes()
    p.write_bytes(raw[:-3])
    assert _load_status(built_lib, p) == ERR_IO
    flipped = bytearray(raw)
    flipped[50] ^= 1
    p.write_bytes(bytes(flipped))
    assert _load_status(built_lib, p) == ERR_IO
    p.write_bytes(raw + b"\0")
    assert _load_status(built_lib, p) == ERR_IO


def test_oracle_layout_with_tombstones_passes_the_host_checks(built_lib, tmp_path):
    """The state the GPU snapshot test saves: R-MAT scale 12, half the edges
    inserted, every fifth of them deleted again (tombstones in the file)."""
    import gpma_bfs_gb300 as G
    from oracle.oracle import OracleGPMA

    src, dst = G.gen_rmat(12, 8, seed=11)
    n = 1 << 12
    first = G.edges_to_keys(src, dst)[: len(src) // 2]
    o = OracleGPMA(n, threads=2)
    o.update(first, np.ones(len(first), np.uint8))
    o.update(first[::5], np.zeros(len(first[::5]), np.uint8))
    keys, vals, ro = o.export_layout()
    assert np.count_nonzero((keys != KEY_NONE) & (vals == 0)) > 0
    _write(tmp_path / "g.snap", n, keys, vals, ro)
    assert _load_status(built_lib, tmp_path / "g.snap") in (0, ERR_CUDA), built_lib.gpma_last_error()
