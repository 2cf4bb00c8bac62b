"""Workload scripts for the reference driver and the shared digest.

Test infrastructure only. ``write_script`` encodes a sequence of operations
("update", keys, values) / ("bfs", src) / ("dump",) / ("timed_update", keys,
values: the update alone, timed, no layout digest) in the binary format read
by oracle/ref/ref_driver.cu; ``read_output`` decodes its results; ``digest``
is the order-sensitive 64-bit digest both sides use.
"""
from __future__ import annotations

import struct

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def digest(x: np.ndarray) -> int:
    """sum_i mix64(x_i + (i+1) * golden) mod 2^64, elements widened to u64."""
    z = np.asarray(x).astype(np.uint64, copy=True).ravel()
    with np.errstate(over="ignore"):
        z += (np.arange(1, len(z) + 1, dtype=np.uint64) * _GOLD)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
        return int(z.sum(dtype=np.uint64))


def write_script(path, row_num: int, ops) -> None:
    with open(path, "wb") as f:
        f.write(b"GPWS" + struct.pack("<III", 1, row_num, len(ops)))
        for op in ops:
            if op[0] == "update":
                k = np.ascontiguousarray(op[1], np.uint64)
                v = np.ascontiguousarray(op[2], np.uint8)
                f.write(struct.pack("<IQ", 1, len(k)))
                f.write(k.tobytes())
                f.write(v.tobytes())
            elif op[0] == "timed_update":
                k = np.ascontiguousarray(op[1], np.uint64)
                v = np.ascontiguousarray(op[2], np.uint8)
                f.write(struct.pack("<IQ", 4, len(k)))
                f.write(k.tobytes())
                f.write(v.tobytes())
            elif op[0] == "bfs":
                f.write(struct.pack("<II", 2, op[1]))
            elif op[0] == "dump":
                f.write(struct.pack("<I", 3))
            else:
                raise ValueError(op[0])


def read_output(path, row_num: int) -> list[dict]:
    data = open(path, "rb").read()
    assert data[:4] == b"GPWO"
    pos = 8
    out = []

    def take(fmt):
        nonlocal pos
        vals = struct.unpack_from(fmt, data, pos)
        pos += struct.calcsize(fmt)
        return vals

    def arr(dtype, n):
        nonlocal pos
        a = np.frombuffer(data, dtype=dtype, count=n, offset=pos).copy()
        pos += a.nbytes
        return a

    while pos < len(data):
        (tag,) = take("<I")
        if tag == 1:
            size, seg, h, row_num = take("<IIII")
            (live,) = take("<Q")
            d = take("<4Q")
            lower = arr(np.uint32, h + 1)
            upper = arr(np.uint32, h + 1)
            out.append({"op": "update", "size": size, "segment_length": seg, "tree_height": h, "live": live,
                        "d_keys": d[0], "d_values": d[1], "d_row_offset": d[2], "d_compact": d[3],
                        "lower": lower, "upper": upper})
        elif tag == 2:
            src, = take("<I")
            reached, = take("<Q")
            out.append({"op": "bfs", "src": src, "reached": reached, "levels": arr(np.uint32, row_num)})
        elif tag == 3:
            size, row_num = take("<II")
            out.append({"op": "dump", "keys": arr(np.uint64, size), "values": arr(np.uint8, size),
                        "row_offset": arr(np.uint32, row_num + 1)})
        elif tag == 4:
            n, ns = take("<QQ")
            out.append({"op": "timed_update", "keys": n, "seconds": ns * 1e-9})
        else:
            raise ValueError(f"bad tag {tag}")
    return out


def state_record(keys: np.ndarray, masked: np.ndarray, row_offset: np.ndarray, geometry: dict, lower, upper) -> dict:
    """The same per-update record the reference driver writes, from exported arrays."""
    live_mask = (keys != np.uint64(0xFFFFFFFFFFFFFFFF)) & (masked != 0)
    compact = keys[live_mask]
    return {"size": geometry["size"], "segment_length": geometry["segment_length"],
            "tree_height": geometry["tree_height"], "live": int(len(compact)), "d_keys": digest(keys),
            "d_values": digest(masked), "d_row_offset": digest(row_offset), "d_compact": digest(compact),
            "lower": np.asarray(lower, np.uint32), "upper": np.asarray(upper, np.uint32)}
