"""ctypes binding of the C restatement (oracle/gpma_oracle.c).

Test infrastructure only (see oracle/gpma_oracle.h). ``build()`` compiles
oracle/_build/libgpma_oracle.so with the Makefile next to this file.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libgpma_oracle.so"
GRAPHGEN = HERE / "_build" / "libgraphgen.so"


class _Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "updates", "accepted_windows", "accepted_slots", "levels_visited", "root_resizes", "root_drops",
        "significant", "last_inserts")]


class _Gpma(ctypes.Structure):
    _fields_ = [("keys", ctypes.POINTER(ctypes.c_uint64)), ("values", ctypes.POINTER(ctypes.c_uint8)),
                ("size", ctypes.c_uint32), ("segment_length", ctypes.c_uint32), ("tree_height", ctypes.c_uint32),
                ("lower", ctypes.POINTER(ctypes.c_uint32)), ("upper", ctypes.POINTER(ctypes.c_uint32)),
                ("row_num", ctypes.c_uint32), ("row_offset", ctypes.POINTER(ctypes.c_uint32)),
                ("threads", ctypes.c_int), ("stats", _Stats)]


def build() -> Path:
    src = [HERE / "gpma_oracle.c", HERE / "gpma_oracle.h", HERE / "Makefile",
           HERE.parent / "gpma_bfs_gb300" / "csrc" / "graphgen.c"]
    if not LIB.exists() or not GRAPHGEN.exists() or any(
            p.stat().st_mtime > min(LIB.stat().st_mtime, GRAPHGEN.stat().st_mtime) for p in src if p.exists()):
        subprocess.run(["make", "-C", str(HERE), "oracle"], check=True, capture_output=True)
    return LIB


def gen_chung_lu(n: int, m: int, exponent: float = 2.3, max_degree: int = 9000, seed: int = 2):
    """The seeded Chung-Lu edge list of the benchmarks (same generator source
    as the library, built on its own into oracle/_build/libgraphgen.so), so a
    CPU baseline produces its input without loading the product library."""
    build()
    L = ctypes.CDLL(str(GRAPHGEN))
    L.gpma_gen_chung_lu.restype = ctypes.c_int
    L.gpma_gen_chung_lu.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double, ctypes.c_uint32,
                                    ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    src = np.empty(m, np.uint32)
    dst = np.empty(m, np.uint32)
    rc = L.gpma_gen_chung_lu(n, m, exponent, max_degree, seed, src.ctypes.data, dst.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"gpma_gen_chung_lu failed ({rc})")
    return src, dst


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.c_void_p
        L.oracle_create.restype = ctypes.POINTER(_Gpma)
        L.oracle_create.argtypes = [ctypes.c_uint32, ctypes.c_int]
        L.oracle_destroy.argtypes = [ctypes.POINTER(_Gpma)]
        L.oracle_update.restype = ctypes.c_int
        L.oracle_update.argtypes = [ctypes.POINTER(_Gpma), P, P, ctypes.c_uint64]
        L.oracle_bfs.restype = ctypes.c_int
        L.oracle_bfs.argtypes = [ctypes.POINTER(_Gpma), ctypes.c_uint32, P, ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_bfs_multi.restype = ctypes.c_int
        L.oracle_bfs_multi.argtypes = [ctypes.POINTER(_Gpma), P, ctypes.c_uint32, P, P]
        L.oracle_traversed_edges.restype = ctypes.c_uint64
        L.oracle_traversed_edges.argtypes = [ctypes.POINTER(_Gpma), P]
        L.oracle_compact.restype = ctypes.c_uint64
        L.oracle_compact.argtypes = [ctypes.POINTER(_Gpma), P]
        L.oracle_export.argtypes = [ctypes.POINTER(_Gpma), P, P, P]
        _lib = L
    return _lib


class OracleGPMA:
    """CPU restatement of GPMA<CPU> with the same surface as gpma_bfs_gb300.GPMA."""

    def __init__(self, row_num: int, threads: int | None = None):
        self.row_num = int(row_num)
        t = threads if threads is not None else int(os.environ.get("ORACLE_THREADS", "1"))
        self._g = lib().oracle_create(self.row_num, t)
        if not self._g:
            raise MemoryError("oracle_create failed")

    def close(self):
        if getattr(self, "_g", None):
            lib().oracle_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def _s(self) -> _Gpma:
        return self._g.contents

    def set_threads(self, threads: int) -> None:
        """OpenMP threads of the following calls (results do not depend on it)."""
        self._s.threads = max(1, int(threads))

    def update(self, keys: np.ndarray, values: np.ndarray) -> None:
        k = np.ascontiguousarray(keys, np.uint64)
        v = np.ascontiguousarray(values, np.uint8)
        assert len(k) == len(v)
        rc = lib().oracle_update(self._g, k.ctypes.data, v.ctypes.data, len(k))
        assert rc == 0

    def geometry(self) -> dict:
        s = self._s
        return {"size": s.size, "segment_length": s.segment_length, "tree_height": s.tree_height,
                "row_num": s.row_num}

    def thresholds(self):
        s = self._s
        h = s.tree_height
        return (np.ctypeslib.as_array(s.lower, (h + 1,)).copy(), np.ctypeslib.as_array(s.upper, (h + 1,)).copy())

    def export_layout(self):
        s = self._s
        keys = np.empty(s.size, np.uint64)
        vals = np.empty(s.size, np.uint8)
        ro = np.empty(s.row_num + 1, np.uint32)
        lib().oracle_export(self._g, keys.ctypes.data, vals.ctypes.data, ro.ctypes.data)
        return keys, vals, ro

    def compact_keys(self) -> np.ndarray:
        n = lib().oracle_compact(self._g, None)
        out = np.empty(n, np.uint64)
        lib().oracle_compact(self._g, out.ctypes.data)
        return out

    def bfs(self, src: int):
        levels = np.zeros(self.row_num, np.uint32)
        reached = ctypes.c_uint64()
        rc = lib().oracle_bfs(self._g, int(src), levels.ctypes.data, ctypes.byref(reached))
        if rc:
            raise ValueError("source out of range")
        return levels, reached.value

    def bfs_multi(self, sources):
        src = np.ascontiguousarray(np.asarray(sources, np.uint32))
        levels = np.zeros((len(src), self.row_num), np.uint32)
        reached = np.zeros(len(src), np.uint64)
        rc = lib().oracle_bfs_multi(self._g, src.ctypes.data, len(src), levels.ctypes.data, reached.ctypes.data)
        if rc:
            raise ValueError("source out of range")
        return levels, reached

    def traversed_edges(self, levels: np.ndarray) -> int:
        lv = np.ascontiguousarray(levels, np.uint32)
        return int(lib().oracle_traversed_edges(self._g, lv.ctypes.data))

    def stats(self) -> dict:
        s = self._s.stats
        return {name: getattr(s, name) for name, _ in _Stats._fields_}
