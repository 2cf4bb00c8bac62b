"""GB300-native GPMA+ (dynamic graph in a GPU packed memory array) and BFS.

Python mirror of the reference's C++ interface (recolic/gpma_bfs), over the
C ABI in ``include/gpma_gb300.h`` (``libgpma_gb300.so``, built in-tree for
sm_103a by ``gpma_bfs_gb300/build.py``):

* ``GPMA(row_num)``                      - ``GPMA<GPU>::GPMA`` (gpma.cuh:79-82)
* ``update_gpma(gpma, keys, values)``    - ``update_gpma`` (gpma.cuh:968-1050)
* ``gpma_bfs(gpma, node_size, edge_size, start_node, results)``
                                         - ``gpma_bfs`` (gpma_bfs.cuh:511-533)

Arrays may be numpy arrays (host) or torch tensors (host or CUDA). There is
no CPU fallback: every compute call goes to the CUDA library, and importing
fails loudly if the library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

__all__ = [
    "GPMA", "GPMAError", "update_gpma", "gpma_bfs", "gpma_bfs_multi", "lib", "library_path",
    "KEY_NONE", "KEY_MAX", "COL_IDX_NONE", "VALUE_NONE", "gen_rmat", "gen_chung_lu", "edges_to_keys",
    "read_edges_text", "write_edges_text", "Step", "partition_rows", "shard_first_row",
]

KEY_NONE = 0xFFFFFFFFFFFFFFFF  # gpma.cuh:15
KEY_MAX = KEY_NONE - 1         # gpma.cuh:16
COL_IDX_NONE = 0xFFFFFFFF      # gpma.cuh:19
VALUE_NONE = 0                 # gpma.cuh:18

_PKG = Path(__file__).resolve().parent
library_path = _PKG / "libgpma_gb300.so"

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "out of memory", 4: "capacity exceeded",
          5: "device wait timed out", 6: "I/O error", 7: "device-side check failed", 8: "server queue full",
          9: "HBM admission budget exceeded"}
ERR_BUSY = 8
ERR_BUDGET = 9


class GPMAError(RuntimeError):
    """A C-ABI call returned a non-zero gpma_status."""

    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {detail}")
        self.status = status


class _Geometry(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32), ("segment_length", ctypes.c_uint32),
                ("tree_height", ctypes.c_uint32), ("row_num", ctypes.c_uint32)]


class _Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "updates", "submitted", "last_inserts", "levels_visited", "accepted_windows", "accepted_slots",
        "root_resizes", "root_drops", "significant")]


class _Profile(ctypes.Structure):
    _fields_ = [("sort_ms", ctypes.c_double), ("locate_ms", ctypes.c_double), ("group_ms", ctypes.c_double),
                ("levels_ms", ctypes.c_double), ("update_kernel_ms", ctypes.c_double), ("rebuild_ms", ctypes.c_double),
                ("bfs_ms", ctypes.c_double), ("update_kernels", ctypes.c_uint64), ("bfs_kernels", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("bfs_edges", ctypes.c_uint64), ("sort_fallbacks", ctypes.c_uint64)]


class _Tuning(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("bfs_dense_div", "bfs_blocks_per_sm", "ms_dense_div",
                                               "ms_blocks_per_sm", "update_blocks_per_sm", "update_sort")] + \
               [("reserved", ctypes.c_uint32 * 2)]


class _TestHooks(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("update_stall", "bfs_stall", "wait_limit_us", "noalloc_chunk_cap",
                                               "noalloc_overflows")] + [("reserved", ctypes.c_uint32 * 3)]


class _StepStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("runs", "graph_launches", "builds", "param_updates", "host_runs")] + \
        [("last_ms", ctypes.c_double), ("total_ms", ctypes.c_double)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_round_keys", ctypes.c_uint64),
                ("max_round_bfs_graphs", ctypes.c_uint32), ("max_queued", ctypes.c_uint32),
                ("max_queued_keys", ctypes.c_uint64), ("flags", ctypes.c_uint32), ("lanes", ctypes.c_uint32),
                ("input_ring_bytes", ctypes.c_uint64)]


class _ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("rounds", "requests", "keys", "edges")] + \
        [(n, ctypes.c_double) for n in ("busy_seconds", "update_ms", "bfs_ms")] + \
        [(n, ctypes.c_uint32) for n in ("max_round_requests", "max_inflight_rounds")]


class _RequestInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("graph", ctypes.c_uint32), ("kind", ctypes.c_uint32),
                ("state", ctypes.c_uint32), ("status", ctypes.c_int32), ("arrival", ctypes.c_double),
                ("start", ctypes.c_double), ("done", ctypes.c_double), ("round", ctypes.c_uint64),
                ("keys", ctypes.c_uint64), ("nsrc", ctypes.c_uint32), ("lane", ctypes.c_uint32),
                ("reached", ctypes.c_uint64 * 64)]


class _RoundInfo(ctypes.Structure):
    _fields_ = [("round", ctypes.c_uint64), ("start", ctypes.c_double), ("seconds", ctypes.c_double),
                ("updates", ctypes.c_uint32), ("bfs_requests", ctypes.c_uint32), ("bfs_graphs", ctypes.c_uint32),
                ("failed", ctypes.c_uint32), ("keys", ctypes.c_uint64), ("sources", ctypes.c_uint64),
                ("edges", ctypes.c_uint64), ("update_ms", ctypes.c_double), ("bfs_ms", ctypes.c_double)]


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("GPMA_GB300_LIB", library_path))
    if not path.exists():
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(str(path))
    P, u32, u64, st = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    sig = {
        "gpma_create": (st, [u32, P, ctypes.POINTER(P)]),
        "gpma_destroy": (st, [P]),
        "gpma_update": (st, [P, P, P, u64, P]),
        "gpma_bfs": (st, [P, u32, P, ctypes.POINTER(u64), P]),
        "gpma_bfs_multi": (st, [P, P, u32, P, P, P]),
        "gpma_bfs_noalloc": (st, [P, u32, P, ctypes.POINTER(u64), P]),
        "gpma_get_geometry": (st, [P, ctypes.POINTER(_Geometry)]),
        "gpma_get_thresholds": (st, [P, P, P]),
        "gpma_export_layout": (st, [P, P, P, P, P]),
        "gpma_export_compact": (st, [P, P, u64, ctypes.POINTER(u64), P]),
        "gpma_device_arrays": (st, [P, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P)]),
        "gpma_get_stats": (st, [P, ctypes.POINTER(_Stats)]),
        "gpma_batch_create": (st, [ctypes.POINTER(P)]),
        "gpma_batch_destroy": (st, [P]),
        "gpma_batch_update": (st, [P, P, P, P, P, u32, P]),
        "gpma_batch_bfs_multi": (st, [P, P, P, P, u32, P, P, P]),
        "gpma_batch_update_packed": (st, [P, P, P, P, P, u32, P]),
        "gpma_batch_set_profiling": (st, [P, ctypes.c_int]),
        "gpma_batch_get_profile": (st, [P, ctypes.POINTER(_Profile)]),
        "gpma_batch_reset_profile": (st, [P]),
        "gpma_server_create": (st, [ctypes.POINTER(_ServerConfig), P, ctypes.POINTER(P)]),
        "gpma_server_destroy": (st, [P]),
        "gpma_server_add_graph": (st, [P, u32, u64, ctypes.POINTER(u32)]),
        "gpma_server_graph": (st, [P, u32, ctypes.POINTER(P)]),
        "gpma_server_cancel": (st, [P, u64]),
        "gpma_server_submit_update": (st, [P, u32, P, P, u64, ctypes.c_double, ctypes.POINTER(u64)]),
        "gpma_server_submit_bfs": (st, [P, u32, P, u32, ctypes.c_double, P, ctypes.POINTER(u64)]),
        "gpma_server_run_round": (st, [P, ctypes.c_double, ctypes.POINTER(_RoundInfo)]),
        "gpma_server_poll": (st, [P, u64, ctypes.c_int, ctypes.POINTER(_RequestInfo)]),
        "gpma_server_last_round": (st, [P, P, u32, ctypes.POINTER(u32)]),
        "gpma_server_queued": (st, [P, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_double)]),
        "gpma_server_committed_bytes": (st, [P, ctypes.POINTER(u64)]),
        "gpma_server_start": (st, [P]),
        "gpma_server_clock": (st, [P, ctypes.POINTER(ctypes.c_double)]),
        "gpma_server_drain": (st, [P, ctypes.c_double]),
        "gpma_server_stop": (st, [P]),
        "gpma_server_get_stats": (st, [P, ctypes.POINTER(_ServerStats)]),
        "gpma_get_tuning": (st, [ctypes.POINTER(_Tuning)]),
        "gpma_bfs_level_profile": (st, [P, P, P, P, u32, ctypes.POINTER(u32)]),
        "gpma_set_tuning": (st, [ctypes.POINTER(_Tuning)]),
        "gpma_get_test_hooks": (st, [ctypes.POINTER(_TestHooks)]),
        "gpma_set_test_hooks": (st, [ctypes.POINTER(_TestHooks)]),
        "gpma_set_profiling": (st, [P, ctypes.c_int]),
        "gpma_get_profile": (st, [P, ctypes.POINTER(_Profile)]),
        "gpma_reset_profile": (st, [P]),
        "gpma_status_string": (ctypes.c_char_p, [st]),
        "gpma_last_error": (ctypes.c_char_p, []),
        "gpma_version": (ctypes.c_char_p, []),
        "gpma_gen_rmat": (st, [u32, u32, ctypes.c_double, ctypes.c_double, ctypes.c_double, u64, P, P, u64,
                               ctypes.POINTER(u64)]),
        "gpma_gen_chung_lu": (st, [u32, u64, ctypes.c_double, u32, u64, P, P]),
        "gpma_edges_to_keys": (st, [P, P, u64, P]),
        "gpma_read_edges_text": (st, [ctypes.c_char_p, ctypes.POINTER(u32), ctypes.POINTER(u64), P, P, u64]),
        "gpma_write_edges_text": (st, [ctypes.c_char_p, u32, P, P, u64]),
        "gpma_read_edges_bin": (st, [ctypes.c_char_p, ctypes.POINTER(u32), ctypes.POINTER(u64), P, P, u64]),
        "gpma_write_edges_bin": (st, [ctypes.c_char_p, u32, P, P, u64]),
        "gpma_save": (st, [P, ctypes.c_char_p, P]),
        "gpma_pagerank": (st, [P, ctypes.c_float, u32, ctypes.c_double, P, ctypes.POINTER(u32), P]),
        "gpma_components": (st, [P, P, ctypes.POINTER(u64), ctypes.POINTER(u32), P]),
        "gpma_load": (st, [ctypes.c_char_p, P, ctypes.POINTER(P)]),
        "gpma_validate": (st, [P, ctypes.POINTER(u64), P]),
        "gpma_shard_first_row": (u32, [u32, u32, u32]),
        "gpma_partition_rows": (st, [P, P, u64, u32, u32, ctypes.c_int, P, P, P]),
        "gpma_step_create": (st, [P, ctypes.POINTER(P)]),
        "gpma_step_destroy": (st, [P]),
        "gpma_step_run": (st, [P, P, P, u64, u32, P, ctypes.POINTER(u64), P]),
        "gpma_step_get_stats": (st, [P, ctypes.POINTER(_StepStats)]),
        "gpma_batch_step_create": (st, [P, P, u32, ctypes.POINTER(P)]),
        "gpma_batch_step_destroy": (st, [P]),
        "gpma_batch_step_run": (st, [P, P, P, P, P, P, P, P]),
        "gpma_batch_step_run_many": (st, [P, u32, P, P, P, P, P, P, P]),
        "gpma_batch_step_get_stats": (st, [P, ctypes.POINTER(_StepStats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(status: int, where: str) -> None:
    if status != 0:
        raise GPMAError(status, where, lib().gpma_last_error().decode(errors="replace"))


def _ptr(a) -> tuple[int, object]:
    """(address, keep-alive) of a contiguous numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            a = np.ascontiguousarray(a)
        return a.ctypes.data, a
    data_ptr = getattr(a, "data_ptr", None)
    if data_ptr is not None:
        if not a.is_contiguous():
            a = a.contiguous()
        return a.data_ptr(), a
    raise TypeError(f"expected a numpy array or torch tensor, got {type(a).__name__}")


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


def _is_cuda(a) -> bool:
    return getattr(a, "is_cuda", False)


class GPMA:
    """A dynamic directed graph of ``row_num`` nodes on the current GPU.

    Mirrors ``GPMA<GPU>`` (gpma.cuh:31-102): the constructor inserts one guard
    key per row; ``keys``, ``values`` and ``row_offset`` are exported copies of
    the device arrays; ``segment_length``, ``tree_height``, ``lower_element``
    and ``upper_element`` are the current geometry and density thresholds.
    """

    def __init__(self, row_num: int, stream=None):
        if row_num < 0 or row_num >= 0xFFFFFFFF:
            raise ValueError(f"row_num {row_num} out of range")
        h = ctypes.c_void_p()
        _check(lib().gpma_create(int(row_num), _stream_ptr(stream), ctypes.byref(h)), "gpma_create")
        self._h = h
        self.row_num = int(row_num)
        self._owned = True

    @classmethod
    def _view(cls, handle: ctypes.c_void_p, row_num: int) -> "GPMA":
        """A non-owning wrapper of a graph that something else (a Server) owns."""
        g = cls.__new__(cls)
        g._h = handle
        g.row_num = int(row_num)
        g._owned = False
        return g

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                lib().gpma_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._h:
            raise ValueError("GPMA handle is closed")
        return self._h

    def geometry(self) -> dict:
        g = _Geometry()
        _check(lib().gpma_get_geometry(self.handle, ctypes.byref(g)), "gpma_get_geometry")
        return {"size": g.size, "segment_length": g.segment_length, "tree_height": g.tree_height,
                "row_num": g.row_num}

    def get_size(self) -> int:
        return self.geometry()["size"]

    @property
    def segment_length(self) -> int:
        return self.geometry()["segment_length"]

    @property
    def tree_height(self) -> int:
        return self.geometry()["tree_height"]

    def thresholds(self) -> tuple[np.ndarray, np.ndarray]:
        h = self.tree_height
        lo = np.zeros(h + 1, np.uint32)
        hi = np.zeros(h + 1, np.uint32)
        _check(lib().gpma_get_thresholds(self.handle, lo.ctypes.data, hi.ctypes.data), "gpma_get_thresholds")
        return lo, hi

    @property
    def lower_element(self) -> np.ndarray:
        return self.thresholds()[0]

    @property
    def upper_element(self) -> np.ndarray:
        return self.thresholds()[1]

    def validate(self, stream=None) -> int:
        """Segments whose cached first key differs from the array (0 when
        the structure is consistent)."""
        bad = ctypes.c_uint64()
        _check(lib().gpma_validate(self.handle, ctypes.byref(bad), _stream_ptr(stream)), "gpma_validate")
        return bad.value

    def export_layout(self, stream=None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(keys, masked values, row_offset) as host arrays."""
        size = self.get_size()
        keys = np.empty(size, np.uint64)
        vals = np.empty(size, np.uint8)
        ro = np.empty(self.row_num + 1, np.uint32)
        _check(lib().gpma_export_layout(self.handle, keys.ctypes.data, vals.ctypes.data, ro.ctypes.data,
                                        _stream_ptr(stream)), "gpma_export_layout")
        return keys, vals, ro

    @property
    def keys(self) -> np.ndarray:
        return self.export_layout()[0]

    @property
    def values(self) -> np.ndarray:
        return self.export_layout()[1]

    @property
    def row_offset(self) -> np.ndarray:
        return self.export_layout()[2]

    def compact_keys(self, stream=None) -> np.ndarray:
        n = ctypes.c_uint64()
        _check(lib().gpma_export_compact(self.handle, None, 0, ctypes.byref(n), _stream_ptr(stream)),
               "gpma_export_compact")
        out = np.empty(n.value, np.uint64)
        _check(lib().gpma_export_compact(self.handle, out.ctypes.data, n.value, ctypes.byref(n),
                                         _stream_ptr(stream)), "gpma_export_compact")
        return out

    def stats(self) -> dict:
        s = _Stats()
        _check(lib().gpma_get_stats(self.handle, ctypes.byref(s)), "gpma_get_stats")
        return {name: getattr(s, name) for name, _ in _Stats._fields_}

    def set_profiling(self, enabled: bool = True) -> None:
        """Time each phase with CUDA events on the calling stream."""
        _check(lib().gpma_set_profiling(self.handle, int(bool(enabled))), "gpma_set_profiling")

    def profile(self) -> dict:
        p = _Profile()
        _check(lib().gpma_get_profile(self.handle, ctypes.byref(p)), "gpma_get_profile")
        return {name: getattr(p, name) for name, _ in _Profile._fields_}

    def reset_profile(self) -> None:
        _check(lib().gpma_reset_profile(self.handle), "gpma_reset_profile")

    def bfs_levels_profile(self) -> list[dict]:
        """Per level of the last profiled gpma_bfs: ms, frontier size, dense sweep or row walk."""
        cap = 64
        ms = np.zeros(cap)
        fr = np.zeros(cap, np.uint32)
        de = np.zeros(cap, np.uint8)
        n = ctypes.c_uint32()
        _check(lib().gpma_bfs_level_profile(self.handle, ms.ctypes.data, fr.ctypes.data, de.ctypes.data, cap,
                                            ctypes.byref(n)), "gpma_bfs_level_profile")
        k = min(n.value, cap)
        return [{"ms": float(ms[i]), "frontier": int(fr[i]), "dense": bool(de[i])} for i in range(k)]

    def device_arrays(self) -> tuple[int, int, int]:
        k, v, r = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().gpma_device_arrays(self.handle, ctypes.byref(k), ctypes.byref(v), ctypes.byref(r)),
               "gpma_device_arrays")
        return k.value, v.value, r.value


def update_gpma(gpma: GPMA, update_keys, update_values, stream=None) -> None:
    """Applies one batch: value 0 deletes a key, non-zero inserts or modifies.

    Raises ValueError when the key and value counts differ, as the
    reference's batch entry throws std::invalid_argument (multidev.cuh:107-108).
    The inputs are left unmodified.
    """
    if len(update_keys) != len(update_values):
        raise ValueError("Inconsistant kv size.")
    n = len(update_keys)
    if isinstance(update_keys, np.ndarray):
        update_keys = np.ascontiguousarray(update_keys, dtype=np.uint64)
    if isinstance(update_values, np.ndarray):
        update_values = np.ascontiguousarray(update_values).view(np.uint8) \
            if update_values.dtype.itemsize == 1 else np.ascontiguousarray(update_values, dtype=np.uint8)
    kp, kk = _ptr(update_keys)
    vp, vk = _ptr(update_values)
    _check(lib().gpma_update(gpma.handle, kp, vp, n, _stream_ptr(stream)), "gpma_update")
    del kk, vk


def gpma_bfs(gpma: GPMA, node_size: int, edge_size: int, start_node: int, results=None, stream=None):
    """BFS levels from start_node (1 = start, 0 = unreached) into results.

    ``results`` (numpy uint32 array, or torch int32/uint32 tensor on host or
    GPU, ``node_size`` entries) is allocated when omitted. edge_size is
    accepted for signature parity (the reference sized its queues with it).
    Returns (results, reachable node count).
    """
    del edge_size
    if node_size != gpma.row_num:
        raise ValueError(f"node_size {node_size} != row_num {gpma.row_num}")
    if results is None:
        results = np.zeros(node_size, np.uint32)
    if len(results) < node_size:
        raise ValueError("results holds fewer than node_size entries")
    rp, keep = _ptr(results)
    reached = ctypes.c_uint64()
    _check(lib().gpma_bfs(gpma.handle, int(start_node), rp, ctypes.byref(reached), _stream_ptr(stream)), "gpma_bfs")
    del keep
    return results, reached.value


def shard_first_row(row_num: int, shards: int, s: int) -> int:
    """First row of shard s when row_num rows are split into `shards` row
    ranges (floor(row_num * s / shards))."""
    return int(lib().gpma_shard_first_row(row_num, shards, s))


def partition_rows(keys, values, row_num: int, shards: int, rebase: bool = True):
    """Orders a host batch by the row-range shard of each key's source row,
    stably; returns (keys, values, offsets) with shard s's part at
    offsets[s]:offsets[s+1]. With rebase the source rows become shard-local.
    The exchange step a graph sharded by row range needs per update."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    values = np.ascontiguousarray(values, dtype=np.uint8)
    if len(keys) != len(values):
        raise ValueError("Inconsistant kv size.")
    ok, ov = np.empty_like(keys), np.empty_like(values)
    off = np.zeros(shards + 1, np.uint64)
    _check(lib().gpma_partition_rows(keys.ctypes.data, values.ctypes.data, len(keys), row_num, shards, int(rebase),
                                     ok.ctypes.data, ov.ctypes.data, off.ctypes.data), "gpma_partition_rows")
    return ok, ov, off


class Step:
    """One slide step of a graph -- update_gpma of a batch, then gpma_bfs
    from a source -- recorded as a CUDA graph on first use and replayed for
    every later step (gpma_step_* in the C ABI). ``run`` returns exactly what
    update_gpma followed by gpma_bfs returns. Close the step before its graph.
    """

    def __init__(self, gpma: GPMA):
        self.gpma = gpma
        h = ctypes.c_void_p()
        _check(lib().gpma_step_create(gpma.handle, ctypes.byref(h)), "gpma_step_create")
        self.handle = h

    def run(self, update_keys, update_values, start_node: int, results=None, stream=None) -> int:
        """Applies the batch, runs the BFS from start_node and returns the
        reachable node count; levels go to ``results`` (host or device,
        row_num entries) when given."""
        if len(update_keys) != len(update_values):
            raise ValueError("Inconsistant kv size.")
        if isinstance(update_keys, np.ndarray):
            update_keys = np.ascontiguousarray(update_keys, dtype=np.uint64)
        if isinstance(update_values, np.ndarray):
            update_values = np.ascontiguousarray(update_values).view(np.uint8) \
                if update_values.dtype.itemsize == 1 else np.ascontiguousarray(update_values, dtype=np.uint8)
        n = len(update_keys)
        kp, kk = _ptr(update_keys) if n else (None, None)
        vp, vk = _ptr(update_values) if n else (None, None)
        rp, rk = (None, None)
        if results is not None:
            if len(results) < self.gpma.row_num:
                raise ValueError("results holds fewer than row_num entries")
            rp, rk = _ptr(results)
        reached = ctypes.c_uint64()
        _check(lib().gpma_step_run(self.handle, kp, vp, n, int(start_node), rp, ctypes.byref(reached),
                                   _stream_ptr(stream)), "gpma_step_run")
        del kk, vk, rk
        return reached.value

    def stats(self) -> dict:
        s = _StepStats()
        _check(lib().gpma_step_get_stats(self.handle, ctypes.byref(s)), "gpma_step_get_stats")
        return {n: getattr(s, n) for n, _ in _StepStats._fields_}

    def close(self) -> None:
        if self.handle:
            lib().gpma_step_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def gpma_bfs_multi(gpma: GPMA, sources, results=None, stream=None):
    """Up to 64 BFS at once; results is [k][row_num] uint32. Returns (results, reached[k])."""
    src = np.ascontiguousarray(np.asarray(sources, dtype=np.uint32))
    k = len(src)
    if results is None:
        results = np.zeros((k, gpma.row_num), np.uint32)
    rp, keep = _ptr(results)
    reached = np.zeros(k, np.uint64)
    _check(lib().gpma_bfs_multi(gpma.handle, src.ctypes.data, k, rp, reached.ctypes.data, _stream_ptr(stream)),
           "gpma_bfs_multi")
    del keep
    return results, reached


def pagerank(gpma: GPMA, damping: float = 0.85, iterations: int = 20, tol: float = 0.0, out=None, stream=None):
    """(ranks float32[row_num], iterations run). `out` may be a host array or
    a CUDA tensor of row_num float32."""
    if out is None:
        out = np.zeros(gpma.row_num, np.float32)
    p, keep = _ptr(out)
    it = ctypes.c_uint32()
    _check(lib().gpma_pagerank(gpma.handle, float(damping), int(iterations), float(tol), p, ctypes.byref(it),
                               _stream_ptr(stream)), "gpma_pagerank")
    del keep
    return out, it.value


def components(gpma: GPMA, out=None, stream=None):
    """(labels uint32[row_num]: smallest node id of each node's weakly
    connected component, component count, rounds)."""
    if out is None:
        out = np.zeros(gpma.row_num, np.uint32)
    p, keep = _ptr(out)
    c, r = ctypes.c_uint64(), ctypes.c_uint32()
    _check(lib().gpma_components(gpma.handle, p, ctypes.byref(c), ctypes.byref(r), _stream_ptr(stream)),
           "gpma_components")
    del keep
    return out, c.value, r.value


TUNING_FIELDS = ("bfs_dense_div", "bfs_blocks_per_sm", "ms_dense_div", "ms_blocks_per_sm", "update_blocks_per_sm",
                 "update_sort")


def get_tuning() -> dict:
    """Launch shapes and switch points in effect (they never change results)."""
    t = _Tuning()
    _check(lib().gpma_get_tuning(ctypes.byref(t)), "gpma_get_tuning")
    return {n: getattr(t, n) for n in TUNING_FIELDS}


def set_tuning(**values) -> dict:
    """Changes some tuning fields; returns the previous settings."""
    old = get_tuning()
    unknown = set(values) - set(TUNING_FIELDS)
    if unknown:
        raise ValueError(f"unknown tuning fields {sorted(unknown)}")
    t = _Tuning(*[int(values.get(n, old[n])) for n in TUNING_FIELDS])
    _check(lib().gpma_set_tuning(ctypes.byref(t)), "gpma_set_tuning")
    return old


TEST_HOOK_FIELDS = ("update_stall", "bfs_stall", "wait_limit_us", "noalloc_chunk_cap")


def get_test_hooks() -> dict:
    """Error-path test hooks in effect, plus noalloc_overflows: how often the
    last gpma_bfs_noalloc call found its long-row chunk list full."""
    h = _TestHooks()
    _check(lib().gpma_get_test_hooks(ctypes.byref(h)), "gpma_get_test_hooks")
    return {n: getattr(h, n) for n in TEST_HOOK_FIELDS + ("noalloc_overflows",)}


def set_test_hooks(**values) -> dict:
    """Changes some test-hook fields (update_stall / bfs_stall: the next
    launches' first grid barrier waits for an arrival that never comes and
    gives up after wait_limit_us; noalloc_chunk_cap: entries of the
    no-allocation BFS's chunk list); returns the previous settings."""
    old = get_test_hooks()
    unknown = set(values) - set(TEST_HOOK_FIELDS)
    if unknown:
        raise ValueError(f"unknown test hooks {sorted(unknown)}")
    h = _TestHooks(*[int(values.get(n, old[n])) for n in TEST_HOOK_FIELDS])
    _check(lib().gpma_set_test_hooks(ctypes.byref(h)), "gpma_set_test_hooks")
    return {n: old[n] for n in TEST_HOOK_FIELDS}


# ---- synthetic graphs and the reference's text format -------------------------

def gen_rmat(scale: int, edge_factor: int, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 1):
    """R-MAT edge list (src, dst uint32), self-loops and duplicates removed, shuffled."""
    cap = edge_factor << scale
    src = np.empty(cap, np.uint32)
    dst = np.empty(cap, np.uint32)
    m = ctypes.c_uint64()
    _check(lib().gpma_gen_rmat(scale, edge_factor, a, b, c, seed, src.ctypes.data, dst.ctypes.data, cap,
                               ctypes.byref(m)), "gpma_gen_rmat")
    return src[: m.value].copy(), dst[: m.value].copy()


def gen_chung_lu(n: int, m: int, exponent: float = 2.3, max_degree: int = 9000, seed: int = 2):
    """Power-law edge list with exactly m distinct non-loop edges, shuffled."""
    src = np.empty(m, np.uint32)
    dst = np.empty(m, np.uint32)
    _check(lib().gpma_gen_chung_lu(n, m, exponent, max_degree, seed, src.ctypes.data, dst.ctypes.data),
           "gpma_gen_chung_lu")
    return src, dst


def edges_to_keys(src: np.ndarray, dst: np.ndarray) -> np.ndarray:
    """keys = (src << 32) + dst (gpma_bfs_demo.cu:53)."""
    return (src.astype(np.uint64) << np.uint64(32)) + dst.astype(np.uint64)


def write_edges_text(path: str, n: int, src: np.ndarray, dst: np.ndarray) -> None:
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    _check(lib().gpma_write_edges_text(str(path).encode(), n, src.ctypes.data, dst.ctypes.data, len(src)),
           "gpma_write_edges_text")


def write_edges_bin(path: str, n: int, src: np.ndarray, dst: np.ndarray) -> None:
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    _check(lib().gpma_write_edges_bin(str(path).encode(), n, src.ctypes.data, dst.ctypes.data, len(src)),
           "gpma_write_edges_bin")


def read_edges_bin(path: str):
    """(n, src, dst) from a binary edge list."""
    n = ctypes.c_uint32()
    m = ctypes.c_uint64()
    _check(lib().gpma_read_edges_bin(str(path).encode(), ctypes.byref(n), ctypes.byref(m), None, None, 0),
           "gpma_read_edges_bin")
    src = np.empty(m.value, np.uint32)
    dst = np.empty(m.value, np.uint32)
    _check(lib().gpma_read_edges_bin(str(path).encode(), ctypes.byref(n), ctypes.byref(m), src.ctypes.data,
                                     dst.ctypes.data, m.value), "gpma_read_edges_bin")
    return n.value, src, dst


def save(gpma: GPMA, path: str, stream=None) -> None:
    """Snapshot of the whole structure (exact layout) to `path`."""
    _check(lib().gpma_save(gpma.handle, str(path).encode(), _stream_ptr(stream)), "gpma_save")


def load(path: str, stream=None) -> GPMA:
    """A graph restored from a snapshot, with exactly the saved layout."""
    h = ctypes.c_void_p()
    _check(lib().gpma_load(str(path).encode(), _stream_ptr(stream), ctypes.byref(h)), "gpma_load")
    g = GPMA.__new__(GPMA)
    g._h = h
    g._owned = True
    geo = _Geometry()
    _check(lib().gpma_get_geometry(h, ctypes.byref(geo)), "gpma_get_geometry")
    g.row_num = geo.row_num
    return g


def read_edges_text(path: str):
    """(n, src, dst) from a text edge list in the reference's format."""
    n = ctypes.c_uint32()
    m = ctypes.c_uint64()
    _check(lib().gpma_read_edges_text(str(path).encode(), ctypes.byref(n), ctypes.byref(m), None, None, 0),
           "gpma_read_edges_text")
    src = np.empty(m.value, np.uint32)
    dst = np.empty(m.value, np.uint32)
    _check(lib().gpma_read_edges_text(str(path).encode(), ctypes.byref(n), ctypes.byref(m), src.ctypes.data,
                                      dst.ctypes.data, m.value), "gpma_read_edges_text")
    return n.value, src, dst


class Batch:
    """Many graphs per launch (no reference counterpart).

    ``update(graphs, keys, values)`` applies one batch per graph in a single
    persistent kernel launch; ``bfs_multi(graphs, sources)`` runs up to 64
    searches per graph for all graphs in one launch.
    """

    def __init__(self):
        h = ctypes.c_void_p()
        _check(lib().gpma_batch_create(ctypes.byref(h)), "gpma_batch_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gpma_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, graphs, keys, values, stream=None) -> None:
        k = len(graphs)
        if not (len(keys) == len(values) == k):
            raise ValueError("one key array and one value array per graph")
        keep = []
        kp, vp, cnt = (ctypes.c_void_p * k)(), (ctypes.c_void_p * k)(), (ctypes.c_uint64 * k)()
        hs = (ctypes.c_void_p * k)()
        for i, (g, kk, vv) in enumerate(zip(graphs, keys, values)):
            if len(kk) != len(vv):
                raise ValueError("Inconsistant kv size.")
            if isinstance(kk, np.ndarray):
                kk = np.ascontiguousarray(kk, dtype=np.uint64)
            if isinstance(vv, np.ndarray):
                vv = np.ascontiguousarray(vv).view(np.uint8) if vv.dtype.itemsize == 1 \
                    else np.ascontiguousarray(vv, dtype=np.uint8)
            a, ka = _ptr(kk)
            b, kb = _ptr(vv)
            keep += [ka, kb]
            kp[i], vp[i], cnt[i], hs[i] = a, b, len(kk), g.handle.value
        _check(lib().gpma_batch_update(self._h, hs, kp, vp, cnt, k, _stream_ptr(stream)), "gpma_batch_update")

    def update_packed(self, graphs, keys, values, offsets, stream=None) -> None:
        """All batches in one buffer: graph i gets keys[offsets[i]:offsets[i+1]]."""
        k = len(graphs)
        off = np.ascontiguousarray(np.asarray(offsets, np.uint64))
        if len(off) != k + 1 or len(keys) != len(values) or (k and int(off[-1]) > len(keys)):
            raise ValueError("offsets must have len(graphs) + 1 entries within the key array")
        if isinstance(keys, np.ndarray):
            keys = np.ascontiguousarray(keys, dtype=np.uint64)
        if isinstance(values, np.ndarray):
            values = np.ascontiguousarray(values).view(np.uint8) if values.dtype.itemsize == 1 \
                else np.ascontiguousarray(values, dtype=np.uint8)
        kp, kk = _ptr(keys)
        vp, vk = _ptr(values)
        hs = (ctypes.c_void_p * k)(*[g.handle.value for g in graphs])
        _check(lib().gpma_batch_update_packed(self._h, hs, kp, vp, off.ctypes.data, k, _stream_ptr(stream)),
               "gpma_batch_update_packed")
        del kk, vk

    def bfs_multi(self, graphs, sources, levels: bool = False, stream=None):
        """(levels per graph or None, reached per graph) for up to 64 sources per graph."""
        k = len(graphs)
        srcs = [np.ascontiguousarray(np.asarray(s, np.uint32)) for s in sources]
        hs = (ctypes.c_void_p * k)(*[g.handle.value for g in graphs])
        sp = (ctypes.c_void_p * k)(*[s.ctypes.data for s in srcs])
        ns = (ctypes.c_uint32 * k)(*[len(s) for s in srcs])
        outs = [np.zeros((len(s), g.row_num), np.uint32) for s, g in zip(srcs, graphs)] if levels else None
        lp = (ctypes.c_void_p * k)(*[o.ctypes.data for o in outs]) if levels else None
        reached = np.zeros(sum(len(s) for s in srcs), np.uint64)
        _check(lib().gpma_batch_bfs_multi(self._h, hs, sp, ns, k, lp, reached.ctypes.data, _stream_ptr(stream)),
               "gpma_batch_bfs_multi")
        parts, o = [], 0
        for s in srcs:
            parts.append(reached[o:o + len(s)])
            o += len(s)
        return outs, parts

    def set_profiling(self, enabled: bool = True) -> None:
        _check(lib().gpma_batch_set_profiling(self._h, int(bool(enabled))), "gpma_batch_set_profiling")

    def profile(self) -> dict:
        p = _Profile()
        _check(lib().gpma_batch_get_profile(self._h, ctypes.byref(p)), "gpma_batch_get_profile")
        return {name: getattr(p, name) for name, _ in _Profile._fields_}

    def reset_profile(self) -> None:
        _check(lib().gpma_batch_reset_profile(self._h), "gpma_batch_reset_profile")

    def step(self, graphs) -> "BatchStep":
        """A recorded step over these graphs: update_packed + bfs_multi as one CUDA graph."""
        return BatchStep(self, graphs)


class BatchStep:
    """The batched form's step (gpma_batch_step_*): one packed update of every
    graph and one multi-source BFS over all of them, recorded as a CUDA graph
    and replayed per step; results equal Batch.update_packed followed by
    Batch.bfs_multi (without levels). Close it before its batch and graphs."""

    def __init__(self, batch: Batch, graphs):
        self.batch, self.graphs = batch, list(graphs)
        k = len(self.graphs)
        hs = (ctypes.c_void_p * k)(*[g.handle.value for g in self.graphs])
        h = ctypes.c_void_p()
        _check(lib().gpma_batch_step_create(batch._h, hs, k, ctypes.byref(h)), "gpma_batch_step_create")
        self.handle = h

    def run(self, keys, values, offsets, sources, stream=None):
        """Applies the packed batches (graph i gets keys[offsets[i]:offsets[i+1]])
        and returns the reached counts per graph of the multi-source BFS."""
        k = len(self.graphs)
        off = np.ascontiguousarray(np.asarray(offsets, np.uint64))
        if len(off) != k + 1 or len(keys) != len(values) or int(off[-1]) > len(keys) or len(sources) != k:
            raise ValueError("offsets must have len(graphs) + 1 entries within the key array, one source list per graph")
        if isinstance(keys, np.ndarray):
            keys = np.ascontiguousarray(keys, dtype=np.uint64)
        if isinstance(values, np.ndarray):
            values = np.ascontiguousarray(values).view(np.uint8) if values.dtype.itemsize == 1 \
                else np.ascontiguousarray(values, dtype=np.uint8)
        kp, kk = _ptr(keys)
        vp, vk = _ptr(values)
        srcs = [np.ascontiguousarray(np.asarray(x, np.uint32)) for x in sources]
        sp = (ctypes.c_void_p * k)(*[x.ctypes.data for x in srcs])
        ns = (ctypes.c_uint32 * k)(*[len(x) for x in srcs])
        reached = np.zeros(sum(len(x) for x in srcs), np.uint64)
        _check(lib().gpma_batch_step_run(self.handle, kp, vp, off.ctypes.data, sp, ns, reached.ctypes.data,
                                         _stream_ptr(stream)), "gpma_batch_step_run")
        del kk, vk
        parts, o = [], 0
        for x in srcs:
            parts.append(reached[o:o + len(x)])
            o += len(x)
        return parts

    def run_many(self, keys, values, offsets, sources, stream=None):
        """Several steps in one recorded graph launch: step t applies keys[t] /
        values[t] (device tensors or device pointers) with offsets[t] (len(graphs)
        + 1 entries), each followed by the multi-source BFS from `sources`.
        Returns, per step, the reached counts per graph."""
        k, steps = len(self.graphs), len(keys)
        if len(values) != steps or len(offsets) != steps or len(sources) != k:
            raise ValueError("one key, value and offset array per step, one source list per graph")
        off = np.ascontiguousarray(np.stack([np.asarray(o, np.uint64) for o in offsets])) if steps else \
            np.zeros((0, k + 1), np.uint64)
        if off.shape != (steps, k + 1):
            raise ValueError("offsets must have len(graphs) + 1 entries per step")
        keep, kp, vp = [], (ctypes.c_void_p * max(steps, 1))(), (ctypes.c_void_p * max(steps, 1))()
        for t in range(steps):
            if len(keys[t]) != len(values[t]) or int(off[t, -1]) > len(keys[t]):
                raise ValueError(f"step {t}: offsets past the key array or key/value lengths differ")
            a, ka = _ptr(keys[t])
            b, kb = _ptr(values[t])
            keep += [ka, kb]
            kp[t], vp[t] = a, b
        srcs = [np.ascontiguousarray(np.asarray(x, np.uint32)) for x in sources]
        sp = (ctypes.c_void_p * k)(*[x.ctypes.data for x in srcs])
        ns = (ctypes.c_uint32 * k)(*[len(x) for x in srcs])
        per = sum(len(x) for x in srcs)
        reached = np.zeros(steps * per, np.uint64)
        _check(lib().gpma_batch_step_run_many(self.handle, steps, kp, vp, off.ctypes.data, sp, ns,
                                              reached.ctypes.data, _stream_ptr(stream)), "gpma_batch_step_run_many")
        del keep
        out = []
        for t in range(steps):
            parts, o = [], t * per
            for x in srcs:
                parts.append(reached[o:o + len(x)])
                o += len(x)
            out.append(parts)
        return out

    def stats(self) -> dict:
        st = _StepStats()
        _check(lib().gpma_batch_step_get_stats(self.handle, ctypes.byref(st)), "gpma_batch_step_get_stats")
        return {n: getattr(st, n) for n, _ in _StepStats._fields_}

    def close(self) -> None:
        if self.handle:
            lib().gpma_batch_step_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


PLAN_ONLY = 1


class Server:
    """Served form (no reference counterpart): resident graphs, update batches
    and BFS queries with continuous batching.

    ``submit_update`` / ``submit_bfs`` queue requests with their arrival time
    (raising GPMAError with status ERR_BUSY when the queue is full);
    ``poll(id)`` gives a request's state, times and BFS reach. Either the
    caller drives rounds (``run_round(now)``, on any clock, e.g. virtual time)
    or ``start()`` runs the native serving loop: one worker thread per lane on
    the server's own wall clock (``clock()``), rounds starting as soon as a
    request's arrival has passed and a lane is free; ``drain()`` waits for the
    queue to empty, ``stop()`` ends the loop. With ``lanes`` > 1 that many
    rounds are in flight at once, each on its own stream and buffers.
    ``input_ring_bytes`` sizes a pinned host ring that queued update batches
    are copied into at submission (uploads from pinned memory, however long
    a batch waited).
    """

    def __init__(self, hbm_budget_bytes: int = 120 << 30, max_round_keys: int = 1 << 24,
                 max_round_bfs_graphs: int = 4096, max_queued: int = 1 << 20, max_queued_keys: int = 1 << 28,
                 plan_only: bool = False, stream=None, lanes: int = 1, input_ring_bytes: int = 0):
        cfg = _ServerConfig(int(hbm_budget_bytes), int(max_round_keys), int(max_round_bfs_graphs), int(max_queued),
                            int(max_queued_keys), PLAN_ONLY if plan_only else 0, int(lanes), int(input_ring_bytes))
        h = ctypes.c_void_p()
        _check(lib().gpma_server_create(ctypes.byref(cfg), _stream_ptr(stream), ctypes.byref(h)), "gpma_server_create")
        self._h = h
        self._rows = []
        self._keep = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gpma_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_graph(self, row_num: int, reserve_edges: int = 0) -> int:
        gid = ctypes.c_uint32()
        _check(lib().gpma_server_add_graph(self._h, int(row_num), int(reserve_edges), ctypes.byref(gid)),
               "gpma_server_add_graph")
        self._rows.append(int(row_num))
        return gid.value

    def graph(self, gid: int):
        """The graph as a non-owning GPMA (None in plan-only mode)."""
        h = ctypes.c_void_p()
        _check(lib().gpma_server_graph(self._h, int(gid), ctypes.byref(h)), "gpma_server_graph")
        return GPMA._view(h, self._rows[gid]) if h.value else None

    def submit_update(self, gid: int, keys: np.ndarray, values: np.ndarray, arrival: float) -> int:
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values).view(np.uint8) if np.asarray(values).dtype.itemsize == 1 \
            else np.ascontiguousarray(values, dtype=np.uint8)
        if len(keys) != len(values):
            raise ValueError("Inconsistant kv size.")
        rid = ctypes.c_uint64()
        _check(lib().gpma_server_submit_update(self._h, int(gid), keys.ctypes.data, values.ctypes.data, len(keys),
                                               float(arrival), ctypes.byref(rid)), "gpma_server_submit_update")
        return rid.value

    def submit_bfs(self, gid: int, sources, arrival: float, levels: bool = False) -> int:
        """Queues a search; with levels=True the [k][row_num] level array is
        kept and returned by ``levels(id)`` once the request is done."""
        src = np.ascontiguousarray(np.asarray(sources, np.uint32))
        out = np.zeros((len(src), self._rows[gid]), np.uint32) if levels else None
        rid = ctypes.c_uint64()
        _check(lib().gpma_server_submit_bfs(self._h, int(gid), src.ctypes.data, len(src), float(arrival),
                                            out.ctypes.data if levels else None, ctypes.byref(rid)),
               "gpma_server_submit_bfs")
        if levels:
            self._keep[rid.value] = out
        return rid.value

    def run_round(self, now: float) -> dict:
        ri = _RoundInfo()
        _check(lib().gpma_server_run_round(self._h, float(now), ctypes.byref(ri)), "gpma_server_run_round")
        return {name: getattr(ri, name) for name, _ in _RoundInfo._fields_}

    def cancel(self, rid: int) -> None:
        """Withdraws a request no round has taken yet (state 3 afterwards)."""
        _check(lib().gpma_server_cancel(self._h, int(rid)), "gpma_server_cancel")
        self._keep.pop(int(rid), None)

    def poll(self, rid: int, release: bool = False) -> dict:
        info = _RequestInfo()
        _check(lib().gpma_server_poll(self._h, int(rid), int(bool(release)), ctypes.byref(info)), "gpma_server_poll")
        d = {name: getattr(info, name) for name, _ in _RequestInfo._fields_ if name != "reached"}
        d["reached"] = np.array(info.reached[: info.nsrc], np.uint64)
        return d

    def levels(self, rid: int):
        return self._keep.pop(rid, None)

    def last_round(self) -> list:
        n = ctypes.c_uint32()
        _check(lib().gpma_server_last_round(self._h, None, 0, ctypes.byref(n)), "gpma_server_last_round")
        ids = np.zeros(max(1, n.value), np.uint64)
        _check(lib().gpma_server_last_round(self._h, ids.ctypes.data, n.value, ctypes.byref(n)),
               "gpma_server_last_round")
        return [int(x) for x in ids[: n.value]]

    def queued(self) -> tuple[int, int, float]:
        r, k, t = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        _check(lib().gpma_server_queued(self._h, ctypes.byref(r), ctypes.byref(k), ctypes.byref(t)),
               "gpma_server_queued")
        return r.value, k.value, t.value

    def committed_bytes(self) -> int:
        b = ctypes.c_uint64()
        _check(lib().gpma_server_committed_bytes(self._h, ctypes.byref(b)), "gpma_server_committed_bytes")
        return b.value

    def start(self) -> None:
        """Starts the serving loop (the server's clock starts at 0)."""
        _check(lib().gpma_server_start(self._h), "gpma_server_start")

    def clock(self) -> float:
        t = ctypes.c_double()
        _check(lib().gpma_server_clock(self._h, ctypes.byref(t)), "gpma_server_clock")
        return t.value

    def drain(self, timeout: float = 600.0) -> None:
        """Waits until nothing is queued or running (raises on a failed round or the timeout)."""
        _check(lib().gpma_server_drain(self._h, float(timeout)), "gpma_server_drain")

    def stop(self) -> None:
        _check(lib().gpma_server_stop(self._h), "gpma_server_stop")

    def stats(self) -> dict:
        st = _ServerStats()
        _check(lib().gpma_server_get_stats(self._h, ctypes.byref(st)), "gpma_server_get_stats")
        return {name: getattr(st, name) for name, _ in _ServerStats._fields_}
