"""Replays golden-case scripts through an implementation and compares.

An implementation is any object with update(keys, values), bfs(src) ->
(levels, reached), export_layout() -> (keys, masked values, row_offset),
geometry() and thresholds(); the oracle (oracle.oracle.OracleGPMA) and the
GPU adapter below both qualify.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from oracle.workload import digest, state_record

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_case(name: str):
    """(row_num, ops, golden arrays) of a committed golden case."""
    import cases

    z = dict(np.load(GOLDEN / f"{name}.npz"))
    n = int(z["row_num"])
    if name in cases.SMALL:
        ops = []
        ko = 0
        ui = 0
        for kind, ln, src in zip(z["op_kind"], z["op_len"], z["op_src"]):
            if kind == 1:
                ln = int(ln)
                ops.append(("update", z["upd_keys"][ko:ko + ln], z["upd_vals"][ko:ko + ln]))
                ko += ln
                ui += 1
            elif kind == 2:
                ops.append(("bfs", int(src)))
            else:
                ops.append(("dump",))
    else:
        n2, ops, keys = cases.generated_ops(name)
        assert n2 == n
        assert digest(keys) == int(z["input_digest"]), "generator no longer reproduces the golden input"
    return n, ops, z


class GpuAdapter:
    """gpma_bfs_gb300.GPMA behind the replay interface (all calls through the C ABI)."""

    def __init__(self, n: int):
        import gpma_bfs_gb300 as G

        self.G = G
        self.g = G.GPMA(n)
        self.n = n

    def update(self, keys, values):
        self.G.update_gpma(self.g, np.asarray(keys, np.uint64), np.asarray(values, np.uint8))

    def bfs(self, src):
        levels, reached = self.G.gpma_bfs(self.g, self.n, 0, src)
        return levels, reached

    def export_layout(self):
        return self.g.export_layout()

    def geometry(self):
        return self.g.geometry()

    def thresholds(self):
        return self.g.thresholds()

    def close(self):
        self.g.close()


def record_after_update(impl) -> dict:
    keys, masked, ro = impl.export_layout()
    lo, hi = impl.thresholds()
    return state_record(keys, masked, ro, impl.geometry(), lo, hi)


def replay_and_compare(impl, ops, z, check_full=True, max_ops=None):
    """Runs ops on impl and asserts every per-op result equals the golden one."""
    ui = bi = di = 0
    lo_off = 0
    dump_off = ro_off = 0
    lev_off = 0
    n = int(z["row_num"])
    for oi, op in enumerate(ops[:max_ops]):
        if op[0] == "update":
            impl.update(op[1], op[2])
            r = record_after_update(impl)
            h = int(z["rec_h"][ui])
            ctx = f"op {oi} (update #{ui}, {len(op[1])} keys)"
            assert r["size"] == z["rec_size"][ui], ctx + " size"
            assert r["segment_length"] == z["rec_seg"][ui], ctx + " segment_length"
            assert r["tree_height"] == h, ctx + " tree_height"
            assert np.array_equal(r["lower"], z["rec_lower"][lo_off:lo_off + h + 1]), ctx + " lower_element"
            assert np.array_equal(r["upper"], z["rec_upper"][lo_off:lo_off + h + 1]), ctx + " upper_element"
            assert r["live"] == z["rec_live"][ui], ctx + " live count"
            assert r["d_compact"] == z["rec_dc"][ui], ctx + " compacted key set"
            assert r["d_keys"] == z["rec_dk"][ui], ctx + " key layout"
            assert r["d_values"] == z["rec_dv"][ui], ctx + " values"
            assert r["d_row_offset"] == z["rec_dr"][ui], ctx + " row_offset"
            lo_off += h + 1
            ui += 1
        elif op[0] == "bfs":
            levels, reached = impl.bfs(op[1])
            ctx = f"op {oi} (bfs #{bi} from {op[1]})"
            assert int(z["bfs_src"][bi]) == op[1]
            assert reached == z["bfs_reached"][bi], ctx + " reached"
            if "bfs_levels" in z and check_full:
                assert np.array_equal(levels, z["bfs_levels"][lev_off:lev_off + n]), ctx + " levels"
            assert digest(levels) == z["bfs_digest"][bi], ctx + " levels digest"
            lev_off += n
            bi += 1
        else:
            keys, masked, ro = impl.export_layout()
            size = int(z["dump_size"][di])
            ctx = f"op {oi} (dump #{di})"
            assert np.array_equal(keys, z["dump_keys"][dump_off:dump_off + size]), ctx + " keys"
            assert np.array_equal(masked, z["dump_vals"][dump_off:dump_off + size]), ctx + " values"
            assert np.array_equal(ro, z["dump_ro"][ro_off:ro_off + n + 1]), ctx + " row_offset"
            dump_off += size
            ro_off += n + 1
            di += 1
    return ui, bi, di
