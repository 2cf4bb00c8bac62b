"""Regenerates the golden vectors in tests/golden/*.npz from the reference.

Runs every case of cases.py through oracle/_ref/ref_driver, the reference's
own GPMA<CPU> + update_gpma + CPU BFS (built from the reference sources by
`make -C oracle ref`), and stores the per-operation results:

    python tests/golden/make_golden.py [case ...]

Needs oracle/_ref/ref_driver, built from a reference checkout with
`make -C oracle ref REF=<checkout>`; the fixtures it writes are committed,
so the tests never need the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import cases  # noqa: E402
from oracle.workload import digest, read_output, write_script  # noqa: E402

DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"


def records_to_arrays(n, ops, records, store_ops, input_digest=None) -> dict:
    """The per-operation results of one reference run, as the arrays a fixture holds."""
    kinds, lens, srcs = [], [], []
    uk, uv = [], []
    for op in ops:
        if op[0] == "update":
            kinds.append(1)
            lens.append(len(op[1]))
            srcs.append(0)
            if store_ops:
                uk.append(np.asarray(op[1], np.uint64))
                uv.append(np.asarray(op[2], np.uint8))
        elif op[0] == "bfs":
            kinds.append(2)
            lens.append(0)
            srcs.append(op[1])
        else:
            kinds.append(3)
            lens.append(0)
            srcs.append(0)
    upd = [r for r in records if r["op"] == "update"]
    bfs = [r for r in records if r["op"] == "bfs"]
    dmp = [r for r in records if r["op"] == "dump"]
    out = dict(
        row_num=np.uint32(n), op_kind=np.asarray(kinds, np.uint8), op_len=np.asarray(lens, np.uint64),
        op_src=np.asarray(srcs, np.uint32),
        rec_size=np.asarray([r["size"] for r in upd], np.uint32),
        rec_seg=np.asarray([r["segment_length"] for r in upd], np.uint32),
        rec_h=np.asarray([r["tree_height"] for r in upd], np.uint32),
        rec_live=np.asarray([r["live"] for r in upd], np.uint64),
        rec_dk=np.asarray([r["d_keys"] for r in upd], np.uint64),
        rec_dv=np.asarray([r["d_values"] for r in upd], np.uint64),
        rec_dr=np.asarray([r["d_row_offset"] for r in upd], np.uint64),
        rec_dc=np.asarray([r["d_compact"] for r in upd], np.uint64),
        rec_lower=np.concatenate([r["lower"] for r in upd]) if upd else np.zeros(0, np.uint32),
        rec_upper=np.concatenate([r["upper"] for r in upd]) if upd else np.zeros(0, np.uint32),
        bfs_src=np.asarray([r["src"] for r in bfs], np.uint32),
        bfs_reached=np.asarray([r["reached"] for r in bfs], np.uint64),
        bfs_digest=np.asarray([digest(r["levels"]) for r in bfs], np.uint64),
    )
    if store_ops:
        out["upd_keys"] = np.concatenate(uk) if uk else np.zeros(0, np.uint64)
        out["upd_vals"] = np.concatenate(uv) if uv else np.zeros(0, np.uint8)
        out["bfs_levels"] = np.concatenate([r["levels"] for r in bfs]) if bfs else np.zeros(0, np.uint32)
    if dmp:
        out["dump_size"] = np.asarray([len(r["keys"]) for r in dmp], np.uint64)
        out["dump_keys"] = np.concatenate([r["keys"] for r in dmp])
        out["dump_vals"] = np.concatenate([r["values"] for r in dmp])
        out["dump_ro"] = np.concatenate([r["row_offset"] for r in dmp])
    if input_digest is not None:
        out["input_digest"] = np.uint64(input_digest)
    return out


def encode(name, n, ops, records, store_ops, input_digest=None):
    np.savez_compressed(HERE / f"{name}.npz", **records_to_arrays(n, ops, records, store_ops, input_digest))


def run_reference(n, ops):
    with tempfile.TemporaryDirectory() as td:
        script = Path(td) / "w.gws"
        outp = Path(td) / "w.gwo"
        write_script(script, n, ops)
        env = dict(os.environ, OMP_NUM_THREADS=os.environ.get("OMP_NUM_THREADS", "8"))
        subprocess.run([str(DRIVER), str(script), str(outp)], check=True, env=env)
        return read_output(outp, n)


def main(names):
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref"], check=True, capture_output=True)
    todo = names or list(cases.SMALL) + list(cases.GENERATED)
    for name in todo:
        if name in cases.SMALL:
            n, ops = cases.SMALL[name]()
            recs = run_reference(n, ops)
            encode(name, n, ops, recs, store_ops=True)
        else:
            n, ops, keys = cases.generated_ops(name)
            recs = run_reference(n, ops)
            encode(name, n, ops, recs, store_ops=cases.GENERATED[name]["full"], input_digest=digest(keys))
        print(f"{name}: {sum(1 for o in ops if o[0] == 'update')} updates, "
              f"{(HERE / (name + '.npz')).stat().st_size} bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
