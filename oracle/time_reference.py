"""Times the reference's own GPMA<CPU> update against the oracle port.

Test infrastructure only: runs on a host where oracle/_ref/ref_driver was
built from the reference sources (`make -C oracle ref`). Both sides get the
social sliding window (1,632,803 nodes, 30,622,564 edges, slides of
153,112 inserts + 153,112 deletes): an untimed half-load, W warm-up slides,
then K timed slides. The reference side uses the driver's timed-update
operation (update_gpma alone, no layout digest); both run OpenMP on every
host core.

    python oracle/time_reference.py [K]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
import gpma_bfs_gb300 as G  # noqa: E402
from gpma_bfs_gb300.workloads import make_graph  # noqa: E402
from oracle.oracle import OracleGPMA  # noqa: E402
from oracle.workload import read_output, write_script  # noqa: E402

DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"
WARMUP = 3


def main(steps: int) -> None:
    if not DRIVER.exists():
        sys.exit(f"{DRIVER} is missing: build it with `make -C oracle ref` where the reference sources are")
    n, src, dst = make_graph(bench.GRAPH)
    keys = G.edges_to_keys(src, dst)
    half, step, slide = bench.schedule(keys)
    cores = os.cpu_count() or 1
    ops = [("timed_update", keys[:half], np.ones(half, np.uint8))]
    ops += [("timed_update", *slide(i)) for i in range(WARMUP + steps)]
    with tempfile.TemporaryDirectory() as td:
        write_script(Path(td) / "s.gws", n, ops)
        subprocess.run([str(DRIVER), str(Path(td) / "s.gws"), str(Path(td) / "s.gwo")], check=True,
                       env=dict(os.environ, OMP_NUM_THREADS=str(cores)))
        recs = read_output(Path(td) / "s.gwo", n)
    ref_t = sum(r["seconds"] for r in recs[1 + WARMUP:])
    print(f"reference GPMA<CPU>: load of {half:,} edges {recs[0]['seconds']:.2f} s; {steps} slides of {2 * step:,} "
          f"keys: {steps * 2 * step / ref_t:.3e} updates/s ({1e3 * ref_t / steps:.1f} ms each), {cores} threads")
    o = OracleGPMA(n, threads=cores)
    t0 = time.perf_counter()
    o.update(keys[:half], np.ones(half, np.uint8))
    load = time.perf_counter() - t0
    for i in range(WARMUP):
        o.update(*slide(i))
    port_t = 0.0
    for i in range(WARMUP, WARMUP + steps):
        k, v = slide(i)
        t0 = time.perf_counter()
        o.update(k, v)
        port_t += time.perf_counter() - t0
    o.close()
    print(f"oracle port:         load of {half:,} edges {load:.2f} s; {steps} slides of {2 * step:,} "
          f"keys: {steps * 2 * step / port_t:.3e} updates/s ({1e3 * port_t / steps:.1f} ms each), {cores} threads")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 10)
