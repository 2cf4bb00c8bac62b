"""bench.py --impl reference: the reference algorithm (the oracle's
restatement) timed on the host cores, loading only oracle/ libraries (no GPU
needed)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_params_match_the_social_graph():
    sys.path.insert(0, str(ROOT))
    import bench
    from gpma_bfs_gb300.workloads import GRAPHS

    p = GRAPHS["social"]
    assert bench.SOCIAL == {k: p[k] for k in ("n", "m", "exponent", "max_degree", "seed")}


def test_reference_arm_runs_without_the_product_library(built_lib):
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3'];"
            "import bench; bench.main();"
            "maps = open('/proc/self/maps').read();"
            "print('LOADED', int('libgpma_gb300' in maps), int('libgpma_oracle' in maps))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=str(ROOT), timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["unit"] == "edge updates/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"]["edges"] == 30_622_564 and line["config"]["batch"] == 306_224
    assert lines[-1] == "LOADED 0 1", "the reference arm loaded the product library"
