"""Builds libgpma_gb300.so in-tree for sm_103a (GB300).

Each CUDA translation unit is compiled by nvcc in parallel with one
``-gencode arch=compute_103a,code=sm_103a``; the host-only generators are
compiled by gcc with OpenMP; everything is linked into
``gpma_bfs_gb300/libgpma_gb300.so`` with the CUDA runtime linked statically.
Objects go to ``gpma_bfs_gb300/_build/``. A source newer than its object is
rebuilt; nothing else is.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgpma_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}"]
CC_FLAGS = ["-O2", "-std=c11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}"]

CU_SOURCES = ["update.cu", "bfs.cu", "msbfs.cu", "capi.cu", "server.cu", "analytics.cu", "step.cu"]
C_SOURCES = ["graphgen.c"]
HEADERS = [CSRC / "gpma_internal.cuh", CSRC / "sort.cuh", INCLUDE / "gpma_gb300.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *HEADERS] if p.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("GPMA_BUILD_VERBOSE") and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    """Compiles (if needed) and returns the path of libgpma_gb300.so.

    GPMA_SORT_ITEMS (environment) sets the keys per thread of a radix-sort
    tile and GPMA_BFS_LANE_SLOTS the slots a BFS lane walks per step;
    changing either rebuilds.
    """
    if verbose:
        os.environ["GPMA_BUILD_VERBOSE"] = "1"
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    sort_items = os.environ.get("GPMA_SORT_ITEMS", "8")
    lane_slots = os.environ.get("GPMA_BFS_LANE_SLOTS", "4")
    lookback = os.environ.get("GPMA_SORT_LOOKBACK", "8")
    stamp = BUILD / "options.txt"
    options = f"GPMA_SORT_ITEMS={sort_items}\nGPMA_BFS_LANE_SLOTS={lane_slots}\nGPMA_SORT_LOOKBACK={lookback}\n"
    if not stamp.exists() or stamp.read_text() != options:
        stamp.write_text(options)
    NVCC_FLAGS.append(f"-DGPMA_SORT_ITEMS={sort_items}")
    NVCC_FLAGS.append(f"-DGPMA_BFS_LANE_SLOTS={lane_slots}")
    NVCC_FLAGS.append(f"-DGPMA_SORT_LOOKBACK={lookback}")
    HEADERS.append(stamp)
    jobs = []
    objs = []
    for name in CU_SOURCES:
        src, obj = CSRC / name, BUILD / (name + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)])
    cc = os.environ.get("CC", "gcc")
    for name in C_SOURCES:
        src, obj = CSRC / name, BUILD / (name + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([cc, *CC_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lgomp"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
