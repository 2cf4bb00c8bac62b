"""Builds libgpma_gb300.so in-tree for sm_103a (GB300).

Each CUDA translation unit is compiled by nvcc in parallel with one
``-gencode arch=compute_103a,code=sm_103a``; the host-only generators are
compiled by gcc with OpenMP; everything is linked into
``gpma_bfs_gb300/libgpma_gb300.so`` with the CUDA runtime linked statically.
Objects go to ``gpma_bfs_gb300/_build/``. A source newer than its object is
rebuilt; nothing else is.

``build(checked=True)`` makes the bounds-checked variant
``libgpma_gb300_checked.so`` (objects in ``_build_checked/``): every
data-dependent index range of the kernels is checked before the access and a
failure returns GPMA_ERR_DEVICE instead of touching memory out of range. Point
``GPMA_GB300_LIB`` at it to run a program or the tests against it.
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
BUILD_CHECKED = PKG / "_build_checked"
LIB_CHECKED = PKG / "libgpma_gb300_checked.so"
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


def _stale(obj: Path, src: Path, headers: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *headers] if p.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("GPMA_BUILD_VERBOSE") and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)


def build(verbose: bool = False, ptxas_info: bool = False, checked: bool = False) -> Path:
    """Compiles (if needed) and returns the path of libgpma_gb300.so, or of
    libgpma_gb300_checked.so with ``checked``.

    GPMA_SORT_ITEMS (environment) sets the keys per thread of a radix-sort
    tile, GPMA_BFS_LANE_SLOTS the slots a BFS lane walks per step and
    GPMA_SORT_LOOKBACK the predecessor tiles a look-back step reads;
    changing any of them rebuilds.
    """
    if verbose:
        os.environ["GPMA_BUILD_VERBOSE"] = "1"
    nvcc = _nvcc()
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    build_dir.mkdir(exist_ok=True)
    sort_items = os.environ.get("GPMA_SORT_ITEMS", "8")
    lane_slots = os.environ.get("GPMA_BFS_LANE_SLOTS", "4")
    lookback = os.environ.get("GPMA_SORT_LOOKBACK", "8")
    defines = [f"-DGPMA_SORT_ITEMS={sort_items}", f"-DGPMA_BFS_LANE_SLOTS={lane_slots}",
               f"-DGPMA_SORT_LOOKBACK={lookback}", f"-DGPMA_BOUNDS_CHECK={int(checked)}"]
    stamp = build_dir / "options.txt"
    options = "".join(d[2:] + "\n" for d in defines)
    if not stamp.exists() or stamp.read_text() != options:
        stamp.write_text(options)
    nvcc_flags = [*NVCC_FLAGS, *defines]
    headers = [*HEADERS, stamp]
    jobs = []
    objs = []
    for name in CU_SOURCES:
        src, obj = CSRC / name, build_dir / (name + ".o")
        objs.append(obj)
        if _stale(obj, src, headers) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc, *ARCH, *nvcc_flags, *extra, "-c", str(src), "-o", str(obj)])
    cc = os.environ.get("CC", "gcc")
    for name in C_SOURCES:
        src, obj = CSRC / name, build_dir / (name + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append([cc, *CC_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if jobs or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        tmp = lib.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lgomp"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv, checked="--checked" in sys.argv))
