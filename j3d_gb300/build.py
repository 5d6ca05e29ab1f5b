"""Builds libj3dgpu.so in-tree (j3d_gb300/_lib/) for sm_103a.

nvcc compiles the CUDA translation units, g++ the host-only math; both with
FMA contraction off, because the hit-deciding fp32 arithmetic must round
exactly where it is written. Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_lib"
BUILD_DIR = HERE / "_build"
LIB = OUT_DIR / "libj3dgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread"]

CU_SOURCES = ["build.cu", "render_dispatch.cu", "query.cu", "umma_gemm.cu", "learned.cu", "ingest.cu", "pointcloud.cu",
              "api.cu"]
# render.cu once per BVH width (its kernels are templated on it; namespaces w2 / w4 / w8)
RENDER_WIDTHS = (2, 4, 8)
CXX_SOURCES = ["host_math.cpp", "ingest_parse.cpp", "toplevel.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + [HERE.parent / "include" / "j3dg.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        jobs.append([nv, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    for w in RENDER_WIDTHS:
        obj = BUILD_DIR / f"render_w{w}.cu.o"
        objs.append(obj)
        jobs.append([nv, *NVCC_FLAGS, f"-DJ3DG_W={w}", "-c", str(CSRC / "render.cu"), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD_DIR / (src + ".o")
        objs.append(obj)
        jobs.append([os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nv, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-Xcompiler", "-pthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
