"""Builds libwfgpu.so (the C-ABI library) in-tree for sm_103a.

Every CUDA translation unit is compiled with -fmad=false (no contracted
multiply-add) and IEEE division/square root, so the arithmetic the reference
performs in float is reproduced operation for operation; host code gets
-ffp-contract=off for the same reason (gcc on Arm would otherwise fuse).
Objects are rebuilt only when a source or header is newer.
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
ROOT = PKG.parent
OUT_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libwfgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-I", str(ROOT / "include")]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "include")]

CUDA_SOURCES = ["wf_sort.cu", "wf_bvh.cu", "wf_render.cu", "wf_api.cpp", "wf_loop.cpp", "wf_stages.cpp",
                "wf_static.cu"]
HOST_SOURCES = ["wf_scenes.cpp", "wf_scene_io.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwfgpu.so")
    return cand


def _newest_header() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, obj: Path, cuda: bool, extra: list[str]) -> None:
    if cuda:
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-x", "cu", "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and "-Xptxas" in " ".join(extra):
        sys.stderr.write(r.stderr)


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    BUILD_DIR.mkdir(exist_ok=True)
    hdr = _newest_header()
    jobs = []
    for name, cuda in [(s, True) for s in CUDA_SOURCES] + [(s, False) for s in HOST_SOURCES]:
        src = CSRC / name
        obj = BUILD_DIR / (name + ".o")
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr)
        jobs.append((src, obj, cuda, stale))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, c, extra if c else []) for s, o, c, st in jobs if st]
        for f in futs:
            f.result()
    objs = [str(o) for _, o, _, _ in jobs]
    if force or not LIB.exists() or LIB.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="--ptxas-v" in sys.argv)
    print(LIB)
