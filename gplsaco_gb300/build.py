"""Builds the engine library gplsaco_gb300/_build/libfaco_gb300.so for sm_103a.

    python -m gplsaco_gb300.build [--force]

Translation units compile in parallel with nvcc (one -gencode, sm_103a), then
link into one shared object with the CUDA runtime linked statically.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libfaco_gb300.so"
ROOT = PKG.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]
SOURCES = ["faco_kernels.cu", "faco_engine.cu", "faco_prepare.cpp", "prior_mlp.cu", "faco_noalloc.cu", "faco_knn.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not LIB.exists():
        return True
    newest = max(p.stat().st_mtime for p in list(CSRC.iterdir()) + [ROOT / "include" / "faco_gb300.h"])
    return LIB.stat().st_mtime < newest


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    tag = f"{os.getpid()}"

    def compile_one(src: str) -> Path:
        obj = OUT / f"{Path(src).stem}.{tag}.o"
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        objects = list(pool.map(compile_one, SOURCES))
    tmp = OUT / f"libfaco_gb300.{tag}.so"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects)], check=True)
    os.replace(tmp, LIB)
    for obj in objects:
        obj.unlink(missing_ok=True)
    return LIB


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True)
    print(path)
