"""Build the GB300 decoder library (libtv_gb300.so) in place with nvcc.

One translation unit, one -gencode (sm_103a), so it builds in seconds on the
x86 development host and on the aarch64 GPU host alike.
"""
from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "libtv_gb300.so"
SOURCES = [HERE / "csrc" / "tv_host.cu"]
DEPS = SOURCES + sorted((HERE / "csrc").glob("*.cuh")) + [HERE.parent / "include" / "tv_gb300.h"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the GB300 decoder has no CPU fallback and must be compiled")


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in DEPS if p.exists())


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    if not force and up_to_date():
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *NVCC_FLAGS, "-o", str(tmp), *map(str, SOURCES)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True, cwd=str(HERE))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
