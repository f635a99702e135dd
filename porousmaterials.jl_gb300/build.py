"""Build recipe for libpmgb.so (the sm_103a CUDA library behind include/pmgb.h).

Compiles each translation unit of csrc/ with nvcc for sm_103a in parallel and links the
shared library in-tree at pmgb/libpmgb.so.  Run directly (`python build.py`) or through
`__graft_entry__.build()`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUT_DIR = HERE / "pmgb"
LIB = OUT_DIR / "libpmgb.so"
OBJ_DIR = HERE / "_build"

SOURCES = ["pmgb_kernels.cu", "pmgb_img.cu", "pmgb_batch.cu", "pmgb_refine.cu", "pmgb_api.cu", "pmgb_setup.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so x86 and Arm builds give the same host results
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-ftz=true", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", f"-I{INCLUDE}",
         f"-I{CSRC}"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libpmgb")
    return cand


def _compile(nvcc: str, src: str, verbose: bool) -> Path:
    obj = OBJ_DIR / (Path(src).stem + ".o")
    cmd = [nvcc, *ARCH, *FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ_DIR.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
