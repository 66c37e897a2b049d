"""In-tree build of the native parts: librh.so (CUDA kernels + C ABI, sm_103a)
and the drop-in command-line program cuda_Cell_Detailed.

    python -m ryr_hyperactivity_gb300.build

Translation units compile in parallel; outputs go next to the sources
(csrc/_build/*.o, ./librh.so, ./bin/cuda_Cell_Detailed).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(CSRC, "_build")
LIB = os.path.join(PKG, "librh.so")
BIN = os.path.join(PKG, "bin")
CLI = os.path.join(BIN, "cuda_Cell_Detailed")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-I", os.path.join(ROOT, "include")]
CU_SOURCES = ["step.cu", "window.cu", "rh_api.cu", "mlp.cu"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hs


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.splitext(os.path.basename(src))[0] + ".o")
    if _newer(obj, [src] + _headers() + [os.path.abspath(__file__)]):
        return obj
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs) + 1) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose), srcs))
    if not _newer(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    cli_src = os.path.join(CSRC, "cli_main.cpp")
    if os.path.exists(cli_src) and not _newer(CLI, [cli_src, LIB] + _headers()):
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), cli_src, "-o", CLI,
               "-L", PKG, "-lrh", "-Wl,-rpath,$ORIGIN/..", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
