"""Builds the in-tree CUDA library ``pd_gb300/_lib/libpd_gb300.so`` for sm_103a with nvcc.

Translation units compile in parallel, then link into one shared library. Host code is
compiled with ``-ffp-contract=off`` so that x86-64 and aarch64 hosts round identically.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libpd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "-I" + os.path.join(HERE, "..", "include")]
# Per-unit extra flags: the reference-order kernel must never contract a*b+c into an FMA.
UNITS = {
    "host.cpp": ["-x", "cu"],
    "abi.cu": [],
    "substep_exact.cu": ["-fmad=false"],
    "substep_fast.cu": [],
    "substep_mixed.cu": [],
    "substep_mixed_grid.cu": [],
    "substep_delta.cu": [],
    "substep_delta64.cu": [],
    "substep_corr.cu": [],
    "adjoint.cu": [],
    "solve_noalloc.cu": ["-fmad=false"],
    "state_copy.cu": [],
    "spectrum.cu": ["-fmad=false"],
    "refactor.cu": ["-fmad=false"],
}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()

    def compile_unit(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(obj_dir, unit + ".o")
        cmd = [nvcc] + ARCH + COMMON + UNITS[unit] + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, list(UNITS)))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
