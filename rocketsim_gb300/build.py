"""Builds the in-tree shared library ``rocketsim_gb300/_lib/librsg_gb300.so``.

nvcc compiles the translation units in parallel for sm_103a only and
links them into one library exporting the C ABI of include/rocketsim_gb300.h.
Floating-point contraction is off on both sides (``-fmad=false`` for device
code, ``-ffp-contract=off`` for host code) so that every multiply and add
rounds as written, like the reference's SSE build.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "librsg_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

SOURCES = ["rsg_kernels.cu", "rsg_ballpred.cu", "rsg_air.cu", "rsg_air_noalloc.cu", "rsg_ground.cu", "rsg_ground_sweep.cu", "rsg_capi.cpp",
           "rsg_mesh.cpp"]
# The ground adjoint's reverse sweep only linearises around recomputed intermediates: division and
# square root correct to about 2 ulp are enough there (see rsg_ground_sweep.cu).
EXTRA = {"rsg_ground_sweep.cu": ["-prec-div=false", "-prec-sqrt=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rocketsim_gb300")
    return cand


def _digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            p = os.path.join(d, name)
            if os.path.isfile(p) and name.endswith((".cu", ".cuh", ".cpp", ".h", ".hpp")):
                with open(p, "rb") as f:
                    h.update(name.encode())
                    h.update(f.read())
    h.update(" ".join(ARCH + COMMON).encode())
    h.update(repr(sorted(EXTRA.items())).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if the sources changed) and return the library path."""
    os.makedirs(LIB_DIR, exist_ok=True)
    stamp = LIB_PATH + ".sha256"
    dig = _digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB_PATH
    nvcc = _nvcc()
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)

    def compile_one(src: str) -> str:
        out = os.path.join(obj_dir, src + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *EXTRA.get(src, []), "-c", os.path.join(CSRC, src), "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)
        return out

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", *objs, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
