"""Build libifgf2d.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked with nvcc.  Output:
ifgf2d_gb300/_build/libifgf2d.so.  Used by __graft_entry__.build() and by the package on
first import when the library is missing.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libifgf2d.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["geometry.cpp", "tree.cpp", "ifgf2d_kernels.cu", "ifgf_apply.cu", "ifgf_batch.cu", "rp_precompute.cu", "ifgf2d_capi.cu",
           "batch.cu", "batch_tcgen05.cu", "offsurface.cu", "precond_net.cu", "precond_capi.cu", "noalloc.cu", "gmres_device.cu", "plan_device.cu", "geometry_device.cu", "group.cu", "spectral_precond.cu"]
# translation units whose arithmetic must round like the host restatement (no FMA contraction)
NO_FMAD = {"rp_precompute.cu", "plan_device.cu", "geometry_device.cu"}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libifgf2d.so")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread",
           "-c", os.path.join(CSRC, src), "-o", obj]
    if src in NO_FMAD:
        cmd[1:1] = ["-fmad=false"]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".inc"))]
    deps.append(os.path.join(HERE, "..", "include", "ifgf2d.h"))
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-pthread", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
