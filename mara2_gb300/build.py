"""Build the CUDA library in-tree: mara2_gb300/_lib/libmara_gpu.so.

Each translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked into one shared library that exports the C ABI of include/mara_gpu.h.

* plain_fp64.cu  --fmad=false: the plain FP64 path must round exactly like
                 the reference's CPU build, so no multiply-add is contracted;
* mixed.cu       contraction on: FP32 arithmetic with explicit intrinsics;
* every host compile uses -ffp-contract=off (the host computes the mesh
  constants that the plain path feeds to its kernels).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libmara_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(HERE, "..", "include")] + ARCH
UNITS = {
    "plain_fp64.cu": ["--fmad=false"],
    "mixed.cu": ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "batch.cu": ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "mara_gpu.cu": ["--fmad=false"],
    "no_alloc.cu": ["--fmad=false"],
    "diagnostics.cu": ["--fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh", ".hpp"))]
    headers.append(os.path.join(HERE, "..", "include", "mara_gpu.h"))
    units = [u for u in UNITS if os.path.exists(os.path.join(SRC, u))]
    objs = []
    jobs = []
    for u in units:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src, __file__] + headers):
            jobs.append([nvcc(), "-c", src, "-o", obj] + COMMON + UNITS[u])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for log in ex.map(run, jobs):
            if verbose and log:
                print(log)
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
