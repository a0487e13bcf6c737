"""Build the in-tree CUDA library libthorin_gpu.so for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into a
shared library next to this file.  Device code is compiled with FMA
contraction (--fmad=true): the kernels are bound by the FP64 pipe and a fused
multiply-add is one instruction; host code keeps -ffp-contract=off.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libthorin_gpu.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["kernels_hydro.cu", "kernels_aux.cu", "thorin_api.cu", "thorin_noalloc.cu", "thorin_selftest.cu",
           "warmnet.cu", "thorin_ensemble.cu", "thorin_graph.cu"]
# the control kernels of the device-resident DT repeat host arithmetic and
# are compiled, like the host code, without FMA contraction
NO_FMA = {"thorin_graph.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=true", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "thorin_gpu.h"))
    objs, jobs = [], []
    nv = nvcc()
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            flags = [f.replace("--fmad=true", "--fmad=false") for f in FLAGS] if src in NO_FMA else FLAGS
            cmd = [nv, *ARCH, *flags, *(["-Xptxas", "-v"] if ptxas_v else []), "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([nv, *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
