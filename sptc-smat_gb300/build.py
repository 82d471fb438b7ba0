"""Builds libsmat.so in-tree (sptc-smat_gb300/lib/) for sm_103a.

    python sptc-smat_gb300/build.py [--clean]

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a);
host C++ through g++. Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libsmat.so")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
HOSTFLAGS = ["-fPIC", "-fopenmp", "-ffp-contract=off"]

CU_SOURCES = ["api.cu", "spmm_tc.cu", "spmm24.cu", "convert.cu", "spmm_static.cu", "ref_shims.cu", "spmm_24ref.cu", "group.cu", "tune.cu", "features.cu", "mlp.cu", "reorder_gpu.cu", "tiles.cu"]
CPP_SOURCES = ["reorder.cpp", "bcsr.cpp", "sp24.cpp", "io.cpp"]


def _cmd_cu(src, obj):
    return [NVCC, *ARCH, "-lineinfo", *COMMON, "-Xcompiler", ",".join(HOSTFLAGS), "-c",
            os.path.join(CSRC, src), "-o", obj]


def _cmd_cpp(src, obj):
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    return [CXX, *COMMON, f"-I{cuda_inc}", *HOSTFLAGS, "-c", os.path.join(CSRC, src), "-o", obj]


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "smat.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if _stale(obj, [os.path.join(CSRC, src), *headers]):
            jobs.append(_cmd_cu(src, obj) if src.endswith(".cu") else _cmd_cpp(src, obj))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp"])
    return LIB


if __name__ == "__main__":
    if "--clean" in sys.argv and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    print(build(verbose="-v" in sys.argv))
