"""CPU: the work plan the library builds, replayed as the tensor-core kernel
consumes it (tests/plan_emulation.cpp, compiled here against csrc/bcsr.cpp):
plan invariants, hub rows dealt over the issuing warps and added back by the
epilogue, split panels summed from their parts, C in the original row order,
all against an FP64 CSR product."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plan_replay_matches_fp64(tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda.h")):
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path / "plan_emulation")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", f"-I{ROOT}/include", f"-I{ROOT}/sptc-smat_gb300/csrc",
           f"-I{cuda_inc}", os.path.join(ROOT, "tests", "plan_emulation.cpp"),
           os.path.join(ROOT, "sptc-smat_gb300", "csrc", "bcsr.cpp"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ALL OK"), r.stdout[-3000:] + r.stderr[-2000:]
