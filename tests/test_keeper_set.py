"""CPU: the Keeper scan's pooled red-black set (csrc/keeper_set.h) holds the
same keys in the same order as std::set<std::pair<float, long>> -- the
reference's container -- after every insert and every trim from end()
(tests/keeper_set_check.cpp, compiled here)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_keeper_set_matches_std_set(tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "keeper_set_check")
    cmd = [cxx, "-O2", "-std=c++17", f"-I{ROOT}/sptc-smat_gb300/csrc",
           os.path.join(ROOT, "tests", "keeper_set_check.cpp"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ALL OK"), r.stdout[-3000:] + r.stderr[-2000:]
