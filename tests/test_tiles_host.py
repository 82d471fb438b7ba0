"""CPU: the reference's merged 4 x 4-block tiles (SparseMatrix::bcsrBlocking,
src/cuda_hgemm/src/common/matrix.h:794-1137).

* the oracle's restatement against the golden fixtures made by the reference
  itself (tests/golden/golden_tiles.npz) and, where the reference sources are
  present, against the reference run live on random BCSRs;
* the GPU build's per-element steps (csrc/tiles_core.h), replayed on the CPU
  by tests/tiles_replay.cpp, against the same fixtures and the oracle on
  larger and skewed matrices, and its rejection of malformed BCSRs.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden_tiles.npz")
KEYS = ("rowptr", "colidx", "val", "block_info", "rel_map", "tile_info")


def golden_cases():
    d = np.load(GOLDEN)
    for i in range(int(d["tiles_n"])):
        mr, mc, k = (int(x) for x in d[f"tiles{i}_dims"])
        yield (i, mr, mc, k, d[f"tiles{i}_brp"], d[f"tiles{i}_bci"], d[f"tiles{i}_bval"].view(np.float16),
               {key: d[f"tiles{i}_{key}"] for key in KEYS})


def same(a, b):
    for key in KEYS:
        x, y = np.asarray(a[key]), np.asarray(b[key])
        assert x.shape == y.shape, (key, x.shape, y.shape)
        assert np.array_equal(x.reshape(-1), y.reshape(-1)), key


def random_bcsr(O, rng, k, mr, mc, deg, hub=False, zeros=0.0, empty_tile_rows=False):
    rp, cs = [0], []
    for r in range(mr):
        n = int(rng.integers(0, deg))
        if hub and r % 37 == 0:
            n = mc // 2
        if empty_tile_rows and (r // 64) % 3 == 1:
            n = 0
        c = np.unique(rng.integers(0, mc, n))
        rng.shuffle(c)
        cs += c.tolist()
        rp.append(len(cs))
    v = rng.standard_normal(len(cs)).astype(np.float16)
    v[rng.random(len(v)) < zeros] = 0
    brp, bci, bv, _ = O.csr_to_bcsr(mr, mc, k, np.array(rp, np.int32), np.array(cs, np.int32), v)
    return brp, bci, bv


@pytest.fixture(scope="module")
def replay(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("tiles") / "libtiles_replay.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{ROOT}/sptc-smat_gb300/csrc",
                    os.path.join(ROOT, "tests", "tiles_replay.cpp"), "-o", so],
                   check=True, capture_output=True, text=True, timeout=300)
    L = C.CDLL(so)
    L.replay_tiles.restype = C.c_int64
    L.replay_tiles.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_int64)] + [C.c_void_p] * 6

    def run(mr, mc, k, brp, bci, bval):
        brp = np.ascontiguousarray(brp, np.int32)
        bci = np.ascontiguousarray(bci, np.int32)
        vb = np.ascontiguousarray(np.asarray(bval, np.float16).view(np.uint16)).reshape(-1)
        nrp = C.c_int64()
        args = [mr, mc, k, len(bci), brp.ctypes.data, bci.ctypes.data, vb.ctypes.data, C.byref(nrp)]
        nt = L.replay_tiles(*args, *([None] * 6))
        if nt < 0:
            return int(nt)
        cells = ((mr + 63) // 64) * ((mc + 4 * k - 1) // (4 * k))
        out = {"rowptr": np.zeros(nrp.value, np.int32), "colidx": np.zeros(max(nt, 1), np.int32),
               "val": np.zeros(max(nt, 1) * 256 * k, np.uint16), "block_info": np.zeros(max(cells, 1), np.int32),
               "rel_map": np.zeros(max(cells, 1), np.int32), "tile_info": np.zeros(max(nt, 1) * 16, np.int32)}
        L.replay_tiles(*args, *(out[key].ctypes.data for key in KEYS))
        out["colidx"], out["tile_info"] = out["colidx"][:nt], out["tile_info"][: nt * 16]
        out["val"] = out["val"][: nt * 256 * k].reshape(nt, 256 * k)
        out["block_info"], out["rel_map"] = out["block_info"][:cells], out["rel_map"][:cells]
        return out

    return run


def test_oracle_matches_reference_goldens(oracle_lib):
    n = 0
    for i, mr, mc, k, brp, bci, bval, want in golden_cases():
        same(oracle_lib.bcsr_blocking(mr, mc, k, brp, bci, bval), want)
        n += 1
    assert n >= 14


def test_goldens_cover_the_reference_quirks():
    seen_gap = seen_unsorted = seen_24 = seen_empty = False
    for i, mr, mc, k, brp, bci, bval, want in golden_cases():
        nrr = (mr + 63) // 64
        used = want["block_info"].reshape(nrr, -1).any(1).sum()
        seen_gap |= used < nrr and len(want["colidx"]) > 0          # tile rows without an entry
        rp, ci = want["rowptr"], want["colidx"]
        seen_unsorted |= any(np.any(np.diff(ci[rp[j]:rp[j + 1]]) < 0) for j in range(len(rp) - 1))
        seen_24 |= bool(np.any(want["tile_info"] == 1))
        seen_empty |= len(bci) == 0
    assert seen_gap and seen_unsorted and seen_24 and seen_empty


def test_oracle_matches_live_reference(oracle_lib):
    if not oracle_lib.ref_available():
        pytest.skip("reference build not available")
    rng = np.random.default_rng(7)
    for trial in range(12):
        k = 16 if trial % 2 else 32
        mr, mc = 16 * int(rng.integers(1, 40)), k * int(rng.integers(1, 30))
        brp, bci, bv = random_bcsr(oracle_lib, rng, k, mr, mc, int(rng.integers(1, 30)),
                                   zeros=0.3 * (trial % 3 == 0), empty_tile_rows=trial % 4 == 1)
        same(oracle_lib.bcsr_blocking(mr, mc, k, brp, bci, bv), oracle_lib.ref_bcsr_blocking(mr, mc, k, brp, bci, bv))


def test_replay_of_the_gpu_build_matches_goldens(replay):
    for i, mr, mc, k, brp, bci, bval, want in golden_cases():
        got = replay(mr, mc, k, brp, bci, bval)
        assert not isinstance(got, int), (i, got)
        same(got, want)


@pytest.mark.parametrize("k", [16, 32])
def test_replay_matches_oracle_on_skewed_matrices(replay, oracle_lib, k):
    rng = np.random.default_rng(11 + k)
    for hub, zeros, gaps in [(True, 0.0, False), (False, 0.5, True), (True, 0.2, True)]:
        mr, mc = 16 * 97, k * 61
        brp, bci, bv = random_bcsr(oracle_lib, rng, k, mr, mc, 24, hub=hub, zeros=zeros, empty_tile_rows=gaps)
        same(replay(mr, mc, k, brp, bci, bv), oracle_lib.bcsr_blocking(mr, mc, k, brp, bci, bv))


def test_replay_rejects_malformed_bcsr(replay):
    k = 16
    brp = np.array([0, 2, 3], np.int32)
    bci = np.array([16, 0, 32], np.int32)                    # descending in block row 0
    bval = np.zeros(3 * 256, np.float16)
    assert replay(32, 64, k, brp, bci, bval) == -1 - 4
    assert replay(32, 64, k, brp, np.array([0, 8, 32], np.int32), bval) == -1 - 2   # not a multiple of k
    assert replay(32, 64, k, brp, np.array([0, 64, 32], np.int32), bval) == -1 - 2  # past the last column
    assert replay(32, 64, k, np.array([0, 3, 2], np.int32), bci, bval) < 0          # row pointers decrease
