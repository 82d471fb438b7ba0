"""GPU: the Keeper row reordering with its candidate distances measured on
the device (smat_reorder use_gpu = 1; the seed loop and its commits stay on
the host) gives the reference's result bit for bit: the golden groupings,
permutations and counters of the reference build, the host scan's result on
random patterns (unsorted rows, empty rows, hub rows), and at full size the
R-MAT 2^16 workload's permutation (sha1 prefix 7f14c3e9e4c90b29, the
reference BlockingEngine's)."""
import hashlib
import os
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def test_device_scan_matches_reference_golden(dev, smat_mod):
    g = np.load(os.path.join(GOLD, "golden_preprocess.npz"))
    for i in range(int(g["keep_n"])):
        tau, bb, BB, nc = g[f"keep{i}_params"]
        rp = g[f"keep{i}_rowptr"]
        A = smat_mod.Csr(len(rp) - 1, int(nc), rp, g[f"keep{i}_cols"])
        r = smat_mod.reorder(A, float(tau), int(bb), int(BB), algo=5, force_fixed=True, use_gpu=True)
        name = str(g[f"keep{i}_name"])
        assert np.array_equal(r.grouping, g[f"keep{i}_grouping"]), name
        assert np.array_equal(r.perm, g[f"keep{i}_perm"]), name
        assert (r.comparisons, r.merges) == tuple(g[f"keep{i}_stats"][:2]), name


def random_pattern(rows, cols, seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 40, rows)
    lens[rng.integers(0, rows, 5)] = rng.integers(200, 600, 5)     # hub rows
    lens[rng.integers(0, rows, 20)] = 0                             # empty rows
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    cols_ = np.concatenate([rng.choice(cols, size=n, replace=False) for n in lens]).astype(np.int32)
    return rp, cols_


@pytest.mark.parametrize("seed,sort_rows", [(1, True), (2, False), (3, True)])
@pytest.mark.parametrize("tau,bs", [(0.3, 4), (0.6, 16), (0.9, 8)])
def test_device_scan_matches_host_scan(dev, smat_mod, seed, sort_rows, tau, bs):
    rp, cols = random_pattern(3000, 2500, seed)
    if sort_rows:
        for r in range(len(rp) - 1):
            cols[rp[r]:rp[r + 1]].sort()
    A = smat_mod.Csr(len(rp) - 1, 2500, rp, cols)
    h = smat_mod.reorder(A, tau, bs, 16, algo=5, force_fixed=True)
    d = smat_mod.reorder(A, tau, bs, 16, algo=5, force_fixed=True, use_gpu=True)
    assert np.array_equal(h.grouping, d.grouping)
    assert np.array_equal(h.perm, d.perm)
    assert (h.comparisons, h.merges) == (d.comparisons, d.merges)


def test_device_scan_full_size_rmat(dev, smat_mod):
    from smat import generators as G
    A0 = G.rmat(16, 2_000_000, seed=3)
    t = time.perf_counter()
    r = smat_mod.reorder(A0, tau=0.6, col_block=16, row_block=16, algo=5, force_fixed=True, use_gpu=True)
    dt = time.perf_counter() - t
    sha = hashlib.sha1(np.ascontiguousarray(r.perm, np.int64).tobytes()).hexdigest()[:16]
    print(f"R-MAT 2^16 reorder with device distances: {dt:.1f} s, {r.comparisons} comparisons, "
          f"{r.merges} merges, perm {sha}")
    assert sha == "7f14c3e9e4c90b29"
    assert (r.comparisons, r.merges) == (114193321, 18752)
