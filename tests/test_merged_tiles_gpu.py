"""GPU: the reference's merged 4 x 4-block tiles (SparseMatrix::bcsrBlocking,
src/cuda_hgemm/src/common/matrix.h:794-1137) built on the device by
smat_tiles_create, and the `_tiled` launchers that consume them.

* the device build bit for bit against the golden fixtures the reference
  made (tests/golden/golden_tiles.npz: empty tile rows, tiles first met out
  of column order, explicit zeros, 2:4 labels, an empty matrix) and against
  the oracle on R-MAT, band and random-block matrices at 16 x 16 and
  16 x 32 blocks; malformed BCSRs are rejected;
* mmaOBTKernel_tiled (16 x 16 blocks) and mmaOBTSKernel_tiled_large
  (16 x 32 blocks), called with the merged arrays the way the reference
  harness calls them (tester.h:230-299, 507-548), against the FP64 product
  (1e-3 relative Frobenius, FP16 output), twice in a row (the second call
  reuses the cached handle).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KEYS = ("rowptr", "colidx", "val", "block_info", "rel_map", "tile_info")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def to_dev(a, dev):
    a = np.ascontiguousarray(a)
    if a.dtype in (np.float16, np.uint16):
        return torch.from_numpy(a.reshape(-1).view(np.int16).copy()).to(dev)
    return torch.from_numpy(a.copy()).to(dev)


def build(smat_mod, dev, mr, mc, k, brp, bci, bval):
    bv = np.asarray(bval, np.float16).reshape(-1)
    if bv.size == 0:
        bv = np.zeros(8, np.float16)
    ci = np.asarray(bci, np.int32)
    t = smat_mod.Tiles(mr, mc, k, to_dev(np.asarray(brp, np.int32), dev), to_dev(ci, dev), to_dev(bv, dev))
    return t


def same(a, b):
    for key in KEYS:
        x, y = np.asarray(a[key]).reshape(-1), np.asarray(b[key]).reshape(-1)
        assert x.shape == y.shape, (key, x.shape, y.shape)
        assert np.array_equal(x, y), key


def test_device_build_matches_reference_goldens(dev, smat_mod):
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_tiles.npz"))
    for i in range(int(d["tiles_n"])):
        mr, mc, k = (int(x) for x in d[f"tiles{i}_dims"])
        bci = d[f"tiles{i}_bci"]
        # the device build's Python wrapper takes the block count from col_idx
        t = smat_mod.Tiles(mr, mc, k, to_dev(d[f"tiles{i}_brp"], dev),
                           to_dev(bci if len(bci) else np.zeros(0, np.int32), dev),
                           to_dev(d[f"tiles{i}_bval"] if len(bci) else np.zeros(8, np.uint16), dev))
        same(t.to_host(), {key: d[f"tiles{i}_{key}"] for key in KEYS})


@pytest.mark.parametrize("k", [16, 32])
@pytest.mark.parametrize("family", ["rmat", "band", "random_block"])
def test_device_build_matches_oracle(dev, smat_mod, oracle_lib, k, family):
    from smat import generators as G
    A = {"rmat": lambda: G.rmat(12, 60_000, seed=5), "band": lambda: G.band(3000, 70, seed=6),
         "random_block": lambda: G.random_block(2500, 0.03, 0.2, 0.9, seed=7)}[family]()
    brp, bci, bv = smat_mod.csr_to_bcsr_host(A, block=(16, k))
    mr, mc = (A.rows + 15) // 16 * 16, (A.cols + k - 1) // k * k
    got = build(smat_mod, dev, mr, mc, k, brp, bci, bv).to_host()
    want = oracle_lib.bcsr_blocking(mr, mc, k, brp, bci, bv)
    same(got, want)
    assert len(want["colidx"]) > 10


def test_device_build_rejects_malformed_bcsr(dev, smat_mod):
    brp = np.array([0, 2, 3], np.int32)
    bv = np.zeros(3 * 256, np.float16)
    for bci in ([16, 0, 32], [0, 8, 32], [0, 64, 32]):       # descending, not a multiple of k, past the end
        with pytest.raises(smat_mod.SmatError) as e:
            build(smat_mod, dev, 32, 64, 16, brp, np.array(bci, np.int32), bv)
        assert e.value.status == 1
    with pytest.raises(smat_mod.SmatError):
        build(smat_mod, dev, 32, 64, 16, np.array([0, 3, 2], np.int32), np.array([0, 16, 32], np.int32), bv)
    # the handle keeps working after the rejections
    t = build(smat_mod, dev, 32, 64, 16, brp, np.array([0, 16, 32], np.int32), bv)
    assert t.n_tiles == 1 and t.n_rowptr == 2


def fp64(A, Bh, M):
    import scipy.sparse as sps
    Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
    r = np.zeros((M, Bh.shape[1]))
    r[: A.rows] = Asp @ Bh[: A.cols].astype(np.float64)
    return r


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name,k", [("mmaOBTKernel_tiled", 16), ("mmaOBTSKernel_tiled_large", 32)])
@pytest.mark.parametrize("family", ["band", "gaps"])
def test_tiled_launchers_match_fp64(dev, smat_mod, name, k, family):
    from smat import _lib
    from smat import generators as G
    if family == "band":
        A = G.force_24(G.band(1000, 40, seed=2), 0.4, 16, 16, seed=3)
    else:
        # tile rows without entries and tiles first met out of column order
        A0 = G.random_block(1200, 0.04, 0.3, 0.9, seed=8)
        rows = np.repeat(np.arange(A0.rows), np.diff(A0.row_ptr))
        m = (rows // 64) % 3 != 1
        rp = np.concatenate([[0], np.cumsum(np.bincount(rows[m], minlength=A0.rows))]).astype(np.int64)
        A = smat_mod.Csr(A0.rows, A0.cols, rp, A0.col_idx[m], A0.values[m])
    brp, bci, bv = smat_mod.csr_to_bcsr_host(A, block=(16, k))
    M, K = (A.rows + 15) // 16 * 16, (A.cols + k - 1) // k * k
    t = build(smat_mod, dev, M, K, k, brp, bci, bv)
    d = t.desc
    N = 48
    Bh = np.zeros((K, N), np.float16)
    Bh[: A.cols] = np.random.default_rng(5).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    Bc = torch.from_numpy(Bh).to(dev).t().contiguous()          # column-major K x N
    Cm = torch.full((M, N), float("nan"), dtype=torch.float16, device=dev)
    f = _lib.ref_shim(name)
    for _ in range(2):                                           # first call builds, second reuses
        Cm.fill_(float("nan"))
        if name == "mmaOBTKernel_tiled":
            f(d.values, d.row_ptr, d.col_idx, Bc.data_ptr(), Cm.data_ptr(), M, N, K, len(bci), d.block_info,
              d.rel_map)
        else:
            f(d.values, d.row_ptr, d.col_idx, None, None, Bc.data_ptr(), Cm.data_ptr(), M, N, K, len(bci),
              d.block_info, d.rel_map, d.tile_info)
        torch.cuda.synchronize()
        assert smat_mod.lib().smat_ref_shims_last_status() == 0, smat_mod.lib().smat_last_error()
        assert rel(Cm.float().cpu().numpy(), fp64(A, Bh, M)) <= 1e-3
    smat_mod.lib().smat_ref_shims_release()
