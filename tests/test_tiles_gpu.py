"""GPU: the tile-shape axes the autotuner searches, each checked against the
FP64 oracle -- 256-column N tiles (one pass over A for N <= 256; plan class
3, kernel variants with two 128-column subtiles), the pipeline depth (stage
slots in flight) -- and the autotuner over panel height x split threshold x
N-tile width x depth: the shape it picks is no slower (within timing noise)
than any candidate the test measures itself, and handles created with
panel_rows = 0 take it. Tolerances as in the other GPU tests: FP16 1e-3,
BF16 1e-2 relative Frobenius vs FP64."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rel_err(got, ref):
    got = np.asarray(got, np.float64)
    n = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / (n if n > 0 else 1.0))


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def fp64_product(O, A, B):
    return O.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), np.asarray(B, np.float64))


def run(M, B, form, out=None):
    C = M.spmm(B, form=form, out=out)
    torch.cuda.synchronize()
    M.check_device_error()
    return C.float().cpu().numpy()


@pytest.mark.parametrize("R", [4, 8])
@pytest.mark.parametrize("N", [129, 200, 256, 384, 512])
def test_wide_tiles_vs_fp64(dev, smat_mod, oracle_lib, R, N):
    from smat import generators as G
    A = G.rmat(12, 50000, seed=N)
    Bh = np.random.default_rng(R * N).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    ref = fp64_product(oracle_lib, A, Bh)
    B = torch.from_numpy(Bh).to(dev)
    W = smat_mod.Bcsr(A, panel_rows=R, n_tile_cols=256)
    assert W.info["n_tile_cols"] == 256
    cw = run(W, B, smat_mod.FORM_F16)
    assert rel_err(cw, ref) <= 1e-3
    Nn = smat_mod.Bcsr(A, panel_rows=R)
    assert Nn.info["n_tile_cols"] == 128
    cn = run(Nn, B, smat_mod.FORM_F16)
    assert rel_err(cw, cn.astype(np.float64)) <= 1e-5     # same sums, other grouping of the passes
    W.close()
    Nn.close()


def test_wide_tiles_bf16_stencil_and_col_major(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.stencil27(16)
    Bf = np.random.default_rng(3).standard_normal((A.cols, 256)).astype(np.float32)
    ref = fp64_product(oracle_lib, A, Bf)
    W = smat_mod.Bcsr(A, panel_rows=8, n_tile_cols=256, forms=(smat_mod.FORM_F16, smat_mod.FORM_BF16))
    B = torch.from_numpy(Bf).to(dev)
    assert rel_err(run(W, B, smat_mod.FORM_BF16), ref) <= 1e-2
    Bc = B.t().contiguous().t()
    assert rel_err(run(W, Bc, smat_mod.FORM_F16), ref) <= 1e-3
    W.close()


def test_wide_tiles_with_24_path_and_group(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.force_24(G.rmat(12, 60000, seed=9), 0.3, seed=8)
    N = 256
    Bh = np.random.default_rng(7).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    ref = fp64_product(oracle_lib, A, Bh)
    B = torch.from_numpy(Bh).to(dev)
    W = smat_mod.Bcsr(A, panel_rows=8, n_tile_cols=256, use_24=1)
    assert W.info["n_blocks_24"] > 0
    assert rel_err(run(W, B, smat_mod.FORM_F16), ref) <= 1e-3
    W.close()
    W = smat_mod.Bcsr(A, panel_rows=8, n_tile_cols=256)
    Cg = torch.zeros((A.rows, N), dtype=torch.float32, device=dev)
    g = smat_mod.Group([(W, smat_mod.FORM_F16, B, Cg)])
    g.run(0)
    torch.cuda.synchronize()
    assert rel_err(Cg.cpu().numpy(), ref) <= 1e-3
    W.close()


@pytest.mark.parametrize("depth", [2, 3])
def test_pipeline_depth(dev, smat_mod, oracle_lib, depth):
    from smat import generators as G
    A = G.rmat(13, 120000, seed=5)
    Bh = np.random.default_rng(depth).uniform(-1, 1, (A.cols, 128)).astype(np.float16)
    ref = fp64_product(oracle_lib, A, Bh)
    M = smat_mod.Bcsr(A, pipeline_depth=depth)
    assert M.info["pipeline_depth"] == depth
    assert rel_err(run(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16), ref) <= 1e-3
    M.close()


def time_ms(M, B, reps=10):
    C = M.spmm(B)
    for _ in range(3):
        M.spmm(B, out=C)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        M.spmm(B, out=C)
    e1.record()
    torch.cuda.synchronize()
    M.check_device_error()
    return e0.elapsed_time(e1) / reps


def test_autotune_three_axes(dev, smat_mod):
    from smat import generators as G
    smat_mod.lib().smat_autotune_clear()
    A = G.stencil27(32)                                   # 32768 rows, N = 256: both tile widths offered
    N = 256
    r = smat_mod.autotune(A, form=smat_mod.FORM_F16, N=N)
    assert not r["cached"] and r["candidates"] >= 13, r
    assert r["n_tile_cols"] in (128, 256) and r["pipeline_depth"] in (0, 2)
    assert r["ms"] <= r["ms_default"] * 1.0001
    M = smat_mod.Bcsr(A)                                  # panel_rows = 0: the tuned shape
    assert (M.info["panel_rows"], M.info["n_tile_cols"], M.info["pipeline_depth"]) == \
        (r["panel_rows"], r["n_tile_cols"], r["pipeline_depth"])
    B = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, (A.cols, N)).astype(np.float32)).to(dev)
    t_tuned = time_ms(M, B)
    M.close()
    # candidates across the three axes, measured here
    times = {}
    for R in (4, 8, 16):
        for ntc in (128, 256):
            if ntc == 256 and R > 8:
                continue
            for depth in (0, 2):
                C = smat_mod.Bcsr(A, panel_rows=R, n_tile_cols=ntc, pipeline_depth=depth,
                                  split_frac=r["split_frac"])
                times[(R, ntc, depth)] = time_ms(C, B)
                C.close()
    best = min(times.values())
    print("tuned", (r["panel_rows"], r["n_tile_cols"], r["pipeline_depth"]), f"{t_tuned:.4f} ms;",
          {k: round(v, 4) for k, v in sorted(times.items())})
    assert t_tuned <= best * 1.10, (t_tuned, best)
    smat_mod.lib().smat_autotune_clear()
