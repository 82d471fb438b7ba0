"""GPU parity of the tensor-core SpMM (through the C ABI) against the FP64
CPU oracle, against the reference's own BCSR kernel on identical inputs, and
size-independent properties at full size.

Tolerances (relative Frobenius error vs FP64): plain FP16 form 1e-3 (the
spec bound; FP16 inputs are exact in FP64, so the observed error is
FP32 accumulation only, ~1e-6), BF16 form 1e-2 (BF16 rounding of FP32 data),
split-BF16 form 1e-4 (spec bound 1e-3).
"""
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


def spmm(M, B, form, out_dtype=torch.float32):
    C = M.spmm(B, form=form, out_dtype=out_dtype)
    torch.cuda.synchronize()
    M.check_device_error()
    return C.float().cpu().numpy()


def test_band_config1_fp16_vs_fp64(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.band(4096, 64, seed=1)
    Bh = np.random.default_rng(2).uniform(-1, 1, (4096, 64)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    assert M.info["nnzb"] == 2284
    B = torch.from_numpy(Bh).to(dev).t().contiguous().t()
    err = rel_err(spmm(M, B, smat_mod.FORM_F16), fp64_product(oracle_lib, A, Bh))
    assert err <= 1e-3, err


@pytest.mark.parametrize("N", [8, 64, 100, 128, 200, 256, 384])
@pytest.mark.parametrize("layout", ["col", "row"])
def test_random_shapes_and_widths(dev, smat_mod, oracle_lib, N, layout):
    from smat import generators as G
    A0 = G.random_block(1000, 0.06, 0.05, 0.9, seed=N)     # 1000 rows: not a multiple of 16
    keep = A0.col_idx < 997                                 # ragged K: drop columns >= 997
    r = np.repeat(np.arange(A0.rows), np.diff(A0.row_ptr))[keep]
    rp = np.zeros(A0.rows + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    A = smat_mod.Csr(A0.rows, 997, np.cumsum(rp), A0.col_idx[keep], A0.values[keep])
    Bh = np.random.default_rng(N).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    B = torch.from_numpy(Bh).to(dev)
    if layout == "col":
        B = B.t().contiguous().t()
    err = rel_err(spmm(M, B, smat_mod.FORM_F16), fp64_product(oracle_lib, A, Bh))
    assert err <= 1e-3, err


@pytest.mark.parametrize("form,tol", [("bf16", 1e-2), ("split", 1e-4), ("f16_from_f32", 1e-3)])
def test_forms_with_fp32_b(dev, smat_mod, oracle_lib, form, tol):
    from smat import generators as G
    A = G.stencil27(12)                                     # FP32 values, diagonal-dominant
    rng = np.random.default_rng(4)
    Bf = rng.standard_normal((A.cols, 96)).astype(np.float32)
    f = {"bf16": smat_mod.FORM_BF16, "split": smat_mod.FORM_SPLIT_BF16, "f16_from_f32": smat_mod.FORM_F16}[form]
    M = smat_mod.Bcsr(A, forms=(f,))
    ref = fp64_product(oracle_lib, A, Bf)
    err = rel_err(spmm(M, torch.from_numpy(Bf).to(dev), f), ref)
    if form == "f16_from_f32":
        # FP16 rounding of A and B bounds this form; check it against the
        # FP16-rounded inputs in FP64 instead
        A16 = smat_mod.Csr(A.rows, A.cols, A.row_ptr, A.col_idx, A.values.astype(np.float16))
        ref = fp64_product(oracle_lib, A16, Bf.astype(np.float16))
        err = rel_err(spmm(M, torch.from_numpy(Bf).to(dev), f), ref)
    assert err <= tol, err


def test_split_beats_bf16_and_fp16(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.stencil27(10)
    Bf = np.random.default_rng(5).standard_normal((A.cols, 128)).astype(np.float32)
    M = smat_mod.Bcsr(A, forms=(smat_mod.FORM_F16, smat_mod.FORM_BF16, smat_mod.FORM_SPLIT_BF16))
    ref = fp64_product(oracle_lib, A, Bf)
    B = torch.from_numpy(Bf).to(dev)
    e = {f: rel_err(spmm(M, B, f), ref) for f in (smat_mod.FORM_F16, smat_mod.FORM_BF16, smat_mod.FORM_SPLIT_BF16)}
    assert e[smat_mod.FORM_SPLIT_BF16] < 1e-4 < e[smat_mod.FORM_F16] < e[smat_mod.FORM_BF16]


@pytest.mark.parametrize("R,block", [(4, (16, 16)), (8, (16, 16)), (16, (16, 16)), (4, (32, 16)), (8, (32, 16))])
def test_panel_heights_and_block_shapes(dev, smat_mod, oracle_lib, R, block):
    from smat import generators as G
    A = G.rmat(12, 40000, seed=R)
    Bh = np.random.default_rng(1).uniform(-1, 1, (A.cols, 160)).astype(np.float16)
    M = smat_mod.Bcsr(A, block=block, panel_rows=R)
    err = rel_err(spmm(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16), fp64_product(oracle_lib, A, Bh))
    assert err <= 1e-3, err


def test_fp16_output(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.band(2048, 20, seed=3)
    Bh = np.random.default_rng(3).uniform(-1, 1, (2048, 128)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    C = spmm(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16, out_dtype=torch.float16)
    assert rel_err(C, fp64_product(oracle_lib, A, Bh)) <= 1e-3


def test_reorder_pipeline_returns_original_row_order(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.rmat(11, 15000, seed=8)
    r = smat_mod.reorder(A, 0.6, 16, 16)
    M = smat_mod.Bcsr(A, row_perm=r.perm)
    Bh = np.random.default_rng(8).uniform(-1, 1, (A.cols, 64)).astype(np.float16)
    C = spmm(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16)
    assert rel_err(C, fp64_product(oracle_lib, A, Bh)) <= 1e-3
    # the BCSR it built is the reference's blocking of the permuted matrix
    rp, ci, v, _ = M.export()
    rp2, ci2, v2 = smat_mod.csr_to_bcsr_host(A, (16, 16), r.perm)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2) and np.array_equal(v.view(np.uint16), v2.view(np.uint16))


def test_empty_rows_and_empty_matrix(dev, smat_mod):
    rp = np.zeros(101, np.int64)
    rp[50:] = 3
    A = smat_mod.Csr(100, 40, rp, np.array([1, 17, 39]), np.array([1.0, 2.0, 3.0], np.float32))
    M = smat_mod.Bcsr(A)
    B = torch.ones((40, 16), device=dev)
    C = spmm(M, B, smat_mod.FORM_F16)
    expect = np.zeros((100, 16))
    expect[49] = 6.0
    assert np.array_equal(C, expect)
    Z = smat_mod.Csr(64, 64, np.zeros(65, np.int64), np.zeros(0, np.int32), np.zeros(0, np.float32))
    MZ = smat_mod.Bcsr(Z)
    Cz = MZ.spmm(torch.ones((64, 32), device=dev))
    torch.cuda.synchronize()
    assert float(Cz.abs().max()) == 0.0


def test_deterministic_and_host_variant(dev, smat_mod):
    from smat import generators as G
    A = G.rmat(12, 30000, seed=2)
    Bh = np.random.default_rng(2).uniform(-1, 1, (A.cols, 128)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    B = torch.from_numpy(Bh).to(dev)
    c1 = spmm(M, B, smat_mod.FORM_F16)
    c2 = spmm(M, B, smat_mod.FORM_F16)
    assert np.array_equal(c1, c2)
    c3 = M.spmm_host(Bh, smat_mod.FORM_F16)
    assert np.array_equal(c1, c3)


def test_errors_are_statuses(dev, smat_mod):
    from smat import generators as G
    A = G.band(256, 4, seed=1)
    M = smat_mod.Bcsr(A)  # FP16 form only
    B = torch.ones((256, 16), device=dev, dtype=torch.float16)
    with pytest.raises(smat_mod.SmatError) as e:
        M.spmm(B, form=smat_mod.FORM_BF16)
    assert e.value.status == 1
    C = torch.empty((256, 16), device=dev)
    with pytest.raises(smat_mod.SmatError) as e:
        M.spmm_raw(smat_mod.FORM_F16, B, smat_mod.F16, smat_mod.ROW_MAJOR, 16, C, smat_mod.F32, 16, 16, None, 0, 0)
    assert e.value.status == 1


def test_linearity_at_rmat_scale(dev, smat_mod):
    """Full-size property: A(B1 + B2) = A B1 + A B2 for the 65536-row R-MAT
    workload shape (exact up to FP32 accumulation)."""
    from smat import generators as G
    A = G.rmat(16, 2_000_000, seed=3)
    M = smat_mod.Bcsr(A)
    g = torch.Generator(device=dev).manual_seed(1)
    B1 = (torch.rand((A.cols, 128), device=dev, generator=g) - 0.5).half()
    B2 = (torch.rand((A.cols, 128), device=dev, generator=g) - 0.5).half()
    s = (B1.float() + B2.float())
    C1 = M.spmm(B1.float())
    C2 = M.spmm(B2.float())
    C12 = M.spmm(s)
    torch.cuda.synchronize()
    lhs, rhs = C12.double(), (C1.double() + C2.double())
    assert float((lhs - rhs).norm() / rhs.norm()) < 1e-3


def test_reference_kernel_agrees(dev, smat_mod, oracle_lib):
    """Same inputs through the reference's own mmaOBTKernelSparse (FP16
    accumulate, FP16 C) and through ours (FP32 accumulate): both checked
    against FP64, and against each other at 1e-3."""
    import ref_kernel
    if not ref_kernel.available():
        pytest.skip("reference cubin not built")
    from smat import generators as G
    A = G.band(4096, 64, seed=1)
    N = 64
    Bh = np.random.default_rng(2).uniform(-1, 1, (4096, N)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    rp, ci, v, _ = M.export()
    Bcol = torch.from_numpy(Bh).to(dev).t().contiguous()          # (N, K) rows = columns of B
    Cref, keep = ref_kernel.run(torch.from_numpy(v).to(dev), torch.from_numpy(rp).to(dev),
                                torch.from_numpy(ci).to(dev), 4096, 4096, Bcol, N)
    torch.cuda.synchronize()
    ours = spmm(M, Bcol.t(), smat_mod.FORM_F16)
    ref64 = fp64_product(oracle_lib, A, Bh)
    e_ref = rel_err(Cref.float().cpu().numpy(), ref64)
    e_ours = rel_err(ours, ref64)
    e_pair = rel_err(ours, Cref.float().cpu().numpy().astype(np.float64))
    assert e_ours <= 1e-3 and e_ours <= e_ref
    assert e_pair <= 1e-3, (e_pair, e_ref, e_ours)


def e4m3_table():
    """Value of every e4m3 ("e4m3fn": bias 7, no infinities, 0x7f/0xff NaN) code."""
    t = np.zeros(256, np.float64)
    for c in range(256):
        s = -1.0 if c & 0x80 else 1.0
        e, m = (c >> 3) & 0xF, c & 7
        if e == 0xF and m == 7:
            t[c] = np.nan
        elif e == 0:
            t[c] = s * m * 2.0 ** -9
        else:
            t[c] = s * (1 + m / 8) * 2.0 ** (e - 7)
    return t


def test_fp8_form_exact_and_within_budget(dev, smat_mod, oracle_lib):
    """FP8 form: e4m3 A with one FP32 scale per 16x16 block. The kernel must
    reproduce the FP64 product of its own dequantised A (FP32 accumulation,
    1e-5), and that A must stay within the 2e-2 budget of the FP64 product of
    the FP32 matrix (27-point stencil, FP32 B)."""
    import ctypes as C
    from smat import generators as G
    A = G.stencil27(16)
    Bf = np.random.default_rng(12).standard_normal((A.cols, 96)).astype(np.float32)
    M = smat_mod.Bcsr(A, forms=(smat_mod.FORM_FP8, smat_mod.FORM_F16))
    got = spmm(M, torch.from_numpy(Bf).to(dev), smat_mod.FORM_FP8)
    nnzb = M.info["nnzb"]
    codes = np.zeros(nnzb * 256, np.uint8)
    scales = np.zeros(nnzb, np.float32)
    assert smat_mod.lib().smat_bcsr_export_fp8(M.handle, codes.ctypes.data, scales.ctypes.data) == 0
    rp, ci, _, _ = M.export()
    deq = (e4m3_table()[codes].reshape(nnzb, 16, 16) * scales[:, None, None].astype(np.float64))
    deq = deq.astype(np.float32).astype(np.float16).astype(np.float64)     # the FP16 operand the MMA reads
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    Cq = np.zeros((M.info["rows_padded"], 96))
    for b in range(nnzb):
        r0, c0 = rows[b] * 16, ci[b]
        Cq[r0:r0 + 16] += deq[b] @ Bf[c0:c0 + 16].astype(np.float16).astype(np.float64)   # B is packed to FP16
    assert rel_err(got, Cq[: A.rows]) <= 1e-5
    e8 = rel_err(got, fp64_product(oracle_lib, A, Bf))
    assert e8 <= 2e-2, e8
    # plain max-abs scaling (block max -> 448) for comparison: the chosen scales do better
    vals = np.zeros((nnzb, 16, 16))
    Asp = A.to_scipy().tocoo()
    bi = {(int(r), int(c)): k for k, (r, c) in enumerate(zip(rows, ci))}
    for r, c, v in zip(Asp.row, Asp.col, Asp.data):
        vals[bi[(r // 16, c // 16 * 16)], r % 16, c % 16] = v
    amax = np.abs(vals).reshape(nnzb, -1).max(1)
    tab = e4m3_table()
    grid = np.sort(np.unique(np.abs(tab[~np.isnan(tab)])))
    def q(x):
        a = np.abs(x)
        idx = np.clip(np.searchsorted(grid, a), 1, len(grid) - 1)
        lo, hi = grid[idx - 1], grid[idx]
        return np.sign(x) * np.where(a - lo <= hi - a, lo, hi)
    plain = q(vals / (amax / 448)[:, None, None]) * (amax / 448)[:, None, None]
    assert np.sum((deq - vals) ** 2) < np.sum((plain - vals) ** 2)


def test_fp8_form_rejects_out_of_range_values(dev, smat_mod):
    A = smat_mod.Csr(16, 16, np.array([0] * 16 + [1]), np.array([3]), np.array([1e6], np.float32))
    with pytest.raises(smat_mod.SmatError):
        smat_mod.Bcsr(A, forms=(smat_mod.FORM_FP8,))


@pytest.mark.parametrize("layout", ["col", "row"])
def test_host_entry_with_pinned_buffers(dev, smat_mod, oracle_lib, layout):
    """smat_spmm_host on page-locked B and C: the kernels read B and write C in
    place (no staging copies); same result as the device entry point."""
    from smat import generators as G
    A = G.rmat(12, 50000, seed=9)
    N = 96
    Bh = np.random.default_rng(9).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    M = smat_mod.Bcsr(A)
    Bp = torch.empty((N, A.cols) if layout == "col" else (A.cols, N), dtype=torch.float16).pin_memory()
    Bp.copy_(torch.from_numpy(np.ascontiguousarray(Bh.T if layout == "col" else Bh)))
    bview = Bp.numpy().T if layout == "col" else Bp.numpy()
    Cp = torch.full((A.rows, N), float("nan"), dtype=torch.float32).pin_memory()
    M.spmm_host(bview, smat_mod.FORM_F16, out=Cp.numpy())
    M.check_device_error()
    ref = spmm(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16)
    assert np.array_equal(Cp.numpy(), ref)
    assert rel_err(Cp.numpy(), fp64_product(oracle_lib, A, Bh)) <= 1e-3


def test_column_permutation_keeps_the_product(dev, smat_mod, oracle_lib):
    """Blocking with a column permutation (the reference's column reordering):
    the blocks are those of A with its columns permuted, and C = A * B is
    unchanged because B's rows are gathered through the same permutation."""
    from smat import generators as G
    A = G.rmat(11, 30000, seed=21)
    q = smat_mod.reorder_columns(A, tau=0.6)
    assert np.array_equal(np.sort(q), np.arange(A.cols))
    N = 80
    Bh = np.random.default_rng(21).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    M = smat_mod.Bcsr(A, col_perm=q)
    M0 = smat_mod.Bcsr(A)
    for layout in ("row", "col"):
        B = torch.from_numpy(Bh).to(dev)
        if layout == "col":
            B = B.t().contiguous().t()
        got = spmm(M, B, smat_mod.FORM_F16)
        assert rel_err(got, spmm(M0, B, smat_mod.FORM_F16)) <= 1e-6
        assert rel_err(got, fp64_product(oracle_lib, A, Bh)) <= 1e-3
    # the blocks are those of the column-permuted matrix
    inv = np.empty_like(q)
    inv[q] = np.arange(q.size)
    Aq = smat_mod.Csr(A.rows, A.cols, A.row_ptr, inv[A.col_idx], A.values)
    rp, ci, v = smat_mod.csr_to_bcsr_host(Aq)
    erp, eci, ev, _ = M.export()
    assert np.array_equal(rp, erp) and np.array_equal(ci, eci) and np.array_equal(v.view(np.uint16), ev.view(np.uint16))


def hub_matrix(rows, cols, seed):
    """Mostly sparse rows with a few dense hub rows (every 97th and 211th row):
    the planner cuts each hub block row over the four MMA-issuing warps and the
    epilogue adds the parts."""
    from smat import Csr
    rng = np.random.default_rng(seed)
    rp, ci = [0], []
    for r in range(rows):
        d = 0.6 if (r % 97 == 5 or r % 211 == 17) else 0.004
        c = np.flatnonzero(rng.random(cols) < d).astype(np.int32)
        ci.append(c)
        rp.append(rp[-1] + len(c))
    ci = np.concatenate(ci)
    vals = rng.uniform(-1, 1, len(ci)).astype(np.float16).astype(np.float32)
    return Csr(rows, cols, np.array(rp, np.int64), ci, vals)


@pytest.mark.parametrize("R,split_frac,N", [(16, 0.0, 128), (8, 0.0, 128), (16, 0.05, 128), (16, 0.0, 256),
                                            (16, 0.05, 256)])
def test_hub_rows_cut_over_warps(dev, smat_mod, oracle_lib, R, split_frac, N):
    A = hub_matrix(3000, 5000, seed=R + N)
    Bh = np.random.default_rng(5).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    ref = fp64_product(oracle_lib, A, Bh)
    forms = (smat_mod.FORM_F16, smat_mod.FORM_BF16, smat_mod.FORM_SPLIT_BF16)
    M = smat_mod.Bcsr(A, panel_rows=R, split_frac=split_frac, forms=forms)
    B = torch.from_numpy(Bh).to(dev)
    c1 = spmm(M, B, smat_mod.FORM_F16)
    assert rel_err(c1, ref) <= 1e-3
    assert np.array_equal(c1, spmm(M, B, smat_mod.FORM_F16))   # parts are added in a fixed order
    assert rel_err(spmm(M, B, smat_mod.FORM_BF16), ref) <= 1e-2
    assert rel_err(spmm(M, B.float(), smat_mod.FORM_SPLIT_BF16), ref) <= 1e-4
    assert rel_err(spmm(M, B, smat_mod.FORM_F16, out_dtype=torch.float16), ref) <= 1e-3
