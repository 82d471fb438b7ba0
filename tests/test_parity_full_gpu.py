"""GPU parity at the stated workload sizes, against the FP64 oracle.

* R-MAT 2^16 exactly as bench.py builds it (smat.workloads.rmat16: 2.0 M
  distinct entries, rows permuted, Keeper reorder at tau 0.6, 30 % of the
  blocks forced to exact 2:4, about 27.5 M nonzeros after that), B 65536 x 128
  FP16: the plain FP16 form within 1e-3 relative Frobenius error of the FP64
  product, and the uploaded BCSR bit-equal to the host blocking of the
  reordered matrix (csrToBcsr, src/cuda_hgemm/src/common/matrix.h:666-792).
* The same R-MAT workload with its exact-2:4 blocks on the structured-sparse
  path (every such block, and only units of at least 8 of them): FP16
  within 1e-3 of FP64.
* 27-point stencil on 64^3 (262,144 rows, 6.86 M nonzeros), B 262144 x 256
  FP32 N(0,1): FP16 <= 1e-3, BF16 <= 1e-2, split hi+lo BF16 <= 1e-4 (the
  stated bound is 1e-3) and FP8 e4m3 with per-block scales <= 2e-2, all
  against one FP64 product.
* The 512 uneven matrices of the grouped workload in one grouped launch,
  each problem against its own FP64 product (FP16 1e-3, BF16 1e-2).

Each test prints the errors it measured, so the margins are in the log.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_rmat16_workload_plain_fp16(dev, smat_mod, oracle_lib):
    from smat import workloads
    A, perm = workloads.rmat16()
    assert A.rows == 65536 and A.nnz > 20_000_000
    M = smat_mod.Bcsr(A, block=(16, 16), forms=(smat_mod.FORM_F16,), row_perm=perm)
    # the uploaded block structure and values are csrToBcsr of the reordered matrix
    rp, ci, v, _ = M.export()
    hrp, hci, hv = smat_mod.csr_to_bcsr_host(A, block=(16, 16), row_perm=perm)
    assert np.array_equal(rp, hrp) and np.array_equal(ci, hci)
    assert np.array_equal(v.view(np.uint16), hv.view(np.uint16))
    N = 128
    Bh = np.random.default_rng(2).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    B = torch.from_numpy(Bh).to(dev).t().contiguous().t()      # column-major, as the reference's B
    Cm = M.spmm(B, form=smat_mod.FORM_F16)
    torch.cuda.synchronize()
    M.check_device_error()
    ref = oracle_lib.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), Bh.astype(np.float64))
    e = rel(Cm.cpu().numpy(), ref)
    print(f"R-MAT 2^16 workload ({A.nnz} nnz, {M.info['nnzb']} blocks): FP16 rel err vs FP64 {e:.3e}")
    assert e <= 1e-3
    M.close()


@pytest.mark.parametrize("unit_min", [1, 8])
def test_rmat16_workload_with_24_path(dev, smat_mod, oracle_lib, unit_min):
    from smat import workloads
    A, perm = workloads.rmat16()
    M = smat_mod.Bcsr(A, block=(16, 16), forms=(smat_mod.FORM_F16,), row_perm=perm, use_24=unit_min)
    n24 = M.info["n_blocks_24"]
    assert n24 > 0
    N = 128
    Bh = np.random.default_rng(2).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    B = torch.from_numpy(Bh).to(dev).t().contiguous().t()
    Cm = M.spmm(B, form=smat_mod.FORM_F16)
    torch.cuda.synchronize()
    M.check_device_error()
    ref = oracle_lib.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), Bh.astype(np.float64))
    err = rel(Cm.cpu().numpy(), ref)
    print(f"R-MAT 2^16 workload, 2:4 path (units of >= {unit_min}): {n24} of {M.info['nnzb']} blocks on mma.sp, "
          f"rel err vs FP64 {err:.3e}")
    assert err <= 1e-3, err
    M.close()


def test_stencil64_all_forms(dev, smat_mod, oracle_lib):
    from smat import workloads
    A = workloads.stencil64()
    assert A.rows == 262144
    forms = {"f16": (smat_mod.FORM_F16, 1e-3), "bf16": (smat_mod.FORM_BF16, 1e-2),
             "split_bf16": (smat_mod.FORM_SPLIT_BF16, 1e-4), "fp8": (smat_mod.FORM_FP8, 2e-2)}
    M = smat_mod.Bcsr(A, forms=tuple(f for f, _ in forms.values()))
    N = 256
    Bf = np.random.default_rng(7).standard_normal((A.cols, N)).astype(np.float32)
    B = torch.from_numpy(Bf).to(dev)
    ref = oracle_lib.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), Bf.astype(np.float64))
    errs = {}
    for name, (f, tol) in forms.items():
        Cm = M.spmm(B, form=f)
        torch.cuda.synchronize()
        M.check_device_error()
        errs[name] = rel(Cm.cpu().numpy(), ref)
        del Cm
    print("stencil 64^3, N = 256, rel err vs FP64: " + ", ".join(f"{k} {v:.3e}" for k, v in errs.items()))
    for name, (f, tol) in forms.items():
        assert errs[name] <= tol, (name, errs[name], tol)
    M.close()


def test_batched512_grouped_each_problem(dev, smat_mod, oracle_lib):
    from smat import workloads
    probs = []
    for A, N, fk in workloads.batched512():
        form = smat_mod.FORM_F16 if fk == 0 else smat_mod.FORM_BF16
        tdt = torch.float16 if fk == 0 else torch.bfloat16
        M = smat_mod.Bcsr(A, forms=(form,))
        B = torch.randn((A.cols, N), device=dev, generator=None).to(tdt)
        Cm = torch.full((A.rows, N), float("nan"), dtype=torch.float32, device=dev)
        probs.append((A, M, form, B, Cm))
    g = smat_mod.Group([(M, f, B, Cm) for A, M, f, B, Cm in probs])
    g.run(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g.check_device_error()
    worst = {smat_mod.FORM_F16: 0.0, smat_mod.FORM_BF16: 0.0}
    for A, M, form, B, Cm in probs:
        ref = oracle_lib.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64),
                                  B.float().cpu().numpy().astype(np.float64))
        e = rel(Cm.cpu().numpy(), ref)
        worst[form] = max(worst[form], e)
        assert e <= (1e-3 if form == smat_mod.FORM_F16 else 1e-2), e
    print(f"batched 512: worst rel err vs FP64: FP16 {worst[smat_mod.FORM_F16]:.3e}, "
          f"BF16 {worst[smat_mod.FORM_BF16]:.3e}")
    g.close()
    for A, M, *_ in probs:
        M.close()
