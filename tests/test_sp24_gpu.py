"""GPU parity of the structured-sparse (2:4) path: with use_24 the blocks
that are exactly 2:4 leave the dense plan and run on tcgen05.mma.sp (A as
128 rows x 16 kept values plus 2-bit indices), the rest on the dense
kernel. Every result is checked against the FP64 CPU oracle: FP16 form
1e-3, BF16 form 1e-2 (the same bounds as the dense path), for matrices whose
blocks are all 2:4, none 2:4 and mixed, at several widths N, with FP32 and
FP16 C, and against the dense path on the same matrix."""
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


def run(M, B, form, out_dtype=torch.float32):
    C = M.spmm(B, form=form, out_dtype=out_dtype)
    torch.cuda.synchronize()
    M.check_device_error()
    return C.float().cpu().numpy()


def matrix(kind, smat_mod):
    from smat import generators as G
    if kind == "all24":
        A = G.force_24(G.random_block(2000, 0.05, 0.3, 0.9, seed=5), 1.0, seed=7)
    elif kind == "none24":
        A = G.band(2048, 40, seed=3)
    else:
        A = G.force_24(G.rmat(12, 60000, seed=9), 0.3, seed=8)
    return A


@pytest.mark.parametrize("kind", ["all24", "none24", "mixed"])
@pytest.mark.parametrize("N", [64, 128, 200, 256])
def test_fp16_vs_fp64(dev, smat_mod, oracle_lib, kind, N):
    A = matrix(kind, smat_mod)
    Bh = np.random.default_rng(N).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    M = smat_mod.Bcsr(A, use_24=True)
    n24 = M.info["n_blocks_24"]
    if kind == "all24":
        assert n24 == M.info["nnzb"] > 0
    elif kind == "none24":
        assert n24 == 0
    else:
        assert 0 < n24 < M.info["nnzb"]
    ref = fp64_product(oracle_lib, A, Bh)
    err = rel_err(run(M, torch.from_numpy(Bh).to(dev), smat_mod.FORM_F16), ref)
    print(f"2:4 path {kind} N={N}: {n24} of {M.info['nnzb']} blocks on mma.sp, rel err vs FP64 {err:.3e}")
    assert err <= 1e-3, err
    M.close()


@pytest.mark.parametrize("kind", ["all24", "mixed"])
def test_bf16_and_fp16_out(dev, smat_mod, oracle_lib, kind):
    A = matrix(kind, smat_mod)
    Bf = np.random.default_rng(3).standard_normal((A.cols, 128)).astype(np.float32)
    ref = fp64_product(oracle_lib, A, Bf)
    M = smat_mod.Bcsr(A, use_24=True, forms=(smat_mod.FORM_F16, smat_mod.FORM_BF16))
    B = torch.from_numpy(Bf).to(dev)
    e_bf = rel_err(run(M, B, smat_mod.FORM_BF16), ref)
    assert e_bf <= 1e-2, e_bf
    e_h = rel_err(run(M, B, smat_mod.FORM_F16, torch.float16), ref)
    assert e_h <= 2e-3, e_h                     # FP16 C: one more rounding of the result
    M.close()


def test_same_as_dense_path(dev, smat_mod):
    A = matrix("mixed", smat_mod)
    Bh = np.random.default_rng(1).uniform(-1, 1, (A.cols, 128)).astype(np.float16)
    B = torch.from_numpy(Bh).to(dev)
    M0 = smat_mod.Bcsr(A)
    M1 = smat_mod.Bcsr(A, use_24=True)
    assert M0.info["n_blocks_24"] == 0 and M1.info["n_blocks_24"] > 0
    c0 = run(M0, B, smat_mod.FORM_F16)
    c1 = run(M1, B, smat_mod.FORM_F16)
    assert rel_err(c1, c0.astype(np.float64)) <= 1e-5
    c1b = run(M1, B, smat_mod.FORM_F16)             # repeat: deterministic
    assert np.array_equal(c1, c1b)
    M0.close()
    M1.close()


def test_unit_threshold_routing(dev, smat_mod, oracle_lib):
    """use_24 = k routes only the exact-2:4 blocks of units (8 block rows x
    32 columns) holding at least k of them; the rest stay dense."""
    A = matrix("mixed", smat_mod)
    Bh = np.random.default_rng(5).uniform(-1, 1, (A.cols, 128)).astype(np.float16)
    ref = fp64_product(oracle_lib, A, Bh)
    B = torch.from_numpy(Bh).to(dev)
    counts = []
    for k in (1, 2, 4, 8, 17):
        M = smat_mod.Bcsr(A, use_24=k)
        counts.append(M.info["n_blocks_24"])
        err = rel_err(run(M, B, smat_mod.FORM_F16), ref)
        assert err <= 1e-3, (k, err)
        M.close()
    print("2:4 blocks routed for unit thresholds 1, 2, 4, 8, 17:", counts)
    assert counts[0] > counts[1] > counts[2] > 0
    assert all(a >= b for a, b in zip(counts, counts[1:]))
    assert counts[-1] == 0                        # a unit holds at most 16 blocks
