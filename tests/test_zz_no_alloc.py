"""GPU: smat_spmm_static_scratch (packed-B scratch in the library's fixed
device array, nothing allocated) against smat_spmm (caller workspace), both
called through the C ABI, on two calls in a row with different B, N and
form, so that the second call runs over the first call's leftovers. Also
checked against the FP64 oracle (FP16 form: 1e-3; split form: 1e-4), that
repeated calls leave the device's free memory unchanged (no allocation on the
path), and the rejection of a B too large for the array.

The file name sorts last so the test also runs after the whole GPU suite.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def rel_err(got, ref):
    return float(np.linalg.norm(np.asarray(got, np.float64) - ref) / np.linalg.norm(ref))


def call_both(smat_mod, M, form, B, b_dtype, N):
    """(C from smat_spmm_static_scratch, C from smat_spmm), row-major FP32."""
    L = smat_mod._lib.lib()
    Kc = M.info["cols"]
    s = torch.cuda.current_stream().cuda_stream
    C_static = torch.full((M.info["rows"], N), float("nan"), dtype=torch.float32, device=B.device)
    C_ref = torch.full_like(C_static, float("nan"))
    # B is (K, N) row-major
    st = L.smat_spmm_static_scratch(M.handle, form, C.c_void_p(B.data_ptr()), b_dtype, smat_mod.ROW_MAJOR, N,
                                    C.c_void_p(C_static.data_ptr()), smat_mod.F32, N, N, C.c_void_p(s))
    assert st == 0, L.smat_last_error().decode()
    ws_bytes = M.workspace_size(form, b_dtype, N)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=B.device)
    st = L.smat_spmm(M.handle, form, C.c_void_p(B.data_ptr()), b_dtype, smat_mod.ROW_MAJOR, N,
                     C.c_void_p(C_ref.data_ptr()), smat_mod.F32, N, N, C.c_void_p(ws.data_ptr()), ws_bytes,
                     C.c_void_p(s))
    assert st == 0, L.smat_last_error().decode()
    torch.cuda.synchronize()
    M.check_device_error()
    assert B.shape[0] == Kc
    return C_static.cpu().numpy(), C_ref.cpu().numpy()


def test_static_scratch_matches_workspace_entry_point(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.stencil27(14, seed=3)                              # FP32 values, 2744 rows
    M = smat_mod.Bcsr(A, forms=(smat_mod.FORM_F16, smat_mod.FORM_SPLIT_BF16))
    rng = np.random.default_rng(11)
    A64 = (A.row_ptr, A.col_idx, A.values.astype(np.float64))
    # call 1: FP16 form, FP16 B, N = 200 (two 128-column tiles)
    B1 = rng.uniform(-1, 1, (A.cols, 200)).astype(np.float16)
    Cs, Cr = call_both(smat_mod, M, smat_mod.FORM_F16, torch.from_numpy(B1).to(dev), smat_mod.F16, 200)
    assert np.isfinite(Cs).all()
    np.testing.assert_allclose(Cs, Cr, rtol=1e-6, atol=1e-6)
    ref1 = oracle_lib.spmm_f64(*A64, B1.astype(np.float64))
    assert rel_err(Cs, ref1) <= 1e-3
    # call 2: split form, FP32 B, N = 72 (fewer tiles: the array still holds call 1's B)
    B2 = rng.standard_normal((A.cols, 72)).astype(np.float32)
    Cs, Cr = call_both(smat_mod, M, smat_mod.FORM_SPLIT_BF16, torch.from_numpy(B2).to(dev), smat_mod.F32, 72)
    assert np.isfinite(Cs).all()
    np.testing.assert_allclose(Cs, Cr, rtol=1e-6, atol=1e-6)
    ref2 = oracle_lib.spmm_f64(*A64, B2.astype(np.float64))
    assert rel_err(Cs, ref2) <= 1e-4


def test_static_scratch_allocates_nothing(dev, smat_mod):
    from smat import generators as G
    A = G.rmat(12, 60_000, seed=5)
    M = smat_mod.Bcsr(A, forms=(smat_mod.FORM_F16,))
    L = smat_mod._lib.lib()
    N = 256
    B = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, (A.cols, N)).astype(np.float16)).to(dev)
    Cm = torch.empty((A.rows, N), dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream().cuda_stream

    def call():
        st = L.smat_spmm_static_scratch(M.handle, smat_mod.FORM_F16, C.c_void_p(B.data_ptr()), smat_mod.F16,
                                        smat_mod.ROW_MAJOR, N, C.c_void_p(Cm.data_ptr()), smat_mod.F32, N, N,
                                        C.c_void_p(s))
        assert st == 0, L.smat_last_error().decode()

    call()                                                   # the first call looks the array's address up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(50):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    M.check_device_error()
    assert free1 == free0


def test_static_scratch_rejects_oversized_b(dev, smat_mod):
    # K = 65536 columns: the split form at N = 256 needs 64 MiB of packed B
    rows, cols = 64, 65536
    rp = np.arange(rows + 1, dtype=np.int64) * 2
    ci = np.stack([np.arange(rows) * 7, np.arange(rows) * 7 + 40000], 1).reshape(-1).astype(np.int32)
    A = smat_mod.Csr(rows, cols, rp, ci, np.ones(rows * 2, np.float32))
    M = smat_mod.Bcsr(A, forms=(smat_mod.FORM_SPLIT_BF16,))
    N = 256
    assert M.workspace_size(smat_mod.FORM_SPLIT_BF16, smat_mod.F32, N) > (32 << 20)
    L = smat_mod._lib.lib()
    B = torch.zeros((cols, N), dtype=torch.float32, device=dev)
    Cm = torch.zeros((rows, N), dtype=torch.float32, device=dev)
    st = L.smat_spmm_static_scratch(M.handle, smat_mod.FORM_SPLIT_BF16, C.c_void_p(B.data_ptr()), smat_mod.F32,
                                    smat_mod.ROW_MAJOR, N, C.c_void_p(Cm.data_ptr()), smat_mod.F32, N, N, None)
    assert st == 2                                           # SMAT_ERR_UNSUPPORTED
    assert "static scratch" in L.smat_last_error().decode()
