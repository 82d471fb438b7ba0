"""GPU: the bounded-wait error path of the SpMM kernel, exercised without a
fault. A testing hook makes one MMA-issuing thread wait on a barrier that
nothing arrives at; with a 1 ms wait limit the launch must end within that
time scale, report SMAT_ERR_TIMEOUT with the stall's site (205) or the site
of the epilogue wait on the stalled warp's accumulator (301), whichever
limit runs out first (the epilogue starts waiting earlier), leave the
context usable, and the next launch on the same handle must be correct
against FP64 (FP16 form, 1e-3)."""
import time

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
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_expired_wait_reports_timeout_and_handle_recovers(dev, smat_mod, oracle_lib):
    from smat import generators as G
    A = G.rmat(12, 40000, seed=9)
    M = smat_mod.Bcsr(A)
    N = 64
    Bh = np.random.default_rng(4).uniform(-1, 1, (A.cols, N)).astype(np.float16)
    B = torch.from_numpy(Bh).to(dev)
    ref = oracle_lib.spmm_f64(A.row_ptr, A.col_idx, A.values.astype(np.float64), Bh.astype(np.float64))

    M.spmm(B)                                   # warm-up: kernel attributes, workspace
    torch.cuda.synchronize()
    M.check_device_error()

    M.set_wait_limit(1_000_000)                 # 1 ms
    M.debug_stall(1)                            # CTA 0's first MMA thread stalls before its first stage
    t0 = time.perf_counter()
    M.spmm(B)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    with pytest.raises(smat_mod.SmatError) as e:
        M.check_device_error()
    msg = str(e.value)
    assert "timed out" in msg and ("site 205" in msg or "site 301" in msg), msg
    assert dt < 1.0, dt                         # the 1 ms limit, not the 4 s default

    # the hook is one-shot, the handle and the context are intact
    Cm = M.spmm(B)
    torch.cuda.synchronize()
    M.check_device_error()
    e2 = rel(Cm.cpu().numpy(), ref)
    assert e2 <= 1e-3, e2
    M.set_wait_limit(0)
    Cm = M.spmm(B)
    torch.cuda.synchronize()
    M.check_device_error()
    assert rel(Cm.cpu().numpy(), ref) <= 1e-3
    M.close()
