"""GPU: grouped SpMM (smat_group_*) — many problems of uneven sizes, FP16 and
BF16 forms and N in {32, 64, 128}, in one persistent launch — against the
single-problem entry point (1e-5: only the summation order of split panels
differs) and FP64 (FP16 1e-3, BF16 1e-2), and replayed from a CUDA graph."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch.device("cuda", 0)


def make_problems(smat_mod, dev, count, seed):
    from smat import generators as G
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        rows = int(np.exp(rng.uniform(np.log(512), np.log(8192))))
        fam = i % 3
        if fam == 0:
            A = G.band(rows, int(rng.integers(8, 96)), seed=i)
        elif fam == 1:
            scale = max(9, int(np.log2(rows)))
            A = G.rmat(scale, int(rng.integers(8, 40)) * (1 << scale), seed=i)
        else:
            A = G.random_block(rows, float(rng.uniform(0.01, 0.05)), 0.4, 0.9, seed=i)
        N = int(rng.choice([32, 64, 128]))
        form = smat_mod.FORM_F16 if rng.random() < 0.5 else smat_mod.FORM_BF16
        tdt = torch.float16 if form == smat_mod.FORM_F16 else torch.bfloat16
        Bh = rng.uniform(-1, 1, (A.cols, N)).astype(np.float32)
        B = torch.from_numpy(Bh).to(dev).to(tdt)
        if rng.random() < 0.5:
            B = B.t().contiguous().t()                      # column-major
        M = smat_mod.Bcsr(A, forms=(form,))
        Cm = torch.full((A.rows, N), float("nan"), dtype=torch.float32, device=dev)
        probs.append((A, M, form, B, Cm))
    return probs


def fp64(A, B):
    import scipy.sparse as sps
    Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
    return Asp @ B.float().cpu().numpy().astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def test_group_matches_single_calls_and_fp64(dev, smat_mod):
    probs = make_problems(smat_mod, dev, 24, seed=3)
    g = smat_mod.Group([(M, f, B, Cm) for A, M, f, B, Cm in probs])
    g.run(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g.check_device_error()
    for A, M, form, B, Cm in probs:
        single = M.spmm(B, form=form)
        torch.cuda.synchronize()
        got = Cm.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, single.cpu().numpy().astype(np.float64)) <= 1e-5
        tol = 1e-3 if form == smat_mod.FORM_F16 else 1e-2
        assert rel(got, fp64(A, B)) <= tol
    g.close()


def test_group_replays_from_cuda_graph(dev, smat_mod):
    probs = make_problems(smat_mod, dev, 12, seed=8)
    g = smat_mod.Group([(M, f, B, Cm) for A, M, f, B, Cm in probs])
    s = torch.cuda.Stream()
    g.run(s.cuda_stream)                   # first run outside capture
    s.synchronize()
    ref = [Cm.clone() for *_, Cm in probs]
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        g.run(s.cuda_stream)
    for *_, Cm in probs:
        Cm.fill_(float("nan"))
    torch.cuda.synchronize()
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    g.check_device_error()
    for r, (*_, Cm) in zip(ref, probs):
        assert torch.equal(r, Cm)
    g.close()


def test_group_rejects_bad_problems(dev, smat_mod):
    from smat import generators as G
    A = G.band(256, 8, seed=1)
    M = smat_mod.Bcsr(A)
    B = torch.zeros((A.cols, 32), dtype=torch.float16, device=dev)
    Cm = torch.zeros((A.rows, 32), dtype=torch.float32, device=dev)
    with pytest.raises(smat_mod.SmatError):
        smat_mod.Group([(M, smat_mod.FORM_BF16, B, Cm)])   # form not materialised


def test_autotune_picks_the_fastest_and_is_used(dev, smat_mod):
    from smat import generators as G
    smat_mod.lib().smat_autotune_clear()
    A = G.rmat(13, 120000, seed=4)
    r = smat_mod.autotune(A, form=smat_mod.FORM_F16, N=128)
    assert not r["cached"] and r["panel_rows"] in (4, 8, 16) and r["ms"] > 0
    assert r["ms"] <= r["ms_default"] * 1.0001            # the default shape is one of the candidates
    again = smat_mod.autotune(A, form=smat_mod.FORM_F16, N=128)
    assert again["cached"] and again["panel_rows"] == r["panel_rows"]
    M = smat_mod.Bcsr(A)                                   # panel_rows = 0: the tuned shape
    assert M.info["panel_rows"] == r["panel_rows"]
    smat_mod.lib().smat_autotune_clear()


def test_features_match_oracle(dev, smat_mod):
    import features_oracle
    from smat import generators as G
    for A in (G.band(3000, 40, seed=1), G.rmat(12, 30000, seed=2), G.random_block(2000, 0.03, 0.4, 0.9, seed=3),
              G.stencil27(12)):
        got = smat_mod.features(A)
        ref = features_oracle.features(A.rows, A.cols, A.row_ptr, A.col_idx)
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-6), np.abs(got - ref).max()
