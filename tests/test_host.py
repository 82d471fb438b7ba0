"""CPU: libsmat's host side — the C ABI loads and exports what include/smat.h
declares, the reorder and the blocking are bit-identical to the reference
(golden fixtures), malformed input is rejected with a status, and the
synthetic generators and helpers behave."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(smat_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol(smat_mod):
    lib = ctypes.CDLL(smat_mod._lib.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert declared_symbols(), "no declarations found"
    assert not missing, missing


def test_version_and_error_text(smat_mod):
    assert b"sm_103a" in smat_mod.lib().smat_version()


def test_reorder_matches_reference_golden(smat_mod):
    g = np.load(os.path.join(GOLD, "golden_preprocess.npz"))
    for i in range(int(g["keep_n"])):
        tau, bb, BB, nc = g[f"keep{i}_params"]
        rp = g[f"keep{i}_rowptr"]
        A = smat_mod.Csr(len(rp) - 1, int(nc), rp, g[f"keep{i}_cols"])
        r = smat_mod.reorder(A, float(tau), int(bb), int(BB), algo=5, force_fixed=True)
        name = str(g[f"keep{i}_name"])
        assert np.array_equal(r.grouping, g[f"keep{i}_grouping"]), name
        assert np.array_equal(r.perm, g[f"keep{i}_perm"]), name
        assert (r.comparisons, r.merges) == tuple(g[f"keep{i}_stats"][:2]), name


def test_reorder_fixed_blocking(smat_mod):
    A = smat_mod.Csr(10, 10, np.arange(11), np.arange(10))
    r = smat_mod.reorder(A, 0.5, 4, 4, algo=2, force_fixed=False)
    assert r.grouping.tolist() == [i // 4 for i in range(10)]
    assert r.perm.tolist() == list(range(10))


def test_reorder_device_scan_needs_a_device(smat_mod):
    """Without a CUDA device a device scan is refused with a status (never a
    silent host run); with one, tests/test_reorder_gpu.py checks it."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    A = smat_mod.Csr(10, 10, np.arange(11), np.arange(10))
    with pytest.raises(smat_mod.SmatError) as e:
        smat_mod.reorder(A, 0.5, 4, 4, use_gpu=True)
    assert "use_gpu" in str(e.value)


def test_reorder_empty_rows_and_matrix(smat_mod):
    A = smat_mod.Csr(5, 8, np.zeros(6, np.int64), np.zeros(0, np.int32))
    r = smat_mod.reorder(A, 0.5, 4, 2)
    assert sorted(r.perm.tolist()) == list(range(5))
    Z = smat_mod.Csr(0, 0, np.zeros(1, np.int64), np.zeros(0, np.int32))
    assert smat_mod.reorder(Z, 0.5, 4, 2).perm.size == 0


def test_blocking_matches_reference_golden(smat_mod):
    g = np.load(os.path.join(GOLD, "golden_bcsr.npz"))
    for i in range(int(g["bcsr_n"])):
        mr, mc, k = (int(x) for x in g[f"bcsr{i}_dims"])
        A = smat_mod.Csr(mr, mc, g[f"bcsr{i}_rowptr"], g[f"bcsr{i}_cols"], g[f"bcsr{i}_vals"])
        rp, ci, v = smat_mod.csr_to_bcsr_host(A, (16, k))
        assert np.array_equal(rp, g[f"bcsr{i}_brp"]), i
        assert np.array_equal(ci, g[f"bcsr{i}_bci"]), i
        assert np.array_equal(v.view(np.uint16), g[f"bcsr{i}_bval"].view(np.uint16)), i


def test_blocking_with_row_perm_equals_blocking_of_permuted(smat_mod, oracle_lib):
    rng = np.random.default_rng(3)
    from smat import generators as G
    A = G.random_block(333, 0.04, 0.2, 0.9, seed=9)
    perm = rng.permutation(A.rows)
    rp1, ci1, v1 = smat_mod.csr_to_bcsr_host(A, (16, 16), perm)
    Ap = A.permuted(perm)
    mr, mc = (A.rows + 15) // 16 * 16, (A.cols + 15) // 16 * 16
    rpp = np.concatenate([Ap.row_ptr, np.full(mr - A.rows, Ap.row_ptr[-1])]).astype(np.int32)
    rp2, ci2, v2, _ = oracle_lib.csr_to_bcsr(mr, mc, 16, rpp, Ap.col_idx, Ap.values.astype(np.float16))
    assert np.array_equal(rp1, rp2) and np.array_equal(ci1, ci2)
    assert np.array_equal(v1.view(np.uint16), v2.view(np.uint16))


def test_fp64_values_round_directly_to_half(smat_mod):
    # mmio_highlevel.h:608 converts double -> half in one rounding
    x = np.array([1.0 + 2.0 ** -11 + 2.0 ** -40], np.float64)  # just above a tie in double
    A = smat_mod.Csr(1, 1, np.array([0, 1]), np.array([0]), x)
    _, _, v = smat_mod.csr_to_bcsr_host(A, (16, 16))
    assert float(v[0, 0, 0]) == float(np.float16(1.0 + 2.0 ** -10))


@pytest.mark.parametrize("bad", ["rowptr", "col", "perm"])
def test_malformed_input_is_rejected(smat_mod, bad):
    rp = np.array([0, 2, 3]); ci = np.array([0, 1, 1])
    perm = None
    if bad == "rowptr":
        rp = np.array([0, 3, 2])
    elif bad == "col":
        ci = np.array([0, 7, 1])
    else:
        perm = np.array([0, 0])
    A = smat_mod.Csr(2, 2, rp, ci, np.ones(3, np.float32))
    with pytest.raises(smat_mod.SmatError) as e:
        smat_mod.csr_to_bcsr_host(A, (16, 16), perm)
    assert e.value.status == 1  # SMAT_ERR_INVALID


def test_bcsr_create_without_gpu_reports_no_device(smat_mod):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    A = smat_mod.Csr(4, 4, np.arange(5), np.arange(4), np.ones(4, np.float32))
    with pytest.raises(smat_mod.SmatError) as e:
        smat_mod.Bcsr(A)
    assert e.value.status == 6  # SMAT_ERR_NO_DEVICE


def test_generators(smat_mod):
    from smat import generators as G
    b = G.band(4096, 64, seed=1)
    assert b.nnz == 524224  # 4096 * 129 - 64 * 65
    r = np.repeat(np.arange(b.rows), np.diff(b.row_ptr))
    assert np.all(np.abs(r - b.col_idx) <= 64)
    s = G.stencil27(8)
    assert s.nnz == sum((min(x + 1, 7) - max(x - 1, 0) + 1) for x in range(8)) ** 3
    d = s.to_scipy().diagonal()
    assert np.all(d > 20)
    m = G.rmat(10, 5000, seed=3)
    assert m.nnz == 5000 and m.rows == 1024
    assert len(set(zip(np.repeat(np.arange(m.rows), np.diff(m.row_ptr)).tolist(), m.col_idx.tolist()))) == 5000


def test_force_24_makes_exact_24_blocks(smat_mod, oracle_lib):
    from smat import generators as G
    A = G.rmat(9, 3000, seed=4)
    F = G.force_24(A, 0.5, seed=2)
    rp, ci, v = smat_mod.csr_to_bcsr_host(F, (16, 16))
    n24 = sum(oracle_lib.is_block_24(blk) and np.count_nonzero(blk) == 128 for blk in v)
    nb_a = smat_mod.csr_to_bcsr_host(A, (16, 16))[1].size
    assert abs(n24 - round(0.5 * nb_a)) <= 2


def test_partition_rows_covers_all_rows(smat_mod):
    from smat import generators as G
    A = G.rmat(11, 20000, seed=5)
    for world in (1, 2, 3, 8):
        parts = smat_mod.partition_rows(A, world)
        assert parts[0][0] == 0 and parts[-1][1] == A.rows
        assert all(p[1] == q[0] for p, q in zip(parts, parts[1:]))
        assert all(p[0] % 16 == 0 for p in parts)


def test_block_split_matches_reference_labels(smat_mod):
    """smat_csr_to_bcsr_split_host: the reference's blockInfo labels
    (csrToBcsr, frozen in golden_bcsr.npz) and its filterBcsrBlocks split."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_bcsr.npz"))
    for i in range(int(g["bcsr_n"])):
        mr, mc, k = (int(x) for x in g[f"bcsr{i}_dims"])
        A = smat_mod.Csr(mr, mc, g[f"bcsr{i}_rowptr"].astype(np.int64), g[f"bcsr{i}_cols"],
                         g[f"bcsr{i}_vals"].astype(np.float16))
        (rp24, ci24, v24), (rpd, cid, vd), grid = smat_mod.csr_to_bcsr_split_host(A, block_cols=k)
        assert np.array_equal(grid.reshape(-1), g[f"bcsr{i}_info"]), i
        brp, bci = g[f"bcsr{i}_brp"], g[f"bcsr{i}_bci"]
        bval = g[f"bcsr{i}_bval"].view(np.uint16).reshape(-1, 16, k)
        nbc = mc // k
        lab = np.array([grid[r, c // k] for r in range(len(brp) - 1) for c in bci[brp[r]:brp[r + 1]]])
        for want, (rp, ci, v) in ((1, (rp24, ci24, v24)), (2, (rpd, cid, vd))):
            sel = lab == want
            assert np.array_equal(ci, bci[sel]), (i, want)
            assert np.array_equal(v.view(np.uint16), bval[sel]), (i, want)
            rows = np.repeat(np.arange(len(brp) - 1), np.diff(brp))[sel]
            assert np.array_equal(rp, np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=len(brp) - 1))])), i
