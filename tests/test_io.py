"""CPU: the product's file readers and writer (sptc-smat_gb300/csrc/io.cpp)
against the reference's own readers — mmio_allinone
(src/cuda_hgemm/src/common/mmio_highlevel.h:514-680) and
CSR::read_from_edgelist (preprocess/src/general/csr.cpp:166-290) — frozen in
tests/golden/golden_io.npz, and live on fresh files where the reference
build exists. Integer structure and FP16 value bits must match exactly.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_io.npz")


@pytest.fixture(scope="module")
def gio():
    return np.load(GOLD)


def check_mtx(smat_mod, path, k, shape, rowptr, colidx, valbits):
    A = smat_mod.read_mtx(path, col_pad=k)
    m, n, _ = shape
    assert (A.rows, A.cols) == (m, n)
    assert np.array_equal(A.row_ptr, rowptr.astype(np.int64))
    assert np.array_equal(A.col_idx, colidx.astype(np.int32))
    # the reference converts each parsed double straight to FP16 (round to nearest even)
    with np.errstate(over="ignore"):                       # 65520 rounds to inf, as in the reference
        bits = A.values.astype(np.float16).view(np.uint16)
    assert np.array_equal(bits, valbits)


def test_read_mtx_golden(smat_mod, gio, tmp_path):
    for i in range(int(gio["mtx_n"])):
        p = tmp_path / f"m{i}.mtx"
        p.write_text(str(gio[f"mtx{i}_text"]))
        check_mtx(smat_mod, str(p), int(gio[f"mtx{i}_k"]), gio[f"mtx{i}_shape"], gio[f"mtx{i}_rowptr"],
                  gio[f"mtx{i}_colidx"], gio[f"mtx{i}_valbits"])


def test_read_mtx_symmetric_fill_order(smat_mod, tmp_path):
    # mirrored entries land right after their source, in file order
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 2.5\n2 1 -1\n3 2 0.5\n3 3 1e-3\n")
    A = smat_mod.read_mtx(str(p))
    assert (A.rows, A.cols) == (16, 16)
    assert A.row_ptr[:4].tolist() == [0, 2, 4, 6]
    assert A.col_idx.tolist() == [0, 1, 0, 2, 1, 2]
    assert A.values.tolist() == [2.5, -1.0, -1.0, 0.5, 0.5, 1e-3]


def test_read_el_golden(smat_mod, gio, tmp_path):
    for i in range(int(gio["el_n"])):
        p = tmp_path / f"e{i}.el"
        p.write_text(str(gio[f"el{i}_text"]))
        pat = bool(int(gio[f"el{i}_pattern"]))
        A = smat_mod.read_el(str(p), pattern_only=pat)
        rows, cols = (int(x) for x in gio[f"el{i}_shape"])
        assert (A.rows, A.cols) == (rows, cols)
        assert np.array_equal(A.row_ptr, gio[f"el{i}_rowptr"])
        assert np.array_equal(A.col_idx, gio[f"el{i}_colidx"].astype(np.int32))
        if pat:
            assert A.values is None
        else:
            assert np.array_equal(A.values, gio[f"el{i}_vals"])


def test_read_el_rejects_descending_rows(smat_mod, tmp_path):
    # the reference throws std::invalid_argument (csr.cpp:226-227)
    p = tmp_path / "bad.el"
    p.write_text("3 1 1.0\n1 2 1.0\n")
    with pytest.raises(smat_mod.SmatError) as e:
        smat_mod.read_el(str(p))
    assert e.value.status == 1


def test_read_mtx_rejects_bad_files(smat_mod, tmp_path):
    p = tmp_path / "bad.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n4 1 2.0\n")
    with pytest.raises(smat_mod.SmatError):
        smat_mod.read_mtx(str(p))               # row index out of range
    p.write_text("%%MatrixMarket matrix array real general\n3 3\n1\n2\n3\n")
    with pytest.raises(smat_mod.SmatError):
        smat_mod.read_mtx(str(p))               # dense array files are not read by the reference either
    with pytest.raises(smat_mod.SmatError):
        smat_mod.read_mtx(str(tmp_path / "missing.mtx"))


def test_write_el_round_trip(smat_mod, tmp_path):
    from smat import generators as G
    A = G.rmat(9, 3000, seed=4)
    perm = np.random.default_rng(0).permutation(A.rows)
    p = tmp_path / "r_reordered.el"
    smat_mod.write_el(str(p), A, perm)
    B = smat_mod.read_el(str(p), pattern_only=True)
    P = A.permuted(perm)
    last = int(np.max(np.nonzero(np.diff(P.row_ptr))[0])) + 1      # trailing empty rows are not written
    assert B.rows == last
    assert np.array_equal(B.row_ptr, P.row_ptr[: last + 1])
    assert np.array_equal(B.col_idx, P.col_idx)


def test_readers_match_reference_live(smat_mod, oracle_lib, tmp_path):
    if not oracle_lib.ref_available():
        pytest.skip("reference build unavailable")
    rng = np.random.default_rng(99)
    for t in range(6):
        m, n = int(rng.integers(1, 90)), int(rng.integers(1, 90))
        sym = "symmetric" if t % 2 else "general"
        if sym == "symmetric":
            n = m
        ents = []
        for _ in range(int(rng.integers(1, 300))):
            i, j = int(rng.integers(1, m + 1)), int(rng.integers(1, n + 1))
            if sym == "symmetric" and j > i:
                i, j = j, i
            ents.append(f"{i} {j} {float(rng.standard_normal()) * 100:.9g}")
        p = tmp_path / f"l{t}.mtx"
        p.write_text(f"%%MatrixMarket matrix coordinate real {sym}\n{m} {n} {len(ents)}\n" + "\n".join(ents) + "\n")
        k = int(rng.choice([16, 32]))
        mm, nn, s, rp, ci, vb = oracle_lib.ref_read_mtx(str(p), k)
        check_mtx(smat_mod, str(p), k, (mm, nn, s), rp, ci, vb)
        lines, r = [], 0
        for _ in range(int(rng.integers(1, 200))):
            r += int(rng.integers(0, 3))
            lines.append(f"{r} {int(rng.integers(0, 500))} {float(rng.standard_normal()):.7g}")
        q = tmp_path / f"l{t}.el"
        q.write_text("\n".join(lines) + "\n")
        rows, cols, rp, ci, v = oracle_lib.ref_read_el(str(q))
        A = smat_mod.read_el(str(q))
        assert (A.rows, A.cols) == (rows, cols)
        assert np.array_equal(A.row_ptr, rp) and np.array_equal(A.col_idx, ci.astype(np.int32))
        assert np.array_equal(A.values, v)
