"""CPU: the oracle (oracle/smat_oracle.cpp) against the reference's own
outputs, frozen in tests/golden/ by make_golden.py, and — where the reference
build exists (oracle/_ref) — against the reference live on fresh inputs.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def pre():
    return np.load(os.path.join(GOLD, "golden_preprocess.npz"))


def test_jaccard_known_answer(oracle_lib):
    # preprocess/test/general/TEST_similarities.cpp with -b 3: Jaccard 0.5
    d = oracle_lib.jaccard_group([1, 2, 5, 10, 12, 20], 1, [0, 2, 4, 10, 16], 1, 3)
    assert d == 0.5


def test_jaccard_golden(oracle_lib, pre):
    for i in range(int(pre["jac_n"])):
        ga, gb, bs = pre[f"jac{i}_p"]
        d = oracle_lib.jaccard_group(pre[f"jac{i}_a"], int(ga), pre[f"jac{i}_b"], int(gb), int(bs))
        assert np.float32(d) == pre[f"jac{i}_d"], i


def test_merge_rows_golden(oracle_lib, pre):
    for i in range(int(pre["mer_n"])):
        r = oracle_lib.merge_rows(pre[f"mer{i}_a"], pre[f"mer{i}_b"])
        assert np.array_equal(r, pre[f"mer{i}_r"]), i


def test_merge_rows_drops_tail_like_reference(oracle_lib):
    # utilities.cpp:145-173 stops copying A once B runs past it
    assert oracle_lib.merge_rows([1, 5, 9], [3]).tolist() == [1, 3]
    assert oracle_lib.merge_rows([1, 5], [3, 10]).tolist() == [1, 3, 10]


def test_keeper_reorder_golden(oracle_lib, pre):
    for i in range(int(pre["keep_n"])):
        tau, bb, BB, _ = pre[f"keep{i}_params"]
        perm, g, st = oracle_lib.reorder(pre[f"keep{i}_rowptr"], pre[f"keep{i}_cols"], float(tau), int(bb), int(BB))
        name = str(pre[f"keep{i}_name"])
        assert np.array_equal(g, pre[f"keep{i}_grouping"]), name
        assert np.array_equal(perm, pre[f"keep{i}_perm"]), name
        assert st[0] == pre[f"keep{i}_stats"][0] and st[1] == pre[f"keep{i}_stats"][1], name


def test_csr_to_bcsr_golden(oracle_lib):
    g = np.load(os.path.join(GOLD, "golden_bcsr.npz"))
    for i in range(int(g["bcsr_n"])):
        mr, mc, k = (int(x) for x in g[f"bcsr{i}_dims"])
        brp, bci, bv, info = oracle_lib.csr_to_bcsr(mr, mc, k, g[f"bcsr{i}_rowptr"], g[f"bcsr{i}_cols"],
                                                    g[f"bcsr{i}_vals"])
        assert np.array_equal(brp, g[f"bcsr{i}_brp"]), i
        assert np.array_equal(bci, g[f"bcsr{i}_bci"]), i
        assert np.array_equal(bv.view(np.uint16), g[f"bcsr{i}_bval"].view(np.uint16)), i
        assert np.array_equal(info, g[f"bcsr{i}_info"]), i


def test_csr_multiply_golden(oracle_lib):
    g = np.load(os.path.join(GOLD, "golden_multiply.npz"))
    rows = len(g["rowptr"]) - 1
    C = oracle_lib.csr_multiply_f32(g["rowptr"], g["cols"], g["vals"], g["B"], int(g["bcols"]), rows)
    assert np.array_equal(C, g["C"])


def test_fp64_oracle_matches_scipy(oracle_lib):
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(5)
    m = sp.random(200, 150, density=0.05, random_state=5, format="csr")
    B = rng.standard_normal((150, 9))
    C = oracle_lib.spmm_f64(m.indptr, m.indices, m.data, B)
    assert np.allclose(C, m @ B, rtol=1e-12, atol=1e-12)


def test_oracle_matches_reference_live(oracle_lib):
    if not oracle_lib.ref_available():
        pytest.skip("reference build unavailable")
    rng = np.random.default_rng(77)
    for t in range(12):
        rows, cols = int(rng.integers(1, 600)), int(rng.integers(1, 400))
        rp, cs = [0], []
        for _ in range(rows):
            c = np.unique(rng.integers(0, cols, int(rng.integers(0, 25))))
            cs.extend(c.tolist())
            rp.append(len(cs))
        rp, cs = np.array(rp), np.array(cs, np.int64)
        tau = float(rng.choice([0.2, 0.5, 0.6, 0.9]))
        b, B = int(rng.choice([1, 3, 8, 16])), int(rng.choice([2, 4, 16]))
        p1, g1, s1 = oracle_lib.reorder(rp, cs, tau, b, B)
        p2, g2, s2 = oracle_lib.ref_reorder(rp, cs, cols, tau, b, B)
        assert np.array_equal(g1, g2) and np.array_equal(p1, p2) and s1[0] == s2[0] and s1[1] == s2[1]
