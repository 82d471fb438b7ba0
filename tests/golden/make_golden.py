"""Generates the golden fixtures in this directory by running the REFERENCE's
own code (built from its sources by oracle/Makefile into oracle/_ref/):

* golden_preprocess.npz — Jaccard distances and merge_rows results
  (preprocess/src/general/blocking.cpp, utilities.cpp), and Keeper groupings,
  permutations and counters (BlockingEngine::GetGrouping with
  `-a 5 -b b -B B -F f -t tau`) on the reference's TEST matrix, on its
  bcsstk18_r minitest graph and on seeded random patterns;
* golden_bcsr.npz — SparseMatrix::csrToBcsr (src/cuda_hgemm/src/common/matrix.h)
  block structure and values on seeded random CSRs with file-order columns;
* golden_multiply.npz — CSR::multiply (preprocess/src/general/csr.cpp) on a
  seeded case;
* golden_io.npz — mmio_allinone (src/cuda_hgemm/src/common/mmio_highlevel.h)
  on seeded MatrixMarket files (general, symmetric, pattern, integer,
  hermitian complex, FP16 rounding edge values) and CSR::read_from_edgelist
  on seeded edge lists, with the file texts;
* golden_tiles.npz — SparseMatrix::bcsrBlocking (matrix.h:794-1137), the
  merged 4 x 4-block tiles, on the csrToBcsr output of seeded CSRs (16 x 16
  and 16 x 32 blocks, empty tile rows, explicit zeros, 2:4-patterned rows,
  an empty matrix).

Run it where the reference sources are present:

    python tests/golden/make_golden.py [--reference /path/to/sptc-smat] [--only tiles]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def read_el(path):
    """Edge list as CSR::read_from_edgelist reads it (rows ascending, `row col [value]`,
    rows = last row + 1, cols = max column + 1)."""
    rows, cols, vals = [], [], []
    with open(path) as f:
        for line in f:
            if not line.strip() or line[0] in "#%":
                continue
            t = line.split()
            rows.append(int(t[0]))
            cols.append(int(t[1]))
            vals.append(float(t[2]) if len(t) > 2 else 1.0)
    r = np.array(rows, np.int64)
    n_rows = int(r[-1]) + 1
    rp = np.zeros(n_rows + 1, np.int64)
    np.add.at(rp, r + 1, 1)
    rp = np.cumsum(rp)
    return rp, np.array(cols, np.int64), np.array(vals, np.float32), n_rows, int(max(cols)) + 1


def rand_pattern(rng, rows, cols, deg, shuffle=False):
    rp = [0]
    cs = []
    for _ in range(rows):
        c = np.unique(rng.integers(0, cols, int(rng.integers(0, deg))))
        if shuffle:
            rng.shuffle(c)
        cs.extend(c.tolist())
        rp.append(len(cs))
    return np.array(rp, np.int64), np.array(cs, np.int64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SMAT_REFERENCE"),
                    help="reference source tree (default: $SMAT_REFERENCE, else the oracle recipe's default)")
    ap.add_argument("--only", choices=["tiles"], help="write only this fixture file")
    args = ap.parse_args()
    import oracle as O
    if args.reference:
        os.environ["SMAT_REFERENCE"] = args.reference
    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("reference build not available")
    if args.only == "tiles":
        make_tiles(O)
        return
    rng = np.random.default_rng(20261203)
    out = {}

    # --- Jaccard / merge_rows
    a = np.array([1, 2, 5, 10, 12, 20]); b = np.array([0, 2, 4, 10, 16])
    jac = [(a, 1, b, 1, 3)]
    for _ in range(200):
        A = np.unique(rng.integers(0, 300, rng.integers(0, 40)))
        B = np.unique(rng.integers(0, 300, rng.integers(0, 40)))
        jac.append((A, int(rng.integers(1, 16)), B, 1, int(rng.integers(1, 33))))
    out["jac_n"] = np.array(len(jac))
    for i, (A, ga, B, gb, bs) in enumerate(jac):
        out[f"jac{i}_a"], out[f"jac{i}_b"] = A.astype(np.int64), B.astype(np.int64)
        out[f"jac{i}_p"] = np.array([ga, gb, bs], np.int64)
        out[f"jac{i}_d"] = np.array(O.jaccard_group(A, ga, B, gb, bs, ref=True), np.float32)
    mer = []
    for _ in range(200):
        A = np.unique(rng.integers(0, 100, rng.integers(0, 20)))
        B = np.unique(rng.integers(0, 100, rng.integers(0, 20)))
        mer.append((A, B))
    out["mer_n"] = np.array(len(mer))
    for i, (A, B) in enumerate(mer):
        out[f"mer{i}_a"], out[f"mer{i}_b"] = A.astype(np.int64), B.astype(np.int64)
        out[f"mer{i}_r"] = O.merge_rows(A, B, ref=True)

    # --- Keeper reorder cases
    cases = []
    test_el = os.path.join(args.reference, "preprocess/data/TEST/TEST_matrix_weighted.el")
    rp, cs, _, nr, nc = read_el(test_el)
    for tau, bb, BB in [(0.5, 3, 3), (0.6, 3, 3), (0.5, 16, 16), (0.3, 2, 4), (0.9, 1, 2)]:
        cases.append(("TEST_matrix_weighted", rp, cs, nc, tau, bb, BB))
    bc = os.path.join(args.reference, "preprocess/data/minitest/bcsstk18_r.el")
    rp, cs, _, nr, nc = read_el(bc)
    cases.append(("bcsstk18_r", rp, cs, nc, 0.5, 16, 16))
    cases.append(("bcsstk18_r", rp, cs, nc, 0.6, 16, 16))
    for k in range(6):
        rows = int(rng.integers(50, 1500)); cols = int(rng.integers(30, 800))
        rp, cs = rand_pattern(rng, rows, cols, int(rng.integers(2, 30)))
        cases.append((f"random{k}", rp, cs, cols, float(rng.choice([0.3, 0.5, 0.6, 0.8])),
                      int(rng.choice([4, 8, 16])), int(rng.choice([4, 8, 16]))))
    out["keep_n"] = np.array(len(cases))
    for i, (name, rp, cs, nc, tau, bb, BB) in enumerate(cases):
        perm, g, st = O.ref_reorder(rp, cs, nc, tau, bb, BB, algo=5, force_fixed=True)
        out[f"keep{i}_name"] = np.array(name)
        out[f"keep{i}_rowptr"] = rp.astype(np.int64)
        out[f"keep{i}_cols"] = cs.astype(np.int32)
        out[f"keep{i}_params"] = np.array([tau, bb, BB, nc], np.float64)
        out[f"keep{i}_perm"] = perm.astype(np.int32)
        out[f"keep{i}_grouping"] = g.astype(np.int64)
        out[f"keep{i}_stats"] = st.astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "golden_preprocess.npz"), **out)

    # --- csrToBcsr cases
    out = {}
    bcases = []
    for k in range(8):
        mr = 16 * int(rng.integers(1, 24)); kk = int(rng.choice([16, 32]))
        mc = kk * int(rng.integers(1, 12))
        rp, cs = rand_pattern(rng, mr, mc, int(rng.integers(1, 60)), shuffle=True)
        v = rng.standard_normal(len(cs)).astype(np.float16)
        bcases.append((mr, mc, kk, rp, cs, v))
    out["bcsr_n"] = np.array(len(bcases))
    for i, (mr, mc, kk, rp, cs, v) in enumerate(bcases):
        brp, bci, bv, info = O.ref_csr_to_bcsr(mr, mc, kk, rp.astype(np.int32), cs.astype(np.int32), v)
        out[f"bcsr{i}_dims"] = np.array([mr, mc, kk], np.int64)
        out[f"bcsr{i}_rowptr"] = rp.astype(np.int32)
        out[f"bcsr{i}_cols"] = cs.astype(np.int32)
        out[f"bcsr{i}_vals"] = v
        out[f"bcsr{i}_brp"], out[f"bcsr{i}_bci"] = brp, bci
        out[f"bcsr{i}_bval"], out[f"bcsr{i}_info"] = bv, info
    np.savez_compressed(os.path.join(HERE, "golden_bcsr.npz"), **out)

    # --- CSR::multiply
    rows = 300
    rp, cs = rand_pattern(rng, rows, rows, 20)
    v = rng.standard_normal(len(cs)).astype(np.float32)
    bcols = 7
    Bc = rng.uniform(-1, 1, rows * bcols).astype(np.float32)
    Cref = O.ref_csr_multiply(rp, cs, v, rows, Bc, bcols, rows)
    np.savez_compressed(os.path.join(HERE, "golden_multiply.npz"), rowptr=rp, cols=cs.astype(np.int32), vals=v,
                        B=Bc, bcols=np.array(bcols), C=Cref)
    # --- file readers: mmio_allinone (MatrixMarket) and CSR::read_from_edgelist (edge lists)
    import tempfile
    out = {}
    tmp = tempfile.mkdtemp()
    mtx_cases = []

    def mtx_text(field, sym, m, n, entries, comment=True):
        lines = [f"%%MatrixMarket matrix coordinate {field} {sym}"]
        if comment:
            lines.append("% generated by make_golden.py")
        lines.append(f"{m} {n} {len(entries)}")
        for e in entries:
            lines.append(" ".join(str(x) for x in e))
        return "\n".join(lines) + "\n"

    def rand_entries(m, n, cnt, kind, lower=False):
        es = []
        for _ in range(cnt):
            i, j = int(rng.integers(1, m + 1)), int(rng.integers(1, n + 1))
            if lower and j > i:
                i, j = j, i
            if kind == "real":
                es.append((i, j, repr(float(rng.standard_normal() * 10.0 ** int(rng.integers(-3, 3))))))
            elif kind == "integer":
                es.append((i, j, int(rng.integers(-50, 50))))
            elif kind == "complex":
                es.append((i, j, repr(float(rng.standard_normal())), repr(float(rng.standard_normal()))))
            else:
                es.append((i, j))
        return es

    mtx_cases.append((mtx_text("real", "general", 37, 53, rand_entries(37, 53, 300, "real")), 16))
    mtx_cases.append((mtx_text("real", "symmetric", 50, 50, rand_entries(50, 50, 200, "real", lower=True)), 16))
    mtx_cases.append((mtx_text("pattern", "general", 70, 41, rand_entries(70, 41, 250, "pattern")), 32))
    mtx_cases.append((mtx_text("integer", "symmetric", 33, 33, rand_entries(33, 33, 90, "integer", lower=True)), 16))
    mtx_cases.append((mtx_text("complex", "hermitian", 20, 20, rand_entries(20, 20, 60, "complex", lower=True)), 16))
    # values that sit on FP16 rounding boundaries (ties, subnormals, overflow)
    edge_vals = ["1.00048828125", "1.0009765625", "1.00146484375", "6.103515625e-05", "2.98e-08", "65504",
                 "65520", "-65519.99", "1e-9", "3.0517578125e-05"]
    mtx_cases.append((mtx_text("real", "general", 16, 16, [(k + 1, k + 1, v) for k, v in enumerate(edge_vals)]), 16))
    out["mtx_n"] = np.array(len(mtx_cases))
    for i, (text, k) in enumerate(mtx_cases):
        path = os.path.join(tmp, f"m{i}.mtx")
        with open(path, "w") as f:
            f.write(text)
        m, n, sym, rp, ci, vb = O.ref_read_mtx(path, k)
        out[f"mtx{i}_text"] = np.array(text)
        out[f"mtx{i}_k"] = np.array(k)
        out[f"mtx{i}_shape"] = np.array([m, n, sym], np.int64)
        out[f"mtx{i}_rowptr"], out[f"mtx{i}_colidx"], out[f"mtx{i}_valbits"] = rp, ci, vb

    el_cases = []
    lines = ["# comment", "% another"]
    r = 0
    for _ in range(120):
        r += int(rng.integers(0, 3))
        lines.append(f"{r} {int(rng.integers(0, 90))} {float(rng.standard_normal()):.6g}")
    el_cases.append(("\n".join(lines) + "\n", 0))
    lines = []
    r = 2
    for _ in range(80):
        r += int(rng.integers(0, 2))
        lines.append(f"{r} {int(rng.integers(0, 200))}")
    el_cases.append(("\n".join(lines) + "\n", 1))
    out["el_n"] = np.array(len(el_cases))
    for i, (text, pat) in enumerate(el_cases):
        path = os.path.join(tmp, f"e{i}.el")
        with open(path, "w") as f:
            f.write(text)
        rows, cols, rp, ci, v = O.ref_read_el(path, pattern_only=bool(pat))
        out[f"el{i}_text"] = np.array(text)
        out[f"el{i}_pattern"] = np.array(pat)
        out[f"el{i}_shape"] = np.array([rows, cols], np.int64)
        out[f"el{i}_rowptr"], out[f"el{i}_colidx"], out[f"el{i}_vals"] = rp, ci, v
    np.savez_compressed(os.path.join(HERE, "golden_io.npz"), **out)
    make_tiles(O)
    print("golden fixtures written to", HERE)


def tile_cases(rng):
    """(m_row, m_col, k, rowptr, cols, values fp16) CSRs for the merged-tile fixtures."""
    cases = []
    for i in range(12):
        k = 16 if i % 2 == 0 else 32
        mr = 16 * int(rng.integers(1, 30))
        mc = k * int(rng.integers(1, 24))
        rp, cs = rand_pattern(rng, mr, mc, int(rng.integers(1, 50)), shuffle=True)
        v = rng.standard_normal(len(cs)).astype(np.float16)
        if i % 3 == 1:                      # explicit zeros
            v[rng.random(len(v)) < 0.4] = 0
        if i % 4 == 2:                      # whole tile rows without entries
            keep = np.ones(len(cs), bool)
            for r in range(mr):
                if (r // 64) % 2 == 1:
                    keep[rp[r]:rp[r + 1]] = False
            counts = np.array([keep[rp[r]:rp[r + 1]].sum() for r in range(mr)])
            rp = np.concatenate([[0], np.cumsum(counts)])
            cs, v = cs[keep], v[keep]
        cases.append((mr, mc, k, rp, cs, v))
    # rows with exactly two entries in every group of four columns (2:4 labels)
    mr, mc, k = 128, 256, 16
    rp, cs = [0], []
    for r in range(mr):
        c = []
        for g4 in range(0, mc, 4):
            if rng.random() < 0.3:
                c += sorted(rng.choice(4, 2, replace=False) + g4)
        cs += c
        rp.append(len(cs))
    cases.append((mr, mc, k, np.array(rp), np.array(cs), rng.standard_normal(len(cs)).astype(np.float16)))
    cases.append((64, 64, 16, np.zeros(65, np.int64), np.zeros(0, np.int64), np.zeros(0, np.float16)))
    # tiles first met out of column order inside a tile row (later block rows
    # reach further left), so the merged column array is not sorted there
    entries = {0: [200], 16: [5, 130], 40: [100, 255], 70: [250], 80: [10, 70], 127: [3]}
    rp, cs = [0], []
    for r in range(128):
        cs += entries.get(r, [])
        rp.append(len(cs))
    cases.append((128, 256, 16, np.array(rp), np.array(cs), np.linspace(-2, 2, len(cs)).astype(np.float16)))
    return cases


def make_tiles(O):
    rng = np.random.default_rng(20261204)
    out = {}
    cases = tile_cases(rng)
    out["tiles_n"] = np.array(len(cases))
    for i, (mr, mc, k, rp, cs, v) in enumerate(cases):
        brp, bci, bv, _ = O.ref_csr_to_bcsr(mr, mc, k, rp.astype(np.int32), cs.astype(np.int32), v)
        t = O.ref_bcsr_blocking(mr, mc, k, brp, bci, bv)
        out[f"tiles{i}_dims"] = np.array([mr, mc, k], np.int64)
        out[f"tiles{i}_brp"], out[f"tiles{i}_bci"] = brp, bci
        out[f"tiles{i}_bval"] = bv.reshape(-1).view(np.uint16)
        for key in O.TILE_KEYS:
            out[f"tiles{i}_{key}"] = t[key]
    np.savez_compressed(os.path.join(HERE, "golden_tiles.npz"), **out)


if __name__ == "__main__":
    main()
