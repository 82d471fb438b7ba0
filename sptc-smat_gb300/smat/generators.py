"""Seeded synthetic matrix families (numpy), standing in for the SuiteSparse
and generated matrices the reference benchmarks on.

The reference's own generators (src/generate_matrices.py:6-136) make band and
2:4 band matrices with all values 1; the families below add the value
distributions, R-MAT, the 27-point stencil and random-block matrices of the
workloads this package is measured on. Every function is deterministic in
its seed.
"""
from __future__ import annotations

import numpy as np

from . import Csr


def _csr_from_coo(rows: int, cols: int, r: np.ndarray, c: np.ndarray, v: np.ndarray | None) -> Csr:
    order = np.lexsort((c, r))
    r, c = r[order], c[order]
    if v is not None:
        v = v[order]
    rp = np.zeros(rows + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=rows), out=rp[1:])
    return Csr(rows, cols, rp, c.astype(np.int32), v)


def band(n: int, half_bw: int, seed: int = 1, dtype=np.float16) -> Csr:
    """A_ij != 0 iff |i - j| <= half_bw; values U[-1, 1] rounded to `dtype`."""
    rng = np.random.default_rng(seed)
    i = np.arange(n, dtype=np.int64)
    lo = np.maximum(i - half_bw, 0)
    hi = np.minimum(i + half_bw, n - 1)
    lens = hi - lo + 1
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    starts = np.repeat(lo - rp[:-1], lens)
    cols = (np.arange(rp[-1], dtype=np.int64) + starts).astype(np.int32)
    vals = rng.uniform(-1.0, 1.0, rp[-1]).astype(dtype)
    return Csr(n, n, rp, cols, vals)


def rmat(scale: int, n_unique: int, a=0.57, b=0.19, c=0.19, seed: int = 3, dtype=np.float16,
         permute_rows: bool = True) -> Csr:
    """R-MAT graph 2^scale x 2^scale: edges drawn (with recursive quadrant
    probabilities a, b, c, d = 1-a-b-c) until `n_unique` distinct entries exist;
    rows then randomly permuted; values N(0, 1)."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    keys = np.zeros(0, np.int64)
    p = np.array([a, b, c, 1.0 - a - b - c])
    cum = np.cumsum(p)
    while keys.size < n_unique:
        m = int((n_unique - keys.size) * 1.2) + 1024
        u = rng.random((m, scale))
        q = np.searchsorted(cum, u, side="right")  # 0..3 per level
        q = np.minimum(q, 3)
        bits = 1 << np.arange(scale - 1, -1, -1, dtype=np.int64)
        r = ((q >> 1) & 1).astype(np.int64) @ bits
        cc = (q & 1).astype(np.int64) @ bits
        keys = np.unique(np.concatenate([keys, r * n + cc]))
    if keys.size > n_unique:
        keys = np.sort(rng.choice(keys, n_unique, replace=False))
    r, cc = keys // n, keys % n
    if permute_rows:
        perm = rng.permutation(n)
        r = perm[r]
    v = rng.standard_normal(keys.size).astype(dtype)
    return _csr_from_coo(n, n, r, cc, v)


def stencil27(nx: int, seed: int = 4, dtype=np.float32) -> Csr:
    """27-point stencil on an nx^3 grid, natural order; off-diagonals N(1, 0.1),
    diagonal 27 + N(0, 1)."""
    rng = np.random.default_rng(seed)
    n = nx ** 3
    idx = np.arange(n, dtype=np.int64)
    z, y, x = idx // (nx * nx), (idx // nx) % nx, idx % nx
    rs, cs = [], []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ok = (z + dz >= 0) & (z + dz < nx) & (y + dy >= 0) & (y + dy < nx) & (x + dx >= 0) & (x + dx < nx)
                rs.append(idx[ok])
                cs.append(idx[ok] + dz * nx * nx + dy * nx + dx)
    r = np.concatenate(rs)
    c = np.concatenate(cs)
    v = rng.normal(1.0, 0.1, r.size)
    diag = r == c
    v[diag] = 27.0 + rng.standard_normal(int(diag.sum()))
    return _csr_from_coo(n, n, r, c, v.astype(dtype))


def random_block(n: int, block_density: float, fill_lo: float, fill_hi: float, bs: int = 16,
                 seed: int = 5, dtype=np.float16) -> Csr:
    """Random 16x16 blocks at the given block density, each filled to a
    random fraction in [fill_lo, fill_hi]; values N(0, 1)."""
    rng = np.random.default_rng(seed)
    nb = (n + bs - 1) // bs
    nblk = max(1, int(round(nb * nb * block_density)))
    flat = rng.choice(nb * nb, size=min(nblk, nb * nb), replace=False).astype(np.int64)
    br, bc = np.divmod(flat, nb)
    fill = rng.uniform(fill_lo, fill_hi, size=flat.size).astype(np.float32)
    m = rng.random((flat.size, bs, bs), dtype=np.float32) < fill[:, None, None]
    k, rr, cc = np.nonzero(m)
    r = rr.astype(np.int64) + br[k] * bs
    c = cc.astype(np.int64) + bc[k] * bs
    ok = (r < n) & (c < n)
    r, c = r[ok], c[ok]
    v = rng.standard_normal(r.size).astype(dtype)
    return _csr_from_coo(n, n, r, c, v)


def force_24(csr: Csr, fraction: float, bh: int = 16, bw: int = 16, seed: int = 6) -> Csr:
    """Rewrite a seeded `fraction` of the nonzero bh x bw blocks to an exact
    2:4 pattern: in every row of such a block, exactly 2 nonzeros in every
    aligned group of 4 columns (values N(0, 1)); nnz changes accordingly."""
    rng = np.random.default_rng(seed)
    r = np.repeat(np.arange(csr.rows, dtype=np.int64), np.diff(csr.row_ptr))
    c = csr.col_idx.astype(np.int64)
    v = csr.values if csr.values is not None else np.ones(csr.nnz, np.float32)
    nbc = (csr.cols + bw - 1) // bw
    bkey = (r // bh) * nbc + c // bw
    ublocks = np.unique(bkey)
    chosen = np.sort(rng.choice(ublocks, size=int(round(fraction * ublocks.size)), replace=False))
    keep = ~np.isin(bkey, chosen)
    # new 2:4 entries for each chosen block
    nch = chosen.size
    groups = bw // 4
    # per (block, row, group): choose 2 of 4 positions
    pairs = np.array([(i, j) for i in range(4) for j in range(i + 1, 4)], np.int64)  # 6 choices
    pick = pairs[rng.integers(0, 6, size=(nch, bh, groups))]  # (nch, bh, groups, 2)
    br = (chosen // nbc)[:, None, None, None]
    bc = (chosen % nbc)[:, None, None, None]
    rows = br * bh + np.arange(bh)[None, :, None, None]
    cols = bc * bw + (np.arange(groups) * 4)[None, None, :, None] + pick
    rows = np.broadcast_to(rows, cols.shape).reshape(-1)
    cols = cols.reshape(-1)
    ok = (rows < csr.rows) & (cols < csr.cols)
    rows, cols = rows[ok], cols[ok]
    vals = rng.standard_normal(rows.size).astype(v.dtype)
    return _csr_from_coo(csr.rows, csr.cols, np.concatenate([r[keep], rows]), np.concatenate([c[keep], cols]),
                         np.concatenate([v[keep], vals]))
