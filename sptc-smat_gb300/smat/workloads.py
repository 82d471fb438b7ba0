"""The benchmark workloads, built the same way for bench.py and the
full-size parity tests (all inputs synthetic and seeded).

rmat16():     R-MAT 2^16 x 2^16 (a=0.57, b=c=0.19, d=0.05), 2,000,000 distinct
              entries, rows randomly permuted, FP16 N(0,1) values; Jaccard row
              reordering (Keeper, tau 0.6, 16-column blocks, 16-row groups,
              fixed-size regrouping); 30 % of the nonzero 16 x 16 blocks of the
              reordered matrix rewritten to an exact 2:4 pattern. Returns A in
              its ORIGINAL row order and the reorder permutation. The
              permutation (~30 s of host cores) is cached on disk.
stencil64():  27-point stencil on a 64^3 grid, natural order, FP32 values.
batched512(): the 512 uneven matrices of the grouped workload (band / R-MAT /
              random-block, rows log-uniform in [1024, 32768], N in {32, 64,
              128}, FP16 or BF16).
"""
from __future__ import annotations

import hashlib
import os

import numpy as np

CACHE = os.environ.get("SMAT_CACHE", os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__)))), "_build", "bench_cache"))


def rmat16(cache: bool = True):
    """(A in original row order, perm) of the R-MAT 2^16 workload."""
    from . import reorder
    from . import generators as G

    A0 = G.rmat(16, 2_000_000, seed=3)
    perm = None
    pfile = None
    if cache:
        key = hashlib.sha1(A0.row_ptr.tobytes() + A0.col_idx.tobytes()).hexdigest()[:16]
        os.makedirs(CACHE, exist_ok=True)
        pfile = os.path.join(CACHE, f"perm_{key}_t0.6_b16_B16.npy")
        if os.path.exists(pfile):
            perm = np.load(pfile)
    if perm is None:
        perm = reorder(A0, tau=0.6, col_block=16, row_block=16, algo=5, force_fixed=True).perm
        if pfile:
            np.save(pfile, perm)
    Ar = A0.permuted(perm)                       # reordered row order
    Ar = G.force_24(Ar, 0.3, 16, 16, seed=6)     # exact 2:4 in 30 % of the blocks
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    return Ar.permuted(inv), perm                # back to the original row order


def stencil64():
    from . import generators as G
    return G.stencil27(64, seed=4)


def batched512(count: int = 512, seed: int = 11):
    """[(A, N, form)] of the grouped workload (form: 0 FP16, 1 BF16)."""
    from . import generators as G
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        rows = int(np.exp(rng.uniform(np.log(1024), np.log(32768))))
        fam = i % 3
        if fam == 0:
            A = G.band(rows, int(np.exp(rng.uniform(np.log(8), np.log(256)))), seed=i)
        elif fam == 1:
            scale = int(np.ceil(np.log2(rows)))
            A = G.rmat(scale, int(rng.uniform(8, 64) * (1 << scale)), seed=i)
        else:
            A = G.random_block(rows, float(rng.uniform(0.01, 0.05)), 0.4, 0.9, seed=i)
        N = int(rng.choice([32, 64, 128]))
        out.append((A, N, 0 if i % 2 == 0 else 1))
    return out
