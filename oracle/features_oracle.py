"""TEST INFRASTRUCTURE ONLY — numpy restatement of the 64 matrix features that
sptc-smat_gb300/csrc/features.cu computes on the GPU (same bins, same
normalisation), used by tests as the checker."""
from __future__ import annotations

import numpy as np


def features(rows, cols, row_ptr, col_idx):
    rp = np.asarray(row_ptr, np.int64)
    ci = np.asarray(col_idx, np.int64)
    nnz = int(rp[-1]) if len(rp) else 0
    out = np.zeros(64, np.float64)
    R, Z = max(1, rows), max(1, nnz)
    lens = np.diff(rp)
    bins = np.where(lens == 0, 0, np.minimum(15, 1 + np.floor(np.log2(np.maximum(lens, 1))).astype(np.int64)))
    out[0:16] = np.bincount(bins, minlength=16)[:16] / R
    r = np.repeat(np.arange(rows, dtype=np.int64), lens)
    d = np.abs(ci - r)
    span = float(max(rows, cols))
    out[16:32] = np.bincount(np.minimum(15, (d / span * 16.0).astype(np.int64)), minlength=16)[:16] / Z
    nbc = (cols + 15) // 16
    keys, counts = np.unique((r >> 4) * nbc + (ci >> 4), return_counts=True)
    T = max(1, len(keys))
    tb = np.minimum(15, np.floor(2.0 * np.log2(counts.astype(np.float64))).astype(np.int64))
    out[32:48] = np.bincount(tb, minlength=16)[:16] / T
    mean = lens.sum() / R
    var = max(0.0, (lens.astype(np.float64) ** 2).sum() / R - mean * mean)
    density = nnz / max(1.0, rows * max(1, cols))
    s = out[48:]
    s[0] = np.log2(rows + 1) / 20
    s[1] = np.log2(cols + 1) / 20
    s[2] = np.log2(nnz + 1) / 30
    s[3] = min(1.0, 100 * density)
    s[4] = mean / 64
    s[5] = np.sqrt(var) / mean if mean > 0 else 0.0
    s[6] = (lens.max() / mean / 100) if mean > 0 else 0.0
    s[7] = (d == 0).sum() / Z
    s[8] = (lens == 0).sum() / R
    s[9] = len(keys) / max(1.0, np.ceil(rows / 16.0)) / 64
    s[10] = counts.sum() / T / 256
    s[11] = np.log2(len(keys) + 1) / 25
    s[12] = (d < 64).sum() / Z
    return out
