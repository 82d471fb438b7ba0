"""Learned choice of the reordering threshold tau and the BCSR block shape.

For a matrix the pipeline can run the exhaustive sweep -- reorder with every
tau in {0.1, ..., 0.9} (Keeper, fixed-size groups) for every block shape
{8x8, 16x16, 32x16}, block, and time the SpMM at N = 128 in BF16 -- or ask a
small MLP (64 GPU-computed features -> 64-128-128-(9+3), trained with
libsmat's own kernels on sweeps the pipeline ran over seeded synthetic
matrices) for the shape in one forward pass. The sweep stays the fallback and
the judge: regret = t(predicted) / t(sweep best) - 1. The tensor-core SpMM
needs 16-column blocks, so the 8x8 shape is never available (never a label).

    python -m smat.selector --out DIR [--train 600] [--test 200] [--seed 1]
                            [--rows-min 8192] [--rows-max 32768]

builds the dataset (sweeps), trains, and writes DIR/selector_sweep.npz,
DIR/selector_weights.npz and a JSON summary line with the regrets. The
reorders of the sweep run in a pool of single-threaded worker processes,
one matrix per job (each regenerates its matrix from its seed), while the
parent times the SpMMs of the matrices already reordered on the GPU.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np

TAUS = [round(0.1 * i, 1) for i in range(1, 10)]
BLOCKS = [(8, 8), (16, 16), (32, 16)]          # (rows, cols) per block
DEFAULT = (TAUS.index(0.6), 1)                 # the method without the learned part: tau 0.6, 16x16
N_SWEEP = 128


# ------------------------------------------------------------------------------------------ matrices

def family_matrix(family: int, rows: int, rng: np.random.Generator):
    """A seeded synthetic matrix of one of four families, rows shuffled."""
    from . import generators as G
    seed = int(rng.integers(1 << 30))
    if family == 0:
        A = G.band(rows, int(rng.integers(4, 128)), seed=seed)
    elif family == 1:
        scale = max(8, int(np.ceil(np.log2(rows))))
        A = G.rmat(scale, int(rng.integers(4, 48)) * (1 << scale), seed=seed)
    elif family == 2:
        # block density 0.5-2 %, fill 20-95 %: at most ~2 % of the entries, as the sweep's families are stated
        A = G.random_block(rows, float(rng.uniform(0.005, 0.02)), float(rng.uniform(0.2, 0.9)), 0.95, seed=seed)
    else:
        A = G.stencil27(max(8, int(round(rows ** (1 / 3)))), seed=seed)
    perm = rng.permutation(A.rows)                 # scrambled rows: the reordering has work to do
    return A.permuted(perm)


def spec_matrix(spec):
    """The matrix of a dataset entry (family, rows, seed), regenerated deterministically."""
    family, rows, mseed = spec
    return family_matrix(int(family), int(rows), np.random.default_rng(int(mseed)))


def _sweep_job(job):
    """(index, {(t, b): perm}) for one matrix: every tau and supported block
    shape, in a worker process (CPU only, one thread)."""
    i, spec = job
    from . import reorder
    A = spec_matrix(spec)
    out = {}
    for t, tau in enumerate(TAUS):
        for b, (bh, bw) in enumerate(BLOCKS):
            if bw != 16:
                continue
            out[(t, b)] = reorder(A, tau=tau, col_block=bw, row_block=bh, algo=5,
                                  force_fixed=True).perm.astype(np.int32)
    return i, out


def _reorder_job(args):
    """(perm for one tau and block shape) in a worker process (CPU only)."""
    rows, cols, rp, ci, tau, bh, bw = args
    from . import Csr, reorder
    A = Csr(rows, cols, rp, ci, None)
    return reorder(A, tau=tau, col_block=bw, row_block=bh, algo=5, force_fixed=True).perm


def sweep_perms(mats, workers=None):
    """Permutations for every (matrix, tau, supported block shape), computed in a spawned process pool."""
    import multiprocessing as mp
    jobs, keys = [], []
    for m, A in enumerate(mats):
        for t, tau in enumerate(TAUS):
            for b, (bh, bw) in enumerate(BLOCKS):
                if bw != 16:
                    continue
                jobs.append((A.rows, A.cols, A.row_ptr, A.col_idx, tau, bh, bw))
                keys.append((m, t, b))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers or os.cpu_count()) as pool:
        perms = pool.map(_reorder_job, jobs, chunksize=4)
    return dict(zip(keys, perms))


def time_spmm(A, perm, block, device=0, reps=10):
    """Milliseconds of one BF16 SpMM (pack B + contraction) at N = 128."""
    import torch

    from . import FORM_BF16, Bcsr
    M = Bcsr(A, block=block, forms=(FORM_BF16,), row_perm=perm, device=device)
    B = torch.ones((A.cols, N_SWEEP), dtype=torch.bfloat16, device=f"cuda:{device}")
    out = torch.empty((A.rows, N_SWEEP), dtype=torch.float32, device=B.device)
    ws = torch.empty(M.workspace_size(FORM_BF16, 2, N_SWEEP), dtype=torch.uint8, device=B.device)
    for _ in range(3):
        M.spmm(B, form=FORM_BF16, out=out, workspace=ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        M.spmm(B, form=FORM_BF16, out=out, workspace=ws)
    e1.record()
    torch.cuda.synchronize()
    M.check_device_error()
    M.close()
    return e0.elapsed_time(e1) / reps


def dataset_specs(n: int, seed: int, rows_range=(8192, 32768)):
    """(family, rows, matrix seed) per entry: families in turn, rows log-uniform."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        rows = int(np.exp(rng.uniform(np.log(rows_range[0]), np.log(rows_range[1]))))
        specs.append((i % 4, rows, int(rng.integers(1 << 62))))
    return np.array(specs, np.int64)


def build_dataset(n: int, seed: int, rows_range=(8192, 32768), device=0, log=print, workers=None):
    """(specs [n, 3], features [n, 64], sweep times [n, 9, 3]; inf where a
    shape is unavailable). Largest matrices are reordered first."""
    import multiprocessing as mp

    from . import features
    specs = dataset_specs(n, seed, rows_range)
    X = np.zeros((n, 64), np.float32)
    T = np.full((n, len(TAUS), len(BLOCKS)), np.inf)
    order = sorted(range(n), key=lambda i: -int(specs[i][1]))
    jobs = [(i, tuple(specs[i])) for i in order]
    t0 = time.time()
    nproc = workers or max(1, (os.cpu_count() or 2) - 1)
    old = os.environ.get("OMP_NUM_THREADS")
    os.environ["OMP_NUM_THREADS"] = "1"           # one core per worker process
    try:
        ctx = mp.get_context("spawn")
        with ctx.Pool(nproc) as pool:
            done = 0
            for i, perms in pool.imap_unordered(_sweep_job, jobs):
                A = spec_matrix(specs[i])
                X[i] = features(A, device)
                for (t, b), perm in perms.items():
                    T[i, t, b] = time_spmm(A, perm.astype(np.int64), BLOCKS[b], device)
                done += 1
                if done % 50 == 0 or done == n:
                    log(f"[selector] {done}/{n} matrices swept, {time.time() - t0:.0f}s")
    finally:
        if old is None:
            os.environ.pop("OMP_NUM_THREADS", None)
        else:
            os.environ["OMP_NUM_THREADS"] = old
    return specs, X, T


def labels(T):
    flat = T.reshape(len(T), -1).argmin(1)
    return (flat // len(BLOCKS)).astype(np.int32), (flat % len(BLOCKS)).astype(np.int32)


# --------------------------------------------------------------------------------------------- model

class Selector:
    """The MLP on the GPU (smat_mlp_*)."""

    def __init__(self, device=0, seed=1234, params=None):
        from ._lib import check, lib
        self._lib, self._check = lib(), check
        h = C.c_void_p()
        check(self._lib.smat_mlp_create(device, seed, C.byref(h)))
        self._h = h
        if params is not None:
            p = np.ascontiguousarray(params, np.float32)
            check(self._lib.smat_mlp_set_params(self._h, p.ctypes.data))

    def params(self):
        p = np.zeros(self._lib.smat_mlp_num_params(), np.float32)
        self._check(self._lib.smat_mlp_get_params(self._h, p.ctypes.data))
        return p

    def train(self, X, yt, yb, epochs=400, lr=2e-3, batch=64, seed=0):
        rng = np.random.default_rng(seed)
        X = np.ascontiguousarray(X, np.float32)
        loss = np.zeros(1, np.float32)
        hist = []
        for ep in range(epochs):
            order = rng.permutation(len(X))
            for s in range(0, len(X), batch):
                idx = order[s:s + batch]
                xb = np.ascontiguousarray(X[idx])
                tb = np.ascontiguousarray(yt[idx], np.int32)
                bb = np.ascontiguousarray(yb[idx], np.int32)
                self._check(self._lib.smat_mlp_train_step(self._h, xb.ctypes.data, tb.ctypes.data, bb.ctypes.data,
                                                          len(idx), C.c_float(lr), loss.ctypes.data))
            hist.append(float(loss[0]))
        return hist

    def predict(self, X):
        """(tau index, block index) per row of X; the block head chooses among available shapes."""
        X = np.ascontiguousarray(X, np.float32)
        L = np.zeros((len(X), 12), np.float32)
        self._check(self._lib.smat_mlp_predict(self._h, X.ctypes.data, len(X), L.ctypes.data))
        blk_logits = L[:, 9:].copy()
        for b, (bh, bw) in enumerate(BLOCKS):
            if bw != 16:
                blk_logits[:, b] = -np.inf
        return L[:, :9].argmax(1), blk_logits.argmax(1)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.smat_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def load_default(device=0):
    """The selector trained on the committed sweep (data/selector_weights.npz)."""
    return Selector(device=device, params=np.load(os.path.join(DATA, "selector_weights.npz"))["params"])


def choose(csr, selector=None, device=0):
    """(tau, (block rows, block cols)) for csr: the selector's prediction, or,
    without one, the exhaustive sweep's best (the fallback)."""
    from . import features
    if selector is not None:
        ti, bi = selector.predict(features(csr, device)[None, :])
        return TAUS[int(ti[0])], BLOCKS[int(bi[0])]
    perms = sweep_perms([csr])
    best, arg = np.inf, None
    for (m, t, b), perm in perms.items():
        ms = time_spmm(csr, perm, BLOCKS[b], device)
        if ms < best:
            best, arg = ms, (TAUS[t], BLOCKS[b])
    return arg


def regret(T, ti, bi):
    best = T.reshape(len(T), -1).min(1)
    return T[np.arange(len(T)), ti, bi] / best - 1.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--train", type=int, default=600)
    ap.add_argument("--test", type=int, default=200)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=400)
    ap.add_argument("--rows-min", type=int, default=8192)
    ap.add_argument("--rows-max", type=int, default=32768)
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    n = args.train + args.test
    t0 = time.time()
    specs, X, T = build_dataset(n, args.seed, (args.rows_min, args.rows_max))
    sweep_s = time.time() - t0
    np.savez_compressed(os.path.join(args.out, "selector_sweep.npz"), X=X, T=T, specs=specs, taus=np.array(TAUS),
                        blocks=np.array(BLOCKS), train=np.array(args.train),
                        rows_range=np.array([args.rows_min, args.rows_max]))
    yt, yb = labels(T)
    sel = Selector(seed=args.seed)
    hist = sel.train(X[:args.train], yt[:args.train], yb[:args.train], epochs=args.epochs)
    ti, bi = sel.predict(X[args.train:])
    Tt = T[args.train:]
    r = regret(Tt, ti, bi)
    r0 = regret(Tt, np.full(len(Tt), DEFAULT[0]), np.full(len(Tt), DEFAULT[1]))
    np.savez_compressed(os.path.join(args.out, "selector_weights.npz"), params=sel.params())
    print(json.dumps({"train": args.train, "test": args.test, "rows": [args.rows_min, args.rows_max],
                      "sweep_seconds": sweep_s, "final_loss": hist[-1], "first_loss": hist[0],
                      "regret_mean": float(r.mean()), "regret_p90": float(np.quantile(r, 0.9)),
                      "regret_default_mean": float(r0.mean()), "regret_default_p90": float(np.quantile(r0, 0.9)),
                      "best_is_default_frac": float(np.mean(r0 == 0))}), flush=True)


if __name__ == "__main__":
    main()
