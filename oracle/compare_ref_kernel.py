"""TEST INFRASTRUCTURE ONLY — times the reference's own plain BCSR kernel
(mmaOBTKernelSparse, run from oracle/_ref by ref_kernel.py) beside libsmat's
tensor-core SpMM on identical inputs, and reports both errors against FP64.

    python oracle/compare_ref_kernel.py [--workload band|rmat] [--reps 20]

Prints one JSON line per workload: kernel times (CUDA events on the launching
stream, after warm-up), useful TFLOP/s (2 nnz N / t), and relative Frobenius
errors vs the FP64 product.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "sptc-smat_gb300"))
sys.path.insert(0, ROOT)


def timeit(fn, reps, stream):
    import torch
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="both", choices=["band", "rmat", "both"])
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args()
    import scipy.sparse as sps
    import torch

    import ref_kernel
    import smat
    from smat import generators as G
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    loads = []
    if args.workload in ("band", "both"):
        loads.append(("band4096_hb64_N64", G.band(4096, 64, seed=1), None, 64))
    if args.workload in ("rmat", "both"):
        import bench
        A, perm = bench.build_matrix()
        loads.append(("rmat16_2M_reordered_24frac0.3_N128", A, perm, 128))
    for name, A, perm, N in loads:
        M = smat.Bcsr(A, row_perm=perm)
        rp, ci, v, _ = M.export()
        K = M.info["cols_padded"]
        Mrows = M.info["rows_padded"]
        Bh = np.random.default_rng(2).uniform(-1, 1, (A.cols, N)).astype(np.float16)
        Bpad = np.zeros((K, N), np.float16)
        Bpad[: A.cols] = Bh
        Bcol = torch.from_numpy(Bpad).to(dev).t().contiguous()   # (N, K): column-major K x N
        vals = torch.from_numpy(v).to(dev)
        rpd, cid = torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev)
        holder = {}

        def ref_call():
            C, keep = ref_kernel.run(vals, rpd, cid, Mrows, K, Bcol, N)
            holder["C"], holder["keep"] = C, keep

        ws_bytes = M.workspace_size(smat.FORM_F16, smat.F16, N)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        Cours = torch.empty((A.rows, N), dtype=torch.float32, device=dev)
        Bours = Bcol.t()[: A.cols]
        s = stream.cuda_stream

        def ours_call():
            M.spmm_raw(smat.FORM_F16, Bours, smat.F16, smat.COL_MAJOR, K, Cours, smat.F32, N, N, ws, ws_bytes, s)

        t_ref = timeit(ref_call, args.reps, stream)
        t_ours = timeit(ours_call, args.reps, stream)
        # errors vs FP64 (both in the ORIGINAL row order)
        Asp = sps.csr_matrix((A.values.astype(np.float64), A.col_idx, A.row_ptr), shape=(A.rows, A.cols))
        ref64 = Asp @ Bh.astype(np.float64)
        Cr = holder["C"].float().cpu().numpy()[: A.rows]
        if perm is not None:  # the reference writes C in the blocked (reordered) row order
            Cr2 = np.empty_like(Cr)
            Cr2[perm] = Cr
            Cr = Cr2
        Co = Cours.cpu().numpy()
        nrm = np.linalg.norm(ref64)
        useful = 2.0 * A.nnz * N
        print(json.dumps({
            "workload": name, "N": N, "nnz": A.nnz, "nnzb": int(ci.size),
            "reference_mmaOBTKernelSparse": {"ms": t_ref, "useful_tflops": useful / t_ref / 1e9,
                                             "rel_err_vs_fp64": float(np.linalg.norm(Cr - ref64) / nrm),
                                             "note": "FP16 accumulate, FP16 C (mmaOBT.cu)"},
            "smat_spmm_f16": {"ms": t_ours, "useful_tflops": useful / t_ours / 1e9,
                              "rel_err_vs_fp64": float(np.linalg.norm(Co - ref64) / nrm),
                              "note": "pack B + tcgen05 kind::f16, FP32 accumulate, FP32 C"},
            "speedup": t_ref / t_ours,
        }), flush=True)


if __name__ == "__main__":
    main()
