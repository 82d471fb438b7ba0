"""TEST INFRASTRUCTURE ONLY — runs the reference's own plain BCSR SpMM kernel,
mmaOBTKernelSparse (src/cuda_hgemm/src/mma/mmaOBT.cu:18-169), compiled from
its source for sm_103a by oracle/Makefile into oracle/_ref/mmaOBT.sm_103a.cubin,
and its 2:4 compressors preprocessing_mmaSTKernelSparse (mmaST.cu:22-140,
oracle/_ref/mmaST.sm_103a.cubin) and preprocessing_mmaSTKernelSparse_large
(mmaST_large.cu:22-152, oracle/_ref/mmaST_large.sm_103a.cubin).

The kernel is launched through the CUDA driver API on torch tensors, with the
reference's launch shape grid(ceil(N/8), M/16) x 32 threads (mmaOBT.cu:164-168)
and arguments (values, rowPtr, colIdx, B column-major, C row-major FP16,
M, N, K, nnzb, blockInfo, relativeBlockIndexMapping).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "mmaOBT.sm_103a.cubin")
SYMBOL = b"_Z18mmaOBTKernelSparseP6__halfPiS1_S0_S0_mmmmS1_S1_"

_cu = None
_fn = None


def available() -> bool:
    return os.path.exists(CUBIN)


def _load():
    global _cu, _fn
    if _fn is None:
        _cu = C.CDLL("libcuda.so.1")
        mod = C.c_void_p()
        r = _cu.cuModuleLoad(C.byref(mod), CUBIN.encode())
        if r != 0:
            raise RuntimeError(f"cuModuleLoad failed: {r}")
        fn = C.c_void_p()
        r = _cu.cuModuleGetFunction(C.byref(fn), mod, SYMBOL)
        if r != 0:
            raise RuntimeError(f"cuModuleGetFunction failed: {r}")
        _fn = fn
    return _fn


def run(vals_f16, rowptr, colidx, M, K, B_colmajor_f16, N, stream=None):
    """C (M x N, FP16, row-major) = reference kernel(A, B); all torch CUDA tensors.
    vals_f16: [nnzb, 16, 16]; rowptr [M/16 + 1]; colidx [nnzb] (column starts);
    B: K x N column-major FP16 (a tensor whose element (k, n) is at k + n*K)."""
    import torch
    fn = _load()
    dev = vals_f16.device
    nnzb = int(colidx.numel())
    ncr = K // 16
    # relativeBlockIndexMapping over the dense block grid: ptr of each block
    rel = torch.full(((M // 16) * ncr,), -1, dtype=torch.int32)
    rp = rowptr.cpu().numpy()
    ci = colidx.cpu().numpy()
    rows = np.repeat(np.arange(M // 16), np.diff(rp))
    rel_np = rel.numpy()
    rel_np[rows * ncr + ci // 16] = np.arange(nnzb, dtype=np.int32)
    rel = torch.from_numpy(rel_np).to(dev)
    info = torch.zeros_like(rel)
    Cm = torch.zeros((M, N), dtype=torch.float16, device=dev)
    args = [C.c_void_p(vals_f16.data_ptr()), C.c_void_p(rowptr.data_ptr()), C.c_void_p(colidx.data_ptr()),
            C.c_void_p(B_colmajor_f16.data_ptr()), C.c_void_p(Cm.data_ptr()), C.c_size_t(M), C.c_size_t(N),
            C.c_size_t(K), C.c_size_t(nnzb), C.c_void_p(info.data_ptr()), C.c_void_p(rel.data_ptr())]
    params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
    s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    r = _cu.cuLaunchKernel(fn, (N + 7) // 8, M // 16, 1, 32, 1, 1, 0, C.c_void_p(s), params, None)
    if r != 0:
        raise RuntimeError(f"cuLaunchKernel failed: {r}")
    return Cm, (args, params, rel, info)


CUBIN_ST = os.path.join(HERE, "_ref", "mmaST.sm_103a.cubin")
SYMBOL_ST = b"_Z31preprocessing_mmaSTKernelSparseP6__halfPcS0_mmmmPiS2_"
_fn_st = None


def compress_available() -> bool:
    return os.path.exists(CUBIN_ST)


CUBIN_ST_LARGE = os.path.join(HERE, "_ref", "mmaST_large.sm_103a.cubin")
SYMBOL_ST_LARGE = b"_Z37preprocessing_mmaSTKernelSparse_largeP6__halfPcS0_mmmmPiS2_"
_fn_st_large = None


def compress_large_available() -> bool:
    return os.path.exists(CUBIN_ST_LARGE)


def _function(cubin, symbol):
    _load()
    mod = C.c_void_p()
    r = _cu.cuModuleLoad(C.byref(mod), cubin.encode())
    if r != 0:
        raise RuntimeError(f"cuModuleLoad failed: {r}")
    fn = C.c_void_p()
    r = _cu.cuModuleGetFunction(C.byref(fn), mod, symbol)
    if r != 0:
        raise RuntimeError(f"cuModuleGetFunction failed: {r}")
    return fn


def compress24(vals_f16, block_info, rel_map, M, N, K, metadata, sparse, stream=None, large=False):
    """The reference compressor with its launch shape grid(ceil(N/8), ceil(M/16)) x 32
    (mmaST.cu:316-326; mmaST_large.cu:324-335 with large=True, 16 x 32 blocks),
    writing into the given metadata (int8) and sparse (FP16) tensors."""
    import torch
    global _fn_st, _fn_st_large
    if large:
        if _fn_st_large is None:
            _fn_st_large = _function(CUBIN_ST_LARGE, SYMBOL_ST_LARGE)
        fn = _fn_st_large
    else:
        if _fn_st is None:
            _fn_st = _function(CUBIN_ST, SYMBOL_ST)
        fn = _fn_st
    dev = vals_f16.device
    args = [C.c_void_p(vals_f16.data_ptr()), C.c_void_p(metadata.data_ptr()), C.c_void_p(sparse.data_ptr()),
            C.c_size_t(M), C.c_size_t(N), C.c_size_t(K), C.c_size_t(0), C.c_void_p(block_info.data_ptr()),
            C.c_void_p(rel_map.data_ptr())]
    params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
    s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    r = _cu.cuLaunchKernel(fn, (N + 7) // 8, (M + 15) // 16, 1, 32, 1, 1, 0, C.c_void_p(s), params, None)
    if r != 0:
        raise RuntimeError(f"cuLaunchKernel failed: {r}")
    return args, params
