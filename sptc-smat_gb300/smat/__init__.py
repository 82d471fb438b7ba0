"""smat — Python front end of libsmat, the GB300 SMaT pipeline.

Mirrors the reference's three-step surface:

* ``reorder``   — ``Matrix_Blocking -a 5 ... -F 1 -t tau`` / ``BlockingEngine::GetGrouping``
  (preprocess/src/general/blocking.cpp:616-657) as driven by ``reorder_using_paolo``
  (src/reorder.py:107-139), returning the reference's permutation;
* ``Bcsr``      — the ``SparseMatrix`` constructor (src/cuda_hgemm/src/common/matrix.h:161-246):
  CSR -> BCSR on the device;
* ``Bcsr.spmm`` — the SpMM launchers (src/cuda_hgemm/src/main.cu:20-28), on tcgen05 tensor cores.

Every call goes through the C ABI of ``include/smat.h``; there is no Python
or CPU fallback for the SpMM: without the built library or an sm_103 device
the calls raise ``SmatError``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from ._lib import (BF16, COL_MAJOR, E4M3, F16, F32, F64, FORM_BF16, FORM_F16, FORM_FP8, FORM_SPLIT_BF16,
                   ROW_MAJOR, BcsrInfo, BcsrOpts, CsrFile, CsrStruct, Problem, ReorderStats, SmatError, TilesDesc,
                   TuneResult, check, lib, ptr)

__all__ = ["Csr", "Bcsr", "Group", "Tiles", "autotune", "features", "transpose", "reorder_columns", "reorder", "read_mtx", "read_el", "write_el", "csr_to_bcsr_host", "partition_rows", "row_slice", "ReorderResult", "SmatError", "lib", "FORM_F16", "FORM_BF16",
           "FORM_FP8", "FORM_SPLIT_BF16", "F32", "F16", "BF16", "F64", "E4M3", "ROW_MAJOR", "COL_MAJOR"]

_VAL_DTYPES = {np.dtype(np.float32): F32, np.dtype(np.float16): F16, np.dtype(np.float64): F64}


@dataclass
class Csr:
    """CSR on the host. Column order inside a row is kept as given."""
    rows: int
    cols: int
    row_ptr: np.ndarray
    col_idx: np.ndarray
    values: np.ndarray | None = None

    def __post_init__(self):
        self.row_ptr = np.ascontiguousarray(self.row_ptr, dtype=np.int64)
        self.col_idx = np.ascontiguousarray(self.col_idx, dtype=np.int32)
        if self.values is not None:
            v = np.asarray(self.values)
            if v.dtype not in _VAL_DTYPES:
                v = v.astype(np.float32)
            self.values = np.ascontiguousarray(v)

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1]) if len(self.row_ptr) else 0

    def struct(self) -> CsrStruct:
        s = CsrStruct()
        s.rows, s.cols, s.nnz = self.rows, self.cols, self.nnz
        s.row_ptr = self.row_ptr.ctypes.data
        s.col_idx = self.col_idx.ctypes.data if self.nnz else None
        if self.values is not None:
            s.values = self.values.ctypes.data
            s.values_dtype = _VAL_DTYPES[self.values.dtype]
        else:
            s.values = None
            s.values_dtype = F32
        return s

    @classmethod
    def from_scipy(cls, m, keep_order: bool = True) -> "Csr":
        m = m.tocsr()
        if not keep_order:
            m.sort_indices()
        return cls(m.shape[0], m.shape[1], m.indptr, m.indices, m.data)

    def to_scipy(self):
        import scipy.sparse as sp
        vals = self.values if self.values is not None else np.ones(self.nnz, np.float32)
        return sp.csr_matrix((vals, self.col_idx, self.row_ptr), shape=(self.rows, self.cols))

    def permuted(self, perm: np.ndarray) -> "Csr":
        """Rows reordered: new row r = old row perm[r] (CSR::permute_rows, csr.cpp:65-74)."""
        perm = np.asarray(perm, np.int64)
        lens = np.diff(self.row_ptr)[perm]
        rp = np.zeros(self.rows + 1, np.int64)
        np.cumsum(lens, out=rp[1:])
        idx = np.concatenate([np.arange(self.row_ptr[p], self.row_ptr[p + 1]) for p in perm]) if self.rows else \
            np.zeros(0, np.int64)
        vals = None if self.values is None else self.values[idx]
        return Csr(self.rows, self.cols, rp, self.col_idx[idx], vals)


def _take_file(f: CsrFile) -> Csr:
    """Copy a library-owned CSR into numpy arrays and release it."""
    try:
        c = f.csr
        rp = np.ctypeslib.as_array(C.cast(c.row_ptr, C.POINTER(C.c_int64)), (c.rows + 1,)).copy()
        ci = (np.ctypeslib.as_array(C.cast(c.col_idx, C.POINTER(C.c_int32)), (c.nnz,)).copy() if c.nnz
              else np.zeros(0, np.int32))
        vals = None
        if c.values:
            ct = {F64: C.c_double, F32: C.c_float}[c.values_dtype]
            vals = (np.ctypeslib.as_array(C.cast(c.values, C.POINTER(ct)), (c.nnz,)).copy() if c.nnz
                    else np.zeros(0, {F64: np.float64, F32: np.float32}[c.values_dtype]))
        return Csr(int(c.rows), int(c.cols), rp, ci, vals)
    finally:
        lib().smat_csr_file_free(C.byref(f))


def read_mtx(path: str, col_pad: int = 16) -> Csr:
    """MatrixMarket -> Csr the way the SpMM harness reads it (padded, file order, symmetric expanded)."""
    f = CsrFile()
    check(lib().smat_read_mtx(os.fsencode(path), col_pad, C.byref(f)))
    return _take_file(f)


def read_el(path: str, pattern_only: bool = False) -> Csr:
    """Edge list -> Csr the way the preprocessing tool reads it."""
    f = CsrFile()
    check(lib().smat_read_el(os.fsencode(path), 1 if pattern_only else 0, C.byref(f)))
    return _take_file(f)


def write_el(path: str, csr: Csr, row_perm=None) -> None:
    """Pattern edge list with new row r = old row row_perm[r] (the *_reordered.el file)."""
    perm = None if row_perm is None else np.ascontiguousarray(row_perm, np.int64)
    s = csr.struct()
    check(lib().smat_write_el(os.fsencode(path), C.byref(s), None if perm is None else perm.ctypes.data))


@dataclass
class ReorderResult:
    perm: np.ndarray
    grouping: np.ndarray
    comparisons: int
    merges: int


def reorder(csr: Csr, tau: float = 0.5, col_block: int = 16, row_block: int = 16, algo: int = 5,
            force_fixed: bool = True, use_gpu: bool = False) -> ReorderResult:
    """Row reordering with the reference's result: new row r = old row perm[r].
    use_gpu=True measures the candidate distances on the current CUDA device
    (the seed loop and its commits stay on the host); same result."""
    perm = np.zeros(csr.rows, np.int64)
    grouping = np.zeros(csr.rows, np.int64)
    st = ReorderStats()
    s = csr.struct()
    check(lib().smat_reorder(C.byref(s), C.c_float(tau), col_block, row_block, algo, 1 if force_fixed else 0,
                             1 if use_gpu else 0, perm.ctypes.data, grouping.ctypes.data, C.byref(st)))
    return ReorderResult(perm, grouping, st.comparisons, st.merges)


def transpose(csr: Csr) -> Csr:
    """The transposed pattern (and values), rows in column order."""
    r = np.repeat(np.arange(csr.rows, dtype=np.int64), np.diff(csr.row_ptr))
    order = np.argsort(csr.col_idx, kind="stable")
    rp = np.zeros(csr.cols + 1, np.int64)
    np.add.at(rp, csr.col_idx.astype(np.int64) + 1, 1)
    vals = None if csr.values is None else csr.values[order]
    return Csr(csr.cols, csr.rows, np.cumsum(rp), r[order].astype(np.int32), vals)


def reorder_columns(csr: Csr, tau: float = 0.5, col_block: int = 16, row_block: int = 16, row_perm=None) -> np.ndarray:
    """Column permutation from the reference's second pass (src/reorder.py:140-182):
    Keeper on the rows of the transposed (row-reordered) matrix; new column c =
    old column result[c]. Use it as Bcsr(..., col_perm=...)."""
    A = csr if row_perm is None else csr.permuted(np.asarray(row_perm))
    return reorder(transpose(A), tau=tau, col_block=col_block, row_block=row_block, algo=5, force_fixed=True).perm


def csr_to_bcsr_host(csr: Csr, block=(16, 16), row_perm=None):
    """Host-only blocking: (row_ptr, col_idx (column starts), values fp16 [nnzb, bh, bw])."""
    bh, bw = block
    perm = None if row_perm is None else np.ascontiguousarray(row_perm, np.int64)
    s = csr.struct()
    nnzb = C.c_int64()
    pp = None if perm is None else perm.ctypes.data
    check(lib().smat_csr_to_bcsr_host(C.byref(s), bh, bw, pp, C.byref(nnzb), None, None, None))
    n = nnzb.value
    rows_p = (csr.rows + bh - 1) // bh * bh
    rp = np.zeros(rows_p // bh + 1, np.int32)
    ci = np.zeros(max(n, 1), np.int32)
    vals = np.zeros(max(n, 1) * bh * bw, np.uint16)
    check(lib().smat_csr_to_bcsr_host(C.byref(s), bh, bw, pp, C.byref(nnzb), rp.ctypes.data, ci.ctypes.data,
                                      vals.ctypes.data))
    return rp, ci[:n], vals[: n * bh * bw].view(np.float16).reshape(n, bh, bw)


def csr_to_bcsr_split_host(csr: Csr, block_cols: int = 16, row_perm=None):
    """The reference's 2:4 / dense block split (smat_csr_to_bcsr_split_host):
    ((row_ptr, col_idx, values) of the "2:4" blocks, the same of the dense
    blocks, the label grid)."""
    perm = None if row_perm is None else np.ascontiguousarray(row_perm, np.int64)
    s = csr.struct()
    n24, nd = C.c_int64(), C.c_int64()
    pp = None if perm is None else perm.ctypes.data
    check(lib().smat_csr_to_bcsr_split_host(C.byref(s), block_cols, pp, C.byref(n24), C.byref(nd), None, None, None,
                                            None, None, None, None))
    nbr = (csr.rows + 15) // 16
    nbc = (csr.cols + block_cols - 1) // block_cols
    bsz = 16 * block_cols
    out = []
    for n in (n24.value, nd.value):
        out.append((np.zeros(nbr + 1, np.int32), np.zeros(max(n, 1), np.int32), np.zeros(max(n, 1) * bsz, np.uint16)))
    grid = np.zeros(max(nbr * nbc, 1), np.int32)
    (a_rp, a_ci, a_v), (d_rp, d_ci, d_v) = out
    check(lib().smat_csr_to_bcsr_split_host(C.byref(s), block_cols, pp, C.byref(n24), C.byref(nd), a_rp.ctypes.data,
                                            a_ci.ctypes.data, a_v.ctypes.data, d_rp.ctypes.data, d_ci.ctypes.data,
                                            d_v.ctypes.data, grid.ctypes.data))
    n1, n2 = n24.value, nd.value
    return ((a_rp, a_ci[:n1], a_v[:n1 * bsz].view(np.float16).reshape(n1, 16, block_cols)),
            (d_rp, d_ci[:n2], d_v[:n2 * bsz].view(np.float16).reshape(n2, 16, block_cols)),
            grid[:nbr * nbc].reshape(nbr, nbc))


def _torch_dt(dt):
    import torch
    return {torch.float32: F32, torch.float16: F16, torch.bfloat16: BF16}[dt]


def _torch_layout(t):
    """(layout, ld) of a 2-D torch tensor viewed as (K, N)."""
    if t.dim() != 2:
        raise ValueError("B must be 2-D (K, N)")
    s0, s1 = t.stride()
    if s0 == 1 and (s1 >= t.shape[0] or t.shape[1] == 1):
        return COL_MAJOR, max(s1, t.shape[0])
    if s1 == 1:
        return ROW_MAJOR, max(s0, t.shape[1])
    raise ValueError("B must have a unit stride in one dimension")


class Bcsr:
    """A BCSR matrix resident on one GPU (the reference's ``SparseMatrix``)."""

    def __init__(self, csr: Csr, block=(16, 16), forms=(FORM_F16,), row_perm=None, panel_rows: int = 0,
                 device: int = 0, use_24: bool = False, split_frac: float = 0.0, col_perm=None,
                 n_tile_cols: int = 0, pipeline_depth: int = 0):
        o = BcsrOpts()
        o.block_rows, o.block_cols = block
        o.forms = 0
        for f in forms:
            o.forms |= 1 << f
        o.use_24 = int(use_24)          # True: every exact-2:4 block; k > 1: units of >= k such blocks
        o.n_tile_cols = n_tile_cols
        o.pipeline_depth = pipeline_depth
        self._perm = None if row_perm is None else np.ascontiguousarray(row_perm, np.int64)
        o.row_perm = None if self._perm is None else self._perm.ctypes.data
        o.device = device
        o.panel_rows = panel_rows
        o.split_frac = split_frac
        self._cperm = None if col_perm is None else np.ascontiguousarray(col_perm, np.int64)
        o.col_perm = None if self._cperm is None else self._cperm.ctypes.data
        h = C.c_void_p()
        s = csr.struct()
        check(lib().smat_bcsr_create(C.byref(s), C.byref(o), C.byref(h)))
        self._h = h
        self.device = device
        self.forms = tuple(forms)
        inf = BcsrInfo()
        check(lib().smat_bcsr_get_info(self._h, C.byref(inf)))
        self.info = {k: getattr(inf, k) for k, _ in BcsrInfo._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().smat_bcsr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def export(self):
        """(row_ptr int32, col_idx int32 (column starts), values fp16 [nnzb, bh, bw], is_24 uint8)."""
        i = self.info
        nbr = i["rows_padded"] // i["block_rows"]
        rp = np.zeros(nbr + 1, np.int32)
        ci = np.zeros(max(i["nnzb"], 1), np.int32)
        vals = np.zeros(max(i["nnzb"], 1) * i["block_rows"] * i["block_cols"], np.uint16)
        is24 = np.zeros(max(i["nnzb"], 1), np.uint8)
        check(lib().smat_bcsr_export(self._h, rp.ctypes.data, ci.ctypes.data, vals.ctypes.data, is24.ctypes.data))
        n = i["nnzb"]
        return (rp, ci[:n], vals[: n * i["block_rows"] * i["block_cols"]].view(np.float16)
                .reshape(n, i["block_rows"], i["block_cols"]), is24[:n])

    def set_wait_limit(self, ns: int):
        """Limit of every device-side wait of this matrix's SpMMs (0: 4 s)."""
        check(lib().smat_bcsr_set_wait_limit(self._h, int(ns)))

    def debug_stall(self, stage: int):
        """Testing hook: the next SpMM stalls before the given stage until its wait limit."""
        check(lib().smat_bcsr_debug_stall(self._h, int(stage)))

    def workspace_size(self, form: int, b_dtype: int, N: int) -> int:
        n = C.c_size_t()
        check(lib().smat_spmm_workspace_size(self._h, form, b_dtype, N, C.byref(n)))
        return n.value

    def spmm_raw(self, form, B, b_dtype, b_layout, ldb, Cmat, c_dtype, ldc, N, workspace=None,
                 workspace_bytes=0, stream=0):
        """Direct C-ABI call on device pointers (ints or tensors)."""
        check(lib().smat_spmm(self._h, form, ptr(B), b_dtype, b_layout, ldb, ptr(Cmat), c_dtype, ldc, N,
                              ptr(workspace), workspace_bytes, stream))

    def pack_b(self, form, B, b_dtype, b_layout, ldb, N, workspace, workspace_bytes, stream=0):
        """smat_spmm_pack_b: B into the packed tile layout in `workspace`."""
        check(lib().smat_spmm_pack_b(self._h, form, ptr(B), b_dtype, b_layout, ldb, N, ptr(workspace),
                                     workspace_bytes, stream))

    def spmm_packed(self, form, packed_b, N, Cmat, c_dtype, ldc, stream=0):
        """smat_spmm_packed: the contraction alone, from a packed B."""
        check(lib().smat_spmm_packed(self._h, form, ptr(packed_b), N, ptr(Cmat), c_dtype, ldc, stream))

    def spmm(self, B, form: int = FORM_F16, out=None, out_dtype=None, workspace=None, stream=None):
        """C = A @ B for a torch CUDA tensor B of shape (K, N); returns C (rows, N)."""
        import torch
        K, N = B.shape
        if K != self.info["cols"]:
            raise ValueError(f"B has {K} rows, A has {self.info['cols']} columns")
        b_dtype = {torch.float32: F32, torch.float16: F16, torch.bfloat16: BF16}[B.dtype]
        layout, ldb = _torch_layout(B)
        if out is None:
            out = torch.empty((self.info["rows"], N), device=B.device,
                              dtype=out_dtype if out_dtype is not None else torch.float32)
        c_dtype = {torch.float32: F32, torch.float16: F16}[out.dtype]
        ws_bytes = self.workspace_size(form, b_dtype, N)
        if workspace is None and ws_bytes:
            workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=B.device)
        s = stream if stream is not None else torch.cuda.current_stream(B.device).cuda_stream
        self.spmm_raw(form, B, b_dtype, layout, ldb, out, c_dtype, out.stride(0), N,
                      workspace, 0 if workspace is None else workspace.numel(), s)
        return out

    def spmm_host(self, B: np.ndarray, form: int = FORM_F16, out_dtype=np.float32, out=None,
                  stream=0) -> np.ndarray:
        """Host-buffer SpMM (smat_spmm_host): B (K, N) numpy in, C (rows, N) numpy out.
        With page-locked B and C (e.g. views of torch pin_memory tensors) the
        kernels read B and write C in place over the CPU-GPU link."""
        B = np.asarray(B)
        K, N = B.shape
        b_dtype = {np.dtype(np.float32): F32, np.dtype(np.float16): F16}[B.dtype]
        if B.flags.c_contiguous:
            layout, ldb = ROW_MAJOR, N
        elif B.flags.f_contiguous:
            layout, ldb = COL_MAJOR, K
        else:
            B = np.ascontiguousarray(B)
            layout, ldb = ROW_MAJOR, N
        if out is None:
            out = np.empty((self.info["rows"], N), dtype=out_dtype)
        if not out.flags.c_contiguous or out.shape != (self.info["rows"], N):
            raise ValueError("out must be a C-contiguous (rows, N) array")
        c_dtype = F32 if out.dtype == np.float32 else F16
        check(lib().smat_spmm_host(self._h, form, B.ctypes.data, b_dtype, layout, ldb, out.ctypes.data, c_dtype,
                                   N, N, stream))
        return out

    def check_device_error(self):
        check(lib().smat_bcsr_check_device_error(self._h))


def autotune(csr: Csr, form: int = FORM_F16, N: int = 128, block=(16, 16), row_perm=None, device: int = 0) -> dict:
    """Measure the launch shapes for this matrix and cache the fastest (smat_autotune)."""
    o = BcsrOpts()
    o.block_rows, o.block_cols = block
    perm = None if row_perm is None else np.ascontiguousarray(row_perm, np.int64)
    o.row_perm = None if perm is None else perm.ctypes.data
    o.device = device
    r = TuneResult()
    s = csr.struct()
    check(lib().smat_autotune(C.byref(s), C.byref(o), form, N, C.byref(r)))
    return {"panel_rows": r.panel_rows, "split_frac": r.split_frac, "ms": r.ms, "ms_default": r.ms_default,
            "cached": bool(r.cached), "n_tile_cols": r.n_tile_cols, "pipeline_depth": r.pipeline_depth,
            "candidates": r.candidates}


def features(csr: Csr, device: int = 0) -> np.ndarray:
    """The 64 matrix features of smat_features (computed on the GPU)."""
    out = np.zeros(64, np.float32)
    s = csr.struct()
    check(lib().smat_features(C.byref(s), device, out.ctypes.data))
    return out


class Group:
    """Many SpMMs in one persistent launch (smat_group_*). problems: list of
    (Bcsr, form, B, C) with torch CUDA tensors; B is (K, N) in either layout,
    C is (rows, N) row-major FP32 or FP16. The tensors must stay alive and in
    place while the group is used."""

    def __init__(self, problems):
        arr = (Problem * len(problems))()
        self._keep = []
        for i, (M, form, B, Cm) in enumerate(problems):
            layout, ld = _torch_layout(B)
            arr[i].A = M.handle.value if hasattr(M.handle, "value") else M.handle
            arr[i].form = form
            arr[i].B = B.data_ptr()
            arr[i].b_dtype = _torch_dt(B.dtype)
            arr[i].b_layout = layout
            arr[i].ldb = ld
            arr[i].C = Cm.data_ptr()
            arr[i].c_dtype = _torch_dt(Cm.dtype)
            arr[i].ldc = Cm.stride(0)
            arr[i].N = B.shape[1]
            self._keep.append((M, B, Cm))
        h = C.c_void_p()
        check(lib().smat_group_create(arr, len(problems), C.byref(h)))
        self._h = h

    def run(self, stream=0):
        check(lib().smat_group_run(self._h, stream))

    def check_device_error(self):
        check(lib().smat_group_check_device_error(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().smat_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TILE_KEYS = ("rowptr", "colidx", "val", "block_info", "rel_map", "tile_info")


class Tiles:
    """The reference's merged 4 x 4-block tiles (SparseMatrix::bcsrBlocking,
    src/cuda_hgemm/src/common/matrix.h:794-1137) built on the GPU from a
    device BCSR (smat_tiles_create): row_ptr, col_idx, values are torch CUDA
    tensors (int32, int32, FP16 or int16 of nnzb * 16 * block_cols) in the
    layout csrToBcsr leaves; rows and cols padded to the block shape."""

    def __init__(self, rows: int, cols: int, block_cols: int, row_ptr, col_idx, values, stream=0):
        h = C.c_void_p()
        check(lib().smat_tiles_create(int(rows), int(cols), int(block_cols), int(col_idx.numel()),
                                      row_ptr.data_ptr(), col_idx.data_ptr(), values.data_ptr(), stream,
                                      C.byref(h)))
        self._h = h
        d = TilesDesc()
        check(lib().smat_tiles_describe(h, C.byref(d)))
        self.desc = d
        self.n_tiles, self.n_rowptr = d.n_tiles, d.n_rowptr
        self.grid = (d.tile_rows, d.tile_cols)

    @property
    def handle(self):
        return self._h

    def to_host(self) -> dict:
        """The merged arrays on the host, keyed by TILE_KEYS (values as FP16
        bits, [n_tiles, 256 * block_cols])."""
        d, nt = self.desc, self.n_tiles
        cells = d.tile_rows * d.tile_cols
        out = {"rowptr": np.zeros(self.n_rowptr, np.int32), "colidx": np.zeros(max(nt, 1), np.int32),
               "val": np.zeros(max(nt, 1) * 256 * d.block_cols, np.uint16),
               "block_info": np.zeros(max(cells, 1), np.int32), "rel_map": np.zeros(max(cells, 1), np.int32),
               "tile_info": np.zeros(max(nt, 1) * 16, np.int32)}
        check(lib().smat_tiles_copy_to_host(self._h, *(out[k].ctypes.data for k in TILE_KEYS)))
        out["colidx"], out["tile_info"] = out["colidx"][:nt], out["tile_info"][: nt * 16]
        out["val"] = out["val"][: nt * 256 * d.block_cols].reshape(nt, 256 * d.block_cols)
        out["block_info"], out["rel_map"] = out["block_info"][:cells], out["rel_map"][:cells]
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().smat_tiles_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def partition_rows(csr: Csr, world: int, block_rows: int = 16):
    """1-D partition of the rows into `world` contiguous ranges of whole block
    rows, balanced by nonzeros: the natural sharding of the SpMM (each shard
    owns its rows of C; B is replicated; no exchange is needed)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    nbr = (csr.rows + block_rows - 1) // block_rows
    ends = np.minimum(np.arange(1, nbr + 1) * block_rows, csr.rows)
    cum = csr.row_ptr[ends]
    total = int(csr.row_ptr[-1])
    cuts = [0]
    for w in range(1, world):
        target = total * w / world
        b = int(np.searchsorted(cum, target, side="left"))
        cuts.append(max(cuts[-1], min(int(ends[b]) if b < nbr else csr.rows, csr.rows)))
    cuts.append(csr.rows)
    return [(cuts[i], cuts[i + 1]) for i in range(world)]


def row_slice(csr: Csr, r0: int, r1: int) -> Csr:
    """Rows [r0, r1) as their own CSR (same columns)."""
    a, b = int(csr.row_ptr[r0]), int(csr.row_ptr[r1])
    vals = None if csr.values is None else csr.values[a:b]
    return Csr(r1 - r0, csr.cols, csr.row_ptr[r0:r1 + 1] - a, csr.col_idx[a:b], vals)
