"""TEST INFRASTRUCTURE ONLY — ctypes front end of the CPU oracle.

Loads ``oracle/_build/libsmat_oracle.so`` (the restatement in
``smat_oracle.cpp``) and, where it was built, the reference's own code in
``oracle/_ref/`` (``ref_preprocess_shim.cpp``, ``ref_bcsr_shim.cu``).
Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")

_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(ref: bool = False) -> None:
    """Compile the oracle (and, if asked and available, the reference build)."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


_lib = None
_ref_pre = None
_ref_bcsr = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(BUILD, "libsmat_oracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_jaccard_group.restype = C.c_float
        L.orc_jaccard_group.argtypes = [_i64p, C.c_int64, C.c_int64, _i64p, C.c_int64, C.c_int64, C.c_int64]
        L.orc_merge_rows.restype = C.c_int64
        L.orc_merge_rows.argtypes = [_i64p, C.c_int64, _i64p, C.c_int64, _i64p]
        L.orc_keeper_grouping.restype = None
        L.orc_keeper_grouping.argtypes = [C.c_int64, _i64p, _i64p, C.c_float, C.c_int64, C.c_int64, _i64p, _i64p]
        L.orc_permutation.restype = None
        L.orc_permutation.argtypes = [_i64p, C.c_int64, _i64p]
        L.orc_fixed_size_grouping.restype = None
        L.orc_fixed_size_grouping.argtypes = [_i64p, C.c_int64, C.c_int64, _i64p]
        L.orc_reorder.restype = None
        L.orc_reorder.argtypes = [C.c_int64, _i64p, _i64p, C.c_float, C.c_int64, C.c_int64, C.c_int,
                                  _i64p, _i64p, _i64p]
        L.orc_csr_to_bcsr.restype = C.c_int64
        L.orc_csr_to_bcsr.argtypes = [C.c_int64, C.c_int64, C.c_int, _i32p, _i32p, _u16p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_bcsr_blocking.restype = C.c_int64
        L.orc_bcsr_blocking.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int64, _i32p, _i32p, _u16p,
                                        C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
        L.orc_is_block_24.restype = C.c_int
        L.orc_is_block_24.argtypes = [_u16p, C.c_int, C.c_int]
        L.orc_spmm_f64.restype = None
        L.orc_spmm_f64.argtypes = [C.c_int64, C.c_int64, _i64p, _i64p, _f64p, _f64p, C.c_int64, C.c_int64,
                                   _f64p, C.c_int64, C.c_int64]
        L.orc_csr_multiply_f32_range.restype = None
        L.orc_csr_multiply_f32_range.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, C.c_int64, C.c_void_p]
        L.orc_csr_multiply_f32.restype = None
        L.orc_csr_multiply_f32.argtypes = [C.c_int64, _i64p, _i64p, _f32p, _f32p, C.c_int64, _f32p]
        _lib = L
    return _lib


def reference_dir():
    """The reference source tree: $SMAT_REFERENCE, else the one the last
    oracle build compiled from (oracle/_ref/source_dir.txt); None when
    neither names an existing directory."""
    d = os.environ.get("SMAT_REFERENCE")
    if not d:
        p = os.path.join(REFDIR, "source_dir.txt")
        if os.path.exists(p):
            with open(p) as f:
                d = f.read().strip()
    return d if d and os.path.isdir(d) else None


def ref_available() -> bool:
    return os.path.exists(os.path.join(REFDIR, "libsmat_ref_preprocess.so"))


def ref_pre():
    global _ref_pre
    if _ref_pre is None:
        L = C.CDLL(os.path.join(REFDIR, "libsmat_ref_preprocess.so"))
        L.ref_jaccard_group.restype = C.c_float
        L.ref_jaccard_group.argtypes = [_i64p, C.c_int64, C.c_int64, _i64p, C.c_int64, C.c_int64, C.c_int64]
        L.ref_hamming_group.restype = C.c_float
        L.ref_hamming_group.argtypes = [_i64p, C.c_int64, C.c_int64, _i64p, C.c_int64, C.c_int64, C.c_int64]
        L.ref_merge_rows.restype = C.c_int64
        L.ref_merge_rows.argtypes = [_i64p, C.c_int64, _i64p, C.c_int64, _i64p]
        L.ref_reorder.restype = None
        L.ref_reorder.argtypes = [C.c_int64, C.c_int64, _i64p, _i64p, C.c_float, C.c_int64, C.c_int64, C.c_int,
                                  C.c_int, _i64p, _i64p, _i64p]
        L.ref_csr_multiply.restype = None
        L.ref_csr_multiply.argtypes = [C.c_int64, C.c_int64, _i64p, _i64p, _f32p, _f32p, C.c_int64, _f32p]
        L.ref_read_el.restype = C.c_int64
        L.ref_read_el.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.POINTER(C.c_int64)),
                                  C.POINTER(C.POINTER(C.c_int64)), C.POINTER(C.POINTER(C.c_float))]
        L.ref_pre_free.restype = None
        L.ref_pre_free.argtypes = [C.c_void_p]
        L.ref_csr_reorder_rows.restype = None
        L.ref_csr_reorder_rows.argtypes = [C.c_int64, C.c_int64, _i64p, _i64p, _f32p, _i64p, _i64p, _i64p, _f32p]
        _ref_pre = L
    return _ref_pre


class _RefBcsr(C.Structure):
    _fields_ = [("nnzb", C.c_int64), ("grid", C.c_int64),
                ("rowptr", C.POINTER(C.c_int32)), ("colidx", C.POINTER(C.c_int32)),
                ("val", C.POINTER(C.c_uint16)), ("block_info", C.POINTER(C.c_int32)),
                ("rel_map", C.POINTER(C.c_int32))]


class _RefTiles(C.Structure):
    _fields_ = [("ntiles", C.c_int64), ("n_rowptr", C.c_int64), ("grid", C.c_int64),
                ("rowptr", C.POINTER(C.c_int32)), ("colidx", C.POINTER(C.c_int32)),
                ("val", C.POINTER(C.c_uint16)), ("block_info", C.POINTER(C.c_int32)),
                ("rel_map", C.POINTER(C.c_int32)), ("tile_info", C.POINTER(C.c_int32))]


def ref_bcsr_lib():
    global _ref_bcsr
    if _ref_bcsr is None:
        L = C.CDLL(os.path.join(REFDIR, "libsmat_ref_bcsr.so"))
        L.ref_bcsr_blocking.restype = C.POINTER(_RefTiles)
        L.ref_bcsr_blocking.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int64, _i32p, _i32p, _u16p]
        L.ref_tiles_free.restype = None
        L.ref_tiles_free.argtypes = [C.POINTER(_RefTiles)]
        L.ref_csr_to_bcsr.restype = C.POINTER(_RefBcsr)
        L.ref_csr_to_bcsr.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int64, _i32p, _i32p, _u16p]
        L.ref_bcsr_free.restype = None
        L.ref_bcsr_free.argtypes = [C.POINTER(_RefBcsr)]
        L.ref_read_mtx.restype = C.c_int
        L.ref_read_mtx.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int),
                                   C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_int32)),
                                   C.POINTER(C.POINTER(C.c_uint16))]
        L.ref_free.restype = None
        L.ref_free.argtypes = [C.c_void_p]
        _ref_bcsr = L
    return _ref_bcsr


# ----------------------------------------------------------------------------- oracle wrappers

def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def jaccard_group(a, ga, b, gb, bs, ref=False):
    a, b = _i64(a), _i64(b)
    L = ref_pre() if ref else lib()
    f = L.ref_jaccard_group if ref else L.orc_jaccard_group
    return float(np.float32(f(a, len(a), ga, b, len(b), gb, bs)))


def merge_rows(a, b, ref=False):
    a, b = _i64(a), _i64(b)
    out = np.zeros(len(a) + len(b) + 1, np.int64)
    L = ref_pre() if ref else lib()
    f = L.ref_merge_rows if ref else L.orc_merge_rows
    n = f(a, len(a), b, len(b), out)
    return out[:n].copy()


def keeper_grouping(rowptr, cols, tau, col_block, max_row_block):
    rowptr, cols = _i64(rowptr), _i64(cols)
    rows = len(rowptr) - 1
    g = np.zeros(rows, np.int64)
    st = np.zeros(2, np.int64)
    lib().orc_keeper_grouping(rows, rowptr, cols, tau, col_block, max_row_block, g, st)
    return g, st


def reorder(rowptr, cols, tau, col_block, row_block, force_fixed=True):
    """Oracle of the whole reorder step: returns (perm, grouping, stats)."""
    rowptr, cols = _i64(rowptr), _i64(cols)
    rows = len(rowptr) - 1
    perm = np.zeros(rows, np.int64)
    g = np.zeros(rows, np.int64)
    st = np.zeros(2, np.int64)
    lib().orc_reorder(rows, rowptr, cols, tau, col_block, row_block, 1 if force_fixed else 0, perm, g, st)
    return perm, g, st


def ref_reorder(rowptr, cols, n_cols, tau, col_block, row_block, algo=5, force_fixed=True):
    """The reference's own BlockingEngine run in-process: (perm, grouping, stats)."""
    rowptr, cols = _i64(rowptr), _i64(cols)
    rows = len(rowptr) - 1
    perm = np.zeros(rows, np.int64)
    g = np.zeros(rows, np.int64)
    st = np.zeros(5, np.int64)
    ref_pre().ref_reorder(rows, n_cols, rowptr, cols, tau, col_block, row_block, algo,
                          1 if force_fixed else 0, g, perm, st)
    return perm, g, st


def permutation(grouping):
    g = _i64(grouping)
    p = np.zeros(len(g), np.int64)
    lib().orc_permutation(g, len(g), p)
    return p


def csr_to_bcsr(m_row, m_col, k, rowptr, colidx, val_f16):
    """Oracle of SparseMatrix::csrToBcsr: (rowptr, colidx, values[nnzb,16,k] fp16, block_info)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    vbits = np.ascontiguousarray(np.asarray(val_f16, np.float16).view(np.uint16))
    L = lib()
    nnzb = L.orc_csr_to_bcsr(m_row, m_col, k, rowptr, colidx, vbits, None, None, None, None)
    brp = np.zeros(m_row // 16 + 1, np.int32)
    bci = np.zeros(max(nnzb, 1), np.int32)
    bv = np.zeros(max(nnzb, 1) * 16 * k, np.uint16)
    grid = ((m_row + 15) // 16) * ((m_col + k - 1) // k)
    info = np.zeros(max(grid, 1), np.int32)
    L.orc_csr_to_bcsr(m_row, m_col, k, rowptr, colidx, vbits, brp.ctypes.data, bci.ctypes.data,
                      bv.ctypes.data, info.ctypes.data)
    return brp, bci[:nnzb], bv[: nnzb * 16 * k].view(np.float16).reshape(nnzb, 16, k), info[:grid]


def ref_csr_to_bcsr(m_row, m_col, k, rowptr, colidx, val_f16):
    """The reference's own csrToBcsr (matrix.h:666-792), run on the CPU."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    vbits = np.ascontiguousarray(np.asarray(val_f16, np.float16).view(np.uint16))
    L = ref_bcsr_lib()
    p = L.ref_csr_to_bcsr(m_row, m_col, k, len(colidx), rowptr, colidx, vbits)
    b = p.contents
    nnzb, grid = b.nnzb, b.grid
    brp = np.ctypeslib.as_array(b.rowptr, shape=(m_row // 16 + 1,)).copy()
    bci = np.ctypeslib.as_array(b.colidx, shape=(max(nnzb, 1),))[:nnzb].copy()
    bv = np.ctypeslib.as_array(b.val, shape=(max(nnzb, 1) * 16 * k,))[: nnzb * 16 * k].copy()
    info = np.ctypeslib.as_array(b.block_info, shape=(max(grid, 1),))[:grid].copy()
    L.ref_bcsr_free(p)
    return brp, bci, bv.view(np.float16).reshape(nnzb, 16, k), info


TILE_KEYS = ("rowptr", "colidx", "val", "block_info", "rel_map", "tile_info")


def bcsr_blocking(m_row, m_col, k, brp, bci, bval_f16):
    """Oracle of SparseMatrix::bcsrBlocking (matrix.h:794-1137): the 4 x 4-block
    merged tiles of a BCSR, as a dict of TILE_KEYS (values as FP16 bits,
    [ntiles, 256 * k])."""
    brp = np.ascontiguousarray(brp, np.int32)
    bci = np.ascontiguousarray(bci, np.int32)
    vb = np.ascontiguousarray(np.asarray(bval_f16, np.float16).view(np.uint16)).reshape(-1)
    L = lib()
    nnzb = len(bci)
    nrp = C.c_int64()
    nt = L.orc_bcsr_blocking(m_row, m_col, k, nnzb, brp, bci, vb, C.byref(nrp), None, None, None, None, None,
                             None)
    grid = ((m_row + 63) // 64) * ((m_col + 4 * k - 1) // (4 * k))
    out = {"rowptr": np.zeros(nrp.value, np.int32), "colidx": np.zeros(max(nt, 1), np.int32),
           "val": np.zeros(max(nt, 1) * 256 * k, np.uint16), "block_info": np.zeros(max(grid, 1), np.int32),
           "rel_map": np.zeros(max(grid, 1), np.int32), "tile_info": np.zeros(max(nt, 1) * 16, np.int32)}
    L.orc_bcsr_blocking(m_row, m_col, k, nnzb, brp, bci, vb, C.byref(nrp), *(out[n].ctypes.data for n in TILE_KEYS))
    out["colidx"], out["tile_info"] = out["colidx"][:nt], out["tile_info"][: nt * 16]
    out["val"] = out["val"][: nt * 256 * k].reshape(nt, 256 * k)
    out["block_info"], out["rel_map"] = out["block_info"][:grid], out["rel_map"][:grid]
    return out


def ref_bcsr_blocking(m_row, m_col, k, brp, bci, bval_f16):
    """The reference's own bcsrBlocking, run on the CPU (same dict as bcsr_blocking)."""
    brp = np.ascontiguousarray(brp, np.int32)
    bci = np.ascontiguousarray(bci, np.int32)
    vb = np.ascontiguousarray(np.asarray(bval_f16, np.float16).view(np.uint16)).reshape(-1)
    L = ref_bcsr_lib()
    p = L.ref_bcsr_blocking(m_row, m_col, k, len(bci), brp, bci, vb)
    t = p.contents
    nt, nrp, grid = t.ntiles, t.n_rowptr, t.grid
    take = lambda ptr, n: np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].copy()
    out = {"rowptr": take(t.rowptr, nrp), "colidx": take(t.colidx, nt),
           "val": take(t.val, nt * 256 * k).reshape(nt, 256 * k), "block_info": take(t.block_info, grid),
           "rel_map": take(t.rel_map, grid), "tile_info": take(t.tile_info, nt * 16)}
    L.ref_tiles_free(p)
    return out


def spmm_f64(rowptr, colidx, val, B):
    """FP64 product C = A @ B, A in CSR, B a (K, N) array (any layout)."""
    rowptr, colidx = _i64(rowptr), _i64(colidx)
    val = np.ascontiguousarray(val, np.float64)
    B = np.asarray(B, np.float64)
    Bc = np.ascontiguousarray(B)
    rows = len(rowptr) - 1
    N = Bc.shape[1]
    Cm = np.zeros((rows, N), np.float64)
    lib().orc_spmm_f64(rows, N, rowptr, colidx, val, Bc, N, 1, Cm, N, 1)
    return Cm


def csr_multiply_f32(rowptr, colidx, val, B_colmajor, b_cols, rows):
    """Restatement of CSR::multiply; B, C column-major with ld = rows."""
    C_ = np.zeros(rows * b_cols, np.float32)
    lib().orc_csr_multiply_f32(rows, _i64(rowptr), _i64(colidx), np.ascontiguousarray(val, np.float32),
                               np.ascontiguousarray(B_colmajor, np.float32), b_cols, C_)
    return C_


def ref_csr_multiply(rowptr, colidx, val, n_cols, B_colmajor, b_cols, rows):
    """The reference's CSR::multiply itself (oracle/_ref)."""
    C_ = np.zeros(rows * b_cols, np.float32)
    Bc = np.ascontiguousarray(B_colmajor, np.float32).copy()
    ref_pre().ref_csr_multiply(rows, n_cols, _i64(rowptr), _i64(colidx),
                               np.ascontiguousarray(val, np.float32), Bc, b_cols, C_)
    return C_


def is_block_24(blk):
    b = np.ascontiguousarray(np.asarray(blk, np.float16).view(np.uint16))
    return bool(lib().orc_is_block_24(b, b.shape[0], b.shape[1]))


def csr_multiply_f32_range(ld, r0, r1, rowptr, colidx, val, B_colmajor, b_cols, C_colmajor):
    """CSR::multiply's loop over rows [r0, r1); arrays must stay alive (raw pointers)."""
    lib().orc_csr_multiply_f32_range(ld, r0, r1, rowptr.ctypes.data, colidx.ctypes.data, val.ctypes.data,
                                     B_colmajor.ctypes.data, b_cols, C_colmajor.ctypes.data)


def ref_read_mtx(path, k=16):
    """The reference's mmio_allinone (mmio_highlevel.h:523-680) on a file:
    (rows, cols, symmetric, rowptr int32, colidx int32, values as FP16 bits)."""
    L = ref_bcsr_lib()
    m, n, z = C.c_int64(), C.c_int64(), C.c_int64()
    sym = C.c_int()
    rp, ci, v = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)(), C.POINTER(C.c_uint16)()
    rc = L.ref_read_mtx(os.fsencode(path), k, C.byref(m), C.byref(n), C.byref(z), C.byref(sym), C.byref(rp),
                        C.byref(ci), C.byref(v))
    if rc != 0:
        raise RuntimeError(f"reference mmio_allinone failed: {rc}")
    try:
        rowptr = np.ctypeslib.as_array(rp, (m.value + 1,)).copy()
        colidx = np.ctypeslib.as_array(ci, (z.value,)).copy() if z.value else np.zeros(0, np.int32)
        vals = np.ctypeslib.as_array(v, (z.value,)).copy() if z.value else np.zeros(0, np.uint16)
    finally:
        for p in (rp, ci, v):
            L.ref_free(C.cast(p, C.c_void_p))
    return m.value, n.value, sym.value, rowptr, colidx, vals


def ref_read_el(path, pattern_only=False):
    """The reference's CSR::read_from_edgelist (csr.cpp:166-290) on a file:
    (rows, cols, rowptr int64, colidx int64, values float32), or None if it threw."""
    L = ref_pre()
    cols = C.c_int64()
    rp, ci, v = C.POINTER(C.c_int64)(), C.POINTER(C.c_int64)(), C.POINTER(C.c_float)()
    rows = L.ref_read_el(os.fsencode(path), 1 if pattern_only else 0, C.byref(cols), C.byref(rp), C.byref(ci),
                         C.byref(v))
    if rows < 0:
        return None
    try:
        rowptr = np.ctypeslib.as_array(rp, (rows + 1,)).copy()
        nnz = int(rowptr[-1])
        colidx = np.ctypeslib.as_array(ci, (nnz,)).copy() if nnz else np.zeros(0, np.int64)
        vals = np.ctypeslib.as_array(v, (nnz,)).copy() if nnz else np.zeros(0, np.float32)
    finally:
        for p in (rp, ci, v):
            L.ref_pre_free(C.cast(p, C.c_void_p))
    return rows, cols.value, rowptr, colidx, vals
