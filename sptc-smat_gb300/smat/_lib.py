"""ctypes binding of libsmat (include/smat.h)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libsmat.so")

SMAT_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "UNSUPPORTED", 3: "CUDA", 4: "NOMEM", 5: "TIMEOUT", 6: "NO_DEVICE"}

F32, F16, BF16, F64, E4M3 = 0, 1, 2, 3, 4
FORM_F16, FORM_BF16, FORM_FP8, FORM_SPLIT_BF16 = 0, 1, 2, 3
ROW_MAJOR, COL_MAJOR = 0, 1


class SmatError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"smat {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class CsrStruct(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("values", C.c_void_p),
                ("values_dtype", C.c_int32)]


class BcsrOpts(C.Structure):
    _fields_ = [("block_rows", C.c_int32), ("block_cols", C.c_int32), ("forms", C.c_uint32),
                ("use_24", C.c_int32), ("row_perm", C.c_void_p), ("device", C.c_int32),
                ("panel_rows", C.c_int32), ("split_frac", C.c_float), ("col_perm", C.c_void_p),
                ("n_tile_cols", C.c_int32), ("pipeline_depth", C.c_int32)]


class CsrFile(C.Structure):
    _fields_ = [("csr", CsrStruct), ("symmetric", C.c_int32)]


class Problem(C.Structure):
    _fields_ = [("A", C.c_void_p), ("form", C.c_int32), ("B", C.c_void_p), ("b_dtype", C.c_int32),
                ("b_layout", C.c_int32), ("ldb", C.c_int64), ("C", C.c_void_p), ("c_dtype", C.c_int32),
                ("ldc", C.c_int64), ("N", C.c_int64)]


class TuneResult(C.Structure):
    _fields_ = [("panel_rows", C.c_int32), ("split_frac", C.c_float), ("ms", C.c_double),
                ("ms_default", C.c_double), ("cached", C.c_int32), ("n_tile_cols", C.c_int32),
                ("pipeline_depth", C.c_int32), ("candidates", C.c_int32)]


class BcsrInfo(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("rows_padded", C.c_int64),
                ("cols_padded", C.c_int64), ("nnz", C.c_int64), ("nnzb", C.c_int64),
                ("n_blocks_24", C.c_int64), ("block_rows", C.c_int32), ("block_cols", C.c_int32),
                ("panel_rows", C.c_int32), ("n_panels", C.c_int32), ("n_union_cols", C.c_int64),
                ("fill", C.c_double), ("n_tile_cols", C.c_int32), ("pipeline_depth", C.c_int32)]


class TilesDesc(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("block_cols", C.c_int32), ("device", C.c_int32),
                ("n_tiles", C.c_int64), ("n_rowptr", C.c_int64), ("tile_rows", C.c_int64),
                ("tile_cols", C.c_int64), ("values", C.c_void_p), ("row_ptr", C.c_void_p),
                ("col_idx", C.c_void_p), ("block_info", C.c_void_p), ("rel_map", C.c_void_p),
                ("tile_info", C.c_void_p)]


class ReorderStats(C.Structure):
    _fields_ = [("comparisons", C.c_int64), ("merges", C.c_int64)]


# every symbol include/smat.h declares, with its ctypes signature
_SIGS = {
    "smat_read_mtx": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(CsrFile)]),
    "smat_read_el": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(CsrFile)]),
    "smat_write_el": (C.c_int, [C.c_char_p, C.POINTER(CsrStruct), C.c_void_p]),
    "smat_csr_file_free": (C.c_int, [C.POINTER(CsrFile)]),
    "smat_reorder": (C.c_int, [C.POINTER(CsrStruct), C.c_float, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                               C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(ReorderStats)]),
    "smat_bcsr_create": (C.c_int, [C.POINTER(CsrStruct), C.POINTER(BcsrOpts), C.POINTER(C.c_void_p)]),
    "smat_bcsr_create_from_bcsr": (C.c_int, [C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.POINTER(BcsrOpts), C.POINTER(C.c_void_p)]),
    "smat_bcsr_destroy": (C.c_int, [C.c_void_p]),
    "smat_bcsr_export_fp8": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "smat_bcsr_get_info": (C.c_int, [C.c_void_p, C.POINTER(BcsrInfo)]),
    "smat_bcsr_export": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "smat_csr_to_bcsr_host": (C.c_int, [C.POINTER(CsrStruct), C.c_int32, C.c_int32, C.c_void_p,
                                         C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p]),
    "smat_csr_to_bcsr_split_host": (C.c_int, [C.POINTER(CsrStruct), C.c_int32, C.c_void_p, C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p]),
    "smat_tiles_create": (C.c_int, [C.c_int64, C.c_int64, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.POINTER(C.c_void_p)]),
    "smat_tiles_describe": (C.c_int, [C.c_void_p, C.POINTER(TilesDesc)]),
    "smat_tiles_copy_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "smat_tiles_destroy": (C.c_int, [C.c_void_p]),
    "smat_spmm_workspace_size": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_size_t)]),
    "smat_spmm": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                            C.c_int32, C.c_int64, C.c_int64, C.c_void_p, C.c_size_t, C.c_void_p]),
    "smat_spmm_pack_b": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_int64,
                                   C.c_void_p, C.c_size_t, C.c_void_p]),
    "smat_spmm_packed": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_int64,
                                   C.c_void_p]),
    "smat_spmm_static_scratch": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int64,
                                           C.c_void_p, C.c_int32, C.c_int64, C.c_int64, C.c_void_p]),
    "smat_autotune": (C.c_int, [C.POINTER(CsrStruct), C.POINTER(BcsrOpts), C.c_int32, C.c_int64,
                                C.POINTER(TuneResult)]),
    "smat_autotune_clear": (C.c_int, []),
    "smat_features": (C.c_int, [C.POINTER(CsrStruct), C.c_int32, C.c_void_p]),
    "smat_mlp_create": (C.c_int, [C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "smat_mlp_num_params": (C.c_int32, []),
    "smat_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smat_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smat_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_void_p]),
    "smat_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float,
                                      C.c_void_p]),
    "smat_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "smat_mlp_destroy": (C.c_int, [C.c_void_p]),
    "smat_group_create": (C.c_int, [C.POINTER(Problem), C.c_int32, C.POINTER(C.c_void_p)]),
    "smat_group_run": (C.c_int, [C.c_void_p, C.c_void_p]),
    "smat_group_check_device_error": (C.c_int, [C.c_void_p]),
    "smat_group_destroy": (C.c_int, [C.c_void_p]),
    "smat_spmm_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                                 C.c_int32, C.c_int64, C.c_int64, C.c_void_p]),
    "smat_bcsr_check_device_error": (C.c_int, [C.c_void_p]),
    "smat_bcsr_set_wait_limit": (C.c_int, [C.c_void_p, C.c_uint64]),
    "smat_bcsr_debug_stall": (C.c_int, [C.c_void_p, C.c_int32]),
    "smat_ref_shims_last_status": (C.c_int, []),
    "smat_ref_shims_release": (C.c_int, []),
    "smat_last_error": (C.c_char_p, []),
    "smat_version": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load libsmat.so (building it first if it is missing). Raises if it cannot load."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("smat_build", os.path.join(PKG_ROOT, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != SMAT_OK:
        raise SmatError(status, lib().smat_last_error().decode())


def ptr(a) -> int:
    """Address of a numpy array, a torch tensor, or an int."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


# The reference's kernel launchers (C++ linkage, include/smat_ref_shims.h), by
# their Itanium-mangled names, with ctypes signatures.
_HP, _IP, _SZ = C.c_void_p, C.c_void_p, C.c_size_t
REF_SHIMS = {
    "mmaOBTKernel": ("_Z12mmaOBTKernelP6__halfPiS1_S0_S0_mmmmS1_S1_",
                     [_HP, _IP, _IP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "mmaOBTKernel_large": ("_Z18mmaOBTKernel_largeP6__halfPiS1_S0_S0_mmmmS1_S1_",
                           [_HP, _IP, _IP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "mmaOBTSKernel": ("_Z13mmaOBTSKernelP6__halfPiS1_PcS0_S0_S0_mmmmS1_S1_",
                      [_HP, _IP, _IP, C.c_void_p, _HP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "mmaOBTSKernel_large": ("_Z19mmaOBTSKernel_largeP6__halfPiS1_PcS0_S0_S0_mmmmS1_S1_",
                            [_HP, _IP, _IP, C.c_void_p, _HP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "mmaOBTSKernel_large_separate": ("_Z28mmaOBTSKernel_large_separateP6__halfPiS1_S0_S1_S1_PcS0_S0_S0_mmmmS1_S1_",
                                     [_HP, _IP, _IP, _HP, _IP, _IP, C.c_void_p, _HP, _HP, _HP, _SZ, _SZ, _SZ, _SZ,
                                      _IP, _IP]),
    "mmaOBTKernel_tiled": ("_Z18mmaOBTKernel_tiledP6__halfPiS1_S0_S0_mmmmS1_S1_",
                           [_HP, _IP, _IP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "mmaOBTSKernel_tiled_large": ("_Z25mmaOBTSKernel_tiled_largeP6__halfPiS1_PcS0_S0_S0_mmmmS1_S1_S1_",
                                  [_HP, _IP, _IP, C.c_void_p, _HP, _HP, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP, _IP]),
    "preprocessing_mmaSTKernel": ("_Z25preprocessing_mmaSTKernelP6__halfPcS0_mmmmPiS2_",
                                  [_HP, C.c_void_p, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
    "preprocessing_mmaSTKernel_large": ("_Z31preprocessing_mmaSTKernel_largeP6__halfPcS0_mmmmPiS2_",
                                        [_HP, C.c_void_p, _HP, _SZ, _SZ, _SZ, _SZ, _IP, _IP]),
}


def ref_shim(name):
    """A reference launcher exported by libsmat, callable through ctypes."""
    mangled, args = REF_SHIMS[name]
    f = getattr(lib(), mangled)
    f.restype = None
    f.argtypes = args
    return f
