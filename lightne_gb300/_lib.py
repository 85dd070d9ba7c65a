"""ctypes binding of liblightne_gb300.so (the C ABI in include/lightne_gb300.h).

The shared library is the product: importing this module loads it and fails
loudly when it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblightne_gb300.so")

LNE_OK = 0
LNE_ERR_INVALID = 1
LNE_ERR_ALLOC = 2
LNE_ERR_TABLE_FULL = 3
LNE_ERR_CUDA = 4
LNE_ERR_UNSUPPORTED = 5
LNE_ERR_NUMERIC = 6

LNE_PREC_FP32 = 0
LNE_PREC_BF16 = 1
LNE_PREC_FP8 = 2
LNE_PREC_FP16 = 3

_STATUS_NAMES = {
    LNE_ERR_INVALID: "LNE_ERR_INVALID",
    LNE_ERR_ALLOC: "LNE_ERR_ALLOC",
    LNE_ERR_TABLE_FULL: "LNE_ERR_TABLE_FULL",
    LNE_ERR_CUDA: "LNE_ERR_CUDA",
    LNE_ERR_UNSUPPORTED: "LNE_ERR_UNSUPPORTED",
    LNE_ERR_NUMERIC: "LNE_ERR_NUMERIC",
}


class LneError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (%d): %s" % (_STATUS_NAMES.get(status, "LNE_ERR"), status, msg))
        self.status = status


class SparsifyParams(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("walk_len", ctypes.c_int64),
        ("table_size", ctypes.c_int64),
        ("negative", ctypes.c_int64),
        ("sample", ctypes.c_int32),
        ("upper", ctypes.c_int32),
        ("sample_ratio", ctypes.c_float),
        ("mem_ratio", ctypes.c_float),
    ]


class SparsifyStats(ctypes.Structure):
    _fields_ = [
        ("logn", ctypes.c_double),
        ("total_samples", ctypes.c_double),
        ("inv_lambda", ctypes.c_double),
        ("frac", ctypes.c_double),
        ("factor", ctypes.c_double),
        ("m_exact", ctypes.c_double),
        ("exp_rv_rounded", ctypes.c_int64),
        ("table_size", ctypes.c_int64),
        ("capacity", ctypes.c_int64),
        ("samples_emitted", ctypes.c_int64),
        ("distinct", ctypes.c_int64),
        ("nnz_upper", ctypes.c_int64),
        ("nnz", ctypes.c_int64),
        ("ms_sample", ctypes.c_float),
        ("ms_trunclog", ctypes.c_float),
        ("ms_csr", ctypes.c_float),
        ("kernel_launches", ctypes.c_int32),
        ("sliced", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RandsvdParams(ctypes.Structure):
    _fields_ = [
        ("rank", ctypes.c_int64),
        ("dim", ctypes.c_int64),
        ("normalize", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("random_project_only", ctypes.c_int32),
        ("sparse_project", ctypes.c_int32),
        ("sparse_project_s", ctypes.c_double),
    ]


class RandsvdStats(ctypes.Structure):
    _fields_ = [
        ("ms_sketch", ctypes.c_float),
        ("ms_qr", ctypes.c_float),
        ("ms_spmm2", ctypes.c_float),
        ("ms_core", ctypes.c_float),
        ("ms_total", ctypes.c_float),
        ("jacobi_sweeps", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int32),
        ("spmm_nnz", ctypes.c_double),
        ("jacobi_sweeps_fp32", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class PropagateParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int64),
        ("order", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("mu", ctypes.c_double),
        ("s", ctypes.c_double),
    ]


class PropagateStats(ctypes.Structure):
    _fields_ = [
        ("ms_total", ctypes.c_float),
        ("kernel_launches", ctypes.c_int32),
        ("spmm_calls", ctypes.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


VP = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int32
PVP = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes).  Every symbol include/lightne_gb300.h declares.
SIGNATURES = {
    "lne_last_error": (ctypes.c_char_p, []),
    "lne_version": (ctypes.c_char_p, []),
    "lne_ctx_create": (ctypes.c_int, [PVP, ctypes.c_int, VP]),
    "lne_ctx_destroy": (ctypes.c_int, [VP]),
    "lne_ctx_synchronize": (ctypes.c_int, [VP]),
    "lne_ctx_launch_count": (ctypes.c_int, [VP, ctypes.POINTER(I64)]),
    "lne_ctx_set_spmm_panel_bytes": (ctypes.c_int, [VP, I64]),
    "lne_ctx_set_sparsify_slices": (ctypes.c_int, [VP, I32, I32]),
    "lne_ctx_set_sparsify_batch": (ctypes.c_int, [VP, I64]),
    "lne_ctx_set_sparsify_rounds": (ctypes.c_int, [VP, I32, I32]),
    "lne_ctx_set_row_sort_window": (ctypes.c_int, [VP, I64]),
    "lne_ctx_set_core_svd_fp64": (ctypes.c_int, [VP, I32]),
    "lne_device_alloc": (ctypes.c_int, [VP, I64, PVP]),
    "lne_device_free": (ctypes.c_int, [VP, VP]),
    "lne_copy_to_host": (ctypes.c_int, [VP, VP, VP, I64]),
    "lne_copy_to_device": (ctypes.c_int, [VP, VP, VP, I64]),
    "lne_graph_upload": (ctypes.c_int, [VP, I64, VP, VP, PVP]),
    "lne_graph_upload_device": (ctypes.c_int, [VP, I64, VP, VP, PVP]),
    "lne_graph_free": (ctypes.c_int, [VP]),
    "lne_sparsify": (ctypes.c_int, [VP, VP, ctypes.POINTER(SparsifyParams), PVP, ctypes.POINTER(SparsifyStats)]),
    "lne_trunc_log_values": (ctypes.c_int, [VP, VP, I64, VP]),
    "lne_spmm": (ctypes.c_int, [VP, VP, ctypes.c_int, VP, I64, I64, ctypes.c_float, ctypes.c_float, VP, I64]),
    "lne_randsvd": (ctypes.c_int, [VP, VP, ctypes.POINTER(RandsvdParams), VP, VP, ctypes.POINTER(RandsvdStats)]),
    "lne_gaussian": (ctypes.c_int, [VP, ctypes.c_uint64, ctypes.c_uint64, I64, I64, VP, I64]),
    "lne_sparse_projection": (ctypes.c_int, [VP, ctypes.c_uint64, I64, I64, ctypes.c_double, VP, I64, VP]),
    "lne_ne_zhang_matrix": (ctypes.c_int, [VP, VP, VP]),
    "lne_propagate": (ctypes.c_int, [VP, VP, ctypes.POINTER(PropagateParams), VP, VP, VP,
                                     ctypes.POINTER(PropagateStats)]),
    "lne_propagate_adjoint": (ctypes.c_int, [VP, VP, ctypes.POINTER(PropagateParams), VP, VP, VP,
                                             ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(PropagateStats)]),
    "lne_chebyshev_coefficients": (ctypes.c_int, [ctypes.c_int32, ctypes.c_double, VP]),
    "lne_dense_embed": (ctypes.c_int, [VP, VP, I64, I64, VP, VP]),
    "lne_core_svd": (ctypes.c_int, [VP, VP, ctypes.c_int32, VP, VP, VP]),
    "lne_gram": (ctypes.c_int, [VP, VP, I64, I64, VP, I64, I64, I64, VP]),
    "lne_gemm_tall": (ctypes.c_int, [VP, VP, I64, I64, VP, I64, I64, VP, I64]),
    "lne_gram_noalloc": (ctypes.c_int, [VP, VP, I64, I64, VP, I64, I64, I64, VP]),
    "lne_csr_info": (ctypes.c_int, [VP, ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    "lne_csr_download": (ctypes.c_int, [VP, VP, VP, VP, VP]),
    "lne_csr_device_ptrs": (ctypes.c_int, [VP, PVP, PVP, PVP]),
    "lne_csr_wrap_device": (ctypes.c_int, [VP, I64, I64, VP, VP, VP, PVP]),
    "lne_csr_free": (ctypes.c_int, [VP]),
}

_lib = None


def load():
    """Load the library (once).  Raises ImportError if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("liblightne_gb300.so not found at %s: run `python -m lightne_gb300.build` "
                          "(the CUDA library is required; there is no CPU path)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != LNE_OK:
        raise LneError(status, load().lne_last_error().decode(errors="replace"))
