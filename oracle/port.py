"""ctypes binding of oracle/sparsify_port.c (the C restatement of the
reference sparsifier).  Test infrastructure only."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

I64P = ctypes.POINTER(ctypes.c_int64)
I32P = ctypes.POINTER(ctypes.c_int32)
F32P = ctypes.POINTER(ctypes.c_float)
F64P = ctypes.POINTER(ctypes.c_double)

STAT_NAMES = ["logn", "M", "inv_lambda", "exp_rv_rounded", "frac", "table_size", "capacity",
              "samples", "M_exact", "factor", "nnz_upper", "nnz", "sec_sample", "sec_csr",
              "threads", "distinct"]


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
    return os.path.join(_HERE, "_build", "libsparsify_port.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "libsparsify_port.so")
        src = os.path.join(_HERE, "sparsify_port.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        L.lne_port_hash64_2.restype = ctypes.c_uint64
        L.lne_port_hash64_2.argtypes = [ctypes.c_uint64]
        L.lne_port_map_uint64.restype = ctypes.c_double
        L.lne_port_map_uint64.argtypes = [ctypes.c_uint64]
        L.lne_port_params.restype = None
        L.lne_port_params.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_float, ctypes.c_float, F64P]
        L.lne_port_sparsify.restype = ctypes.c_int
        L.lne_port_sparsify.argtypes = [ctypes.c_int64, I64P, I32P, ctypes.c_uint64, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_int, ctypes.c_int, I64P,
                                        ctypes.POINTER(I32P), ctypes.POINTER(F32P), F64P]
        L.lne_port_sample_range.restype = ctypes.c_int64
        L.lne_port_sample_range.argtypes = [ctypes.c_int64, I64P, I32P, ctypes.c_uint64, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_int64, ctypes.c_int64, ctypes.c_int, F64P]
        L.lne_port_free.restype = None
        L.lne_port_free.argtypes = [ctypes.c_void_p]
        _LIB = L
    return _LIB


def hash64_2(x: int) -> int:
    return lib().lne_port_hash64_2(x)


def params(n, m_dir, walk_len, tablesz, sample_ratio, mem_ratio) -> dict:
    out = (ctypes.c_double * 7)()
    lib().lne_port_params(n, m_dir, walk_len, tablesz, sample_ratio, mem_ratio, out)
    return dict(zip(STAT_NAMES[:7], list(out)))


def sparsify(off, nbrs, seed, walk_len=10, tablesz=0, negative=1, sample=0, sample_ratio=1.0,
             mem_ratio=1.0, upper=0, nthreads=0):
    """Canonical CSR (row_ptr int64, col int32, val float32) and stats dict."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
    n = off.size - 1
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    colp = I32P()
    valp = F32P()
    stats = (ctypes.c_double * 16)()
    rc = lib().lne_port_sparsify(n, off.ctypes.data_as(I64P), nbrs.ctypes.data_as(I32P), seed,
                                 walk_len, tablesz, negative, sample, sample_ratio, mem_ratio, upper,
                                 nthreads, row_ptr.ctypes.data_as(I64P), ctypes.byref(colp),
                                 ctypes.byref(valp), stats)
    st = dict(zip(STAT_NAMES, list(stats)))
    if rc != 0:
        raise RuntimeError("oracle sparsify failed with status %d" % rc)
    nnz = int(row_ptr[-1])
    col = np.ctypeslib.as_array(colp, shape=(max(nnz, 1),))[:nnz].copy()
    val = np.ctypeslib.as_array(valp, shape=(max(nnz, 1),))[:nnz].copy()
    lib().lne_port_free(ctypes.cast(colp, ctypes.c_void_p))
    lib().lne_port_free(ctypes.cast(valp, ctypes.c_void_p))
    return (row_ptr, col, val), st


def sample_range(off, nbrs, seed, e_begin, e_end, walk_len=10, tablesz=0, sample=0,
                 sample_ratio=1.0, mem_ratio=1.0, nthreads=0):
    """Sampler + table insert over directed edges [e_begin, e_end): returns
    (samples emitted, seconds)."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
    sec = ctypes.c_double()
    got = lib().lne_port_sample_range(off.size - 1, off.ctypes.data_as(I64P),
                                      nbrs.ctypes.data_as(I32P), seed, walk_len, tablesz, sample,
                                      sample_ratio, mem_ratio, e_begin, e_end, nthreads,
                                      ctypes.byref(sec))
    if got < 0:
        raise RuntimeError("oracle sample_range failed (%d)" % got)
    return int(got), sec.value
