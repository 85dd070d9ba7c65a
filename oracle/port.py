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
        srcs = [os.path.join(_HERE, f) for f in ("sparsify_port.c", "spmm_port.c")]
        if not os.path.exists(path) or any(os.path.getmtime(path) < os.path.getmtime(s) for s in srcs):
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
        L.lne_port_session_create.restype = ctypes.c_void_p
        L.lne_port_session_create.argtypes = [ctypes.c_int64, I64P, I32P, ctypes.c_uint64, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_int, ctypes.c_int]
        L.lne_port_session_sample.restype = ctypes.c_int64
        L.lne_port_session_sample.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64]
        L.lne_port_session_finish.restype = ctypes.c_int
        L.lne_port_session_finish.argtypes = [ctypes.c_void_p, I64P, ctypes.POINTER(I32P), ctypes.POINTER(F32P),
                                              F64P]
        L.lne_port_session_free.restype = None
        L.lne_port_session_free.argtypes = [ctypes.c_void_p]
        for name, fp in (("lne_port_spmm_f32", F32P), ("lne_port_spmm_f64", F64P)):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [ctypes.c_int64, ctypes.c_int64, I64P, I32P, fp, fp, ctypes.c_int64, ctypes.c_int64, fp,
                           ctypes.c_int64, ctypes.c_int]
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


class Session:
    """The sparsifier in steps (oracle/sparsify_port.c lne_port_session_*):
    sample(u0, u1) runs the per-edge sampler over the out-edges of vertices
    [u0, u1); finish() builds the canonical CSR and returns it with the
    stats, as sparsify() does."""

    def __init__(self, off, nbrs, seed, walk_len=10, tablesz=0, negative=1, sample=0, sample_ratio=1.0,
                 mem_ratio=1.0, upper=0, nthreads=0):
        self.off = np.ascontiguousarray(off, dtype=np.int64)
        self.nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        self.n = self.off.size - 1
        self.h = lib().lne_port_session_create(self.n, self.off.ctypes.data_as(I64P),
                                               self.nbrs.ctypes.data_as(I32P), seed, walk_len, tablesz, negative,
                                               sample, sample_ratio, mem_ratio, upper, nthreads)
        if not self.h:
            raise MemoryError("oracle session: table allocation failed")

    def sample(self, u0, u1):
        got = lib().lne_port_session_sample(self.h, u0, u1)
        if got < 0:
            raise RuntimeError("oracle session: pair table full")
        return int(got)

    def finish(self):
        row_ptr = np.zeros(self.n + 1, dtype=np.int64)
        colp = I32P()
        valp = F32P()
        stats = (ctypes.c_double * 16)()
        rc = lib().lne_port_session_finish(self.h, row_ptr.ctypes.data_as(I64P), ctypes.byref(colp),
                                           ctypes.byref(valp), stats)
        self.h = None
        st = dict(zip(STAT_NAMES, list(stats)))
        if rc != 0:
            raise RuntimeError("oracle sparsify failed with status %d" % rc)
        nnz = int(row_ptr[-1])
        col = np.ctypeslib.as_array(colp, shape=(max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(valp, shape=(max(nnz, 1),))[:nnz].copy()
        lib().lne_port_free(ctypes.cast(colp, ctypes.c_void_p))
        lib().lne_port_free(ctypes.cast(valp, ctypes.c_void_p))
        return (row_ptr, col, val), st

    def free(self):
        if self.h:
            lib().lne_port_session_free(self.h)
            self.h = None

    def __del__(self):
        self.free()


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


def spmm(row_ptr, col, val, X, rows=None, out=None, nthreads=0):
    """Y = A X on the host cores for a CSR A (int64 row_ptr, int32 col) and a
    row-major dense X: FP32 when val and X are float32, FP64 when both are
    float64.  `rows` = (r0, r1) computes only those rows of `out`."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    X = np.ascontiguousarray(X)
    if X.dtype == np.float64:
        fn, fp, dt = lib().lne_port_spmm_f64, F64P, np.float64
    else:
        fn, fp, dt = lib().lne_port_spmm_f32, F32P, np.float32
    val = np.ascontiguousarray(val, dtype=dt)
    X = np.ascontiguousarray(X, dtype=dt)
    n = row_ptr.size - 1
    d = X.shape[1]
    if out is None:
        out = np.empty((n, d), dtype=dt)
    r0, r1 = rows if rows is not None else (0, n)
    fn(r0, r1, row_ptr.ctypes.data_as(I64P), col.ctypes.data_as(I32P), val.ctypes.data_as(fp),
       X.ctypes.data_as(fp), X.strides[0] // X.itemsize, d, out.ctypes.data_as(fp), out.strides[0] // out.itemsize,
       nthreads)
    return out
