"""Host-side mirror of LightNE's in-process interface over the C ABI.

Names and argument meaning follow the reference
(``LightNE/PathEmbed.h``, ``LightNE/mklredsvd/mklredsvd.h``,
``LightNE/SpectralPropagation.h``); errors are raised as :class:`LneError`
with the library's status instead of the reference's ``assert``/``exit(0)``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import LneError, SparsifyParams, SparsifyStats, check

__all__ = ["Context", "Graph", "CSR", "generate_trunc_log_matrix_v2", "LneError"]


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """Device + stream.  ``stream`` is a raw cudaStream_t (int) or None."""

    def __init__(self, device: int = 0, stream: int | None = None):
        L = _lib.load()
        h = ctypes.c_void_p()
        check(L.lne_ctx_create(ctypes.byref(h), device, ctypes.c_void_p(stream or 0)))
        self.handle = h
        self.device = device

    def synchronize(self) -> None:
        check(_lib.load().lne_ctx_synchronize(self.handle))

    def close(self) -> None:
        if self.handle:
            _lib.load().lne_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Graph:
    """Symmetric CSR graph resident on the device (neighbour order kept)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p, n: int, m_dir: int):
        self.ctx = ctx
        self.handle = handle
        self.n = n
        self.m_dir = m_dir

    @classmethod
    def from_numpy(cls, ctx: Context, offsets: np.ndarray, nbrs: np.ndarray) -> "Graph":
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nb = np.ascontiguousarray(nbrs, dtype=np.int32)
        h = ctypes.c_void_p()
        check(_lib.load().lne_graph_upload(ctx.handle, off.size - 1, _ptr(off), _ptr(nb), ctypes.byref(h)))
        return cls(ctx, h, off.size - 1, int(off[-1]))

    @classmethod
    def from_device(cls, ctx: Context, n: int, d_offsets: int, d_nbrs: int, m_dir: int) -> "Graph":
        h = ctypes.c_void_p()
        check(_lib.load().lne_graph_upload_device(ctx.handle, n, ctypes.c_void_p(d_offsets),
                                                  ctypes.c_void_p(d_nbrs), ctypes.byref(h)))
        return cls(ctx, h, n, m_dir)

    def free(self) -> None:
        if self.handle:
            _lib.load().lne_graph_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class CSR:
    """Device CSR (int64 row_ptr, int32 col, float32 val), canonical order."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle
        n = ctypes.c_int64()
        nnz = ctypes.c_int64()
        check(_lib.load().lne_csr_info(handle, ctypes.byref(n), ctypes.byref(nnz)))
        self.n = n.value
        self.nnz = nnz.value

    @classmethod
    def wrap_device(cls, ctx: Context, n: int, nnz: int, d_row_ptr: int, d_col: int, d_val: int) -> "CSR":
        h = ctypes.c_void_p()
        check(_lib.load().lne_csr_wrap_device(ctx.handle, n, nnz, ctypes.c_void_p(d_row_ptr),
                                              ctypes.c_void_p(d_col), ctypes.c_void_p(d_val), ctypes.byref(h)))
        return cls(ctx, h)

    def download(self):
        rp = np.empty(self.n + 1, dtype=np.int64)
        col = np.empty(self.nnz, dtype=np.int32)
        val = np.empty(self.nnz, dtype=np.float32)
        check(_lib.load().lne_csr_download(self.ctx.handle, self.handle, _ptr(rp), _ptr(col), _ptr(val)))
        return rp, col, val

    def device_ptrs(self):
        a, b, c = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(_lib.load().lne_csr_device_ptrs(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def free(self) -> None:
        if self.handle:
            _lib.load().lne_csr_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def generate_trunc_log_matrix_v2(ctx: Context, graph: Graph, seed: int, walk_len: int = 10,
                                 upper: bool = False, sample: bool = False, table_size: int = 0,
                                 negative: int = 1, sample_ratio: float = 1.0,
                                 mem_ratio: float = 1.0):
    """NetSMF sparsifier (``LightNE/PathEmbed.h:81-369``) on the device.

    Returns ``(CSR, stats)``.  ``seed`` replaces the reference's ``time(0)``;
    ``sample_ratio``/``mem_ratio`` are narrowed to float as the reference's
    flag parsing does.  Raises :class:`LneError` with ``LNE_ERR_TABLE_FULL``
    where the reference would print "looping forever" and exit.
    """
    p = SparsifyParams(seed=seed & 0xFFFFFFFFFFFFFFFF, walk_len=walk_len, table_size=table_size,
                       negative=negative, sample=int(bool(sample)), upper=int(bool(upper)),
                       sample_ratio=sample_ratio, mem_ratio=mem_ratio)
    st = SparsifyStats()
    h = ctypes.c_void_p()
    check(_lib.load().lne_sparsify(ctx.handle, graph.handle, ctypes.byref(p), ctypes.byref(h), ctypes.byref(st)))
    return CSR(ctx, h), st.as_dict()
