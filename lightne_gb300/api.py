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
from ._lib import (LNE_PREC_BF16, LNE_PREC_FP16, LNE_PREC_FP32, LneError, PropagateParams, PropagateStats, RandsvdParams,
                   RandsvdStats, SparsifyParams, SparsifyStats, check)

__all__ = ["Context", "Graph", "CSR", "generate_trunc_log_matrix_v2", "randsvd",
           "chebyshev_expansion", "get_embedding_dense", "gaussian", "chebyshev_coefficients", "propagate_adjoint", "ChebyshevPropagation", "LneError"]

PRECISIONS = {"fp32": LNE_PREC_FP32, "bf16": LNE_PREC_BF16, "fp16": LNE_PREC_FP16}


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """Device + stream.  ``stream`` is a raw cudaStream_t (int); by default
    the context runs on torch's current stream of ``device``, so library work
    and torch tensor operations are ordered on one stream."""

    def __init__(self, device: int = 0, stream: int | None = None):
        L = _lib.load()
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(device).cuda_stream
        h = ctypes.c_void_p()
        check(L.lne_ctx_create(ctypes.byref(h), device, ctypes.c_void_p(stream or 0)))
        self.handle = h
        self.device = device

    def synchronize(self) -> None:
        check(_lib.load().lne_ctx_synchronize(self.handle))

    def set_sparsify_slices(self, slots: int = 8192, slice_bits: int = -1) -> None:
        """Shared-memory table size per slice of the sliced pair aggregation
        (0: always the pair table in HBM) and its slice bits (-1: automatic)."""
        check(_lib.load().lne_ctx_set_sparsify_slices(self.handle, slots, slice_bits))

    def set_sparsify_batch(self, keys: int = 0) -> None:
        """Samples per batch of the sparsifier (0: the default 2^30)."""
        check(_lib.load().lne_ctx_set_sparsify_batch(self.handle, keys))

    def set_sparsify_rounds(self, mode: int = 0, row_sort_max: int = 0) -> None:
        """Hash-range rounds above one batch of samples (counts): 0 when the
        pair table does not fit, 1 always, -1 never.  The rounds' CSR rows of
        at most row_sort_max entries (a power of two in [32, 1024]; 0: 1024)
        are sorted by one warp, longer rows through a bitmap of the column
        range."""
        check(_lib.load().lne_ctx_set_sparsify_rounds(self.handle, mode, row_sort_max))

    def set_row_sort_window(self, cols: int = 0) -> None:
        """Columns per window of the rounds' bitmap row sort (a multiple of
        2048; 0: as many as shared memory holds)."""
        check(_lib.load().lne_ctx_set_row_sort_window(self.handle, cols))

    def set_core_svd_fp64(self, mode: int = -1) -> None:
        """FP64 Jacobi sweeps in the core SVDs of lne_randsvd and
        lne_dense_embed after the FP32 ones: 1 until they converge, 0 one
        sweep, -1 (default) one in the 16-bit forms of lne_randsvd, else
        until they converge."""
        check(_lib.load().lne_ctx_set_core_svd_fp64(self.handle, mode))

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


def _torch():
    import torch
    return torch


def _as_device_f32(x, device):
    torch = _torch()
    if isinstance(x, np.ndarray):
        return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(f"cuda:{device}")
    return x.to(device=f"cuda:{device}", dtype=torch.float32).contiguous()


def ne_zhang_matrix(ctx: Context, graph: Graph) -> CSR:
    """path_embed::NE_Zhang_et_al's matrix (LightNE/PathEmbed.h:410-448) on
    the device; factorise it with ``randsvd(..., normalize=True)``."""
    out = ctypes.c_void_p()
    check(_lib.load().lne_ne_zhang_matrix(ctx.handle, graph.handle, ctypes.byref(out)))
    return CSR(ctx, out)


def sparse_projection(ctx: Context, seed: int, n: int, rank: int, s: float = 100.0):
    """The very sparse random projection randsvd uses with sparse_project,
    as a dense torch tensor n x rank, and its nonzero count."""
    torch = _torch()
    out = torch.empty(n, rank, dtype=torch.float32, device=f"cuda:{ctx.device}")
    nnz = ctypes.c_int64()
    check(_lib.load().lne_sparse_projection(ctx.handle, seed, n, rank, s, ctypes.c_void_p(out.data_ptr()), rank,
                                            ctypes.byref(nnz)))
    return out, nnz.value


def gaussian(ctx: Context, seed: int, stream_id: int, rows: int, cols: int):
    """The device Gaussian sketch (stream 0: Omega, 1: P) as a torch tensor."""
    torch = _torch()
    out = torch.empty(rows, cols, dtype=torch.float32, device=f"cuda:{ctx.device}")
    check(_lib.load().lne_gaussian(ctx.handle, seed, stream_id, rows, cols, ctypes.c_void_p(out.data_ptr()), cols))
    ctx.synchronize()
    return out


def randsvd(ctx: Context, A: CSR, rank: int, dim: int, normalize: bool = False, precision: str = "fp32",
            seed: int = 777, random_project_only: bool = False, sparse_project: bool = False,
            sparse_project_s: float = 100.0):
    """MKLRedSVD(...).run() + compute_u_sigma_root on the device
    (LightNE/mklredsvd/mklredsvd.cc:93-403, LightNE/PathEmbed.h:371-408).
    ``sparse_project`` takes the very sparse random projection sketch
    (mklredsvd.cc:148-226) instead of the Gaussian one.
    Returns (emb torch n x dim, S numpy[rank], stats)."""
    torch = _torch()
    emb = torch.empty(A.n, dim, dtype=torch.float32, device=f"cuda:{ctx.device}")
    S = np.zeros(rank, dtype=np.float32)
    p = RandsvdParams(rank=rank, dim=dim, normalize=int(bool(normalize)), precision=PRECISIONS[precision],
                      seed=seed, random_project_only=int(bool(random_project_only)),
                      sparse_project=int(bool(sparse_project)), sparse_project_s=float(sparse_project_s))
    st = RandsvdStats()
    check(_lib.load().lne_randsvd(ctx.handle, A.handle, ctypes.byref(p), ctypes.c_void_p(emb.data_ptr()),
                                  _ptr(S), ctypes.byref(st)))
    return emb, S, st.as_dict()


def chebyshev_expansion(ctx: Context, graph: Graph, a, dim: int, order: int = 10, mu: float = 0.2,
                        s: float = 0.5, precision: str = "fp32", return_a: bool = False):
    """spectral_propagation::chebyshev_expansion up to (A+I)a
    (LightNE/SpectralPropagation.h:45-221).  ``a`` is n x dim (numpy or
    torch); returns y (torch), and a - conv when ``return_a``."""
    torch = _torch()
    da = _as_device_f32(a, ctx.device)
    y = torch.empty_like(da)
    a_out = torch.empty_like(da) if return_a else None
    p = PropagateParams(dim=dim, order=order, precision=PRECISIONS[precision], mu=mu, s=s)
    st = PropagateStats()
    check(_lib.load().lne_propagate(ctx.handle, graph.handle, ctypes.byref(p), ctypes.c_void_p(da.data_ptr()),
                                    ctypes.c_void_p(y.data_ptr()),
                                    ctypes.c_void_p(a_out.data_ptr() if return_a else 0), ctypes.byref(st)))
    return (y, a_out, st.as_dict()) if return_a else (y, st.as_dict())


def get_embedding_dense(ctx: Context, x, dim: int):
    """SVD of x (n x dim) -> U sqrt(S), rows normalised
    (LightNE/SpectralPropagation.h:16-43).  Returns (emb torch, S numpy)."""
    torch = _torch()
    dx = _as_device_f32(x, ctx.device)
    n = dx.shape[0]
    emb = torch.empty(n, dim, dtype=torch.float32, device=f"cuda:{ctx.device}")
    S = np.zeros(dim, dtype=np.float32)
    check(_lib.load().lne_dense_embed(ctx.handle, ctypes.c_void_p(dx.data_ptr()), n, dim,
                                      ctypes.c_void_p(emb.data_ptr()), _ptr(S)))
    return emb, S


def core_svd(ctx: Context, C):
    """SVD of a small dense r x r matrix on the device, the core step of the
    randomized SVD (LAPACKE_gesvd at LightNE/mklredsvd/mklredsvd.cc:357-371):
    returns (U torch float64 r x r, S torch float64 r, (fp64 sweeps, fp32
    sweeps)); C = U diag(S) V^T, S descending."""
    torch = _torch()
    dc = torch.as_tensor(C, dtype=torch.float64).to(f"cuda:{ctx.device}").contiguous()
    r = dc.shape[0]
    if dc.dim() != 2 or dc.shape[1] != r:
        raise ValueError("core_svd: C must be square")
    U = torch.empty(r, r, dtype=torch.float64, device=dc.device)
    S = torch.empty(r, dtype=torch.float64, device=dc.device)
    sw = np.zeros(2, dtype=np.int32)
    check(_lib.load().lne_core_svd(ctx.handle, ctypes.c_void_p(dc.data_ptr()), r, ctypes.c_void_p(U.data_ptr()),
                                   ctypes.c_void_p(S.data_ptr()), _ptr(sw)))
    return U, S, (int(sw[0]), int(sw[1]))


def chebyshev_coefficients(order: int, s: float = 0.5) -> np.ndarray:
    out = np.zeros(max(order, 2), dtype=np.float32)
    check(_lib.load().lne_chebyshev_coefficients(order, s, _ptr(out)))
    return out


def propagate_adjoint(ctx: Context, graph: Graph, a, gy, dim: int, order: int = 10, mu: float = 0.2,
                      s: float = 0.5, precision: str = "fp32", need_params: bool = True):
    """Adjoint of :func:`chebyshev_expansion`: returns (dL/da torch, dL/dmu,
    dL/ds) for the output gradient ``gy`` (no counterpart in the reference)."""
    torch = _torch()
    da = _as_device_f32(a, ctx.device)
    dg = _as_device_f32(gy, ctx.device)
    ga = torch.empty_like(dg)
    dmu = ctypes.c_double(0.0)
    ds = ctypes.c_double(0.0)
    p = PropagateParams(dim=dim, order=order, precision=PRECISIONS[precision], mu=mu, s=s)
    st = PropagateStats()
    check(_lib.load().lne_propagate_adjoint(
        ctx.handle, graph.handle, ctypes.byref(p), ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(dg.data_ptr()),
        ctypes.c_void_p(ga.data_ptr()), ctypes.byref(dmu) if need_params else None,
        ctypes.byref(ds) if need_params else None, ctypes.byref(st)))
    return ga, dmu.value, ds.value


def _make_autograd_function():
    torch = _torch()

    class _ChebyshevPropagation(torch.autograd.Function):
        """y = (A + I)(a - sum_k c_k(s) T_k(X(mu)) a) on the device, with the
        hand-written adjoint (lne_propagate_adjoint) as its backward."""

        @staticmethod
        def forward(fctx, a, mu, s, lctx, graph, order, precision):
            a = a.contiguous().float()
            y, _ = chebyshev_expansion(lctx, graph, a, a.shape[1], order=order, mu=float(mu), s=float(s),
                                       precision=precision)
            fctx.save_for_backward(a)
            fctx.lctx, fctx.graph, fctx.order, fctx.precision = lctx, graph, order, precision
            fctx.mu, fctx.s = float(mu), float(s)
            fctx.need_mu = torch.is_tensor(mu) and mu.requires_grad
            fctx.need_s = torch.is_tensor(s) and s.requires_grad
            return y

        @staticmethod
        def backward(fctx, gy):
            (a,) = fctx.saved_tensors
            need = fctx.need_mu or fctx.need_s
            ga, dmu, ds = propagate_adjoint(fctx.lctx, fctx.graph, a, gy.contiguous(), a.shape[1],
                                            order=fctx.order, mu=fctx.mu, s=fctx.s, precision=fctx.precision,
                                            need_params=need)
            gmu = torch.tensor(dmu, dtype=torch.float32, device=a.device) if fctx.need_mu else None
            gs = torch.tensor(ds, dtype=torch.float32, device=a.device) if fctx.need_s else None
            return ga, gmu, gs, None, None, None, None

    return _ChebyshevPropagation


_AUTOGRAD = None


def ChebyshevPropagation(a, mu, s, lctx: Context, graph: Graph, order: int = 10, precision: str = "fp32"):
    """Differentiable spectral propagation (``torch.autograd.Function``):
    gradients flow to ``a`` and to ``mu`` / ``s`` when they are tensors that
    require grad."""
    global _AUTOGRAD
    if _AUTOGRAD is None:
        _AUTOGRAD = _make_autograd_function()
    return _AUTOGRAD.apply(a, mu, s, lctx, graph, order, precision)
