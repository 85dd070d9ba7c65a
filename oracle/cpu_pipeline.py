"""ORACLE — test infrastructure, not product code.

The reference's dense stages restated op-for-op in FP32 over torch CPU, for
the timed CPU baseline of the benchmark (the reference's own MKL build is not
available: MKL is absent from the reference tree and from the benchmark host).
Sparse products are CSR x dense (`torch.sparse.mm`), QR is
`torch.linalg.qr` (Householder, as geqrf + orgqr), small SVDs are
`torch.linalg.svd`; every thread the host offers is used.

  randsvd       LightNE/mklredsvd/mklredsvd.cc:93-403 + PathEmbed.h:371-408
  propagate     LightNE/SpectralPropagation.h:45-221
  dense_embed   LightNE/SpectralPropagation.h:16-43
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch


def set_threads(n: int | None = None) -> int:
    n = n or os.cpu_count() or 1
    torch.set_num_threads(n)
    return n


def csr_tensor(row_ptr, col, val, n):
    return torch.sparse_csr_tensor(torch.from_numpy(np.ascontiguousarray(row_ptr, dtype=np.int64)),
                                   torch.from_numpy(np.ascontiguousarray(col, dtype=np.int64)),
                                   torch.from_numpy(np.ascontiguousarray(val, dtype=np.float32)), size=(n, n))


def operator_csr(offsets, nbrs, mu=0.2):
    """The CSR of M the reference builds (self loop first, SpectralPropagation.h:51-75)."""
    n = offsets.size - 1
    deg = np.diff(offsets)
    dt = (deg + 1).astype(np.float32).astype(np.float64)
    mu_f = float(np.float32(mu))
    diag = (1.0 - mu_f - 1.0 / dt).astype(np.float32)
    offv = (-1.0 / dt).astype(np.float32)
    rp = offsets + np.arange(n + 1)
    col = np.empty(rp[-1], dtype=np.int64)
    val = np.empty(rp[-1], dtype=np.float32)
    col[rp[:-1]] = np.arange(n)
    val[rp[:-1]] = diag
    mask = np.ones(rp[-1], dtype=bool)
    mask[rp[:-1]] = False
    col[mask] = nbrs
    val[mask] = np.repeat(offv, deg)
    return csr_tensor(rp, col, val, n)


def randsvd(A, rank, dim, seed=777):
    g = torch.Generator().manual_seed(seed)
    n = A.shape[0]
    O = torch.randn(n, rank, generator=g)
    Y = torch.sparse.mm(A, O)
    Q, _ = torch.linalg.qr(Y)
    B = torch.sparse.mm(A, Q)
    P = torch.randn(rank, rank, generator=g)
    Z, _ = torch.linalg.qr(B @ P)
    C = Z.T @ B
    U, S, _ = torch.linalg.svd(C)
    return (Z @ U[:, :dim]) * torch.sqrt(S[:dim]), S


def propagate(M, Adj_plus_I, a, order=10, s=0.5):
    import scipy.special as ss
    sf = float(np.float32(s))
    Lx0 = a.clone()
    tmp = torch.sparse.mm(M, a)
    Lx1 = 0.5 * torch.sparse.mm(M, tmp) - a
    conv = float(np.float32(ss.iv(0, sf))) * Lx0 + float(np.float32(-2 * ss.iv(1, sf))) * Lx1
    for k in range(2, order):
        tmp = torch.sparse.mm(M, Lx1)
        Lx2 = torch.sparse.mm(M, tmp) - Lx0 - 2 * Lx1
        conv += float(np.float32((-2 if k & 1 else 2) * ss.iv(k, sf))) * Lx2
        Lx0, Lx1 = Lx1, Lx2
    a = a - conv
    return torch.sparse.mm(Adj_plus_I, a)


def dense_embed(x):
    U, S, _ = torch.linalg.svd(x, full_matrices=False)
    e = U * torch.sqrt(S)
    nrm = e.norm(dim=1, keepdim=True)
    return torch.where(nrm > 1e-5, e / nrm, e)


def timed(fn, *a, **k):
    t0 = time.perf_counter()
    out = fn(*a, **k)
    return out, time.perf_counter() - t0


def dense_stage_seconds(row_ptr, col, val, offsets, nbrs, rank=138, dim=128, order=10, row_frac=0.05,
                        seed=0):
    """Seconds of the reference's dense stages on this host, measured on a
    bounded sample and scaled by operation count:
      - one A x Omega product over a random `row_frac` of A's rows, scaled
        by nnz to the two products of the randomized SVD;
      - Householder QR, the B P and Z U GEMMs and the core SVD on the full
        n x rank panels (QR and GEMMs once each, scaled to their counts);
      - two operator products of the propagation, scaled to its 19;
      - the n x dim dense SVD.
    Returns a dict of per-stage seconds."""
    n = offsets.size - 1
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(n, max(1, int(n * row_frac)), replace=False))
    lens = row_ptr[rows + 1] - row_ptr[rows]
    sub_rp = np.zeros(rows.size + 1, np.int64)
    np.cumsum(lens, out=sub_rp[1:])
    idx = np.concatenate([np.arange(row_ptr[r], row_ptr[r + 1]) for r in rows]) if lens.sum() else np.zeros(0, int)
    Asub = torch.sparse_csr_tensor(torch.from_numpy(sub_rp), torch.from_numpy(col[idx].astype(np.int64)),
                                   torch.from_numpy(val[idx]), size=(rows.size, n))
    O = torch.randn(n, rank)
    _, t_sub = timed(torch.sparse.mm, Asub, O)
    frac_nnz = max(lens.sum(), 1) / max(row_ptr[-1], 1)
    t_spmm = t_sub / frac_nnz
    Y = torch.randn(n, rank)
    _, t_qr = timed(torch.linalg.qr, Y)
    P = torch.randn(rank, rank)
    _, t_gemm = timed(torch.matmul, Y, P)
    C = torch.randn(rank, rank)
    _, t_svd = timed(torch.linalg.svd, C)
    M = operator_csr(offsets, nbrs)
    a = torch.randn(n, dim)
    _, t_op = timed(torch.sparse.mm, M, a)
    _, t_op2 = timed(torch.sparse.mm, M, a)
    x = torch.randn(n, dim)
    _, t_dense = timed(dense_embed, x)
    return {
        "randsvd": 2 * t_spmm + 2 * t_qr + 3 * t_gemm + t_svd,
        "propagate": 19 * 0.5 * (t_op + t_op2),
        "dense_embed": t_dense,
        "spmm_sample_rows": int(rows.size),
    }
