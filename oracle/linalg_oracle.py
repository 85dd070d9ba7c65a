"""ORACLE — test infrastructure, not product code.

FP64 NumPy/SciPy restatement of the reference's dense stages, used as the
checker of the device randomized SVD, spectral propagation and dense
embedding.  Parity for these stages is measured by error metrics, not bit
patterns: the reference's arithmetic runs in Intel MKL (not in the reference
tree, no pinned version; README.md:22-37 asks for a conda/Parallel Studio
MKL), whose summation order and VSL SFMT19937 Gaussian stream cannot be
reproduced.  The oracle therefore takes the same Gaussian sketches as the
device run (exported by lne_gaussian) and evaluates the reference's
algorithm exactly in FP64.

Reference correspondence (paths inside the reference project):
  randsvd            LightNE/mklredsvd/mklredsvd.cc:93-403 (Y = A O, QR, B = A Q,
                     Z = qr(B P), C = Z^T B, gesvd(C), matU = Z U_C)
  gram_schmidt       LightNE/mklredsvd/util.cc:40-79 (geqrf + orgqr)
  u_sigma_root       LightNE/PathEmbed.h:371-408
  propagation        LightNE/SpectralPropagation.h:45-221
  dense_embed        LightNE/SpectralPropagation.h:16-43
  Bessel weights     LightNE/SpectralPropagation.h:12 (boost cyl_bessel_i)

QR sign convention: the device uses CholeskyQR, whose R has a positive
diagonal; Householder QR is unique up to column signs, so the oracle flips
signs to make diag(R) positive.  Singular vectors are compared after
orthogonal Procrustes alignment.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.special as ss


def spmm64(A: sp.csr_matrix, X: np.ndarray) -> np.ndarray:
    """A @ X in FP64 on every host core (the row-parallel C product of
    oracle/spmm_port.c; FP64 values, operand and sums)."""
    from oracle import port
    A = A.tocsr()
    if A.shape[0] >= 2 ** 31 or A.shape[1] >= 2 ** 31:
        return A @ X
    X = np.ascontiguousarray(X, dtype=np.float64)
    return port.spmm(A.indptr, A.indices, A.data.astype(np.float64), X)


def qr_pos(Y: np.ndarray) -> np.ndarray:
    """Thin Q of Y with diag(R) > 0 (the CholeskyQR factor)."""
    Q, R = np.linalg.qr(Y, mode="reduced")
    sgn = np.sign(np.diag(R))
    sgn[sgn == 0] = 1.0
    return Q * sgn


def u_sigma_root(U: np.ndarray, S, dim: int, normalize: bool, eps: float = 1e-5) -> np.ndarray:
    """emb[:, j] = sqrt(S_j) U[:, j] for j < dim; optional row normalisation
    (rows with norm <= eps are left as they are)."""
    sig = np.ones(dim) if S is None else np.sqrt(np.asarray(S[:dim], dtype=np.float64))
    emb = U[:, :dim] * sig
    if normalize:
        nrm = np.linalg.norm(emb, axis=1)
        ok = nrm > eps
        emb[ok] /= nrm[ok, None]
    return emb


def randsvd(A: sp.csr_matrix, omega: np.ndarray, P: np.ndarray, dim: int, normalize: bool = False,
            random_project_only: bool = False):
    """MKLRedSVD::run + compute_u_sigma_root in FP64.  Returns (emb, S)."""
    A = A.astype(np.float64)
    Y = spmm64(A, omega)
    if random_project_only:
        return u_sigma_root(Y, None, dim, normalize), None
    Q = qr_pos(Y)
    B = spmm64(A, Q)
    Z = qr_pos(B @ P)
    C = Z.T @ B
    Uc, S, _ = np.linalg.svd(C)
    matU = Z @ Uc
    return u_sigma_root(matU, S, dim, normalize), S


def ne_zhang_matrix(offsets: np.ndarray, nbrs: np.ndarray) -> sp.csr_matrix:
    """The matrix NE_Zhang_et_al factorises (LightNE/PathEmbed.h:410-448):
    the graph's structure with values (float)(log(1/d_i) - log(neg_v /
    sum neg)), neg_v = (sum over neighbours u of v of 1/d_u)^0.75, FP64
    before the narrowing (each neg_v summed in file order)."""
    n = offsets.size - 1
    deg = np.diff(offsets).astype(np.float64)
    inv = np.zeros(n)
    inv[deg > 0] = 1.0 / deg[deg > 0]
    contrib = inv[nbrs]
    neg = np.zeros(n)
    for j in range(n):
        s = 0.0
        for e in range(offsets[j], offsets[j + 1]):
            s += contrib[e]
        neg[j] = s ** 0.75
    neg_sum = float(np.sum(neg))
    src = np.repeat(np.arange(n), np.diff(offsets))
    val = (np.log(1.0 / deg[src]) - np.log(neg[nbrs] / neg_sum)).astype(np.float32)
    return sp.csr_matrix((val, nbrs.astype(np.int64), offsets.astype(np.int64)), shape=(n, n))


def operator_values(deg: np.ndarray, mu: float, narrow: bool = True):
    """Per-row diagonal and off-diagonal values of M as the reference stores
    them (floats computed in double, SpectralPropagation.h:62-72); with
    narrow=False the exact real-valued operator (for derivatives)."""
    dt = (deg + 1).astype(np.float64)
    if not narrow:
        return 1.0 - mu - 1.0 / dt, -1.0 / dt
    mu_f = float(np.float32(mu))
    diag = (1.0 - mu_f - 1.0 / dt).astype(np.float32).astype(np.float64)
    off = (-1.0 / dt).astype(np.float32).astype(np.float64)
    return diag, off


def chebyshev_coefficients(order: int, s: float, narrow: bool = True) -> np.ndarray:
    s_f = float(np.float32(s)) if narrow else float(s)
    c = np.zeros(max(order, 2))
    c[0] = ss.iv(0, s_f)
    c[1] = -2.0 * ss.iv(1, s_f)
    for k in range(2, order):
        c[k] = (-2.0 if k & 1 else 2.0) * ss.iv(k, s_f)
    return c.astype(np.float32).astype(np.float64) if narrow else c


def propagate(offsets: np.ndarray, nbrs: np.ndarray, a: np.ndarray, order: int = 10, mu: float = 0.2,
              s: float = 0.5, narrow: bool = True):
    """chebyshev_expansion up to tmp = (A + I)(a - conv), in FP64.  With
    narrow=False mu, s, M and the weights are not rounded to float (the
    real-valued map, for finite differences).  Returns (y, a - conv)."""
    n = offsets.size - 1
    deg = np.diff(offsets)
    diag, off = operator_values(deg, mu, narrow)
    rows = np.repeat(np.arange(n), deg)
    Adj = sp.csr_matrix((np.ones(nbrs.size), nbrs.astype(np.int64), offsets), shape=(n, n))
    M = (sp.diags(diag) + sp.diags(off) @ Adj).tocsr()
    c = chebyshev_coefficients(order, s, narrow)
    a = a.astype(np.float64)
    Lx0 = a.copy()
    tmp = spmm64(M, a)
    Lx1 = 0.5 * spmm64(M, tmp) - a
    conv = c[0] * Lx0 + c[1] * Lx1
    for k in range(2, order):
        tmp = spmm64(M, Lx1)
        Lx2 = spmm64(M, tmp) - Lx0 - 2.0 * Lx1
        conv = conv + c[k] * Lx2
        Lx0, Lx1 = Lx1, Lx2
    a2 = a - conv
    y = a2 + spmm64(Adj, a2)
    del rows
    return y, a2


def dense_embed(x: np.ndarray, normalize: bool = True):
    """get_embedding_dense: gesvd(x) -> U sqrt(S), rows normalised."""
    U, S, _ = np.linalg.svd(x.astype(np.float64), full_matrices=False)
    d = x.shape[1]
    return u_sigma_root(U, S, d, normalize), S


# ---------------------------------------------------------------------------
# Error metrics
# ---------------------------------------------------------------------------
def procrustes_rel_error(E: np.ndarray, Eref: np.ndarray) -> float:
    """min over orthogonal R of ||E R - Eref||_F / ||Eref||_F."""
    E = E.astype(np.float64)
    Eref = Eref.astype(np.float64)
    U, _, Vt = np.linalg.svd(E.T @ Eref)
    R = U @ Vt
    return float(np.linalg.norm(E @ R - Eref) / np.linalg.norm(Eref))


def max_principal_angle(U1: np.ndarray, U2: np.ndarray) -> float:
    """Largest principal angle (radians) between the column spans."""
    Q1 = sla.orth(U1.astype(np.float64))
    Q2 = sla.orth(U2.astype(np.float64))
    s = np.linalg.svd(Q1.T @ Q2, compute_uv=False)
    return float(np.arccos(np.clip(s.min(), -1.0, 1.0)))


def rel_sv_error(S: np.ndarray, Sref: np.ndarray) -> float:
    S = np.asarray(S, dtype=np.float64)
    Sref = np.asarray(Sref, dtype=np.float64)
    return float(np.max(np.abs(S - Sref) / np.maximum(np.abs(Sref), 1e-300)))
