"""ORACLE — test infrastructure, not product code.

The reference's whole pipeline on the host cores, for the timed CPU baseline
of the benchmark: the C port of the sparsifier (oracle/sparsify_port.c), then
the dense stages in FP32 as the reference runs them through MKL — CSR x dense
products on every core (oracle/spmm_port.c, in place of mkl_sparse_s_mm),
Householder QR (`torch.linalg.qr`, as geqrf + orgqr), GEMMs and small SVDs
(`torch.linalg`, every thread).  The reference's own MKL build is not
available (MKL is absent from the reference tree and from the benchmark
host), so this is a port, not the reference binary.

The pipeline is an ordered list of work units; running every unit once, in
order, is one whole embedding of the workload.  The benchmark's CPU arm times
its steps as consecutive groups of units, so that its steps together run the
pipeline exactly once, with nothing scaled or extrapolated.

  sparsifier    LightNE/PathEmbed.h:81-369 (port: oracle/sparsify_port.c)
  randsvd       LightNE/mklredsvd/mklredsvd.cc:93-403 + PathEmbed.h:371-408
  propagate     LightNE/SpectralPropagation.h:45-221
  dense_embed   LightNE/SpectralPropagation.h:16-43
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from oracle import port


def set_threads(n: int | None = None) -> int:
    n = n or os.cpu_count() or 1
    torch.set_num_threads(n)
    return n


def operator_csr(offsets, nbrs, mu=0.2):
    """The CSR of M the reference builds (self loop first, values computed in
    double and narrowed to float, SpectralPropagation.h:51-75)."""
    n = offsets.size - 1
    deg = np.diff(offsets)
    dt = (deg + 1).astype(np.float64)
    mu_f = float(np.float32(mu))
    diag = (1.0 - mu_f - 1.0 / dt).astype(np.float32)
    offv = (-1.0 / dt).astype(np.float32)
    rp = offsets + np.arange(n + 1)
    col = np.empty(rp[-1], dtype=np.int32)
    val = np.empty(rp[-1], dtype=np.float32)
    col[rp[:-1]] = np.arange(n)
    val[rp[:-1]] = diag
    mask = np.ones(rp[-1], dtype=bool)
    mask[rp[:-1]] = False
    col[mask] = nbrs
    val[mask] = np.repeat(offv, deg)
    return rp.astype(np.int64), col, val


def bessel_weights(order, s):
    import scipy.special as ss
    sf = float(np.float32(s))
    c = [float(np.float32(ss.iv(0, sf))), float(np.float32(-2 * ss.iv(1, sf)))]
    c += [float(np.float32((-2 if k & 1 else 2) * ss.iv(k, sf))) for k in range(2, order)]
    return c


def _blocks(total, parts):
    """parts + 1 boundaries splitting [0, total) into near-equal ranges."""
    return [total * i // parts for i in range(parts + 1)]


class Pipeline:
    """One whole embedding of a workload on the host cores, as work units.

    w: dict with walk_len, tablesz, sample_ratio (float), rank, dim, order.
    Units, in order: the sampler over `sample_units` vertex ranges of equal
    directed-edge counts; the trunc-log + CSR build; the sketch; A Omega in
    `row_units` row blocks; QR; A Q in row blocks; B P, QR, C = Z^T B, core
    SVD and U sqrt(S); the operator build; one unit per Chebyshev order; the
    (A + I) product; the dense SVD embedding."""

    def __init__(self, off, nbrs, w, seed, nthreads=0, sample_units=32, row_units=16, mu=0.2, s=0.5,
                 svd_seed=777):
        self.off = np.ascontiguousarray(off, dtype=np.int64)
        self.nbrs = np.ascontiguousarray(nbrs, dtype=np.int32)
        self.n = self.off.size - 1
        self.w = w
        self.seed = seed
        self.cores = set_threads(nthreads or None)
        self.mu, self.s, self.svd_seed = mu, s, svd_seed
        self.stage_s: dict[str, float] = {}
        self.units = []
        # sampler ranges cut on directed-edge counts
        m_dir = int(self.off[-1])
        cuts = np.searchsorted(self.off, np.array(_blocks(m_dir, sample_units)), side="left")
        cuts[0], cuts[-1] = 0, self.n
        cuts = np.maximum.accumulate(cuts)
        self.units.append(("sparsify", self._u_session))
        for i in range(sample_units):
            self.units.append(("sparsify", lambda a=int(cuts[i]), b=int(cuts[i + 1]): self._u_sample(a, b)))
        self.units.append(("sparsify", self._u_finish))
        rb = _blocks(self.n, row_units)
        self.units.append(("randsvd", self._u_sketch))
        for i in range(row_units):
            self.units.append(("randsvd", lambda a=rb[i], b=rb[i + 1]: self._u_spmm("O", "Y", a, b)))
        self.units.append(("randsvd", self._u_qr1))
        for i in range(row_units):
            self.units.append(("randsvd", lambda a=rb[i], b=rb[i + 1]: self._u_spmm("Q", "B", a, b)))
        self.units.append(("randsvd", self._u_core))
        self.units.append(("propagate", self._u_operator))
        for k in range(1, max(w["order"], 2)):
            self.units.append(("propagate", lambda k=k: self._u_order(k)))
        self.units.append(("propagate", self._u_aplusi))
        self.units.append(("dense_embed", self._u_dense))

    # -- sparsifier -------------------------------------------------------
    def _u_session(self):
        w = self.w
        self.sess = port.Session(self.off, self.nbrs, self.seed, walk_len=w["walk_len"], tablesz=w["tablesz"],
                                 sample_ratio=float(np.float32(w["sample_ratio"])), nthreads=self.cores)

    def _u_sample(self, a, b):
        self.sess.sample(a, b)

    def _u_finish(self):
        self.csr, self.sp_stats = self.sess.finish()
        self.sess = None

    # -- randomized SVD (mklredsvd.cc:93-403) ------------------------------
    def _u_sketch(self):
        r = self.w["rank"]
        self.gen = torch.Generator().manual_seed(self.svd_seed)
        self.O = torch.randn(self.n, r, generator=self.gen).numpy()
        self.Y = np.empty((self.n, r), np.float32)

    def _u_spmm(self, src, dst, a, b):
        rp, col, val = self.csr
        port.spmm(rp, col, val, getattr(self, src), rows=(a, b), out=getattr(self, dst), nthreads=self.cores)

    def _u_qr1(self):
        self.Q = torch.linalg.qr(torch.from_numpy(self.Y)).Q.contiguous().numpy()
        self.B = np.empty_like(self.Q)
        self.O = self.Y = None

    def _u_core(self):
        r, d = self.w["rank"], self.w["dim"]
        B = torch.from_numpy(self.B)
        P = torch.randn(r, r, generator=self.gen)
        Z = torch.linalg.qr(B @ P).Q
        C = Z.T @ B
        U, S, _ = torch.linalg.svd(C)
        self.emb = ((Z @ U[:, :d]) * torch.sqrt(S[:d])).contiguous().numpy()
        self.S = S.numpy()
        self.Q = self.B = None

    # -- spectral propagation (SpectralPropagation.h:45-221) ---------------
    def _u_operator(self):
        self.M = operator_csr(self.off, self.nbrs, self.mu)
        self.c = bessel_weights(max(self.w["order"], 2), self.s)

    def _mm(self, x):
        rp, col, val = self.M
        return port.spmm(rp, col, val, x, nthreads=self.cores)

    def _u_order(self, k):
        if k == 1:
            a = self.emb
            self.L0 = a
            tmp = self._mm(a)
            self.L1 = 0.5 * self._mm(tmp) - a
            self.conv = self.c[0] * self.L0 + self.c[1] * self.L1
            return
        tmp = self._mm(self.L1)
        L2 = self._mm(tmp) - self.L0 - 2 * self.L1
        self.conv += self.c[k] * L2
        self.L0, self.L1 = self.L1, L2

    def _u_aplusi(self):
        a = (self.emb - self.conv).astype(np.float32)
        ones = np.ones(self.nbrs.size, np.float32)
        self.y = a + port.spmm(self.off, self.nbrs, ones, a, nthreads=self.cores)
        self.L0 = self.L1 = self.conv = None

    def _u_dense(self):
        U, S, _ = torch.linalg.svd(torch.from_numpy(self.y), full_matrices=False)
        e = U * torch.sqrt(S)
        nrm = e.norm(dim=1, keepdim=True)
        self.out = torch.where(nrm > 1e-5, e / nrm, e).numpy()

    # -- driving ------------------------------------------------------------
    def run(self, lo=0, hi=None):
        """Runs units [lo, hi) in order; returns their wall seconds."""
        hi = len(self.units) if hi is None else hi
        total = 0.0
        for name, fn in self.units[lo:hi]:
            t0 = time.perf_counter()
            fn()
            dt = time.perf_counter() - t0
            self.stage_s[name] = self.stage_s.get(name, 0.0) + dt
            total += dt
        return total

    @property
    def samples(self) -> int:
        return int(self.sp_stats["samples"])


def step_groups(units: int, steps: int):
    """Boundaries cutting `units` consecutive units into `steps` groups (as
    equal in count as possible; every group non-empty while steps <= units)."""
    steps = max(1, min(steps, units))
    return _blocks(units, steps)


def warmup(off, nbrs, w, seed, nthreads, units):
    """Warm-up for the timed CPU steps: the sampler over the first `units`
    of 64 edge ranges in a throwaway table, and one small host product."""
    sess = port.Session(off, nbrs, seed, walk_len=w["walk_len"], tablesz=w["tablesz"],
                        sample_ratio=float(np.float32(w["sample_ratio"])), nthreads=nthreads)
    n = off.size - 1
    cuts = np.searchsorted(off, np.array(_blocks(int(off[-1]), 64)), side="left")
    for i in range(min(units, 64)):
        sess.sample(int(cuts[i]), int(min(cuts[i + 1], n)))
    sess.free()
    x = np.ones((n, 8), np.float32)
    port.spmm(off, nbrs, np.ones(nbrs.size, np.float32), x, nthreads=nthreads)
