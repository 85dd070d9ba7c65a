"""Adjoint of the spectral propagation (lne_propagate_adjoint and the
torch.autograd.Function) against an FP64 dense-operator autograd reference
and FP64 central finite differences (step 1e-6).  Tolerances: dL/da and
dL/dmu, dL/ds within 1e-4 relative (FP32 form).  The 16-bit forms gather
16-bit vectors for dL/da (within 1e-3 for FP16, 3e-3 for BF16) and compute
the parameter gradients in FP32 (within 1e-4)."""
import math

import numpy as np
import pytest
import torch

from lightne_gb300 import graphs
from lightne_gb300.api import ChebyshevPropagation, Graph, propagate_adjoint
from oracle import linalg_oracle as lo

pytestmark = pytest.mark.gpu


def bessel_i_series(k, s, terms=30):
    out = torch.zeros((), dtype=torch.float64)
    for m in range(terms):
        out = out + (s / 2) ** (2 * m + k) / float(math.factorial(m) * math.factorial(m + k))
    return out


def dense_forward(off, nbrs, a, mu, s, order):
    """The real-valued map in FP64 on a dense operator, differentiable."""
    n = off.size - 1
    A = torch.zeros(n, n, dtype=torch.float64)
    src = np.repeat(np.arange(n), np.diff(off))
    A[src, nbrs.astype(np.int64)] = 1.0
    dt = torch.tensor(np.diff(off) + 1, dtype=torch.float64)
    At = A + torch.eye(n, dtype=torch.float64)
    M = (1.0 - mu) * torch.eye(n, dtype=torch.float64) - At / dt[:, None]
    c = [bessel_i_series(0, s), -2 * bessel_i_series(1, s)] + \
        [(-2 if k & 1 else 2) * bessel_i_series(k, s) for k in range(2, order)]
    Lx0 = a
    Lx1 = 0.5 * (M @ (M @ a)) - a
    conv = c[0] * Lx0 + c[1] * Lx1
    for k in range(2, order):
        Lx2 = M @ (M @ Lx1) - 2 * Lx1 - Lx0
        conv = conv + c[k] * Lx2
        Lx0, Lx1 = Lx1, Lx2
    return At @ (a - conv)


@pytest.mark.parametrize("order", [10, 3, 2])
def test_adjoint_matches_dense_autograd(ctx, order):
    off, nbrs = graphs.chung_lu(400, 2500, 2.1, seed=41)
    g = Graph.from_numpy(ctx, off, nbrs)
    dim = 12
    rng = np.random.default_rng(5)
    a = rng.standard_normal((400, dim))
    W = rng.standard_normal((dim, 4))
    mu0, s0 = 0.2, 0.5
    at = torch.tensor(a, requires_grad=True)
    mut = torch.tensor(mu0, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(s0, dtype=torch.float64, requires_grad=True)
    y = dense_forward(off, nbrs, at, mut, st, order)
    loss = ((y @ torch.tensor(W)) ** 2).sum()
    loss.backward()
    yd = y.detach().numpy()
    gy = 2 * (yd @ W) @ W.T
    ga, dmu, ds = propagate_adjoint(ctx, g, a.astype(np.float32), gy.astype(np.float32), dim, order=order, mu=mu0,
                                    s=s0)
    ref = at.grad.numpy()
    rel = np.linalg.norm(ga.double().cpu().numpy() - ref) / np.linalg.norm(ref)
    assert rel < 1e-4, rel
    assert abs(dmu - mut.grad.item()) <= 1e-4 * abs(mut.grad.item()) + 1e-6, (dmu, mut.grad.item())
    assert abs(ds - st.grad.item()) <= 1e-4 * abs(st.grad.item()) + 1e-6, (ds, st.grad.item())
    g.free()


@pytest.mark.parametrize("precision,tol", [("fp16", 1e-3), ("bf16", 3e-3)])
@pytest.mark.parametrize("a_scale,g_scale", [(1.0, 1.0), (1e-5, 4e3)])
def test_adjoint_16bit_forms(ctx, precision, tol, a_scale, g_scale):
    """The 16-bit forms against the FP64 dense autograd; the second case puts
    the input and the output gradient far outside FP16's normal range (the
    FP16 form scales the output gradient by a power of two and unscales the
    results).  dL/dmu and dL/ds come from the FP32 tangent pass."""
    off, nbrs = graphs.chung_lu(400, 2500, 2.1, seed=43)
    g = Graph.from_numpy(ctx, off, nbrs)
    dim, order = 16, 10
    rng = np.random.default_rng(7)
    a = a_scale * rng.standard_normal((400, dim))
    W = rng.standard_normal((dim, 4))
    at = torch.tensor(a, requires_grad=True)
    mut = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    y = dense_forward(off, nbrs, at, mut, st, order)
    gy = g_scale * rng.standard_normal(tuple(y.shape))
    (y * torch.tensor(gy)).sum().backward()
    ga, dmu, ds = propagate_adjoint(ctx, g, a.astype(np.float32), gy.astype(np.float32), dim, order=order,
                                    precision=precision)
    ref = at.grad.numpy()
    ga = ga.double().cpu().numpy()
    assert np.isfinite(ga).all()
    rel = np.linalg.norm(ga - ref) / np.linalg.norm(ref)
    assert rel < tol, rel
    assert abs(dmu - mut.grad.item()) <= 1e-4 * abs(mut.grad.item()), (dmu, mut.grad.item())
    assert abs(ds - st.grad.item()) <= 1e-4 * abs(st.grad.item()), (ds, st.grad.item())
    g.free()


def test_autograd_function_and_finite_differences(ctx):
    off, nbrs = graphs.chung_lu(3000, 20000, 2.1, seed=42)
    g = Graph.from_numpy(ctx, off, nbrs)
    n, dim, order = 3000, 16, 10
    rng = np.random.default_rng(6)
    a = rng.standard_normal((n, dim))
    W = rng.standard_normal((dim, 4))
    at = torch.tensor(a, dtype=torch.float32, device="cuda", requires_grad=True)
    mut = torch.tensor(0.2, device="cuda", requires_grad=True)
    st = torch.tensor(0.5, device="cuda", requires_grad=True)
    y = ChebyshevPropagation(at, mut, st, ctx, g, order)
    loss = ((y @ torch.tensor(W, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()

    def L(aa, mu, s):
        yy, _ = lo.propagate(off, nbrs, aa, order=order, mu=mu, s=s, narrow=False)
        return float(((yy @ W) ** 2).sum())

    h = 1e-6
    fd_mu = (L(a, 0.2 + h, 0.5) - L(a, 0.2 - h, 0.5)) / (2 * h)
    fd_s = (L(a, 0.2, 0.5 + h) - L(a, 0.2, 0.5 - h)) / (2 * h)
    assert abs(mut.grad.item() - fd_mu) <= 1e-4 * abs(fd_mu), (mut.grad.item(), fd_mu)
    assert abs(st.grad.item() - fd_s) <= 1e-4 * abs(fd_s), (st.grad.item(), fd_s)
    ga = at.grad.double().cpu().numpy()
    for (i, j) in [(0, 0), (5, 3), (100, 15), (2999, 7), (1234, 1), (17, 11)]:
        ap, am = a.copy(), a.copy()
        ap[i, j] += h
        am[i, j] -= h
        fd = (L(ap, 0.2, 0.5) - L(am, 0.2, 0.5)) / (2 * h)
        assert abs(ga[i, j] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(ga).max()), (i, j, ga[i, j], fd)
    g.free()
