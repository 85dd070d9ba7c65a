"""Differentiation form at full size: spectral propagation forward + adjoint
on the Chung-Lu graph with n = 1,138,499 and m = 2,990,443 (seed 2), input
embedding n x 128 (FP32, standard normal, seed 4), K = 10, mu = 0.2,
s = 0.5; loss = sum of squares of the output projected onto a fixed 128 x 16
Gaussian matrix (seed 5).  The device gradients (FP32 form, hand-written
adjoint through lne_propagate_adjoint) are checked against FP64 central
finite differences (step 1e-6) of the real-valued map on 64 random
coordinates of the embedding and on both filter parameters; the bar is 1e-4
relative (for the coordinates: norm-wise over the 64, and each entry
against the largest).

The FP64 side uses two exact identities of the map, so that it runs in
minutes on the host: the propagation acts on rows, hence y(a) R = y(a R)
(the loss needs a 16-column forward), and it is linear in a, hence
y(a +- h e_ic) R = y(a) R +- h y(e_i) R[c, :] (one forward of the 64 unit
vectors); the loss at both points is then evaluated and differenced in
FP64 as a central difference, entry by entry before the sum."""
import numpy as np
import pytest
import torch

from lightne_gb300 import graphs
from lightne_gb300.api import Graph, chebyshev_expansion, propagate_adjoint
from oracle import linalg_oracle as lo

pytestmark = pytest.mark.gpu

N, M_EDGES, DIM, ORDER, MU, S = 1138499, 2990443, 128, 10, 0.2, 0.5
H = 1e-6


def test_adjoint_matches_fd_at_config_size(ctx):
    off, nbrs = graphs.chung_lu(N, M_EDGES, 2.1, seed=2)
    g = Graph.from_numpy(ctx, off, nbrs)
    a = np.random.default_rng(4).standard_normal((N, DIM)).astype(np.float32)
    R = np.random.default_rng(5).standard_normal((DIM, 16))
    # device: forward, dL/dy = 2 (y R) R^T, adjoint
    y, _ = chebyshev_expansion(ctx, g, a, DIM, order=ORDER, mu=MU, s=S)
    Rt = torch.tensor(R, dtype=torch.float64, device="cuda")
    gy = (2.0 * (y.double() @ Rt) @ Rt.T).float()
    del y
    ga, dmu, ds = propagate_adjoint(ctx, g, a, gy, DIM, order=ORDER, mu=MU, s=S)
    del gy

    # FP64 central differences of L(a, mu, s) = |y(a R; mu, s)|^2
    aR = a.astype(np.float64) @ R

    def L16(mu, s):
        yy, _ = lo.propagate(off, nbrs, aR, order=ORDER, mu=mu, s=s, narrow=False)
        return float((yy ** 2).sum())

    fd_mu = (L16(MU + H, S) - L16(MU - H, S)) / (2 * H)
    fd_s = (L16(MU, S + H) - L16(MU, S - H)) / (2 * H)
    assert abs(dmu - fd_mu) <= 1e-4 * abs(fd_mu), (dmu, fd_mu)
    assert abs(ds - fd_s) <= 1e-4 * abs(fd_s), (ds, fd_s)

    Y, _ = lo.propagate(off, nbrs, aR, order=ORDER, mu=MU, s=S, narrow=False)  # y(a) R
    rng = np.random.default_rng(7)
    rows = rng.integers(0, N, 64)
    cols = rng.integers(0, DIM, 64)
    ga_h = ga.double().cpu().numpy()
    got, fd = np.zeros(64), np.zeros(64)
    E = np.zeros((N, 64))
    E[rows, np.arange(64)] = 1.0
    zz, _ = lo.propagate(off, nbrs, E, order=ORDER, mu=MU, s=S, narrow=False)  # y(e_i), one column each
    for k, (i, c) in enumerate(zip(rows, cols)):
        Z = zz[:, k:k + 1] * R[c][None, :]                                           # y(e_ic) R
        # L(a + h e) - L(a - h e), differenced entry by entry before the
        # sum (the totals are ~1e9; their difference would cancel)
        fd[k] = float((((Y + H * Z) ** 2) - ((Y - H * Z) ** 2)).sum()) / (2 * H)
        got[k] = ga_h[i, c]
    # FP32 evaluation of (I - f(M)) cancels for some vertices, so single
    # coordinates are compared on the scale of the gradient: the error of
    # the 64 sampled entries relative to their norm, and every entry's error
    # relative to the largest entry
    rel = np.linalg.norm(got - fd) / np.linalg.norm(fd)
    worst = np.abs(got - fd).max() / np.abs(fd).max()
    print("config-4 adjoint vs FP64 FD: dmu %.3e ds %.3e coords norm-wise %.3e worst %.3e" %
          (abs(dmu - fd_mu) / abs(fd_mu), abs(ds - fd_s) / abs(fd_s), rel, worst))
    assert rel <= 1e-4, rel
    assert worst <= 1e-4, worst
    g.free()
