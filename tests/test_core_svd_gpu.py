"""Core SVD of the randomized SVD (lne_core_svd, the LAPACKE_gesvd call at
LightNE/mklredsvd/mklredsvd.cc:357-371) against numpy's FP64 SVD.

C = U diag(sigma) V^T is built in FP64 from random orthogonal factors with
chosen spectra: smooth decay, a condition number of 1e8, repeated singular
values, exact rank deficiency.  The device result must give the singular
values to 1e-12 of the largest, orthonormal left vectors, C C^T U = U S^2,
and the same vectors as numpy where the spectrum separates them.  Sizes
cover the FP32-preconditioned path (r <= 160, both its odd and even
pairings) and the plain FP64 path above it."""
import numpy as np
import pytest
import torch

from lightne_gb300.api import core_svd

pytestmark = pytest.mark.gpu


def _orth(rng, r):
    q, _ = np.linalg.qr(rng.standard_normal((r, r)))
    return q


def _spectrum(kind, r, rng):
    if kind == "decay":
        return np.exp(-np.linspace(0.0, np.log(1e3), r)) * (1.0 + 0.01 * rng.standard_normal(r))
    if kind == "ill":
        return np.logspace(0.0, -8.0, r)
    if kind == "repeated":
        return np.repeat(np.linspace(1.0, 0.2, 5), (r + 4) // 5)[:r]
    if kind == "deficient":
        s = np.exp(-np.linspace(0.0, 3.0, r))
        s[max(1, r // 2):] = 0.0
        return s
    raise ValueError(kind)


@pytest.mark.parametrize("r", [1, 2, 3, 17, 64, 128, 138, 160, 161, 200])
@pytest.mark.parametrize("kind", ["decay", "ill", "repeated", "deficient"])
def test_core_svd_matches_numpy(ctx, r, kind):
    rng = np.random.default_rng(1000 * r + len(kind))
    sig = np.abs(_spectrum(kind, r, rng))
    C = (_orth(rng, r) * sig) @ _orth(rng, r).T
    U, S, (sw64, sw32) = core_svd(ctx, C)
    U = U.cpu().numpy()
    S = S.cpu().numpy()
    ref = np.sort(sig)[::-1]
    smax = ref[0]
    assert np.all(np.diff(S) <= 0.0)
    assert np.abs(S - ref).max() <= 1e-12 * smax, (np.abs(S - ref).max(), smax)
    keep = ref > 1e-10 * smax
    Uk = U[:, keep]
    assert np.abs(Uk.T @ Uk - np.eye(Uk.shape[1])).max() <= 1e-12
    resid = C @ (C.T @ Uk) - Uk * S[keep] ** 2
    assert np.abs(resid).max() <= 1e-12 * smax ** 2
    # vectors of well-separated singular values agree with numpy's up to sign
    Un, Sn, _ = np.linalg.svd(C)
    gap = np.full(r, np.inf)
    if r > 1:
        d = np.abs(np.diff(Sn))
        gap[:-1] = np.minimum(gap[:-1], d)
        gap[1:] = np.minimum(gap[1:], d)
    sep = keep & (gap > 1e-3 * smax)
    if sep.any():
        cos = np.abs(np.sum(U[:, sep] * Un[:, sep], axis=0))
        assert (1.0 - cos).max() <= 1e-9, (1.0 - cos).max()
    if 2 <= r <= 160:
        assert sw32 >= 1
    if r > 160:
        assert sw32 == 0
    assert 1 <= sw64 <= 60


def test_core_svd_input_untouched(ctx):
    rng = np.random.default_rng(3)
    C = torch.tensor(rng.standard_normal((138, 138)), dtype=torch.float64, device="cuda")
    C0 = C.clone()
    core_svd(ctx, C)
    assert torch.equal(C, C0)
