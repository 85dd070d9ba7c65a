"""Pins the dense stages' oracle (and through it the device) to the
reference's own code.

Randomized SVD: tests/golden/randsvd_*.npz hold the singular values and the
embedding of the reference's MKLRedSVD::run + compute_u_sigma_root
(LightNE/mklredsvd/mklredsvd.cc:93-403, LightNE/PathEmbed.h:371-408,
compiled by oracle/ref_randsvd_harness.cc) on golden sparsifier matrices,
with Gaussian sketches drawn by numpy from a stored seed.  The FP64
restatement must agree: singular values <= 1e-5 relative, embedding
<= 2e-5 after Procrustes.  The device's randomized SVD is checked against
the same restatement with its own sketches (tests/test_dense_stages_gpu.py).

Spectral propagation:

tests/golden/propagate_*.npz hold the outputs of the reference's
chebyshev_expansion (LightNE/SpectralPropagation.h:45-229, compiled from its
sources by oracle/ref_propagate_harness.cc with the MKL and Boost calls it
needs defined in oracle/mkl_shim/mkl_defs.h and oracle/boost_shim), made by
tests/golden/make_golden.py: a - conv (the reference mutates its argument),
the (A + I)(a - conv) product it hands to get_embedding_dense, and the
returned embedding.  The reference computes in FP32.

  - the FP64 restatement (oracle/linalg_oracle.py) against them: relative
    Frobenius error <= 2e-6 (the reference's FP32 rounding), the dense
    embedding <= 2e-5 after Procrustes;
  - the device (lne_propagate, lne_dense_embed) against them: FP32 form
    <= 1e-5, FP16 form <= 1e-3, BF16 form <= 1e-2 (the star's hub row sums
    2499 BF16 values); lne_dense_embed on the
    reference's (A + I)(a - conv) <= 1e-4 after Procrustes.
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import linalg_oracle as lo

CASES = sorted(glob.glob(os.path.join(GOLDEN, "propagate_*.npz")))
IDS = [os.path.basename(c)[10:-4] for c in CASES]
SVD_CASES = sorted(glob.glob(os.path.join(GOLDEN, "randsvd_*.npz")))


@pytest.mark.parametrize("path", SVD_CASES, ids=[os.path.basename(c)[8:-4] for c in SVD_CASES])
def test_oracle_matches_reference_randsvd(path):
    import scipy.sparse as sp
    z = np.load(path)
    prm = json.loads(str(z["params"]))
    m = np.load(os.path.join(GOLDEN, "sparsify_%s.npz" % prm["matrix"]))
    rp, col, val = m["row_ptr"], m["col"], m["val"]
    n = rp.size - 1
    rng = np.random.default_rng(prm["sketch_seed"])
    omega = rng.standard_normal((n, prm["rank"])).astype(np.float32)
    P = rng.standard_normal((prm["rank"], prm["rank"])).astype(np.float32)
    A = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    emb, S = lo.randsvd(A, omega.astype(np.float64), P.astype(np.float64), prm["dim"],
                        normalize=bool(prm["normalize"]))
    assert lo.rel_sv_error(z["S"][:prm["dim"]], S[:prm["dim"]]) < 1e-5
    assert lo.procrustes_rel_error(z["emb"].astype(np.float64), emb) < 2e-5


def load(path):
    z = np.load(path)
    return z["offsets"], z["nbrs"], z["a"], json.loads(str(z["params"])), z["a_out"], z["y"], z["emb"]


def rel(x, ref):
    return float(np.linalg.norm(np.asarray(x, np.float64) - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_oracle_matches_reference_propagation(path):
    off, nbrs, a, prm, a_out, y, emb = load(path)
    yref, a2 = lo.propagate(off, nbrs, a, order=prm["order"], mu=prm["mu"], s=prm["s"])
    assert rel(a_out, a2) < 2e-6
    assert rel(y, yref) < 2e-6
    fin, _ = lo.dense_embed(y)
    assert lo.procrustes_rel_error(emb, fin) < 2e-5


def test_fixtures_present():
    assert len(CASES) >= 5 and len(SVD_CASES) >= 3


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("fp16", 1e-3), ("bf16", 1e-2)])
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_device_matches_reference_propagation(ctx, path, precision, tol):
    from lightne_gb300.api import Graph, chebyshev_expansion
    off, nbrs, a, prm, a_out, y, emb = load(path)
    g = Graph.from_numpy(ctx, off, nbrs)
    yd, a2, _ = chebyshev_expansion(ctx, g, a, prm["dim"], order=prm["order"], mu=prm["mu"], s=prm["s"],
                                    precision=precision, return_a=True)
    g.free()
    assert rel(yd.double().cpu().numpy(), y.astype(np.float64)) < tol
    assert rel(a2.double().cpu().numpy(), a_out.astype(np.float64)) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_device_dense_embed_matches_reference(ctx, path):
    from lightne_gb300.api import get_embedding_dense
    off, nbrs, a, prm, a_out, y, emb = load(path)
    out, _ = get_embedding_dense(ctx, y, prm["dim"])
    assert lo.procrustes_rel_error(out.double().cpu().numpy(), emb.astype(np.float64)) < 1e-4
