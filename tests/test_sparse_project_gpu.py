"""-sparse_project: the very sparse random projection sketch of the
randomized SVD (LightNE/mklredsvd/mklredsvd.cc:148-226).  The sketch's
statistics (Binomial(rank, 1/s) nonzeros per row at distinct columns,
values +-sqrt(s), s = sqrt(n) below 1), its reproducibility, the product
Y = A O against FP64, and the whole SVD against the FP64 oracle run on the
same sketch (FP32 form: <= 1e-4 relative embedding error after Procrustes,
as the Gaussian sketch)."""
import math

import numpy as np
import pytest
import scipy.sparse as sp

from lightne_gb300 import graphs
from lightne_gb300.api import Graph, generate_trunc_log_matrix_v2, gaussian, randsvd, sparse_projection
from oracle import linalg_oracle as lo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def netsmf_matrix(ctx):
    off, nbrs = graphs.chung_lu(3000, 30000, 2.1, seed=21)
    g = Graph.from_numpy(ctx, off, nbrs)
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, 5, walk_len=10, table_size=3_000_000, sample_ratio=1.0)
    rp, col, val = csr.download()
    yield csr, sp.csr_matrix((val.astype(np.float64), col, rp), shape=(3000, 3000))
    csr.free()
    g.free()


@pytest.mark.parametrize("n,rank,s", [(40000, 138, 100.0), (5000, 64, 4.0), (10000, 32, 0.0)])
def test_sketch_statistics(ctx, n, rank, s):
    O, nnz = sparse_projection(ctx, 777, n, rank, s)
    O2, nnz2 = sparse_projection(ctx, 777, n, rank, s)
    o = O.cpu().numpy()
    assert nnz == nnz2 and (o == O2.cpu().numpy()).all()  # reproducible
    s_eff = s if s >= 1.0 else math.sqrt(n)
    v = np.float32(math.sqrt(np.float32(s_eff)))
    nz = o[o != 0]
    assert nz.size == nnz
    assert np.isin(np.abs(nz), [v]).all()
    # nonzeros ~ Binomial(n * rank, 1/s): within 6 standard deviations
    p = 1.0 / s_eff
    mean, sd = n * rank * p, math.sqrt(n * rank * p * (1 - p))
    assert abs(nnz - mean) < 6 * sd, (nnz, mean, sd)
    # signs balanced, columns spread
    assert abs((nz > 0).mean() - 0.5) < 6 * 0.5 / math.sqrt(max(nz.size, 1))
    per_col = (o != 0).sum(axis=0)
    cmean, csd = n * p, math.sqrt(n * p * (1 - p))
    assert (np.abs(per_col - cmean) < 7 * csd + 1).all()
    # another seed gives another sketch
    O3, _ = sparse_projection(ctx, 778, n, rank, s)
    assert (O3.cpu().numpy() != o).any()


def test_product_matches_fp64(ctx, netsmf_matrix):
    csr, A = netsmf_matrix
    rank, s = 40, 9.0
    emb, _, _ = randsvd(ctx, csr, rank, rank, random_project_only=True, sparse_project=True, sparse_project_s=s,
                        seed=31)
    O, _ = sparse_projection(ctx, 31, A.shape[0], rank, s)
    ref = A @ O.double().cpu().numpy()
    bound = 1e-5 * (abs(A) @ np.abs(O.double().cpu().numpy())) + 1e-30
    err = np.abs(emb.double().cpu().numpy() - ref)
    assert (err <= bound).all(), (err / bound).max()


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp16", 1e-3), ("bf16", 3e-3)])
def test_randsvd_sparse_project_matches_fp64(ctx, netsmf_matrix, precision, tol):
    csr, A = netsmf_matrix
    rank, dim, seed, s = 48, 32, 777, 4.0
    emb, S, st = randsvd(ctx, csr, rank, dim, precision=precision, seed=seed, sparse_project=True,
                         sparse_project_s=s)
    O, _ = sparse_projection(ctx, seed, A.shape[0], rank, s)
    P = gaussian(ctx, seed, 1, rank, rank)
    ref, Sref = lo.randsvd(A, O.double().cpu().numpy(), P.double().cpu().numpy(), dim)
    e = emb.double().cpu().numpy()
    assert np.isfinite(e).all()
    err = lo.procrustes_rel_error(e, ref)
    assert err < tol, err
    assert lo.rel_sv_error(S[:dim], Sref[:dim]) < tol
    assert st["jacobi_sweeps_fp32"] > 0
    assert st["jacobi_sweeps"] > 0 if precision == "fp32" else st["jacobi_sweeps"] == 1
