"""Randomized SVD, spectral propagation and dense embedding on the device
against the FP64 oracle (oracle/linalg_oracle.py) with the same Gaussian
sketches.  Tolerances (relative embedding error after Procrustes, relative
Frobenius error of the propagation): the FP32 form <= 1e-4 / 1e-5; the FP16
form <= 1e-3, the gate the 16-bit forms are held to; the BF16 form, whose
operands carry 2^-9 relative rounding, <= 3e-3 (it does not meet the gate on
every input: its measured errors are recorded beside the benchmark)."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from lightne_gb300 import graphs
from lightne_gb300.api import (CSR, Graph, chebyshev_expansion, gaussian, generate_trunc_log_matrix_v2,
                               get_embedding_dense, randsvd)
from oracle import linalg_oracle as lo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def netsmf_matrix(ctx):
    off, nbrs = graphs.chung_lu(3000, 30000, 2.1, seed=21)
    g = Graph.from_numpy(ctx, off, nbrs)
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, 5, walk_len=10, table_size=3_000_000, sample_ratio=1.0)
    rp, col, val = csr.download()
    yield csr, sp.csr_matrix((val.astype(np.float64), col, rp), shape=(3000, 3000)), (off, nbrs)
    csr.free()
    g.free()


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp16", 1e-3), ("bf16", 3e-3)])
@pytest.mark.parametrize("normalize", [False, True])
def test_randsvd_matches_fp64(ctx, netsmf_matrix, precision, tol, normalize):
    csr, A, _ = netsmf_matrix
    rank, dim, seed = 48, 32, 777
    emb, S, st = randsvd(ctx, csr, rank, dim, normalize=normalize, precision=precision, seed=seed)
    om = gaussian(ctx, seed, 0, A.shape[0], rank)
    # the 16-bit forms gather the sketch from an FP8 copy: exact
    assert torch.equal(om.to(torch.float8_e4m3fn).float(), om)
    P = gaussian(ctx, seed, 1, rank, rank)
    ref, Sref = lo.randsvd(A, om.double().cpu().numpy(), P.double().cpu().numpy(), dim, normalize=normalize)
    e = emb.double().cpu().numpy()
    assert np.isfinite(e).all()
    err = lo.procrustes_rel_error(e, ref)
    assert err < tol, err
    assert lo.rel_sv_error(S[:dim], Sref[:dim]) < tol
    # FP64 sweeps after the FP32 ones: until they converge in the FP32 form,
    # one in the 16-bit forms (by default)
    assert st["jacobi_sweeps_fp32"] > 0
    assert st["jacobi_sweeps"] > 0 if precision == "fp32" else st["jacobi_sweeps"] == 1


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_core_svd_one_fp64_sweep(ctx, netsmf_matrix, precision):
    # one FP64 sweep after the FP32 ones gives the embedding of the FP64
    # sweeps run to convergence, to far below the forms' tolerances
    csr, A, _ = netsmf_matrix
    rank, dim, seed = 48, 32, 777
    out = {}
    try:
        for mode in (1, 0):
            ctx.set_core_svd_fp64(mode)
            out[mode] = randsvd(ctx, csr, rank, dim, precision=precision, seed=seed)
    finally:
        ctx.set_core_svd_fp64(-1)
    (e1, S1, st1), (e0, S0, st0) = out[1], out[0]
    assert st0["jacobi_sweeps"] == 1 and st1["jacobi_sweeps"] >= 1
    assert lo.procrustes_rel_error(e0.double().cpu().numpy(), e1.double().cpu().numpy()) < 1e-5
    assert lo.rel_sv_error(S0[:dim], S1[:dim]) < 1e-8
    if precision == "fp32":
        om = gaussian(ctx, seed, 0, A.shape[0], rank)
        P = gaussian(ctx, seed, 1, rank, rank)
        ref, _ = lo.randsvd(A, om.double().cpu().numpy(), P.double().cpu().numpy(), dim)
        assert lo.procrustes_rel_error(e0.double().cpu().numpy(), ref) < 1e-4


def test_random_project_only(ctx, netsmf_matrix):
    csr, A, _ = netsmf_matrix
    emb, S, _ = randsvd(ctx, csr, 40, 24, random_project_only=True, seed=9)
    om = gaussian(ctx, 9, 0, A.shape[0], 40).double().cpu().numpy()
    ref, _ = lo.randsvd(A, om, None, 24, random_project_only=True)
    np.testing.assert_allclose(emb.double().cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * np.abs(ref).max())


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("fp16", 1e-3), ("bf16", 3e-3)])
@pytest.mark.parametrize("order,dim", [(10, 128), (10, 20), (2, 16), (3, 16)])
def test_propagate_matches_fp64(ctx, netsmf_matrix, precision, tol, order, dim):
    _, _, (off, nbrs) = netsmf_matrix
    g = Graph.from_numpy(ctx, off, nbrs)
    a = np.random.default_rng(3).standard_normal((off.size - 1, dim)).astype(np.float32)
    y, a2, _ = chebyshev_expansion(ctx, g, a, dim, order=order, precision=precision, return_a=True)
    yref, a2ref = lo.propagate(off, nbrs, a, order=order)
    y = y.double().cpu().numpy()
    rel = np.linalg.norm(y - yref) / np.linalg.norm(yref)
    assert rel < tol, rel
    rel2 = np.linalg.norm(a2.double().cpu().numpy() - a2ref) / np.linalg.norm(a2ref)
    assert rel2 < tol, rel2
    g.free()


@pytest.mark.parametrize("scale", [1e-6, 1.0, 3e3])
def test_propagate_fp16_input_scaling(ctx, netsmf_matrix, scale):
    """The FP16 form scales its input by a power of two into FP16's range:
    inputs far below or above it give the same relative error."""
    _, _, (off, nbrs) = netsmf_matrix
    g = Graph.from_numpy(ctx, off, nbrs)
    a = (scale * np.random.default_rng(5).standard_normal((off.size - 1, 32))).astype(np.float32)
    y, a2, _ = chebyshev_expansion(ctx, g, a, 32, order=10, precision="fp16", return_a=True)
    yref, a2ref = lo.propagate(off, nbrs, a, order=10)
    y = y.double().cpu().numpy()
    assert np.isfinite(y).all()
    rel = np.linalg.norm(y - yref) / np.linalg.norm(yref)
    assert rel < 1e-3, rel
    g.free()


def test_propagate_long_rows(ctx):
    # a star: the hub's adjacency row exceeds the SpMM chunk (2048 entries)
    off, nbrs = graphs.star_graph(9000)
    g = Graph.from_numpy(ctx, off, nbrs)
    a = np.random.default_rng(4).standard_normal((9000, 24)).astype(np.float32)
    y, _ = chebyshev_expansion(ctx, g, a, 24, order=10)
    yref, _ = lo.propagate(off, nbrs, a, order=10)
    rel = np.linalg.norm(y.double().cpu().numpy() - yref) / np.linalg.norm(yref)
    assert rel < 1e-5, rel
    g.free()


@pytest.mark.parametrize("dim", [16, 64, 128])
def test_dense_embed_matches_fp64(ctx, dim):
    rng = np.random.default_rng(dim)
    n = 5000
    U, _ = np.linalg.qr(rng.standard_normal((n, dim)))
    V, _ = np.linalg.qr(rng.standard_normal((dim, dim)))
    s = np.logspace(0, -2.5, dim)
    x = (U * s) @ V.T
    emb, S = get_embedding_dense(ctx, x.astype(np.float32), dim)
    ref, Sref = lo.dense_embed(x.astype(np.float32))
    err = lo.procrustes_rel_error(emb.double().cpu().numpy(), ref)
    assert err < 1e-4, err
    assert lo.rel_sv_error(S, Sref) < 1e-4
    nr = np.linalg.norm(emb.double().cpu().numpy(), axis=1)
    np.testing.assert_allclose(nr, 1.0, rtol=1e-5)
    # with one FP64 sweep
    try:
        ctx.set_core_svd_fp64(0)
        emb0, S0 = get_embedding_dense(ctx, x.astype(np.float32), dim)
    finally:
        ctx.set_core_svd_fp64(-1)
    assert lo.procrustes_rel_error(emb0.double().cpu().numpy(), ref) < 1e-4
    assert lo.rel_sv_error(S0, Sref) < 1e-4
