"""Tensor-core (tcgen05, split-TF32) tall GEMM and Gram (lne_gemm_tall,
lne_gram) against FP64 products.  Tolerance: FP32-level, |err| <= 2e-6 x
(|In| |W|) elementwise for the GEMM, <= 2e-6 x (|A|^T |B|) for the Gram."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k,c2,ldo", [(1000, 138, 138, 144), (5000, 144, 128, 128), (300, 16, 16, 16),
                                        (4097, 8, 200, 200), (2000, 130, 256, 256), (1500, 40, 300, 304)])
def test_gemm_tall(ctx, lib, n, k, c2, ldo):
    rng = np.random.default_rng(n + k + c2)
    ldi = (k + 7) // 8 * 8
    In = np.zeros((n, ldi), np.float32)
    In[:, :k] = rng.standard_normal((n, k))
    W = rng.standard_normal((k, c2)).astype(np.float32)
    dIn, dW = torch.from_numpy(In).cuda(), torch.from_numpy(W).cuda()
    dOut = torch.full((n, ldo), 7.0, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lne_gemm_tall(ctx.handle, ctypes.c_void_p(dIn.data_ptr()), ldi, k, ctypes.c_void_p(dW.data_ptr()), c2,
                           n, ctypes.c_void_p(dOut.data_ptr()), ldo)
    assert rc == 0, lib.lne_last_error()
    out = dOut.cpu().numpy()
    ref = In[:, :k].astype(np.float64) @ W.astype(np.float64)
    bound = 2e-6 * (np.abs(In[:, :k]).astype(np.float64) @ np.abs(W).astype(np.float64)) + 1e-30
    err = np.abs(out[:, :c2] - ref)
    assert (err <= bound).all(), (err / bound).max()
    assert (out[:, c2:] == 0).all()


@pytest.mark.parametrize("n,c1,c2", [(10000, 138, 138), (4096, 128, 128), (2049, 16, 16), (3000, 200, 40),
                                     (7000, 144, 256), (1000, 60, 270)])
def test_gram(ctx, lib, n, c1, c2):
    rng = np.random.default_rng(n + c1)
    lda, ldb = (c1 + 7) // 8 * 8, (c2 + 7) // 8 * 8
    A = np.zeros((n, lda), np.float32)
    B = np.zeros((n, ldb), np.float32)
    A[:, :c1] = rng.standard_normal((n, c1))
    B[:, :c2] = rng.standard_normal((n, c2))
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dG = torch.zeros((c1, c2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lne_gram(ctx.handle, ctypes.c_void_p(dA.data_ptr()), lda, c1, ctypes.c_void_p(dB.data_ptr()), ldb, c2,
                      n, ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    G = dG.cpu().numpy()
    ref = A[:, :c1].astype(np.float64).T @ B[:, :c2].astype(np.float64)
    bound = 2e-6 * (np.abs(A[:, :c1]).astype(np.float64).T @ np.abs(B[:, :c2]).astype(np.float64))
    assert (np.abs(G - ref) <= bound).all(), (np.abs(G - ref) / bound).max()


@pytest.mark.parametrize("n,c", [(10000, 138), (4096, 128), (2049, 16), (33, 144), (1, 138), (7001, 250),
                                 (200003, 144), (50001, 131), (5000, 160), (3000, 100), (70, 7)])
def test_gram_symmetric(ctx, lib, n, c):
    """A^T A with the same pointer for both operands (the CholeskyQR case):
    the second 128-column tile only computes columns >= 128 and the rest
    is mirrored, so the result is exactly symmetric."""
    rng = np.random.default_rng(n + 7 * c)
    lda = (c + 7) // 8 * 8
    A = np.zeros((n, lda), np.float32)
    A[:, :c] = rng.standard_normal((n, c))
    dA = torch.from_numpy(A).cuda()
    dG = torch.zeros((c, c), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    p = ctypes.c_void_p(dA.data_ptr())
    rc = lib.lne_gram(ctx.handle, p, lda, c, p, lda, c, n, ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    G = dG.cpu().numpy()
    A64 = A[:, :c].astype(np.float64)
    ref = A64.T @ A64
    bound = 2e-6 * (np.abs(A64).T @ np.abs(A64))
    assert (np.abs(G - ref) <= bound).all(), (np.abs(G - ref) / bound).max()
    assert (G == G.T).all()


@pytest.mark.parametrize("n,c1,c2", [(3001, 137, 137), (999, 61, 45)])
def test_gram_unaligned_rows(ctx, lib, n, c1, c2):
    """Row strides that are not a multiple of 16 bytes take the per-block
    tensor-core Gram instead of the streaming one; same result bound."""
    rng = np.random.default_rng(n)
    lda, ldb = c1 + 1, c2 + 2
    A = rng.standard_normal((n, lda)).astype(np.float32)
    B = rng.standard_normal((n, ldb)).astype(np.float32)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dG = torch.zeros((c1, c2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lne_gram(ctx.handle, ctypes.c_void_p(dA.data_ptr()), lda, c1, ctypes.c_void_p(dB.data_ptr()), ldb, c2,
                      n, ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    A64, B64 = A[:, :c1].astype(np.float64), B[:, :c2].astype(np.float64)
    ref = A64.T @ B64
    bound = 2e-6 * (np.abs(A64).T @ np.abs(B64))
    G = dG.cpu().numpy()
    assert (np.abs(G - ref) <= bound).all(), (np.abs(G - ref) / bound).max()


@pytest.mark.parametrize("n,k,c2,ldi", [(3001, 137, 137, 138), (130, 5, 20, 7), (200003, 138, 138, 144),
                                        (257, 138, 128, 144)])
def test_gemm_tall_shapes(ctx, lib, n, k, c2, ldi):
    """Ragged tiles (n not a multiple of 128), K not a multiple of 16, and
    row strides that are not 16-byte multiples (per-tile kernel)."""
    rng = np.random.default_rng(n + k)
    In = rng.standard_normal((n, ldi)).astype(np.float32)
    W = rng.standard_normal((k, c2)).astype(np.float32)
    ldo = c2
    dIn, dW = torch.from_numpy(In).cuda(), torch.from_numpy(W).cuda()
    dOut = torch.full((n, ldo), 7.0, device="cuda")
    torch.cuda.synchronize()
    rc = lib.lne_gemm_tall(ctx.handle, ctypes.c_void_p(dIn.data_ptr()), ldi, k, ctypes.c_void_p(dW.data_ptr()), c2,
                           n, ctypes.c_void_p(dOut.data_ptr()), ldo)
    assert rc == 0, lib.lne_last_error()
    out = dOut.cpu().numpy()
    I64 = In[:, :k].astype(np.float64)
    ref = I64 @ W.astype(np.float64)
    bound = 2e-6 * (np.abs(I64) @ np.abs(W).astype(np.float64)) + 1e-30
    err = np.abs(out - ref)
    assert (err <= bound).all(), (err / bound).max()
