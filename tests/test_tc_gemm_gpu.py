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
