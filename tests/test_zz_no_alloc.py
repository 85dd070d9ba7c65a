"""The allocation-free Gram (lne_gram_noalloc): for callers that cannot
allocate device memory when they need A^T B (their device memory belongs to
another allocator, or they run under a hard memory cap).  Checked through
the C ABI against lne_gram on two calls in a row (the fixed scratch array
keeps the previous call's contents), with the same tolerance as the other
Gram tests, and its size limit.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from lightne_gb300._lib import LNE_ERR_UNSUPPORTED

pytestmark = pytest.mark.gpu


def _gram(lib, ctx, fn, dA, lda, c1, dB, ldb, c2, n):
    dG = torch.full((c1, c2), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = fn(ctx.handle, ctypes.c_void_p(dA.data_ptr()), lda, c1, ctypes.c_void_p(dB.data_ptr()), ldb, c2, n,
            ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    return dG.cpu().numpy()


def test_gram_noalloc_matches_gram_on_two_calls(ctx, lib):
    for call, (n, c1, c2) in enumerate([(60000, 138, 138), (20000, 100, 40)]):
        rng = np.random.default_rng(100 + call)
        lda, ldb = (c1 + 7) // 8 * 8, (c2 + 7) // 8 * 8
        A = np.zeros((n, lda), np.float32)
        B = np.zeros((n, ldb), np.float32)
        A[:, :c1] = rng.standard_normal((n, c1))
        B[:, :c2] = rng.standard_normal((n, c2))
        dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        ref = _gram(lib, ctx, lib.lne_gram, dA, lda, c1, dB, ldb, c2, n)
        got = _gram(lib, ctx, lib.lne_gram_noalloc, dA, lda, c1, dB, ldb, c2, n)
        bound = 2e-6 * (np.abs(A[:, :c1]).astype(np.float64).T @ np.abs(B[:, :c2]).astype(np.float64))
        assert np.isfinite(got).all()
        assert (np.abs(got - ref) <= bound).all(), (np.abs(got - ref) / bound).max()


def test_gram_noalloc_rejects_oversize(ctx, lib):
    n, c = 2048 * 300, 128  # 300 * 128 * 128 partial sums > 4,194,304
    dA = torch.zeros((1, c), device="cuda")
    dG = torch.zeros((c, c), dtype=torch.float64, device="cuda")
    rc = lib.lne_gram_noalloc(ctx.handle, ctypes.c_void_p(dA.data_ptr()), c, c, ctypes.c_void_p(dA.data_ptr()), c, c,
                              n, ctypes.c_void_p(dG.data_ptr()))
    assert rc == LNE_ERR_UNSUPPORTED
    assert b"16 MiB" in lib.lne_last_error()
