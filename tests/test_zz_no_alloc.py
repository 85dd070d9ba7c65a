"""The allocation-free Gram (lne_gram_noalloc): for callers that cannot
allocate device memory when they need A^T B (their device memory belongs to
another allocator, or they run under a hard memory cap).  Checked through
the C ABI against an FP64 NumPy product, with the bound of the other Gram
tests (|err| <= 2e-6 x (|A|^T |B|) elementwise), and against lne_gram, on
calls in a row that share the fixed scratch array (each keeps the previous
call's contents): the tensor-core Gram of two operands, the symmetric A^T A
form (one pointer for both), a leading dimension off the 16-byte grid (the
CUDA-core Gram), a B wider than the tensor-core path takes, and n = 0.
Then the size limit, and that the caller's current device is kept.
Collected last on purpose: its module-scope array is set up by its first
call, after every other test has run."""
import ctypes

import numpy as np
import pytest
import torch

from lightne_gb300._lib import LNE_ERR_UNSUPPORTED

pytestmark = pytest.mark.gpu


def _call(lib, ctx, fn, dA, lda, c1, dB, ldb, c2, n):
    dG = torch.full((c1, c2), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = fn(ctx.handle, ctypes.c_void_p(dA.data_ptr()), lda, c1, ctypes.c_void_p(dB.data_ptr()), ldb, c2, n,
            ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    return dG.cpu().numpy()


# (n, c1, c2, lda, ldb, same): same = B is A (one pointer, the A^T A form)
CASES = [
    (60000, 138, 138, 144, 144, False),  # tensor-core Gram of two operands
    (60000, 144, 144, 144, 144, True),   # symmetric tensor-core Gram
    (20000, 37, 29, 37, 29, False),      # rows off the 16-byte grid: CUDA-core Gram
    (4096, 40, 300, 40, 304, False),     # B wider than 256 columns: CUDA-core Gram
    (0, 24, 16, 24, 16, False),          # no rows: G = 0
]


def test_gram_noalloc_matches_fp64_on_calls_in_a_row(ctx, lib):
    for call, (n, c1, c2, lda, ldb, same) in enumerate(CASES):
        rng = np.random.default_rng(100 + call)
        A = np.zeros((max(n, 1), lda), np.float32)
        A[:n, :c1] = rng.standard_normal((n, c1))
        if same:
            B = A
        else:
            B = np.zeros((max(n, 1), ldb), np.float32)
            B[:n, :c2] = rng.standard_normal((n, c2))
        dA = torch.from_numpy(A).cuda()
        dB = dA if same else torch.from_numpy(B).cuda()
        got = _call(lib, ctx, lib.lne_gram_noalloc, dA, lda, c1, dB, ldb, c2, n)
        ref = A[:n, :c1].astype(np.float64).T @ B[:n, :c2].astype(np.float64)
        bound = 2e-6 * (np.abs(A[:n, :c1]).astype(np.float64).T @ np.abs(B[:n, :c2]).astype(np.float64))
        assert np.isfinite(got).all(), call
        assert (np.abs(got - ref) <= bound).all(), (call, (np.abs(got - ref) / np.maximum(bound, 1e-300)).max())
        if n > 0:
            base = _call(lib, ctx, lib.lne_gram, dA, lda, c1, dB, ldb, c2, n)
            assert (np.abs(got - base) <= 2 * bound).all(), call
        else:
            assert (got == 0).all()


def test_gram_noalloc_rejects_oversize(ctx, lib):
    n, c = 2048 * 300, 128  # 300 * 128 * 128 partial sums > 4,194,304
    dA = torch.zeros((1, c), device="cuda")
    dG = torch.zeros((c, c), dtype=torch.float64, device="cuda")
    rc = lib.lne_gram_noalloc(ctx.handle, ctypes.c_void_p(dA.data_ptr()), c, c, ctypes.c_void_p(dA.data_ptr()), c, c,
                              n, ctypes.c_void_p(dG.data_ptr()))
    assert rc == LNE_ERR_UNSUPPORTED
    assert b"16 MiB" in lib.lne_last_error()


def test_gram_noalloc_keeps_current_device(ctx, lib):
    dA = torch.ones((2048, 8), device="cuda")
    dG = torch.zeros((8, 8), dtype=torch.float64, device="cuda")
    before = torch.cuda.current_device()
    rc = lib.lne_gram_noalloc(ctx.handle, ctypes.c_void_p(dA.data_ptr()), 8, 8, ctypes.c_void_p(dA.data_ptr()), 8,
                              8, 2048, ctypes.c_void_p(dG.data_ptr()))
    assert rc == 0, lib.lne_last_error()
    assert torch.cuda.current_device() == before
    assert (dG.cpu().numpy() == 2048.0).all()
