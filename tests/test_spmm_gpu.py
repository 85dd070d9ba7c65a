"""lne_spmm (explicit CSR x dense, FP32, BF16, FP16 or FP8 dense operand) against an
FP64 numpy product of the same operands.  Tolerance: FP32 accumulation,
|err| <= 1e-5 * (|A| |X|) elementwise."""
import ctypes

import numpy as np
import pytest
import torch

from lightne_gb300 import _lib
from lightne_gb300._lib import LNE_PREC_BF16, LNE_PREC_FP8, LNE_PREC_FP16, LNE_PREC_FP32
from lightne_gb300.api import CSR

pytestmark = pytest.mark.gpu


def random_csr(n, avg, long_rows=(), seed=0):
    rng = np.random.default_rng(seed)
    lens = rng.poisson(avg, n).astype(np.int64)
    for r, L in long_rows:
        lens[r] = L
    lens = np.minimum(lens, n)
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    col = np.concatenate([np.sort(rng.choice(n, L, replace=False)) for L in lens]).astype(np.int32)
    val = rng.standard_normal(rp[-1]).astype(np.float32)
    return rp, col, val


DTYPES = {LNE_PREC_FP32: torch.float32, LNE_PREC_BF16: torch.bfloat16, LNE_PREC_FP8: torch.float8_e4m3fn,
          LNE_PREC_FP16: torch.float16}


@pytest.mark.parametrize("d,prec", [(128, LNE_PREC_FP32), (138, LNE_PREC_FP32), (20, LNE_PREC_FP32),
                                    (600, LNE_PREC_FP32), (128, LNE_PREC_BF16), (138, LNE_PREC_BF16),
                                    (60, LNE_PREC_BF16), (1100, LNE_PREC_BF16), (144, LNE_PREC_FP8),
                                    (138, LNE_PREC_FP8), (16, LNE_PREC_FP8), (700, LNE_PREC_FP8),
                                    (2100, LNE_PREC_FP8), (144, LNE_PREC_FP16), (138, LNE_PREC_FP16),
                                    (40, LNE_PREC_FP16)])
def test_spmm_matches_fp64(ctx, lib, d, prec):
    n = 3000
    rp, col, val = random_csr(n, 12, long_rows=[(5, 2500), (77, 2049), (2999, 2048)], seed=d)
    ld = (d + 15) // 16 * 16 if prec == LNE_PREC_FP8 else (d + 7) // 8 * 8
    rng = np.random.default_rng(1)
    X = np.zeros((n, ld), np.float32)
    X[:, :d] = rng.standard_normal((n, d)).astype(np.float32)
    dX = torch.from_numpy(X).to(DTYPES[prec]).cuda()
    Y0 = rng.standard_normal((n, ld)).astype(np.float32)
    dY = torch.from_numpy(Y0).cuda()
    d_rp, d_col, d_val = (torch.from_numpy(a).cuda() for a in (rp, col, val))
    A = CSR.wrap_device(ctx, n, int(rp[-1]), d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr())
    torch.cuda.synchronize()
    alpha, beta = 0.75, -0.5
    rc = lib.lne_spmm(ctx.handle, A.handle, prec, ctypes.c_void_p(dX.data_ptr()), ld, d, alpha, beta,
                      ctypes.c_void_p(dY.data_ptr()), ld)
    assert rc == 0, lib.lne_last_error()
    ctx.synchronize()
    got = dY.cpu().numpy()
    Xd = dX.cpu().to(torch.float64).numpy()  # the operand's values as stored
    import scipy.sparse as sp
    Am = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    ref = alpha * (Am @ Xd[:, :d]) + beta * Y0[:, :d].astype(np.float64)
    bound = 1e-5 * (abs(alpha) * (abs(Am) @ np.abs(Xd[:, :d])) + abs(beta) * np.abs(Y0[:, :d])) + 1e-30
    err = np.abs(got[:, :d] - ref)
    assert (err <= bound).all(), (err / bound).max()
    # columns beyond d are untouched
    assert np.array_equal(got[:, d:], Y0[:, d:])
    # bitwise reproducible
    dY2 = torch.from_numpy(Y0).cuda()
    lib.lne_spmm(ctx.handle, A.handle, prec, ctypes.c_void_p(dX.data_ptr()), ld, d, alpha, beta,
                 ctypes.c_void_p(dY2.data_ptr()), ld)
    ctx.synchronize()
    assert torch.equal(dY, dY2)
    A.free()


def test_spmm_rejects_misaligned(ctx, lib):
    n = 10
    rp = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    col = torch.zeros(1, dtype=torch.int32, device="cuda")
    val = torch.zeros(1, dtype=torch.float32, device="cuda")
    A = CSR.wrap_device(ctx, n, 0, rp.data_ptr(), col.data_ptr(), val.data_ptr())
    X = torch.zeros(n, 12, device="cuda")
    rc = lib.lne_spmm(ctx.handle, A.handle, LNE_PREC_FP32, ctypes.c_void_p(X.data_ptr()), 12, 12, 1.0, 0.0,
                      ctypes.c_void_p(X.data_ptr()), 12)
    assert rc == _lib.LNE_ERR_INVALID
    A.free()


@pytest.mark.parametrize("prec", [LNE_PREC_FP32, LNE_PREC_BF16])
def test_spmm_column_panels(ctx, lib, prec):
    # a panel budget far below the operand size forces many column panels
    n, d = 6000, 138
    rp, col, val = random_csr(n, 40, long_rows=[(3, 5000), (4000, 3000)], seed=7)
    ld = 144
    rng = np.random.default_rng(2)
    X = np.zeros((n, ld), np.float32)
    X[:, :d] = rng.standard_normal((n, d))
    dt = torch.float32 if prec == LNE_PREC_FP32 else torch.bfloat16
    dX = torch.from_numpy(X).to(dt).cuda()
    d_rp, d_col, d_val = (torch.from_numpy(a).cuda() for a in (rp, col, val))
    A = CSR.wrap_device(ctx, n, int(rp[-1]), d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr())
    outs = []
    for budget in (64 << 20, 100 * ld * 4, 777 * ld * 4):
        assert lib.lne_ctx_set_spmm_panel_bytes(ctx.handle, budget) == 0
        dY = torch.zeros((n, ld), device="cuda")
        torch.cuda.synchronize()
        rc = lib.lne_spmm(ctx.handle, A.handle, prec, ctypes.c_void_p(dX.data_ptr()), ld, d, 1.0, 0.0,
                          ctypes.c_void_p(dY.data_ptr()), ld)
        assert rc == 0, lib.lne_last_error()
        ctx.synchronize()
        outs.append(dY.cpu().numpy()[:, :d].astype(np.float64))
    lib.lne_ctx_set_spmm_panel_bytes(ctx.handle, 64 << 20)
    Xd = dX.cpu().to(torch.float64).numpy()  # the operand's values as stored
    import scipy.sparse as sp
    Am = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    ref = Am @ Xd[:, :d]
    bound = 1e-5 * (abs(Am) @ np.abs(Xd[:, :d])) + 1e-30
    for o in outs:
        assert (np.abs(o - ref) <= bound).all()
    A.free()
