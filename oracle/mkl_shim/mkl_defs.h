/*
 * Test infrastructure (oracle): definitions, for the oracle harnesses only,
 * of the few MKL routines the reference's spectral propagation calls
 * (LightNE/SpectralPropagation.h:45-229 through
 * LightNE/mklredsvd/mklhelper.h): the CSR handle, the sparse x dense product,
 * the BLAS-1 calls and the dense SVD of get_embedding_dense.  Include it after
 * the declarations-only mkl.h and before the reference headers.
 *
 * They follow MKL's documented semantics, not its arithmetic (MKL is not
 * available here): mkl_sparse_?_mm computes y = alpha * A x + beta * y for a
 * GENERAL, non-transposed, row-major CSR with each row's sum in CSR order in
 * the operand type; LAPACKE_?gesvd (jobu 'S', jobvt 'N', row-major) is a
 * one-sided Jacobi SVD in double, and records its input matrix so that the
 * harness can write the (A + I)(a - conv) product the reference passes to it.
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <numeric>
#include <vector>

struct sparse_matrix {
  MKL_INT rows, cols;
  const MKL_INT* rows_start;
  const MKL_INT* rows_end;
  const MKL_INT* col;
  const void* val;
};

namespace lne_shim {

// The last matrix handed to LAPACKE_?gesvd (row-major, as doubles).
inline std::vector<double>& last_svd_input() {
  static std::vector<double> v;
  return v;
}

template <class FP>
sparse_status_t create_csr(sparse_matrix_t* A, MKL_INT rows, MKL_INT cols, MKL_INT* rows_start, MKL_INT* rows_end,
                           MKL_INT* col, FP* val) {
  *A = new sparse_matrix{rows, cols, rows_start, rows_end, col, val};
  return SPARSE_STATUS_SUCCESS;
}

template <class FP>
sparse_status_t mm(sparse_operation_t op, FP alpha, const sparse_matrix_t A, matrix_descr descr,
                   sparse_layout_t layout, const FP* x, MKL_INT columns, MKL_INT ldx, FP beta, FP* y, MKL_INT ldy) {
  if (op != SPARSE_OPERATION_NON_TRANSPOSE || layout != SPARSE_LAYOUT_ROW_MAJOR ||
      descr.type != SPARSE_MATRIX_TYPE_GENERAL)
    return SPARSE_STATUS_NOT_INITIALIZED;
  const FP* val = static_cast<const FP*>(A->val);
  std::vector<FP> acc(columns);
  for (MKL_INT i = 0; i < A->rows; ++i) {
    std::fill(acc.begin(), acc.end(), FP(0));
    for (MKL_INT e = A->rows_start[i]; e < A->rows_end[i]; ++e) {
      const FP v = val[e];
      const FP* xr = x + A->col[e] * ldx;
      for (MKL_INT j = 0; j < columns; ++j) acc[j] += v * xr[j];
    }
    FP* yr = y + i * ldy;
    for (MKL_INT j = 0; j < columns; ++j) yr[j] = beta == FP(0) ? alpha * acc[j] : alpha * acc[j] + beta * yr[j];
  }
  return SPARSE_STATUS_SUCCESS;
}

// One-sided Jacobi SVD of the m x n row-major a (m >= n): U (m x n, ldu), S
// descending; V is not formed (jobvt 'N').
template <class FP>
lapack_int gesvd_s_n(lapack_int m, lapack_int n, const FP* a, lapack_int lda, FP* s, FP* u, lapack_int ldu) {
  std::vector<double> W((size_t)m * n);
  for (lapack_int i = 0; i < m; ++i)
    for (lapack_int j = 0; j < n; ++j) W[(size_t)j * m + i] = (double)a[i * lda + j];  // column j contiguous
  last_svd_input().assign((size_t)m * n, 0.0);
  for (lapack_int i = 0; i < m; ++i)
    for (lapack_int j = 0; j < n; ++j) last_svd_input()[(size_t)i * n + j] = (double)a[i * lda + j];
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (lapack_int p = 0; p < n; ++p)
      for (lapack_int q = p + 1; q < n; ++q) {
        double* x = &W[(size_t)p * m];
        double* y = &W[(size_t)q * m];
        double app = 0, aqq = 0, apq = 0;
        for (lapack_int i = 0; i < m; ++i) {
          app += x[i] * x[i];
          aqq += y[i] * y[i];
          apq += x[i] * y[i];
        }
        if (app == 0.0 || aqq == 0.0) continue;
        const double c0 = std::fabs(apq) / std::sqrt(app * aqq);
        off = std::max(off, c0);
        if (c0 < 1e-15) continue;
        const double zeta = (aqq - app) / (2.0 * apq);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
        for (lapack_int i = 0; i < m; ++i) {
          const double xi = x[i], yi = y[i];
          x[i] = c * xi - sn * yi;
          y[i] = sn * xi + c * yi;
        }
      }
    if (off < 1e-15) break;
  }
  std::vector<double> nrm(n);
  for (lapack_int j = 0; j < n; ++j) {
    double t = 0;
    for (lapack_int i = 0; i < m; ++i) t += W[(size_t)j * m + i] * W[(size_t)j * m + i];
    nrm[j] = std::sqrt(t);
  }
  std::vector<lapack_int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](lapack_int p, lapack_int q) { return nrm[p] > nrm[q]; });
  for (lapack_int k = 0; k < n; ++k) {
    const lapack_int j = ord[k];
    s[k] = (FP)nrm[j];
    for (lapack_int i = 0; i < m; ++i) u[i * ldu + k] = (FP)(nrm[j] > 0 ? W[(size_t)j * m + i] / nrm[j] : 0.0);
  }
  return 0;
}

}  // namespace lne_shim

// Plain functions: overload resolution prefers them over the variadic
// declarations of mkl.h.
inline sparse_status_t mkl_sparse_optimize(sparse_matrix_t) { return SPARSE_STATUS_SUCCESS; }
inline sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
  delete A;
  return SPARSE_STATUS_SUCCESS;
}
inline sparse_status_t mkl_sparse_s_create_csr(sparse_matrix_t* M, sparse_index_base_t, MKL_INT r, MKL_INT c,
                                               MKL_INT* rs, MKL_INT* re, MKL_INT* ci, float* v) {
  return lne_shim::create_csr(M, r, c, rs, re, ci, v);
}
inline sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t* M, sparse_index_base_t, MKL_INT r, MKL_INT c,
                                               MKL_INT* rs, MKL_INT* re, MKL_INT* ci, double* v) {
  return lne_shim::create_csr(M, r, c, rs, re, ci, v);
}
inline sparse_status_t mkl_sparse_s_mm(sparse_operation_t op, float alpha, sparse_matrix_t M, matrix_descr d,
                                       sparse_layout_t l, const float* x, MKL_INT cols, MKL_INT ldx, float beta,
                                       float* y, MKL_INT ldy) {
  return lne_shim::mm<float>(op, alpha, M, d, l, x, cols, ldx, beta, y, ldy);
}
inline sparse_status_t mkl_sparse_d_mm(sparse_operation_t op, double alpha, sparse_matrix_t M, matrix_descr d,
                                       sparse_layout_t l, const double* x, MKL_INT cols, MKL_INT ldx, double beta,
                                       double* y, MKL_INT ldy) {
  return lne_shim::mm<double>(op, alpha, M, d, l, x, cols, ldx, beta, y, ldy);
}
inline void cblas_saxpy(MKL_INT n, float a, const float* x, MKL_INT incx, float* y, MKL_INT incy) {
  for (MKL_INT i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}
inline void cblas_scopy(MKL_INT n, const float* x, MKL_INT incx, float* y, MKL_INT incy) {
  for (MKL_INT i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}
inline void cblas_sscal(MKL_INT n, float a, float* x, MKL_INT incx) {
  for (MKL_INT i = 0; i < n; ++i) x[i * incx] *= a;
}
inline float cblas_snrm2(MKL_INT n, const float* x, MKL_INT incx) {
  double t = 0;
  for (MKL_INT i = 0; i < n; ++i) t += (double)x[i * incx] * x[i * incx];
  return (float)std::sqrt(t);
}
inline lapack_int LAPACKE_sgesvd(int layout, char jobu, char jobvt, lapack_int m, lapack_int n, float* a,
                                 lapack_int lda, float* s, float* u, lapack_int ldu, float*, lapack_int, float*) {
  if (layout != LAPACK_ROW_MAJOR || jobu != 'S' || jobvt != 'N' || m < n) return -1;
  return lne_shim::gesvd_s_n<float>(m, n, a, lda, s, u, ldu);
}

// ---------------------------------------------------------------------------
// The randomized SVD (LightNE/mklredsvd/mklredsvd.cc:93-403, util.cc:21-79).
// ---------------------------------------------------------------------------
namespace lne_shim {

// The Gaussian stream: vsRngGaussian hands out the values the harness
// queued, in order (the reference draws Omega, then P, from one stream).
inline std::vector<float>& gaussian_queue() {
  static std::vector<float> q;
  return q;
}
inline size_t& gaussian_pos() {
  static size_t p = 0;
  return p;
}

// Householder QR in double of the row-major m x n a (m >= n): geqrf keeps
// the factors aside; orgqr writes the thin Q (m x n) into a.  R's diagonal
// takes LAPACK's sign (-sign(a_kk) |x|).
inline std::vector<double>& qr_q() {
  static std::vector<double> q;
  return q;
}
template <class FP>
lapack_int geqrf(lapack_int m, lapack_int n, FP* a, lapack_int lda) {
  if (m < n) return -2;
  std::vector<double> A((size_t)m * n);
  for (lapack_int i = 0; i < m; ++i)
    for (lapack_int j = 0; j < n; ++j) A[(size_t)j * m + i] = (double)a[i * lda + j];  // column-major
  std::vector<double> V((size_t)m * n, 0.0), beta(n, 0.0);
  for (lapack_int k = 0; k < n; ++k) {
    double* x = &A[(size_t)k * m];
    double nrm = 0;
    for (lapack_int i = k; i < m; ++i) nrm += x[i] * x[i];
    nrm = std::sqrt(nrm);
    double* v = &V[(size_t)k * m];
    if (nrm == 0.0) continue;
    const double alpha = x[k] >= 0 ? -nrm : nrm;
    for (lapack_int i = k; i < m; ++i) v[i] = x[i];
    v[k] -= alpha;
    double vv = 0;
    for (lapack_int i = k; i < m; ++i) vv += v[i] * v[i];
    beta[k] = vv > 0 ? 2.0 / vv : 0.0;
    for (lapack_int j = k; j < n; ++j) {
      double* y = &A[(size_t)j * m];
      double d = 0;
      for (lapack_int i = k; i < m; ++i) d += v[i] * y[i];
      d *= beta[k];
      for (lapack_int i = k; i < m; ++i) y[i] -= d * v[i];
    }
  }
  // Q = H_0 H_1 ... H_{n-1} applied to the first n columns of I
  std::vector<double>& Q = qr_q();
  Q.assign((size_t)m * n, 0.0);
  for (lapack_int j = 0; j < n; ++j) Q[(size_t)j * m + j] = 1.0;
  for (lapack_int k = n - 1; k >= 0; --k) {
    const double* v = &V[(size_t)k * m];
    for (lapack_int j = 0; j < n; ++j) {
      double* y = &Q[(size_t)j * m];
      double d = 0;
      for (lapack_int i = k; i < m; ++i) d += v[i] * y[i];
      d *= beta[k];
      for (lapack_int i = k; i < m; ++i) y[i] -= d * v[i];
    }
  }
  for (lapack_int i = 0; i < m; ++i)
    for (lapack_int j = 0; j < n; ++j) a[i * lda + j] = (FP)(j >= i ? A[(size_t)j * m + i] : 0.0);
  return 0;
}
template <class FP>
lapack_int orgqr(lapack_int m, lapack_int n, FP* a, lapack_int lda) {
  const std::vector<double>& Q = qr_q();
  if ((lapack_int)Q.size() != m * n) return -1;
  for (lapack_int i = 0; i < m; ++i)
    for (lapack_int j = 0; j < n; ++j) a[i * lda + j] = (FP)Q[(size_t)j * m + i];
  return 0;
}

}  // namespace lne_shim

inline void* mkl_calloc(MKL_INT num, size_t size, int) { return std::calloc((size_t)num, size); }
template <class T>
inline void mkl_free(T* p) {
  std::free((void*)p);
}
inline int vslNewStream(VSLStreamStatePtr* s, int, int) {
  *s = (VSLStreamStatePtr)&lne_shim::gaussian_pos();
  return VSL_STATUS_OK;
}
inline int vslDeleteStream(VSLStreamStatePtr*) { return VSL_STATUS_OK; }
inline int vsRngGaussian(MKL_INT, VSLStreamStatePtr, MKL_INT n, float* r, float a, float sigma) {
  std::vector<float>& q = lne_shim::gaussian_queue();
  size_t& p = lne_shim::gaussian_pos();
  if (p + (size_t)n > q.size()) return -1;
  for (MKL_INT i = 0; i < n; ++i) r[i] = a + sigma * q[p + (size_t)i];
  p += (size_t)n;
  return VSL_STATUS_OK;
}
inline sparse_status_t mkl_sparse_set_mm_hint(sparse_matrix_t, sparse_operation_t, matrix_descr, sparse_layout_t,
                                              MKL_INT, MKL_INT) {
  return SPARSE_STATUS_SUCCESS;
}
inline sparse_status_t mkl_sparse_set_memory_hint(sparse_matrix_t, sparse_memory_usage_t) {
  return SPARSE_STATUS_SUCCESS;
}
inline lapack_int LAPACKE_sgeqrf(int layout, lapack_int m, lapack_int n, float* a, lapack_int lda, float*) {
  if (layout != LAPACK_ROW_MAJOR) return -1;
  return lne_shim::geqrf<float>(m, n, a, lda);
}
inline lapack_int LAPACKE_sorgqr(int layout, lapack_int m, lapack_int n, lapack_int, float* a, lapack_int lda,
                                 const float*) {
  if (layout != LAPACK_ROW_MAJOR) return -1;
  return lne_shim::orgqr<float>(m, n, a, lda);
}
// Row-major C = alpha op(A) op(B) + beta C, FP32 sums in k order.
inline void cblas_sgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, MKL_INT m, MKL_INT n, MKL_INT k,
                        float alpha, const float* a, MKL_INT lda, const float* b, MKL_INT ldb, float beta, float* c,
                        MKL_INT ldc) {
  if (layout != CblasRowMajor) std::abort();
  for (MKL_INT i = 0; i < m; ++i)
    for (MKL_INT j = 0; j < n; ++j) {
      float s = 0.0f;
      for (MKL_INT p = 0; p < k; ++p) {
        const float x = ta == CblasNoTrans ? a[i * lda + p] : a[p * lda + i];
        const float y = tb == CblasNoTrans ? b[p * ldb + j] : b[j * ldb + p];
        s += x * y;
      }
      c[i * ldc + j] = beta == 0.0f ? alpha * s : alpha * s + beta * c[i * ldc + j];
    }
}

// Routines of run()'s sparse-projection branch (mklredsvd.cc:148-226), which
// the harness never takes: defined only so that run() links; reaching one
// is a harness error.
template <class... A>
int viRngBinomial(A...) {
  std::abort();
}
template <class... A>
sparse_status_t mkl_sparse_s_spmmd(A...) {
  std::abort();
}
