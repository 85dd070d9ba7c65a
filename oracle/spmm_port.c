/*
 * ORACLE — test infrastructure, not product code.
 *
 * Row-parallel CSR x dense products on the host cores (OpenMP), for the FP64
 * oracle of the dense stages and for the timed CPU baseline of the
 * reference's dense stages.  Only tests/, __graft_entry__.smoke() and the
 * CPU legs of bench.py load this library.
 *
 * Reference correspondence (paths inside the reference project): the
 * products the reference hands to MKL's sparse inspector-executor,
 * mkl_sparse_s_mm with SPARSE_LAYOUT_ROW_MAJOR and a GENERAL descriptor
 * (LightNE/mklredsvd/mklredsvd.cc:233-251, :270-283; the propagation's
 * operator products, LightNE/SpectralPropagation.h:94-221): Y = A X for a
 * row-major dense X.  Each output row is one thread's sum over its row's
 * nonzeros in CSR order.
 */
#include <stdint.h>
#include <omp.h>

/* Y[i, 0:d] = sum_j A[i, j] X[j, 0:d] for rows i in [r0, r1); FP32. */
void lne_port_spmm_f32(int64_t r0, int64_t r1, const int64_t* rp, const int32_t* col, const float* val,
                       const float* X, int64_t ldx, int64_t d, float* Y, int64_t ldy, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = r0; i < r1; ++i) {
    float* y = Y + i * ldy;
    for (int64_t k = 0; k < d; ++k) y[k] = 0.0f;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
      const float v = val[e];
      const float* x = X + (int64_t)col[e] * ldx;
      for (int64_t k = 0; k < d; ++k) y[k] += v * x[k];
    }
  }
}

/* The same product in FP64 (values, operand and sums), for the oracle. */
void lne_port_spmm_f64(int64_t r0, int64_t r1, const int64_t* rp, const int32_t* col, const double* val,
                       const double* X, int64_t ldx, int64_t d, double* Y, int64_t ldy, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = r0; i < r1; ++i) {
    double* y = Y + i * ldy;
    for (int64_t k = 0; k < d; ++k) y[k] = 0.0;
    for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
      const double v = val[e];
      const double* x = X + (int64_t)col[e] * ldx;
      for (int64_t k = 0; k < d; ++k) y[k] += v * x[k];
    }
  }
}
