// Very sparse random projection sketch (-sparse_project) of the randomized SVD.
#pragma once
#include <stdint.h>

#include "lne_internal.h"

namespace lne {

// The sketch O (n x rank) in CSR on the device.
struct SparseProjection {
  lne_ctx* ctx = nullptr;
  int64_t n = 0;
  int rank = 0;
  int64_t nnz = 0;
  int64_t* rp = nullptr;   // [n + 1]
  int32_t* col = nullptr;  // [nnz], ascending within a row
  float* val = nullptr;    // [nnz], +-sqrt(s)
  ~SparseProjection();
};

// s (sqrt(n) unless s_flag >= 1), the density 1/s and the value sqrt(s).
void sparse_projection_scale(int64_t n, double s_flag, float* s, double* density, float* value);
// Draws O for the seed (synchronises once, to size the arrays).
int sparse_projection_build(lne_ctx* ctx, int64_t n, int rank, uint64_t seed, double s_flag, SparseProjection* O,
                            int* launches);
// Y (n x ld, FP32) = A O; columns rank..ld-1 of Y are written as zeros.
int sparse_projection_product(lne_ctx* ctx, const lne_csr* A, const SparseProjection& O, float* Y, int64_t ld,
                              int* launches);
// O as a dense n x ld matrix.
int sparse_projection_dense(lne_ctx* ctx, const SparseProjection& O, float* out, int64_t ld);

}  // namespace lne
