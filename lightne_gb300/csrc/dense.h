// Dense building blocks of the randomized SVD and of the dense embedding
// (host-side launchers; all work on ctx->stream).
//
// Tall matrices are row-major n x ld (ld = pad_ld(cols), 16-byte rows,
// padding columns kept at zero).  Small r x r matrices are row-major FP64.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include "dense_common.cuh"
#include "lne_internal.h"

namespace lne {

// N(0,1) entries from a counter-based generator: entry (i, j) of stream
// `stream_id` is a Box-Muller transform of two 24-bit uniforms hashed from
// (seed, stream_id, i, j), rounded to an e4m3-representable value for
// stream 0 (the sketch) and to a BF16-representable one otherwise.
// Independent of the launch shape.  The FP8 fill writes the e4m3 bytes of
// the same values (always e4m3-rounded).
int gaussian_fill_f32(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols, float* out,
                      int64_t ld);
int gaussian_fill_fp8(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols,
                      __nv_fp8_e4m3* out, int64_t ld);

// G (c1 x c2, FP64, row-major, ldg = c2) = A^T B for A (n x c1, lda),
// B (n x c2, ldb).  FP32 products summed per 2048-row block, blocks summed
// in FP64 in block order (reproducible).
int gram(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
         double* G);

// Out (n x c2, ldo) = In (n x k, ldi) * W (k x c2, FP32 row-major, ldw = c2).
// Optional 16-bit copy of Out (same ld; BF16, or FP16 of scale * Out).
// Columns c2..ldo-1 of Out are zeroed.
int gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
              int64_t ldo, Copy16 OutB = Copy16());

// Cholesky G + shift*I = L L^T (FP64, in place on a device r x r buffer) and
// W = L^-T as FP32 (r x r row-major, upper triangular).  Returns
// LNE_ERR_NUMERIC when a pivot is not positive.
// Kernel launches of one cholesky_inv call for an r x r matrix.
int cholesky_inv_launches(lne_ctx* ctx, int r);
int cholesky_inv(lne_ctx* ctx, double* G, int r, double shift, float* W);

// One-sided Jacobi SVD of C (r x r, FP64 row-major, device; overwritten):
// U (r x r FP64, columns = left singular vectors, sorted by singular value,
// descending), S (r, FP64).  For r <= 160 the FP64 sweeps start from an
// FP32 Jacobi preconditioning; *sweeps32_out (may be NULL) gets its sweeps
// (0 without it), *sweeps_out the FP64 sweeps.  fp64_sweep_cap > 0 caps
// the FP64 sweeps after the preconditioning (r <= 160); 0: until they
// converge.  One FP64 sweep takes the FP32 stopping level (|cos| <= 4e-6)
// to about its square.
int jacobi_svd(lne_ctx* ctx, double* C, int r, double* U, double* S, int* sweeps_out, int* sweeps32_out = nullptr,
               int fp64_sweep_cap = 0);
// Kernel launches of one jacobi_svd call.
int jacobi_svd_launches(lne_ctx* ctx, int r);
// The FP64 sweep cap of the pipeline's core SVDs (the context's setting;
// `full_by_default` says what the automatic setting does for the caller).
inline int core_svd_sweep_cap(const lne_ctx* ctx, bool full_by_default) {
  const bool full = ctx->core_svd_fp64 < 0 ? full_by_default : ctx->core_svd_fp64 != 0;
  return full ? 0 : 1;
}

// tcgen05 tensor-core versions (3xTF32, FP32-level accuracy) of gram and
// gemm_tall for up to 256 columns; gram/gemm_tall use them when they apply.
bool tc_supported(int c2);
int tc_gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
                 int64_t ldo, Copy16 OutB);
// Streaming tensor-core Gram: applies when both operands are 16-byte aligned
// with row strides that are multiples of 4 floats and the shape fits.  Uses
// at most max_blocks CTAs; `partial` (NULL: allocated here) holds
// blocks * c1 * c2 floats.
bool tc_gram_stream_supported(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb,
                              int c2);
int tc_gram_stream(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
                   double* G, float* partial, int64_t max_blocks);
// CUDA-core Gram with caller-provided partial storage (ceil(n / 2048) * c1 *
// c2 floats); allocates nothing.
int gram_simt_into(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
                   double* G, float* partial);

// Copies an FP32 tall matrix into a BF16 copy (same ld).
int to_bf16(lne_ctx* ctx, const float* X, int64_t n, int64_t ld, __nv_bfloat16* Y);

// Row-wise L2 normalisation of an n x d FP32 matrix (rows with norm <= eps
// are left unchanged), as PathEmbed.h:390-405.
int normalize_rows(lne_ctx* ctx, float* X, int64_t n, int d, int64_t ld, float eps);

// Trace of a device FP64 r x r matrix, read back to the host (synchronises).
int trace_host(lne_ctx* ctx, const double* G, int r, double* out);
// ||G - I||_F of an r x r FP64 matrix, read back to the host (synchronises).
int identity_distance_host(lne_ctx* ctx, const double* G, int r, double* out);

}  // namespace lne
