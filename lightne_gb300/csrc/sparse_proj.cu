// Very sparse random projection sketch of the randomized SVD (-sparse_project):
// LightNE/mklredsvd/mklredsvd.cc:148-226, after Li, Hastie and Church, "Very
// sparse random projections" (KDD 2006).
//
// The sketch O is n x rank with, per row i, k_i ~ Binomial(rank, 1/s)
// nonzeros at distinct columns, each +sqrt(s) or -sqrt(s) with equal
// probability; s = sqrt(n) unless -sparse_project_s >= 1 gives it.  The
// reference draws k_i from MKL's VSL stream and the columns by a partial
// Fisher-Yates shuffle seeded with time(0); neither stream can be
// reproduced, so row i here uses its own counter-based generator
// fork(seed, i) (the pbbs::random construction of the sampler): rank
// Bernoulli(1/s) draws give k_i, Floyd's algorithm (Bentley and Floyd, CACM
// 1987) picks the k_i distinct columns, sorted ascending, and one draw per
// entry gives its sign.  The same seed gives the same sketch.
//
// Y = A O (mkl_sparse_spmmd, mklredsvd.cc:219) is one warp per row of A:
// lanes load 32 nonzeros (j, a) of the row at a time, the lanes whose O row
// j is not empty are taken in lane order, and every entry (c, o) of O row j
// adds a * o to output column c, held by lane c % 32.  Each output sum runs
// in the order of A's nonzeros, so Y is reproducible.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <string>

#include "lne_internal.h"
#include "lne_math.cuh"
#include "sparse_proj.h"

namespace lne {

namespace {

constexpr int kSpPer = 5;  // output columns per lane: rank up to 160

__device__ __forceinline__ int sp_row_count(uint64_t& s, int rank, double density) {
  int k = 0;
  for (int t = 0; t < rank; ++t) k += map_uint64(rng_draw(s)) < density ? 1 : 0;
  return k;
}

__global__ void k_sp_count(int64_t n, int rank, uint64_t seed, double density, int64_t* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s = rng_fork(seed, (uint64_t)i);
  cnt[i] = sp_row_count(s, rank, density);
}

__global__ void k_sp_fill(int64_t n, int rank, uint64_t seed, double density, float value,
                          const int64_t* __restrict__ rp, int32_t* __restrict__ col, float* __restrict__ val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t s = rng_fork(seed, (uint64_t)i);
  const int k = sp_row_count(s, rank, density);
  const int64_t b = rp[i];
  // Floyd: for j = rank - k .. rank - 1 take t uniform in [0, j]; if t was
  // taken already, take j instead
  for (int m = 0, j = rank - k; j < rank; ++j, ++m) {
    const int t = (int)(rng_draw(s) % (uint64_t)(j + 1));
    bool dup = false;
    for (int e = 0; e < m; ++e) dup |= col[b + e] == t;
    col[b + m] = dup ? j : t;
  }
  for (int m = 1; m < k; ++m) {  // ascending columns
    const int x = col[b + m];
    int e = m - 1;
    while (e >= 0 && col[b + e] > x) {
      col[b + e + 1] = col[b + e];
      --e;
    }
    col[b + e + 1] = x;
  }
  for (int m = 0; m < k; ++m) val[b + m] = (rng_draw(s) & 1ULL) ? value : -value;
}

__global__ void k_sp_dense(int64_t n, int rank, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                           const float* __restrict__ val, float* __restrict__ out, int64_t ld) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* row = out + i * ld;
  for (int c = 0; c < ld; ++c) row[c] = 0.0f;
  for (int64_t e = rp[i]; e < rp[i + 1]; ++e) row[col[e]] = val[e];
  (void)rank;
}

__global__ void __launch_bounds__(256) k_spmm_sparse_proj(int64_t n, const int64_t* __restrict__ arp,
                                                          const int32_t* __restrict__ acol,
                                                          const float* __restrict__ aval,
                                                          const int64_t* __restrict__ orp,
                                                          const int32_t* __restrict__ ocol,
                                                          const float* __restrict__ oval, float* __restrict__ Y,
                                                          int64_t ld) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += nwarps) {
    float acc[kSpPer];
#pragma unroll
    for (int t = 0; t < kSpPer; ++t) acc[t] = 0.0f;
    const int64_t a0 = arp[row], a1 = arp[row + 1];
    for (int64_t base = a0; base < a1; base += 32) {
      const int64_t idx = base + lane;
      const bool valid = idx < a1;
      const int j = valid ? acol[idx] : 0;
      const float a = valid ? aval[idx] : 0.0f;
      const int64_t o0 = valid ? orp[j] : 0;
      const int k = valid ? (int)(orp[j + 1] - o0) : 0;
      unsigned m = __ballot_sync(0xffffffffu, k > 0);
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const float as = __shfl_sync(0xffffffffu, a, src);
        const int64_t os = __shfl_sync(0xffffffffu, o0, src);
        const int ks = __shfl_sync(0xffffffffu, k, src);
        for (int e = 0; e < ks; ++e) {
          const int c = ocol[os + e];
          const float ov = oval[os + e];
          if ((c & 31) == lane) {
#pragma unroll
            for (int t = 0; t < kSpPer; ++t)
              if ((c >> 5) == t) acc[t] = fmaf(as, ov, acc[t]);
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < kSpPer; ++t) {
      const int c = lane + 32 * t;
      if (c < ld) Y[row * ld + c] = acc[t];
    }
  }
}

}  // namespace

SparseProjection::~SparseProjection() {
  if (ctx) {
    dfree(ctx, rp);
    dfree(ctx, col);
    dfree(ctx, val);
  }
}

// s and the value sqrt(s) as the reference's FP (float) arithmetic gives
// them (mklredsvd.cc:150-155, 188); the density 1/s is taken in double, as
// viRngBinomial receives it.
void sparse_projection_scale(int64_t n, double s_flag, float* s_out, double* density, float* value) {
  float s = sqrtf((float)n);
  if (s_flag >= 1.0) s = (float)s_flag;
  *s_out = s;
  *density = 1.0 / (double)s;
  *value = sqrtf(s);
}

int sparse_projection_build(lne_ctx* ctx, int64_t n, int rank, uint64_t seed, double s_flag, SparseProjection* O,
                            int* launches) {
  O->ctx = ctx;
  O->n = n;
  O->rank = rank;
  float s = 0.0f, value = 0.0f;
  double density = 0.0;
  sparse_projection_scale(n, s_flag, &s, &density, &value);
  cudaStream_t st = ctx->stream;
  int64_t* cnt = nullptr;
  void* tmp = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&O->rp, sizeof(int64_t) * (n + 1), "sparse projection row_ptr"))) return rc;
  if ((rc = dalloc(ctx, (void**)&cnt, sizeof(int64_t) * (n > 0 ? n : 1), "sparse projection counts"))) return rc;
  if ((rc = dalloc(ctx, &tmp, scan_tmp_bytes(n), "sparse projection scan"))) {
    dfree(ctx, cnt);
    return rc;
  }
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (n > 0) k_sp_count<<<grid, 256, 0, st>>>(n, rank, seed, density, cnt);
  scan_exclusive_i64(cnt, O->rp, n, tmp, st);
  int64_t nnz = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&nnz, O->rp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  dfree(ctx, tmp);
  dfree(ctx, cnt);
  O->nnz = nnz;
  if ((rc = dalloc(ctx, (void**)&O->col, sizeof(int32_t) * (nnz > 0 ? nnz : 1), "sparse projection col")) ||
      (rc = dalloc(ctx, (void**)&O->val, sizeof(float) * (nnz > 0 ? nnz : 1), "sparse projection val")))
    return rc;
  if (n > 0) k_sp_fill<<<grid, 256, 0, st>>>(n, rank, seed, density, value, O->rp, O->col, O->val);
  if (launches) *launches += 5;  // count, 3-launch scan, fill
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int sparse_projection_product(lne_ctx* ctx, const lne_csr* A, const SparseProjection& O, float* Y, int64_t ld,
                              int* launches) {
  if (ld > 32 * kSpPer) {
    set_error("sparse projection: rank above 160 is not supported");
    return LNE_ERR_UNSUPPORTED;
  }
  if (A->n <= 0) return LNE_OK;
  const int64_t warps = std::min<int64_t>(A->n, (int64_t)ctx->num_sms * 64);
  k_spmm_sparse_proj<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, ctx->stream>>>(
      A->n, A->row_ptr, A->col, A->val, O.rp, O.col, O.val, Y, ld);
  if (launches) *launches += 1;
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int sparse_projection_dense(lne_ctx* ctx, const SparseProjection& O, float* out, int64_t ld) {
  if (O.n <= 0) return LNE_OK;
  k_sp_dense<<<(unsigned)((O.n + 255) / 256), 256, 0, ctx->stream>>>(O.n, O.rank, O.rp, O.col, O.val, out, ld);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

}  // namespace lne

using namespace lne;

extern "C" int lne_sparse_projection(lne_ctx* ctx, uint64_t seed, int64_t n, int64_t rank, double s, float* d_out,
                                     int64_t ld, int64_t* nnz_out) {
  LNE_CHECK_ARG(ctx && d_out && n >= 0 && rank >= 1 && rank <= 1 << 20 && ld >= rank,
                "lne_sparse_projection: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  SparseProjection O;
  int rc = sparse_projection_build(ctx, n, (int)rank, seed, s, &O, nullptr);
  if (rc) return rc;
  if ((rc = sparse_projection_dense(ctx, O, d_out, ld))) return rc;
  if (nnz_out) *nnz_out = O.nnz;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return LNE_OK;
}
