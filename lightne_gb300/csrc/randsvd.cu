// Randomized SVD of the sparsifier matrix and the U * sqrt(Sigma) embedding.
//
// Reference: mkl_redsvd::MKLRedSVD<FP>::run (LightNE/mklredsvd/mklredsvd.cc:93-403)
// and path_embed::compute_u_sigma_root (LightNE/PathEmbed.h:371-408):
//   Y = A * Omega, Q = qr(Y), B = A * Q, Z = qr(B * P), C = Z^T B,
//   C = U_C S V^T, matU = Z * U_C, emb[:, j] = sqrt(S_j) * matU[:, j], j < dim.
// Orthonormalisation is CholeskyQR (a shifted pass, then one or two plain
// passes) instead of Householder geqrf+orgqr; R has a positive diagonal, so Q is the
// unique thin-QR factor with that sign convention.  The core SVD is a
// one-sided FP64 Jacobi.  The Gaussian sketches come from a counter-based
// generator (MKL's SFMT19937 stream cannot be reproduced without MKL).  The
// sketch's values are e4m3-representable, so the 16-bit forms gather it from
// an exact FP8 copy; their product A * Q gathers a 16-bit copy of Q (BF16,
// or FP16 of 2^12 Q) that the last CholeskyQR GEMM writes beside the FP32 Q.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "dense.h"
#include "sparse_proj.h"
#include "dense_common.cuh"
#include "lne_internal.h"
#include "spmm_core.cuh"
#include "spmm_dispatch.cuh"

namespace lne {

namespace {

struct Buf {
  lne_ctx* ctx;
  std::vector<void*> ptrs;
  explicit Buf(lne_ctx* c) : ctx(c) {}
  template <typename T>
  int get(T** out, size_t count, const char* what) {
    void* p = nullptr;
    int rc = dalloc(ctx, &p, sizeof(T) * (count > 0 ? count : 1), what);
    if (rc == LNE_OK) ptrs.push_back(p);
    *out = (T*)p;
    return rc;
  }
  ~Buf() {
    for (void* p : ptrs) dfree(ctx, p);
  }
};

// Y = scale * (A * X) with FP32 output, X FP32, BF16, FP16 or FP8 (scale
// undoes the power-of-two scaling of an FP16 copy; 1 otherwise); `add`
// accumulates the later column panels of the cache-blocked SpMM.
struct EpiStore {
  float* __restrict__ Y;
  int64_t ldy;
  int d;
  bool add;
  float scale = 1.0f;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&a)[N]) const {
    float* y = Y + r * ldy + e0;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (e0 + i < d) y[i] = add ? fmaf(scale, a[i], y[i]) : scale * a[i];
  }
};

__global__ void k_scale_cols(const double* __restrict__ U, const double* __restrict__ S, int r, int dim,
                             float* __restrict__ W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= r * dim) return;
  const int i = t / dim, j = t % dim;
  // compute_u_sigma_root takes sqrt of the float singular value
  W[t] = (float)U[(int64_t)i * r + j] * sqrtf((float)S[j]);
}

__global__ void k_copy_cols(const float* __restrict__ X, int64_t ldx, int64_t n, int dim, float* __restrict__ E) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * dim; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / dim;
    const int j = (int)(t - i * dim);
    E[t] = X[i * ldx + j];
  }
}

}  // namespace

// CholeskyQR on X (n x ld FP32, r columns) with tmp as the ping-pong
// partner; the two pointers are swapped so that the result ends in X.  Xb
// (optional) receives a 16-bit copy of the result from the last GEMM.
//
// The first pass is shifted (Fukaya et al. 2020: G + s I with s = 64 u tr G,
// the shift growing x10 while a pivot fails), then plain passes follow.
// After the first pass the Gram of its result G1 = Q1^T Q1 measures how
// orthogonal Q1 is: with ||G1 - I||_F <= 0.5, kappa(Q1)^2 <= 3 and one more
// plain pass leaves Q orthogonal to FP32 rounding (CholeskyQR2); otherwise a
// third pass follows (shifted CholeskyQR3), as for the second QR of the
// randomized SVD, whose Z = B P has kappa ~ 5e3.
static constexpr double kCholQR2Tol = 0.5;
static int cholqr3(lne_ctx* ctx, float*& X, float*& tmp, int64_t n, int64_t ld, int r, Copy16 Xb,
                   int* launches) {
  Buf B(ctx);
  double* G = nullptr;
  float* W = nullptr;
  int rc;
  if ((rc = B.get(&G, (size_t)r * r, "gram")) || (rc = B.get(&W, (size_t)r * r, "R^-1"))) return rc;
  float* src = X;
  float* dst = tmp;
  const double u32 = 5.9604644775390625e-08;
  for (int pass = 0; pass < 3; ++pass) {
    double shift = 0.0;
    bool last = pass == 2;
    for (int attempt = 0; attempt < 6; ++attempt) {
      if ((rc = gram(ctx, src, ld, r, src, ld, r, n, G))) return rc;
      *launches += 2;
      if (pass == 1 && attempt == 0) {
        double e = 0.0;
        if ((rc = identity_distance_host(ctx, G, r, &e))) return rc;
        *launches += 1;
        last = e <= kCholQR2Tol;
      }
      if (pass == 0 || attempt > 0) {
        double tr = 0.0;
        if ((rc = trace_host(ctx, G, r, &tr))) return rc;
        *launches += 1;
        shift = (pass == 0 && attempt == 0 ? 64.0 : 64.0 * pow(10.0, attempt)) * u32 * tr;
      }
      rc = cholesky_inv(ctx, G, r, shift, W);
      *launches += cholesky_inv_launches(ctx, r);
      if (rc == LNE_OK) break;
      if (rc != LNE_ERR_NUMERIC || attempt == 5) return rc;
    }
    if ((rc = gemm_tall(ctx, src, ld, r, W, r, n, dst, ld, last ? Xb : Copy16()))) return rc;
    *launches += 1;
    float* t = src;
    src = dst;
    dst = t;
    if (last) break;
  }
  // the result is in src: the buffer X came in after two passes, tmp's
  // after three
  X = src;
  tmp = dst;
  return LNE_OK;
}

template <typename XT>
static int spmm_store(lne_ctx* ctx, lne_csr* A, const XT* X, int64_t ld, int d, float* Y, int* launches,
                      float scale = 1.0f, int64_t panel_bytes = 0) {
  EpiStore epi{Y, ld, d, false, scale};
  return spmm_csr_panels<XT>(ctx, A, X, ld, d, epi, launches, panel_bytes);
}

// The product A * Q of the 16-bit forms gathers Q in two column panels when
// Q's lowest-id rows up to this many bytes receive at least half of A's
// entries (power-law graphs numbered hubs first): their gathers then stay
// in L2 (1.1M x 144 FP16 at nnz 351M: 14.7 -> 13.3 ms alone).
static constexpr int64_t kHubPanelBytes = (int64_t)64 << 20;

// Scale of the FP16 copy of Q: |Q| <= 1 (orthonormal columns), so 2^12 Q
// stays below 4097, and entries down to 2^-26 stay in FP16's normal range.
static constexpr float kQHalfScale = 4096.0f;

}  // namespace lne

using namespace lne;

extern "C" int lne_gaussian(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols,
                            float* d_out, int64_t ld) {
  LNE_CHECK_ARG(ctx && d_out && rows >= 0 && cols >= 0 && ld >= cols, "lne_gaussian: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  return gaussian_fill_f32(ctx, seed, stream_id, rows, cols, d_out, ld);
}

extern "C" int lne_randsvd(lne_ctx* ctx, const lne_csr* Acsr, const lne_randsvd_params* p, float* d_emb,
                           float* h_S, lne_randsvd_stats* stats) {
  LNE_CHECK_ARG(ctx && Acsr && p && d_emb, "lne_randsvd: NULL argument");
  LNE_CHECK_ARG(p->rank >= 1 && p->dim >= 1 && p->dim <= p->rank, "lne_randsvd: need 1 <= dim <= rank");
  LNE_CHECK_ARG(p->rank <= Acsr->n, "lne_randsvd: rank above n");
  LNE_CHECK_ARG(p->precision == LNE_PREC_FP32 || p->precision == LNE_PREC_BF16 || p->precision == LNE_PREC_FP16,
                "lne_randsvd: bad precision");
  if (p->rank > 1024) {
    set_error("lne_randsvd: rank above 1024 is not supported by the one-block Jacobi core");
    return LNE_ERR_UNSUPPORTED;
  }
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, ctx->stream));
  lne_csr* A = const_cast<lne_csr*>(Acsr);
  const int64_t n = A->n;
  const int r = (int)p->rank, dim = (int)p->dim;
  const int64_t ld = pad_ld(r);
  const bool f16 = p->precision == LNE_PREC_FP16;
  const bool low = p->precision != LNE_PREC_FP32;  // a 16-bit form
  cudaStream_t st = ctx->stream;
  int launches = 0;
  if (!A->plan_ready) launches += kPlanLaunches;
  int rc = build_plan_csr(ctx, A);
  if (rc) return rc;

  cudaEvent_t ev[6];
  for (auto& e : ev) cudaEventCreate(&e);
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() { for (int i = 0; i < 6; ++i) cudaEventDestroy(e[i]); }
  } evg{ev};

  Buf B(ctx);
  float *Y = nullptr, *T = nullptr, *Bm = nullptr, *P = nullptr, *Wf = nullptr;
  __nv_fp8_e4m3* Xq = nullptr;  // the sketch's FP8 copy (16-bit forms)
  uint16_t* Q16 = nullptr;       // the 16-bit copy of Q (16-bit forms)
  const int64_t ldq = pad_ld_fp8(r);
  double *C = nullptr, *U = nullptr, *S = nullptr;
  if ((rc = B.get(&Y, (size_t)n * ld, "Y")) || (rc = B.get(&T, (size_t)n * ld, "QR scratch")) ||
      (low && !p->sparse_project && (rc = B.get(&Xq, (size_t)n * ldq, "FP8 sketch"))))
    return rc;

  cudaEventRecord(ev[0], st);
  // Y = A * Omega
  if (p->sparse_project) {
    // Omega = the very sparse random projection (mklredsvd.cc:148-226): the
    // product only touches A's nonzeros whose O row is not empty
    SparseProjection O;
    if ((rc = sparse_projection_build(ctx, n, r, p->seed, p->sparse_project_s, &O, &launches))) return rc;
    if ((rc = sparse_projection_product(ctx, A, O, Y, ld, &launches))) return rc;
    launches -= 1;  // the Gaussian draw counted below does not happen
  } else if (low) {
    // the sketch's values are e4m3-representable: its FP8 copy is exact
    if ((rc = gaussian_fill_fp8(ctx, p->seed, 0, n, r, Xq, ldq))) return rc;
    if ((rc = spmm_store<__nv_fp8_e4m3>(ctx, A, Xq, ldq, (int)ld, Y, &launches))) return rc;
  } else {
    if ((rc = gaussian_fill_f32(ctx, p->seed, 0, n, r, T, ld))) return rc;
    if ((rc = spmm_store<float>(ctx, A, T, ld, (int)ld, Y, &launches))) return rc;
  }
  launches += 1;
  cudaEventRecord(ev[1], st);

  if (p->random_project_only) {
    // matU = Y, S = NULL: emb = Y[:, :dim] (PathEmbed.h:380 uses sigma = 1)
    k_copy_cols<<<(unsigned)std::min<int64_t>((n * dim + 255) / 256, (int64_t)ctx->num_sms * 32), 256, 0, st>>>(
        Y, ld, n, dim, d_emb);
    launches += 1;
    if (p->normalize && (rc = normalize_rows(ctx, d_emb, n, dim, dim, 1e-5f))) return rc;
    if (h_S)
      for (int i = 0; i < r; ++i) h_S[i] = 1.0f;
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    if (p->normalize) launches += 1;
    if (stats) {
      memset(stats, 0, sizeof(*stats));
      cudaEventElapsedTime(&stats->ms_sketch, ev[0], ev[1]);
      stats->kernel_launches = launches;
    }
    ctx->launch_count += launches;
    return LNE_OK;
  }

  // Q = qr(Y), with its 16-bit copy in the 16-bit forms
  Copy16 q16;
  if (low) {
    if ((rc = B.get(&Q16, (size_t)n * ld, "16-bit Q"))) return rc;
    q16.p = Q16;
    q16.kind = f16 ? 2 : 1;
    q16.scale = f16 ? kQHalfScale : 1.0f;
  }
  if ((rc = cholqr3(ctx, Y, T, n, ld, r, q16, &launches))) return rc;
  cudaEventRecord(ev[2], st);
  // B = A * Q
  if ((rc = B.get(&Bm, (size_t)n * ld, "B"))) return rc;
  if (f16)
    rc = spmm_store<__half>(ctx, A, (const __half*)Q16, ld, (int)ld, Bm, &launches, 1.0f / kQHalfScale,
                            -kHubPanelBytes);
  else if (low)
    rc = spmm_store<__nv_bfloat16>(ctx, A, (const __nv_bfloat16*)Q16, ld, (int)ld, Bm, &launches, 1.0f,
                                   -kHubPanelBytes);
  else
    rc = spmm_store<float>(ctx, A, Y, ld, (int)ld, Bm, &launches);
  if (rc) return rc;
  cudaEventRecord(ev[3], st);
  // Z = qr(B * P); Y holds Z from here on
  if ((rc = B.get(&P, (size_t)r * r, "P"))) return rc;
  if ((rc = gaussian_fill_f32(ctx, p->seed, 1, r, r, P, r))) return rc;
  if ((rc = gemm_tall(ctx, Bm, ld, r, P, r, n, Y, ld))) return rc;
  launches += 2;
  if ((rc = cholqr3(ctx, Y, T, n, ld, r, Copy16(), &launches))) return rc;
  cudaEventRecord(ev[4], st);
  // C = Z^T B, C = U_C S V^T
  if ((rc = B.get(&C, (size_t)r * r, "C")) || (rc = B.get(&U, (size_t)r * r, "U_C")) ||
      (rc = B.get(&S, (size_t)r, "S")))
    return rc;
  if ((rc = gram(ctx, Y, ld, r, Bm, ld, r, n, C))) return rc;
  int sweeps = 0, sweeps32 = 0;
  // FP64 sweeps to convergence in the FP32 form, one in the 16-bit forms
  // (unless the context says otherwise)
  const int cap = core_svd_sweep_cap(ctx, !low);
  if ((rc = jacobi_svd(ctx, C, r, U, S, &sweeps, &sweeps32, cap))) return rc;
  launches += 2 + jacobi_svd_launches(ctx, r);  // Gram + reduction, Jacobi
  // emb = Z * (U_C[:, :dim] * diag(sqrt(S[:dim])))
  if ((rc = B.get(&Wf, (size_t)r * dim, "U sqrt(S)"))) return rc;
  k_scale_cols<<<(r * dim + 255) / 256, 256, 0, st>>>(U, S, r, dim, Wf);
  if ((rc = gemm_tall(ctx, Y, ld, r, Wf, dim, n, d_emb, dim))) return rc;
  launches += 2;
  if (p->normalize) {
    if ((rc = normalize_rows(ctx, d_emb, n, dim, dim, 1e-5f))) return rc;
    launches += 1;
  }
  cudaEventRecord(ev[5], st);
  if (h_S) {
    std::vector<double> hs(r);
    LNE_CUDA_TRY(cudaMemcpyAsync(hs.data(), S, sizeof(double) * r, cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < r; ++i) h_S[i] = (float)hs[i];
  }
  LNE_CUDA_TRY(cudaEventSynchronize(ev[5]));
  LNE_CUDA_TRY(cudaGetLastError());
  {
    int hf = 0;
    LNE_CUDA_TRY(cudaMemcpy(&hf, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
    if (hf == 2) {
      set_error("lne_randsvd: a tensor-core wait timed out");
      return LNE_ERR_CUDA;
    }
  }
  if (stats) {
    cudaEventElapsedTime(&stats->ms_sketch, ev[0], ev[1]);
    cudaEventElapsedTime(&stats->ms_qr, ev[1], ev[2]);
    cudaEventElapsedTime(&stats->ms_spmm2, ev[2], ev[3]);
    cudaEventElapsedTime(&stats->ms_core, ev[3], ev[5]);
    cudaEventElapsedTime(&stats->ms_total, ev[0], ev[5]);
    stats->jacobi_sweeps = sweeps;
    stats->jacobi_sweeps_fp32 = sweeps32;
    stats->kernel_launches = launches;
    stats->spmm_nnz = (double)A->nnz;
  }
  ctx->launch_count += launches;
  return LNE_OK;
}

extern "C" int lne_core_svd(lne_ctx* ctx, const double* d_C, int32_t r, double* d_U, double* d_S,
                            int32_t* h_sweeps) {
  LNE_CHECK_ARG(ctx && d_C && d_U && d_S && r >= 1, "lne_core_svd: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  Buf B(ctx);
  double* C = nullptr;
  int rc;
  if ((rc = B.get(&C, (size_t)r * r, "core copy"))) return rc;
  LNE_CUDA_TRY(cudaMemcpyAsync(C, d_C, sizeof(double) * r * r, cudaMemcpyDeviceToDevice, ctx->stream));
  int sw = 0, sw32 = 0;
  if ((rc = jacobi_svd(ctx, C, r, d_U, d_S, &sw, &sw32))) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (h_sweeps) {
    h_sweeps[0] = sw;
    h_sweeps[1] = sw32;
  }
  return LNE_OK;
}

extern "C" int lne_dense_embed(lne_ctx* ctx, const float* d_x, int64_t n, int64_t dim, float* d_emb, float* h_S) {
  LNE_CHECK_ARG(ctx && d_x && d_emb && n >= 1 && dim >= 1 && dim <= n, "lne_dense_embed: bad argument");
  if (dim > 1024) {
    set_error("lne_dense_embed: dim above 1024 is not supported by the one-block Jacobi core");
    return LNE_ERR_UNSUPPORTED;
  }
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, st));
  const int d = (int)dim;
  const int64_t ld = pad_ld(d);
  Buf B(ctx);
  float *X = nullptr, *Q = nullptr, *T = nullptr, *W = nullptr;
  double *C = nullptr, *U = nullptr, *S = nullptr;
  int rc, launches = 0;
  if ((rc = B.get(&X, (size_t)n * ld, "X")) || (rc = B.get(&Q, (size_t)n * ld, "Q")) ||
      (rc = B.get(&T, (size_t)n * ld, "QR scratch")) || (rc = B.get(&C, (size_t)d * d, "R")) ||
      (rc = B.get(&U, (size_t)d * d, "U_R")) || (rc = B.get(&S, (size_t)d, "S")) ||
      (rc = B.get(&W, (size_t)d * d, "U sqrt(S)")))
    return rc;
  // padded copy (the pad columns are zero)
  LNE_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(float) * n * ld, st));
  LNE_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(float) * ld, d_x, sizeof(float) * d, sizeof(float) * d, n,
                                 cudaMemcpyDeviceToDevice, st));
  LNE_CUDA_TRY(cudaMemcpyAsync(Q, X, sizeof(float) * n * ld, cudaMemcpyDeviceToDevice, st));
  // X = Q R with Q from CholeskyQR; R = Q^T X; R = U_R S V^T; U = Q U_R
  if ((rc = cholqr3(ctx, Q, T, n, ld, d, Copy16(), &launches))) return rc;
  if ((rc = gram(ctx, Q, ld, d, X, ld, d, n, C))) return rc;
  int sweeps = 0;
  if ((rc = jacobi_svd(ctx, C, d, U, S, &sweeps, nullptr, core_svd_sweep_cap(ctx, true)))) return rc;
  k_scale_cols<<<(d * d + 255) / 256, 256, 0, st>>>(U, S, d, d, W);
  if ((rc = gemm_tall(ctx, Q, ld, d, W, d, n, d_emb, d))) return rc;
  // get_embedding_dense normalises unconditionally (SpectralPropagation.h:40)
  if ((rc = normalize_rows(ctx, d_emb, n, d, d, 1e-5f))) return rc;
  // Gram + reduction, Jacobi, column scaling, GEMM, row normalisation
  launches += 2 + jacobi_svd_launches(ctx, d) + 1 + 1 + 1;
  if (h_S) {
    std::vector<double> hs(d);
    LNE_CUDA_TRY(cudaMemcpyAsync(hs.data(), S, sizeof(double) * d, cudaMemcpyDeviceToHost, st));
    LNE_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < d; ++i) h_S[i] = (float)hs[i];
  }
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  LNE_CUDA_TRY(cudaGetLastError());
  int hf = 0;
  LNE_CUDA_TRY(cudaMemcpy(&hf, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
  if (hf == 2) {
    set_error("lne_dense_embed: a tensor-core wait timed out");
    return LNE_ERR_CUDA;
  }
  ctx->launch_count += launches;
  return LNE_OK;
}
