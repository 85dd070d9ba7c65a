// Dense kernels of the randomized SVD (mklredsvd.cc:93-403 replaced by
// CholeskyQR and a one-sided Jacobi core SVD) and of the dense embedding.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <string>

#include "dense.h"
#include "dense_common.cuh"
#include "lne_math.cuh"

namespace lne {

// ---------------------------------------------------------------------------
// Gaussian sketch
// ---------------------------------------------------------------------------
// FP8 (e4m3) nearest value of x, as a float (and its byte in *b).
__device__ __forceinline__ float round_e4m3(float x, __nv_fp8_storage_t* b) {
  *b = __nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3);
  const __half_raw h = __nv_cvt_fp8_to_halfraw(*b, __NV_E4M3);
  return __half2float(*reinterpret_cast<const __half*>(&h));
}

// Box-Muller draw `idx` of the stream, rounded to an FP8 (e4m3)-representable
// value (e4m3 set) or a BF16-representable one, so that the FP32 and
// BF16 forms of the randomized SVD use the same sketch.
__device__ __forceinline__ float gaussian_at(uint64_t base, uint64_t idx, bool e4m3, __nv_fp8_storage_t* b) {
  const uint64_t x1 = hash64_2(base + 2 * idx), x2 = hash64_2(base + 2 * idx + 1);
  const float u1 = (float)((x1 >> 40) + 1) * 5.9604644775390625e-08f;  // (0, 1]
  const float u2 = (float)(x2 >> 40) * 5.9604644775390625e-08f;        // [0, 1)
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  const float z = sqrtf(-2.0f * logf(u1)) * c;
  if (e4m3) return round_e4m3(z, b);
  *b = 0;
  return __bfloat162float(__float2bfloat16_rn(z));
}

template <typename T>
__global__ void k_gaussian(uint64_t base, int64_t rows, int64_t cols, T* __restrict__ out, int64_t ld, bool e4m3) {
  const int64_t total = rows * ld;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / ld, j = t - i * ld;
    __nv_fp8_storage_t b = 0;
    const float z = j < cols ? gaussian_at(base, (uint64_t)(i * cols + j), e4m3, &b) : 0.0f;
    if constexpr (sizeof(T) == 1)
      reinterpret_cast<__nv_fp8_storage_t*>(out)[t] = b;
    else
      out[t] = (T)z;
  }
}

static uint64_t gaussian_base(uint64_t seed, uint64_t stream_id) {
  return hash64_2(seed ^ hash64_2(stream_id + 0x9E3779B97F4A7C15ULL));
}

static unsigned grid1d(int64_t items, int threads, int64_t cap) {
  int64_t b = (items + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

// Stream 0 (the sketch Omega) is rounded to e4m3, the others to BF16.
int gaussian_fill_f32(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols, float* out,
                      int64_t ld) {
  k_gaussian<float><<<grid1d(rows * ld, 256, (int64_t)ctx->num_sms * 32), 256, 0, ctx->stream>>>(
      gaussian_base(seed, stream_id), rows, cols, out, ld, stream_id == 0);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int gaussian_fill_fp8(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols,
                      __nv_fp8_e4m3* out, int64_t ld) {
  k_gaussian<__nv_fp8_e4m3><<<grid1d(rows * ld, 256, (int64_t)ctx->num_sms * 32), 256, 0, ctx->stream>>>(
      gaussian_base(seed, stream_id), rows, cols, out, ld, true);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

// ---------------------------------------------------------------------------
// Gram: partial[b] = A_b^T B_b over row blocks of kGramRows, 64 x 64 output
// tiles, 256 threads with 4 x 4 outputs each; then a fixed-order FP64 sum.
// ---------------------------------------------------------------------------
static constexpr int kGramRows = 2048;

__global__ void __launch_bounds__(256) k_gram_partial(const float* __restrict__ A, int64_t lda, int c1,
                                                      const float* __restrict__ B, int64_t ldb, int c2, int64_t n,
                                                      float* __restrict__ partial, int tiles_j) {
  __shared__ __align__(16) float As[32][64];
  __shared__ __align__(16) float Bs[32][64];
  const int ti = blockIdx.x / tiles_j, tj = blockIdx.x % tiles_j;
  const int64_t rb = blockIdx.y;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t r0 = rb * kGramRows;
  const int64_t r1 = std::min<int64_t>(n, r0 + kGramRows);
  float acc[4][4] = {};
  for (int64_t k0 = r0; k0 < r1; k0 += 32) {
    for (int idx = tid; idx < 32 * 64; idx += 256) {
      const int rr = idx >> 6, cc = idx & 63;
      const int64_t row = k0 + rr;
      const int ca = ti * 64 + cc, cb = tj * 64 + cc;
      As[rr][cc] = (row < r1 && ca < c1) ? A[row * lda + ca] : 0.f;
      Bs[rr][cc] = (row < r1 && cb < c2) ? B[row * ldb + cb] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(av[p], bv[q], acc[p][q]);
    }
    __syncthreads();
  }
  float* out = partial + rb * (int64_t)c1 * c2;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = ti * 64 + ty * 4 + p;
    if (i >= c1) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = tj * 64 + tx * 4 + q;
      if (j < c2) out[(int64_t)i * c2 + j] = acc[p][q];
    }
  }
}

__global__ void k_gram_reduce(const float* __restrict__ partial, int64_t nb, int64_t cnt, double* __restrict__ G) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  double s = 0.0;
  for (int64_t b = 0; b < nb; ++b) s += (double)partial[b * cnt + t];
  G[t] = s;
}

int gram_simt_into(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
                   double* G, float* partial) {
  const int64_t nb = std::max<int64_t>(1, (n + kGramRows - 1) / kGramRows);
  const int tiles_i = (c1 + 63) / 64, tiles_j = (c2 + 63) / 64;
  dim3 grid((unsigned)(tiles_i * tiles_j), (unsigned)nb);
  k_gram_partial<<<grid, 256, 0, ctx->stream>>>(A, lda, c1, B, ldb, c2, n, partial, tiles_j);
  const int64_t cnt = (int64_t)c1 * c2;
  k_gram_reduce<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(partial, nb, cnt, G);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int gram(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
         double* G) {
  if (tc_supported(c2) && tc_gram_stream_supported(ctx, A, lda, c1, B, ldb, c2))
    return tc_gram_stream(ctx, A, lda, c1, B, ldb, c2, n, G, nullptr, ctx->num_sms);
  const int64_t nb = std::max<int64_t>(1, (n + kGramRows - 1) / kGramRows);
  float* partial = nullptr;
  int rc = dalloc(ctx, (void**)&partial, sizeof(float) * nb * c1 * c2, "gram partials");
  if (rc) return rc;
  rc = gram_simt_into(ctx, A, lda, c1, B, ldb, c2, n, G, partial);
  dfree(ctx, partial);
  return rc;
}

// ---------------------------------------------------------------------------
// Tall GEMM: Out = In * W, 128 x 64 output tiles, 256 threads, 8 x 4 each.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gemm_tall(const float* __restrict__ In, int64_t ldi, int k,
                                                   const float* __restrict__ W, int c2, int64_t n,
                                                   float* __restrict__ Out, int64_t ldo, Copy16 OutB) {
  __shared__ __align__(16) float As[16][128 + 4];
  __shared__ __align__(16) float Ws[16][64];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t row0 = (int64_t)blockIdx.x * 128;
  const int col0 = blockIdx.y * 64;
  float acc[8][4] = {};
  for (int k0 = 0; k0 < k; k0 += 16) {
    for (int idx = tid; idx < 128 * 16; idx += 256) {
      const int rr = idx >> 4, kk = idx & 15;
      const int64_t row = row0 + rr;
      As[kk][rr] = (row < n && k0 + kk < k) ? In[row * ldi + k0 + kk] : 0.f;
    }
    for (int idx = tid; idx < 16 * 64; idx += 256) {
      const int kk = idx >> 6, cc = idx & 63;
      Ws[kk][cc] = (k0 + kk < k && col0 + cc < c2) ? W[(int64_t)(k0 + kk) * c2 + col0 + cc] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 8]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][ty * 8 + 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Ws[kk][tx * 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int p = 0; p < 8; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(av[p], bv[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const int64_t row = row0 + ty * 8 + p;
    if (row >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = col0 + tx * 4 + q;
      if (c < ldo) {
        const float v = c < c2 ? acc[p][q] : 0.f;
        Out[row * ldo + c] = v;
        copy16_put(OutB, row * ldo + c, v);
      }
    }
  }
}

int gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
              int64_t ldo, Copy16 OutB) {
  if (n <= 0) return LNE_OK;
  if (tc_supported((int)std::max<int64_t>(c2, ldo))) return tc_gemm_tall(ctx, In, ldi, k, W, c2, n, Out, ldo, OutB);
  dim3 grid((unsigned)((n + 127) / 128), (unsigned)((ldo + 63) / 64));
  k_gemm_tall<<<grid, 256, 0, ctx->stream>>>(In, ldi, k, W, c2, n, Out, ldo, OutB);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

// ---------------------------------------------------------------------------
// FP64 Cholesky (right-looking, one block) and W = L^-T in FP32.
// ---------------------------------------------------------------------------
__global__ void k_cholesky(double* __restrict__ G, int r, double shift, int* __restrict__ status) {
  __shared__ double dk;
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  for (int i = threadIdx.x; i < r; i += blockDim.x) G[(int64_t)i * r + i] += shift;
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (threadIdx.x == 0) {
      const double d = G[(int64_t)k * r + k];
      if (!(d > 0.0) || !isfinite(d)) {
        bad = 1;
        dk = 1.0;
      } else {
        dk = sqrt(d);
      }
      G[(int64_t)k * r + k] = dk;
    }
    __syncthreads();
    if (bad) break;
    const double piv = dk;
    for (int i = k + 1 + threadIdx.x; i < r; i += blockDim.x) G[(int64_t)i * r + k] /= piv;
    __syncthreads();
    const int m = r - k - 1;
    for (int64_t t = threadIdx.x; t < (int64_t)m * m; t += blockDim.x) {
      const int i = k + 1 + (int)(t / m), j = k + 1 + (int)(t % m);
      if (j <= i) G[(int64_t)i * r + j] -= G[(int64_t)i * r + k] * G[(int64_t)j * r + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *status = bad;
}

// X = L^-1 by forward substitution, one column per thread; W[i][j] = X[j][i].
__global__ void k_tri_inv_t(const double* __restrict__ L, int r, float* __restrict__ W, double* __restrict__ X) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= r) return;
  for (int i = 0; i < r; ++i) {
    double x;
    if (i < j) {
      x = 0.0;
    } else if (i == j) {
      x = 1.0 / L[(int64_t)j * r + j];
    } else {
      double s = 0.0;
      for (int k = j; k < i; ++k) s += L[(int64_t)i * r + k] * X[(int64_t)k * r + j];
      x = -s / L[(int64_t)i * r + i];
    }
    X[(int64_t)i * r + j] = x;
    W[(int64_t)j * r + i] = (float)x;
  }
}

// The same factorisation and inverse with the matrix in shared memory (one
// CTA, r <= 160): L in the lower triangle, X = L^-1 stored transposed in the
// upper triangle (X[i][j] at [j][i]) and its diagonal apart, so W = X^T is
// the upper triangle.  Same operations in the same order as the two kernels
// above; the matrix is read from global memory once and W written once.
constexpr int kCholSmemMax = 160;

__global__ void __launch_bounds__(1024) k_chol_inv_smem(const double* __restrict__ G, int r, double shift,
                                                        float* __restrict__ W, int* __restrict__ status) {
  extern __shared__ double A[];  // r * r, then the diagonal of X (r)
  double* xd = A + (int64_t)r * r;
  __shared__ double dk;
  __shared__ int bad;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  for (int t = tid; t < r * r; t += blockDim.x) A[t] = G[t];
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int i = tid; i < r; i += blockDim.x) A[i * r + i] += shift;
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (tid == 0) {
      const double d = A[k * r + k];
      if (!(d > 0.0) || !isfinite(d)) {
        bad = 1;
        dk = 1.0;
      } else {
        dk = sqrt(d);
      }
      A[k * r + k] = dk;
    }
    __syncthreads();
    if (bad) break;
    const double piv = dk;
    for (int i = k + 1 + tid; i < r; i += blockDim.x) A[i * r + k] /= piv;
    __syncthreads();
    for (int i = k + 1 + ty; i < r; i += 32) {
      const double lik = A[i * r + k];
      for (int j = k + 1 + tx; j <= i; j += 32) A[i * r + j] -= lik * A[j * r + k];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) *status = 1;
    return;
  }
  // rows of X = L^-1 in order; thread j < i computes X[i][j]
  for (int i = 0; i < r; ++i) {
    for (int j = tid; j <= i; j += blockDim.x) {
      if (j == i) {
        xd[i] = 1.0 / A[i * r + i];
      } else {
        double sacc = A[i * r + j] * xd[j];  // k = j
        for (int k = j + 1; k < i; ++k) sacc += A[i * r + k] * A[j * r + k];
        A[j * r + i] = -sacc / A[i * r + i];
      }
    }
    __syncthreads();
  }
  for (int t = tid; t < r * r; t += blockDim.x) {
    const int j = t / r, i = t - (t / r) * r;  // W[j][i] = X[i][j]
    W[t] = i < j ? 0.0f : (i == j ? (float)xd[i] : (float)A[j * r + i]);
  }
  if (tid == 0) *status = 0;
}

// Thread-block cluster primitives: barrier, rank, distributed shared memory.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t dsmem_map(uint32_t saddr, uint32_t rank) {
  uint32_t a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(saddr), "r"(rank));
  return a;
}
__device__ __forceinline__ double dsmem_ld(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ int dsmem_ld32(uint32_t a) {
  int v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void dsmem_st(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}

// The same factorisation on one thread-block cluster (16 CTAs where the
// device allows that size, else 8), r <= kCholClusterMax, blocked by panels
// of kCholPanel columns: panel q (columns 8q .. 8q + 7) lives in CTA
// q % size.  Step q: the owner factors the panel in its shared memory
// (pivot, scale, update of the panel's later columns, column by column), a
// cluster barrier publishes it, every CTA copies it (distributed shared
// memory) and applies it to its own later columns (rank-8 update).  One
// cluster barrier per panel instead of one per pivot; the sums of a trailing
// update run in panel order (not bit-identical to the one-CTA form, the
// same FP64 arithmetic otherwise).  Then every CTA gathers L and the
// cluster's warps solve L x = e_j for their columns j (each entry a
// lane-parallel dot product), writing row j of W = L^-T.
constexpr int kCholClusterMax = 144;
constexpr int kCholPanel = 8;

__global__ void __launch_bounds__(256) k_chol_inv_cluster(const double* __restrict__ G, int r, double shift,
                                                          float* __restrict__ W, int* __restrict__ status) {
  extern __shared__ double chs[];
  __shared__ int bad;
  __shared__ double prcp;  // 1 / pivot
  const int csize = gridDim.x;
  const int rank = (int)cluster_rank();
  const int npan = (r + kCholPanel - 1) / kCholPanel;
  const int nps = (npan + csize - 1) / csize;  // panel slots per CTA
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  double* col = chs;                                       // [nps * 8][r]: my columns
  double* pan = col + (size_t)nps * kCholPanel * r;        // [8][r]: the panel of this step
  double* Lf = pan + (size_t)kCholPanel * r;               // [r][r]: all of L (inverse phase)
  double* xw = Lf + (size_t)r * r;                         // [nw][r]: a warp's solution column; then r reciprocals
  // local column c (slot c / 8, offset c % 8) is global column j_of(c)
  auto j_of = [&](int c) { return ((c / kCholPanel) * csize + rank) * kCholPanel + (c % kCholPanel); };
  const int ncols = nps * kCholPanel;
  for (int c = 0; c < ncols; ++c) {
    const int j = j_of(c);
    if (j < r)
      for (int i = tid; i < r; i += blockDim.x) col[(size_t)c * r + i] = G[(size_t)j * r + i] + (i == j ? shift : 0.0);
  }
  if (tid == 0) bad = 0;
  const uint32_t col_s = (uint32_t)__cvta_generic_to_shared(col);
  const uint32_t bad_s = (uint32_t)__cvta_generic_to_shared(&bad);
  cluster_barrier();
  bool failed = false;
  for (int q = 0; q < npan; ++q) {
    const int own = q % csize, qs = q / csize;
    const int k0 = q * kCholPanel, k1 = min(k0 + kCholPanel, r);
    if (rank == own) {
      for (int k = k0; k < k1; ++k) {
        double* ck = col + (size_t)(qs * kCholPanel + (k - k0)) * r;
        // FP64 division and square root are long instruction sequences on
        // this part: one square root and one reciprocal per pivot, then
        // the column is scaled by multiplications spread over all warps
        if (warp == 0) {  // one warp evaluates the pivot
          const double d = ck[k];
          const bool ok = d > 0.0 && isfinite(d);
          const double piv = ok ? sqrt(d) : 1.0;
          if (lane == 0) {
            prcp = 1.0 / piv;
            ck[k] = piv;
            if (!ok) bad = 1;
          }
        }
        __syncthreads();
        if (bad) break;
        const double rp = prcp;
        for (int i = k + 1 + tid; i < r; i += blockDim.x) ck[i] *= rp;
        __syncthreads();
        for (int j = k + 1 + warp; j < k1; j += nw) {
          double* cj = col + (size_t)(qs * kCholPanel + (j - k0)) * r;
          const double ljk = ck[j];
          for (int i = j + lane; i < r; i += 32) cj[i] -= ck[i] * ljk;
        }
        __syncthreads();
      }
    }
    cluster_barrier();
    if (dsmem_ld32(dsmem_map(bad_s, (uint32_t)own))) {
      failed = true;
      break;
    }
    // the panel's rows k0.. into pan (column t of the panel at pan + t r)
    const uint32_t src = dsmem_map(col_s + (uint32_t)(qs * kCholPanel * r) * 8u, (uint32_t)own);
    for (int e = tid; e < (k1 - k0) * r; e += blockDim.x)
      if (e - (e / r) * r >= k0) pan[e] = dsmem_ld(src + 8u * (uint32_t)e);
    __syncthreads();
    // rank-(k1 - k0) update of my columns after the panel
    for (int c = warp; c < ncols; c += nw) {
      const int j = j_of(c);
      if (j < k1 || j >= r) continue;
      double lj[kCholPanel];
#pragma unroll
      for (int t = 0; t < kCholPanel; ++t) lj[t] = k0 + t < k1 ? pan[(size_t)t * r + j] : 0.0;
      double* cj = col + (size_t)c * r;
      for (int i = j + lane; i < r; i += 32) {
        double v = cj[i];
#pragma unroll
        for (int t = 0; t < kCholPanel; ++t)
          if (k0 + t < k1) v -= pan[(size_t)t * r + i] * lj[t];
        cj[i] = v;
      }
    }
    __syncthreads();
  }
  cluster_barrier();
  if (!failed) {
    // L column-major in every CTA (Lc[k][i] = column k, row i >= k) and
    // the reciprocals of its diagonal
    double* Lc = Lf;
    double* idg = xw + (size_t)nw * r;
    for (int k = warp; k < r; k += nw) {
      const int qk = k / kCholPanel;
      const uint32_t src =
          dsmem_map(col_s + (uint32_t)(((qk / csize) * kCholPanel + (k % kCholPanel)) * r) * 8u, (uint32_t)(qk % csize));
      for (int i = k + lane; i < r; i += 32) Lc[(size_t)k * r + i] = dsmem_ld(src + 8u * (uint32_t)i);
    }
    __syncthreads();
    for (int i = tid; i < r; i += blockDim.x) idg[i] = 1.0 / Lc[(size_t)i * r + i];
    __syncthreads();
    // column j of X = L^-1 by column-oriented forward substitution:
    // x_k = b_k / L_kk, then b_i -= L_ik x_k for i > k (lane-parallel, no
    // reductions); row j of W = X^T
    double* x = xw + (size_t)warp * r;
    for (int j = warp * csize + rank; j < r; j += nw * csize) {
      for (int i = lane; i < r; i += 32) x[i] = i == j ? 1.0 : 0.0;
      __syncwarp();
      for (int k = j; k < r; ++k) {
        const double xk = x[k] * idg[k];
        __syncwarp();
        if (lane == 0) x[k] = xk;
        const double* lk = Lc + (size_t)k * r;
        for (int i = k + 1 + lane; i < r; i += 32) x[i] = fma(-lk[i], xk, x[i]);
        __syncwarp();
      }
      for (int i = lane; i < r; i += 32) W[(size_t)j * r + i] = i < j ? 0.0f : (float)x[i];
      __syncwarp();
    }
  }
  if (rank == 0 && tid == 0) *status = failed ? 1 : 0;
  cluster_barrier();  // no CTA leaves while another may still read its shared memory
}

static size_t chol_cluster_smem(int r, int csize) {
  const size_t npan = (size_t)(r + kCholPanel - 1) / kCholPanel;
  const size_t nps = (npan + csize - 1) / csize;
  return sizeof(double) * (nps * kCholPanel * r + (size_t)kCholPanel * r + (size_t)r * r + 9 * (size_t)r);
}

// Launches k_chol_inv_cluster on a 16- or 8-CTA cluster; false if neither
// size can be launched.
static bool chol_inv_cluster_launch(lne_ctx* ctx, const double* G, int r, double shift, float* W, int* status) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(256, 1, 1);
  cfg.stream = ctx->stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  for (int cl : {16, 8}) {
    const size_t smem = chol_cluster_smem(r, cl);
    if (smem > ctx->smem_optin) continue;
    if (cl == 16 &&
        cudaFuncSetAttribute(k_chol_inv_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (cudaFuncSetAttribute(k_chol_inv_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cfg.gridDim = dim3(cl, 1, 1);
    cfg.dynamicSmemBytes = smem;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_chol_inv_cluster, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    if (cudaLaunchKernelEx(&cfg, k_chol_inv_cluster, G, r, shift, W, status) == cudaSuccess) return true;
    cudaGetLastError();
  }
  return false;
}

int cholesky_inv_launches(lne_ctx* ctx, int r) {
  if (r <= kCholClusterMax) return 1;
  return (r <= kCholSmemMax && sizeof(double) * ((size_t)r * r + r) <= ctx->smem_optin) ? 1 : 2;
}

int cholesky_inv(lne_ctx* ctx, double* G, int r, double shift, float* W) {
  double* X = nullptr;
  int* status = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&X, sizeof(double) * r * r + 16, "triangular inverse"))) return rc;
  status = (int*)(X + (int64_t)r * r);
  const size_t csmem = sizeof(double) * ((size_t)r * r + r);
  if (r <= kCholClusterMax && chol_inv_cluster_launch(ctx, G, r, shift, W, status)) {
    // done on the cluster
  } else if (r <= kCholSmemMax && csmem <= ctx->smem_optin) {
    cudaFuncSetAttribute(k_chol_inv_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem);
    k_chol_inv_smem<<<1, 1024, csmem, ctx->stream>>>(G, r, shift, W, status);
  } else {
    k_cholesky<<<1, 1024, 0, ctx->stream>>>(G, r, shift, status);
    k_tri_inv_t<<<(r + 127) / 128, 128, 0, ctx->stream>>>(G, r, W, X);
  }
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, X);
  LNE_CUDA_TRY(cudaGetLastError());
  if (h) {
    set_error("Cholesky of the Gram matrix failed (matrix not numerically positive definite)");
    return LNE_ERR_NUMERIC;
  }
  return LNE_OK;
}

// ---------------------------------------------------------------------------
// One-sided Jacobi SVD (Hestenes), FP64.  Columns of the working copy are
// rotated pairwise in round-robin order until every pair is orthogonal to
// 1e-15 relative; singular values are the column norms, left singular
// vectors the normalised columns.  Dot products, rotations and the
// convergence test are FP64; the distributed-shared-memory form computes
// the rotation angle in FP32 and then makes (c, s) orthogonal in FP64.
//
// The sweeps run on one thread-block cluster (16 CTAs where the device
// allows that size, else 8): each warp of the cluster takes pairs of the
// current round-robin step, and a cluster barrier (release/acquire at
// cluster scope) separates the steps.  The columns live in the CTAs' shared
// memory (column c in CTA c % size) and are read and written through
// distributed shared memory; a lane keeps its elements of both columns in
// registers between the dot products and the rotation.  When the columns do
// not fit there, they stay in global memory (L2), read with ld.global.cg so
// that no CTA sees a stale L1 line of a column another CTA rotated.  FP64
// runs at 1/68 of the FP32 rate on this part, so one SM would spend about
// 30 ms on a 138 x 138 core; 16 SMs share the work.
// ---------------------------------------------------------------------------
__global__ void k_jacobi_init(const double* __restrict__ C, int r, double* __restrict__ Wc,
                              int* __restrict__ rotated, int max_sweeps) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)r * r;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / r), j = (int)(t % r);
    Wc[(int64_t)j * r + i] = C[t];
  }
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < max_sweeps; t += gridDim.x * blockDim.x) rotated[t] = 0;
}

__global__ void __launch_bounds__(256) k_jacobi_sweeps(int r, double* __restrict__ Wc, int* __restrict__ rotated,
                                                       int max_sweeps, int* __restrict__ sweeps_out) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;  // the grid is one cluster
  // pairs go to the CTAs round-robin (pair pk -> CTA pk % size), so that
  // every SM's FP64 units share the step's work
  const int gw = (int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x;
  const int rp = (r + 1) & ~1;  // even number of players (index r is a dummy when r is odd)
  // below sqrt(r) eps a rotation only chases the rounding of the dot product
  const double tol = fmax(1e-15, 2.220446049250313e-16 * sqrt((double)r));
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    for (int s = 0; s < rp - 1; ++s) {
      for (int pk = gw; pk < rp / 2; pk += nwarps) {
        int p, q;
        if (pk == 0) {
          p = rp - 1;
          q = s;
        } else {
          p = (s + pk) % (rp - 1);
          q = (s - pk + rp - 1) % (rp - 1);
        }
        if (p >= r || q >= r) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        double* wp = Wc + (int64_t)p * r;
        double* wq = Wc + (int64_t)q * r;
        double a = 0.0, b = 0.0, g = 0.0;
        for (int i = lane; i < r; i += 32) {
          const double x = __ldcg(wp + i), y = __ldcg(wq + i);
          a = fma(x, x, a);
          b = fma(y, y, b);
          g = fma(x, y, g);
        }
        for (int o = 16; o > 0; o >>= 1) {
          a += __shfl_xor_sync(0xffffffffu, a, o);
          b += __shfl_xor_sync(0xffffffffu, b, o);
          g += __shfl_xor_sync(0xffffffffu, g, o);
        }
        if (fabs(g) > tol * sqrt(a * b) && g != 0.0) {
          const double zeta = (b - a) / (2.0 * g);
          const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
          for (int i = lane; i < r; i += 32) {
            const double x = __ldcg(wp + i), y = __ldcg(wq + i);
            wp[i] = c * x - sn * y;
            wq[i] = sn * x + c * y;
          }
          if (lane == 0) rotated[sweep] = 1;
        }
      }
      cluster_barrier();
    }
    if (__ldcg(rotated + sweep) == 0) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *sweeps_out = sweep < max_sweeps ? sweep + 1 : max_sweeps;
}

constexpr int kJacobiPer = 5;  // column elements per lane held in registers (r <= 160)
constexpr int kJacobiMaxSweeps = 60;

// Same sweeps, same arithmetic, with the columns in distributed shared
// memory (r <= 32 * kJacobiPer).
__global__ void __launch_bounds__(256) k_jacobi_sweeps_dsmem(int r, double* __restrict__ Wc, int* __restrict__ rotated,
                                                             int max_sweeps, int* __restrict__ sweeps_out) {
  extern __shared__ double jcols[];  // slot s: column s * csize + rank; then the slots' squared norms
  __shared__ int rot_flag[kJacobiMaxSweeps];  // this CTA rotated some pair in sweep k
  const int lane = threadIdx.x & 31;
  for (int k = threadIdx.x; k < kJacobiMaxSweeps; k += blockDim.x) rot_flag[k] = 0;
  const int csize = gridDim.x;  // the grid is one cluster (8 or 16 CTAs)
  const uint32_t rank = cluster_rank();
  const int nslots = (r + csize - 1) / csize;
  __shared__ double wsum[8], csum;  // this CTA's sum of squares (rotations keep the total)
  double sq = 0.0;
  for (int s = 0; s < nslots; ++s) {
    const int c = s * csize + (int)rank;
    if (c < r)
      for (int i = threadIdx.x; i < r; i += blockDim.x) {
        const double v = Wc[(int64_t)c * r + i];
        jcols[(int64_t)s * r + i] = v;
        sq = fma(v, v, sq);
      }
  }
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  if (lane == 0) wsum[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    csum = t;
  }
  cluster_barrier();
  // A column below about r eps of the Frobenius norm is rounding noise of
  // its partners (each rotation leaves eps |x| in it): it is not rotated,
  // or noise pairs would rotate forever on a rank-deficient matrix.
  double fro2 = 0.0;
  {
    const uint32_t ca = (uint32_t)__cvta_generic_to_shared(&csum);
    for (int c = 0; c < csize; ++c) fro2 += dsmem_ld(dsmem_map(ca, (uint32_t)c));
  }
  const double tiny = fro2 * 1.9721522630525295e-31 * (double)r * (double)r;  // fro2 (2 r 2^-52)^2
  double* cnorm = jcols + (int64_t)nslots * r;
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(jcols);
  const uint32_t nbase = (uint32_t)__cvta_generic_to_shared(cnorm);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  // pairs go to the CTAs round-robin (pair pk -> CTA pk % size), so that
  // every SM's FP64 units share the step's work
  const int gw = (int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x;
  const int rp = (r + 1) & ~1;
  const int m = rp - 1;
  const int cshift = __ffs(csize) - 1;  // csize is a power of two
  const double tol2 = fmax(1e-30, 4.930380657631324e-32 * r);  // (2^-52)^2 r
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // squared column norms, fresh every sweep; within the sweep each
    // rotation updates the two norms it changes (only x.y needs a dot)
    for (int sl = (int)(threadIdx.x >> 5); sl < nslots; sl += (int)(blockDim.x >> 5)) {
      double a = 0.0;
      const double* col = jcols + (int64_t)sl * r;
      for (int i = lane; i < r; i += 32) a = fma(col[i], col[i], a);
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) cnorm[sl] = a;
    }
    cluster_barrier();
    for (int s = 0; s < m; ++s) {
      for (int pk = gw; pk < rp / 2; pk += nwarps) {
        // the round-robin pairs of step s: (s + pk, s - pk) mod m, and (m, s)
        int p, q;
        if (pk == 0) {
          p = m;
          q = s;
        } else {
          p = s + pk;
          if (p >= m) p -= m;
          q = s - pk;
          if (q < 0) q += m;
        }
        if (p >= r || q >= r) continue;
        if (p > q) { const int t = p; p = q; q = t; }
        const uint32_t ap = dsmem_map(base + (uint32_t)((p >> cshift) * r) * 8u, (uint32_t)(p & (csize - 1)));
        const uint32_t aq = dsmem_map(base + (uint32_t)((q >> cshift) * r) * 8u, (uint32_t)(q & (csize - 1)));
        const uint32_t np_ = dsmem_map(nbase + (uint32_t)(p >> cshift) * 8u, (uint32_t)(p & (csize - 1)));
        const uint32_t nq_ = dsmem_map(nbase + (uint32_t)(q >> cshift) * 8u, (uint32_t)(q & (csize - 1)));
        const double a = dsmem_ld(np_), b = dsmem_ld(nq_);
        double x[kJacobiPer], y[kJacobiPer];
#pragma unroll
        for (int k = 0; k < kJacobiPer; ++k) {
          const int i = lane + 32 * k;
          x[k] = i < r ? dsmem_ld(ap + 8u * i) : 0.0;
          y[k] = i < r ? dsmem_ld(aq + 8u * i) : 0.0;
        }
        double g = 0.0;
#pragma unroll
        for (int k = 0; k < kJacobiPer; ++k)
          if (lane + 32 * k < r) g = fma(x[k], y[k], g);
        for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
        // |g| > tol sqrt(ab), without the square root; tol = max(1e-15,
        // sqrt(r) eps): the rounding of a length-r FP64 dot product, below
        // which a rotation would only chase noise
        if (g != 0.0 && a > tiny && b > tiny && g * g > tol2 * (a * b)) {
          // Rotation angle in FP32 (the FP64 units are scarce on this part;
          // an angle accurate to 2^-24 leaves a residual of that size in
          // g, which the next sweep removes), then (c, s) made orthogonal
          // to FP64 precision by two Newton steps on c^2 + s^2 = 1.
          const float zeta = (float)(b - a) / (float)(2.0 * g);
          const float az = fabsf(zeta);
          const float t32 = az < 1e18f ? copysignf(1.0f, zeta) / (az + sqrtf(fmaf(az, az, 1.0f))) : 0.5f / zeta;
          const float c32 = rsqrtf(fmaf(t32, t32, 1.0f));
          double c = (double)c32, sn = (double)c32 * (double)t32;
#pragma unroll
          for (int it = 0; it < 2; ++it) {
            const double f = fma(-0.5, fma(c, c, sn * sn), 1.5);
            c *= f;
            sn *= f;
          }
#pragma unroll
          for (int k = 0; k < kJacobiPer; ++k) {
            const int i = lane + 32 * k;
            if (i < r) {
              dsmem_st(ap + 8u * i, c * x[k] - sn * y[k]);
              dsmem_st(aq + 8u * i, sn * x[k] + c * y[k]);
            }
          }
          if (lane == 0) {
            rot_flag[sweep] = 1;
            const double cc = c * c, ss = sn * sn, cs2 = 2.0 * c * sn * g;
            dsmem_st(np_, fmax(fma(cc, a, fma(ss, b, -cs2)), 0.0));
            dsmem_st(nq_, fmax(fma(ss, a, fma(cc, b, cs2)), 0.0));
          }
        }
      }
      cluster_barrier();
    }
    int any = 0;
    const uint32_t fa = (uint32_t)__cvta_generic_to_shared(&rot_flag[sweep]);
    for (int c = 0; c < csize; ++c) any |= dsmem_ld32(dsmem_map(fa, (uint32_t)c));
    if (!any) break;
  }
  (void)rotated;
  cluster_barrier();  // no CTA leaves while another may still read its flags
  for (int s = 0; s < nslots; ++s) {
    const int c = s * csize + (int)rank;
    if (c < r)
      for (int i = threadIdx.x; i < r; i += blockDim.x) Wc[(int64_t)c * r + i] = jcols[(int64_t)s * r + i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *sweeps_out = sweep < max_sweeps ? sweep + 1 : max_sweeps;
}

// FP32 preconditioning of the FP64 sweeps (r <= 32 * kJacobiPer, one CTA):
// one-sided Jacobi on an FP32 copy of C (scaled to unit largest entry), the
// rotations accumulated in V from I, until no pair has |x.y| > kJacobiTol32
// |x| |y| (or kJacobi32MaxSweeps).  FP32 runs at many times the FP64 rate
// on this part, so these early sweeps are cheap; the FP64 sweeps then start
// from W = C V', V' = V re-orthogonalised in FP64 (k_jacobi_pm,
// k_jacobi_ns), whose columns are orthogonal to about the FP32 tolerance,
// and finish in a few sweeps.  The result is the same FP64-accurate
// one-sided Jacobi SVD: only the starting basis of the FP64 sweeps differs.
//
// Layout: columns of W and V at a stride of rq = r rounded up to 32 floats
// (zero padded).  A pair is handled by 8 lanes (4 pairs per warp), lane l
// holding the float4 vectors l, l + 8, ... of the two columns, so that one
// 8-lane group reads 128 contiguous bytes per load.
constexpr float kJacobiTol32 = 4e-6f;
constexpr int kJacobi32MaxSweeps = 30;
constexpr int kJacobi32Vec = 5;  // float4 vectors per lane: r <= 8 * 4 * 5 = 160

__host__ __device__ inline int jacobi32_stride(int r) { return (r + 31) & ~31; }

__global__ void __launch_bounds__(1024) k_jacobi_precond32(const double* __restrict__ C, int r,
                                                           double* __restrict__ Vout, int* __restrict__ sweeps_out) {
  extern __shared__ float4 jw4[];
  const int rq = jacobi32_stride(r);
  float* W = reinterpret_cast<float*>(jw4);  // column j at j * rq
  float* V = W + (size_t)r * rq;
  __shared__ double red[32];
  __shared__ int rot_flag[kJacobi32MaxSweeps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int gl = lane & 7, grp = lane >> 3;
  for (int k = tid; k < kJacobi32MaxSweeps; k += blockDim.x) rot_flag[k] = 0;
  double mx = 0.0;
  for (int t = tid; t < r * r; t += blockDim.x) mx = fmax(mx, fabs(C[t]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[warp] = mx;
  __syncthreads();
  mx = 0.0;
  for (int w = 0; w < nw; ++w) mx = fmax(mx, red[w]);
  const double sc = (mx > 0.0 && isfinite(mx)) ? 1.0 / mx : 1.0;
  double sq = 0.0;
  for (int t = tid; t < r * rq; t += blockDim.x) {
    const int j = t / rq, i = t - (t / rq) * rq;  // column j, row i
    const float w = i < r ? (float)(C[(int64_t)i * r + j] * sc) : 0.0f;
    W[t] = w;
    V[t] = i == j ? 1.0f : 0.0f;
    sq = fma((double)w, (double)w, sq);
  }
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  __syncthreads();  // every thread has read red[] above
  if (lane == 0) red[warp] = sq;
  __syncthreads();
  double fro2 = 0.0;
  for (int w = 0; w < nw; ++w) fro2 += red[w];
  // columns below about r eps32 of the Frobenius norm are left to the FP64
  // sweeps (in FP32 they are rounding noise of their partners)
  const float tiny = (float)(fro2 * 1.4210854715202004e-14 * (double)r * (double)r);  // fro2 (2 r 2^-24)^2
  const int rp = (r + 1) & ~1;
  const int m = rp - 1;
  const int nv = rq / 32;  // float4 vectors per lane actually used
  const float tol2 = kJacobiTol32 * kJacobiTol32;
  int sweep = 0;
  for (; sweep < kJacobi32MaxSweeps; ++sweep) {
    for (int s = 0; s < m; ++s) {
      for (int pk0 = warp * 4; pk0 < rp / 2; pk0 += nw * 4) {
        const int pk = pk0 + grp;
        int p = 0, q = 0;
        bool live = pk < rp / 2;
        if (live) {
          if (pk == 0) {
            p = m;
            q = s;
          } else {
            p = s + pk;
            if (p >= m) p -= m;
            q = s - pk;
            if (q < 0) q += m;
          }
          if (p >= r || q >= r) live = false;
          if (p > q) { const int t = p; p = q; q = t; }
        }
        float4 x[kJacobi32Vec], y[kJacobi32Vec];
        float a = 0.f, b = 0.f, g = 0.f;
        const float4* wp = reinterpret_cast<const float4*>(W + (size_t)p * rq);
        const float4* wq = reinterpret_cast<const float4*>(W + (size_t)q * rq);
#pragma unroll
        for (int k = 0; k < kJacobi32Vec; ++k) {
          if (live && k < nv) {
            x[k] = wp[gl + 8 * k];
            y[k] = wq[gl + 8 * k];
          } else {
            x[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            y[k] = x[k];
          }
          a = fmaf(x[k].x, x[k].x, fmaf(x[k].y, x[k].y, fmaf(x[k].z, x[k].z, fmaf(x[k].w, x[k].w, a))));
          b = fmaf(y[k].x, y[k].x, fmaf(y[k].y, y[k].y, fmaf(y[k].z, y[k].z, fmaf(y[k].w, y[k].w, b))));
          g = fmaf(x[k].x, y[k].x, fmaf(x[k].y, y[k].y, fmaf(x[k].z, y[k].z, fmaf(x[k].w, y[k].w, g))));
        }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
          a += __shfl_xor_sync(0xffffffffu, a, o);
          b += __shfl_xor_sync(0xffffffffu, b, o);
          g += __shfl_xor_sync(0xffffffffu, g, o);
        }
        if (live && g != 0.f && a > tiny && b > tiny && g * g > tol2 * (a * b)) {
          // the rotation need not be exact here: V is re-orthogonalised
          // in FP64 before the FP64 sweeps
          const float zeta = __fdividef(b - a, 2.0f * g);
          const float az = fabsf(zeta);
          const float t = az < 1e18f ? copysignf(1.0f, zeta) / (az + sqrtf(fmaf(az, az, 1.0f))) : 0.5f / zeta;
          const float c = rsqrtf(fmaf(t, t, 1.0f)), sn = c * t;
          float4* vp = reinterpret_cast<float4*>(V + (size_t)p * rq);
          float4* vq = reinterpret_cast<float4*>(V + (size_t)q * rq);
          float4* wpw = reinterpret_cast<float4*>(W + (size_t)p * rq);
          float4* wqw = reinterpret_cast<float4*>(W + (size_t)q * rq);
#pragma unroll
          for (int k = 0; k < kJacobi32Vec; ++k) {
            if (k < nv) {
              const int e = gl + 8 * k;
              wpw[e] = make_float4(c * x[k].x - sn * y[k].x, c * x[k].y - sn * y[k].y, c * x[k].z - sn * y[k].z,
                                   c * x[k].w - sn * y[k].w);
              wqw[e] = make_float4(sn * x[k].x + c * y[k].x, sn * x[k].y + c * y[k].y, sn * x[k].z + c * y[k].z,
                                   sn * x[k].w + c * y[k].w);
              const float4 u = vp[e], v = vq[e];
              vp[e] = make_float4(c * u.x - sn * v.x, c * u.y - sn * v.y, c * u.z - sn * v.z, c * u.w - sn * v.w);
              vq[e] = make_float4(sn * u.x + c * v.x, sn * u.y + c * v.y, sn * u.z + c * v.z, sn * u.w + c * v.w);
            }
          }
          if (gl == 0) rot_flag[sweep] = 1;
        }
      }
      __syncthreads();
    }
    if (!rot_flag[sweep]) break;
  }
  for (int t = tid; t < r * r; t += blockDim.x) {
    const int j = t / r, i = t - (t / r) * r;
    Vout[t] = (double)V[(size_t)j * rq + i];  // column-major r x r
  }
  if (tid == 0) *sweeps_out = sweep < kJacobi32MaxSweeps ? sweep + 1 : sweep;
}

// M = V^T V and, when C is given, P = C V (column-major: P[j * r + i]),
// FP64; V column-major.  One 16 x 16 output tile per CTA: tiles [0, nt^2)
// are M, [nt^2, 2 nt^2) are P.
__global__ void __launch_bounds__(256) k_jacobi_pm(const double* __restrict__ C, const double* __restrict__ Vc, int r,
                                                   double* __restrict__ Pc, double* __restrict__ M) {
  extern __shared__ double mt[];
  const int ldk = r + 1;  // odd: the 16 rows of a tile fall in distinct banks
  double* As = mt;
  double* Bs = mt + 16 * ldk;
  const int nt = (r + 15) / 16;
  int t = blockIdx.x;
  const bool isP = t >= nt * nt;
  if (isP) t -= nt * nt;
  const int i0 = (t / nt) * 16, j0 = (t % nt) * 16;
  for (int e = threadIdx.x; e < 16 * r; e += blockDim.x) {
    const int a = e / r, k = e - (e / r) * r;
    const int i = i0 + a, j = j0 + a;
    As[a * ldk + k] = i < r ? (isP ? C[(int64_t)i * r + k] : Vc[(int64_t)i * r + k]) : 0.0;
    Bs[a * ldk + k] = j < r ? Vc[(int64_t)j * r + k] : 0.0;
  }
  __syncthreads();
  const int ti = threadIdx.x >> 4, tj = threadIdx.x & 15;
  double acc = 0.0;
  for (int k = 0; k < r; ++k) acc = fma(As[ti * ldk + k], Bs[tj * ldk + k], acc);
  const int i = i0 + ti, j = j0 + tj;
  if (i < r && j < r) {
    if (isP)
      Pc[(int64_t)j * r + i] = acc;
    else
      M[(int64_t)i * r + j] = acc;
  }
}

// Y = X (3 I - M) / 2 for X = X1 and, when given, X2 (column-major r x r,
// M symmetric): one Newton-Schulz step towards orthogonality when
// M = V^T V (V^T V = I + E becomes I + O(E^2)).  Tiles [nt^2, 2 nt^2) do X2.
__global__ void __launch_bounds__(256) k_jacobi_ns(const double* __restrict__ X1, const double* __restrict__ X2,
                                                   const double* __restrict__ M, int r, double* __restrict__ Y1,
                                                   double* __restrict__ Y2) {
  extern __shared__ double mt[];
  const int ldk = r + 1;
  double* As = mt;  // As[a][k] = X[i0 + a][k] = Xc[k * r + i0 + a]
  double* Bs = mt + 16 * ldk;
  const int nt = (r + 15) / 16;
  int t = blockIdx.x;
  const bool second = t >= nt * nt;
  if (second) t -= nt * nt;
  const double* X = second ? X2 : X1;
  double* Y = second ? Y2 : Y1;
  const int i0 = (t / nt) * 16, j0 = (t % nt) * 16;
  for (int e = threadIdx.x; e < 16 * r; e += blockDim.x) {
    const int a = e & 15, k = e >> 4;
    As[a * ldk + k] = i0 + a < r ? X[(int64_t)k * r + i0 + a] : 0.0;
  }
  for (int e = threadIdx.x; e < 16 * r; e += blockDim.x) {
    const int b = e / r, k = e - (e / r) * r;
    Bs[b * ldk + k] = j0 + b < r ? M[(int64_t)(j0 + b) * r + k] : 0.0;
  }
  __syncthreads();
  const int ti = threadIdx.x >> 4, tj = threadIdx.x & 15;
  double acc = 0.0;
  for (int k = 0; k < r; ++k) acc = fma(As[ti * ldk + k], Bs[tj * ldk + k], acc);
  const int i = i0 + ti, j = j0 + tj;
  if (i < r && j < r) Y[(int64_t)j * r + i] = fma(1.5, X[(int64_t)j * r + i], -0.5 * acc);
}

__global__ void k_jacobi_finish(int r, const double* __restrict__ Wc, double* __restrict__ U,
                                double* __restrict__ S) {
  __shared__ int order[1024];
  __shared__ double norms[1024];
  for (int j = threadIdx.x; j < r; j += blockDim.x) {
    double s2 = 0.0;
    for (int i = 0; i < r; ++i) s2 = fma(Wc[(int64_t)j * r + i], Wc[(int64_t)j * r + i], s2);
    norms[j] = sqrt(s2);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < r; j += blockDim.x) {
    int rank = 0;
    for (int k = 0; k < r; ++k) rank += (norms[k] > norms[j]) || (norms[k] == norms[j] && k < j);
    order[rank] = j;
  }
  __syncthreads();
  for (int64_t t = threadIdx.x; t < (int64_t)r * r; t += blockDim.x) {
    const int i = (int)(t / r), jn = (int)(t % r);
    const int j = order[jn];
    const double nrm = norms[j];
    U[t] = nrm > 0.0 ? Wc[(int64_t)j * r + i] / nrm : 0.0;
  }
  for (int jn = threadIdx.x; jn < r; jn += blockDim.x) S[jn] = norms[order[jn]];
}

static size_t jacobi_precond_smem(int r) { return sizeof(float) * 2 * (size_t)r * jacobi32_stride(r); }

static bool jacobi_precond_applies(lne_ctx* ctx, int r) {
  return r <= 32 * kJacobi32Vec && jacobi_precond_smem(r) + 1024 <= ctx->smem_optin;
}

int jacobi_svd_launches(lne_ctx* ctx, int r) { return jacobi_precond_applies(ctx, r) ? 7 : 3; }

int jacobi_svd(lne_ctx* ctx, double* C, int r, double* U, double* S, int* sweeps_out, int* sweeps32_out,
               int fp64_sweep_cap) {
  if (r > 1024) {
    set_error("jacobi_svd: rank above 1024 is not supported");
    return LNE_ERR_UNSUPPORTED;
  }
  const int kMaxSweeps = kJacobiMaxSweeps;
  const bool pre = jacobi_precond_applies(ctx, r);
  // after the FP32 preconditioning, at most fp64_sweep_cap FP64 sweeps
  const int max_sweeps = pre && fp64_sweep_cap > 0 && fp64_sweep_cap < kMaxSweeps ? fp64_sweep_cap : kMaxSweeps;
  const size_t rr = (size_t)r * r;
  double* Wc = nullptr;
  int rc;
  // Wc, then (preconditioned) V, P, M, V1, P1 (FP64 r x r each)
  const size_t bytes = sizeof(double) * rr * (pre ? 6 : 1) + sizeof(int) * (kMaxSweeps + 4);
  if ((rc = dalloc(ctx, (void**)&Wc, bytes, "jacobi work"))) return rc;
  double* Vd = Wc + rr;
  double* Pc = Vd + rr;
  double* M = Pc + rr;
  double* V1 = M + rr;
  double* P1 = V1 + rr;
  int* rotated = (int*)(Wc + rr * (pre ? 6 : 1));
  int* d_sw = rotated + kMaxSweeps;  // [0]: FP64 sweeps, [1]: FP32 sweeps
  LNE_CUDA_TRY(cudaMemsetAsync(d_sw + 1, 0, sizeof(int), ctx->stream));
  if (pre) {
    // FP32 sweeps give V; two Newton-Schulz steps make it orthogonal to
    // FP64 precision (V^T V - I: about 1e-5 -> 1e-10 -> 1e-16); W = C V
    const size_t psmem = jacobi_precond_smem(r);
    cudaFuncSetAttribute(k_jacobi_precond32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem);
    k_jacobi_precond32<<<1, 1024, psmem, ctx->stream>>>(C, r, Vd, d_sw + 1);
    const int nt = (r + 15) / 16;
    const size_t msmem = sizeof(double) * 32 * (size_t)(r + 1);
    k_jacobi_pm<<<2 * nt * nt, 256, msmem, ctx->stream>>>(C, Vd, r, Pc, M);              // M = V^T V, P = C V
    k_jacobi_ns<<<2 * nt * nt, 256, msmem, ctx->stream>>>(Vd, Pc, M, r, V1, P1);         // V1, P1 = (V, P)(3I - M)/2
    k_jacobi_pm<<<nt * nt, 256, msmem, ctx->stream>>>(nullptr, V1, r, nullptr, M);       // M = V1^T V1
    k_jacobi_ns<<<nt * nt, 256, msmem, ctx->stream>>>(P1, nullptr, M, r, Wc, nullptr);   // W = P1 (3I - M)/2
  } else {
    k_jacobi_init<<<64, 256, 0, ctx->stream>>>(C, r, Wc, rotated, kMaxSweeps);
  }
  // one cluster: 16 CTAs if the device accepts that (non-portable) size
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = ctx->stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaErrorUnknown;
  const bool dsmem = r <= 32 * kJacobiPer;
  auto kern = dsmem ? k_jacobi_sweeps_dsmem : k_jacobi_sweeps;
  for (int cl : {16, 8}) {
    if (cl == 16 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cfg.gridDim = dim3(cl, 1, 1);
    cfg.dynamicSmemBytes = dsmem ? sizeof(double) * (size_t)((r + cl - 1) / cl) * (r + 1) : 0;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    e = cudaLaunchKernelEx(&cfg, kern, r, Wc, rotated, max_sweeps, d_sw);
    if (e == cudaSuccess) break;
    cudaGetLastError();
  }
  if (e != cudaSuccess) {
    dfree(ctx, Wc);
    set_error(std::string("jacobi_svd: cluster launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  k_jacobi_finish<<<1, 1024, 0, ctx->stream>>>(r, Wc, U, S);
  int h[2] = {0, 0};
  LNE_CUDA_TRY(cudaMemcpyAsync(h, d_sw, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, Wc);
  LNE_CUDA_TRY(cudaGetLastError());
  if (sweeps_out) *sweeps_out = h[0];
  if (sweeps32_out) *sweeps32_out = h[1];
  return LNE_OK;
}

// ---------------------------------------------------------------------------
// Small helpers
// ---------------------------------------------------------------------------
__global__ void k_to_bf16(const float* __restrict__ X, int64_t total, __nv_bfloat16* __restrict__ Y) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    Y[t] = __float2bfloat16_rn(X[t]);
}

int to_bf16(lne_ctx* ctx, const float* X, int64_t n, int64_t ld, __nv_bfloat16* Y) {
  k_to_bf16<<<grid1d(n * ld, 256, (int64_t)ctx->num_sms * 32), 256, 0, ctx->stream>>>(X, n * ld, Y);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

// One warp per row: norm in FP32 (as cblas_snrm2 on FP32 data), scale by
// 1/norm when norm > eps.
__global__ void k_normalize_rows(float* __restrict__ X, int64_t n, int d, int64_t ld, float eps) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float* x = X + r * ld;
    float s = 0.f;
    for (int j = lane; j < d; j += 32) s = fmaf(x[j], x[j], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float nrm = sqrtf(s);
    if (nrm > eps) {
      const float inv = (float)(1.0 / (double)nrm);
      for (int j = lane; j < d; j += 32) x[j] *= inv;
    }
  }
}

int normalize_rows(lne_ctx* ctx, float* X, int64_t n, int d, int64_t ld, float eps) {
  k_normalize_rows<<<grid1d(n * 32, 256, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(X, n, d, ld, eps);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

__global__ void k_trace(const double* G, int r, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < r; ++i) s += G[(int64_t)i * r + i];
    *out = s;
  }
}

// ||G - I||_F in FP64 (one block; r x r row-major).
__global__ void k_identity_distance(const double* __restrict__ G, int r, double* __restrict__ out) {
  __shared__ double part[32];
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < (int64_t)r * r; t += blockDim.x) {
    const int64_t i = t / r, j = t - i * r;
    const double e = G[t] - (i == j ? 1.0 : 0.0);
    s = fma(e, e, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += part[w];
    *out = sqrt(tot);
  }
}

int identity_distance_host(lne_ctx* ctx, const double* G, int r, double* out) {
  double* d = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&d, sizeof(double), "identity distance"))) return rc;
  k_identity_distance<<<1, 256, 0, ctx->stream>>>(G, r, d);
  LNE_CUDA_TRY(cudaMemcpyAsync(out, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d);
  return LNE_OK;
}

int trace_host(lne_ctx* ctx, const double* G, int r, double* out) {
  double* d = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&d, sizeof(double), "trace"))) return rc;
  k_trace<<<1, 32, 0, ctx->stream>>>(G, r, d);
  LNE_CUDA_TRY(cudaMemcpyAsync(out, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d);
  return LNE_OK;
}

}  // namespace lne

using namespace lne;

extern "C" int lne_gram(lne_ctx* ctx, const float* A, int64_t lda, int64_t c1, const float* B, int64_t ldb,
                        int64_t c2, int64_t n, double* G) {
  LNE_CHECK_ARG(ctx && A && B && G && n >= 0 && c1 >= 1 && c2 >= 1 && lda >= c1 && ldb >= c2,
                "lne_gram: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, ctx->stream));
  int rc = gram(ctx, A, lda, (int)c1, B, ldb, (int)c2, n, G);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpy(&h, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == 2) { set_error("lne_gram: tensor-core wait timed out"); return LNE_ERR_CUDA; }
  return LNE_OK;
}

extern "C" int lne_gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int64_t k, const float* W, int64_t c2,
                             int64_t n, float* Out, int64_t ldo) {
  LNE_CHECK_ARG(ctx && In && W && Out && n >= 0 && k >= 1 && c2 >= 1 && ldi >= k && ldo >= c2,
                "lne_gemm_tall: bad argument");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  LNE_CUDA_TRY(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int) * kFlagWords, ctx->stream));
  int rc = gemm_tall(ctx, In, ldi, (int)k, W, (int)c2, n, Out, ldo);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpy(&h, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == 2) { set_error("lne_gemm_tall: tensor-core wait timed out"); return LNE_ERR_CUDA; }
  return LNE_OK;
}
