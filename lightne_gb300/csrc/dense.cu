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
__device__ __forceinline__ float gaussian_at(uint64_t base, uint64_t idx) {
  const uint64_t x1 = hash64_2(base + 2 * idx), x2 = hash64_2(base + 2 * idx + 1);
  const float u1 = (float)((x1 >> 40) + 1) * 5.9604644775390625e-08f;  // (0, 1]
  const float u2 = (float)(x2 >> 40) * 5.9604644775390625e-08f;        // [0, 1)
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  // rounded to a BF16-representable value, so that the FP32 and BF16 forms
  // of the randomized SVD use the same sketch
  return __bfloat162float(__float2bfloat16_rn(sqrtf(-2.0f * logf(u1)) * c));
}

template <typename T>
__global__ void k_gaussian(uint64_t base, int64_t rows, int64_t cols, T* __restrict__ out, int64_t ld) {
  const int64_t total = rows * ld;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / ld, j = t - i * ld;
    const float z = j < cols ? gaussian_at(base, (uint64_t)(i * cols + j)) : 0.0f;
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

int gaussian_fill_f32(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols, float* out,
                      int64_t ld) {
  k_gaussian<float><<<grid1d(rows * ld, 256, (int64_t)ctx->num_sms * 32), 256, 0, ctx->stream>>>(
      gaussian_base(seed, stream_id), rows, cols, out, ld);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int gaussian_fill_bf16(lne_ctx* ctx, uint64_t seed, uint64_t stream_id, int64_t rows, int64_t cols,
                       __nv_bfloat16* out, int64_t ld) {
  k_gaussian<__nv_bfloat16><<<grid1d(rows * ld, 256, (int64_t)ctx->num_sms * 32), 256, 0, ctx->stream>>>(
      gaussian_base(seed, stream_id), rows, cols, out, ld);
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
                                                   float* __restrict__ Out, int64_t ldo,
                                                   __nv_bfloat16* __restrict__ OutB) {
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
        if (OutB) OutB[row * ldo + c] = __float2bfloat16_rn(v);
      }
    }
  }
}

int gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
              int64_t ldo, __nv_bfloat16* OutB) {
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
// device allows that size, else 8), r <= kCholClusterMax: column j in CTA
// j % size.  Step k: the owner of column k takes the pivot and scales the
// column, a cluster barrier publishes it, every CTA copies it (distributed
// shared memory) and updates its own later columns, element by element in
// the same operations and order as k_cholesky.  Then every CTA gathers L and
// the cluster's warps solve L x = e_j for their columns j (each entry a
// lane-parallel dot product), writing row j of W = L^-T.
constexpr int kCholClusterMax = 144;

__global__ void __launch_bounds__(256) k_chol_inv_cluster(const double* __restrict__ G, int r, double shift,
                                                          float* __restrict__ W, int* __restrict__ status) {
  extern __shared__ double chs[];
  __shared__ int bad;
  const int csize = gridDim.x;
  const int rank = (int)cluster_rank();
  const int nslots = (r + csize - 1) / csize;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  double* col = chs;                          // [nslots][r]: my columns
  double* colk = col + (size_t)nslots * r;    // [r]: column k of this step
  double* Lf = colk + r;                      // [r][r]: all of L (inverse phase)
  double* xw = Lf + (size_t)r * r;            // [nw][r]: a warp's solution column
  for (int s = 0; s < nslots; ++s) {
    const int j = s * csize + rank;
    if (j < r)
      for (int i = tid; i < r; i += blockDim.x) col[(size_t)s * r + i] = G[(size_t)j * r + i] + (i == j ? shift : 0.0);
  }
  if (tid == 0) bad = 0;
  const uint32_t col_s = (uint32_t)__cvta_generic_to_shared(col);
  const uint32_t bad_s = (uint32_t)__cvta_generic_to_shared(&bad);
  cluster_barrier();
  bool failed = false;
  for (int k = 0; k < r; ++k) {
    const int own = k % csize, ks = k / csize;
    if (rank == own && warp == 0) {
      double* c = col + (size_t)ks * r;
      const double d = c[k];
      const bool ok = d > 0.0 && isfinite(d);
      const double piv = ok ? sqrt(d) : 1.0;
      for (int i = k + 1 + lane; i < r; i += 32) c[i] /= piv;
      __syncwarp();
      if (lane == 0) {
        c[k] = piv;
        if (!ok) bad = 1;
      }
    }
    cluster_barrier();
    if (dsmem_ld32(dsmem_map(bad_s, (uint32_t)own))) {
      failed = true;
      break;
    }
    const uint32_t src = dsmem_map(col_s + (uint32_t)(ks * r) * 8u, (uint32_t)own);
    for (int i = k + tid; i < r; i += blockDim.x) colk[i] = dsmem_ld(src + 8u * (uint32_t)i);
    __syncthreads();
    for (int s = warp; s < nslots; s += nw) {
      const int j = s * csize + rank;
      if (j > k && j < r) {
        const double ljk = colk[j];
        double* c = col + (size_t)s * r;
        for (int i = j + lane; i < r; i += 32) c[i] -= colk[i] * ljk;
      }
    }
    __syncthreads();
  }
  cluster_barrier();
  if (!failed) {
    // L row-major in every CTA: Lf[i][k] = column k, row i (i >= k)
    for (int k = warp; k < r; k += nw) {
      const uint32_t src = dsmem_map(col_s + (uint32_t)((k / csize) * r) * 8u, (uint32_t)(k % csize));
      for (int i = k + lane; i < r; i += 32) Lf[(size_t)i * r + k] = dsmem_ld(src + 8u * (uint32_t)i);
    }
    __syncthreads();
    double* x = xw + (size_t)warp * r;
    for (int j = warp * csize + rank; j < r; j += nw * csize) {
      if (lane == 0) x[j] = 1.0 / Lf[(size_t)j * r + j];
      __syncwarp();
      for (int i = j + 1; i < r; ++i) {
        double sacc = 0.0;
        for (int k = j + lane; k < i; k += 32) sacc = fma(Lf[(size_t)i * r + k], x[k], sacc);
        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        if (lane == 0) x[i] = -sacc / Lf[(size_t)i * r + i];
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
  const size_t nslots = (size_t)(r + csize - 1) / csize;
  return sizeof(double) * (nslots * r + r + (size_t)r * r + 8 * (size_t)r);
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
        if (fabs(g) > 1e-15 * sqrt(a * b) && g != 0.0) {
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
  if (blockIdx.x == 0 && threadIdx.x == 0) *sweeps_out = sweep + 1;
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
  for (int s = 0; s < nslots; ++s) {
    const int c = s * csize + (int)rank;
    if (c < r)
      for (int i = threadIdx.x; i < r; i += blockDim.x) jcols[(int64_t)s * r + i] = Wc[(int64_t)c * r + i];
  }
  cluster_barrier();
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
        // |g| > 1e-15 sqrt(ab), without the square root
        if (g != 0.0 && g * g > 1e-30 * (a * b)) {
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
  if (blockIdx.x == 0 && threadIdx.x == 0) *sweeps_out = sweep + 1;
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

int jacobi_svd(lne_ctx* ctx, double* C, int r, double* U, double* S, int* sweeps_out) {
  if (r > 1024) {
    set_error("jacobi_svd: rank above 1024 is not supported");
    return LNE_ERR_UNSUPPORTED;
  }
  const int kMaxSweeps = kJacobiMaxSweeps;
  double* Wc = nullptr;
  int rc;
  if ((rc = dalloc(ctx, (void**)&Wc, sizeof(double) * r * r + sizeof(int) * (kMaxSweeps + 4), "jacobi work")))
    return rc;
  int* rotated = (int*)(Wc + (int64_t)r * r);
  int* d_sw = rotated + kMaxSweeps;
  k_jacobi_init<<<64, 256, 0, ctx->stream>>>(C, r, Wc, rotated, kMaxSweeps);
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
    e = cudaLaunchKernelEx(&cfg, kern, r, Wc, rotated, kMaxSweeps, d_sw);
    if (e == cudaSuccess) break;
    cudaGetLastError();
  }
  if (e != cudaSuccess) {
    dfree(ctx, Wc);
    set_error(std::string("jacobi_svd: cluster launch failed: ") + cudaGetErrorString(e));
    return LNE_ERR_CUDA;
  }
  k_jacobi_finish<<<1, 1024, 0, ctx->stream>>>(r, Wc, U, S);
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpyAsync(&h, d_sw, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dfree(ctx, Wc);
  LNE_CUDA_TRY(cudaGetLastError());
  if (sweeps_out) *sweeps_out = h;
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
  int rc = gemm_tall(ctx, In, ldi, (int)k, W, (int)c2, n, Out, ldo, nullptr);
  if (rc) return rc;
  LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int h = 0;
  LNE_CUDA_TRY(cudaMemcpy(&h, ctx->d_flags + kFlagNumeric, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == 2) { set_error("lne_gemm_tall: tensor-core wait timed out"); return LNE_ERR_CUDA; }
  return LNE_OK;
}
