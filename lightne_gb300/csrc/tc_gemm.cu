// Tall-skinny GEMMs of the randomized SVD on the tcgen05 tensor core:
//   update  Out (n x c2) = In (n x K) * W (K x c2)      [Q = Y R^-1, Z = B P, U = Z U_C]
//   Gram    G   (c1 x c2) = A^T B over 2048-row blocks   [CholeskyQR, C = Z^T B]
// Both accumulate in TMEM with kind::tf32 MMAs on operands split into a
// TF32 high part and a TF32 low part (x = hi + lo): D += hi*hi + hi*lo +
// lo*hi, which keeps FP32-level accuracy (the products dropped are ~2^-22
// relative), needed by CholeskyQR.  The CTA stages each 16-wide K slice of
// both operands in shared memory (converting and splitting on the way),
// one thread issues the MMAs, and tcgen05.commit on a per-stage mbarrier
// tells the stagers when a stage may be refilled.  Every wait is bounded:
// on a timeout the kernel sets the context's numeric flag to 2, waits once
// more (bounded), frees its TMEM and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "dense.h"
#include "lne_internal.h"
#include "tcgen05.cuh"

namespace lne {

namespace {

constexpr int kTcThreads = 128;  // 4 warps: the 128 TMEM lanes of an M = 128 tile
constexpr int kKc = 16;          // K elements staged per stage (two K = 8 MMAs)
constexpr int kStages = 2;
constexpr uint32_t kTileA = 128 * kKc * 4;  // bytes of one A part (hi or lo)
constexpr uint32_t kTileB = 256 * kKc * 4;  // bytes of one B part, sized for N = 256
constexpr uint32_t kStageBytes = 2 * kTileA + 2 * kTileB;
constexpr uint32_t kSmemBytes = kStages * kStageBytes + 64;
constexpr uint32_t kTmemCols = 256;
constexpr long long kWaitCycles = 2000000000LL;  // about one second

struct StageBufs {
  uint8_t* a_hi;
  uint8_t* a_lo;
  uint8_t* b_hi;
  uint8_t* b_lo;
};

__device__ __forceinline__ StageBufs stage_bufs(uint8_t* smem, int st) {
  uint8_t* base = smem + (size_t)st * kStageBytes;
  return StageBufs{base, base + kTileA, base + 2 * kTileA, base + 2 * kTileA + kTileB};
}

// Writes 16 K values of one operand row (hi and lo parts) to a stage.
__device__ __forceinline__ void put_row(uint8_t* hi, uint8_t* lo, uint32_t row, const float (&v)[kKc]) {
#pragma unroll
  for (int q = 0; q < kKc; q += 4) {
    float4 h, l;
    h.x = tc::to_tf32(v[q]);
    h.y = tc::to_tf32(v[q + 1]);
    h.z = tc::to_tf32(v[q + 2]);
    h.w = tc::to_tf32(v[q + 3]);
    l.x = v[q] - h.x;
    l.y = v[q + 1] - h.y;
    l.z = v[q + 2] - h.z;
    l.w = v[q + 3] - h.w;
    const uint32_t off = tc::kmajor_off(row, (uint32_t)q, kKc);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

// Issues the 3 x 2 MMAs of one stage (thread 0 only).
__device__ __forceinline__ void issue_stage(const StageBufs& b, uint32_t tmem, uint32_t idesc, bool first) {
  const uint32_t lbo = 128, sbo = (kKc / 4) * 128;
#pragma unroll
  for (int ks = 0; ks < kKc / 8; ++ks) {
    const uint32_t koff = (uint32_t)ks * 256;  // two core matrices along K per K = 8 step
    const uint64_t ah = tc::smem_desc(tc::smem_addr(b.a_hi) + koff, lbo, sbo);
    const uint64_t al = tc::smem_desc(tc::smem_addr(b.a_lo) + koff, lbo, sbo);
    const uint64_t bh = tc::smem_desc(tc::smem_addr(b.b_hi) + koff, lbo, sbo);
    const uint64_t bl = tc::smem_desc(tc::smem_addr(b.b_lo) + koff, lbo, sbo);
    tc::mma_tf32(tmem, ah, bh, idesc, (first && ks == 0) ? 0u : 1u);
    tc::mma_tf32(tmem, ah, bl, idesc, 1u);
    tc::mma_tf32(tmem, al, bh, idesc, 1u);
  }
}

struct TcShared {
  unsigned long long mbar[kStages];
  uint32_t tmem_base;
};

// Shared K-loop: stage(c, bufs) fills stage buffers for K slice c.
template <class StageFn>
__device__ __forceinline__ bool tc_kloop(uint8_t* smem, TcShared* sh, uint32_t tmem, uint32_t idesc, int nchunks,
                                         const volatile int* abort, StageFn stage) {
  bool ok = true;
  for (int c = 0; c < nchunks; ++c) {
    const int st = c % kStages;
    if (c >= kStages) {
      const uint32_t parity = (uint32_t)((c / kStages - 1) & 1);
      if (!tc::mbar_wait(tc::smem_addr(&sh->mbar[st]), parity, kWaitCycles, abort)) ok = false;
    }
    const StageBufs b = stage_bufs(smem, st);
    stage(c, b);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      issue_stage(b, tmem, idesc, c == 0);
      tc::commit(tc::smem_addr(&sh->mbar[st]));
    }
  }
  // the commit of the last stage arrives when every MMA issued before it is done
  if (nchunks > 0) {
    const int last = nchunks - 1;
    const uint32_t parity = (uint32_t)((last / kStages) & 1);
    if (!tc::mbar_wait(tc::smem_addr(&sh->mbar[last % kStages]), parity, kWaitCycles, abort)) ok = false;
  }
  // block-uniform verdict: the epilogue's tcgen05.ld is warp-synchronous
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  tc::fence_after_sync();
  return ok;
}

__device__ __forceinline__ void tc_setup(TcShared* sh) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) tc::mbar_init(tc::smem_addr(&sh->mbar[i]), 1);
    tc::fence_mbar_init();
  }
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tc::smem_addr(&sh->tmem_base), kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

__device__ __forceinline__ void tc_teardown(TcShared* sh, uint32_t tmem) {
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

// Out (rows m0..m0+127) = In * W;  B operand row j = column j of W.
__global__ void __launch_bounds__(kTcThreads) k_tc_gemm_tall(const float* __restrict__ In, int64_t ldi, int K,
                                                             const float* __restrict__ W, int c2, int nmma, int64_t n,
                                                             float* __restrict__ Out, int64_t ldo,
                                                             __nv_bfloat16* __restrict__ OutB, int* flags) {
  extern __shared__ __align__(128) uint8_t smem[];
  TcShared* sh = reinterpret_cast<TcShared*>(smem + kStages * kStageBytes);
  tc_setup(sh);
  const uint32_t tmem = sh->tmem_base;
  const int64_t m0 = (int64_t)blockIdx.x * 128;
  const int t = threadIdx.x;
  const int nchunks = (K + kKc - 1) / kKc;
  const uint32_t idesc = tc::idesc_tf32(128, nmma);
  const bool ok = tc_kloop(smem, sh, tmem, idesc, nchunks, flags + kFlagNumeric, [&](int c, const StageBufs& b) {
    const int k0 = c * kKc;
    // A: row t of the tile = In row m0 + t
    {
      float v[kKc];
      const int64_t row = m0 + t;
#pragma unroll
      for (int k = 0; k < kKc; ++k) v[k] = (row < n && k0 + k < K) ? In[row * ldi + k0 + k] : 0.0f;
      put_row(b.a_hi, b.a_lo, (uint32_t)t, v);
    }
    // B: rows j = t, t + 128 < nmma
    for (int j = t; j < nmma; j += kTcThreads) {
      float v[kKc];
#pragma unroll
      for (int k = 0; k < kKc; ++k) v[k] = (j < c2 && k0 + k < K) ? W[(int64_t)(k0 + k) * c2 + j] : 0.0f;
      put_row(b.b_hi, b.b_lo, (uint32_t)j, v);
    }
  });
  if (!ok) {
    // record the timeout; give the MMAs in flight one more bounded wait
    // before the TMEM they write is released
    if (t == 0) atomicExch(flags + kFlagNumeric, 2);
    const int last = nchunks - 1;
    if (last >= 0)
      tc::mbar_wait(tc::smem_addr(&sh->mbar[last % kStages]), (uint32_t)((last / kStages) & 1), kWaitCycles,
                    flags + kFlagTimeoutGuard);
  } else {
    const int w = t >> 5, lane = t & 31;
    const int64_t row = m0 + 32 * w + lane;
    for (int cc = 0; cc < nmma; cc += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)cc, v);
      if (row < n) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int col = cc + i;
          if (col < ldo) {
            const float x = col < c2 ? v[i] : 0.0f;
            Out[row * ldo + col] = x;
            if (OutB) OutB[row * ldo + col] = __float2bfloat16_rn(x);
          }
        }
      }
    }
    // columns beyond the MMA width (ldo > nmma cannot happen: nmma >= ldo)
  }
  tc_teardown(sh, tmem);
}

// partial[rb] (c1 x c2) = A[rows]^T B[rows] for the 2048-row block rb and the
// 128-row tile blockIdx.x of the output.
__global__ void __launch_bounds__(kTcThreads) k_tc_gram(const float* __restrict__ A, int64_t lda, int c1,
                                                        const float* __restrict__ B, int64_t ldb, int c2, int nmma,
                                                        int64_t n, float* __restrict__ partial, int* flags) {
  extern __shared__ __align__(128) uint8_t smem[];
  TcShared* sh = reinterpret_cast<TcShared*>(smem + kStages * kStageBytes);
  tc_setup(sh);
  const uint32_t tmem = sh->tmem_base;
  const int mt = blockIdx.x;
  const int64_t rb = blockIdx.y;
  const int64_t r0 = rb * 2048;
  const int64_t r1 = std::min<int64_t>(n, r0 + 2048);
  const int t = threadIdx.x;
  const int nchunks = (int)((r1 - r0 + kKc - 1) / kKc);
  const uint32_t idesc = tc::idesc_tf32(128, nmma);
  const int ca = mt * 128 + t;
  const bool ok = tc_kloop(smem, sh, tmem, idesc, nchunks, flags + kFlagNumeric, [&](int c, const StageBufs& b) {
    const int64_t k0 = r0 + (int64_t)c * kKc;
    {
      float v[kKc];
#pragma unroll
      for (int k = 0; k < kKc; ++k) v[k] = (k0 + k < r1 && ca < c1) ? A[(k0 + k) * lda + ca] : 0.0f;
      put_row(b.a_hi, b.a_lo, (uint32_t)t, v);
    }
    for (int j = t; j < nmma; j += kTcThreads) {
      float v[kKc];
#pragma unroll
      for (int k = 0; k < kKc; ++k) v[k] = (k0 + k < r1 && j < c2) ? B[(k0 + k) * ldb + j] : 0.0f;
      put_row(b.b_hi, b.b_lo, (uint32_t)j, v);
    }
  });
  if (!ok) {
    // record the timeout; give the MMAs in flight one more bounded wait
    // before the TMEM they write is released
    if (t == 0) atomicExch(flags + kFlagNumeric, 2);
    const int last = nchunks - 1;
    if (last >= 0)
      tc::mbar_wait(tc::smem_addr(&sh->mbar[last % kStages]), (uint32_t)((last / kStages) & 1), kWaitCycles,
                    flags + kFlagTimeoutGuard);
  } else {
    const int w = t >> 5, lane = t & 31;
    const int i = mt * 128 + 32 * w + lane;
    float* out = partial + rb * (int64_t)c1 * c2;
    for (int cc = 0; cc < nmma; cc += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)cc, v);
      if (i < c1) {
#pragma unroll
        for (int q = 0; q < 16; ++q)
          if (cc + q < c2) out[(int64_t)i * c2 + cc + q] = v[q];
      }
    }
  }
  tc_teardown(sh, tmem);
}

__global__ void k_gram_reduce_tc(const float* __restrict__ partial, int64_t nb, int64_t cnt, double* __restrict__ G) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  double s = 0.0;
  for (int64_t b = 0; b < nb; ++b) s += (double)partial[b * cnt + t];
  G[t] = s;
}

}  // namespace

bool tc_supported(int c2) { return c2 >= 1 && c2 <= 256; }

int tc_gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
                 int64_t ldo, __nv_bfloat16* OutB) {
  if (n <= 0) return LNE_OK;
  const int nmma = std::max(16, (int)((std::max<int64_t>(c2, ldo) + 15) / 16 * 16));
  if (nmma > 256) {
    set_error("tc_gemm_tall: more than 256 output columns");
    return LNE_ERR_UNSUPPORTED;
  }
  cudaFuncSetAttribute(k_tc_gemm_tall, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  k_tc_gemm_tall<<<(unsigned)((n + 127) / 128), kTcThreads, kSmemBytes, ctx->stream>>>(In, ldi, k, W, c2, nmma, n, Out,
                                                                                       ldo, OutB, ctx->d_flags);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

int tc_gram(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
            double* G) {
  const int nmma = std::max(16, (c2 + 15) / 16 * 16);
  if (nmma > 256) {
    set_error("tc_gram: more than 256 columns");
    return LNE_ERR_UNSUPPORTED;
  }
  const int64_t nb = std::max<int64_t>(1, (n + 2047) / 2048);
  float* partial = nullptr;
  int rc = dalloc(ctx, (void**)&partial, sizeof(float) * nb * c1 * c2, "gram partials");
  if (rc) return rc;
  cudaFuncSetAttribute(k_tc_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  dim3 grid((unsigned)((c1 + 127) / 128), (unsigned)nb);
  k_tc_gram<<<grid, kTcThreads, kSmemBytes, ctx->stream>>>(A, lda, c1, B, ldb, c2, nmma, n, partial, ctx->d_flags);
  const int64_t cnt = (int64_t)c1 * c2;
  k_gram_reduce_tc<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(partial, nb, cnt, G);
  dfree(ctx, partial);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

// Gram with caller-provided partial-sum storage (nb * c1 * c2 floats,
// nb = ceil(n / 2048)); the tensor-core path only (c2 <= 256).  Every
// partial is overwritten, so the storage needs no clearing.
int tc_gram_into(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
                 double* G, float* partial) {
  const int nmma = std::max(16, (c2 + 15) / 16 * 16);
  if (nmma > 256) {
    set_error("tc_gram_into: more than 256 columns");
    return LNE_ERR_UNSUPPORTED;
  }
  const int64_t nb = std::max<int64_t>(1, (n + 2047) / 2048);
  cudaFuncSetAttribute(k_tc_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  dim3 grid((unsigned)((c1 + 127) / 128), (unsigned)nb);
  k_tc_gram<<<grid, kTcThreads, kSmemBytes, ctx->stream>>>(A, lda, c1, B, ldb, c2, nmma, n, partial, ctx->d_flags);
  const int64_t cnt = (int64_t)c1 * c2;
  k_gram_reduce_tc<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(partial, nb, cnt, G);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

}  // namespace lne
