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
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
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
  // one outcome for the whole block: the epilogue's tcgen05.ld is warp-synchronous
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
                                                             Copy16 OutB, int* flags) {
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
            copy16_put(OutB, row * ldo + col, x);
          }
        }
      }
    }
    // columns beyond the MMA width (ldo > nmma cannot happen: nmma >= ldo)
  }
  tc_teardown(sh, tmem);
}


// ---------------------------------------------------------------------------
// Streaming forms (persistent CTAs, one per SM).  The operand rows are copied
// with 16-byte cp.async straight into the K-major core-matrix positions of a
// ring of raw slices (so up to kRing - 1 slices are in flight while the tensor
// core works), split into TF32 high and low parts by an elementwise pass into
// one of two operand buffers, and consumed by the same three-MMA scheme.
// Raw slots are free once converted, so refills never wait for the tensor
// core; operand buffers are reused after the commit of the MMAs that read
// them.
// ---------------------------------------------------------------------------
constexpr int kSThreads = 256;
constexpr int kSlice = 16;                                 // K per slice
constexpr uint32_t kSliceRowBytes = kSlice * 4;            // one operand row of a slice
constexpr uint32_t kASlice = 128 * kSliceRowBytes;         // 8 KB: 128 rows x 16 K
constexpr int kGemmRing = 4;
constexpr int kGramRing = 6;

struct StreamShared {
  unsigned long long mbar[2];
  uint32_t tmem_base;
};

__device__ __forceinline__ void split4(const float4& x, float4& h, float4& l) {
  h.x = tc::to_tf32(x.x);
  h.y = tc::to_tf32(x.y);
  h.z = tc::to_tf32(x.z);
  h.w = tc::to_tf32(x.w);
  l.x = x.x - h.x;
  l.y = x.y - h.y;
  l.z = x.z - h.z;
  l.w = x.w - h.w;
}

// 2 K = 8 steps x (hi*hi + hi*lo + lo*hi) on one slice.  The descriptors
// of the slice's first K step are passed in; the start address field is
// address >> 4 (shared memory addresses stay below 2^18, so the 14-bit field
// never carries), so the next K step (256 bytes on) is descriptor + 16.
template <int SL = kSlice>
__device__ __forceinline__ void issue_slice(uint32_t tmem_d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                            uint32_t idesc, bool first) {
#pragma unroll
  for (int ks = 0; ks < SL / 8; ++ks) {
    const uint64_t ko = (uint64_t)(ks * 16);
    tc::mma_tf32(tmem_d, ah + ko, bh + ko, idesc, (first && ks == 0) ? 0u : 1u);
    tc::mma_tf32(tmem_d, ah + ko, bl + ko, idesc, 1u);
    tc::mma_tf32(tmem_d, al + ko, bh + ko, idesc, 1u);
  }
}
// The same with the A descriptors advanced by `a_step` (in 16-byte units)
// per K = 8 step and the B descriptors by 16.
__device__ __forceinline__ void issue_slice_a(uint32_t tmem_d, uint64_t ah, uint64_t al, uint32_t a_step, uint64_t bh,
                                              uint64_t bl, uint32_t idesc, bool first) {
#pragma unroll
  for (int ks = 0; ks < kSlice / 8; ++ks) {
    const uint64_t ka = (uint64_t)(ks * a_step), kb = (uint64_t)(ks * 16);
    tc::mma_tf32(tmem_d, ah + ka, bh + kb, idesc, (first && ks == 0) ? 0u : 1u);
    tc::mma_tf32(tmem_d, ah + ka, bl + kb, idesc, 1u);
    tc::mma_tf32(tmem_d, al + ka, bh + kb, idesc, 1u);
  }
}
template <int SL = kSlice>
__device__ __forceinline__ uint64_t slice_desc(uint32_t saddr) {
  return tc::smem_desc(saddr, 128, (SL / 4) * 128);
}

__device__ __forceinline__ void stream_setup(StreamShared* sh, uint32_t cols) {
  if (threadIdx.x == 0) {
    tc::mbar_init(tc::smem_addr(&sh->mbar[0]), 1);
    tc::mbar_init(tc::smem_addr(&sh->mbar[1]), 1);
    tc::fence_mbar_init();
  }
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tc::smem_addr(&sh->tmem_base), cols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// After a timed-out wait: record it, wait (bounded, not abortable) for the
// last commit so that no MMA still writes the TMEM being released, drain the
// copies in flight, release the TMEM.
__device__ __forceinline__ void stream_finish(StreamShared* sh, uint32_t tmem, uint32_t cols, bool ok,
                                              int64_t last_commit, int* flags) {
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(flags + kFlagNumeric, 2);
    if (last_commit >= 0)
      tc::mbar_wait(tc::smem_addr(&sh->mbar[last_commit & 1]), (uint32_t)((last_commit >> 1) & 1), kWaitCycles,
                    flags + kFlagTimeoutGuard);
  }
  tc::cp_async_wait<0>();
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, cols);
  }
}

// Out (n x ldo) = In (n x K) * W (K x c2), persistent over 128-row tiles.
// W (split, K-major per 16-K slice) stays in shared memory.
__global__ void __launch_bounds__(kSThreads, 1) k_tc_gemm_stream(const float* __restrict__ In, int64_t ldi, int K,
                                                                 const float* __restrict__ W, int c2, int nmma,
                                                                 int64_t n, float* __restrict__ Out, int64_t ldo,
                                                                 Copy16 OutB, int* flags) {
  extern __shared__ __align__(1024) uint8_t stream_smem[];
  const int nsl = (K + kSlice - 1) / kSlice;
  const uint32_t wslice = (uint32_t)nmma * kSliceRowBytes;
  uint8_t* w_hi = stream_smem;
  uint8_t* w_lo = stream_smem + (size_t)nsl * wslice;
  uint8_t* raw = w_lo + (size_t)nsl * wslice;
  uint8_t* conv = raw + (size_t)kGemmRing * kASlice;  // 2 x (hi, lo)
  StreamShared* sh = reinterpret_cast<StreamShared*>(conv + 4 * kASlice);
  const int t = threadIdx.x;

  // W into shared memory: element (j, k) of the B operand is W[k][j]
  for (int idx = t; idx < nsl * 4 * nmma; idx += kSThreads) {
    const int j = idx % nmma, sq = idx / nmma, sl = sq >> 2, q = sq & 3;
    float4 x;
    float* xv = reinterpret_cast<float*>(&x);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = sl * kSlice + 4 * q + e;
      xv[e] = (j < c2 && k < K) ? W[(int64_t)k * c2 + j] : 0.0f;
    }
    float4 h, l;
    split4(x, h, l);
    const uint32_t off = (uint32_t)sl * wslice + tc::kmajor_off((uint32_t)j, (uint32_t)(4 * q), kSlice);
    *reinterpret_cast<float4*>(w_hi + off) = h;
    *reinterpret_cast<float4*>(w_lo + off) = l;
  }
  stream_setup(sh, 256);
  const uint32_t tmem = sh->tmem_base;
  const uint32_t idesc = tc::idesc_tf32(128, nmma);
  const int64_t ntiles = (n + 127) / 128;
  const int64_t my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t total = my_tiles * nsl;

  auto issue_load = [&](int64_t g) {
    const int64_t tile = blockIdx.x + (g / nsl) * gridDim.x;
    const int k0 = (int)(g % nsl) * kSlice;
    const uint32_t dst0 = tc::smem_addr(raw + (size_t)(g % kGemmRing) * kASlice);
    for (int idx = t; idx < 128 * 4; idx += kSThreads) {
      const int r = idx >> 2, q = idx & 3;
      const int64_t row = tile * 128 + r;
      const int k = k0 + 4 * q;
      const int kb = K - k;
      const uint32_t bytes = (row < n && kb > 0) ? (uint32_t)(kb >= 4 ? 16 : 4 * kb) : 0u;
      const float* src = bytes ? In + row * ldi + k : In;
      tc::cp_async16(dst0 + tc::kmajor_off((uint32_t)r, (uint32_t)(4 * q), kSlice), src, bytes);
    }
  };

  bool ok = true;
  int64_t last_commit = -1;
  for (int64_t g = 0; g < kGemmRing - 1; ++g) {
    if (g < total) issue_load(g);
    tc::cp_async_commit();
  }
  for (int64_t g = 0; g < total && ok; ++g) {
    if (g + kGemmRing - 1 < total) issue_load(g + kGemmRing - 1);
    tc::cp_async_commit();
    tc::cp_async_wait<kGemmRing - 1>();
    const int cb = (int)(g & 1);
    // operand buffer cb is free once the MMAs of slice g - 2 are done: one
    // thread waits, the barrier releases the others
    if (g >= 2 && t == 0 &&
        !tc::mbar_wait(tc::smem_addr(&sh->mbar[cb]), (uint32_t)(((g - 2) >> 1) & 1), kWaitCycles,
                       flags + kFlagNumeric))
      ok = false;
    __syncthreads();  // slice g visible to every thread; operand buffer cb free
    {
      const float4* src = reinterpret_cast<const float4*>(raw + (size_t)(g % kGemmRing) * kASlice);
      float4* hi = reinterpret_cast<float4*>(conv + (size_t)cb * 2 * kASlice);
      float4* lo = reinterpret_cast<float4*>(conv + (size_t)cb * 2 * kASlice + kASlice);
      for (int idx = t; idx < (int)(kASlice / 16); idx += kSThreads) {
        float4 h, l;
        split4(src[idx], h, l);
        hi[idx] = h;
        lo[idx] = l;
      }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok) break;
    const int sl = (int)(g % nsl);
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t a_hi = tc::smem_addr(conv + (size_t)cb * 2 * kASlice);
      issue_slice(tmem, slice_desc(a_hi), slice_desc(a_hi + kASlice), slice_desc(tc::smem_addr(w_hi) + sl * wslice),
                  slice_desc(tc::smem_addr(w_lo) + sl * wslice), idesc, sl == 0);
      tc::commit(tc::smem_addr(&sh->mbar[cb]));
    }
    last_commit = g;
    if (sl == nsl - 1) {
      // tile done: wait for its MMAs, then write it out
      if (!tc::mbar_wait(tc::smem_addr(&sh->mbar[cb]), (uint32_t)((g >> 1) & 1), kWaitCycles, flags + kFlagNumeric))
        ok = false;
      ok = __syncthreads_and(ok ? 1 : 0) != 0;
      if (!ok) break;
      tc::fence_after_sync();
      const int64_t tile = blockIdx.x + (g / nsl) * gridDim.x;
      const int w = t >> 5, lane = t & 31, lg = w & 3;
      const int64_t row = tile * 128 + 32 * lg + lane;
      const bool vec = ((ldo & 3) == 0) && ((reinterpret_cast<uintptr_t>(Out) & 15) == 0);
      for (int cg = w >> 2; cg * 16 < nmma; cg += 2) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * lg) << 16) + (uint32_t)(cg * 16), v);
        if (row < n) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cg * 16 + i >= c2) v[i] = 0.0f;
          float* orow = Out + row * ldo + cg * 16;
          if (vec && cg * 16 + 16 <= ldo) {
#pragma unroll
            for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(orow + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (cg * 16 + i < ldo) orow[i] = v[i];
          }
          copy16_put_row16(OutB, row, ldo, cg * 16, v, (int)std::min<int64_t>(16, ldo - cg * 16));
        }
      }
      tc::fence_before_sync();  // the next tile's first MMA follows a __syncthreads
    }
  }
  stream_finish(sh, tmem, 256, ok, last_commit, flags);
}

// Warp-specialised form of the update GEMM (same operands, layouts and
// MMAs as k_tc_gemm_stream), for W of at most kWsMaxCols columns:
//   warps 8-9 (loaders)  cp.async of raw 16-K slices of In into a ring of
//                        `ring` slots; raw_full[s] completes when they land
//   warps 0-3 (split)    raw slot -> TF32 hi/lo operand stage (2 stages),
//                        releases the raw slot, publishes the stage
//   warp 10 lane 0 (MMA) 6 MMAs per slice into one of two TMEM accumulators;
//                        its commits release the stage and, after a tile's
//                        last slice, hand the accumulator to the epilogue
//   warps 4-7 (store)    TMEM -> registers -> Out (and OutB), then release
//                        the accumulator
// so that loads, splitting, MMAs and stores of successive slices and tiles
// overlap instead of meeting at block-wide barriers.  Every wait is bounded;
// a timeout sets the context's numeric flag to 2, which ends every other
// wait within 64 polls.
constexpr int kWsLoadWarps = 4;  // warps 8 .. 8 + kWsLoadWarps - 1
constexpr int kWsThreads = 32 * (9 + kWsLoadWarps);
constexpr int kWsLoadWarp = 8;
constexpr int kWsMmaWarp = 8 + kWsLoadWarps;
constexpr int kWsMaxRing = 8;
constexpr int kWsMaxCols = 256;  // two accumulators of up to 256 TMEM columns
constexpr int kWsPrefetchTiles = 2;  // tiles of In prefetched into L2 ahead of the TMA ring

struct WsShared {
  unsigned long long raw_full[kWsMaxRing], raw_empty[kWsMaxRing];
  unsigned long long conv_full[2], conv_empty[2], acc_full[2], acc_empty[2];
  uint32_t tmem_base;
};

template <bool TMA>
__global__ void __launch_bounds__(kWsThreads, 1) k_tc_gemm_ws(const __grid_constant__ CUtensorMap tmap,
                                                             const float* __restrict__ In, int64_t ldi, int K,
                                                             const float* __restrict__ W, int c2, int nmma, int ring,
                                                             int64_t n, float* __restrict__ Out, int64_t ldo,
                                                             Copy16 OutB, int* flags) {
  extern __shared__ __align__(1024) uint8_t stream_smem[];
  const int nsl = (K + kSlice - 1) / kSlice;
  const uint32_t wslice = (uint32_t)nmma * kSliceRowBytes;
  uint8_t* w_hi = stream_smem;
  uint8_t* w_lo = stream_smem + (size_t)nsl * wslice;
  uint8_t* raw = w_lo + (size_t)nsl * wslice;
  uint8_t* conv = raw + (size_t)ring * kASlice;  // 2 stages x (hi, lo)
  WsShared* sh = reinterpret_cast<WsShared*>(conv + 4 * kASlice);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  for (int idx = t; idx < nsl * 4 * nmma; idx += kWsThreads) {
    const int j = idx % nmma, sq = idx / nmma, sl = sq >> 2, q = sq & 3;
    float4 x;
    float* xv = reinterpret_cast<float*>(&x);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = sl * kSlice + 4 * q + e;
      xv[e] = (j < c2 && k < K) ? W[(int64_t)k * c2 + j] : 0.0f;
    }
    float4 h, l;
    split4(x, h, l);
    const uint32_t off = (uint32_t)sl * wslice + tc::kmajor_off((uint32_t)j, (uint32_t)(4 * q), kSlice);
    *reinterpret_cast<float4*>(w_hi + off) = h;
    *reinterpret_cast<float4*>(w_lo + off) = l;
  }
  if (t == 0) {
    for (int s = 0; s < ring; ++s) {
      tc::mbar_init(tc::smem_addr(&sh->raw_full[s]), TMA ? 1 : 32 * kWsLoadWarps);
      tc::mbar_init(tc::smem_addr(&sh->raw_empty[s]), 4);
    }
    for (int c = 0; c < 2; ++c) {
      tc::mbar_init(tc::smem_addr(&sh->conv_full[c]), 4);
      tc::mbar_init(tc::smem_addr(&sh->conv_empty[c]), 1);
      tc::mbar_init(tc::smem_addr(&sh->acc_full[c]), 1);
      tc::mbar_init(tc::smem_addr(&sh->acc_empty[c]), 4);
    }
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&sh->tmem_base), 512);
  tc::fence_proxy_async_smem();  // W, written by every thread, is read by the tensor core
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sh->tmem_base;
  const int64_t ntiles = (n + 127) / 128;
  const int64_t my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t total = my_tiles * nsl;
  int* abortf = flags + kFlagNumeric;
  auto fail = [&]() { atomicExch(abortf, 2); };
  int64_t last_commit = -1;  // MMA thread: slice of its last commit

  if (TMA && warp == kWsLoadWarp) {
    // one thread: a 16 x 128 box (8 KB, 64-byte swizzle) per slice; at the
    // start of each tile the boxes of the tile kWsPrefetchTiles on are
    // prefetched into L2, so that the ring's loads wait on L2, not DRAM
    if (lane == 0) {
      for (int64_t g = 0; g < total; ++g) {
        const int s = (int)(g % ring);
        if (g % nsl == 0) {
          const int64_t pj = g / nsl + kWsPrefetchTiles;
          if (pj < my_tiles) {
            const int64_t ptile = blockIdx.x + pj * gridDim.x;
            for (int q = 0; q < nsl; ++q) tc::tma_prefetch_2d(&tmap, q * kSlice, (int)(ptile * 128));
          }
          if (g == 0)  // the first tiles
            for (int64_t j0 = 1; j0 < kWsPrefetchTiles && j0 < my_tiles; ++j0)
              for (int q = 0; q < nsl; ++q)
                tc::tma_prefetch_2d(&tmap, q * kSlice, (int)((blockIdx.x + j0 * gridDim.x) * 128));
        }
        if (g >= ring &&
            !tc::mbar_wait(tc::smem_addr(&sh->raw_empty[s]), (uint32_t)((g / ring - 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        const int64_t tile = blockIdx.x + (g / nsl) * gridDim.x;
        const uint32_t mb = tc::smem_addr(&sh->raw_full[s]);
        tc::mbar_arrive_expect_tx(mb, kASlice);
        tc::tma_load_2d(tc::smem_addr(raw + (size_t)s * kASlice), &tmap, (int)(g % nsl) * kSlice, (int)(tile * 128),
                        mb);
      }
    }
    __syncwarp();
  } else if (TMA && warp > kWsLoadWarp && warp < kWsLoadWarp + kWsLoadWarps) {
    // idle loader warps of the TMA form
  } else if (warp >= kWsLoadWarp && warp < kWsLoadWarp + kWsLoadWarps) {
    const int ll = t - 32 * kWsLoadWarp;  // loader lane
    for (int64_t g = 0; g < total; ++g) {
      const int s = (int)(g % ring);
      if (g >= ring &&
          !tc::mbar_wait(tc::smem_addr(&sh->raw_empty[s]), (uint32_t)((g / ring - 1) & 1), kWaitCycles, abortf)) {
        if (lane == 0) fail();
        break;
      }
      const int64_t tile = blockIdx.x + (g / nsl) * gridDim.x;
      const int k0 = (int)(g % nsl) * kSlice;
      const uint32_t dst0 = tc::smem_addr(raw + (size_t)s * kASlice);
      for (int idx = ll; idx < 128 * 4; idx += 32 * kWsLoadWarps) {
        const int r = idx >> 2, q = idx & 3;
        const int64_t row = tile * 128 + r;
        const int k = k0 + 4 * q;
        const int kb = K - k;
        const uint32_t bytes = (row < n && kb > 0) ? (uint32_t)(kb >= 4 ? 16 : 4 * kb) : 0u;
        const float* src = bytes ? In + row * ldi + k : In;
        tc::cp_async16(dst0 + tc::kmajor_off((uint32_t)r, (uint32_t)(4 * q), kSlice), src, bytes);
      }
      tc::cp_async_mbar_arrive(tc::smem_addr(&sh->raw_full[s]));
    }
    tc::cp_async_wait_all();
  } else if (warp < 4) {
    for (int64_t g = 0; g < total; ++g) {
      const int s = (int)(g % ring), c = (int)(g & 1);
      if (!tc::mbar_wait(tc::smem_addr(&sh->raw_full[s]), (uint32_t)((g / ring) & 1), kWaitCycles, abortf) ||
          (g >= 2 &&
           !tc::mbar_wait(tc::smem_addr(&sh->conv_empty[c]), (uint32_t)(((g >> 1) - 1) & 1), kWaitCycles, abortf))) {
        if (lane == 0) fail();
        break;
      }
      const float4* src = reinterpret_cast<const float4*>(raw + (size_t)s * kASlice);
      float4* hi = reinterpret_cast<float4*>(conv + (size_t)c * 2 * kASlice);
      float4* lo = reinterpret_cast<float4*>(conv + (size_t)c * 2 * kASlice + kASlice);
#pragma unroll
      for (int idx = t; idx < (int)(kASlice / 16); idx += 128) {
        float4 h, l;
        split4(src[idx], h, l);
        hi[idx] = h;
        lo[idx] = l;
      }
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(tc::smem_addr(&sh->raw_empty[s]));
        tc::mbar_arrive(tc::smem_addr(&sh->conv_full[c]));
      }
    }
  } else if (warp == kWsMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_tf32(128, nmma);
      for (int64_t g = 0; g < total; ++g) {
        const int c = (int)(g & 1);
        const int sl = (int)(g % nsl);
        const int64_t j = g / nsl;
        const int b = (int)(j & 1);
        if (sl == 0 && j >= 2 &&
            !tc::mbar_wait(tc::smem_addr(&sh->acc_empty[b]), (uint32_t)(((j >> 1) - 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        if (!tc::mbar_wait(tc::smem_addr(&sh->conv_full[c]), (uint32_t)((g >> 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        tc::fence_after_sync();
        const uint32_t a_hi = tc::smem_addr(conv + (size_t)c * 2 * kASlice);
        // A: the TMA's 64-byte swizzle (8-row atoms 512 bytes apart; the
        // second K = 8 step 32 bytes into the atom) or the no-swizzle
        // core-matrix layout of the cp.async form
        const uint64_t ah = TMA ? tc::smem_desc_sw64(a_hi, 512) : slice_desc(a_hi);
        const uint64_t al = TMA ? tc::smem_desc_sw64(a_hi + kASlice, 512) : slice_desc(a_hi + kASlice);
        issue_slice_a(tmem + (uint32_t)(b * kWsMaxCols), ah, al, TMA ? 2u : 16u,
                      slice_desc(tc::smem_addr(w_hi) + sl * wslice), slice_desc(tc::smem_addr(w_lo) + sl * wslice),
                      idesc, sl == 0);
        tc::commit(tc::smem_addr(&sh->conv_empty[c]));
        if (sl == nsl - 1) tc::commit(tc::smem_addr(&sh->acc_full[b]));
        last_commit = g;
      }
      // nothing may still write TMEM when it is released: wait (bounded,
      // not abortable) for the last commit
      if (last_commit >= 0)
        tc::mbar_wait(tc::smem_addr(&sh->conv_empty[last_commit & 1]), (uint32_t)((last_commit >> 1) & 1),
                      kWaitCycles, flags + kFlagTimeoutGuard);
    }
    __syncwarp();
  } else {
    const int lg = warp & 3;  // TMEM lanes 32 lg ..
    const bool vec = ((ldo & 3) == 0) && ((reinterpret_cast<uintptr_t>(Out) & 15) == 0);
    for (int64_t j = 0; j < my_tiles; ++j) {
      const int b = (int)(j & 1);
      if (!tc::mbar_wait(tc::smem_addr(&sh->acc_full[b]), (uint32_t)((j >> 1) & 1), kWaitCycles, abortf)) {
        if (lane == 0) fail();
        break;
      }
      tc::fence_after_sync();
      const int64_t tile = blockIdx.x + j * gridDim.x;
      const int64_t row = tile * 128 + 32 * lg + lane;
      for (int cg = 0; cg * 16 < nmma; ++cg) {
        float v[16];
        tc::tmem_ld16(tmem + (uint32_t)(b * kWsMaxCols) + ((uint32_t)(32 * lg) << 16) + (uint32_t)(cg * 16), v);
        if (row < n) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cg * 16 + i >= c2) v[i] = 0.0f;
          float* orow = Out + row * ldo + cg * 16;
          if (vec && cg * 16 + 16 <= ldo) {
#pragma unroll
            for (int i = 0; i < 16; i += 4)
              *reinterpret_cast<float4*>(orow + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (cg * 16 + i < ldo) orow[i] = v[i];
          }
          copy16_put_row16(OutB, row, ldo, cg * 16, v, (int)std::min<int64_t>(16, ldo - cg * 16));
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_addr(&sh->acc_empty[b]));
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// Partial Gram of one contiguous range of SL-row slices per CTA (SL = 32
// where the stages fit in shared memory, else 16):
// partial[b] (c1 x c2) = A[rows]^T B[rows].  Both 128-column tiles of A are
// accumulated by the CTA (D0 for columns 0..127 of A, D1 for 128..255; D1
// sits right after D0 in the TMEM column space).  When A and B are the same
// matrix (sym), D1 only computes columns >= 128 and the reduction mirrors
// the lower triangle.
//
// The tensor core accumulates in FP32 without rounding to nearest (the
// low bits of each addition are dropped), so a long accumulation chain
// drifts towards zero by about 2^-25 of the sum per MMA.  Every kGroup
// slices (64 rows) the TMEM sums are therefore added into FP32 registers
// (rounded to nearest) and the next group starts a fresh TMEM sum.  (A group
// is 64 / SL slices.)  With
// room for two TMEM sets the group just finished is read while the next
// one accumulates in the other set; otherwise the drain waits for the
// group's MMAs.
constexpr int kGroupRows = 64;
constexpr int kMaxChunks = 9;  // 16-column chunks per thread: sets up to 288 columns

template <int SL, int RING>
__global__ void __launch_bounds__(kSThreads, 1) k_tc_gram_stream(const float* __restrict__ A, int64_t lda, int c1,
                                                                 const float* __restrict__ B, int64_t ldb, int c2,
                                                                 int nmma, int64_t n, int sym, int64_t per,
                                                                 float* __restrict__ partial, int* flags) {
  extern __shared__ __align__(1024) uint8_t stream_smem[];
  const int mt = c1 > 128 ? 2 : 1;
  constexpr uint32_t kRowBytes = SL * 4;   // one operand row of a slice
  constexpr int kGroup = kGroupRows / SL;
  constexpr int kTpr = kSThreads / SL;     // loading threads per slice row
  constexpr int kQ = SL / 4;               // K groups per slice
  const uint32_t a_part = (uint32_t)(128 * mt) * kRowBytes;   // one part (hi or lo) of the A operand
  const uint32_t b_part = sym ? 0u : (uint32_t)nmma * kRowBytes;
  const uint32_t stage = 2 * a_part + 2 * b_part;
  const int c1p = (c1 + 3) & ~3, c2p = sym ? 0 : (c2 + 3) & ~3;
  const uint32_t raw_slot = (uint32_t)(SL * (c1p + c2p) * 4);
  uint8_t* conv = stream_smem;
  uint8_t* raw = stream_smem + 2 * (size_t)stage;
  StreamShared* sh = reinterpret_cast<StreamShared*>(raw + (size_t)RING * raw_slot);
  const int t = threadIdx.x;
  stream_setup(sh, 512);
  const uint32_t tmem = sh->tmem_base;
  const int n1 = sym ? nmma - 128 : nmma;  // N of D1
  const int set_cols = mt == 2 ? nmma + n1 : nmma;
  const bool dbuf = 2 * set_cols <= 512;
  const uint32_t idesc0 = tc::idesc_tf32(128, nmma);
  const uint32_t idesc1 = tc::idesc_tf32(128, n1 > 0 ? n1 : 16);
  const int64_t nslices = (n + SL - 1) / SL;
  const int64_t s0 = (int64_t)blockIdx.x * per;
  const int64_t left = nslices - s0;
  const int64_t total = left <= 0 ? 0 : (left < per ? left : per);
  const int qa = c1p >> 2, qb = c2p >> 2;
  const int w = t >> 5, lane = t & 31, lg = w & 3, half = w >> 2;
  const int nchunks = set_cols / 16;
  const uint32_t lane_addr = (uint32_t)(32 * lg) << 16;

  float acc[kMaxChunks][16];
#pragma unroll
  for (int i = 0; i < kMaxChunks; ++i)
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[i][e] = 0.0f;
  // adds the TMEM set at column `base` into acc (warp-collective loads)
  auto drain = [&](uint32_t base) {
#pragma unroll
    for (int i = 0; i < kMaxChunks; ++i) {
      const int ch = half + 2 * i;
      if (ch < nchunks) {
        float v[16];
        tc::tmem_ld16(tmem + lane_addr + base + (uint32_t)(ch * 16), v);
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[i][e] += v[e];
      }
    }
  };
  auto set_base = [&](int64_t g) -> uint32_t { return dbuf ? (uint32_t)(((g / kGroup) & 1) * 256) : 0u; };

  // Loads: thread t copies row t / kTpr of the slice, 16-byte chunks
  // t % kTpr, t % kTpr + kTpr, ...; rows past n land as zeros.
  const int lk = t / kTpr, lq = t % kTpr;
  auto issue_load = [&](int64_t g) {
    const int64_t row = (s0 + g) * SL + lk;
    const bool rv = row < n;
    const uint32_t dst0 = tc::smem_addr(raw + (size_t)(g % RING) * raw_slot);
    const float* arow = A + (rv ? row : 0) * lda;
    for (int q = lq; q < qa; q += kTpr) {
      const int cb = c1 - 4 * q;
      tc::cp_async16(dst0 + (uint32_t)((lk * c1p + 4 * q) * 4), arow + 4 * q,
                     rv ? (uint32_t)(cb >= 4 ? 16 : 4 * cb) : 0u);
    }
    if (!sym) {
      const float* brow = B + (rv ? row : 0) * ldb;
      for (int q = lq; q < qb; q += kTpr) {
        const int cb = c2 - 4 * q;
        tc::cp_async16(dst0 + (uint32_t)((SL * c1p + lk * c2p + 4 * q) * 4), brow + 4 * q,
                       rv ? (uint32_t)(cb >= 4 ? 16 : 4 * cb) : 0u);
      }
    }
  };
  // Conversion of operand row j (a column of the data), K group q (raw rows
  // 4q..4q+3).  Thread t takes column t % 128 with groups q0 = (t / 128)
  // kQ / 2 .. q0 + kQ / 2 - 1, and the columns past 128 are spread one
  // (column, group) per thread: e -> (128 + e / kQ, e % kQ).
  auto convert_one = [&](const float* rs, int ld, int j, int q, uint8_t* hi, uint32_t part) {
    const float* col = rs + (4 * q) * ld + j;
    const float4 x = make_float4(col[0], col[ld], col[2 * ld], col[3 * ld]);
    float4 h, l;
    split4(x, h, l);
    const uint32_t off = tc::kmajor_off((uint32_t)j, (uint32_t)(4 * q), SL);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(hi + part + off) = l;
  };
  auto convert = [&](const float* rs, int ld, int cn, uint8_t* hi, uint32_t part) {
    const int j = t & 127, q0 = (t >> 7) * (kQ / 2);
    if (j < cn) {
#pragma unroll
      for (int q = 0; q < kQ / 2; ++q) convert_one(rs, ld, j, q0 + q, hi, part);
    }
    for (int e = t; e < kQ * (cn - 128); e += kSThreads) convert_one(rs, ld, 128 + e / kQ, e % kQ, hi, part);
  };

  bool ok = true;
  int64_t last_commit = -1;
  for (int64_t g = 0; g < RING - 1; ++g) {
    if (g < total) issue_load(g);
    tc::cp_async_commit();
  }
  for (int64_t g = 0; g < total && ok; ++g) {
    if (g + RING - 1 < total) issue_load(g + RING - 1);
    tc::cp_async_commit();
    tc::cp_async_wait<RING - 1>();
    const int cb = (int)(g & 1);
    const bool drain_now = dbuf && g % kGroup == 1 && g > kGroup;
    // operand buffer cb is free once the MMAs of slice g - 2 are done: one
    // thread waits and the barrier below releases the others (every thread
    // waits when TMEM is read next)
    if (g >= 2 && (t == 0 || drain_now) &&
        !tc::mbar_wait(tc::smem_addr(&sh->mbar[cb]), (uint32_t)(((g - 2) >> 1) & 1), kWaitCycles,
                       flags + kFlagNumeric))
      ok = false;
    // the MMAs of slice g - 2 are done, hence (dbuf) every MMA of the group
    // that ended with slice g - 2: add that set into the registers
    if (drain_now) {
      ok = __syncthreads_and(ok ? 1 : 0) != 0;
      if (!ok) break;
      tc::fence_after_sync();
      drain(set_base(g - 2));
      tc::fence_before_sync();
    }
    __syncthreads();
    {
      const float* rs = reinterpret_cast<const float*>(raw + (size_t)(g % RING) * raw_slot);
      uint8_t* st = conv + (size_t)cb * stage;
      convert(rs, c1p, c1, st, a_part);
      if (!sym) convert(rs + SL * c1p, c2p, c2, st + 2 * a_part, b_part);
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (!ok) break;
    const uint32_t sb = set_base(g);
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t a_hi = tc::smem_addr(conv + (size_t)cb * stage);
      const uint32_t a_lo = a_hi + a_part;
      const uint32_t b_hi = sym ? a_hi : a_hi + 2 * a_part;
      const uint32_t b_lo = sym ? a_lo : b_hi + b_part;
      const bool first = g % kGroup == 0;
      issue_slice<SL>(tmem + sb, slice_desc<SL>(a_hi), slice_desc<SL>(a_lo), slice_desc<SL>(b_hi),
                      slice_desc<SL>(b_lo), idesc0, first);
      if (mt == 2 && n1 > 0) {
        const uint32_t m1 = 128 * kRowBytes;  // row 128 of the A operand
        const uint32_t b1 = sym ? m1 : 0u;
        issue_slice<SL>(tmem + sb + (uint32_t)nmma, slice_desc<SL>(a_hi + m1), slice_desc<SL>(a_lo + m1),
                        slice_desc<SL>(b_hi + b1), slice_desc<SL>(b_lo + b1), idesc1, first);
      }
      tc::commit(tc::smem_addr(&sh->mbar[cb]));
    }
    last_commit = g;
    if (!dbuf && (g % kGroup == kGroup - 1 || g == total - 1)) {
      // one TMEM set: wait for this group's MMAs, then drain it
      if (!tc::mbar_wait(tc::smem_addr(&sh->mbar[cb]), (uint32_t)((g >> 1) & 1), kWaitCycles, flags + kFlagNumeric))
        ok = false;
      ok = __syncthreads_and(ok ? 1 : 0) != 0;
      if (!ok) break;
      tc::fence_after_sync();
      drain(0);
      tc::fence_before_sync();
    }
  }
  if (ok && total > 0 && dbuf) {
    const int64_t g = total - 1;
    if (!tc::mbar_wait(tc::smem_addr(&sh->mbar[g & 1]), (uint32_t)((g >> 1) & 1), kWaitCycles, flags + kFlagNumeric))
      ok = false;
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    if (ok) {
      tc::fence_after_sync();
      // groups whose drain point (first slice + kGroup + 1) was not reached
      const int64_t last_group = g / kGroup;
      if (last_group >= 1 && (last_group * kGroup + 1) >= total) drain(set_base((last_group - 1) * kGroup));
      drain(set_base(g));
    }
  }
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  if (ok) {
    float* out = partial + (int64_t)blockIdx.x * c1 * c2;
#pragma unroll
    for (int i = 0; i < kMaxChunks; ++i) {
      const int ch = half + 2 * i;
      if (ch < nchunks) {
        const bool d1 = ch * 16 >= nmma;
        const int row = (d1 ? 128 : 0) + 32 * lg + lane;
        const int j0 = d1 ? (sym ? 128 : 0) + ch * 16 - nmma : ch * 16;
        if (row < c1) {
#pragma unroll
          for (int e = 0; e < 16; ++e)
            if (j0 + e < c2) out[(int64_t)row * c2 + j0 + e] = acc[i][e];
        }
      }
    }
  }
  stream_finish(sh, tmem, 512, ok, last_commit, flags);
}

// Warp-specialised form of the symmetric Gram (A = B, c1 = c2 <= 192), with
// the slices, operand layout, MMAs, TMEM sets and 64-row drains of
// k_tc_gram_stream<32, R>:
//   warp 12 lane 0 (load) one TMA box per raw 32-row slice into a ring of
//                        `ring` slots (raw_full[s] completes when it lands),
//                        with an L2 prefetch of the slice 8 on (warp 13 idles)
//   warps 8-11 (split)   raw slot -> TF32 hi/lo operand stage (2 stages),
//                        releases the raw slot, publishes the stage
//   warp 14 lane 0 (MMA) D0 (and D1) MMAs of a slice into the TMEM set of
//                        its 64-row group; its commits release the stage and,
//                        after the group's last slice, hand the set over
//   warps 0-7 (drain)    TMEM set -> FP32 registers (rounded to nearest),
//                        release the set; the sums go to partial[b] at the end
// Unlike the block-synchronous form (two block barriers per slice) the
// stages overlap.  Timed per slice on one CTA (n = 1.14M, 144 columns): with
// cp.async loaders (two warps, 1,152 16-byte copies per slice) the loads
// took about 3,000 of the 3,400 cycles per slice; the split takes ~1,400
// and the 24 MMAs ~1,500, so the TMA box (one instruction per slice) took
// the call from 0.51 to 0.35 ms.  The number of MMAs per K step hardly
// matters (three, one or none: 0.515, 0.509, 0.491 ms before the TMA
// loads).  Every wait is bounded; a timeout sets the context's numeric flag
// to 2, which ends every other wait within 64 polls.
constexpr int kGwsSL = 32;
constexpr int kGwsGroup = kGroupRows / kGwsSL;  // slices per TMEM set fill
constexpr int kGwsDrainWarps = 8;
constexpr int kGwsSplitWarp = 8, kGwsLoadWarp = 12, kGwsMmaWarp = 14;
constexpr int kGwsThreads = 32 * 15;
constexpr int kGwsChunks = 6;      // 16-column chunks per drain thread: sets up to 192 columns
constexpr int kGwsMaxRing = 8;
constexpr int kGwsPrefetch = 8;    // slices prefetched into L2 ahead of the TMA ring

struct GwsShared {
  unsigned long long raw_full[kGwsMaxRing], raw_empty[kGwsMaxRing];
  unsigned long long conv_full[2], conv_empty[2], set_full[2], set_empty[2];
  uint32_t tmem_base;
};

__global__ void __launch_bounds__(kGwsThreads, 1) k_tc_gram_ws(const __grid_constant__ CUtensorMap tmap,
                                                              const float* __restrict__ A, int64_t lda, int c1,
                                                              int nmma, int ring, int64_t n, int64_t per,
                                                              float* __restrict__ partial, int* flags) {
  extern __shared__ __align__(1024) uint8_t stream_smem[];
  constexpr uint32_t kRowBytes = kGwsSL * 4;
  constexpr int kQ = kGwsSL / 4;
  const int mt = c1 > 128 ? 2 : 1;
  const uint32_t a_part = (uint32_t)(128 * mt) * kRowBytes;
  const uint32_t stage = 2 * a_part;
  const int c1p = (c1 + 3) & ~3;
  const uint32_t raw_slot = (uint32_t)(kGwsSL * c1p * 4);
  uint8_t* conv = stream_smem;
  uint8_t* raw = stream_smem + 2 * (size_t)stage;
  GwsShared* sh = reinterpret_cast<GwsShared*>(raw + (size_t)ring * raw_slot);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int n1 = mt == 2 ? nmma - 128 : 0;  // N of D1 (columns >= 128 only)
  const int set_cols = nmma + n1;
  const int nchunks = set_cols / 16;
  const int64_t nslices = (n + kGwsSL - 1) / kGwsSL;
  const int64_t s0 = (int64_t)blockIdx.x * per;
  const int64_t left = nslices - s0;
  const int64_t total = left <= 0 ? 0 : (left < per ? left : per);
  const int64_t ngroups = (total + kGwsGroup - 1) / kGwsGroup;

  if (t == 0) {
    for (int s = 0; s < ring; ++s) {
      tc::mbar_init(tc::smem_addr(&sh->raw_full[s]), 1);
      tc::mbar_init(tc::smem_addr(&sh->raw_empty[s]), 4);
    }
    for (int c = 0; c < 2; ++c) {
      tc::mbar_init(tc::smem_addr(&sh->conv_full[c]), 4);
      tc::mbar_init(tc::smem_addr(&sh->conv_empty[c]), 1);
      tc::mbar_init(tc::smem_addr(&sh->set_full[c]), 1);
      tc::mbar_init(tc::smem_addr(&sh->set_empty[c]), kGwsDrainWarps);
    }
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tc::smem_addr(&sh->tmem_base), 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sh->tmem_base;
  int* abortf = flags + kFlagNumeric;
  auto fail = [&]() { atomicExch(abortf, 2); };
  bool ok = true;

  if (warp == kGwsLoadWarp) {
    // one thread: a TMA box of 32 rows x c1p columns per slice (rows past n
    // and columns past c1 land as zeros), and an L2 prefetch of the slice
    // kGwsPrefetch slices on, so that the ring's loads wait on L2
    if (lane == 0) {
      for (int64_t g = 0; g < total && g < kGwsPrefetch; ++g)
        tc::tma_prefetch_2d(&tmap, 0, (int)((s0 + g) * kGwsSL));
      for (int64_t g = 0; g < total; ++g) {
        const int s = (int)(g % ring);
        if (g + kGwsPrefetch < total) tc::tma_prefetch_2d(&tmap, 0, (int)((s0 + g + kGwsPrefetch) * kGwsSL));
        if (g >= ring &&
            !tc::mbar_wait(tc::smem_addr(&sh->raw_empty[s]), (uint32_t)((g / ring - 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        const uint32_t mb = tc::smem_addr(&sh->raw_full[s]);
        tc::mbar_arrive_expect_tx(mb, raw_slot);
        tc::tma_load_2d(tc::smem_addr(raw + (size_t)s * raw_slot), &tmap, 0, (int)((s0 + g) * kGwsSL), mb);
      }
    }
    __syncwarp();
  } else if (warp >= kGwsSplitWarp && warp < kGwsLoadWarp) {
    const int ct = t - 32 * kGwsSplitWarp;  // 0..127
    for (int64_t g = 0; g < total; ++g) {
      const int s = (int)(g % ring), c = (int)(g & 1);
      if (!tc::mbar_wait(tc::smem_addr(&sh->raw_full[s]), (uint32_t)((g / ring) & 1), kWaitCycles, abortf) ||
          (g >= 2 &&
           !tc::mbar_wait(tc::smem_addr(&sh->conv_empty[c]), (uint32_t)(((g >> 1) - 1) & 1), kWaitCycles, abortf))) {
        if (lane == 0) fail();
        break;
      }
      const float* rs = reinterpret_cast<const float*>(raw + (size_t)s * raw_slot);
      uint8_t* hi = conv + (size_t)c * stage;
      // operand row j (a column of A), K group q (slice rows 4q .. 4q + 3)
      auto one = [&](int j, int q) {
        const float* col = rs + (4 * q) * c1p + j;
        const float4 x = make_float4(col[0], col[c1p], col[2 * c1p], col[3 * c1p]);
        float4 h, l;
        split4(x, h, l);
        const uint32_t off = tc::kmajor_off((uint32_t)j, (uint32_t)(4 * q), kGwsSL);
        *reinterpret_cast<float4*>(hi + off) = h;
        *reinterpret_cast<float4*>(hi + a_part + off) = l;
      };
      if (ct < c1) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) one(ct, q);
      }
      for (int e = ct; e < kQ * (c1 - 128); e += 128) one(128 + e / kQ, e % kQ);
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(tc::smem_addr(&sh->raw_empty[s]));
        tc::mbar_arrive(tc::smem_addr(&sh->conv_full[c]));
      }
    }
  } else if (warp == kGwsMmaWarp) {
    if (lane == 0) {
      const uint32_t idesc0 = tc::idesc_tf32(128, nmma);
      const uint32_t idesc1 = tc::idesc_tf32(128, n1 > 0 ? n1 : 16);
      int64_t last_commit = -1;
      for (int64_t g = 0; g < total; ++g) {
        const int c = (int)(g & 1);
        const int64_t gi = g / kGwsGroup;
        const int b = (int)(gi & 1);
        const bool first = g % kGwsGroup == 0;
        if (first && gi >= 2 &&
            !tc::mbar_wait(tc::smem_addr(&sh->set_empty[b]), (uint32_t)(((gi >> 1) - 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        if (!tc::mbar_wait(tc::smem_addr(&sh->conv_full[c]), (uint32_t)((g >> 1) & 1), kWaitCycles, abortf)) {
          fail();
          break;
        }
        tc::fence_after_sync();
        const uint32_t a_hi = tc::smem_addr(conv + (size_t)c * stage);
        const uint32_t a_lo = a_hi + a_part;
        const uint32_t d = tmem + (uint32_t)(b * 256);
        issue_slice<kGwsSL>(d, slice_desc<kGwsSL>(a_hi), slice_desc<kGwsSL>(a_lo), slice_desc<kGwsSL>(a_hi),
                            slice_desc<kGwsSL>(a_lo), idesc0, first);
        if (n1 > 0) {
          const uint32_t m1 = 128 * kRowBytes;  // operand row 128
          issue_slice<kGwsSL>(d + (uint32_t)nmma, slice_desc<kGwsSL>(a_hi + m1), slice_desc<kGwsSL>(a_lo + m1),
                              slice_desc<kGwsSL>(a_hi + m1), slice_desc<kGwsSL>(a_lo + m1), idesc1, first);
        }
        tc::commit(tc::smem_addr(&sh->conv_empty[c]));
        if (g % kGwsGroup == kGwsGroup - 1 || g == total - 1) tc::commit(tc::smem_addr(&sh->set_full[b]));
        last_commit = g;
      }
      // nothing may still write TMEM when it is released
      if (last_commit >= 0)
        tc::mbar_wait(tc::smem_addr(&sh->conv_empty[last_commit & 1]), (uint32_t)((last_commit >> 1) & 1),
                      kWaitCycles, flags + kFlagTimeoutGuard);
    }
    __syncwarp();
  } else if (warp < kGwsDrainWarps) {
    const int lg = warp & 3, half = warp >> 2;
    const uint32_t lane_addr = (uint32_t)(32 * lg) << 16;
    float acc[kGwsChunks][16];
#pragma unroll
    for (int i = 0; i < kGwsChunks; ++i)
#pragma unroll
      for (int e = 0; e < 16; ++e) acc[i][e] = 0.0f;
    for (int64_t gi = 0; gi < ngroups; ++gi) {
      const int b = (int)(gi & 1);
      if (!tc::mbar_wait(tc::smem_addr(&sh->set_full[b]), (uint32_t)((gi >> 1) & 1), kWaitCycles, abortf)) {
        if (lane == 0) fail();
        ok = false;
        break;
      }
      tc::fence_after_sync();
#pragma unroll
      for (int i = 0; i < kGwsChunks; ++i) {
        const int ch = half + 2 * i;
        if (ch < nchunks) {
          float v[16];
          tc::tmem_ld16(tmem + lane_addr + (uint32_t)(b * 256 + ch * 16), v);
#pragma unroll
          for (int e = 0; e < 16; ++e) acc[i][e] += v[e];
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_addr(&sh->set_empty[b]));
    }
    if (ok && *reinterpret_cast<volatile int*>(abortf) == 0) {
      float* out = partial + (int64_t)blockIdx.x * c1 * c1;
#pragma unroll
      for (int i = 0; i < kGwsChunks; ++i) {
        const int ch = half + 2 * i;
        if (ch < nchunks) {
          const bool d1 = ch * 16 >= nmma;
          const int row = (d1 ? 128 : 0) + 32 * lg + lane;
          const int j0 = d1 ? 128 + ch * 16 - nmma : ch * 16;
          if (row < c1) {
#pragma unroll
            for (int e = 0; e < 16; ++e)
              if (j0 + e < c1) out[(int64_t)row * c1 + j0 + e] = acc[i][e];
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

// G[i][j] = sum over CTAs of partial[b][i][j] in FP64, in CTA order; with
// sym, the lower triangle is the mirror of the upper one (so G is exactly
// symmetric; entries i >= 128, j < 128 are not computed by the CTAs).
__global__ void k_gram_reduce_stream(const float* __restrict__ partial, int64_t nb, int c1, int c2, int sym,
                                     double* __restrict__ G) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t cnt = (int64_t)c1 * c2;
  if (t >= cnt) return;
  int i = (int)(t / c2), j = (int)(t % c2);
  if (sym && i > j) {
    const int x = i;
    i = j;
    j = x;
  }
  const int64_t e = (int64_t)i * c2 + j;
  double s = 0.0;
  for (int64_t b = 0; b < nb; ++b) s += (double)partial[b * cnt + e];
  G[t] = s;
}

}  // namespace

bool tc_supported(int c2) { return c2 >= 1 && c2 <= 256; }

// Shared memory of the streaming kernels (0 when the shape does not fit).
static size_t gemm_stream_smem(int K, int nmma) {
  const size_t nsl = (size_t)(K + kSlice - 1) / kSlice;
  return 2 * nsl * nmma * kSliceRowBytes + (size_t)kGemmRing * kASlice + 4 * kASlice + sizeof(StreamShared);
}
static size_t gram_stream_smem(int c1, int c2, int nmma, bool sym, int sl, int ring) {
  const int mt = c1 > 128 ? 2 : 1;
  const size_t a_part = (size_t)(128 * mt) * sl * 4;
  const size_t b_part = sym ? 0 : (size_t)nmma * sl * 4;
  const size_t c1p = (c1 + 3) & ~3, c2p = sym ? 0 : (c2 + 3) & ~3;
  return 2 * (2 * a_part + 2 * b_part) + (size_t)ring * sl * (c1p + c2p) * 4 + sizeof(StreamShared);
}
static size_t gram_ws_smem(int c1, int ring) {
  const size_t a_part = (size_t)(128 * (c1 > 128 ? 2 : 1)) * kGwsSL * 4;
  return 4 * a_part + (size_t)ring * kGwsSL * ((c1 + 3) & ~3) * 4 + sizeof(GwsShared);
}
// Slice rows: 32 (ring of 5) when that fits, else 16 (ring of 6); 0: neither fits.
static int gram_slice_rows(lne_ctx* ctx, int c1, int c2, int nmma, bool sym) {
  if (gram_stream_smem(c1, c2, nmma, sym, 32, 5) <= ctx->smem_optin) return 32;
  if (gram_stream_smem(c1, c2, nmma, sym, 16, kGramRing) <= ctx->smem_optin) return 16;
  return 0;
}
static bool aligned16(const void* p, int64_t ld) {
  return (reinterpret_cast<uintptr_t>(p) & 15) == 0 && (ld & 3) == 0;
}

// cuTensorMapEncodeTiled, from the driver (no link against libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// Tensor map of a row-major FP32 matrix (rows x cols, ld elements between
// rows) read in 16-column x 128-row boxes with the 64-byte swizzle; columns
// and rows past the matrix read as zeros.
static bool tmap_rows16x128(CUtensorMap* m, const float* base, int64_t rows, int cols, int64_t ld) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || rows < 1 || cols < 1 || rows > 0x7fffffffLL) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)kSlice, 128};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of a row-major FP32 matrix (rows x cols, ld elements between
// rows) read in boxes of box_rows full rows of box_cols columns (cols rounded
// up to 4), without swizzle; what lies past the matrix reads as zeros.
static bool tmap_row_slices(CUtensorMap* m, const float* base, int64_t rows, int cols, int64_t ld, int box_cols,
                            int box_rows) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || rows < 1 || cols < 1 || rows > 0x7fffffffLL || box_cols > 256 || (box_cols & 3)) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int tc_gemm_tall(lne_ctx* ctx, const float* In, int64_t ldi, int k, const float* W, int c2, int64_t n, float* Out,
                 int64_t ldo, Copy16 OutB) {
  if (n <= 0) return LNE_OK;
  const int nmma = std::max(16, (int)((std::max<int64_t>(c2, ldo) + 15) / 16 * 16));
  if (nmma > 256) {
    set_error("tc_gemm_tall: more than 256 output columns");
    return LNE_ERR_UNSUPPORTED;
  }
  // warp-specialised kernel: the deepest raw ring (up to kWsMaxRing, at
  // least 2) that fits beside W and the two operand stages
  const size_t ws_fixed = gemm_stream_smem(k, nmma) - (size_t)kGemmRing * kASlice - sizeof(StreamShared) +
                          sizeof(WsShared);
  const int ws_ring = ctx->smem_optin > ws_fixed
                          ? (int)std::min<size_t>(kWsMaxRing, (ctx->smem_optin - ws_fixed) / kASlice)
                          : 0;
  if (aligned16(In, ldi) && k >= 1 && nmma <= kWsMaxCols && ws_ring >= 2) {
    const int64_t ntiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, ctx->num_sms);
    const size_t wsmem = ws_fixed + (size_t)ws_ring * kASlice;
    // a CTA allocates all 512 TMEM columns: one CTA per SM, which the
    // shared memory request also ensures
    const size_t lsmem = std::max(wsmem, ctx->smem_optin / 2 + 1);
    CUtensorMap tmap;
    memset(&tmap, 0, sizeof(tmap));
    if (tmap_rows16x128(&tmap, In, n, k, ldi)) {
      cudaFuncSetAttribute(k_tc_gemm_ws<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);
      k_tc_gemm_ws<true><<<grid, kWsThreads, lsmem, ctx->stream>>>(tmap, In, ldi, k, W, c2, nmma, ws_ring, n, Out, ldo,
                                                                  OutB, ctx->d_flags);
    } else {
      cudaFuncSetAttribute(k_tc_gemm_ws<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);
      k_tc_gemm_ws<false><<<grid, kWsThreads, lsmem, ctx->stream>>>(tmap, In, ldi, k, W, c2, nmma, ws_ring, n, Out,
                                                                   ldo, OutB, ctx->d_flags);
    }
    LNE_CUDA_TRY(cudaGetLastError());
    return LNE_OK;
  }
  const size_t ssmem = gemm_stream_smem(k, nmma);
  if (aligned16(In, ldi) && ssmem <= ctx->smem_optin && k >= 1) {
    const int64_t ntiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, ctx->num_sms);
    // at most two CTAs per SM: each holds 256 TMEM columns
    const size_t lsmem = std::max(ssmem, std::min(ctx->smem_optin, (size_t)80 * 1024));
    cudaFuncSetAttribute(k_tc_gemm_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);
    k_tc_gemm_stream<<<grid, kSThreads, lsmem, ctx->stream>>>(In, ldi, k, W, c2, nmma, n, Out, ldo, OutB,
                                                              ctx->d_flags);
    LNE_CUDA_TRY(cudaGetLastError());
    return LNE_OK;
  }
  cudaFuncSetAttribute(k_tc_gemm_tall, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
  k_tc_gemm_tall<<<(unsigned)((n + 127) / 128), kTcThreads, kSmemBytes, ctx->stream>>>(In, ldi, k, W, c2, nmma, n, Out,
                                                                                       ldo, OutB, ctx->d_flags);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

bool tc_gram_stream_supported(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb,
                               int c2) {
  if (c1 < 1 || c2 < 1 || c1 > 256 || c2 > 256) return false;
  const int nmma = std::max(16, (c2 + 15) / 16 * 16);
  const bool sym = A == B && lda == ldb && c1 == c2;
  const int set_cols = c1 > 128 ? nmma + (sym ? nmma - 128 : nmma) : nmma;
  return aligned16(A, lda) && aligned16(B, ldb) && set_cols <= 32 * kMaxChunks &&
         gram_slice_rows(ctx, c1, c2, nmma, sym) > 0;
}

int tc_gram_stream(lne_ctx* ctx, const float* A, int64_t lda, int c1, const float* B, int64_t ldb, int c2, int64_t n,
                   double* G, float* partial, int64_t max_blocks) {
  if (!tc_gram_stream_supported(ctx, A, lda, c1, B, ldb, c2)) {
    set_error("tc_gram_stream: shape or alignment not supported");
    return LNE_ERR_UNSUPPORTED;
  }
  if (n <= 0) {
    LNE_CUDA_TRY(cudaMemsetAsync(G, 0, sizeof(double) * c1 * c2, ctx->stream));
    return LNE_OK;
  }
  const int nmma = std::max(16, (c2 + 15) / 16 * 16);
  const bool sym = A == B && lda == ldb && c1 == c2;
  if (sym) {
    // warp-specialised form: two TMEM sets of at most 2 x kGwsChunks chunks
    const int set_cols = nmma + (c1 > 128 ? nmma - 128 : 0);
    const size_t slot = (size_t)kGwsSL * ((c1 + 3) & ~3) * 4;
    const size_t fixed = gram_ws_smem(c1, 0);
    const int ring = ctx->smem_optin > fixed ? (int)std::min<size_t>(kGwsMaxRing, (ctx->smem_optin - fixed) / slot)
                                             : 0;
    CUtensorMap tmap;
    memset(&tmap, 0, sizeof(tmap));
    if (set_cols <= 32 * kGwsChunks && ring >= 2 &&
        tmap_row_slices(&tmap, A, n, c1, lda, (c1 + 3) & ~3, kGwsSL)) {
      const int64_t nslices = (n + kGwsSL - 1) / kGwsSL;
      const int64_t want =
          std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(nslices, ctx->num_sms), max_blocks));
      const int64_t per = (nslices + want - 1) / want;
      const int64_t nb = (nslices + per - 1) / per;  // <= want
      float* own = nullptr;
      if (!partial) {
        int rc = dalloc(ctx, (void**)&own, sizeof(float) * nb * c1 * c2, "gram partials");
        if (rc) return rc;
        partial = own;
      }
      // the CTA allocates all 512 TMEM columns: one CTA per SM
      const size_t lsmem = std::max(gram_ws_smem(c1, ring), ctx->smem_optin / 2 + 1);
      cudaFuncSetAttribute(k_tc_gram_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);
      k_tc_gram_ws<<<(unsigned)nb, kGwsThreads, lsmem, ctx->stream>>>(tmap, A, lda, c1, nmma, ring, n, per, partial,
                                                                      ctx->d_flags);
      const int64_t cnt = (int64_t)c1 * c2;
      k_gram_reduce_stream<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(partial, nb, c1, c2, 1, G);
      if (own) dfree(ctx, own);
      LNE_CUDA_TRY(cudaGetLastError());
      return LNE_OK;
    }
  }
  const int sl = gram_slice_rows(ctx, c1, c2, nmma, sym);
  const int ring = sl == 32 ? 5 : kGramRing;
  const size_t ssmem = gram_stream_smem(c1, c2, nmma, sym, sl, ring);
  const int64_t nslices = (n + sl - 1) / sl;
  const int64_t want = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(nslices, ctx->num_sms), max_blocks));
  const int64_t per = (nslices + want - 1) / want;
  const int64_t nb = (nslices + per - 1) / per;  // <= want
  float* own = nullptr;
  if (!partial) {
    int rc = dalloc(ctx, (void**)&own, sizeof(float) * nb * c1 * c2, "gram partials");
    if (rc) return rc;
    partial = own;
  }
  // the CTA allocates all 512 TMEM columns: one CTA per SM
  const size_t lsmem = std::max(ssmem, std::min(ctx->smem_optin, (size_t)120 * 1024));
  auto kern = sl == 32 ? k_tc_gram_stream<32, 5> : k_tc_gram_stream<16, kGramRing>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsmem);
  kern<<<(unsigned)nb, kSThreads, lsmem, ctx->stream>>>(A, lda, c1, B, ldb, c2, nmma, n, sym ? 1 : 0, per, partial,
                                                        ctx->d_flags);
  const int64_t cnt = (int64_t)c1 * c2;
  k_gram_reduce_stream<<<(unsigned)((cnt + 255) / 256), 256, 0, ctx->stream>>>(partial, nb, c1, c2, sym ? 1 : 0, G);
  if (own) dfree(ctx, own);
  LNE_CUDA_TRY(cudaGetLastError());
  return LNE_OK;
}

}  // namespace lne
