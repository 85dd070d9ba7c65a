// Row-parallel SpMM core: Y[i,:] = epi(i, sum_j v_ij * X[c_ij, :]).
//
// Work is split into items so that no warp walks more than kChunkNnz
// nonzeros: a row with at most kChunkNnz entries is one item; a longer row
// is cut into chunks whose partial sums go to a scratch buffer and are added
// in chunk order by a second kernel.  Every output is therefore a sum in a
// fixed order: results are bitwise reproducible run to run.
//
// Within an item the warp is split into P = 32/G groups of G lanes; lane gl
// of a group owns the 16-byte column vectors gl, gl+G, ... of the row, and
// group g takes the nonzeros t with t % P == g.  Column ids (and values) are
// loaded up to 32 at a time, one per lane, and broadcast with shuffles; the
// gathers of several nonzeros are issued before their FMAs so that every
// lane keeps several 16-byte loads in flight (SpmmTune).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "dense_common.cuh"
#include "lne_internal.h"

namespace lne {

static constexpr unsigned kFull = 0xffffffffu;

// Access to a sparse operator's rows.
struct CsrRows {  // explicit CSR: int64 row_ptr, int32 col, float val
  const int64_t* __restrict__ row_ptr;
  const int32_t* __restrict__ col;
  const float* __restrict__ val;
  __device__ __forceinline__ int64_t begin(int64_t r) const { return __ldg(row_ptr + r); }
  __device__ __forceinline__ int64_t end(int64_t r) const { return __ldg(row_ptr + r + 1); }
  __device__ __forceinline__ uint32_t c(int64_t j) const { return (uint32_t)__ldg(col + j); }
  __device__ __forceinline__ float v(int64_t j) const { return __ldg(val + j); }
  static constexpr bool kHasVal = true;
};

// The entries of a CSR row whose columns fall in one column panel.
struct PanelRows {
  const int64_t* __restrict__ row_ptr;
  const int32_t* __restrict__ seg;  // n x (np1) relative panel starts
  const int32_t* __restrict__ col;
  const float* __restrict__ val;
  int np1;                          // panels + 1
  int p;                            // this panel
  __device__ __forceinline__ int64_t begin(int64_t r) const {
    return __ldg(row_ptr + r) + __ldg(seg + r * np1 + p);
  }
  __device__ __forceinline__ int64_t end(int64_t r) const {
    return __ldg(row_ptr + r) + __ldg(seg + r * np1 + p + 1);
  }
  __device__ __forceinline__ uint32_t c(int64_t j) const { return (uint32_t)__ldg(col + j); }
  __device__ __forceinline__ float v(int64_t j) const { return __ldg(val + j); }
  static constexpr bool kHasVal = true;
};

struct GraphRows {  // graph adjacency: {offset, degree} per vertex, unit values
  const Vertex* __restrict__ vdata;
  const uint32_t* __restrict__ nbrs;
  __device__ __forceinline__ int64_t begin(int64_t r) const { return (int64_t)__ldg(&vdata[r].off); }
  __device__ __forceinline__ int64_t end(int64_t r) const {
    return (int64_t)__ldg(&vdata[r].off) + (int64_t)__ldg(&vdata[r].deg);
  }
  __device__ __forceinline__ uint32_t c(int64_t j) const { return __ldg(nbrs + j); }
  __device__ __forceinline__ float v(int64_t) const { return 1.0f; }
  static constexpr bool kHasVal = false;
};

// Gather depth of the raw-staged path (FP8 operands, 9-lane groups and
// 128-element 16-bit rows): each lane issues the gathers of kU nonzeros
// before their FMAs, kept as raw 16-byte words (4 registers each).  Column
// ids are loaded in batches of kBatch <= 32, a multiple of the P kU
// nonzeros a warp takes per step, so that no step of a batch runs
// part-empty, and a step whose nonzeros are all in the batch loads without
// predicates.  Measured at n = 1.14M, nnz = 351M (`B = A Q`, the sketch
// product, the 19 SpMMs of the propagation), unpredicated full steps
// included: a 144-element FP16 row at kU = 2 (batch 30) 11.1 ms against
// 11.6 at 3 and 12.8 at 4; 144-element FP8 rows at kU = 5 (batch 30) 8.0
// against 8.4 at 4 and 9.2 at 6; 128-element 16-bit rows on the graph
// (the propagation) at kU = 5 (batch 30) 13.0 against 13.2 at 4 and 13.3
// at 6.  Deeper staging spills (64 registers a thread at 4 CTAs of 256 per
// SM); compiled for 3 CTAs per SM it lost more warps than it gained in
// flight.  Other operands are widened at the load and staged kUnroll deep.
template <typename XT, int G, int VPL>
struct SpmmTune {
  static constexpr int E = Vec16<XT>::E;
  static constexpr int P = 32 / G;
  static constexpr bool kRaw = E == 16 || (G & (G - 1)) != 0 || (E == 8 && G == 16 && VPL == 1);
  static constexpr int kWant = (G == 9 && VPL == 2)                               ? 2
                               : VPL == 1 && (G == 9 || (G == 16 && E == 8)) ? 5
                                                                                  : (VPL >= 4 ? 1 : 4 / VPL);
  static constexpr int kU = kWant * P <= 32 ? kWant : 32 / P;
  static constexpr int kBatch = (32 / (P * kU)) * (P * kU);
  static_assert(kBatch >= 1 && kBatch <= 32, "a batch of column ids is one per lane");
};

template <typename XT, int VPL>
struct Acc {
  static constexpr int E = Vec16<XT>::E;
  float a[VPL][E];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int k = 0; k < VPL; ++k)
#pragma unroll
      for (int e = 0; e < E; ++e) a[k][e] = 0.f;
  }
};

// Accumulate nonzeros [j0, j1) of the operator into acc (per group), then
// reduce across the P groups so that the lanes of group 0 hold the sums.
template <typename XT, int G, int VPL, class Rows>
__device__ __forceinline__ void spmm_accumulate(const Rows& R, int64_t j0, int64_t j1, const XT* __restrict__ X,
                                                int64_t ldx, int C, Acc<XT, VPL>& acc) {
  constexpr int P = 32 / G;
  constexpr int E = Vec16<XT>::E;
  const int lane = threadIdx.x & 31;
  const int grp = lane / G, gl = lane % G;
  if constexpr (SpmmTune<XT, G, VPL>::kRaw) {
    // FP8 vectors, a group of 9 lanes or 16 lanes of 16-bit vectors: the
    // gathers of kU nonzeros are staged as raw 16-byte words, widened at
    // the FMAs
    constexpr int kU = SpmmTune<XT, G, VPL>::kU;
    // G = 9 (a 144-element row: 9 FP8 vectors, or 18 BF16 / FP16 vectors
    // at two per lane): three groups of 9 lanes, lanes 27..31 idle
    const bool in_grp = grp < P;
    constexpr int kB = SpmmTune<XT, G, VPL>::kBatch;
    // a step whose P kU nonzeros are all in the batch, on a slab that fills
    // the lane layout, loads without predicates: lanes past the groups
    // (27..31) read rows of valid columns too and their sums are not used
    const bool full_cols = C == G * VPL;
    for (int64_t base = j0; base < j1; base += kB) {
      const int cnt = (int)((j1 - base) < kB ? (j1 - base) : kB);
      const uint32_t c = lane < cnt ? R.c(base + lane) : 0u;
      const float v = Rows::kHasVal ? (lane < cnt ? R.v(base + lane) : 0.f) : 1.f;
      auto step = [&](int t0, auto checked) {
        constexpr bool kChecked = decltype(checked)::value;
        uint4 raw[kU][VPL];
        float vv[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int t = t0 + u * P + grp;
          const uint32_t cc = __shfl_sync(kFull, c, t & 31);
          vv[u] = Rows::kHasVal ? __shfl_sync(kFull, v, t & 31) : 1.f;
          const XT* xr = X + (int64_t)cc * ldx;
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            const int ch = gl + G * k;
            if constexpr (kChecked)
              raw[u][k] = (in_grp && t < cnt && ch < C) ? __ldg(reinterpret_cast<const uint4*>(xr + ch * E))
                                                         : make_uint4(0, 0, 0, 0);
            else
              raw[u][k] = __ldg(reinterpret_cast<const uint4*>(xr + ch * E));
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u)
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            float x[E];
            Vec16<XT>::unpack(raw[u][k], x);
            // paired FP32 FMAs: each element rounded as by fmaf
#pragma unroll
            for (int e = 0; e < E; e += 2) {
              const float2 r = __ffma2_rn(make_float2(vv[u], vv[u]), make_float2(x[e], x[e + 1]),
                                          make_float2(acc.a[k][e], acc.a[k][e + 1]));
              acc.a[k][e] = r.x;
              acc.a[k][e + 1] = r.y;
            }
          }
      };
      for (int t0 = 0; t0 < cnt; t0 += P * kU) {
        if (full_cols && t0 + P * kU <= cnt)
          step(t0, std::false_type{});
        else
          step(t0, std::true_type{});
      }
    }
    if constexpr ((G & (G - 1)) == 0) {
#pragma unroll
      for (int o = G; o < 32; o <<= 1)
#pragma unroll
        for (int k = 0; k < VPL; ++k)
#pragma unroll
          for (int e = 0; e < E; ++e) acc.a[k][e] += __shfl_xor_sync(kFull, acc.a[k][e], o);
    } else {
      static_assert(P == 3, "non-power-of-two groups: three groups per warp");
#pragma unroll
      for (int k = 0; k < VPL; ++k)
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const float g1 = __shfl_down_sync(kFull, acc.a[k][e], G);
          const float g2 = __shfl_down_sync(kFull, acc.a[k][e], 2 * G);
          acc.a[k][e] = (acc.a[k][e] + g1) + g2;
        }
    }
  } else {
    // nonzeros whose gathers are in flight per lane: about 16 staged floats
    constexpr int kStaged = 16 / (VPL * E);
    constexpr int kUnroll = kStaged < 1 ? 1 : (kStaged > 4 ? 4 : kStaged);
    for (int64_t base = j0; base < j1; base += 32) {
      const int cnt = (int)((j1 - base) < 32 ? (j1 - base) : 32);
      const uint32_t c = lane < cnt ? R.c(base + lane) : 0u;
      const float v = Rows::kHasVal ? (lane < cnt ? R.v(base + lane) : 0.f) : 1.f;
      for (int t0 = 0; t0 < cnt; t0 += P * kUnroll) {
        uint32_t cc[kUnroll];
        float vv[kUnroll];
        float x[kUnroll][VPL][E];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          const int t = t0 + u * P + grp;
          cc[u] = __shfl_sync(kFull, c, t & 31);
          vv[u] = Rows::kHasVal ? __shfl_sync(kFull, v, t & 31) : 1.f;
          const XT* xr = X + (int64_t)cc[u] * ldx;
#pragma unroll
          for (int k = 0; k < VPL; ++k) {
            const int ch = gl + G * k;
            if (t < cnt && ch < C) {
              Vec16<XT>::load(xr + ch * E, x[u][k]);
            } else {
#pragma unroll
              for (int e = 0; e < E; ++e) x[u][k][e] = 0.f;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
          for (int k = 0; k < VPL; ++k)
#pragma unroll
            for (int e = 0; e < E; ++e) acc.a[k][e] = fmaf(vv[u], x[u][k][e], acc.a[k][e]);
      }
    }
#pragma unroll
    for (int o = G; o < 32; o <<= 1)
#pragma unroll
      for (int k = 0; k < VPL; ++k)
#pragma unroll
        for (int e = 0; e < E; ++e) acc.a[k][e] += __shfl_xor_sync(kFull, acc.a[k][e], o);
  }
}

// Main kernel: short rows call the epilogue directly; chunks of long rows
// store partial sums (FP32, ld = ldp) for k_spmm_finish.
template <typename XT, int G, int VPL, class Rows, class Epi>
__global__ void __launch_bounds__(256, 4) k_spmm(Rows R, SpmmPlan plan, const XT* __restrict__ X, int64_t ldx, int C,
                                              float* __restrict__ partial, int64_t ldp, int e_base, Epi epi) {
  constexpr int E = Vec16<XT>::E;
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t items = plan.n_short + plan.n_chunks;
  for (int64_t it = warp; it < items; it += nwarps) {
    Acc<XT, VPL> acc;
    acc.zero();
    if (it < plan.n_short) {
      const uint32_t r = __ldg(plan.short_rows + it);
      spmm_accumulate<XT, G, VPL>(R, R.begin(r), R.end(r), X, ldx, C, acc);
      if (lane < G) {
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          const int ch = gl + G * k;
          if (ch < C) epi(r, e_base + ch * E, acc.a[k]);
        }
      }
    } else {
      const int64_t ci = it - plan.n_short;
      const int64_t b = __ldg(plan.chunk_begin + ci);
      const uint32_t r = __ldg(plan.chunk_row + ci);
      int64_t e = R.end(r);
      const int64_t lim = b + kChunkNnz;
      e = e < lim ? e : lim;
      spmm_accumulate<XT, G, VPL>(R, b, e, X, ldx, C, acc);
      if (lane < G) {
#pragma unroll
        for (int k = 0; k < VPL; ++k) {
          const int ch = gl + G * k;
          if (ch < C) {
            float* p = partial + ci * ldp + ch * E;
#pragma unroll
            for (int q = 0; q < E; q += 4)
              *reinterpret_cast<float4*>(p + q) = make_float4(acc.a[k][q], acc.a[k][q + 1], acc.a[k][q + 2],
                                                             acc.a[k][q + 3]);
          }
        }
      }
    }
  }
}

// Long rows: add the chunk partials in order and apply the epilogue.
// One warp per long row; lanes cover the row in 16-byte (4-float) vectors.
template <class Epi>
__global__ void k_spmm_finish(SpmmPlan plan, const float* __restrict__ partial, int64_t ldp, int cols, int e_base,
                              Epi epi) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp; w < plan.n_long; w += nwarps) {
    const uint32_t r = plan.long_rows[w];
    const int64_t c0 = plan.long_first[w], c1 = plan.long_first[w + 1];
    for (int q = lane * 4; q < cols; q += 128) {
      float s[4] = {0.f, 0.f, 0.f, 0.f};
      for (int64_t ci = c0; ci < c1; ++ci) {
        const float4 v = *reinterpret_cast<const float4*>(partial + ci * ldp + q);
        s[0] += v.x; s[1] += v.y; s[2] += v.z; s[3] += v.w;
      }
      epi(r, e_base + q, s);
    }
  }
}

}  // namespace lne
