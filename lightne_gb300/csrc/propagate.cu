// Spectral propagation: the Bessel-weighted Chebyshev filter on
// M = I - D~^-1 A~ - mu I (A~ = A + I, D~ = D + I), then (A + I) a.
//
// Reference: spectral_propagation::chebyshev_expansion
// (LightNE/SpectralPropagation.h:45-221):
//   Lx0 = a;  tmp = M a;  Lx1 = 0.5 M tmp - a;  conv = I0(s) Lx0 - 2 I1(s) Lx1
//   for k = 2 .. order-1:  tmp = M Lx1;  Lx2 = M tmp - Lx0 - 2 Lx1;
//                          conv += (k odd ? -2 : 2) I_k(s) Lx2;  rotate
//   a -= conv;  y = (A + I) a
// M is applied as an implicit operator: row i has the value
// (float)(1 - mu - 1/d~_i) on the diagonal and (float)(-1/d~_i) on each
// neighbour (the reference stores these floats in a CSR, :59-75), so
// (M x)_i = m_i x_i + o_i * sum_{j in N(i)} x_j with the neighbour sum
// gathered by the SpMM core.  Every half-step is one kernel whose epilogue
// applies the recursion's axpbys while the row is in registers.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <cmath>
#include <string>
#include <type_traits>
#include <vector>

#include "dense.h"
#include "dense_common.cuh"
#include "lne_internal.h"
#include "spmm_core.cuh"
#include "spmm_dispatch.cuh"

namespace lne {

// Modified Bessel function of the first kind I_k(x) by its power series
// sum_m (x/2)^(2m+k) / (m! (m+k)!), summed in long double until the terms
// vanish (x = 0.5 in LightNE; the series converges for every x).
double bessel_i(int k, double x) {
  long double h = (long double)x / 2.0L, term = 1.0L;
  for (int i = 1; i <= k; ++i) term *= h / (long double)i;
  long double sum = term;
  for (int m = 1; m < 500; ++m) {
    term *= h * h / ((long double)m * (long double)(m + k));
    sum += term;
    if (term < sum * 1e-21L) break;
  }
  return (double)sum;
}

void chebyshev_coeffs(int order, double s, std::vector<float>& c) {
  // the reference evaluates iv(k, s) with s a float and narrows each axpy
  // coefficient to float (SpectralPropagation.h:129-197)
  const double sf = (double)(float)s;
  c.assign(order > 2 ? order : 2, 0.0f);
  c[0] = (float)bessel_i(0, sf);
  c[1] = (float)(-2.0 * bessel_i(1, sf));
  for (int k = 2; k < order; ++k) c[k] = (float)(((k & 1) ? -2.0 : 2.0) * bessel_i(k, sf));
}

namespace {

// Type of the 16-bit shadow copies of the propagation vectors that the
// SpMM gathers: the operand type itself in the 16-bit forms (the FP32 form
// keeps no shadows; its shadow pointers stay null).
template <typename XT>
struct ShadowOf {
  using type = __nv_bfloat16;
};
template <>
struct ShadowOf<__half> {
  using type = __half;
};

// Per-row operator data: x = diagonal m_i, y = off-diagonal o_i (the floats
// the reference stores), z = d~_i = deg + 1, w = 1 / d~_i.
__global__ void k_op_coef(const Vertex* __restrict__ vd, int64_t n, float mu, float4* __restrict__ coef) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float dt = (float)(vd[i].deg + 1u);
  const double inv = 1.0 / (double)dt;
  coef[i] = make_float4((float)(1.0 - (double)mu - inv), (float)(-inv), dt, (float)inv);
}

// Loads N elements (N a multiple of 4, e0 a multiple of 4) of row r of a
// dense operand as floats: 16-byte loads for FP32, 8-byte loads for BF16
// and FP16 (so an e0 that is 4 mod 8 stays aligned).
template <typename T, int N>
__device__ __forceinline__ void load_row(const T* __restrict__ X, int64_t ld, int64_t r, int e0, float (&o)[N]) {
  const T* p = X + r * ld + e0;
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(p + i));
      o[i] = v.x; o[i + 1] = v.y; o[i + 2] = v.z; o[i + 3] = v.w;
    }
  } else if constexpr (std::is_same<T, __half>::value) {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(p + i));
      const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
      const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
      o[i] = a.x; o[i + 1] = a.y; o[i + 2] = b.x; o[i + 3] = b.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(p + i));
      o[i] = __uint_as_float(v.x << 16); o[i + 1] = __uint_as_float(v.x & 0xffff0000u);
      o[i + 2] = __uint_as_float(v.y << 16); o[i + 3] = __uint_as_float(v.y & 0xffff0000u);
    }
  }
}
template <int N>
__device__ __forceinline__ void load_f32(const float* __restrict__ X, int64_t ld, int64_t r, int e0, float (&o)[N]) {
  const float* p = X + r * ld + e0;
#pragma unroll
  for (int i = 0; i < N; i += 4) {
    const float4 v = *reinterpret_cast<const float4*>(p + i);
    o[i] = v.x; o[i + 1] = v.y; o[i + 2] = v.z; o[i + 3] = v.w;
  }
}
template <int N>
__device__ __forceinline__ void store_f32(float* __restrict__ X, int64_t ld, int64_t r, int e0, const float (&o)[N]) {
  float* p = X + r * ld + e0;
#pragma unroll
  for (int i = 0; i < N; i += 4) *reinterpret_cast<float4*>(p + i) = make_float4(o[i], o[i + 1], o[i + 2], o[i + 3]);
}
template <typename HT, int N>
__device__ __forceinline__ void store_16(HT* __restrict__ X, int64_t ld, int64_t r, int e0, const float (&o)[N]) {
  HT* p = X + r * ld + e0;
#pragma unroll
  for (int i = 0; i < N; i += 2) *reinterpret_cast<uint32_t*>(p + i) = pack2_16<HT>(o[i], o[i + 1]);
}

// tmp = M x: out = m_i x_i + o_i acc (operand x of type XT); FP32 and/or
// 16-bit outputs.
template <typename XT>
struct EpiApplyM {
  using HT = typename ShadowOf<XT>::type;
  const float4* __restrict__ coef;
  const XT* __restrict__ X;  // the operand (diagonal term)
  int64_t ld;
  float* __restrict__ out_f;
  HT* __restrict__ out_b;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&a)[N]) const {
    const float4 c = __ldg(coef + r);
    float x[N], y[N];
    load_row<XT, N>(X, ld, r, e0, x);
#pragma unroll
    for (int i = 0; i < N; ++i) y[i] = fmaf(c.x, x[i], c.y * a[i]);
    if (out_f) store_f32<N>(out_f, ld, r, e0, y);
    if (out_b) store_16<HT, N>(out_b, ld, r, e0, y);
  }
};

// Final vector of a filter: fin = base - (scale_dt ? d~_i : 1) * conv.
template <typename HT>
struct FinalOut {
  const float* __restrict__ base;  // null: not the final step
  bool scale_dt;
  float* __restrict__ out;
  HT* __restrict__ outb;
  template <int N>
  __device__ __forceinline__ void apply(int64_t r, int e0, int64_t ld, const float4 c, const float (&cv)[N]) const {
    float b[N], f[N];
    load_f32<N>(base, ld, r, e0, b);
    const float sc = scale_dt ? c.z : 1.0f;
#pragma unroll
    for (int i = 0; i < N; ++i) f[i] = fmaf(-sc, cv[i], b[i]);
    store_f32<N>(out, ld, r, e0, f);
    if (outb) store_16<HT, N>(outb, ld, r, e0, f);
  }
};

// First order: Lx1 = 0.5 M tmp - x;  conv = c0 x + c1 Lx1 (conv may be null:
// the tangent pass keeps no sum);  or the final vector when order <= 2.
template <typename XT>
struct EpiFirst {
  using HT = typename ShadowOf<XT>::type;
  const float4* __restrict__ coef;
  const XT* __restrict__ T;        // tmp (operand)
  const float* __restrict__ A;     // x (FP32)
  float* __restrict__ L1;          // Lx1 FP32
  HT* __restrict__ L1b;            // Lx1 16-bit copy (16-bit forms) or null
  float* __restrict__ conv;
  FinalOut<HT> fin;
  int64_t ld;
  float c0, c1;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    const float4 c = __ldg(coef + r);
    float t[N], a[N], l1[N], cv[N];
    load_row<XT, N>(T, ld, r, e0, t);
    load_f32<N>(A, ld, r, e0, a);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const float mt = fmaf(c.x, t[i], c.y * acc[i]);
      l1[i] = fmaf(0.5f, mt, -a[i]);
      cv[i] = fmaf(c1, l1[i], c0 * a[i]);
    }
    store_f32<N>(L1, ld, r, e0, l1);
    if (L1b) store_16<HT, N>(L1b, ld, r, e0, l1);
    if (fin.base)
      fin.template apply<N>(r, e0, ld, c, cv);
    else if (conv)
      store_f32<N>(conv, ld, r, e0, cv);
  }
};

// Order k >= 2: Lx2 = M tmp - Lx0 - 2 Lx1 [- 2 extra];  conv += ck Lx2 (conv
// may be null);  or the final vector on the last order.  L0 == null means a
// zero Lx0; `extra` (FP32, may be null) is the tangent pass's M T_k term.
// The sum is read and written every second order: `skip` leaves conv alone
// and the next order adds ck_prev Lx1 (the skipped order's vector) as well.
template <typename XT>
struct EpiStep {
  using HT = typename ShadowOf<XT>::type;
  const float4* __restrict__ coef;
  const XT* __restrict__ T;
  const float* __restrict__ L0;
  const float* __restrict__ L1;
  const float* __restrict__ extra;
  float* __restrict__ L2;
  HT* __restrict__ L2b;
  float* __restrict__ conv;
  FinalOut<HT> fin;
  int64_t ld;
  float ck;
  float ck_prev = 0.0f;
  bool skip = false;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    const float4 c = __ldg(coef + r);
    float t[N], l0[N], l1[N], l2[N], cv[N];
    load_row<XT, N>(T, ld, r, e0, t);
    if (L0) {
      load_f32<N>(L0, ld, r, e0, l0);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) l0[i] = 0.0f;
    }
    load_f32<N>(L1, ld, r, e0, l1);
    if (conv && !skip) {
      load_f32<N>(conv, ld, r, e0, cv);
#pragma unroll
      for (int i = 0; i < N; ++i) cv[i] = fmaf(ck_prev, l1[i], cv[i]);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) cv[i] = 0.0f;
    }
    float ex[N];
    if (extra) {
      load_f32<N>(extra, ld, r, e0, ex);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) ex[i] = 0.0f;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const float mt = fmaf(c.x, t[i], c.y * acc[i]);
      l2[i] = fmaf(-2.0f, ex[i], fmaf(-2.0f, l1[i], mt - l0[i]));
      cv[i] = fmaf(ck, l2[i], cv[i]);
    }
    if (fin.base) {
      fin.template apply<N>(r, e0, ld, c, cv);
    } else {
      store_f32<N>(L2, ld, r, e0, l2);
      if (L2b) store_16<HT, N>(L2b, ld, r, e0, l2);
      if (conv && !skip) store_f32<N>(conv, ld, r, e0, cv);
    }
  }
};

// y = (A + I) x: out = out_scale * (x_i + acc), written with leading
// dimension ldy for columns < d (out_scale undoes the input scaling of the
// FP16 form; 1 otherwise).
template <typename XT>
struct EpiAPlusI {
  const XT* __restrict__ X;
  int64_t ld;
  float* __restrict__ Y;
  int64_t ldy;
  int d;
  float out_scale;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    float x[N];
    load_row<XT, N>(X, ld, r, e0, x);
    float* y = Y + r * ldy + e0;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (e0 + i < d) y[i] = out_scale * (x[i] + acc[i]);
  }
};

// Adjoint start: h = (A + I) g;  b = h / d~_i (FP32 and BF16 copy).
template <typename XT>
struct EpiAdjInit {
  using HT = typename ShadowOf<XT>::type;
  const float4* __restrict__ coef;
  const XT* __restrict__ G;
  int64_t ld;
  float* __restrict__ H;
  float* __restrict__ Bf;
  HT* __restrict__ Bb;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    const float4 c = __ldg(coef + r);
    float gr[N], h[N], b[N];
    load_row<XT, N>(G, ld, r, e0, gr);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      h[i] = gr[i] + acc[i];
      b[i] = h[i] * c.w;
    }
    store_f32<N>(H, ld, r, e0, h);
    store_f32<N>(Bf, ld, r, e0, b);
    if (Bb) store_16<HT, N>(Bb, ld, r, e0, b);
  }
};

// dst (n x ld, zero padding) = scale * src (n x d) and its 16-bit copy.
template <typename HT>
__global__ void k_pad_copy(const float* __restrict__ src, int64_t n, int d, float scale, float* __restrict__ dst,
                           int64_t ld, HT* __restrict__ dstb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * ld; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / ld;
    const int j = (int)(t - i * ld);
    const float v = j < d ? scale * src[i * d + j] : 0.0f;
    dst[t] = v;
    if (dstb) {
      if constexpr (std::is_same<HT, __half>::value)
        dstb[t] = __float2half_rn(v);
      else
        dstb[t] = __float2bfloat16_rn(v);
    }
  }
}

// dst (n x d) = scale * src (n x ld).
__global__ void k_unpad_copy(const float* __restrict__ src, int64_t ld, int64_t n, int d, float scale,
                             float* __restrict__ dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * d; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / d;
    dst[t] = scale * src[i * ld + (t - i * d)];
  }
}

// y = alpha x (FP32) and its 16-bit copy.
template <typename HT>
__global__ void k_scale_copy(const float* __restrict__ x, int64_t total, float alpha, float* __restrict__ y,
                             HT* __restrict__ yb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const float v = alpha * x[t];
    y[t] = v;
    if (yb) {
      if constexpr (std::is_same<HT, __half>::value)
        yb[t] = __float2half_rn(v);
      else
        yb[t] = __float2bfloat16_rn(v);
    }
  }
}

// Largest |x| over an n x d FP32 matrix (row stride d): one float per
// block; non-finite values count as +inf.
static constexpr int kAmaxBlocks = 512;
__global__ void k_amax_partial(const float* __restrict__ x, int64_t total, float* __restrict__ out) {
  float m = 0.0f;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const float a = fabsf(x[t]);
    m = (a <= m) ? m : (isfinite(a) ? a : INFINITY);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  __shared__ float ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = fmaxf(t, ws[i]);
    out[blockIdx.x] = t;
  }
}

// <h, x> partial sums: FP32 within a thread, FP64 across threads, one
// value per block (summed in block order on the host).
static constexpr int kDotBlocks = 1024;
__global__ void k_dot_partial(const float* __restrict__ h, const float* __restrict__ x, int64_t total,
                              double* __restrict__ out) {
  float s = 0.0f;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    s = fmaf(h[t], x[t], s);
  double d = (double)s;
  for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
    out[blockIdx.x] = t;
  }
}

struct Bufs {
  lne_ctx* ctx;
  std::vector<void*> ptrs;
  explicit Bufs(lne_ctx* c) : ctx(c) {}
  template <typename T>
  int get(T** out, size_t count, const char* what) {
    void* p = nullptr;
    int rc = dalloc(ctx, &p, sizeof(T) * (count > 0 ? count : 1), what);
    if (rc == LNE_OK) ptrs.push_back(p);
    *out = (T*)p;
    return rc;
  }
  ~Bufs() {
    for (void* p : ptrs) dfree(ctx, p);
  }
};

// Shared state of one filter evaluation.
template <typename XT>
struct Filter {
  static constexpr bool k16 = sizeof(XT) == 2;
  using HT = typename ShadowOf<XT>::type;
  lne_ctx* ctx;
  lne_graph* g;
  GraphRows R;
  int64_t n, ld;
  const float4* coef;
  int* launches;
  Bufs* B;
  size_t sz() const { return (size_t)n * ld; }

  // operand view of an FP32 vector with an optional 16-bit copy
  const XT* op(const float* f, const HT* b) const { return k16 ? (const XT*)b : (const XT*)f; }

  int apply_m(const XT* X, float* out_f, HT* out_b) {
    EpiApplyM<XT> epi{coef, X, ld, out_f, out_b};
    return spmm_run<XT>(ctx, R, g->plan, X, ld, ld, epi, launches);
  }

  // The Chebyshev filter on x (FP32 xf, operand copy xb): fin = base -
  // scale * sum_k c_k T_k(X) x written to finf / finb.
  int run(const float* xf, const HT* xb, int order, const std::vector<float>& c, const float* base,
          bool scale_dt, float* finf, HT* finb) {
    int rc;
    float *conv = nullptr, *Tf = nullptr;
    HT* Tb = nullptr;
    float* ring[3] = {nullptr, nullptr, nullptr};
    HT* ringb[3] = {nullptr, nullptr, nullptr};
    const int nring = order > 2 ? 3 : 1;
    if ((rc = B->get(&conv, sz(), "conv"))) return rc;
    for (int i = 0; i < nring; ++i) {
      if ((rc = B->get(&ring[i], sz(), "Chebyshev vector"))) return rc;
      if (k16 && (rc = B->get(&ringb[i], sz(), "Chebyshev vector 16-bit"))) return rc;
    }
    if (k16) {
      if ((rc = B->get(&Tb, sz(), "tmp 16-bit"))) return rc;
    } else if ((rc = B->get(&Tf, sz(), "tmp"))) {
      return rc;
    }
    const XT* X0 = op(xf, xb);
    const XT* Tx = k16 ? (const XT*)Tb : (const XT*)Tf;
    if ((rc = apply_m(X0, k16 ? nullptr : Tf, k16 ? Tb : nullptr))) return rc;  // tmp = M x
    const bool first_is_last = order <= 2;
    {
      FinalOut<HT> fo{first_is_last ? base : nullptr, scale_dt, finf, finb};
      EpiFirst<XT> epi{coef, Tx, xf, ring[0], ringb[0], conv, fo, ld, c[0], c[1]};
      if ((rc = spmm_run<XT>(ctx, R, g->plan, Tx, ld, ld, epi, launches))) return rc;
    }
    const float* l0 = xf;
    int j1 = 0;
    for (int k = 2; k < order; ++k) {
      const int j2 = (j1 + 1) % 3;
      if ((rc = apply_m(op(ring[j1], ringb[j1]), k16 ? nullptr : Tf, k16 ? Tb : nullptr))) return rc;
      const bool last = k == order - 1;
      FinalOut<HT> fo{last ? base : nullptr, scale_dt, finf, finb};
      // conv is updated on odd orders (and on the last): even orders are
      // added with the next one
      const bool skip = !last && (k % 2 == 0);
      const float ck_prev = (k % 2 == 1) ? c[k - 1] : 0.0f;
      EpiStep<XT> epi{coef, Tx, l0, ring[j1], nullptr, ring[j2], ringb[j2], conv, fo, ld, c[k], ck_prev, skip};
      if ((rc = spmm_run<XT>(ctx, R, g->plan, Tx, ld, ld, epi, launches))) return rc;
      l0 = ring[j1];
      j1 = j2;
    }
    return LNE_OK;
  }
};

template <typename XT>
int setup_filter(lne_ctx* ctx, lne_graph* g, const lne_propagate_params* p, Bufs& B, int* launches, Filter<XT>& F,
                 float4** coef_out) {
  const int64_t n = g->n;
  float4* coef = nullptr;
  int rc;
  if ((rc = B.get(&coef, n, "operator coefficients"))) return rc;
  k_op_coef<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(g->vdata, n, (float)p->mu, coef);
  *launches += 1;
  F = Filter<XT>{ctx, g, GraphRows{g->vdata, g->nbrs}, n, pad_ld(p->dim), coef, launches, &B};
  *coef_out = coef;
  return LNE_OK;
}

// Power-of-two input scale of the FP16 form.  The propagation is linear in
// its input, and scaling FP32 values by a power of two is exact, so the
// filter runs on scale * x and the outputs are multiplied by 1 / scale.
// The scale puts the input's largest |value| in [2^6, 2^7): the Chebyshev
// vectors keep 2^9 of headroom below FP16's largest finite value (65504),
// and entries down to 2^-18 of the largest stay in FP16's normal range.
// The FP32 and BF16 forms (BF16 has FP32's exponent range) use 1.
template <typename XT>
int input_scale(lne_ctx* ctx, const float* x, int64_t total, Bufs& B, int* launches, float* scale) {
  *scale = 1.0f;
  if constexpr (!std::is_same<XT, __half>::value) {
    return LNE_OK;
  } else {
    float* part = nullptr;
    int rc;
    if ((rc = B.get(&part, kAmaxBlocks, "amax partials"))) return rc;
    k_amax_partial<<<kAmaxBlocks, 256, 0, ctx->stream>>>(x, total, part);
    *launches += 1;
    std::vector<float> h(kAmaxBlocks);
    LNE_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(float) * kAmaxBlocks, cudaMemcpyDeviceToHost, ctx->stream));
    LNE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    float m = 0.0f;
    for (float v : h) m = v > m ? v : m;
    if (!(m > 0.0f) || !std::isfinite(m)) return LNE_OK;
    int e = 0;
    frexpf(m, &e);  // m in [2^(e-1), 2^e)
    int k = 7 - e;
    k = k < -126 ? -126 : (k > 126 ? 126 : k);
    *scale = ldexpf(1.0f, k);
    return LNE_OK;
  }
}

template <typename XT>
int propagate_impl(lne_ctx* ctx, lne_graph* g, const lne_propagate_params* p, const float* d_a, float* d_y,
                   float* d_a_out, lne_propagate_stats* stats) {
  constexpr bool k16 = sizeof(XT) == 2;
  using HT = typename ShadowOf<XT>::type;
  const int64_t n = g->n;
  const int d = (int)p->dim;
  const int64_t ld = pad_ld(d);
  cudaStream_t st = ctx->stream;
  int launches = 0;
  std::vector<float> c;
  chebyshev_coeffs(p->order, p->s, c);
  Bufs B(ctx);
  Filter<XT> F;
  float4* coef = nullptr;
  int rc;
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, st);
  if ((rc = setup_filter<XT>(ctx, g, p, B, &launches, F, &coef))) return rc;
  float sc = 1.0f;
  if ((rc = input_scale<XT>(ctx, d_a, n * d, B, &launches, &sc))) return rc;
  float *A = nullptr, *Af = nullptr;
  HT *Ab = nullptr, *Afb = nullptr;
  const size_t sz = (size_t)n * ld;
  if ((rc = B.get(&A, sz, "a")) || (rc = B.get(&Af, sz, "a - conv"))) return rc;
  if (k16 && ((rc = B.get(&Ab, sz, "a 16-bit")) || (rc = B.get(&Afb, sz, "a - conv 16-bit")))) return rc;
  const unsigned pg = (unsigned)std::min<int64_t>((n * ld + 255) / 256, (int64_t)ctx->num_sms * 32);
  k_pad_copy<HT><<<pg, 256, 0, st>>>(d_a, n, d, sc, A, ld, Ab);
  launches += 1;
  // a - conv, then y = (A + I)(a - conv)
  if ((rc = F.run(A, Ab, p->order, c, A, false, Af, Afb))) return rc;
  {
    const XT* Xf = F.op(Af, Afb);
    EpiAPlusI<XT> epi{Xf, ld, d_y, d, d, 1.0f / sc};
    if ((rc = spmm_run<XT>(ctx, F.R, g->plan, Xf, ld, ld, epi, &launches))) return rc;
  }
  if (d_a_out) {
    k_unpad_copy<<<pg, 256, 0, st>>>(Af, ld, n, d, 1.0f / sc, d_a_out);
    launches += 1;
  }
  cudaEventRecord(ev1, st);
  LNE_CUDA_TRY(cudaEventSynchronize(ev1));
  LNE_CUDA_TRY(cudaGetLastError());
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    cudaEventElapsedTime(&stats->ms_total, ev0, ev1);
    stats->kernel_launches = launches;
    stats->spmm_calls = 2 * (p->order > 2 ? p->order - 1 : 1) + 1;
  }
  ctx->launch_count += launches;
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  return LNE_OK;
}

// Derivatives of the reference's weights with respect to s:
// c_0 = I0(s), c_k = 2 (-1)^k I_k(s);  I0' = I1, I_k' = (I_{k-1} + I_{k+1}) / 2.
void chebyshev_coeffs_ds(int order, double s, std::vector<double>& dc) {
  const double sf = (double)(float)s;
  dc.assign(order > 2 ? order : 2, 0.0);
  dc[0] = bessel_i(1, sf);
  for (int k = 1; k < (int)dc.size(); ++k)
    dc[k] = ((k & 1) ? -1.0 : 1.0) * (bessel_i(k - 1, sf) + bessel_i(k + 1, sf));
}

// dL/dmu and dL/ds in FP32 (P3): the forward pass on a with the mu-tangent
// T'_1 = -M a, T'_{k+1} = M(M T'_k) - 2 T'_k - T'_{k-1} - 2 M T_k, and the
// dots <h, T_k a>, <h, T'_k> (h = hscale^-1 H): dL/ds = -sum_k c_k'(s)
// <h, T_k a>, dL/dmu = -sum_k c_k <h, T'_k>.
int param_grads(lne_ctx* ctx, Filter<float>& F, const lne_propagate_params* p, const std::vector<float>& c,
                const float* H, const float* d_a, double hscale, double* h_dmu, double* h_ds) {
  const int64_t n = F.n, ld = F.ld;
  const int d = (int)p->dim;
  const int order = p->order;
  const size_t sz = (size_t)n * ld;
  const int64_t total = (int64_t)sz;
  cudaStream_t st = ctx->stream;
  Bufs& B = *F.B;
  int& launches = *F.launches;
  const float4* coef = F.coef;
  int rc;
  const int K = order > 2 ? order : 2;
  double* partial = nullptr;
  if ((rc = B.get(&partial, (size_t)2 * K * kDotBlocks, "dot partials"))) return rc;
  LNE_CUDA_TRY(cudaMemsetAsync(partial, 0, sizeof(double) * 2 * K * kDotBlocks, st));
  auto dot = [&](int slot, const float* x) {
    k_dot_partial<<<kDotBlocks, 256, 0, st>>>(H, x, total, partial + (int64_t)slot * kDotBlocks);
    launches += 1;
  };
  float *A = nullptr, *Tm = nullptr, *Tpm = nullptr;  // a, M T_k, M T'_k
  float* T[3];
  float* Tp[3];
  if ((rc = B.get(&A, sz, "a")) || (rc = B.get(&Tm, sz, "M T")) || (rc = B.get(&Tpm, sz, "M T'"))) return rc;
  for (int i = 0; i < 3; ++i)
    if ((rc = B.get(&T[i], sz, "T")) || (rc = B.get(&Tp[i], sz, "T'"))) return rc;
  const unsigned pg = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 32);
  k_pad_copy<__nv_bfloat16><<<pg, 256, 0, st>>>(d_a, n, d, 1.0f, A, ld, nullptr);
  launches += 1;
  dot(0, A);  // <h, T_0>
  // tmp = M a;  T_1 = 0.5 M tmp - a;  T'_1 = -tmp
  if ((rc = F.apply_m(A, Tm, nullptr))) return rc;
  {
    FinalOut<__nv_bfloat16> fo{nullptr, false, nullptr, nullptr};
    EpiFirst<float> epi{coef, Tm, A, T[0], nullptr, nullptr, fo, ld, 0.0f, 0.0f};
    if ((rc = spmm_run<float>(ctx, F.R, F.g->plan, Tm, ld, ld, epi, &launches))) return rc;
  }
  k_scale_copy<__nv_bfloat16><<<pg, 256, 0, st>>>(Tm, total, -1.0f, Tp[0], nullptr);
  launches += 1;
  dot(1, T[0]);
  dot(K + 1, Tp[0]);
  const float* t0 = A;         // T_{k-1}
  const float* tp0 = nullptr;  // T'_{k-1} (T'_0 = 0)
  int j1 = 0;
  for (int k = 1; k + 1 < order; ++k) {
    const int j2 = (j1 + 1) % 3;
    // tmp = M T_k; T_{k+1} = M tmp - 2 T_k - T_{k-1}
    if ((rc = F.apply_m(T[j1], Tm, nullptr))) return rc;
    {
      FinalOut<__nv_bfloat16> fo{nullptr, false, nullptr, nullptr};
      EpiStep<float> epi{coef, Tm, t0, T[j1], nullptr, T[j2], nullptr, nullptr, fo, ld, 0.0f};
      if ((rc = spmm_run<float>(ctx, F.R, F.g->plan, Tm, ld, ld, epi, &launches))) return rc;
    }
    // tmp' = M T'_k; T'_{k+1} = M tmp' - 2 T'_k - T'_{k-1} - 2 M T_k
    if ((rc = F.apply_m(Tp[j1], Tpm, nullptr))) return rc;
    {
      FinalOut<__nv_bfloat16> fo{nullptr, false, nullptr, nullptr};
      EpiStep<float> epi{coef, Tpm, tp0, Tp[j1], Tm, Tp[j2], nullptr, nullptr, fo, ld, 0.0f};
      if ((rc = spmm_run<float>(ctx, F.R, F.g->plan, Tpm, ld, ld, epi, &launches))) return rc;
    }
    dot(k + 1, T[j2]);
    dot(K + k + 1, Tp[j2]);
    t0 = T[j1];
    tp0 = Tp[j1];
    j1 = j2;
  }
  std::vector<double> hp((size_t)2 * K * kDotBlocks);
  LNE_CUDA_TRY(cudaMemcpyAsync(hp.data(), partial, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, st));
  LNE_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<double> dots(2 * K, 0.0);
  for (int sidx = 0; sidx < 2 * K; ++sidx) {
    for (int b = 0; b < kDotBlocks; ++b) dots[sidx] += hp[(size_t)sidx * kDotBlocks + b];
    dots[sidx] *= hscale;
  }
  std::vector<double> dc;
  chebyshev_coeffs_ds(order, p->s, dc);
  // only the terms the forward filter uses: k < max(order, 2)
  double gs = 0.0, gmu = 0.0;
  for (int k = 0; k < K; ++k) gs -= dc[k] * dots[k];
  for (int k = 1; k < K; ++k) gmu -= (double)c[k] * dots[K + k];
  if (h_ds) *h_ds = gs;
  if (h_dmu) *h_dmu = gmu;
  return LNE_OK;
}

template <typename XT>
int adjoint_impl(lne_ctx* ctx, lne_graph* g, const lne_propagate_params* p, const float* d_a, const float* d_gy,
                 float* d_ga, double* h_dmu, double* h_ds, lne_propagate_stats* stats) {
  constexpr bool k16 = sizeof(XT) == 2;
  using HT = typename ShadowOf<XT>::type;
  const int64_t n = g->n;
  const int d = (int)p->dim;
  const int64_t ld = pad_ld(d);
  const int order = p->order;
  cudaStream_t st = ctx->stream;
  int launches = 0;
  std::vector<float> c;
  chebyshev_coeffs(order, p->s, c);
  Bufs B(ctx);
  Filter<XT> F;
  float4* coef = nullptr;
  int rc;
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, st);
  if ((rc = setup_filter<XT>(ctx, g, p, B, &launches, F, &coef))) return rc;
  const size_t sz = (size_t)n * ld;
  const int64_t total = (int64_t)sz;
  // the FP16 form runs on a scaled output gradient sg * g (dL/da is linear
  // in g; the FP32 parameter-gradient pass unscales its dots by 1 / sg)
  float sg = 1.0f;
  if ((rc = input_scale<XT>(ctx, d_gy, n * d, B, &launches, &sg))) return rc;
  float *G = nullptr, *H = nullptr, *Bf = nullptr, *GA = nullptr;
  HT *Gb = nullptr, *Bb = nullptr;
  if ((rc = B.get(&G, sz, "g")) || (rc = B.get(&H, sz, "h")) || (rc = B.get(&Bf, sz, "b")) ||
      (rc = B.get(&GA, sz, "grad a")))
    return rc;
  if (k16 && ((rc = B.get(&Gb, sz, "g 16-bit")) || (rc = B.get(&Bb, sz, "b 16-bit")))) return rc;
  const unsigned pg = (unsigned)std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 32);
  k_pad_copy<HT><<<pg, 256, 0, st>>>(d_gy, n, d, sg, G, ld, Gb);
  launches += 1;
  // h = (A + I) g, b = D~^-1 h
  {
    const XT* Gx = F.op(G, Gb);
    EpiAdjInit<XT> epi{coef, Gx, ld, H, Bf, Bb};
    if ((rc = spmm_run<XT>(ctx, F.R, g->plan, Gx, ld, ld, epi, &launches))) return rc;
  }
  // grad a = h - D~ sum_k c_k T_k(X) b      (M^T = D~ M D~^-1)
  if ((rc = F.run(Bf, Bb, order, c, H, true, GA, nullptr))) return rc;
  if (d_ga) {
    k_unpad_copy<<<pg, 256, 0, st>>>(GA, ld, n, d, 1.0f / sg, d_ga);
    launches += 1;
  }
  if (h_dmu || h_ds) {
    // The parameter gradients run in FP32 in every form: they are sums over
    // the orders whose terms cancel, so 16-bit gathers would cost them far
    // more relative accuracy than they cost dL/da.  The 16-bit forms first
    // form an FP32 h = (A + I) g from the FP32 copy of (scaled) g.
    Filter<float> F32{ctx, g, F.R, n, ld, coef, &launches, &B};
    const float* H32 = H;
    if (k16) {
      float *H2 = nullptr, *Bs = nullptr;
      if ((rc = B.get(&H2, sz, "h fp32")) || (rc = B.get(&Bs, sz, "b fp32"))) return rc;
      EpiAdjInit<float> epi{coef, G, ld, H2, Bs, nullptr};
      if ((rc = spmm_run<float>(ctx, F32.R, g->plan, G, ld, ld, epi, &launches))) return rc;
      H32 = H2;
    }
    if ((rc = param_grads(ctx, F32, p, c, H32, d_a, 1.0 / (double)sg, h_dmu, h_ds))) return rc;
  }
  cudaEventRecord(ev1, st);
  LNE_CUDA_TRY(cudaEventSynchronize(ev1));
  LNE_CUDA_TRY(cudaGetLastError());
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    cudaEventElapsedTime(&stats->ms_total, ev0, ev1);
    stats->kernel_launches = launches;
  }
  ctx->launch_count += launches;
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  return LNE_OK;
}

}  // namespace

}  // namespace lne

using namespace lne;

extern "C" int lne_propagate(lne_ctx* ctx, const lne_graph* g, const lne_propagate_params* p, const float* d_a,
                             float* d_y, float* d_a_out, lne_propagate_stats* stats) {
  LNE_CHECK_ARG(ctx && g && p && d_a && d_y, "lne_propagate: NULL argument");
  LNE_CHECK_ARG(p->dim >= 1 && p->order >= 0, "lne_propagate: bad dim/order");
  LNE_CHECK_ARG(p->precision == LNE_PREC_FP32 || p->precision == LNE_PREC_BF16 || p->precision == LNE_PREC_FP16,
                "lne_propagate: bad precision");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  lne_graph* gm = const_cast<lne_graph*>(g);
  if (!gm->plan_ready) ctx->launch_count += kPlanLaunches;
  int rc = build_plan_graph(ctx, gm);
  if (rc) return rc;
  if (p->precision == LNE_PREC_BF16) return propagate_impl<__nv_bfloat16>(ctx, gm, p, d_a, d_y, d_a_out, stats);
  if (p->precision == LNE_PREC_FP16) return propagate_impl<__half>(ctx, gm, p, d_a, d_y, d_a_out, stats);
  return propagate_impl<float>(ctx, gm, p, d_a, d_y, d_a_out, stats);
}

extern "C" int lne_propagate_adjoint(lne_ctx* ctx, const lne_graph* g, const lne_propagate_params* p,
                                     const float* d_a, const float* d_gy, float* d_ga, double* h_dmu, double* h_ds,
                                     lne_propagate_stats* stats) {
  LNE_CHECK_ARG(ctx && g && p && d_gy, "lne_propagate_adjoint: NULL argument");
  LNE_CHECK_ARG(d_a || (!h_dmu && !h_ds), "lne_propagate_adjoint: the parameter gradients need a");
  LNE_CHECK_ARG(p->dim >= 1 && p->order >= 0, "lne_propagate_adjoint: bad dim/order");
  LNE_CHECK_ARG(p->precision == LNE_PREC_FP32 || p->precision == LNE_PREC_BF16 || p->precision == LNE_PREC_FP16,
                "lne_propagate_adjoint: bad precision");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  lne_graph* gm = const_cast<lne_graph*>(g);
  if (!gm->plan_ready) ctx->launch_count += kPlanLaunches;
  int rc = build_plan_graph(ctx, gm);
  if (rc) return rc;
  if (p->precision == LNE_PREC_BF16)
    return adjoint_impl<__nv_bfloat16>(ctx, gm, p, d_a, d_gy, d_ga, h_dmu, h_ds, stats);
  if (p->precision == LNE_PREC_FP16) return adjoint_impl<__half>(ctx, gm, p, d_a, d_gy, d_ga, h_dmu, h_ds, stats);
  return adjoint_impl<float>(ctx, gm, p, d_a, d_gy, d_ga, h_dmu, h_ds, stats);
}

extern "C" int lne_chebyshev_coefficients(int32_t order, double s, float* out) {
  LNE_CHECK_ARG(out && order >= 0, "lne_chebyshev_coefficients: bad argument");
  std::vector<float> c;
  chebyshev_coeffs(order, s, c);
  for (size_t i = 0; i < c.size(); ++i) out[i] = c[i];
  return LNE_OK;
}
