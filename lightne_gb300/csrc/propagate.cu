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
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
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

__global__ void k_op_coef(const Vertex* __restrict__ vd, int64_t n, float mu, float2* __restrict__ coef) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float dt = (float)(vd[i].deg + 1u);
  const double inv = 1.0 / (double)dt;
  coef[i] = make_float2((float)(1.0 - (double)mu - inv), (float)(-inv));
}

// Loads N elements (N a multiple of 4, e0 a multiple of 4) of row r of a
// dense operand as floats: 16-byte loads for FP32, 8-byte loads for BF16
// (so an e0 that is 4 mod 8 stays aligned).
template <typename T, int N>
__device__ __forceinline__ void load_row(const T* __restrict__ X, int64_t ld, int64_t r, int e0, float (&o)[N]) {
  const T* p = X + r * ld + e0;
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(p + i));
      o[i] = v.x; o[i + 1] = v.y; o[i + 2] = v.z; o[i + 3] = v.w;
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
template <int N>
__device__ __forceinline__ void store_bf16(__nv_bfloat16* __restrict__ X, int64_t ld, int64_t r, int e0,
                                          const float (&o)[N]) {
  __nv_bfloat16* p = X + r * ld + e0;
#pragma unroll
  for (int i = 0; i < N; i += 2) *reinterpret_cast<__nv_bfloat162*>(p + i) = __floats2bfloat162_rn(o[i], o[i + 1]);
}

// tmp = M x: out = m_i x_i + o_i acc (operand x of type XT).
template <typename XT>
struct EpiApplyM {
  const float2* __restrict__ coef;
  const XT* __restrict__ X;  // the operand (diagonal term)
  int64_t ld;
  float* __restrict__ out_f;           // FP32 output (FP32 form) or null
  __nv_bfloat16* __restrict__ out_b;   // BF16 output (BF16 form) or null
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&a)[N]) const {
    const float2 c = __ldg(coef + r);
    float x[N], y[N];
    load_row<XT, N>(X, ld, r, e0, x);
#pragma unroll
    for (int i = 0; i < N; ++i) y[i] = fmaf(c.x, x[i], c.y * a[i]);
    if (out_f) store_f32<N>(out_f, ld, r, e0, y);
    if (out_b) store_bf16<N>(out_b, ld, r, e0, y);
  }
};

// First order: Lx1 = 0.5 M tmp - a;  conv = c0 a + c1 Lx1;  optionally the
// final a - conv when the filter has order <= 2.
template <typename XT>
struct EpiFirst {
  const float2* __restrict__ coef;
  const XT* __restrict__ T;        // tmp (operand)
  const float* __restrict__ A;     // a (FP32)
  float* __restrict__ L1;          // Lx1 FP32
  __nv_bfloat16* __restrict__ L1b; // Lx1 BF16 copy (BF16 form) or null
  float* __restrict__ conv;
  float* __restrict__ afin;        // a - conv, or null
  __nv_bfloat16* __restrict__ afinb;
  int64_t ld;
  float c0, c1;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    const float2 c = __ldg(coef + r);
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
    if (L1b) store_bf16<N>(L1b, ld, r, e0, l1);
    if (afin) {
#pragma unroll
      for (int i = 0; i < N; ++i) cv[i] = a[i] - cv[i];
      store_f32<N>(afin, ld, r, e0, cv);
      if (afinb) store_bf16<N>(afinb, ld, r, e0, cv);
    } else {
      store_f32<N>(conv, ld, r, e0, cv);
    }
  }
};

// Order k >= 2: Lx2 = M tmp - Lx0 - 2 Lx1;  conv += ck Lx2;  optionally
// a - conv on the last order.
template <typename XT>
struct EpiStep {
  const float2* __restrict__ coef;
  const XT* __restrict__ T;
  const float* __restrict__ L0;
  const float* __restrict__ L1;
  float* __restrict__ L2;
  __nv_bfloat16* __restrict__ L2b;
  float* __restrict__ conv;
  const float* __restrict__ A;
  float* __restrict__ afin;
  __nv_bfloat16* __restrict__ afinb;
  int64_t ld;
  float ck;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    const float2 c = __ldg(coef + r);
    float t[N], l0[N], l1[N], l2[N], cv[N];
    load_row<XT, N>(T, ld, r, e0, t);
    load_f32<N>(L0, ld, r, e0, l0);
    load_f32<N>(L1, ld, r, e0, l1);
    load_f32<N>(conv, ld, r, e0, cv);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const float mt = fmaf(c.x, t[i], c.y * acc[i]);
      l2[i] = fmaf(-2.0f, l1[i], mt - l0[i]);
      cv[i] = fmaf(ck, l2[i], cv[i]);
    }
    if (!afin) {
      store_f32<N>(L2, ld, r, e0, l2);
      if (L2b) store_bf16<N>(L2b, ld, r, e0, l2);
      store_f32<N>(conv, ld, r, e0, cv);
    } else {
      float a[N];
      load_f32<N>(A, ld, r, e0, a);
#pragma unroll
      for (int i = 0; i < N; ++i) a[i] -= cv[i];
      store_f32<N>(afin, ld, r, e0, a);
      if (afinb) store_bf16<N>(afinb, ld, r, e0, a);
    }
  }
};

// y = (A + I) x: out = x_i + acc, written with leading dimension ldy for
// columns < d.
template <typename XT>
struct EpiAPlusI {
  const XT* __restrict__ X;
  int64_t ld;
  float* __restrict__ Y;
  int64_t ldy;
  int d;
  template <int N>
  __device__ __forceinline__ void operator()(int64_t r, int e0, const float (&acc)[N]) const {
    float x[N];
    load_row<XT, N>(X, ld, r, e0, x);
    float* y = Y + r * ldy + e0;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (e0 + i < d) y[i] = x[i] + acc[i];
  }
};

__global__ void k_pad_copy(const float* __restrict__ src, int64_t n, int d, float* __restrict__ dst, int64_t ld,
                           __nv_bfloat16* __restrict__ dstb) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * ld; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / ld;
    const int j = (int)(t - i * ld);
    const float v = j < d ? src[i * d + j] : 0.0f;
    dst[t] = v;
    if (dstb) dstb[t] = __float2bfloat16_rn(v);
  }
}

__global__ void k_unpad_copy(const float* __restrict__ src, int64_t ld, int64_t n, int d, float* __restrict__ dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * d; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / d;
    dst[t] = src[i * ld + (t - i * d)];
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

template <typename XT>
int propagate_impl(lne_ctx* ctx, lne_graph* g, const lne_propagate_params* p, const float* d_a, float* d_y,
                   float* d_a_out, lne_propagate_stats* stats) {
  constexpr bool kBF16 = sizeof(XT) == 2;
  const int64_t n = g->n;
  const int d = (int)p->dim;
  const int64_t ld = pad_ld(d);
  const int order = p->order;
  cudaStream_t st = ctx->stream;
  int launches = 0;
  std::vector<float> c;
  chebyshev_coeffs(order, p->s, c);
  Bufs B(ctx);
  float2* coef = nullptr;
  float *A = nullptr, *conv = nullptr, *Tf = nullptr, *Af = nullptr;
  float* ring[3] = {nullptr, nullptr, nullptr};            // Chebyshev vectors, FP32
  __nv_bfloat16* ringb[3] = {nullptr, nullptr, nullptr};   // their BF16 copies (BF16 form)
  __nv_bfloat16 *Ab = nullptr, *Tb = nullptr, *Afb = nullptr;
  const size_t sz = (size_t)n * ld;
  const int nring = order > 2 ? 3 : 1;
  int rc;
  if ((rc = B.get(&coef, n, "operator coefficients")) || (rc = B.get(&A, sz, "a")) ||
      (rc = B.get(&conv, sz, "conv")) || (rc = B.get(&Af, sz, "a - conv")))
    return rc;
  for (int i = 0; i < nring; ++i)
    if ((rc = B.get(&ring[i], sz, "Chebyshev vector"))) return rc;
  if (kBF16) {
    if ((rc = B.get(&Ab, sz, "a bf16")) || (rc = B.get(&Tb, sz, "tmp bf16")) || (rc = B.get(&Afb, sz, "a - conv bf16")))
      return rc;
    for (int i = 0; i < nring; ++i)
      if ((rc = B.get(&ringb[i], sz, "Chebyshev vector bf16"))) return rc;
  } else {
    if ((rc = B.get(&Tf, sz, "tmp"))) return rc;
  }
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, st);
  k_op_coef<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g->vdata, n, (float)p->mu, coef);
  const unsigned pg = (unsigned)std::min<int64_t>((n * ld + 255) / 256, (int64_t)ctx->num_sms * 32);
  k_pad_copy<<<pg, 256, 0, st>>>(d_a, n, d, A, ld, Ab);
  launches += 2;
  GraphRows R{g->vdata, g->nbrs};
  const XT* Xa = kBF16 ? (const XT*)Ab : (const XT*)A;
  XT* Tx = kBF16 ? (XT*)Tb : (XT*)Tf;
  // tmp = M a
  {
    EpiApplyM<XT> epi{coef, Xa, ld, kBF16 ? nullptr : Tf, kBF16 ? Tb : nullptr};
    if ((rc = spmm_run<XT>(ctx, R, g->plan, Xa, ld, ld, epi, &launches))) return rc;
  }
  // Lx1 = 0.5 M tmp - a; conv = c0 a + c1 Lx1 (and a - conv when order <= 2)
  const bool first_is_last = order <= 2;
  {
    EpiFirst<XT> epi{coef, Tx, A, ring[0], ringb[0], conv, first_is_last ? Af : nullptr,
                     first_is_last ? Afb : nullptr, ld, c[0], c[1]};
    if ((rc = spmm_run<XT>(ctx, R, g->plan, Tx, ld, ld, epi, &launches))) return rc;
  }
  // Lx0 = a (never overwritten), Lx1 = ring[0]; each order writes Lx2 into
  // the ring slot that holds neither Lx0 nor Lx1.
  const float* l0 = A;
  int j1 = 0;
  for (int k = 2; k < order; ++k) {
    const int j2 = (j1 + 1) % 3;
    const XT* X1 = kBF16 ? (const XT*)ringb[j1] : (const XT*)ring[j1];
    {
      EpiApplyM<XT> epi{coef, X1, ld, kBF16 ? nullptr : Tf, kBF16 ? Tb : nullptr};
      if ((rc = spmm_run<XT>(ctx, R, g->plan, X1, ld, ld, epi, &launches))) return rc;
    }
    const bool last = k == order - 1;
    {
      EpiStep<XT> epi{coef, Tx, l0, ring[j1], ring[j2], ringb[j2], conv, A, last ? Af : nullptr,
                      last ? Afb : nullptr, ld, c[k]};
      if ((rc = spmm_run<XT>(ctx, R, g->plan, Tx, ld, ld, epi, &launches))) return rc;
    }
    l0 = ring[j1];
    j1 = j2;
  }
  // y = (A + I)(a - conv)
  {
    const XT* Xf = kBF16 ? (const XT*)Afb : (const XT*)Af;
    EpiAPlusI<XT> epi{Xf, ld, d_y, d, d};
    if ((rc = spmm_run<XT>(ctx, R, g->plan, Xf, ld, ld, epi, &launches))) return rc;
  }
  if (d_a_out) {
    k_unpad_copy<<<pg, 256, 0, st>>>(Af, ld, n, d, d_a_out);
    launches += 1;
  }
  cudaEventRecord(ev1, st);
  LNE_CUDA_TRY(cudaEventSynchronize(ev1));
  LNE_CUDA_TRY(cudaGetLastError());
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    cudaEventElapsedTime(&stats->ms_total, ev0, ev1);
    stats->kernel_launches = launches;
    stats->spmm_calls = 2 * (order > 2 ? order - 1 : 1) + 1;
  }
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
  LNE_CHECK_ARG(p->precision == LNE_PREC_FP32 || p->precision == LNE_PREC_BF16, "lne_propagate: bad precision");
  LNE_CUDA_TRY(cudaSetDevice(ctx->device));
  lne_graph* gm = const_cast<lne_graph*>(g);
  int rc = build_plan_graph(ctx, gm);
  if (rc) return rc;
  if (p->precision == LNE_PREC_BF16) return propagate_impl<__nv_bfloat16>(ctx, gm, p, d_a, d_y, d_a_out, stats);
  return propagate_impl<float>(ctx, gm, p, d_a, d_y, d_a_out, stats);
}

extern "C" int lne_chebyshev_coefficients(int32_t order, double s, float* out) {
  LNE_CHECK_ARG(out && order >= 0, "lne_chebyshev_coefficients: bad argument");
  std::vector<float> c;
  chebyshev_coeffs(order, s, c);
  for (size_t i = 0; i < c.size(); ++i) out[i] = c[i];
  return LNE_OK;
}
