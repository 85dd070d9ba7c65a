// Arithmetic shared by the sparsifier kernels and their host-side tests.
//
// Everything here is __host__ __device__ so that the same code can be
// compiled by g++ for the CPU unit tests (tests/test_math_host.py) and by
// nvcc for the kernels.
#pragma once
#include <stdint.h>
#include <math.h>

#ifdef __CUDACC__
#define LNE_HD __host__ __device__ __forceinline__
#else
#define LNE_HD static inline
#endif

namespace lne {

// ---------------------------------------------------------------------------
// Counter-based generator of the reference (pbbslib/random.h:38-51): a state
// word, rand() = h(state), next() = h(h(state)), fork(i) = h(h(i + state)),
// with h the splitmix64-style finaliser hash64_2 (pbbslib/utilities.h:154-159).
// ---------------------------------------------------------------------------
LNE_HD uint64_t hash64_2(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}
LNE_HD uint64_t rng_rand(uint64_t s) { return hash64_2(s); }
LNE_HD uint64_t rng_next(uint64_t s) { return hash64_2(hash64_2(s)); }
LNE_HD uint64_t rng_fork(uint64_t s, uint64_t i) { return hash64_2(hash64_2(i + s)); }

// map_uint64_t (LightNE/PathEmbed.h:25-30): u64 -> double rounds to nearest,
// and the divide by 2^64 is exact, so it is a scale by 2^-64.
LNE_HD double map_uint64(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(__ull2double_rn(u), 5.421010862427522170037264004349708557128906250e-20);
#else
  return (double)u * 5.421010862427522170037264004349708557128906250e-20;
#endif
}

// One draw of the generator: returns rand() and advances the state with
// next(), sharing the h(state) the two have in common.
LNE_HD uint64_t rng_draw(uint64_t& s) {
  const uint64_t x = hash64_2(s);
  s = hash64_2(x);
  return x;
}

// x mod d for a 64-bit x and a 32-bit d >= 1: the reference takes
// `rand() % degree` in 64-bit unsigned arithmetic (LightNE/PathEmbed.h:43).
LNE_HD uint32_t mod_u64_u32(uint64_t x, uint32_t d) {
  return (uint32_t)(x % (uint64_t)d);
}

// Division by an invariant 32-bit divisor with a precomputed multiplier,
// after Granlund and Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), Figure 4.1 (unsigned, N = 64):
//   l = ceil(log2 d),  m' = floor(2^64 (2^l - d) / d) + 1,
//   t1 = MULUH(m', x),  q = (t1 + ((x - t1) >> min(l,1))) >> max(l-1,0).
// Exact for every 64-bit x and 1 <= d < 2^32.
LNE_HD uint32_t ceil_log2_u32(uint32_t d) {
#ifdef __CUDA_ARCH__
  return d <= 1 ? 0u : 32u - (uint32_t)__clz(d - 1);
#else
  return d <= 1 ? 0u : 32u - (uint32_t)__builtin_clz(d - 1);
#endif
}
LNE_HD uint64_t gm_magic(uint32_t d) {
  const uint32_t l = ceil_log2_u32(d);
  const uint64_t hi = ((uint64_t)1 << l) - (uint64_t)d;  // < d
  // floor(hi * 2^64 / d) by two base-2^32 long-division steps
  const uint64_t t1 = hi << 32;
  const uint64_t q1 = t1 / d, r1 = t1 % d;
  const uint64_t q2 = (r1 << 32) / d;
  return ((q1 << 32) + q2) + 1;
}
LNE_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
LNE_HD uint32_t gm_mod(uint64_t x, uint32_t d, uint64_t magic) {
  const uint32_t l = ceil_log2_u32(d);
  const uint32_t sh1 = l < 1 ? l : 1u, sh2 = l > 0 ? l - 1 : 0u;
  const uint64_t t1 = umulhi64(magic, x);
  const uint64_t q = (t1 + ((x - t1) >> sh1)) >> sh2;
  return (uint32_t)(x - q * (uint64_t)d);
}

// ---------------------------------------------------------------------------
// Double-double arithmetic (Dekker 1971; Knuth TAOCP vol. 2, 4.2.2) for the
// slow path of the trunc-log value.  Each operation is written with explicit
// round-to-nearest intrinsics on the device so that the compiler cannot fuse
// or reassociate it; the host build must use -ffp-contract=off.
// ---------------------------------------------------------------------------
struct dd { double hi, lo; };

#ifdef __CUDA_ARCH__
#define LNE_ADD(a, b) __dadd_rn((a), (b))
#define LNE_SUB(a, b) __dsub_rn((a), (b))
#define LNE_MUL(a, b) __dmul_rn((a), (b))
#define LNE_FMA(a, b, c) __fma_rn((a), (b), (c))
#define LNE_DIV(a, b) __ddiv_rn((a), (b))
#else
#define LNE_ADD(a, b) ((a) + (b))
#define LNE_SUB(a, b) ((a) - (b))
#define LNE_MUL(a, b) ((a) * (b))
#define LNE_FMA(a, b, c) fma((a), (b), (c))
#define LNE_DIV(a, b) ((a) / (b))
#endif

LNE_HD dd two_sum(double a, double b) {
  double s = LNE_ADD(a, b);
  double bb = LNE_SUB(s, a);
  double e = LNE_ADD(LNE_SUB(a, LNE_SUB(s, bb)), LNE_SUB(b, bb));
  return dd{s, e};
}
LNE_HD dd quick_two_sum(double a, double b) {  // requires |a| >= |b|
  double s = LNE_ADD(a, b);
  return dd{s, LNE_SUB(b, LNE_SUB(s, a))};
}
LNE_HD dd two_prod(double a, double b) {
  double p = LNE_MUL(a, b);
  return dd{p, LNE_FMA(a, b, -p)};
}
LNE_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo = LNE_ADD(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = LNE_ADD(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
LNE_HD dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = LNE_ADD(p.lo, LNE_ADD(LNE_MUL(a.hi, b.lo), LNE_MUL(a.lo, b.hi)));
  return quick_two_sum(p.hi, p.lo);
}
LNE_HD dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo = LNE_ADD(p.lo, LNE_MUL(a.lo, b));
  return quick_two_sum(p.hi, p.lo);
}
// a / b by long division with one correction term.
LNE_HD dd dd_div(dd a, dd b) {
  double q1 = LNE_DIV(a.hi, b.hi);
  dd r = dd_add(a, dd_mul_d(dd{-b.hi, -b.lo}, q1));
  double q2 = LNE_DIV(r.hi, b.hi);
  r = dd_add(r, dd_mul_d(dd{-b.hi, -b.lo}, q2));
  double q3 = LNE_DIV(r.hi, b.hi);
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}

// ln 2 split into a double-double: the nearest double, then the nearest
// double to the remainder (ln 2 = 0.693147180559945309417232121458176568...).
#define LNE_LN2_HI 6.93147180559945286226763982995180413e-01
#define LNE_LN2_LO 2.31904681384629955842e-17

// Natural log of a positive normal double to about 104 bits, from
//   x = 2^e * m, m in [sqrt(1/2), sqrt(2)),  s = (m - 1) / (m + 1),
//   ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...),
// with |s| <= 0.1716, so 24 terms of the series reach 2^-106.
LNE_HD dd log_dd(double x) {
  int e = 0;
  double m = frexp(x, &e);  // m in [0.5, 1)
  if (m < 0.70710678118654752440) { m = LNE_MUL(m, 2.0); e -= 1; }
  dd num = dd{LNE_SUB(m, 1.0), 0.0};  // exact: m in [0.5, 2]
  dd den = two_sum(m, 1.0);
  dd s = dd_div(num, den);
  dd s2 = dd_mul(s, s);
  const int K = 24;
  dd t = dd_div(dd{1.0, 0.0}, dd{(double)(2 * K + 1), 0.0});
  for (int k = K - 1; k >= 0; --k) {
    t = dd_add(dd_mul(t, s2), dd_div(dd{1.0, 0.0}, dd{(double)(2 * k + 1), 0.0}));
  }
  dd lm = dd_mul(dd_mul_d(s, 2.0), t);
  dd el = dd_mul_d(dd{LNE_LN2_HI, LNE_LN2_LO}, (double)e);
  return dd_add(el, lm);
}

// True when a double's rounding to float could change if the double moved
// by up to two units in its last place: the low 29 bits of the significand
// (the bits a double -> float conversion drops) lie within 4 of the halfway
// pattern 2^28.
LNE_HD bool float_rounding_is_close(double y) {
  uint64_t b;
#ifdef __CUDA_ARCH__
  b = (uint64_t)__double_as_longlong(y);
#else
  __builtin_memcpy(&b, &y, 8);
#endif
  int64_t low = (int64_t)(b & ((1ULL << 29) - 1));
  int64_t dist = low - (int64_t)(1ULL << 28);
  return dist >= -4 && dist <= 4;
}

}  // namespace lne
