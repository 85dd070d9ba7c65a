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
// hash64_2 is a bijection of the 64-bit words: x ^= x >> s is undone by
// xoring in the shifts by s, 2s, ... below 64, and a multiply by an odd
// constant by a multiply by its inverse mod 2^64.  So a pair key can travel
// as its hash and be recovered exactly.
LNE_HD uint64_t hash64_2_inv(uint64_t y) {
  y ^= (y >> 31) ^ (y >> 62);
  y *= 0x319642b2d24d8ec3ULL;  // 0x94d049bb133111eb^-1 mod 2^64
  y ^= (y >> 27) ^ (y >> 54);
  y *= 0x96de1b173f119089ULL;  // 0xbf58476d1ce4e5b9^-1 mod 2^64
  return y ^ (y >> 30) ^ (y >> 60);
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
// The remainder x - q d is below d < 2^32, so it is exact modulo 2^32 and
// only the low 32 bits of q = y >> sh2 (sh2 <= 31) are needed: one funnel
// shift instead of a 64-bit variable shift, one 32-bit multiply-add.
LNE_HD uint32_t shr64_lo32(uint64_t y, uint32_t sh) {
#ifdef __CUDA_ARCH__
  return __funnelshift_r((uint32_t)y, (uint32_t)(y >> 32), sh);
#else
  return (uint32_t)(y >> sh);
#endif
}
LNE_HD uint32_t gm_mod(uint64_t x, uint32_t d, uint64_t magic) {
  const uint32_t l = ceil_log2_u32(d);
  const uint32_t sh1 = l < 1 ? l : 1u, sh2 = l > 0 ? l - 1 : 0u;
  const uint64_t t1 = umulhi64(magic, x);
  const uint64_t y = t1 + ((x - t1) >> sh1);
  return (uint32_t)x - shr64_lo32(y, sh2) * d;
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


// ---------------------------------------------------------------------------
// Exact emulation, in integer arithmetic, of the reference's trunc-log input
//   adj = ((w * factor) / d_u) / d_v        (LightNE/PathEmbed.h:210)
// with every operation rounded to nearest-even in IEEE double, as the
// reference's double arithmetic does.  A positive normal double is held as
// (m, e): value = m * 2^e with 2^52 <= m < 2^53.
// ---------------------------------------------------------------------------
struct XDouble {
  uint64_t m;
  int32_t e;
};

LNE_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

LNE_HD XDouble xd_from_double(double x) {  // x positive normal
  uint64_t b;
#ifdef __CUDA_ARCH__
  b = (uint64_t)__double_as_longlong(x);
#else
  __builtin_memcpy(&b, &x, 8);
#endif
  const int be = (int)((b >> 52) & 0x7ff);
  return XDouble{(b & ((1ull << 52) - 1)) | (1ull << 52), be - 1075};
}

LNE_HD double xd_to_double(XDouble x) {  // exponent in normal range
  const uint64_t b = ((uint64_t)(x.e + 1075) << 52) | (x.m & ((1ull << 52) - 1));
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  __builtin_memcpy(&d, &b, 8);
  return d;
#endif
}

LNE_HD XDouble xd_from_u64(uint64_t w) {  // exact for w < 2^53, w >= 1
  const int lz = clz64(w);
  return XDouble{w << (lz - 11), -(lz - 11)};
}

// Rounds the 128-bit value (hi, lo) * 2^e (nonzero) to 53 bits, nearest
// even; `sticky` marks nonzero bits below lo.
LNE_HD XDouble xd_round128(uint64_t hi, uint64_t lo, int e, bool sticky) {
  int lz = hi ? clz64(hi) : 64 + clz64(lo);
  // normalise so that the leading one is bit 127
  if (lz >= 64) {
    hi = lo;
    lo = 0;
    lz -= 64;
    e -= 64;
  }
  if (lz > 0) {
    hi = (hi << lz) | (lo >> (64 - lz));
    lo <<= lz;
    e -= lz;
  }
  // keep bits 127..75 (53 bits): m = hi >> 11; round bit = bit 74 = hi bit 10
  uint64_t m = hi >> 11;
  const bool round = (hi >> 10) & 1;
  const bool rest = sticky || (hi & ((1ull << 10) - 1)) || lo;
  e += 75;
  if (round && (rest || (m & 1))) {
    ++m;
    if (m == (1ull << 53)) {
      m >>= 1;
      ++e;
    }
  }
  return XDouble{m, e};
}

LNE_HD XDouble xd_mul(XDouble a, XDouble b) {
  const uint64_t lo = a.m * b.m;
  const uint64_t hi = umulhi64(a.m, b.m);
  return xd_round128(hi, lo, a.e + b.e, false);
}

LNE_HD uint64_t gm_div(uint64_t x, uint32_t d, uint64_t magic) {
  const uint32_t l = ceil_log2_u32(d);
  const uint32_t sh1 = l < 1 ? l : 1u, sh2 = l > 0 ? l - 1 : 0u;
  const uint64_t t1 = umulhi64(magic, x);
  return (t1 + ((x - t1) >> sh1)) >> sh2;
}

// a / d for a 32-bit integer d >= 1 (with its Granlund-Montgomery multiplier):
// long division of a.m * 2^34 in base-2^32 digits, then rounding.
LNE_HD XDouble xd_div_u32(XDouble a, uint32_t d, uint64_t magic) {
  const uint64_t nhi = a.m >> 30, nlo = a.m << 34;  // a.m * 2^34 as 128 bits
  const uint32_t dig[4] = {(uint32_t)(nhi >> 32), (uint32_t)nhi, (uint32_t)(nlo >> 32), (uint32_t)nlo};
  uint64_t rem = 0, q[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint64_t cur = (rem << 32) | dig[i];
    q[i] = gm_div(cur, d, magic);
    rem = cur - q[i] * (uint64_t)d;
  }
  const uint64_t qhi = (q[0] << 32) | q[1], qlo = (q[2] << 32) | q[3];
  return xd_round128(qhi, qlo, a.e - 34, rem != 0);
}

// adj of the trunc-log map, exactly as the reference's double arithmetic.
LNE_HD XDouble trunc_log_adj(uint64_t wcount, bool diag, XDouble factor, uint32_t du, uint64_t mu_, uint32_t dv,
                             uint64_t mv) {
  XDouble w = xd_from_u64(wcount);
  if (diag) w.e += 1;  // w * 2 is exact
  return xd_div_u32(xd_div_u32(xd_mul(w, factor), du, mu_), dv, mv);
}

// ---------------------------------------------------------------------------
// log(adj) in double-float (pairs of floats, ~2^-46 relative) for deciding
// the float the reference obtains by narrowing its double log:
//   adj = 2^E * m, m in [1, 2); c_j = 1 + j/128 (j = top 7 fraction bits);
//   log adj = E ln2 + log c_j + log(1 + r),  r = (m - c_j) / c_j in [0, 2^-7)
// The table log(c_j), 1/c_j (double-float) is built on the host.
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
};

#ifdef __CUDA_ARCH__
#define LNE_FADD(a, b) __fadd_rn((a), (b))
#define LNE_FSUB(a, b) __fsub_rn((a), (b))
#define LNE_FMUL(a, b) __fmul_rn((a), (b))
#define LNE_FFMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define LNE_FADD(a, b) ((a) + (b))
#define LNE_FSUB(a, b) ((a) - (b))
#define LNE_FMUL(a, b) ((a) * (b))
#define LNE_FFMA(a, b, c) fmaf((a), (b), (c))
#endif

LNE_HD df df_two_sum(float a, float b) {
  const float s = LNE_FADD(a, b);
  const float bb = LNE_FSUB(s, a);
  return df{s, LNE_FADD(LNE_FSUB(a, LNE_FSUB(s, bb)), LNE_FSUB(b, bb))};
}
LNE_HD df df_fast_two_sum(float a, float b) {
  const float s = LNE_FADD(a, b);
  return df{s, LNE_FSUB(b, LNE_FSUB(s, a))};
}
LNE_HD df df_add(df a, df b) {
  df s = df_two_sum(a.hi, b.hi);
  const df t = df_two_sum(a.lo, b.lo);
  s.lo = LNE_FADD(s.lo, t.hi);
  s = df_fast_two_sum(s.hi, s.lo);
  s.lo = LNE_FADD(s.lo, t.lo);
  return df_fast_two_sum(s.hi, s.lo);
}
LNE_HD df df_mul(df a, df b) {
  const float p = LNE_FMUL(a.hi, b.hi);
  float e = LNE_FFMA(a.hi, b.hi, -p);
  e = LNE_FFMA(a.hi, b.lo, e);
  e = LNE_FFMA(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
LNE_HD df df_mul_f(df a, float b) {
  const float p = LNE_FMUL(a.hi, b);
  float e = LNE_FFMA(a.hi, b, -p);
  e = LNE_FFMA(a.lo, b, e);
  return df_fast_two_sum(p, e);
}

struct LogTable {
  float log_hi[128], log_lo[128];  // log(c_j) as a double-float
  float inv_hi[128], inv_lo[128];  // 1 / c_j as a double-float
};

// ln 2 = LN2_A + LN2_B + LN2_C: LN2_A = 2839/4096 carries 12 significant
// bits, so E * LN2_A is exact for |E| < 2^12; LN2_B is the float nearest to
// ln 2 - LN2_A and LN2_C the float nearest to the remainder.
#define LNE_LN2_A 6.93115234375000000e-01f
#define LNE_LN2_B 3.19461832987144589e-05f
#define LNE_LN2_C 1.64659496974806085e-12f

// Returns log(m * 2^E) as a double-float.
LNE_HD df log_df(XDouble x, const LogTable& T) {
  const int E = x.e + 52;                              // adj = (x.m / 2^52) * 2^E
  const uint32_t j = (uint32_t)((x.m >> 45) & 127u);   // top 7 fraction bits
  const uint64_t cm = (1ull << 52) | ((uint64_t)j << 45);
  const uint64_t dnum = x.m - cm;                      // < 2^45, exact
  // dnum * 2^-52 as a double-float, exactly: the high 24 bits scaled by
  // 2^-31 and the low 21 bits by 2^-52 (powers of two: exact products)
  const float dh = LNE_FMUL((float)(uint32_t)(dnum >> 21), 4.6566128730773925781250000e-10f);
  const float dl = LNE_FMUL((float)(uint32_t)(dnum & ((1u << 21) - 1)), 2.2204460492503130808472633e-16f);
  const df d = df_two_sum(dh, dl);
  const df r = df_mul(d, df{T.inv_hi[j], T.inv_lo[j]});
  // log(1+r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6 + r^7/7 ...; the tail
  // from r^4 on is below 2^-28 relative to r and is evaluated in float
  float t = LNE_FFMA(r.hi, 1.0f / 7.0f, -1.0f / 6.0f);
  t = LNE_FFMA(t, r.hi, 0.2f);
  t = LNE_FFMA(t, r.hi, -0.25f);
  // q = ((t r + 1/3) r - 1/2) r + 1, in double-float
  df q = df_add(df_mul_f(r, t), df{3.33333343267440796e-01f, -9.93410775862457740e-09f});
  q = df_add(df_mul(q, r), df{-0.5f, 0.0f});
  q = df_add(df_mul(q, r), df{1.0f, 0.0f});
  const df l1 = df_mul(q, r);
  // E ln2: E * A exact; E * B as an exact product; E * C rounded (tiny)
  const float Ef = (float)E;
  const float ea = LNE_FMUL(Ef, LNE_LN2_A);
  const float eb = LNE_FMUL(Ef, LNE_LN2_B);
  const float eb_err = LNE_FFMA(Ef, LNE_LN2_B, -eb);
  const float ec = LNE_FMUL(Ef, LNE_LN2_C);
  df el = df_fast_two_sum(ea, eb);
  el = df_add(el, df{eb_err, 0.0f});
  el = df_add(el, df{ec, 0.0f});
  df res = df_add(el, df{T.log_hi[j], T.log_lo[j]});
  res = df_add(res, l1);
  return res;
}

// Narrowed result of the reference's double log if the double-float value
// decides it, else returns false (the caller takes the slow path).  The
// margin 2^-42 relative covers the double-float error (below 2^-44
// relative: every term of the sum is positive for adj > 1) and the half-ulp
// of the double the reference rounds through.
LNE_HD bool float_of_log_fast(df L, float* out) {
  uint32_t hb;
#ifdef __CUDA_ARCH__
  hb = __float_as_uint(L.hi);
#else
  __builtin_memcpy(&hb, &L.hi, 4);
#endif
  const uint32_t expo = (hb >> 23) & 0xff;
  if ((hb & 0x7fffffu) == 0 || expo == 0 || expo >= 254) return false;  // binade edge, tiny or huge
  const float half_ulp = ldexpf(1.0f, (int)expo - 127 - 24);
  const float margin = ldexpf(fabsf(L.hi), -42);
  if (half_ulp - fabsf(L.lo) <= margin) return false;
  *out = L.hi;
  return true;
}

}  // namespace lne
