// Dense-operand helpers shared by the SpMM, propagation and dense kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lne {

// A 16-byte vector of the dense operand, widened to float.
template <typename T>
struct Vec16;

template <>
struct Vec16<float> {
  static constexpr int E = 4;  // elements per 16 B
  __device__ __forceinline__ static void load(const float* p, float (&o)[4]) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  __device__ __forceinline__ static void load_cg(const float* p, float (&o)[4]) {
    const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  __device__ __forceinline__ static void store(float* p, const float (&o)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
  }
};

template <>
struct Vec16<__nv_bfloat16> {
  static constexpr int E = 8;
  __device__ __forceinline__ static void unpack(const uint4 v, float (&o)[8]) {
    o[0] = __uint_as_float(v.x << 16); o[1] = __uint_as_float(v.x & 0xffff0000u);
    o[2] = __uint_as_float(v.y << 16); o[3] = __uint_as_float(v.y & 0xffff0000u);
    o[4] = __uint_as_float(v.z << 16); o[5] = __uint_as_float(v.z & 0xffff0000u);
    o[6] = __uint_as_float(v.w << 16); o[7] = __uint_as_float(v.w & 0xffff0000u);
  }
  __device__ __forceinline__ static void load(const __nv_bfloat16* p, float (&o)[8]) {
    unpack(__ldg(reinterpret_cast<const uint4*>(p)), o);
  }
  __device__ __forceinline__ static void load_cg(const __nv_bfloat16* p, float (&o)[8]) {
    unpack(__ldcg(reinterpret_cast<const uint4*>(p)), o);
  }
  __device__ __forceinline__ static uint32_t pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half)
    return *reinterpret_cast<const uint32_t*>(&h);
  }
  __device__ __forceinline__ static void store(__nv_bfloat16* p, const float (&o)[8]) {
    uint4 v;
    v.x = pack2(o[0], o[1]); v.y = pack2(o[2], o[3]); v.z = pack2(o[4], o[5]); v.w = pack2(o[6], o[7]);
    *reinterpret_cast<uint4*>(p) = v;
  }
};

// FP16 operand: 8 elements per 16 bytes.  FP16 keeps 11 significant bits
// (BF16: 8) in the same two bytes; callers scale by a power of two so that
// the values sit in its normal range (an exact, invertible scaling).
template <>
struct Vec16<__half> {
  static constexpr int E = 8;
  __device__ __forceinline__ static void unpack(const uint4 v, float (&o)[8]) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w[i]));
      o[2 * i] = f.x;
      o[2 * i + 1] = f.y;
    }
  }
  __device__ __forceinline__ static void load(const __half* p, float (&o)[8]) {
    unpack(__ldg(reinterpret_cast<const uint4*>(p)), o);
  }
  __device__ __forceinline__ static void load_cg(const __half* p, float (&o)[8]) {
    unpack(__ldcg(reinterpret_cast<const uint4*>(p)), o);
  }
  __device__ __forceinline__ static uint32_t pack2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);  // .x = a (low half)
    return *reinterpret_cast<const uint32_t*>(&h);
  }
  __device__ __forceinline__ static void store(__half* p, const float (&o)[8]) {
    uint4 v;
    v.x = pack2(o[0], o[1]); v.y = pack2(o[2], o[3]); v.z = pack2(o[4], o[5]); v.w = pack2(o[6], o[7]);
    *reinterpret_cast<uint4*>(p) = v;
  }
};

// Two elements of a 16-bit copy (BF16 or FP16), round to nearest.
template <typename H>
__device__ __forceinline__ uint32_t pack2_16(float a, float b);
template <>
__device__ __forceinline__ uint32_t pack2_16<__nv_bfloat16>(float a, float b) {
  return Vec16<__nv_bfloat16>::pack2(a, b);
}
template <>
__device__ __forceinline__ uint32_t pack2_16<__half>(float a, float b) {
  return Vec16<__half>::pack2(a, b);
}

// A 16-bit copy written beside an FP32 result: kind 0 none, 1 BF16, 2 FP16;
// the copy holds scale * value (scale a power of two, 1 for BF16).
struct Copy16 {
  void* p = nullptr;
  int kind = 0;
  float scale = 1.0f;
};

// One element of the copy at index idx.
__device__ __forceinline__ void copy16_put(const Copy16& c, int64_t idx, float v) {
  if (c.kind == 1)
    reinterpret_cast<__nv_bfloat16*>(c.p)[idx] = __float2bfloat16_rn(v);
  else if (c.kind == 2)
    reinterpret_cast<__half*>(c.p)[idx] = __float2half_rn(v * c.scale);
}

// Elements [col0, col0 + 16) of row `row` (leading dimension ld), of which
// the first `valid` are in the row: 16-byte stores where ld is a multiple
// of 8 and the copy is 16-byte aligned, element stores otherwise.
__device__ __forceinline__ void copy16_put_row16(const Copy16& c, int64_t row, int64_t ld, int col0,
                                                 const float (&v)[16], int valid) {
  if (c.kind == 0) return;
  const int64_t base = row * ld + col0;
  const bool vec = (ld & 7) == 0 && (col0 & 7) == 0 && ((reinterpret_cast<uintptr_t>(c.p) & 15) == 0);
  if (vec) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (8 * h + 8 > valid) break;
      uint4 q;
      if (c.kind == 1) {
        q.x = pack2_16<__nv_bfloat16>(v[8 * h], v[8 * h + 1]);
        q.y = pack2_16<__nv_bfloat16>(v[8 * h + 2], v[8 * h + 3]);
        q.z = pack2_16<__nv_bfloat16>(v[8 * h + 4], v[8 * h + 5]);
        q.w = pack2_16<__nv_bfloat16>(v[8 * h + 6], v[8 * h + 7]);
      } else {
        const float s = c.scale;
        q.x = pack2_16<__half>(s * v[8 * h], s * v[8 * h + 1]);
        q.y = pack2_16<__half>(s * v[8 * h + 2], s * v[8 * h + 3]);
        q.z = pack2_16<__half>(s * v[8 * h + 4], s * v[8 * h + 5]);
        q.w = pack2_16<__half>(s * v[8 * h + 6], s * v[8 * h + 7]);
      }
      *reinterpret_cast<uint4*>(reinterpret_cast<uint16_t*>(c.p) + base + 8 * h) = q;
    }
    if ((valid & 7) == 0) return;
    for (int i = valid & ~7; i < valid && i < 16; ++i) copy16_put(c, base + i, v[i]);
    return;
  }
  for (int i = 0; i < valid && i < 16; ++i) copy16_put(c, base + i, v[i]);
}

// FP8 (e4m3) operand: 16 elements per 16 bytes, widened exactly to float
// (every e4m3 value is a half), two at a time.  Read-only (the sketch).
template <>
struct Vec16<__nv_fp8_e4m3> {
  static constexpr int E = 16;
  __device__ __forceinline__ static void unpack(const uint4 v, float (&o)[16]) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const __half2_raw r = __nv_cvt_fp8x2_to_halfraw2((__nv_fp8x2_storage_t)(w[i] >> (16 * h)), __NV_E4M3);
        const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&r));
        o[4 * i + 2 * h] = f.x;
        o[4 * i + 2 * h + 1] = f.y;
      }
  }
  __device__ __forceinline__ static void load(const __nv_fp8_e4m3* p, float (&o)[16]) {
    unpack(__ldg(reinterpret_cast<const uint4*>(p)), o);
  }
  __device__ __forceinline__ static void load_cg(const __nv_fp8_e4m3* p, float (&o)[16]) {
    unpack(__ldcg(reinterpret_cast<const uint4*>(p)), o);
  }
};

// Padded leading dimension: rows of the dense operands start on 16-byte
// boundaries and hold a whole number of 16-byte vectors for both FP32 and
// BF16 copies (multiple of 8 elements).
__host__ __device__ __forceinline__ int64_t pad_ld(int64_t d) { return (d + 7) / 8 * 8; }

}  // namespace lne

namespace lne {
// Leading dimension of an FP8 copy: rows of 16-byte multiples.
__host__ __device__ __forceinline__ int64_t pad_ld_fp8(int64_t d) { return (d + 15) / 16 * 16; }
}  // namespace lne
