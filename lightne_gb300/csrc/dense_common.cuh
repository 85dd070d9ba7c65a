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
