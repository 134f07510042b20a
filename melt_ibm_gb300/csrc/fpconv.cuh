// fpconv.cuh -- IEEE 754 binary64 <-> binary32 conversions on the integer
// pipe.
//
// On this part an FP64<->FP32 conversion instruction issues at the FP64 rate
// (2 per clock per SM), like an FP64 FMA, while integer operations issue at
// 64 per clock per SM.  The precision form converts every FP32 increment it
// adds to an FP64 field and every updated field back to its FP32 mirror, so
// these conversions, written with integer operations on the bit patterns,
// take most of its FP64 issue off that pipe.  Both follow IEEE 754:
//   f2d_bits: exact widening (normal and subnormal inputs, signed zeros,
//             infinities; NaN stays NaN with its payload shifted up);
//   d2f_bits: round to nearest, ties to even, with gradual underflow to
//             subnormals and overflow to infinity; NaN stays a quiet NaN.
// mibm_selftest_ checks both, bit for bit, against the hardware conversions
// on edge cases and on random bit patterns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mibm {

__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t m = u & 0x7fffffu;
  uint64_t r;
  if (e - 1u < 254u) {                       // normal: rebias the exponent (127 -> 1023)
    r = sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
  } else if (e == 255u) {                    // infinity or NaN
    r = sign | 0x7ff0000000000000ull | ((uint64_t)m << 29);
  } else if (m == 0u) {                      // signed zero
    r = sign;
  } else {                                   // subnormal float: normalise (value m * 2^-149)
    const int p = 31 - __clz(m);             // leading bit, 0..22
    const uint64_t mm = ((uint64_t)m << (52 - p)) & 0x000fffffffffffffull;
    r = sign | ((uint64_t)(p + 874) << 52) | mm;
  }
  return __longlong_as_double((long long)r);
}

__device__ __forceinline__ float d2f_bits(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu);
  const uint64_t m = b & 0x000fffffffffffffull;
  if (e == 0x7ff)                            // infinity, or a quiet NaN keeping the top payload bits
    return __uint_as_float(sign | 0x7f800000u | (m ? 0x00400000u | (uint32_t)(m >> 29) : 0u));
  const int ef = e - 1023 + 127;             // biased float exponent
  if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);   // beyond the float range: infinity
  if (ef >= 1) {                             // normal result (rounding may carry into the exponent)
    const uint32_t q = (uint32_t)(m >> 29);
    const uint32_t rem = (uint32_t)(m & 0x1fffffffu);
    const uint32_t up = (rem > 0x10000000u) | ((rem == 0x10000000u) & (q & 1u));
    return __uint_as_float(sign | (((uint32_t)ef << 23) + q + up));
  }
  // subnormal or zero result: the 53-bit significand (0 for a double zero or
  // subnormal, which all round to a signed zero here) shifted right by 29 + 1 - ef
  const int sh = 30 - ef;                    // >= 30
  if (e == 0 || sh > 54) return __uint_as_float(sign);
  const uint64_t M = m | 0x0010000000000000ull;
  const uint32_t q = (uint32_t)(M >> sh);
  const uint64_t rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  const uint32_t up = (rem > half) | ((rem == half) & (q & 1u));
  return __uint_as_float(sign | (q + up));   // q + up == 2^23 is the smallest normal
}

// the compute type R of a templated kernel from / to FP64 (identity for FP64)
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f2d_bits(x); }
template <typename R> __device__ __forceinline__ R narrow(double x);
template <> __device__ __forceinline__ double narrow<double>(double x) { return x; }
template <> __device__ __forceinline__ float narrow<float>(double x) { return d2f_bits(x); }

}  // namespace mibm
