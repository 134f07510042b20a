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

// ---------------------------------------------------------------------
// Sums of FP64 values on the integer pipe: (a1 - a0) + (b1 - b0) + (c1 - c0)
// (sum3_diff_*), a + b + c + d + e + f (sum6_*), |a1 + a0| + |b1 + b0| +
// |c1 + c0| (sum3_abs_pair_f64) and |a| + |b| + |c| (sum3_abs_f64), rounded
// once to FP32 or FP64.  Each value's 53-bit significand is shifted right to the weight of
// the last bit of the largest input (exponent E), given its sign, and the
// six are summed in 64-bit integers (|sum| < 2^56); the sum is rounded to
// nearest, ties to even.  The shifts drop bits below that weight only, so
// the result is within 6 * 2^-52 times the largest |input| of the exact sum
// before its rounding (FP64 arithmetic: within about 8 * 2^-52), and it is
// the correctly rounded exact sum when every input is a multiple of that
// weight (zeros and subnormals included; in the difference form a zero or a
// subnormal counts as a value below 2^-1021 unless it cancels); a sum below
// the normal range of the result type is flushed to a signed zero, one above
// it is infinity; an infinite or NaN input gives NaN.  FP64 instructions issue at 1/32 of the integer rate on
// this part, so a stencil that only adds and subtracts FP64 neighbours is
// cheaper this way.
// ---------------------------------------------------------------------
// the exponent field; EXACT0: 1 for zero and subnormals (their weight)
template <bool EXACT0 = true>
__device__ __forceinline__ int fx_exp(double x) {
  const int e = (int)(((uint32_t)((uint64_t)__double_as_longlong(x) >> 32) >> 20) & 0x7ffu);
  if constexpr (EXACT0) return e > 0 ? e : 1;
  return e;
}

// x's significand shifted right by sh >= 0, signed.  EXACT0: the implicit
// bit for normal x only; otherwise for every x, which takes a zero or a
// subnormal as a value below 2^-1021 -- exact enough where such inputs come
// in pairs that cancel or beside normal values that shift them out (the
// difference forms), and two operations cheaper
template <bool EXACT0 = true>
__device__ __forceinline__ int64_t fx_aligned(double x, int sh) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  uint64_t m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
  if constexpr (EXACT0) m = (b & 0x7ff0000000000000ull) ? m : (b & 0x000fffffffffffffull);
  const uint64_t s = (uint64_t)((int64_t)b >> 63);           // 0 or all ones
  return (int64_t)(((m >> (sh < 63 ? sh : 63)) ^ s) - s);
}

// |S| normalised (leading one at bit 63) with its sign and leading-zero count
__device__ __forceinline__ uint64_t fx_norm(int64_t S, uint64_t& sign, int& lz) {
  const uint64_t s = (uint64_t)(S >> 63);
  const uint64_t A0 = ((uint64_t)S ^ s) - s;
  sign = s & 0x8000000000000000ull;
  lz = __clzll((long long)A0);
  return A0 << lz;
}

// S * 2^(E - 1075) to FP32, round to nearest even (E == 0x7ff: NaN)
__device__ __forceinline__ float fx_round_f32(int64_t S, int E) {
  if (E == 0x7ff) return __uint_as_float(0x7fc00000u);
  if (S == 0) return 0.0f;
  uint64_t sg;
  int lz;
  const uint64_t A = fx_norm(S, sg, lz);
  const uint32_t sign = (uint32_t)(sg >> 32);
  uint32_t q = (uint32_t)(A >> 40);                          // 24 significant bits
  const uint32_t r = (uint32_t)(A >> 39) & 1u, sticky = (uint32_t)((A & 0x7fffffffffull) != 0);
  q += r & (sticky | (q & 1u));
  const int ef = 63 - lz + E - 1075 + 127;                   // biased exponent of the leading one
  if (ef <= 0) return __uint_as_float(sign);
  if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
  const uint32_t bits = ((uint32_t)ef << 23) + (q - 0x800000u);   // a carry of q moves into the exponent
  return __uint_as_float(sign | (bits >= 0x7f800000u ? 0x7f800000u : bits));
}

// S * 2^(E - 1075) to FP64, round to nearest even (E == 0x7ff: NaN)
__device__ __forceinline__ double fx_round_f64(int64_t S, int E) {
  if (E == 0x7ff) return __longlong_as_double(0x7ff8000000000000ll);
  if (S == 0) return 0.0;
  uint64_t sign;
  int lz;
  const uint64_t A = fx_norm(S, sign, lz);
  uint64_t q = A >> 11;                                      // 53 significant bits
  const uint64_t r = (A >> 10) & 1u, sticky = (uint64_t)((A & 0x3ffull) != 0);
  q += r & (sticky | (q & 1u));
  const int ef = 63 - lz + E - 1075 + 1023;                  // biased exponent of the leading one
  if (ef <= 0) return __longlong_as_double((long long)sign);
  if (ef >= 2047) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull));
  const uint64_t bits = ((uint64_t)ef << 52) + (q - 0x0010000000000000ull);
  return __longlong_as_double((long long)(sign | (bits >= 0x7ff0000000000000ull ? 0x7ff0000000000000ull : bits)));
}

__device__ __forceinline__ int fx_max6(int a, int b, int c, int d, int e, int f) {
  return max(max(max(a, b), max(c, d)), max(e, f));
}

// the difference form: equal inputs cancel exactly whatever their decoding,
// so zeros take the cheaper one
__device__ __forceinline__ int64_t fx_sum3_diff(double a1, double a0, double b1, double b0, double c1, double c0,
                                                int& E) {
  const int ea1 = fx_exp<false>(a1), ea0 = fx_exp<false>(a0), eb1 = fx_exp<false>(b1), eb0 = fx_exp<false>(b0),
            ec1 = fx_exp<false>(c1), ec0 = fx_exp<false>(c0);
  E = fx_max6(ea1, ea0, eb1, eb0, ec1, ec0);
  return (fx_aligned<false>(a1, E - ea1) - fx_aligned<false>(a0, E - ea0)) +
         (fx_aligned<false>(b1, E - eb1) - fx_aligned<false>(b0, E - eb0)) +
         (fx_aligned<false>(c1, E - ec1) - fx_aligned<false>(c0, E - ec0));
}

__device__ __forceinline__ int64_t fx_sum6(double a, double b, double c, double d, double e, double f, int& E) {
  const int ea = fx_exp(a), eb = fx_exp(b), ec = fx_exp(c), ed = fx_exp(d), ee = fx_exp(e), ef = fx_exp(f);
  E = fx_max6(ea, eb, ec, ed, ee, ef);
  return (fx_aligned(a, E - ea) + fx_aligned(b, E - eb)) + (fx_aligned(c, E - ec) + fx_aligned(d, E - ed)) +
         (fx_aligned(e, E - ee) + fx_aligned(f, E - ef));
}

// |a1 + a0| + |b1 + b0| + |c1 + c0| (each pair summed exactly, then its
// magnitude), rounded once to FP64
__device__ __forceinline__ double sum3_abs_pair_f64(double a1, double a0, double b1, double b0, double c1,
                                                    double c0) {
  const int ea1 = fx_exp(a1), ea0 = fx_exp(a0), eb1 = fx_exp(b1), eb0 = fx_exp(b0), ec1 = fx_exp(c1),
            ec0 = fx_exp(c0);
  const int E = fx_max6(ea1, ea0, eb1, eb0, ec1, ec0);
  int64_t sa = fx_aligned(a1, E - ea1) + fx_aligned(a0, E - ea0);
  int64_t sb = fx_aligned(b1, E - eb1) + fx_aligned(b0, E - eb0);
  int64_t sc = fx_aligned(c1, E - ec1) + fx_aligned(c0, E - ec0);
  sa = sa < 0 ? -sa : sa;
  sb = sb < 0 ? -sb : sb;
  sc = sc < 0 ? -sc : sc;
  return fx_round_f64(sa + sb + sc, E);
}

// |a| + |b| + |c|, rounded once to FP64
__device__ __forceinline__ double sum3_abs_f64(double a, double b, double c) {
  const double x = __longlong_as_double(__double_as_longlong(a) & 0x7fffffffffffffffll);
  const double y = __longlong_as_double(__double_as_longlong(b) & 0x7fffffffffffffffll);
  const double z = __longlong_as_double(__double_as_longlong(c) & 0x7fffffffffffffffll);
  const int ex = fx_exp(x), ey = fx_exp(y), ez = fx_exp(z);
  const int E = max(max(ex, ey), ez);
  return fx_round_f64(fx_aligned(x, E - ex) + fx_aligned(y, E - ey) + fx_aligned(z, E - ez), E);
}

__device__ __forceinline__ float sum3_diff_f32(double a1, double a0, double b1, double b0, double c1, double c0) {
  int E;
  const int64_t S = fx_sum3_diff(a1, a0, b1, b0, c1, c0, E);
  return fx_round_f32(S, E);
}

__device__ __forceinline__ double sum3_diff_f64(double a1, double a0, double b1, double b0, double c1, double c0) {
  int E;
  const int64_t S = fx_sum3_diff(a1, a0, b1, b0, c1, c0, E);
  return fx_round_f64(S, E);
}

__device__ __forceinline__ double sum6_f64(double a, double b, double c, double d, double e, double f) {
  int E;
  const int64_t S = fx_sum6(a, b, c, d, e, f, E);
  return fx_round_f64(S, E);
}

// the compute type R of a templated kernel from / to FP64 (identity for FP64)
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f2d_bits(x); }
template <typename R> __device__ __forceinline__ R narrow(double x);
template <> __device__ __forceinline__ double narrow<double>(double x) { return x; }
template <> __device__ __forceinline__ float narrow<float>(double x) { return d2f_bits(x); }

}  // namespace mibm
