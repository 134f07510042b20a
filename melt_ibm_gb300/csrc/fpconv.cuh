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
//
// Every function here also compiles as plain host C++ (g++, no CUDA), so that
// the CPU tests check the same source against exact rational arithmetic.
#pragma once

#include <stdint.h>

#include <cstring>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define FPC_FN __host__ __device__ __forceinline__
#else
#define FPC_FN inline
#endif

namespace mibm {

// bit casts, leading zeros and an integer maximum for both compilations
namespace fpc {
FPC_FN uint64_t bits64(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}
FPC_FN double from64(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}
FPC_FN uint32_t bits32(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}
FPC_FN float from32(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}
FPC_FN int clz32(uint32_t x) {   // x != 0
#if defined(__CUDA_ARCH__)
  return __clz((int)x);
#else
  return __builtin_clz(x);
#endif
}
FPC_FN int clz64(uint64_t x) {   // x != 0
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}
FPC_FN int imax(int a, int b) { return a > b ? a : b; }
}  // namespace fpc

FPC_FN double f2d_bits(float f) {
  const uint32_t u = fpc::bits32(f);
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
    const int p = 31 - fpc::clz32(m);        // leading bit, 0..22
    const uint64_t mm = ((uint64_t)m << (52 - p)) & 0x000fffffffffffffull;
    r = sign | ((uint64_t)(p + 874) << 52) | mm;
  }
  return fpc::from64(r);
}

FPC_FN float d2f_bits(double d) {
  const uint64_t b = fpc::bits64(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu);
  const uint64_t m = b & 0x000fffffffffffffull;
  if (e == 0x7ff)                            // infinity, or a quiet NaN keeping the top payload bits
    return fpc::from32(sign | 0x7f800000u | (m ? 0x00400000u | (uint32_t)(m >> 29) : 0u));
  const int ef = e - 1023 + 127;             // biased float exponent
  if (ef >= 255) return fpc::from32(sign | 0x7f800000u);   // beyond the float range: infinity
  if (ef >= 1) {                             // normal result (rounding may carry into the exponent)
    const uint32_t q = (uint32_t)(m >> 29);
    const uint32_t rem = (uint32_t)(m & 0x1fffffffu);
    const uint32_t up = (rem > 0x10000000u) | ((rem == 0x10000000u) & (q & 1u));
    return fpc::from32(sign | (((uint32_t)ef << 23) + q + up));
  }
  // subnormal or zero result: the 53-bit significand (0 for a double zero or
  // subnormal, which all round to a signed zero here) shifted right by 29 + 1 - ef
  const int sh = 30 - ef;                    // >= 30
  if (e == 0 || sh > 54) return fpc::from32(sign);
  const uint64_t M = m | 0x0010000000000000ull;
  const uint32_t q = (uint32_t)(M >> sh);
  const uint64_t rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  const uint32_t up = (rem > half) | ((rem == half) & (q & 1u));
  return fpc::from32(sign | (q + up));   // q + up == 2^23 is the smallest normal
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
// weight (zeros of either sign and subnormals included); a sum below the
// normal range of the result type is flushed to a signed zero, one above it
// is infinity; an infinite or NaN input gives NaN.  FP64 instructions issue at 1/32 of the integer rate on
// this part, so a stencil that only adds and subtracts FP64 neighbours is
// cheaper this way.
// ---------------------------------------------------------------------
// the exponent field, 1 for zero and subnormals (their weight)
FPC_FN int fx_exp(double x) {
  const int e = (int)(((uint32_t)(fpc::bits64(x) >> 32) >> 20) & 0x7ffu);
  return e > 0 ? e : 1;
}

// x's significand (the implicit bit for normal x only) shifted right by
// sh >= 0, signed; zeros of either sign give 0
FPC_FN int64_t fx_aligned(double x, int sh) {
  const uint64_t b = fpc::bits64(x);
  const uint64_t m = (b & 0x000fffffffffffffull) | ((b & 0x7ff0000000000000ull) ? 0x0010000000000000ull : 0ull);
  const uint64_t s = (uint64_t)((int64_t)b >> 63);           // 0 or all ones
  return (int64_t)(((m >> (sh < 63 ? sh : 63)) ^ s) - s);
}

// |S| normalised (leading one at bit 63) with its sign and leading-zero count
FPC_FN uint64_t fx_norm(int64_t S, uint64_t& sign, int& lz) {
  const uint64_t s = (uint64_t)(S >> 63);
  const uint64_t A0 = ((uint64_t)S ^ s) - s;
  sign = s & 0x8000000000000000ull;
  lz = fpc::clz64(A0);
  return A0 << lz;
}

// S * 2^(E - 1075) to FP32, round to nearest even (E == 0x7ff: NaN)
FPC_FN float fx_round_f32(int64_t S, int E) {
  if (E == 0x7ff) return fpc::from32(0x7fc00000u);
  if (S == 0) return 0.0f;
  uint64_t sg;
  int lz;
  const uint64_t A = fx_norm(S, sg, lz);
  const uint32_t sign = (uint32_t)(sg >> 32);
  uint32_t q = (uint32_t)(A >> 40);                          // 24 significant bits
  const uint32_t r = (uint32_t)(A >> 39) & 1u, sticky = (uint32_t)((A & 0x7fffffffffull) != 0);
  q += r & (sticky | (q & 1u));
  const int ef = 63 - lz + E - 1075 + 127;                   // biased exponent of the leading one
  if (ef <= 0) return fpc::from32(sign);
  if (ef >= 255) return fpc::from32(sign | 0x7f800000u);
  const uint32_t bits = ((uint32_t)ef << 23) + (q - 0x800000u);   // a carry of q moves into the exponent
  return fpc::from32(sign | (bits >= 0x7f800000u ? 0x7f800000u : bits));
}

// S * 2^(E - 1075) to FP64, round to nearest even (E == 0x7ff: NaN)
FPC_FN double fx_round_f64(int64_t S, int E) {
  if (E == 0x7ff) return fpc::from64(0x7ff8000000000000ull);
  if (S == 0) return 0.0;
  uint64_t sign;
  int lz;
  const uint64_t A = fx_norm(S, sign, lz);
  uint64_t q = A >> 11;                                      // 53 significant bits
  const uint64_t r = (A >> 10) & 1u, sticky = (uint64_t)((A & 0x3ffull) != 0);
  q += r & (sticky | (q & 1u));
  const int ef = 63 - lz + E - 1075 + 1023;                  // biased exponent of the leading one
  if (ef <= 0) return fpc::from64(sign);
  if (ef >= 2047) return fpc::from64(sign | 0x7ff0000000000000ull);
  const uint64_t bits = ((uint64_t)ef << 52) + (q - 0x0010000000000000ull);
  return fpc::from64(sign | (bits >= 0x7ff0000000000000ull ? 0x7ff0000000000000ull : bits));
}

FPC_FN int fx_max6(int a, int b, int c, int d, int e, int f) {
  return fpc::imax(fpc::imax(fpc::imax(a, b), fpc::imax(c, d)), fpc::imax(e, f));
}

FPC_FN int64_t fx_sum3_diff(double a1, double a0, double b1, double b0, double c1, double c0, int& E) {
  const int ea1 = fx_exp(a1), ea0 = fx_exp(a0), eb1 = fx_exp(b1), eb0 = fx_exp(b0), ec1 = fx_exp(c1),
            ec0 = fx_exp(c0);
  E = fx_max6(ea1, ea0, eb1, eb0, ec1, ec0);
  return (fx_aligned(a1, E - ea1) - fx_aligned(a0, E - ea0)) + (fx_aligned(b1, E - eb1) - fx_aligned(b0, E - eb0)) +
         (fx_aligned(c1, E - ec1) - fx_aligned(c0, E - ec0));
}

FPC_FN int64_t fx_sum6(double a, double b, double c, double d, double e, double f, int& E) {
  const int ea = fx_exp(a), eb = fx_exp(b), ec = fx_exp(c), ed = fx_exp(d), ee = fx_exp(e), ef = fx_exp(f);
  E = fx_max6(ea, eb, ec, ed, ee, ef);
  return (fx_aligned(a, E - ea) + fx_aligned(b, E - eb)) + (fx_aligned(c, E - ec) + fx_aligned(d, E - ed)) +
         (fx_aligned(e, E - ee) + fx_aligned(f, E - ef));
}

// |a1 + a0| + |b1 + b0| + |c1 + c0| (each pair summed exactly, then its
// magnitude), rounded once to FP64
FPC_FN double sum3_abs_pair_f64(double a1, double a0, double b1, double b0, double c1,
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
FPC_FN double sum3_abs_f64(double a, double b, double c) {
  const double x = fpc::from64(fpc::bits64(a) & 0x7fffffffffffffffull);
  const double y = fpc::from64(fpc::bits64(b) & 0x7fffffffffffffffull);
  const double z = fpc::from64(fpc::bits64(c) & 0x7fffffffffffffffull);
  const int ex = fx_exp(x), ey = fx_exp(y), ez = fx_exp(z);
  const int E = fpc::imax(fpc::imax(ex, ey), ez);
  return fx_round_f64(fx_aligned(x, E - ex) + fx_aligned(y, E - ey) + fx_aligned(z, E - ez), E);
}

FPC_FN float sum3_diff_f32(double a1, double a0, double b1, double b0, double c1, double c0) {
  int E;
  const int64_t S = fx_sum3_diff(a1, a0, b1, b0, c1, c0, E);
  return fx_round_f32(S, E);
}

FPC_FN double sum3_diff_f64(double a1, double a0, double b1, double b0, double c1, double c0) {
  int E;
  const int64_t S = fx_sum3_diff(a1, a0, b1, b0, c1, c0, E);
  return fx_round_f64(S, E);
}

FPC_FN double sum6_f64(double a, double b, double c, double d, double e, double f) {
  int E;
  const int64_t S = fx_sum6(a, b, c, d, e, f, E);
  return fx_round_f64(S, E);
}

// the compute type R of a templated kernel from / to FP64 (identity for FP64)
FPC_FN double widen(double x) { return x; }
FPC_FN double widen(float x) { return f2d_bits(x); }
template <typename R> FPC_FN R narrow(double x);
template <> FPC_FN double narrow<double>(double x) { return x; }
template <> FPC_FN float narrow<float>(double x) { return d2f_bits(x); }

}  // namespace mibm
