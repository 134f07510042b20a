// mls_exp.h -- exp(x) of the MLS Gaussian weights (geom.f90:24-53),
// evaluated with IEEE double operations in one fixed order, so that the
// library's device code and the CPU oracle obtain the same bits.
//
// Why not the system exp: the reference calls the Fortran runtime's exp, and
// two correct libm implementations (the host's and the device's) differ in
// the last bit for some arguments.  The reference builds its MLS moment
// matrices in absolute coordinates (mlsWeight.f90:105-108, mls_heatFlux.f90:
// 267-270), with condition numbers of 1e7 .. 1e8 at 128^3 .. 256^3, which turn
// that bit into differences of ~1e-8 in the heat-flux and load gradients.
// One exp, written out here and used on both sides, removes that noise from
// the comparison of the two implementations.
//
// Method (Cody & Waite 1980, "Software Manual for the Elementary
// Functions"): x = n ln2 + r with n = rint(x / ln2), ln2 split into a head
// of 29 significant bits (n * head is exact for |n| < 2^24) and a tail,
// |r| <= ln2 / 2 (to rounding); e^r by its Taylor polynomial of degree 13
// (truncation below 6e-18 relative) by Horner's rule, 1 + (r + r^2 q(r));
// the result is p * 2^n by exponent arithmetic.  Within 1 ulp of the true
// value for -708 <= x <= 709 (checked against the host libm); x < -745.2
// gives 0, x > 709.78 gives +inf, NaN propagates.  The Horner coefficients
// are 1/k! rounded to double.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MIBM_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define MIBM_HD inline
#endif

namespace mibm {

// round-to-nearest IEEE operations, never contracted into FMAs
MIBM_HD double mexp_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
MIBM_HD double mexp_add(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
MIBM_HD double mexp_rint(double x) {
#if defined(__CUDA_ARCH__)
  return rint(x);
#else
  return std::nearbyint(x);
#endif
}
// 2^n for -1022 <= n <= 1023
MIBM_HD double mexp_pow2(int n) {
  uint64_t b = (uint64_t)(n + 1023) << 52;
  double d;
#if defined(__CUDA_ARCH__)
  d = __longlong_as_double((long long)b);
#else
  memcpy(&d, &b, sizeof d);
#endif
  return d;
}

MIBM_HD double mls_exp(double x) {
  const double kInvLn2 = 0x1.71547652b82fep+0;      // 1/ln2 rounded
  const double kLn2Hi = 0x1.62e42ffp-1;             // ln2 to 29 significant bits
  const double kLn2Lo = -0x1.718432a1b0e26p-35;     // ln2 - kLn2Hi rounded
  if (x != x) return x;
  if (x > 709.782712893384) return mexp_mul(mexp_pow2(1023), 2.0);   // overflows to +inf
  if (x < -745.2) return 0.0;
  const double nd = mexp_rint(mexp_mul(x, kInvLn2));
  const int n = (int)nd;
  const double r = mexp_add(mexp_add(x, -mexp_mul(nd, kLn2Hi)), -mexp_mul(nd, kLn2Lo));
  // q(r) = 1/2! + r/3! + ... + r^11/13!
  double q = 1.6059043836821613e-10;                // 1/13!
  q = mexp_add(mexp_mul(q, r), 2.08767569878681e-09);      // 1/12!
  q = mexp_add(mexp_mul(q, r), 2.505210838544172e-08);     // 1/11!
  q = mexp_add(mexp_mul(q, r), 2.755731922398589e-07);     // 1/10!
  q = mexp_add(mexp_mul(q, r), 2.7557319223985893e-06);    // 1/9!
  q = mexp_add(mexp_mul(q, r), 2.48015873015873e-05);      // 1/8!
  q = mexp_add(mexp_mul(q, r), 0.0001984126984126984);     // 1/7!
  q = mexp_add(mexp_mul(q, r), 0.001388888888888889);      // 1/6!
  q = mexp_add(mexp_mul(q, r), 0.008333333333333333);      // 1/5!
  q = mexp_add(mexp_mul(q, r), 0.041666666666666664);      // 1/4!
  q = mexp_add(mexp_mul(q, r), 0.16666666666666666);       // 1/3!
  q = mexp_add(mexp_mul(q, r), 0.5);                       // 1/2!
  const double p = mexp_add(1.0, mexp_add(r, mexp_mul(mexp_mul(r, r), q)));
  if (n >= -1022) return mexp_mul(p, mexp_pow2(n));
  // subnormal results: two exact-until-the-last scalings
  return mexp_mul(mexp_mul(p, mexp_pow2(n + 600)), mexp_pow2(-600));
}

}  // namespace mibm

#undef MIBM_HD
