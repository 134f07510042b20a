// selftest.cu -- mibm_selftest_: device checks of the library's own
// arithmetic helpers against the hardware.  The integer-pipe conversions of
// fpconv.cuh must equal the conversion instructions bit for bit (NaN: any
// NaN) on edge cases (signed zeros, subnormals of both formats, the float
// range limits, ties at every rounding boundary, infinities, NaNs) and on
// random bit patterns.  The line-solve factor table evaluated on the device
// (the allocation-free x-line solve builds it there) must equal the host's
// evaluation bit for bit.  The written-out exp of the MLS weights (mls_exp.h)
// must give the host's bits on the device.  The integer-pipe sums of FP64
// values (sum3_diff_f32/f64, sum6_f64, sum3_abs_pair_f64, sum3_abs_f64) must give FP64 arithmetic's bits
// where that is exact, and agree with it to their error bound elsewhere.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fpconv.cuh"
#include "mls_exp.h"

namespace mibm {

// splitmix64 of the thread's index: random bit patterns without host data
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z + 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ bool same_f(float a, float b) {
  return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}
__device__ __forceinline__ bool same_d(double a, double b) {
  return (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
}

// edge[] then n_random random patterns; bad[0] counts d2f mismatches, bad[1]
// f2d mismatches, bad[2..3] keep the first failing input bits
__global__ void conv_selftest_kernel(const unsigned long long* __restrict__ edge, int n_edge, long long n_random,
                                     unsigned long long* __restrict__ bad) {
  const long long n = n_edge + n_random;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    uint64_t bits;
    if (t < n_edge) bits = edge[t];
    else {
      bits = mix64((uint64_t)t);
      // half of the random doubles near the float range, where rounding is exercised
      if (t & 1) bits = (bits & 0x800fffffffffffffull) | ((uint64_t)(0x340 + (bits >> 52) % 0x140) << 52);
    }
    const double d = __longlong_as_double((long long)bits);
    if (!same_f(d2f_bits(d), (float)d)) {
      if (atomicAdd(&bad[0], 1ull) == 0) bad[2] = bits;
    }
    const float f = __uint_as_float((uint32_t)(bits >> 16));
    if (!same_d(f2d_bits(f), (double)f)) {
      if (atomicAdd(&bad[1], 1ull) == 0) bad[3] = (uint32_t)(bits >> 16);
    }
  }
}

static void edge_cases(std::vector<unsigned long long>& v) {
  auto d = [&](double x) { unsigned long long b; memcpy(&b, &x, 8); v.push_back(b); };
  auto f = [&](uint32_t fb) {          // a float pattern, placed so that (bits >> 16) is it
    unsigned long long b = (unsigned long long)fb << 16;
    v.push_back(b);
  };
  const double specials[] = {0.0, -0.0, 1.0, -1.0, 0.5, 3.0, 1e-300, -1e-300, 1e300, -1e300,
                             3.4028234663852886e38, 3.4028235677973366e38, 3.4028235677973362e38,
                             3.402823567797337e38, 1.1754943508222875e-38, 1.1754942106924411e-38,
                             1.401298464324817e-45, 7.006492321624085e-46, 7.006492321624087e-46,
                             2.1019476964872256e-45, 1e-45, 1e-46, 4.9e-324, 2.2250738585072014e-308};
  for (double x : specials) { d(x); d(-x); }
  const unsigned long long raw[] = {0x7ff0000000000000ull, 0xfff0000000000000ull, 0x7ff8000000000000ull,
                                    0x7ff0000000000001ull, 0xfff8000000000123ull, 0x000fffffffffffffull,
                                    0x0000000000000001ull, 0x3ff0000010000000ull, 0x3ff0000030000000ull,
                                    0x3ff0000010000001ull, 0x3ff000000fffffffull, 0x47efffffefffffffull,
                                    0x47effffff0000000ull, 0x380fffffffffffffull, 0x36a0000000000000ull,
                                    0x3690000000000000ull, 0x3690000000000001ull};
  for (unsigned long long b : raw) { v.push_back(b); v.push_back(b ^ 0x8000000000000000ull); }
  // ties and neighbours at every float exponent, normal and subnormal
  for (int e = 0x340; e < 0x480; ++e)
    for (unsigned long long low : {0x10000000ull, 0x30000000ull, 0x0fffffffull, 0x10000001ull, 0x1fffffffull})
      v.push_back(((unsigned long long)e << 52) | (0x5555500000000ull & ~0x1fffffffull) | low);
  const uint32_t fr[] = {0x00000000u, 0x80000000u, 0x00000001u, 0x007fffffu, 0x00400000u, 0x00800000u,
                         0x7f7fffffu, 0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f800001u, 0x3f800000u,
                         0x80000001u, 0x807fffffu, 0x00000100u, 0x00012345u};
  for (uint32_t x : fr) f(x);
}

// sum3_diff_f32, sum3_diff_f64, sum6_f64, sum3_abs_pair_f64 and sum3_abs_f64
// against FP64 arithmetic on n random sextuples.  Even t: k * 2^s with |k| < 2^50 and one s per
// sextuple, where FP64 arithmetic is exact, so both must give the same bits;
// odd t: values of random sign and exponent spread over 2^-40 .. 2^40,
// within 2^-48 (FP32: plus two units of the result) or 2^-47 (FP64) of the
// largest |input|.  bad[0] counts failures, bad[1] keeps
// the first t.
__global__ void sum3_selftest_kernel(long long n, unsigned long long* __restrict__ bad) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    double x[6];
    const uint64_t r0 = mix64((uint64_t)t * 7u + 1u);
    const int s = (int)(r0 % 81u) - 60;
    double amax = 0.0;
    for (int q = 0; q < 6; ++q) {
      const uint64_t r = mix64((uint64_t)t * 7u + 2u + (uint64_t)q);
      if ((t & 1) == 0) {
        const int64_t k = (int64_t)(r >> 14) - (int64_t)(1ll << 49);            // |k| < 2^50
        x[q] = ldexp((double)(k >> (r & 31)), s);                                 // spread the magnitudes
      } else {
        const double m = 1.0 + (double)(r >> 12) * 0x1.0p-52;
        x[q] = ldexp((r & 1) ? -m : m, (int)((r >> 1) % 81u) - 40);
      }
      amax = fmax(amax, fabs(x[q]));
    }
    if ((t & 7) == 3) x[1] = x[0];                                               // exact cancellations
    if ((t & 15) == 5) { x[3] = x[2]; x[5] = x[4]; }
    const float got = sum3_diff_f32(x[0], x[1], x[2], x[3], x[4], x[5]);
    const double got64 = sum3_diff_f64(x[0], x[1], x[2], x[3], x[4], x[5]);
    const double six64 = sum6_f64(x[0], x[1], x[2], x[3], x[4], x[5]);
    const double fp = ((x[0] - x[1]) + (x[2] - x[3])) + (x[4] - x[5]);
    const double fp6 = ((x[0] + x[1]) + (x[2] + x[3])) + (x[4] + x[5]);
    const double ap64 = sum3_abs_pair_f64(x[0], x[1], x[2], x[3], x[4], x[5]);
    const double fpap = (fabs(x[0] + x[1]) + fabs(x[2] + x[3])) + fabs(x[4] + x[5]);
    const double a364 = sum3_abs_f64(x[0], x[2], x[4]);
    const double fpa3 = (fabs(x[0]) + fabs(x[2])) + fabs(x[4]);
    bool ok;
    if ((t & 1) == 0) {
      ok = __float_as_uint(got) == __float_as_uint(d2f_bits(fp)) && same_d(got64, fp) && same_d(six64, fp6) &&
           same_d(ap64, fpap) && same_d(a364, fpa3);
    } else {
      const float ref = d2f_bits(fp);
      const double ulp = ldexp(1.0, ilogb(fmax(fabs((double)ref), fabs((double)got)) + 1e-300) - 23);
      ok = fabs((double)got - (double)ref) <= ldexp(amax, -48) + 2.0 * ulp;
      // FP64 results: both within 8 * 2^-52 of the largest |input| of the
      // exact sum (truncations and the final rounding; FP64 arithmetic's five
      // roundings), so within 2^-47 of each other
      ok = ok && fabs(got64 - fp) <= ldexp(amax, -47) && fabs(six64 - fp6) <= ldexp(amax, -47) &&
           fabs(ap64 - fpap) <= ldexp(amax, -47) && fabs(a364 - fpa3) <= ldexp(amax, -47);
    }
    if (t == 0) {          // equal pairs give +0; an infinity or a NaN gives NaN; zeros
      const double inf = __longlong_as_double(0x7ff0000000000000ll), nan = __longlong_as_double(0x7ff8000000000000ll);
      const float z = sum3_diff_f32(1.5, 1.5, -2.0, -2.0, 0.0, 0.0);
      const float a = sum3_diff_f32(inf, 1.0, 0.0, 0.0, 0.0, 0.0), b = sum3_diff_f32(1.0, 1.0, 2.0, nan, 0.0, 0.0);
      const double z64 = sum3_diff_f64(1.5, 1.5, -2.0, -2.0, 0.0, 0.0), a64 = sum6_f64(inf, 1.0, 0.0, 0.0, 0.0, 0.0);
      ok = ok && __float_as_uint(z) == 0u && a != a && b != b && __double_as_longlong(z64) == 0ll && a64 != a64;
      // zeros contribute nothing; a sum below the normal range is flushed to zero
      const double sub = __longlong_as_double(3ll);                     // 3 * 2^-1074
      ok = ok && __double_as_longlong(sum6_f64(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)) == 0ll &&
           __double_as_longlong(sum3_abs_pair_f64(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)) == 0ll &&
           __double_as_longlong(sum3_abs_f64(0.0, -0.0, 0.0)) == 0ll &&
           __float_as_uint(sum3_diff_f32(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)) == 0u &&
           sum6_f64(1.0, 0.0, 0.0, 0.0, 0.0, 0.0) == 1.0 && sum3_abs_f64(-2.5, 0.0, 0.0) == 2.5 &&
           sum6_f64(sub, sub, 0.0, 0.0, 0.0, 0.0) == 0.0 && sum3_diff_f64(1.0, sub, 0.0, 0.0, 0.0, 0.0) == 1.0;
    }
    if (!ok && atomicAdd(&bad[0], 1ull) == 0) bad[1] = (unsigned long long)t;
  }
}

static long long sum3_selftest() {
  unsigned long long* d = nullptr;
  unsigned long long h[2] = {0, 0};
  if (cudaMalloc(&d, 16) != cudaSuccess) { cudaGetLastError(); return -1; }
  bool ok = cudaMemset(d, 0, 16) == cudaSuccess;
  if (ok) {
    sum3_selftest_kernel<<<1216, 256>>>(1ll << 24, d);
    ok = cudaDeviceSynchronize() == cudaSuccess && cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  if (!ok) { cudaGetLastError(); return -1; }
  if (h[0]) fprintf(stderr, "mibm_selftest_: the integer-pipe sums fail at %llu sextuples (first t = %llu)\n", h[0], h[1]);
  return (long long)h[0];
}

long long tri_factors_selftest();   // tridiag.cu

// mls_exp on the device over n arguments spread over [-750, 712] and the
// weights' range [-11.2, 0]; out[t] = bits of the result
__global__ void mls_exp_selftest_kernel(long long n, unsigned long long* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double x = (t & 1) ? -11.2 * (double)(t >> 1) / (double)(n >> 1) : -750.0 + 1462.0 * (double)t / (double)n;
    out[t] = (unsigned long long)__double_as_longlong(mls_exp(x));
  }
}

static long long mls_exp_selftest() {
  const long long n = 1 << 20;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, n * 8) != cudaSuccess) { cudaGetLastError(); return -1; }
  std::vector<unsigned long long> h(n);
  mls_exp_selftest_kernel<<<608, 256>>>(n, d);
  bool ok = cudaMemcpy(h.data(), d, n * 8, cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok) { cudaGetLastError(); return -1; }
  long long bad = 0;
  for (long long t = 0; t < n; ++t) {
    const double x = (t & 1) ? -11.2 * (double)(t >> 1) / (double)(n >> 1) : -750.0 + 1462.0 * (double)t / (double)n;
    const double r = mls_exp(x);
    unsigned long long b;
    memcpy(&b, &r, 8);
    if (b != h[t]) ++bad;
  }
  return bad;
}

}  // namespace mibm

using namespace mibm;

extern "C" int mibm_selftest_(void) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) { cudaGetLastError(); return -1; }
  std::vector<unsigned long long> edge;
  edge_cases(edge);
  unsigned long long *dedge = nullptr, *dbad = nullptr;
  unsigned long long hbad[4] = {0, 0, 0, 0};
  const long long n_random = 1ll << 26;
  bool ok = cudaMalloc(&dedge, edge.size() * 8) == cudaSuccess && cudaMalloc(&dbad, 32) == cudaSuccess &&
            cudaMemcpy(dedge, edge.data(), edge.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(dbad, 0, 32) == cudaSuccess;
  if (ok) {
    conv_selftest_kernel<<<1216, 256>>>(dedge, (int)edge.size(), n_random, dbad);
    ok = cudaDeviceSynchronize() == cudaSuccess && cudaMemcpy(hbad, dbad, 32, cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(dedge);
  cudaFree(dbad);
  if (!ok) { cudaGetLastError(); return -1; }
  if (hbad[0] || hbad[1])
    fprintf(stderr, "mibm_selftest_: d2f %llu mismatches (first 0x%016llx), f2d %llu (first 0x%08llx)\n", hbad[0],
            hbad[2], hbad[1], hbad[3]);
  const long long tbad = tri_factors_selftest();
  if (tbad < 0) return -1;
  if (tbad) fprintf(stderr, "mibm_selftest_: %lld line-solve factor entries differ between host and device\n", tbad);
  const long long ebad = mls_exp_selftest();
  if (ebad < 0) return -1;
  if (ebad) fprintf(stderr, "mibm_selftest_: mls_exp differs between host and device at %lld arguments\n", ebad);
  const long long sbad = sum3_selftest();
  if (sbad < 0) return -1;
  return (int)std::min<unsigned long long>(hbad[0] + hbad[1] + (unsigned long long)tbad + (unsigned long long)ebad +
                                               (unsigned long long)sbad,
                                           1000000);
}

// ---------------------------------------------------------------------
// Bounds build: the registry of the translation units' hit counters and the
// two entry points (include/mibm.h).  Every unit that includes common.cuh
// registers its counter from a static constructor.
// ---------------------------------------------------------------------
namespace mibm {

static std::vector<unsigned (*)()>& bounds_units() {
  static std::vector<unsigned (*)()> units;
  return units;
}

void bounds_register(unsigned (*take)()) { bounds_units().push_back(take); }

#ifdef MIBM_BOUNDS
// one checked access at index n of an array of n elements: the check skips
// it and counts it
__global__ void bounds_selftest_kernel(int* __restrict__ buf, int n) {
  if (MIBM_IDX_OK(n, n)) buf[n] = 1;
}
#endif

}  // namespace mibm

extern "C" int mibm_bounds_check_(void) {
#ifdef MIBM_BOUNDS
  if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); return -2; }
  unsigned long long hits = 0;
  for (auto take : mibm::bounds_units()) hits += take();
  return (int)std::min<unsigned long long>(hits, 1u << 30);
#else
  return -1;
#endif
}

extern "C" int mibm_bounds_selftest_(void) {
#ifdef MIBM_BOUNDS
  int* d = nullptr;
  if (cudaMalloc(&d, 4 * sizeof(int)) != cudaSuccess) { cudaGetLastError(); return -2; }
  const int before = mibm_bounds_check_();
  mibm::bounds_selftest_kernel<<<1, 1>>>(d, 4);
  const int hits = mibm_bounds_check_();
  cudaFree(d);
  return (before == 0 && hits == 1) ? 0 : 1;
#else
  return -1;
#endif
}
