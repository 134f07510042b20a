// Host build of the library's integer-pipe arithmetic (melt_ibm_gb300/csrc/
// fpconv.cuh, compiled here by g++ without CUDA) for the CPU tests: the same
// source the kernels use, exported over a C ABI in batches.
#include <stdint.h>

#include "fpconv.cuh"

extern "C" {

// which: 0 sum3_diff_f64, 1 sum6_f64, 2 sum3_abs_pair_f64, 3 sum3_abs_f64
// (first, third and fifth value of each sextuple), 4 sum3_diff_f32 (widened
// exactly to double); x holds n sextuples
void fpconv_sums(int which, long long n, const double* x, double* out) {
  for (long long t = 0; t < n; ++t) {
    const double* v = x + 6 * t;
    switch (which) {
      case 0: out[t] = mibm::sum3_diff_f64(v[0], v[1], v[2], v[3], v[4], v[5]); break;
      case 1: out[t] = mibm::sum6_f64(v[0], v[1], v[2], v[3], v[4], v[5]); break;
      case 2: out[t] = mibm::sum3_abs_pair_f64(v[0], v[1], v[2], v[3], v[4], v[5]); break;
      case 3: out[t] = mibm::sum3_abs_f64(v[0], v[2], v[4]); break;
      default: out[t] = (double)mibm::sum3_diff_f32(v[0], v[1], v[2], v[3], v[4], v[5]); break;
    }
  }
}

// d2f_bits and f2d_bits over bit patterns
void fpconv_d2f(long long n, const uint64_t* in, uint32_t* out) {
  for (long long t = 0; t < n; ++t) out[t] = mibm::fpc::bits32(mibm::d2f_bits(mibm::fpc::from64(in[t])));
}

void fpconv_f2d(long long n, const uint32_t* in, uint64_t* out) {
  for (long long t = 0; t < n; ++t) out[t] = mibm::fpc::bits64(mibm::f2d_bits(mibm::fpc::from32(in[t])));
}
}
