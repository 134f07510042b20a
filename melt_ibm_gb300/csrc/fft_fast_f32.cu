// fft_fast_f32.cu -- instances of the fixed-length Poisson FFT passes for
// float2 spectra (see fft_fast.cuh); one translation unit per precision so the
// two compile in parallel.
#include "fft_fast.cuh"

namespace mibm {

template <>
bool fastfft_x_fwd<float2, float>(Ctx* c, const FftArgs<float2>& F, const float* src, float2* spec) {
  switch (c->g.n1m) {
#define CASE(N) case N: fastfft::launch_x_fwd<float2, float, N>(c, F, src, spec); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_x_inv<float2>(Ctx* c, const FftArgs<float2>& F, const float2* spec, float* dst) {
  switch (c->g.n1m) {
#define CASE(N) case N: fastfft::launch_x_inv<float2, N>(c, F, spec, dst); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_y<float2>(Ctx* c, const FftArgs<float2>& F, float2* spec, int sign) {
  switch (c->g.n2m) {
#define CASE(N) case N: fastfft::launch_y<float2, N>(c, F, spec, sign); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_z_solve<float2>(Ctx* c, const FftArgs<float2>& F, float2* spec) {
  switch (c->g.n3m) {
#define CASE(N) case N: fastfft::launch_z<float2, N>(c, F, spec); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

}  // namespace mibm
