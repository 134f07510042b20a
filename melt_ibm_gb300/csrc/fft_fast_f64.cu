// fft_fast_f64.cu -- instances of the fixed-length Poisson FFT passes for
// double2 spectra (see fft_fast.cuh); one translation unit per precision so the
// two compile in parallel.
#include "fft_fast.cuh"

namespace mibm {

template <>
bool fastfft_x_fwd<double2, double>(Ctx* c, const FftArgs<double2>& F, const double* src, double2* spec) {
  switch (c->g.n1m) {
#define CASE(N) case N: fastfft::launch_x_fwd<double2, double, N>(c, F, src, spec); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_x_inv<double2>(Ctx* c, const FftArgs<double2>& F, const double2* spec, double* dst) {
  switch (c->g.n1m) {
#define CASE(N) case N: fastfft::launch_x_inv<double2, N>(c, F, spec, dst); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_y<double2>(Ctx* c, const FftArgs<double2>& F, double2* spec, int sign) {
  switch (c->g.n2m) {
#define CASE(N) case N: fastfft::launch_y<double2, N>(c, F, spec, sign); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

template <>
bool fastfft_z_solve<double2>(Ctx* c, const FftArgs<double2>& F, double2* spec) {
  switch (c->g.n3m) {
#define CASE(N) case N: fastfft::launch_z<double2, N>(c, F, spec); return true;
    MIBM_FFT_SIZES(CASE)
#undef CASE
  }
  return false;
}

}  // namespace mibm
