// fft_common.cuh -- types shared by the Poisson-solve FFT kernels (fft.cu,
// the generic mixed-radix path, and fft_fast.cuh, the kernels specialised for
// fixed line lengths).
#pragma once

#include "common.cuh"

namespace mibm {

struct Plan1D {
  int n = 0;
  int nst = 0;
  int radix[16];
};

inline Plan1D make_plan(int n) {
  Plan1D p;
  p.n = n;
  int m = n;
  while (m % 4 == 0) { p.radix[p.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p.radix[p.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { p.radix[p.nst++] = 3; m /= 3; }
  return p;
}

// complex helpers for double2 / float2
template <typename C> struct Real;
template <> struct Real<double2> { typedef double T; };
template <> struct Real<float2> { typedef float T; };
template <typename C> __device__ __forceinline__ C mk(typename Real<C>::T x, typename Real<C>::T y) { C r; r.x = x; r.y = y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) { return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C conjc(C a) { return mk<C>(a.x, -a.y); }

template <typename C>
struct FftArgs {
  typedef typename Real<C>::T R;
  Grid g;
  Plan1D px, py, pz;
  const C* twx;
  const C* twy;
  const C* twz;
  const R* ak1;
  const R* ak2;
  const R* ak3;
  R inv_nn;
  // inv_nn / (-ak3(k) - ak1(kx) - ak2(j)) at kx + H*(j + n2m*k), 0 at the
  // zero mode: the scale and the eigenvalue division of the z pass as one
  // multiply (an FP64 division is a long sequence of FP64 operations)
  const R* eig;
  // z-line solve tables (fft.cu make_ztri), nullptr: z passes by FFT
  const R* ztri;
  int zt_lines;
  int zt_m;            // chunk length of the chunked z-line tables, 0: one thread per line
};

// chunk length of the chunked z-line Poisson solve for `lines` lines of n
// cells: M = 16 or 8 with 2..kZtMaxChunks chunks (warps of a block), 0 =
// none (one thread per line).  Chunking costs 10 FP64 operations per complex
// cell against 8 for one sweep per line, so it only pays where one thread
// per line leaves the GPU short of warps (measured: 128^3, 8320 lines, 97
// -> 48 us per solve; 256^3, 33024 lines, 233 -> 289 us).
constexpr int kZtMaxChunks = 16;
constexpr int kZtChunkLines = 16384;
inline int zt_chunk(int n, int lines) {
  if (lines >= kZtChunkLines) return 0;
  if (n % 16 == 0 && n / 16 >= 2 && n / 16 <= kZtMaxChunks) return 16;
  if (n % 8 == 0 && n / 8 >= 2 && n / 8 <= kZtMaxChunks) return 8;
  return 0;
}

template <typename C>
__device__ __forceinline__ void load_tw(C* s, const C* tw, int n) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) s[m] = tw[m];
}

constexpr int kRowPairs = 4;   // X passes: 4 complex lines (8 real rows) per CTA
constexpr int kCols = 8;       // Y/Z passes: 8 adjacent kx columns per CTA

// Kernels specialised at compile time for one line length; each returns
// false when the length has no instance (the caller then uses the generic
// kernels of fft.cu).  S is the element type of the real input.
template <typename C, typename S>
bool fastfft_x_fwd(Ctx* c, const FftArgs<C>& F, const S* src, C* spec);
template <typename C>
bool fastfft_y(Ctx* c, const FftArgs<C>& F, C* spec, int sign);
template <typename C>
bool fastfft_z_solve(Ctx* c, const FftArgs<C>& F, C* spec);
template <typename C>
bool fastfft_x_inv(Ctx* c, const FftArgs<C>& F, const C* spec, typename Real<C>::T* dst);

// instances (fft_fast_f64.cu, fft_fast_f32.cu)
template <> bool fastfft_x_fwd<double2, double>(Ctx*, const FftArgs<double2>&, const double*, double2*);
template <> bool fastfft_x_fwd<float2, float>(Ctx*, const FftArgs<float2>&, const float*, float2*);
template <> bool fastfft_x_inv<double2>(Ctx*, const FftArgs<double2>&, const double2*, double*);
template <> bool fastfft_x_inv<float2>(Ctx*, const FftArgs<float2>&, const float2*, float*);
template <> bool fastfft_y<double2>(Ctx*, const FftArgs<double2>&, double2*, int);
template <> bool fastfft_y<float2>(Ctx*, const FftArgs<float2>&, float2*, int);
template <> bool fastfft_z_solve<double2>(Ctx*, const FftArgs<double2>&, double2*);
template <> bool fastfft_z_solve<float2>(Ctx*, const FftArgs<float2>&, float2*);

}  // namespace mibm
