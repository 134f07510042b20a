// fft.cu -- pressure Poisson solve (phcalc.f90:11-97).
//
// The reference solves  lap_h(phi) = dph  with FFTW: a 2-D r2c transform per
// k-plane (x halved, then y), a 1-D c2c transform along z, division by
// N^3 and by the modified-wavenumber eigenvalue -(ak1+ak2+ak3)
// (phini.f90:28-56), the zero mode set to 0, and the inverse chain.  Here the
// same chain runs as five passes over a padded complex spectrum
// spec[k][j][kx] (kx = 0..n1m/2, pitch HP), each pass a batch of line FFTs
// staged in shared memory:
//   X  r2c along x   two real rows packed as one complex line
//   Y  c2c along y   tile of 8 adjacent kx columns
//   Z  c2c along z, scale and eigenvalue division, inverse c2c along z
//   Y' inverse along y
//   X' c2r along x   two Hermitian half-rows packed as one complex line
// Line FFTs are Stockham autosort transforms with radix-4/2/3 stages
// (n = 2^a 3^b), twiddles e^{-2 pi i m/n} tabulated on the host in FP64 and
// staged in shared memory.  Unnormalised, FFTW sign convention
// (forward = e^{-i...}).  The c2r pass drops the imaginary parts of the
// kx = 0 and kx = n1m/2 bins, as a Hermitian c2r transform does.
#include <cmath>
#include <vector>

#include "common.cuh"

namespace mibm {

struct Plan1D {
  int n = 0;
  int nst = 0;
  int radix[16];
};

static Plan1D make_plan(int n) {
  Plan1D p;
  p.n = n;
  int m = n;
  while (m % 4 == 0) { p.radix[p.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p.radix[p.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { p.radix[p.nst++] = 3; m /= 3; }
  return p;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }

// Batched Stockham FFT of `nl` lines of length n held in shared memory.
// Element e of line l lives at buf[l*LS + e*ES].  Ping-pong between A and B;
// returns the buffer that holds the result.  sign = -1 forward, +1 inverse.
// tw[m] = e^{-2 pi i m / n}.
__device__ double2* fft_lines(double2* A, double2* B, int n, int nl, int LS, int ES, const Plan1D& plan,
                              const double2* tw, int sign) {
  int Ns = 1;
  for (int st = 0; st < plan.nst; ++st) {
    int R = plan.radix[st];
    int nb = n / R;                 // butterflies per line
    int total = nb * nl;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int l, j;
      if (LS == 1) { l = t % nl; j = t / nl; } else { j = t % nb; l = t / nb; }
      int kk = j % Ns;
      int tstep = n / (Ns * R);     // twiddle index step
      double2 v[4];
      for (int r = 0; r < R; ++r) v[r] = A[l * LS + (j + r * nb) * ES];
      for (int r = 1; r < R; ++r) {
        double2 w = tw[(kk * r * tstep) % n];
        if (sign > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
      if (R == 4) {
        double2 a02p = cadd(v[0], v[2]), a02m = csub(v[0], v[2]);
        double2 a13p = cadd(v[1], v[3]), a13m = csub(v[1], v[3]);
        // -i*(a1-a3) for the forward sign, +i*(a1-a3) for the inverse
        double2 rot = (sign < 0) ? make_double2(a13m.y, -a13m.x) : make_double2(-a13m.y, a13m.x);
        v[0] = cadd(a02p, a13p);
        v[2] = csub(a02p, a13p);
        v[1] = cadd(a02m, rot);
        v[3] = csub(a02m, rot);
      } else if (R == 2) {
        double2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
      } else {  // R == 3
        const double s3 = 0.86602540378443864676;   // sqrt(3)/2
        double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        double2 m = make_double2(v[0].x - 0.5 * t1.x, v[0].y - 0.5 * t1.y);
        // forward: -i*s3*t2 ; inverse: +i*s3*t2
        double2 s = (sign < 0) ? make_double2(s3 * t2.y, -s3 * t2.x) : make_double2(-s3 * t2.y, s3 * t2.x);
        v[0] = cadd(v[0], t1);
        v[1] = cadd(m, s);
        v[2] = csub(m, s);
      }
      int idxD = (j / Ns) * Ns * R + kk;
      for (int r = 0; r < R; ++r) B[l * LS + (idxD + r * Ns) * ES] = v[r];
    }
    __syncthreads();
    double2* t = A; A = B; B = t;
    Ns *= R;
  }
  return A;
}

struct FftArgs {
  Grid g;
  Plan1D px, py, pz;
  const double2* twx;
  const double2* twy;
  const double2* twz;
  const double* ak1;
  const double* ak2;
  const double* ak3;
  double inv_nn;
};

__device__ __forceinline__ void load_tw(double2* s, const double2* tw, int n) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) s[m] = tw[m];
}

constexpr int kRowPairs = 4;   // X passes: 4 complex lines (8 real rows) per CTA
constexpr int kCols = 8;       // Y/Z passes: 8 adjacent kx columns per CTA

// X forward: real rows (j, j+1) of plane k -> spec half spectra
__global__ void fft_x_fwd(FftArgs F, const double* __restrict__ src, double2* __restrict__ spec) {
  extern __shared__ double2 sh[];
  const Grid& g = F.g;
  int n = g.n1m;
  double2* tws = sh;
  double2* A = sh + n;
  double2* B = A + kRowPairs * n;
  load_tw(tws, F.twx, n);
  int k = blockIdx.y;
  int jp0 = blockIdx.x * kRowPairs;               // first row pair
  int npairs = min(kRowPairs, g.n2m / 2 - jp0);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, i = t % n;
    int j = 2 * (jp0 + l);
    A[l * n + i] = make_double2(src[cidx(g, i, j, k)], src[cidx(g, i, j + 1, k)]);
  }
  __syncthreads();
  double2* R = fft_lines(A, B, n, npairs, n, 1, F.px, tws, -1);
  int H = g.H;
  for (int t = threadIdx.x; t < npairs * H; t += blockDim.x) {
    int l = t / H, kx = t % H;
    double2 z = R[l * n + kx];
    double2 zc = conjd(R[l * n + ((n - kx) % n)]);
    // X_a = (Z + conj Z_-)/2 ; X_b = (Z - conj Z_-)/(2i)
    double2 xa = make_double2(0.5 * (z.x + zc.x), 0.5 * (z.y + zc.y));
    double2 d = csub(z, zc);
    double2 xb = make_double2(0.5 * d.y, -0.5 * d.x);
    int j = 2 * (jp0 + l);
    spec[(size_t)kx + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] = xa;
    spec[(size_t)kx + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)] = xb;
  }
}

// X inverse (c2r): half spectra of rows (j, j+1) -> real rows
__global__ void fft_x_inv(FftArgs F, const double2* __restrict__ spec, double* __restrict__ dst) {
  extern __shared__ double2 sh[];
  const Grid& g = F.g;
  int n = g.n1m, H = g.H;
  double2* tws = sh;
  double2* A = sh + n;
  double2* B = A + kRowPairs * n;
  load_tw(tws, F.twx, n);
  int k = blockIdx.y;
  int jp0 = blockIdx.x * kRowPairs;
  int npairs = min(kRowPairs, g.n2m / 2 - jp0);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, kx = t % n;
    int j = 2 * (jp0 + l);
    int src_kx = (kx < H) ? kx : n - kx;
    double2 xa = spec[(size_t)src_kx + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)];
    double2 xb = spec[(size_t)src_kx + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)];
    if (src_kx == 0 || 2 * src_kx == n) { xa.y = 0.0; xb.y = 0.0; }
    if (kx >= H) { xa.y = -xa.y; xb.y = -xb.y; }
    // Z = Xa + i Xb
    A[l * n + kx] = make_double2(xa.x - xb.y, xa.y + xb.x);
  }
  __syncthreads();
  double2* R = fft_lines(A, B, n, npairs, n, 1, F.px, tws, +1);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, i = t % n;
    int j = 2 * (jp0 + l);
    double2 z = R[l * n + i];
    dst[cidx(g, i, j, k)] = z.x;
    dst[cidx(g, i, j + 1, k)] = z.y;
  }
}

// Y pass (forward or inverse) on a tile of kCols kx columns of plane k
__global__ void fft_y(FftArgs F, double2* __restrict__ spec, int sign) {
  extern __shared__ double2 sh[];
  const Grid& g = F.g;
  int n = g.n2m;
  double2* tws = sh;
  double2* A = sh + n;
  double2* B = A + kCols * n;
  load_tw(tws, F.twy, n);
  int kx0 = blockIdx.x * kCols, k = blockIdx.y;
  int nc = min(kCols, g.H - kx0);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int j = t / kCols, l = t % kCols;
    A[t] = (l < nc) ? spec[(size_t)(kx0 + l) + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] : make_double2(0, 0);
  }
  __syncthreads();
  double2* R = fft_lines(A, B, n, kCols, 1, kCols, F.py, tws, sign);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int j = t / kCols, l = t % kCols;
    if (l < nc) spec[(size_t)(kx0 + l) + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] = R[t];
  }
}

// Z pass: forward, scale, eigenvalue division, zero mode, inverse
__global__ void fft_z_solve(FftArgs F, double2* __restrict__ spec) {
  extern __shared__ double2 sh[];
  const Grid& g = F.g;
  int n = g.n3m;
  double2* tws = sh;
  double2* A = sh + n;
  double2* B = A + kCols * n;
  load_tw(tws, F.twz, n);
  int kx0 = blockIdx.x * kCols, j = blockIdx.y;
  int nc = min(kCols, g.H - kx0);
  size_t zstride = (size_t)g.HP * g.n2m;
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    A[t] = (l < nc) ? spec[(size_t)(kx0 + l) + (size_t)g.HP * j + zstride * k] : make_double2(0, 0);
  }
  __syncthreads();
  double2* R = fft_lines(A, B, n, kCols, 1, kCols, F.pz, tws, -1);
  double2* O = (R == A) ? B : A;
  double a2 = F.ak2[j];
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    double2 v = R[t];
    if (l < nc) {
      v.x *= F.inv_nn; v.y *= F.inv_nn;                 // buft / float(n1m*n2m*n3m)
      double d = -F.ak3[k] - F.ak1[kx0 + l] - a2;       // -ak3(k)-ak1(i)-ak2(j)
      if (k == 0 && kx0 + l == 0 && j == 0) v = make_double2(0.0, 0.0);
      else { double rd = 1.0 / d; v.x *= rd; v.y *= rd; }
    } else {
      v = make_double2(0.0, 0.0);
    }
    R[t] = v;
  }
  __syncthreads();
  double2* S = fft_lines(R, O, n, kCols, 1, kCols, F.pz, tws, +1);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    if (l < nc) spec[(size_t)(kx0 + l) + (size_t)g.HP * j + zstride * k] = S[t];
  }
}

// twiddle tables per context
struct FftCache {
  Ctx* c = nullptr;
  double2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
};
static std::vector<FftCache> g_fft;

static double2* make_tw(Ctx* c, int n) {
  std::vector<double2> h(n);
  for (int m = 0; m < n; ++m) {
    double a = 2.0 * M_PI * (double)m / (double)n;
    h[m] = make_double2(std::cos(a), -std::sin(a));
  }
  double2* d = nullptr;
  if (!cuda_ok(c, cudaMalloc(&d, sizeof(double2) * n), "twiddles")) return nullptr;
  cudaMemcpy(d, h.data(), sizeof(double2) * n, cudaMemcpyHostToDevice);
  return d;
}

static FftCache* fft_of(Ctx* c) {
  for (auto& e : g_fft)
    if (e.c == c) return &e;
  FftCache f;
  f.c = c;
  f.twx = make_tw(c, c->g.n1m);
  f.twy = make_tw(c, c->g.n2m);
  f.twz = make_tw(c, c->g.n3m);
  g_fft.push_back(f);
  return &g_fft.back();
}

void fft_free(Ctx* c) {
  for (size_t q = 0; q < g_fft.size(); ++q)
    if (g_fft[q].c == c) {
      cudaFree(g_fft[q].twx); cudaFree(g_fft[q].twy); cudaFree(g_fft[q].twz);
      g_fft.erase(g_fft.begin() + q);
      return;
    }
}

void k_phcalc(Ctx* c) {
  const Grid& g = c->g;
  FftCache* fc = fft_of(c);
  if (!fc->twx || !fc->twy || !fc->twz) return;
  FftArgs F;
  F.g = g;
  F.px = make_plan(g.n1m); F.py = make_plan(g.n2m); F.pz = make_plan(g.n3m);
  F.twx = fc->twx; F.twy = fc->twy; F.twz = fc->twz;
  F.ak1 = c->ak1; F.ak2 = c->ak2; F.ak3 = c->ak3;
  F.inv_nn = 1.0 / ((double)g.n1m * (double)g.n2m * (double)g.n3m);
  double* dph = c->df[MIBM_F_DPH];
  size_t smx = sizeof(double2) * (g.n1m + 2 * kRowPairs * g.n1m);
  size_t smy = sizeof(double2) * (g.n2m + 2 * kCols * g.n2m);
  size_t smz = sizeof(double2) * (g.n3m + 2 * kCols * g.n3m);
  static bool attr_done = false;
  if (!attr_done) {
    cudaFuncSetAttribute((const void*)fft_x_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute((const void*)fft_x_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute((const void*)fft_y, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute((const void*)fft_z_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_done = true;
  }
  dim3 gx(div_up(g.n2m / 2, kRowPairs), g.n3m);
  dim3 gy(div_up(g.H, kCols), g.n3m);
  dim3 gz(div_up(g.H, kCols), g.n2m);
  { MIBM_PROF(c, "fft_x_fwd"); fft_x_fwd<<<gx, 256, smx, c->stream>>>(F, dph, c->spec); }
  { MIBM_PROF(c, "fft_y"); fft_y<<<gy, 256, smy, c->stream>>>(F, c->spec, -1); }
  { MIBM_PROF(c, "fft_z_solve"); fft_z_solve<<<gz, 256, smz, c->stream>>>(F, c->spec); }
  { MIBM_PROF(c, "fft_y"); fft_y<<<gy, 256, smy, c->stream>>>(F, c->spec, +1); }
  { MIBM_PROF(c, "fft_x_inv"); fft_x_inv<<<gx, 256, smx, c->stream>>>(F, c->spec, dph); }
  c->launches += 5;
  MIBM_LAUNCH_CHECK(c, "phcalc");
}

}  // namespace mibm
