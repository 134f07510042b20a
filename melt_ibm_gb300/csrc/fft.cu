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
// staged in shared memory.  Each pass runs the kernel of fft_fast.cuh
// specialised for its line length when the length has one; the kernels
// below take any length (run-time plan).  Unnormalised, FFTW sign convention
// (forward = e^{-i...}).  The c2r pass drops the imaginary parts of the
// kx = 0 and kx = n1m/2 bins, as a Hermitian c2r transform does.
#include <cmath>
#include <vector>

#include "fft_common.cuh"

namespace mibm {

// Batched Stockham FFT of `nl` lines of length n held in shared memory.
// Element e of line l lives at buf[l*LS + e*ES].  Ping-pong between A and B;
// returns the buffer that holds the result.  sign = -1 forward, +1 inverse.
// tw[m] = e^{-2 pi i m / n}.
template <typename C>
__device__ C* fft_lines(C* A, C* B, int n, int nl, int LS, int ES, const Plan1D& plan, const C* tw, int sign) {
  typedef typename Real<C>::T R;
  int Ns = 1;
  for (int st = 0; st < plan.nst; ++st) {
    int Rdx = plan.radix[st];
    int nb = n / Rdx;                 // butterflies per line
    int total = nb * nl;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int l, j;
      if (LS == 1) { l = t % nl; j = t / nl; } else { j = t % nb; l = t / nb; }
      int kk = j % Ns;
      int tstep = n / (Ns * Rdx);     // twiddle index step
      C v[4];
      for (int r = 0; r < Rdx; ++r) v[r] = A[l * LS + (j + r * nb) * ES];
      for (int r = 1; r < Rdx; ++r) {
        C w = tw[(kk * r * tstep) % n];
        if (sign > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
      if (Rdx == 4) {
        C a02p = cadd(v[0], v[2]), a02m = csub(v[0], v[2]);
        C a13p = cadd(v[1], v[3]), a13m = csub(v[1], v[3]);
        // -i*(a1-a3) for the forward sign, +i*(a1-a3) for the inverse
        C rot = (sign < 0) ? mk<C>(a13m.y, -a13m.x) : mk<C>(-a13m.y, a13m.x);
        v[0] = cadd(a02p, a13p);
        v[2] = csub(a02p, a13p);
        v[1] = cadd(a02m, rot);
        v[3] = csub(a02m, rot);
      } else if (Rdx == 2) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
      } else {  // radix 3
        const R s3 = R(0.86602540378443864676);   // sqrt(3)/2
        C t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        C m = mk<C>(v[0].x - R(0.5) * t1.x, v[0].y - R(0.5) * t1.y);
        // forward: -i*s3*t2 ; inverse: +i*s3*t2
        C sv = (sign < 0) ? mk<C>(s3 * t2.y, -s3 * t2.x) : mk<C>(-s3 * t2.y, s3 * t2.x);
        v[0] = cadd(v[0], t1);
        v[1] = cadd(m, sv);
        v[2] = csub(m, sv);
      }
      int idxD = (j / Ns) * Ns * Rdx + kk;
      for (int r = 0; r < Rdx; ++r) B[l * LS + (idxD + r * Ns) * ES] = v[r];
    }
    __syncthreads();
    C* tmp = A; A = B; B = tmp;
    Ns *= Rdx;
  }
  return A;
}

// X forward: real rows (j, j+1) of plane k (source type S) -> half spectra
template <typename C, typename S>
__global__ void fft_x_fwd(FftArgs<C> F, const S* __restrict__ src, C* __restrict__ spec) {
  typedef typename Real<C>::T R;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* sh = (C*)shraw;
  const Grid& g = F.g;
  int n = g.n1m;
  C* tws = sh;
  C* A = sh + n;
  C* B = A + kRowPairs * n;
  load_tw(tws, F.twx, n);
  int k = blockIdx.y;
  int jp0 = blockIdx.x * kRowPairs;               // first row pair
  int npairs = min(kRowPairs, g.n2m / 2 - jp0);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, i = t % n;
    int j = 2 * (jp0 + l);
    A[l * n + i] = mk<C>(R(src[cidx(g, i, j, k)]), R(src[cidx(g, i, j + 1, k)]));
  }
  __syncthreads();
  C* Rr = fft_lines(A, B, n, npairs, n, 1, F.px, tws, -1);
  int H = g.H;
  for (int t = threadIdx.x; t < npairs * H; t += blockDim.x) {
    int l = t / H, kx = t % H;
    C z = Rr[l * n + kx];
    C zc = conjc(Rr[l * n + ((n - kx) % n)]);
    // X_a = (Z + conj Z_-)/2 ; X_b = (Z - conj Z_-)/(2i)
    C xa = mk<C>(R(0.5) * (z.x + zc.x), R(0.5) * (z.y + zc.y));
    C d = csub(z, zc);
    C xb = mk<C>(R(0.5) * d.y, R(-0.5) * d.x);
    int j = 2 * (jp0 + l);
    spec[(size_t)kx + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] = xa;
    spec[(size_t)kx + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)] = xb;
  }
}

// X inverse (c2r): half spectra of rows (j, j+1) -> real rows of type R
template <typename C>
__global__ void fft_x_inv(FftArgs<C> F, const C* __restrict__ spec, typename Real<C>::T* __restrict__ dst) {
  typedef typename Real<C>::T R;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* sh = (C*)shraw;
  const Grid& g = F.g;
  int n = g.n1m, H = g.H;
  C* tws = sh;
  C* A = sh + n;
  C* B = A + kRowPairs * n;
  load_tw(tws, F.twx, n);
  int k = blockIdx.y;
  int jp0 = blockIdx.x * kRowPairs;
  int npairs = min(kRowPairs, g.n2m / 2 - jp0);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, kx = t % n;
    int j = 2 * (jp0 + l);
    int src_kx = (kx < H) ? kx : n - kx;
    C xa = spec[(size_t)src_kx + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)];
    C xb = spec[(size_t)src_kx + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)];
    if (src_kx == 0 || 2 * src_kx == n) { xa.y = R(0); xb.y = R(0); }
    if (kx >= H) { xa.y = -xa.y; xb.y = -xb.y; }
    // Z = Xa + i Xb
    A[l * n + kx] = mk<C>(xa.x - xb.y, xa.y + xb.x);
  }
  __syncthreads();
  C* Rr = fft_lines(A, B, n, npairs, n, 1, F.px, tws, +1);
  for (int t = threadIdx.x; t < npairs * n; t += blockDim.x) {
    int l = t / n, i = t % n;
    int j = 2 * (jp0 + l);
    C z = Rr[l * n + i];
    dst[cidx(g, i, j, k)] = z.x;
    dst[cidx(g, i, j + 1, k)] = z.y;
  }
}

// Y pass (forward or inverse) on a tile of kCols kx columns of plane k
template <typename C>
__global__ void fft_y(FftArgs<C> F, C* __restrict__ spec, int sign) {
  extern __shared__ __align__(16) unsigned char shraw[];
  C* sh = (C*)shraw;
  const Grid& g = F.g;
  int n = g.n2m;
  C* tws = sh;
  C* A = sh + n;
  C* B = A + kCols * n;
  load_tw(tws, F.twy, n);
  int kx0 = blockIdx.x * kCols, k = blockIdx.y;
  int nc = min(kCols, g.H - kx0);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int j = t / kCols, l = t % kCols;
    A[t] = (l < nc) ? spec[(size_t)(kx0 + l) + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] : mk<C>(0, 0);
  }
  __syncthreads();
  C* Rr = fft_lines(A, B, n, kCols, 1, kCols, F.py, tws, sign);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int j = t / kCols, l = t % kCols;
    if (l < nc) spec[(size_t)(kx0 + l) + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] = Rr[t];
  }
}

// Z pass: forward, scale, eigenvalue division, zero mode, inverse
template <typename C>
__global__ void fft_z_solve(FftArgs<C> F, C* __restrict__ spec) {
  typedef typename Real<C>::T R;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* sh = (C*)shraw;
  const Grid& g = F.g;
  int n = g.n3m;
  C* tws = sh;
  C* A = sh + n;
  C* B = A + kCols * n;
  load_tw(tws, F.twz, n);
  int kx0 = blockIdx.x * kCols, j = blockIdx.y;
  int nc = min(kCols, g.H - kx0);
  size_t zstride = (size_t)g.HP * g.n2m;
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    A[t] = (l < nc) ? spec[(size_t)(kx0 + l) + (size_t)g.HP * j + zstride * k] : mk<C>(0, 0);
  }
  __syncthreads();
  C* Rr = fft_lines(A, B, n, kCols, 1, kCols, F.pz, tws, -1);
  C* O = (Rr == A) ? B : A;
  const R* __restrict__ eig = F.eig + (size_t)g.H * j;
  const size_t eig_k = (size_t)g.H * g.n2m;
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    C v = Rr[t];
    if (l < nc) {
      // buft / float(n1m*n2m*n3m) / (-ak3(k)-ak1(i)-ak2(j)), zero mode := 0
      if (k == 0 && kx0 + l == 0 && j == 0) v = mk<C>(0, 0);
      else { const R f = eig[(size_t)(kx0 + l) + eig_k * k]; v.x *= f; v.y *= f; }
    } else {
      v = mk<C>(0, 0);
    }
    Rr[t] = v;
  }
  __syncthreads();
  C* S = fft_lines(Rr, O, n, kCols, 1, kCols, F.pz, tws, +1);
  for (int t = threadIdx.x; t < kCols * n; t += blockDim.x) {
    int k = t / kCols, l = t % kCols;
    if (l < nc) spec[(size_t)(kx0 + l) + (size_t)g.HP * j + zstride * k] = S[t];
  }
}

// twiddle and eigenvalue tables per context (FP64 and FP32)
struct FftCache {
  Ctx* c = nullptr;
  double2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
  float2 *ftwx = nullptr, *ftwy = nullptr, *ftwz = nullptr;
  float *fak1 = nullptr, *fak2 = nullptr, *fak3 = nullptr;
  double* eig = nullptr;    // FftArgs::eig, FP64 (built at the first FP64 solve)
  float* feig = nullptr;    // the same rounded to FP32 (first FP32 solve)
  double* ztri = nullptr;   // FftArgs::ztri, FP64
  float* fztri = nullptr;   // the same rounded to FP32
  int zt_lines = 0;
  int zt_m = 0;             // FftArgs::zt_m
};
static std::vector<FftCache> g_fft;

// inv_nn * (1 / (-ak3(k) - ak1(kx) - ak2(j))) for kx < H, 0 at the zero mode
__global__ void eig_kernel(Grid g, const double* __restrict__ ak1, const double* __restrict__ ak2,
                           const double* __restrict__ ak3, double inv_nn, double* __restrict__ out,
                           float* __restrict__ fout) {
  const size_t n = (size_t)g.H * g.n2m * g.n3m;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(t % g.H);
    const size_t r = t / g.H;
    const int j = (int)(r % g.n2m), k = (int)(r / g.n2m);
    double f = 0.0;
    if (kx != 0 || j != 0 || k != 0) f = inv_nn * (1.0 / (-ak3[k] - ak1[kx] - ak2[j]));
    if (out) out[t] = f;
    if (fout) fout[t] = (float)f;
  }
}

// z-line tables.  After the x and y transforms, the z pass solves, for each
// line (kx, ky), (D_zz - lambda) phi = r with D_zz = dx3q (phi[k+1] - 2 phi[k]
// + phi[k-1]) periodic and lambda = ak1(kx) + ak2(ky): in Fourier space along z
// that is the division of phcalc.f90:57 (the eigenvalues of D_zz are -ak3,
// phini.f90:28-56), so the periodic tridiagonal solve gives the same phi.  It
// costs 10 FP64 operations per complex value against about 45 for the forward
// transform, division and inverse.  D_zz - lambda = -(2 dx3q + lambda) (I -
// rho (S + S^-1)), rho = dx3q / (2 dx3q + lambda), is the system the line
// solver's tables factor (tridiag_periodic.f90) with betadx = dx3q / lambda;
// its solution times -1/lambda, and the n3m / (n1m n2m n3m) of the unscaled
// transforms, is folded into the right-hand-side factors.  ak2(ky) =
// ak2(n2m - ky), so lines ky and n2m - ky share a table.  The line
// kx = ky = 0 (lambda = 0, singular; its mean is the zero mode set to 0,
// phcalc.f90:65) keeps the transform.  Layout, NT = H (n2m/2 + 1) lines,
// lt = kx + H min(ky, n2m - ky): arrays a, b, q, s at e*NT + lt (offsets 0,
// n, 2n, 3n times NT), then 4 scalars per line (ackl_b, api, ami, 1/den).
// Per-line tables of the z-line solves.  Chunked layout (zt_chunk(n) = M >
// 0): the extended table of the chunked line solves (tridiag.cu), entry q of
// line lt at q*NT + lt, with the a entries and the closure's ackl scaled by
// sigma.  Otherwise the base table: a, b, q, s at e*NT + lt (plus k*NS),
// then ackl, api, ami, 1/den per line.  Line 0 (the zero line) stays zero.
static bool make_ztri(Ctx* c, FftCache* f, bool f32) {
  if (f32 ? f->fztri != nullptr : f->ztri != nullptr) return true;
  const Grid& g = c->g;
  const int n = g.n3m, H = g.H, NT = H * (g.n2m / 2 + 1);
  const int zm = zt_chunk(n, H * g.n2m);
  const size_t NS = (size_t)n * NT;
  const size_t E = zm ? tri_ext_len(n, zm) : 0;
  const size_t len = zm ? E * NT : 4 * NS + 4 * (size_t)NT;
  std::vector<double> ak1(g.n1m), ak2(g.n2m);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "z-line tables")) return false;   // ak1/ak2 uploads
  cudaMemcpy(ak1.data(), c->ak1, sizeof(double) * g.n1m, cudaMemcpyDeviceToHost);
  cudaMemcpy(ak2.data(), c->ak2, sizeof(double) * g.n2m, cudaMemcpyDeviceToHost);
  std::vector<double> tab(len, 0.0), t;
  const double nfac = (double)n / ((double)g.n1m * (double)g.n2m * (double)g.n3m);
  for (int kyr = 0; kyr <= g.n2m / 2; ++kyr)
    for (int kx = 0; kx < H; ++kx) {
      const int lt = kx + H * kyr;
      const double lambda = ak1[kx] + ak2[kyr];
      if (kx == 0 && kyr == 0) continue;                 // the zero line: transform path
      const double sigma = -(1.0 / lambda) * nfac;
      if (zm) {
        tri_build_ext_table(n, zm, g.dx3q / lambda, t);
        const size_t S = 7 * (size_t)n + 3 * (size_t)(n / zm);
        for (size_t q = 0; q < E; ++q) tab[q * NT + lt] = (q < (size_t)n || q == S) ? t[q] * sigma : t[q];
        continue;
      }
      tri_build_table(n, g.dx3q / lambda, t);
      for (int e = 0; e < n; ++e) {
        tab[(size_t)e * NT + lt] = t[e] * sigma;
        tab[NS + (size_t)e * NT + lt] = t[n + e];
        tab[2 * NS + (size_t)e * NT + lt] = t[2 * n + e];
        tab[3 * NS + (size_t)e * NT + lt] = t[3 * n + e];
      }
      tab[4 * NS + 4 * (size_t)lt + 0] = t[4 * n + 0] * sigma;
      tab[4 * NS + 4 * (size_t)lt + 1] = t[4 * n + 1];
      tab[4 * NS + 4 * (size_t)lt + 2] = t[4 * n + 2];
      tab[4 * NS + 4 * (size_t)lt + 3] = t[4 * n + 3];
    }
  void* p = nullptr;
  if (!cuda_ok(c, cudaMalloc(&p, len * (f32 ? sizeof(float) : sizeof(double))), "z-line tables")) return false;
  if (f32) {
    std::vector<float> tf(tab.begin(), tab.end());
    cudaMemcpy(p, tf.data(), len * sizeof(float), cudaMemcpyHostToDevice);
    f->fztri = (float*)p;
  } else {
    cudaMemcpy(p, tab.data(), len * sizeof(double), cudaMemcpyHostToDevice);
    f->ztri = (double*)p;
  }
  f->zt_lines = NT;
  f->zt_m = zm;
  return true;
}

static bool make_eig(Ctx* c, FftCache* f, bool f32) {
  if (f32 ? f->feig != nullptr : f->eig != nullptr) return true;
  const Grid& g = c->g;
  const size_t n = (size_t)g.H * g.n2m * g.n3m;
  void* p = nullptr;
  if (!cuda_ok(c, cudaMalloc(&p, n * (f32 ? sizeof(float) : sizeof(double))), "eigenvalue table")) return false;
  const double inv_nn = 1.0 / ((double)g.n1m * (double)g.n2m * (double)g.n3m);
  eig_kernel<<<(unsigned)std::min<size_t>(div_up(n, 256), 4096), 256, 0, c->stream>>>(
      g, c->ak1, c->ak2, c->ak3, inv_nn, f32 ? nullptr : (double*)p, f32 ? (float*)p : nullptr);
  ++c->launches;
  if (f32) f->feig = (float*)p;
  else f->eig = (double*)p;
  return true;
}

template <typename C>
static C* make_tw(Ctx* c, int n) {
  std::vector<C> h(n);
  for (int m = 0; m < n; ++m) {
    double a = 2.0 * M_PI * (double)m / (double)n;
    h[m].x = std::cos(a);
    h[m].y = -std::sin(a);
  }
  C* d = nullptr;
  if (!cuda_ok(c, cudaMalloc(&d, sizeof(C) * n), "twiddles")) return nullptr;
  cudaMemcpy(d, h.data(), sizeof(C) * n, cudaMemcpyHostToDevice);
  return d;
}

static float* make_fak(Ctx* c, const double* ak, int n) {
  std::vector<double> h(n);
  cudaMemcpy(h.data(), ak, sizeof(double) * n, cudaMemcpyDeviceToHost);
  std::vector<float> f(h.begin(), h.end());
  float* d = nullptr;
  if (!cuda_ok(c, cudaMalloc(&d, sizeof(float) * n), "eigenvalues")) return nullptr;
  cudaMemcpy(d, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
  return d;
}

static FftCache* fft_of(Ctx* c) {
  for (auto& e : g_fft)
    if (e.c == c) return &e;
  FftCache f;
  f.c = c;
  f.twx = make_tw<double2>(c, c->g.n1m);
  f.twy = make_tw<double2>(c, c->g.n2m);
  f.twz = make_tw<double2>(c, c->g.n3m);
  f.ftwx = make_tw<float2>(c, c->g.n1m);
  f.ftwy = make_tw<float2>(c, c->g.n2m);
  f.ftwz = make_tw<float2>(c, c->g.n3m);
  f.fak1 = make_fak(c, c->ak1, c->g.n1m);
  f.fak2 = make_fak(c, c->ak2, c->g.n2m);
  f.fak3 = make_fak(c, c->ak3, c->g.n3m);
  g_fft.push_back(f);
  return &g_fft.back();
}

void fft_free(Ctx* c) {
  for (size_t q = 0; q < g_fft.size(); ++q)
    if (g_fft[q].c == c) {
      FftCache& f = g_fft[q];
      cudaFree(f.twx); cudaFree(f.twy); cudaFree(f.twz);
      cudaFree(f.ftwx); cudaFree(f.ftwy); cudaFree(f.ftwz);
      cudaFree(f.fak1); cudaFree(f.fak2); cudaFree(f.fak3);
      cudaFree(f.eig); cudaFree(f.feig); cudaFree(f.ztri); cudaFree(f.fztri);
      g_fft.erase(g_fft.begin() + q);
      return;
    }
}

// Builds the tables the solve of the given form needs before a step is
// launched (and possibly captured into a graph).
bool fft_prepare(Ctx* c, bool f32) {
  FftCache* fc = fft_of(c);
  return make_eig(c, fc, f32) && (f32 || make_ztri(c, fc, false));
}

template <typename C, typename S>
static void phcalc_launch(Ctx* c, FftArgs<C> F, const S* src, typename Real<C>::T* dst, const char* tag) {
  const Grid& g = c->g;
  C* spec = (C*)c->spec;
  size_t smx = sizeof(C) * (g.n1m + 2 * kRowPairs * g.n1m);
  size_t smy = sizeof(C) * (g.n2m + 2 * kCols * g.n2m);
  size_t smz = sizeof(C) * (g.n3m + 2 * kCols * g.n3m);
  cudaFuncSetAttribute((const void*)fft_x_fwd<C, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute((const void*)fft_x_inv<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute((const void*)fft_y<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  cudaFuncSetAttribute((const void*)fft_z_solve<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  dim3 gx(div_up(g.n2m / 2, kRowPairs), g.n3m);
  dim3 gy(div_up(g.H, kCols), g.n3m);
  dim3 gz(div_up(g.H, kCols), g.n2m);
  bool f32 = sizeof(C) == sizeof(float2);
  // each pass: the kernel specialised for its line length where one exists
  { MIBM_PROF(c, f32 ? "fft_x_fwd_f32" : "fft_x_fwd");
    if (!fastfft_x_fwd<C, S>(c, F, src, spec)) fft_x_fwd<C, S><<<gx, 256, smx, c->stream>>>(F, src, spec); }
  { MIBM_PROF(c, f32 ? "fft_y_f32" : "fft_y");
    if (!fastfft_y<C>(c, F, spec, -1)) fft_y<C><<<gy, 256, smy, c->stream>>>(F, spec, -1); }
  { MIBM_PROF(c, f32 ? "fft_z_solve_f32" : "fft_z_solve");
    if (!fastfft_z_solve<C>(c, F, spec)) fft_z_solve<C><<<gz, 256, smz, c->stream>>>(F, spec); }
  { MIBM_PROF(c, f32 ? "fft_y_f32" : "fft_y");
    if (!fastfft_y<C>(c, F, spec, +1)) fft_y<C><<<gy, 256, smy, c->stream>>>(F, spec, +1); }
  { MIBM_PROF(c, f32 ? "fft_x_inv_f32" : "fft_x_inv");
    if (!fastfft_x_inv<C>(c, F, spec, dst)) fft_x_inv<C><<<gx, 256, smx, c->stream>>>(F, spec, dst); }
  c->launches += 5;
  MIBM_LAUNCH_CHECK(c, tag);
}

void k_phcalc(Ctx* c) {
  const Grid& g = c->g;
  FftCache* fc = fft_of(c);
  if (!fc->twx || !fc->twy || !fc->twz) return;
  FftArgs<double2> F;
  F.g = g;
  F.px = make_plan(g.n1m); F.py = make_plan(g.n2m); F.pz = make_plan(g.n3m);
  F.twx = fc->twx; F.twy = fc->twy; F.twz = fc->twz;
  F.ak1 = c->ak1; F.ak2 = c->ak2; F.ak3 = c->ak3;
  F.inv_nn = 1.0 / ((double)g.n1m * (double)g.n2m * (double)g.n3m);
  if (!make_eig(c, fc, false) || !make_ztri(c, fc, false)) return;
  F.eig = fc->eig;
  F.ztri = fc->ztri; F.zt_lines = fc->zt_lines; F.zt_m = fc->zt_m;
  phcalc_launch<double2, double>(c, F, c->df[MIBM_F_DPH], c->df[MIBM_F_DPH], "phcalc");
}

// Precision form: the same solve in FP32 on the FP32 right-hand side
// `src` (the rounded FP64 residual), result phi in FP32.
void k_phcalc_f32(Ctx* c, const float* src, float* phi) {
  const Grid& g = c->g;
  FftCache* fc = fft_of(c);
  if (!fc->ftwx || !fc->fak1) return;
  FftArgs<float2> F;
  F.g = g;
  F.px = make_plan(g.n1m); F.py = make_plan(g.n2m); F.pz = make_plan(g.n3m);
  F.twx = fc->ftwx; F.twy = fc->ftwy; F.twz = fc->ftwz;
  F.ak1 = fc->fak1; F.ak2 = fc->fak2; F.ak3 = fc->fak3;
  F.inv_nn = (float)(1.0 / ((double)g.n1m * (double)g.n2m * (double)g.n3m));
  if (!make_eig(c, fc, true)) return;
  F.eig = fc->feig;
  // FP32 transforms cost little on the FP32 pipe: the z pass stays a
  // transform (the tridiagonal lines are latency-bound and slower there)
  F.ztri = nullptr; F.zt_lines = 0; F.zt_m = 0;
  phcalc_launch<float2, float>(c, F, src, phi, "phcalc_f32");
}

}  // namespace mibm
