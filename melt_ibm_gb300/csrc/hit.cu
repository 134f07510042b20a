// hit.cu -- HIT forcing into forcx, forcy, forcz (hit.f90).
//
// Eswaran & Pope stochastic forcing (CalcHITRandomForce, hit.f90:1-126):
// the Ornstein-Uhlenbeck update of the mode amplitudes bhat and their
// solenoidal projection Fhat run on the host in the reference's loop order
// (a few hundred modes); the physical-space sums
//   forcx(i,j,k) = Re sum_{l,m,n} Fhat(1,l,m,n) e^{i kl xc_i} e^{i km ym_j} e^{i kn zm_k}
// (and the staggered variants for forcy, forcz) run on the device.  The sum
// factorises one axis at a time:
//   G_c(l, n; j) = sum_m Fhat(c,l,m,n) e^{i km y_j}          (nmodes^3 N)
//   H_c(l; j, k) = sum_n G_c(l, n; j) e^{i kn z_k}            (nmodes^2 N^2)
// and, because only the real part is kept and e^{-i kl x} is the conjugate
// of e^{i kl x}, the modes +l and -l fold into one coefficient:
//   Re(e H(l)) + Re(conj(e) H(-l)) = Re(e (H(l) + conj(H(-l)))),
// so every cell needs (nmodes+1)/2 complex-real products (the l = 0 one is a
// plain real part) instead of nmodes^3 -- the reference's O(nmodes^3 N^3)
// loops become O(nmodes^2 N^2 + nmodes N^3 / 2).  The sums are the
// reference's in another order (agreement to round-off).  The exponential
// tables are the reference's (InitRandomForce, hit.f90:171-202), evaluated
// on the host.  The precision form evaluates the last, per-cell stage in
// FP32 from FP32 copies of the tables (the forcing fields stay FP64).
//
// ABC forcing (CalcABC_HITForce, hit.f90:224-254) uses host tables of the
// sines and cosines of each coordinate line.
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace mibm {

struct HitState {
  int nmodes = 0, n1 = 0, n2 = 0, n3 = 0;
  std::vector<double> bhat;           // 2 * 3 * nmodes^3, (re, im), Fortran order (ndir, l, m, n)
  std::vector<int> waven;
  bool rng_seeded = false;
  uint64_t rng = 0;
  double2* d_fhat = nullptr;          // 3 * nmodes^3
  double2* d_ex = nullptr;            // [xc | xm] x nmodes x n1m  : e^{i k x}
  double2* d_ey = nullptr;            // [ym | yc] x nmodes x n2m
  double2* d_ez = nullptr;            // [zm | zc] x nmodes x n3m
  double2* d_g = nullptr;             // G: 3 x nmodes x nmodes x n2m
  double2* d_h = nullptr;             // folded H: 3 x nb x n3m x n2m, nb = (nmodes + 1) / 2
  float2* d_ex32 = nullptr;           // FP32 copy of d_ex (precision form)
  float2* d_h32 = nullptr;            // FP32 copy of d_h (precision form)
  double2* h_fhat = nullptr;          // pinned staging of Fhat (3 * nmodes^3)
  cudaEvent_t fhat_copied = nullptr;  // the staging buffer has been read by its copy
  double* d_abc = nullptr;            // ABC tables: sin/cos per axis
};

static std::vector<std::pair<Ctx*, HitState*>> g_hit;

static HitState* hit_of(Ctx* c) {
  for (auto& e : g_hit)
    if (e.first == c) return e.second;
  HitState* h = new HitState();
  g_hit.emplace_back(c, h);
  return h;
}

void hit_free(Ctx* c) {
  for (size_t q = 0; q < g_hit.size(); ++q)
    if (g_hit[q].first == c) {
      HitState* h = g_hit[q].second;
      cudaFree(h->d_fhat); cudaFree(h->d_ex); cudaFree(h->d_ey); cudaFree(h->d_ez); cudaFree(h->d_h);
      cudaFree(h->d_g); cudaFree(h->d_ex32); cudaFree(h->d_h32); cudaFreeHost(h->h_fhat);
      if (h->fhat_copied) cudaEventDestroy(h->fhat_copied);
      cudaFree(h->d_abc);
      delete h;
      g_hit.erase(g_hit.begin() + q);
      return;
    }
}

static double ref_pi() { return 2.0 * std::asin(1.0); }   // papero.f90:142

// cordin.f90:74-97 (1-based i): face and centre coordinates
static double coord_c(double len, int n, int i) { return len * ((double)(i - 1) / (double)n); }
static double coord_m(double len, int n, int i) {
  return (len * ((double)(i - 1) / (double)n) + len * ((double)i / (double)n)) * 0.5;
}

static int hit_nmodes(double kf_on_kmin) {
  int nbuffer = (int)std::floor(kf_on_kmin) + 1;   // hit.f90:139
  return (nbuffer - 1) * 2 + 1;
}

// splitmix64 (Steele, Lea & Flood 2014), uniform in (0, 1]
static double hit_uniform(HitState* h) {
  uint64_t z = (h->rng += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)((z >> 11) + 1) * (1.0 / 9007199254740992.0);
}

// (re)build the mode tables when the parameters or the grid change
static bool hit_setup(Ctx* c, HitState* h) {
  const Grid& g = c->g;
  int nm = hit_nmodes(c->S(MIBM_S_KF_ON_KMIN));
  if (nm == h->nmodes && h->n1 == g.n1m && h->n2 == g.n2m && h->n3 == g.n3m && h->d_fhat) return true;
  cudaFree(h->d_fhat); cudaFree(h->d_ex); cudaFree(h->d_ey); cudaFree(h->d_ez); cudaFree(h->d_h);
  cudaFree(h->d_g); cudaFree(h->d_ex32); cudaFree(h->d_h32); cudaFreeHost(h->h_fhat);
  h->d_fhat = nullptr; h->d_ex = h->d_ey = h->d_ez = h->d_h = h->d_g = nullptr;
  h->d_ex32 = nullptr; h->d_h32 = nullptr; h->h_fhat = nullptr;
  h->nmodes = nm; h->n1 = g.n1m; h->n2 = g.n2m; h->n3 = g.n3m;
  if (h->bhat.size() != 6 * (size_t)nm * nm * nm) h->bhat.assign(6 * (size_t)nm * nm * nm, 0.0);
  int nbuffer = (nm - 1) / 2 + 1;
  h->waven.assign(nm, 0);
  for (int i = 1; i <= nbuffer - 1; ++i) h->waven[i - 1] = -(nbuffer - i);   // hit.f90:152-160
  for (int i = 0; i <= nbuffer - 1; ++i) h->waven[nbuffer + i - 1] = i;
  const double pi = ref_pi();
  // e^{i kappa x} tables, hit.f90:171-202 (kappa = float(waveN)*2*pi/len)
  auto table = [&](int n, double len, bool face, std::vector<double2>& out, size_t at) {
    for (int q = 0; q < nm; ++q) {
      double kappa = (double)h->waven[q] * 2.0 * pi / len;
      for (int i = 1; i <= n; ++i) {
        double x = face ? coord_c(len, n, i) : coord_m(len, n, i);
        std::complex<double> e = std::exp(std::complex<double>(0.0, kappa * x));
        out[at + (size_t)q * n + (i - 1)] = make_double2(e.real(), e.imag());
      }
    }
  };
  std::vector<double2> ex(2 * (size_t)nm * g.n1m), ey(2 * (size_t)nm * g.n2m), ez(2 * (size_t)nm * g.n3m);
  table(g.n1m, g.xlen, true, ex, 0);                         // exp_I_kl_xsi (xc)
  table(g.n1m, g.xlen, false, ex, (size_t)nm * g.n1m);       // exp_I_kl_xi  (xm)
  table(g.n2m, g.ylen, false, ey, 0);                        // exp_I_km_yj  (ym)
  table(g.n2m, g.ylen, true, ey, (size_t)nm * g.n2m);        // exp_I_km_ysj (yc)
  table(g.n3m, g.zlen, false, ez, 0);                        // exp_I_kn_zk  (zm)
  table(g.n3m, g.zlen, true, ez, (size_t)nm * g.n3m);        // exp_I_kn_zsk (zc)
  const int nb = (nm + 1) / 2;
  std::vector<float2> ex32(ex.size());
  for (size_t q = 0; q < ex.size(); ++q) ex32[q] = make_float2((float)ex[q].x, (float)ex[q].y);
  bool ok = cuda_ok(c, cudaMalloc(&h->d_fhat, sizeof(double2) * 3 * (size_t)nm * nm * nm), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ex, sizeof(double2) * ex.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ey, sizeof(double2) * ey.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ez, sizeof(double2) * ez.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_g, sizeof(double2) * 3 * (size_t)nm * nm * g.n2m), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_h, sizeof(double2) * 3 * (size_t)nb * g.n2m * g.n3m), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ex32, sizeof(float2) * ex32.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_h32, sizeof(float2) * 3 * (size_t)nb * g.n2m * g.n3m), "hit") &&
            cuda_ok(c, cudaMallocHost(&h->h_fhat, sizeof(double2) * 3 * (size_t)nm * nm * nm), "hit");
  if (!ok) return false;
  if (!h->fhat_copied && !cuda_ok(c, cudaEventCreateWithFlags(&h->fhat_copied, cudaEventDisableTiming), "hit"))
    return false;
  cudaMemcpy(h->d_ex, ex.data(), sizeof(double2) * ex.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(h->d_ey, ey.data(), sizeof(double2) * ey.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(h->d_ez, ez.data(), sizeof(double2) * ez.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(h->d_ex32, ex32.data(), sizeof(float2) * ex32.size(), cudaMemcpyHostToDevice);
  return cuda_ok(c, cudaGetLastError(), "hit tables");
}

__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// G_c(l, n; j) = sum_m Fhat(c,l,m,n) e_y(j,m); one thread per (c, l, n, j)
__global__ void hit_g_kernel(Grid g, int nm, const double2* __restrict__ fhat, const double2* __restrict__ ey,
                             double2* __restrict__ G) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * (size_t)nm * nm * g.n2m) return;
  const int j = (int)(t % g.n2m);
  size_t r = t / g.n2m;
  const int n = (int)(r % nm);
  r /= nm;
  const int l = (int)(r % nm), c = (int)(r / nm);
  // forcx, forcz use ym; forcy uses yc
  const double2* eyc = ey + (c == 1 ? (size_t)nm * g.n2m : 0);
  double2 acc = make_double2(0.0, 0.0);
  for (int m = 0; m < nm; ++m) {
    double2 p = cmul2(fhat[(size_t)c + 3 * ((size_t)l + nm * ((size_t)m + (size_t)nm * n))], eyc[(size_t)m * g.n2m + j]);
    acc.x += p.x; acc.y += p.y;
  }
  G[t] = acc;
}

// H_c(l; j, k) = sum_n G_c(l, n; j) e_z(k, n), folded over +-l:
//   K_c(0) = H_c(l0),  K_c(p) = H_c(l0 + p) + conj(H_c(l0 - p)),  p = 1 .. nb-1,
// l0 = nb - 1 the zero wavenumber (waveN runs -(nb-1) .. nb-1).  One thread
// per (c, p, j, k); K stored [c][p][k][j], with an FP32 copy when wanted.
__global__ void hit_k_kernel(Grid g, int nm, const double2* __restrict__ G, const double2* __restrict__ ez,
                             double2* __restrict__ K, float2* __restrict__ K32) {
  const int nb = (nm + 1) / 2, l0 = nb - 1;
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t plane = (size_t)g.n2m * g.n3m;
  if (t >= 3 * (size_t)nb * plane) return;
  const size_t jk = t % plane;
  const int j = (int)(jk % g.n2m), k = (int)(jk / g.n2m);
  const size_t r = t / plane;
  const int p = (int)(r % nb), c = (int)(r / nb);
  // forcx, forcy use zm; forcz uses zc
  const double2* ezc = ez + (c == 2 ? (size_t)nm * g.n3m : 0);
  auto H = [&](int l) {
    double2 acc = make_double2(0.0, 0.0);
    const double2* Gl = G + (((size_t)c * nm + l) * nm) * g.n2m + j;
    for (int n = 0; n < nm; ++n) {
      double2 q = cmul2(Gl[(size_t)n * g.n2m], ezc[(size_t)n * g.n3m + k]);
      acc.x += q.x; acc.y += q.y;
    }
    return acc;
  };
  double2 v = H(l0 + p);
  if (p > 0) {
    double2 w = H(l0 - p);
    v.x += w.x;
    v.y -= w.y;
  }
  K[t] = v;
  if (K32) K32[t] = make_float2((float)v.x, (float)v.y);
}

// forc_c(i,j,k) = Re K_c(0) + sum_{p>=1} Re(e_x(i, l0+p) K_c(p))
template <typename R, typename R2>
__global__ void hit_force_kernel(Grid g, int nm, const R2* __restrict__ ex, const R2* __restrict__ K,
                                 double* __restrict__ fx, double* __restrict__ fy, double* __restrict__ fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n1m) return;
  const int nb = (nm + 1) / 2, l0 = nb - 1;
  size_t plane = (size_t)g.n2m * g.n3m, jk = (size_t)j + (size_t)g.n2m * k;
  double out[3];
  for (int c = 0; c < 3; ++c) {
    const R2* exc = ex + (c == 0 ? 0 : (size_t)nm * g.n1m);   // forcx at xc, forcy/forcz at xm
    const R2* Kc = K + (size_t)c * nb * plane + jk;
    R s = Kc[0].x;
    for (int p = 1; p < nb; ++p) {
      R2 e = exc[(size_t)(l0 + p) * g.n1m + i];
      R2 kk = Kc[(size_t)p * plane];
      s += e.x * kk.x - e.y * kk.y;
    }
    out[c] = (double)s;
  }
  size_t c0 = cidx(g, i, j, k);
  fx[c0] = out[0]; fy[c0] = out[1]; fz[c0] = out[2];
}

// ABC forcing: tables [sin zm | cos ym | sin xm | cos zm | sin ym | cos xm] of 2 pi x / len
__global__ void hit_abc_kernel(Grid g, double C, const double* __restrict__ tab, double* __restrict__ fx,
                               double* __restrict__ fy, double* __restrict__ fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n1m) return;
  const double* szm = tab;
  const double* cym = szm + g.n3m;
  const double* sxm = cym + g.n2m;
  const double* czm = sxm + g.n1m;
  const double* sym = czm + g.n3m;
  const double* cxm = sym + g.n2m;
  size_t c0 = cidx(g, i, j, k);
  fx[c0] = C * szm[k] + C * cym[j];
  fy[c0] = C * sxm[i] + C * czm[k];
  fz[c0] = C * sym[j] + C * cxm[i];
}

// linear forcing (extension): forc = xlen * C * u at each velocity's position
__global__ void hit_linear_kernel(Grid g, double a, const double* __restrict__ vx, const double* __restrict__ vy,
                                  const double* __restrict__ vz, double* __restrict__ fx, double* __restrict__ fy,
                                  double* __restrict__ fz) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.cells) return;
  fx[t] = a * vx[t];
  fy[t] = a * vy[t];
  fz[t] = a * vz[t];
}

// CalcHITRandomForce, hit.f90:20-60: O-U update and solenoidal projection
static void hit_update_modes(Ctx* c, HitState* h, std::vector<double2>& fhat) {
  const Grid& g = c->g;
  const int nm = h->nmodes;
  const double pi = ref_pi();
  const double dt = c->S(MIBM_S_DT), tl = c->S(MIBM_S_TL), eps = c->S(MIBM_S_EPSSTAR);
  const double kf = c->S(MIBM_S_KF_ON_KMIN) * 2.0 * pi / g.xlen;
  if (!h->rng_seeded) {
    h->rng = (uint64_t)(int64_t)c->I(MIBM_I_HIT_SEED);
    h->rng_seeded = true;
  }
  fhat.assign(3 * (size_t)nm * nm * nm, make_double2(0.0, 0.0));
  const double amp = std::sqrt(2.0 * eps * dt / (tl * tl));
  for (int l = 0; l < nm; ++l) {
    double kl = (double)h->waven[l] * 2.0 * pi / g.xlen;
    for (int m = 0; m < nm; ++m) {
      double km = (double)h->waven[m] * 2.0 * pi / g.ylen;
      for (int n = 0; n < nm; ++n) {
        double kn = (double)h->waven[n] * 2.0 * pi / g.zlen;
        double kmag = std::sqrt(kl * kl + km * km + kn * kn);
        if (!(kmag > 0.0 && kmag < kf)) continue;
        size_t base = 3 * ((size_t)l + nm * ((size_t)m + (size_t)nm * n));
        std::complex<double> b[3];
        for (int d = 0; d < 3; ++d) {
          double u1 = hit_uniform(h), u2 = hit_uniform(h);
          double r = std::sqrt(-2.0 * std::log(u1));
          std::complex<double> rc(r * std::cos(2.0 * pi * u2), r * std::sin(2.0 * pi * u2));
          std::complex<double> old(h->bhat[2 * (base + d)], h->bhat[2 * (base + d) + 1]);
          b[d] = old * (1.0 - dt / tl) + rc * amp;
          h->bhat[2 * (base + d)] = b[d].real();
          h->bhat[2 * (base + d) + 1] = b[d].imag();
        }
        // Fhat = bhat - k (k . bhat) / |k|^2
        std::complex<double> dot = kl * b[0] + km * b[1] + kn * b[2];
        double kk[3] = {kl, km, kn};
        for (int d = 0; d < 3; ++d) {
          std::complex<double> f = b[d] - kk[d] * dot / (kmag * kmag);
          fhat[base + d] = make_double2(f.real(), f.imag());
        }
      }
    }
  }
}

void k_hit_random_force(Ctx* c) {
  HitState* h = hit_of(c);
  if (!hit_setup(c, h)) return;
  std::vector<double2> fhat;
  hit_update_modes(c, h, fhat);
  const Grid& g = c->g;
  const int nm = h->nmodes, nb = (nm + 1) / 2;
  // the pinned staging buffer is reused: its previous copy must have run
  if (!cuda_ok(c, cudaEventSynchronize(h->fhat_copied), "hit")) return;
  memcpy(h->h_fhat, fhat.data(), sizeof(double2) * fhat.size());
  cudaMemcpyAsync(h->d_fhat, h->h_fhat, sizeof(double2) * fhat.size(), cudaMemcpyHostToDevice, c->stream);
  cudaEventRecord(h->fhat_copied, c->stream);
  const bool f32 = c->precision == 1;
  size_t ng = 3 * (size_t)nm * nm * g.n2m, nk = 3 * (size_t)nb * g.n2m * g.n3m;
  { MIBM_PROF(c, "hit_modes");
    hit_g_kernel<<<div_up(ng, 256), 256, 0, c->stream>>>(g, nm, h->d_fhat, h->d_ey, h->d_g);
    hit_k_kernel<<<div_up(nk, 256), 256, 0, c->stream>>>(g, nm, h->d_g, h->d_ez, h->d_h, f32 ? h->d_h32 : nullptr); }
  { MIBM_PROF(c, "hit_force");
    dim3 grid(div_up(g.n1m, 128), g.n2m, g.n3m);
    if (f32)
      hit_force_kernel<float, float2><<<grid, 128, 0, c->stream>>>(
          g, nm, h->d_ex32, h->d_h32, c->df[MIBM_F_FORCX], c->df[MIBM_F_FORCY], c->df[MIBM_F_FORCZ]);
    else
      hit_force_kernel<double, double2><<<grid, 128, 0, c->stream>>>(
          g, nm, h->d_ex, h->d_h, c->df[MIBM_F_FORCX], c->df[MIBM_F_FORCY], c->df[MIBM_F_FORCZ]); }
  c->launches += 3;
  cuda_ok(c, cudaGetLastError(), "hit");
}

void k_hit_abc_force(Ctx* c) {
  HitState* h = hit_of(c);
  const Grid& g = c->g;
  const double pi = ref_pi();
  std::vector<double> tab((size_t)2 * (g.n1m + g.n2m + g.n3m));
  double* szm = tab.data();
  double* cym = szm + g.n3m;
  double* sxm = cym + g.n2m;
  double* czm = sxm + g.n1m;
  double* sym = czm + g.n3m;
  double* cxm = sym + g.n2m;
  for (int k = 1; k <= g.n3m; ++k) {
    szm[k - 1] = std::sin(2.0 * pi * coord_m(g.zlen, g.n3m, k) / g.zlen);
    czm[k - 1] = std::cos(2.0 * pi * coord_m(g.zlen, g.n3m, k) / g.zlen);
  }
  for (int j = 1; j <= g.n2m; ++j) {
    cym[j - 1] = std::cos(2.0 * pi * coord_m(g.ylen, g.n2m, j) / g.ylen);
    sym[j - 1] = std::sin(2.0 * pi * coord_m(g.ylen, g.n2m, j) / g.ylen);
  }
  for (int i = 1; i <= g.n1m; ++i) {
    sxm[i - 1] = std::sin(2.0 * pi * coord_m(g.xlen, g.n1m, i) / g.xlen);
    cxm[i - 1] = std::cos(2.0 * pi * coord_m(g.xlen, g.n1m, i) / g.xlen);
  }
  if (!h->d_abc && !cuda_ok(c, cudaMalloc(&h->d_abc, sizeof(double) * tab.size()), "abc")) return;
  cudaMemcpy(h->d_abc, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice);
  double C = c->S(MIBM_S_C_HIT) * ((2.0 * pi / g.xlen) * (2.0 * pi / g.xlen));   // C_HIT*(2 pi/xlen)**2
  { MIBM_PROF(c, "hit_abc");
    hit_abc_kernel<<<dim3(div_up(g.n1m, 128), g.n2m, g.n3m), 128, 0, c->stream>>>(
        g, C, h->d_abc, c->df[MIBM_F_FORCX], c->df[MIBM_F_FORCY], c->df[MIBM_F_FORCZ]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "abc forcing");
}

void k_hit_linear_force(Ctx* c) {
  const Grid& g = c->g;
  double a = g.xlen * c->S(MIBM_S_C_HIT);
  { MIBM_PROF(c, "hit_linear");
    hit_linear_kernel<<<div_up(g.cells, 256), 256, 0, c->stream>>>(
        g, a, c->df[MIBM_F_VX], c->df[MIBM_F_VY], c->df[MIBM_F_VZ], c->df[MIBM_F_FORCX], c->df[MIBM_F_FORCY],
        c->df[MIBM_F_FORCZ]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "linear forcing");
}

int hit_modes(Ctx* c) { return hit_nmodes(c->S(MIBM_S_KF_ON_KMIN)); }

void hit_bhat(Ctx* c, double* buf, int dir) {
  HitState* h = hit_of(c);
  int nm = hit_nmodes(c->S(MIBM_S_KF_ON_KMIN));
  size_t n = 6 * (size_t)nm * nm * nm;
  if (h->bhat.size() != n) h->bhat.assign(n, 0.0);
  if (dir == 0) std::copy(h->bhat.begin(), h->bhat.end(), buf);
  else std::copy(buf, buf + n, h->bhat.begin());
}

// Position of the Gaussian-increment stream (the splitmix64 counter): read
// (dir 0; before the first draw, the seed the first call would take) or
// set (dir 1), so that a continued run draws what the uninterrupted one would.
void hit_rng(Ctx* c, unsigned long long* state, int dir) {
  HitState* h = hit_of(c);
  if (dir == 0) *state = h->rng_seeded ? h->rng : (uint64_t)(int64_t)c->I(MIBM_I_HIT_SEED);
  else { h->rng = *state; h->rng_seeded = true; }
}

}  // namespace mibm
