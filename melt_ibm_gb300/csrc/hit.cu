// hit.cu -- HIT forcing into forcx, forcy, forcz (hit.f90).
//
// Eswaran & Pope stochastic forcing (CalcHITRandomForce, hit.f90:1-126):
// the Ornstein-Uhlenbeck update of the mode amplitudes bhat and their
// solenoidal projection Fhat run on the host in the reference's loop order
// (a few hundred modes); the physical-space sums
//   forcx(i,j,k) = Re sum_{l,m,n} Fhat(1,l,m,n) e^{i kl xc_i} e^{i km ym_j} e^{i kn zm_k}
// (and the staggered variants for forcy, forcz) run on the device.  The sum
// factorises: H_c(l; j, k) = sum_{m,n} Fhat(c,l,m,n) e^{i km y_j} e^{i kn z_k}
// is formed once per (l, j, k), then every cell needs nmodes complex
// products instead of nmodes^3 -- the reference's O(nmodes^3 N^3) loops
// become O(nmodes^2 N^2 + nmodes N^3).  The exponential tables are the
// reference's (InitRandomForce, hit.f90:171-202), evaluated on the host.
//
// ABC forcing (CalcABC_HITForce, hit.f90:224-254) uses host tables of the
// sines and cosines of each coordinate line.
#include <cmath>
#include <complex>
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
  double2* d_h = nullptr;             // 3 x nmodes x n2m x n3m
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
  h->d_fhat = nullptr; h->d_ex = h->d_ey = h->d_ez = h->d_h = nullptr;
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
  bool ok = cuda_ok(c, cudaMalloc(&h->d_fhat, sizeof(double2) * 3 * (size_t)nm * nm * nm), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ex, sizeof(double2) * ex.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ey, sizeof(double2) * ey.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_ez, sizeof(double2) * ez.size()), "hit") &&
            cuda_ok(c, cudaMalloc(&h->d_h, sizeof(double2) * 3 * (size_t)nm * g.n2m * g.n3m), "hit");
  if (!ok) return false;
  cudaMemcpy(h->d_ex, ex.data(), sizeof(double2) * ex.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(h->d_ey, ey.data(), sizeof(double2) * ey.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(h->d_ez, ez.data(), sizeof(double2) * ez.size(), cudaMemcpyHostToDevice);
  return cuda_ok(c, cudaGetLastError(), "hit tables");
}

__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// H_c(l; j, k) = sum_n sum_m Fhat(c,l,m,n) * (e_y(j,m) * e_z(k,n)); one thread per (c, l, j, k)
__global__ void hit_h_kernel(Grid g, int nm, const double2* __restrict__ fhat, const double2* __restrict__ ey,
                             const double2* __restrict__ ez, double2* __restrict__ H) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t plane = (size_t)g.n2m * g.n3m;
  if (t >= 3 * (size_t)nm * plane) return;
  int c = (int)(t / ((size_t)nm * plane));
  size_t r = t - (size_t)c * nm * plane;
  int l = (int)(r / plane);
  size_t jk = r - (size_t)l * plane;
  int j = (int)(jk % g.n2m), k = (int)(jk / g.n2m);
  // forcx, forcz use ym; forcy uses yc.  forcx, forcy use zm; forcz uses zc.
  const double2* eyc = ey + (c == 1 ? (size_t)nm * g.n2m : 0);
  const double2* ezc = ez + (c == 2 ? (size_t)nm * g.n3m : 0);
  double2 acc = make_double2(0.0, 0.0);
  for (int n = 0; n < nm; ++n) {
    double2 zk = ezc[(size_t)n * g.n3m + k];
    for (int m = 0; m < nm; ++m) {
      double2 b = cmul2(eyc[(size_t)m * g.n2m + j], zk);                       // buff1
      double2 f = fhat[(size_t)c + 3 * ((size_t)l + nm * ((size_t)m + (size_t)nm * n))];
      double2 p = cmul2(f, b);
      acc.x += p.x; acc.y += p.y;
    }
  }
  H[(size_t)c * nm * plane + (size_t)l * plane + jk] = acc;
}

// forc_c(i,j,k) = Re sum_l e_x(i,l) * H_c(l; j, k)
__global__ void hit_force_kernel(Grid g, int nm, const double2* __restrict__ ex, const double2* __restrict__ H,
                                 double* __restrict__ fx, double* __restrict__ fy, double* __restrict__ fz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n1m) return;
  size_t plane = (size_t)g.n2m * g.n3m, jk = (size_t)j + (size_t)g.n2m * k;
  double out[3];
  for (int c = 0; c < 3; ++c) {
    const double2* exc = ex + (c == 0 ? 0 : (size_t)nm * g.n1m);   // forcx at xc, forcy/forcz at xm
    double s = 0.0;
    for (int l = 0; l < nm; ++l) {
      double2 e = exc[(size_t)l * g.n1m + i];
      double2 hh = H[(size_t)c * nm * plane + (size_t)l * plane + jk];
      s += e.x * hh.x - e.y * hh.y;
    }
    out[c] = s;
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
  const int nm = h->nmodes;
  cudaMemcpyAsync(h->d_fhat, fhat.data(), sizeof(double2) * fhat.size(), cudaMemcpyHostToDevice, c->stream);
  size_t nh = 3 * (size_t)nm * g.n2m * g.n3m;
  { MIBM_PROF(c, "hit_modes");
    hit_h_kernel<<<div_up(nh, 256), 256, 0, c->stream>>>(g, nm, h->d_fhat, h->d_ey, h->d_ez, h->d_h); }
  { MIBM_PROF(c, "hit_force");
    hit_force_kernel<<<dim3(div_up(g.n1m, 128), g.n2m, g.n3m), 128, 0, c->stream>>>(
        g, nm, h->d_ex, h->d_h, c->df[MIBM_F_FORCX], c->df[MIBM_F_FORCY], c->df[MIBM_F_FORCZ]); }
  c->launches += 2;
  // the host vector is read by the copy: wait before it goes out of scope
  cuda_ok(c, cudaStreamSynchronize(c->stream), "hit");
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
