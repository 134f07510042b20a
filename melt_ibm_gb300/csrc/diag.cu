// diag.cu -- per-step diagnostics: CalcDissipation (diss.f90:11-201),
// vorticity (vorticity.f90:1-109) and calcFluidVelAvgs (calcSlipVels.f90:
// 17-181).
//
// The three routines sweep the same cells with the same velocity
// differences, so one kernel does all of them: per cell the nine velocity
// gradients of diss.f90:69-105 (the vorticity components are differences of
// the same values, vorticity.f90:45-77), the kinetic energy, the
// dissipation and scalar dissipation rates, and, where the cell is fully
// fluid (VOFp = 1), the 21 running sums.  Each thread sums its cells in a
// fixed grid-stride order, each block combines its threads with a fixed
// shuffle tree, and one block adds the block sums in block order, so the
// result is deterministic (no atomics).  The few derived numbers (eta,
// Re_lambda, ...) are formed on the host from the sums.
//
// With mibm_set_diagnostics_(1) the kernels are part of every tschem_ step
// (and its graph) and the sums come back with the step's end-of-step copies,
// so a host that logs them every step pays no extra synchronisation.
#include <cmath>
#include <cstddef>
#include <cstring>

#include "common.cuh"

namespace mibm {

constexpr int kDiagSums = 21;
constexpr int kDiagThreads = 256;
constexpr int kDiagBlocks = 304;          // 2 per SM on a GB300

struct DiagArgs {
  Grid g;
  const double *u, *v, *w, *t, *vof;
  const double* vcm;                      // vel_CM (device)
  double ren, pec, tliq;
};

__device__ __forceinline__ double sq(double x) { return x * x; }

// sums: [sumVOF, kenerg, diss, chi, enstrophy, count, u(3), u^2(3),
//        u - vel_CM (3), (u - vel_CM)^2 (3), T, T - Tliq, (T - Tliq)^2]
__global__ void __launch_bounds__(kDiagThreads) diag_kernel(DiagArgs a, double* __restrict__ part) {
  const Grid& g = a.g;
  double s[kDiagSums];
  for (int q = 0; q < kDiagSums; ++q) s[q] = 0.0;
  const double udx1 = g.dx1, udx2 = g.dx2, udx3 = g.dx3;
  const double vc0 = a.vcm[0], vc1 = a.vcm[1], vc2 = a.vcm[2];
  const size_t n = (size_t)g.n1m * g.n2m * g.n3m;
  for (size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x; cell < n; cell += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(cell % g.n1m), j = (int)((cell / g.n1m) % g.n2m), k = (int)(cell / ((size_t)g.n1m * g.n2m));
    size_t c0 = cidx(g, i, j, k);
    if (a.vof[c0] != 1.0) continue;                  // only fully fluid cells enter any sum
    int ip = wrap(i + 1, g.n1m), im = wrap(i - 1, g.n1m);
    int jp = wrap(j + 1, g.n2m), jm = wrap(j - 1, g.n2m);
    int kp = wrap(k + 1, g.n3m), km = wrap(k - 1, g.n3m);
    auto U = [&](int ii, int jj, int kk) { return a.u[cidx(g, ii, jj, kk)]; };
    auto V = [&](int ii, int jj, int kk) { return a.v[cidx(g, ii, jj, kk)]; };
    auto W = [&](int ii, int jj, int kk) { return a.w[cidx(g, ii, jj, kk)]; };
    auto T = [&](int ii, int jj, int kk) { return a.t[cidx(g, ii, jj, kk)]; };
    double h11 = (U(ip, j, k) - U(i, j, k)) * udx1;
    double h12 = ((U(i, jp, k) + U(ip, jp, k)) - (U(i, jm, k) + U(ip, jm, k))) * 0.25 * udx2;
    double h13 = ((U(i, j, kp) + U(ip, j, kp)) - (U(i, j, km) + U(ip, j, km))) * 0.25 * udx3;
    double h21 = ((V(ip, j, k) + V(ip, jp, k)) - (V(im, j, k) + V(im, jp, k))) * 0.25 * udx1;
    double h22 = (V(i, jp, k) - V(i, j, k)) * udx2;
    double h23 = ((V(i, j, kp) + V(i, jp, kp)) - (V(i, j, km) + V(i, jp, km))) * 0.25 * udx3;
    double h31 = ((W(ip, j, k) + W(ip, j, kp)) - (W(im, j, k) + W(im, j, kp))) * 0.25 * udx1;
    double h32 = ((W(i, jp, k) + W(i, jp, kp)) - (W(i, jm, k) + W(i, jm, kp))) * 0.25 * udx2;
    double h33 = (W(i, j, kp) - W(i, j, k)) * udx3;
    double uc = U(i, j, k), vcc = V(i, j, k), wc = W(i, j, k), tc = T(i, j, k);
    double tke = (sq(uc) + sq(U(ip, j, k)) + sq(vcc) + sq(V(i, jp, k)) + sq(wc) + sq(W(i, j, kp))) * 0.5;
    tke = tke * 0.5;
    double diss = sq(h11) + sq(h22) + sq(h33) + 0.5 * sq(h21 + h12) + 0.5 * sq(h31 + h13) + 0.5 * sq(h32 + h23);
    diss = diss * 2.0 / a.ren;
    double chi = sq(0.5 * g.dx1 * (T(ip, j, k) - T(im, j, k))) + sq(0.5 * g.dx2 * (T(i, jp, k) - T(i, jm, k))) +
                 sq(0.5 * g.dx3 * (T(i, j, kp) - T(i, j, km)));
    chi = chi / a.pec;
    double vorx = h32 - h23, vory = h13 - h31, vorz = h21 - h12;
    s[0] += 1.0; s[1] += tke; s[2] += diss; s[3] += chi;
    s[4] += sq(vorx) + sq(vory) + sq(vorz);
    s[5] += 1.0;
    s[6] += uc; s[7] += vcc; s[8] += wc;
    s[9] += sq(uc); s[10] += sq(vcc); s[11] += sq(wc);
    s[12] += uc - vc0; s[13] += vcc - vc1; s[14] += wc - vc2;
    s[15] += sq(uc - vc0); s[16] += sq(vcc - vc1); s[17] += sq(wc - vc2);
    s[18] += tc; s[19] += tc - a.tliq; s[20] += sq(tc - a.tliq);
  }
  __shared__ double ws[kDiagThreads / 32][kDiagSums];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < kDiagSums; ++q) {
    double v = s[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) ws[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kDiagSums) {
    double v = ws[0][threadIdx.x];
    for (int w = 1; w < kDiagThreads / 32; ++w) v += ws[w][threadIdx.x];
    part[kDiagSums * (size_t)blockIdx.x + threadIdx.x] = v;
  }
}

__global__ void diag_final_kernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
  int q = threadIdx.x;
  if (q >= kDiagSums) return;
  double v = 0.0;
  for (int b = 0; b < nb; ++b) v += part[kDiagSums * (size_t)b + q];
  out[q] = v;
}

// diss.f90:160-186, vorticity.f90:93-95, calcSlipVels.f90:134-168
static void diag_derive(const double* s, double ren, double* out) {
  double nu = 1.0 / ren;
  double sumvof = s[0];
  double kenerg = s[1] / sumvof, diss = s[2] / sumvof, chi = s[3] / sumvof;
  double urms = std::sqrt(2.0 / 3.0 * kenerg);
  double eta = std::pow(nu * nu * nu / diss, 0.25);
  double Re_L = kenerg * kenerg / (nu * diss);
  double lambda_t = std::sqrt(15.0 * nu * urms * urms / diss);
  double re_lam = urms * lambda_t / nu;
  double L_int = std::sqrt(kenerg * kenerg * kenerg) / diss;
  double n = s[5];
  double o[MIBM_NDIAG] = {diss, kenerg, urms, eta, lambda_t, Re_L, re_lam, L_int, chi, s[4] / sumvof, n,
                          s[6] / n, s[7] / n, s[8] / n, s[9] / n, s[10] / n, s[11] / n,
                          s[12] / n, s[13] / n, s[14] / n, s[15] / n, s[16] / n, s[17] / n,
                          s[18] / n, s[19] / n, s[20] / n};
  memcpy(out, o, sizeof(o));
}

struct DiagState {
  double* part = nullptr;      // device: block sums, then the 21 totals
  double* host = nullptr;      // pinned: totals read back at the end of a step
};
static DiagState* diag_of(Ctx* c) {
  if (!c->diag) c->diag = new DiagState();
  return (DiagState*)c->diag;
}

static bool diag_ensure(Ctx* c) {
  DiagState* d = diag_of(c);
  if (d->part) return true;
  if (!cuda_ok(c, cudaMalloc(&d->part, sizeof(double) * kDiagSums * (kDiagBlocks + 1)), "diagnostics")) return false;
  if (!cuda_ok(c, cudaMallocHost((void**)&d->host, sizeof(double) * kDiagSums), "diagnostics")) return false;
  return true;
}

// Enqueue: re-tag a moving body (diss.f90:47-50), the sweep, the totals and
// their copy into pinned memory.  vcm: device address of vel_CM.
void diag_enqueue(Ctx* c, const double* vcm) {
  if (!diag_ensure(c)) return;
  DiagState* d = diag_of(c);
  if (!c->I(MIBM_I_STATIONARY) && c->I(MIBM_I_IMLSFOR) == 1) lagr_tag_narrow_band(c);
  DiagArgs a;
  a.g = c->g;
  a.u = c->df[MIBM_F_VX]; a.v = c->df[MIBM_F_VY]; a.w = c->df[MIBM_F_VZ]; a.t = c->df[MIBM_F_TEMP];
  a.vof = c->df[MIBM_F_VOFP];
  a.vcm = vcm;
  a.ren = c->S(MIBM_S_REN); a.pec = c->S(MIBM_S_PEC); a.tliq = c->S(MIBM_S_TLIQ);
  double* totals = d->part + (size_t)kDiagSums * kDiagBlocks;
  { MIBM_PROF(c, "diagnostics");
    diag_kernel<<<kDiagBlocks, kDiagThreads, 0, c->stream>>>(a, d->part);
    diag_final_kernel<<<1, 32, 0, c->stream>>>(d->part, kDiagBlocks, totals); }
  c->launches += 2;
  if (MIBM_LAUNCH_CHECK(c, "diagnostics"))
    cudaMemcpyAsync(d->host, totals, sizeof(double) * kDiagSums, cudaMemcpyDeviceToHost, c->stream);
}

// After the stream has completed: the numbers of the last enqueue.
void diag_finish(Ctx* c) {
  DiagState* d = diag_of(c);
  if (!d->host) return;
  diag_derive(d->host, c->S(MIBM_S_REN), c->diag_last);
  c->diag_valid = true;
}

void diag_free(Ctx* c) {
  if (!c->diag) return;
  DiagState* d = (DiagState*)c->diag;
  cudaFree(d->part);
  if (d->host) cudaFreeHost(d->host);
  delete d;
  c->diag = nullptr;
}

}  // namespace mibm
