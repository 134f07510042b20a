// interp.cu -- restart regrid, interp.f90:1-221 (trilinear interpolation of
// a continuation field from an old uniform grid to the current one).
//
// Drop-in semantics of the reference: arrold is the caller's host array
// (n1o, n2o, kstarto-1:kendo+1) and is modified in place exactly as the
// reference does (periodic copies of column n1o / row n2o, extrapolated
// bottom and top slabs); arrnew is the caller's host array (n1, n2,
// kstart:kend) and receives the result.  The old array goes to the device
// once; one thread per new cell searches the old coordinates (the
// reference's first-bracket linear search) and forms the trilinear weights
// in the reference's operation order (this file is compiled without FMA
// contraction, so the bracket decisions and sums match the oracle).
#include <vector>

#include "common.cuh"

namespace mibm {

// gridnew with istr = 0 (interp.f90:265-311): 1-based, padded to n+2 with the
// second-order extrapolated end points at 0 and n+1 (interp.f90:38-53)
static void grid_uniform(int n, double len, std::vector<double>& rc, std::vector<double>& rm, bool extend) {
  rc.assign(n + 2, 0.0);
  rm.assign(n + 2, 0.0);
  for (int i = 1; i <= n; ++i) rc[i] = len * ((double)(i - 1) / (double)(n - 1));
  for (int i = 1; i <= n - 1; ++i) rm[i] = (rc[i] + rc[i + 1]) * 0.5;
  rm[n] = 2 * rc[n] - rm[n - 1];
  if (extend) {
    rc[0] = 2 * rc[1] - rc[2]; rc[n + 1] = 2 * rc[n] - rc[n - 1];
    rm[0] = 2 * rm[1] - rm[2]; rm[n + 1] = 2 * rm[n] - rm[n - 1];
  }
}

struct InterpArgs {
  int n1o, n2o, n3o, klo;      // old array (n1o, n2o, klo:klo+nk-1)
  int n1, n2, n3m;             // new array (n1, n2, 1:n3m)
  const double* xo; const double* yo; const double* zo;   // 0..n+1
  const double* xn; const double* yn; const double* zn;   // 1-based (index 0 unused)
};

__device__ __forceinline__ void bracket(const double* old, int n, double b, int& f, int& c) {
  f = n - 1; c = n;
  for (int l = 1; l <= n; ++l)
    if (old[l] >= b) { f = l - 1; c = l; return; }
}

__global__ void interp_kernel(InterpArgs a, const double* __restrict__ ao, double* __restrict__ an) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t total = (size_t)a.n1 * a.n2 * a.n3m;
  if (t >= total) return;
  int i = (int)(t % a.n1) + 1, j = (int)((t / a.n1) % a.n2) + 1, k = (int)(t / ((size_t)a.n1 * a.n2)) + 1;
  double bix = a.xn[i], biy = a.yn[j], biz = a.zn[k];
  int bifi, bici, bifj, bicj, bifk, bick;
  bracket(a.xo, a.n1o, bix, bifi, bici);
  bracket(a.yo, a.n2o, biy, bifj, bicj);
  bracket(a.zo, a.n3o, biz, bifk, bick);
  double bix1 = a.xo[bifi], bix2 = a.xo[bici], biy1 = a.yo[bifj], biy2 = a.yo[bicj];
  double biz1 = a.zo[bifk], biz2 = a.zo[bick];
  if (bifi == 0) bifi = a.n1o - 1;
  if (bifj == 0) bifj = a.n2o - 1;
  auto A = [&](int ii, int jj, int kk) {
    return ao[(size_t)(ii - 1) + (size_t)a.n1o * ((size_t)(jj - 1) + (size_t)a.n2o * (size_t)(kk - a.klo))];
  };
  double aficjfk = A(bifi, bicj, bifk), afifjfk = A(bifi, bifj, bifk);
  double acicjfk = A(bici, bicj, bifk), acifjfk = A(bici, bifj, bifk);
  double aficjck = A(bifi, bicj, bick), afifjck = A(bifi, bifj, bick);
  double acicjck = A(bici, bicj, bick), acifjck = A(bici, bifj, bick);
  double dxdydz = 1.0 / ((bix2 - bix1) * (biy2 - biy1) * (biz2 - biz1));
  an[(size_t)(i - 1) + (size_t)a.n1 * ((size_t)(j - 1) + (size_t)a.n2 * (size_t)(k - 1))] =
      (aficjfk * (bix2 - bix) * (biy - biy1) * (biz2 - biz) + afifjfk * (bix2 - bix) * (biy2 - biy) * (biz2 - biz) +
       acicjfk * (bix - bix1) * (biy - biy1) * (biz2 - biz) + acifjfk * (bix - bix1) * (biy2 - biy) * (biz2 - biz) +
       aficjck * (bix2 - bix) * (biy - biy1) * (biz - biz1) + afifjck * (bix2 - bix) * (biy2 - biy) * (biz - biz1) +
       acicjck * (bix - bix1) * (biy - biy1) * (biz - biz1) + acifjck * (bix - bix1) * (biy2 - biy) * (biz - biz1)) *
      dxdydz;
}

void k_interp_restart(Ctx* c, double* arrold, double* arrnew, int n1o, int n2o, int n3o, int intvar, int kstarto,
                      int kendo) {
  const Grid& g = c->g;
  if (n1o < 3 || n2o < 3 || n3o < 3 || kstarto < 1 || kendo < kstarto || kendo > n3o || intvar < 1 || intvar > 4) {
    fail(c, MIBM_EINVAL, "interp_: old grid must be >= 3 per direction, 1 <= kstarto <= kendo <= n3o, intvar 1..4");
    return;
  }
  const int klo = kstarto - 1, nk = kendo - kstarto + 3;
  auto AO = [&](int i, int j, int k) -> double& {
    return arrold[(size_t)(i - 1) + (size_t)n1o * ((size_t)(j - 1) + (size_t)n2o * (size_t)(k - klo))];
  };
  // in-place edits of the old array, interp.f90:60-61 and 95-110
  for (int k = klo; k < klo + nk; ++k)
    for (int j = 1; j <= n2o; ++j) AO(n1o, j, k) = AO(1, j, k);
  for (int k = klo; k < klo + nk; ++k)
    for (int i = 1; i <= n1o; ++i) AO(i, n2o, k) = AO(i, 1, k);
  if (kstarto <= 1)
    for (int i = 1; i <= n1o; ++i)
      for (int j = 1; j <= n2o; ++j) AO(i, j, 0) = 2.0 * AO(i, j, 1) - AO(i, j, 2);
  if (kendo >= n3o)
    for (int i = 1; i <= n1o; ++i)
      for (int j = 1; j <= n2o; ++j) AO(i, j, n3o) = 2.0 * AO(i, j, n3o - 1) - AO(i, j, n3o - 2);
  // grids: old (extended) and new, staggering per variable (interp.f90:62-92)
  const int n1 = g.n1m + 1, n2 = g.n2m + 1, n3 = g.n3m + 1;
  std::vector<double> tc, tm, rc, rm, zz, zm, tcn, tmn, rcn, rmn, zzn, zmn;
  grid_uniform(n1o, g.xlen, tc, tm, true); grid_uniform(n2o, g.ylen, rc, rm, true); grid_uniform(n3o, g.zlen, zz, zm, true);
  grid_uniform(n1, g.xlen, tcn, tmn, false); grid_uniform(n2, g.ylen, rcn, rmn, false); grid_uniform(n3, g.zlen, zzn, zmn, false);
  const std::vector<double>* sel[6];
  switch (intvar) {
    case 1: sel[0] = &tc; sel[1] = &rm; sel[2] = &zm; sel[3] = &tcn; sel[4] = &rmn; sel[5] = &zmn; break;
    case 2: sel[0] = &tm; sel[1] = &rc; sel[2] = &zm; sel[3] = &tmn; sel[4] = &rcn; sel[5] = &zmn; break;
    case 3: sel[0] = &tm; sel[1] = &rm; sel[2] = &zz; sel[3] = &tmn; sel[4] = &rmn; sel[5] = &zzn; break;
    default: sel[0] = &tm; sel[1] = &rm; sel[2] = &zm; sel[3] = &tmn; sel[4] = &rmn; sel[5] = &zmn; break;
  }
  size_t nold = (size_t)n1o * n2o * nk, nnew = (size_t)n1 * n2 * g.n3m;
  size_t glen = 0;
  for (auto* v : sel) glen += v->size();
  double *d_old = nullptr, *d_new = nullptr, *d_grid = nullptr;
  bool ok = cuda_ok(c, cudaMalloc(&d_old, sizeof(double) * nold), "interp") &&
            cuda_ok(c, cudaMalloc(&d_new, sizeof(double) * nnew), "interp") &&
            cuda_ok(c, cudaMalloc(&d_grid, sizeof(double) * glen), "interp");
  if (ok) {
    InterpArgs a;
    a.n1o = n1o; a.n2o = n2o; a.n3o = n3o; a.klo = klo; a.n1 = n1; a.n2 = n2; a.n3m = g.n3m;
    const double** dst[6] = {&a.xo, &a.yo, &a.zo, &a.xn, &a.yn, &a.zn};
    size_t at = 0;
    for (int q = 0; q < 6; ++q) {
      cudaMemcpy(d_grid + at, sel[q]->data(), sizeof(double) * sel[q]->size(), cudaMemcpyHostToDevice);
      *dst[q] = d_grid + at;
      at += sel[q]->size();
    }
    cudaMemcpy(d_old, arrold, sizeof(double) * nold, cudaMemcpyHostToDevice);
    { MIBM_PROF(c, "interp");
      interp_kernel<<<div_up(nnew, 256), 256, 0, c->stream>>>(a, d_old, d_new); }
    ++c->launches;
    if (MIBM_LAUNCH_CHECK(c, "interp"))
      cuda_ok(c, cudaMemcpyAsync(arrnew, d_new, sizeof(double) * nnew, cudaMemcpyDeviceToHost, c->stream), "interp");
    cuda_ok(c, cudaStreamSynchronize(c->stream), "interp");
  }
  cudaFree(d_old); cudaFree(d_new); cudaFree(d_grid);
}

}  // namespace mibm
