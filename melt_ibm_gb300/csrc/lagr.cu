// lagr.cu -- immersed-boundary (Lagrangian) part of the substep.
//
// Restates on the device:
//   findCentroidIndices.f90:14-50           centroid cage indices
//   mlsWeight.f90:48-412, geom.f90:24-53     MLS shape functions (FP64 4x4 LU)
//   mlsForce.f90:13-33, forc1/2/3/temp.f90  interpolation + force spreading
//   velforce.f90:13-52, tempforce.f90:13-40 mean removal and field update
//   findProbeIndices.f90:20-74              +/- normal probe cages
//   mls_heatFlux.f90:77-395                 MLS gradient of T, face->vertex
//   stefanCondition.f90:12-31               Stefan front advance
//   triaux.f90:53-323, RigidAuxRoutines.f90:653-780  geometry refresh
//   genSDF.f90:120-365, tagCells.f90:85-111 narrow-band tagging
//   pencil_rayTag.f90:37-460                initial full tagging
//
// Determinism: no floating-point atomics anywhere.  Force spreading is an
// atomics-free sorted scatter: the 27 cage cells of every triangle are keyed
// by cell index and stably radix-sorted once per geometry (the key order
// depends only on the mesh), then each unique cell sums its contributions in
// triangle order -- the reference's summation order.  Face->vertex sums use
// a vertex->face adjacency list in ascending face order.  The narrow band
// takes the minimum distance with 64-bit integer atomicMin on the
// (non-negative) IEEE bit pattern and the earliest triangle among equal
// distances, exactly the strict "<" update rule of genSDF.f90:167.
#include <climits>
#include <string>
#include <cstddef>
#include <cmath>
#include <utility>
#include <vector>

#include "common.cuh"
#include "mls_exp.h"

namespace mibm {

// ---------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------
struct LagArgs {
  Grid g;
  int nf, nv, coff, clen;
  const double* xc; const double* xm; const double* yc; const double* ym; const double* zc; const double* zm;
  double wcon, wscl;
};

static LagArgs lag_args(Ctx* c) {
  LagArgs a;
  a.g = c->g; a.nf = c->maxnf; a.nv = c->maxnv; a.coff = c->coord_off; a.clen = 3 * c->coord_off;
  a.xc = c->xc; a.xm = c->xm; a.yc = c->yc; a.ym = c->ym; a.zc = c->zc; a.zm = c->zm;
  a.wcon = c->S(MIBM_S_WCON); a.wscl = c->S(MIBM_S_WSCL);
  return a;
}

template <typename T> static T* M(Ctx* c, int id) { return (T*)c->dm[id]; }

__device__ __forceinline__ int ffloor(double x) { return (int)floor(x); }
__device__ __forceinline__ int fnint(double x) { return (int)round(x); }
__device__ __forceinline__ double sqd(double x) { return x * x; }

__device__ __forceinline__ double coord(const LagArgs& A, int dir, int sel, int idx) {
  // sel 0 = c (face) coordinates, 1 = m (centre).  The tables span
  // [-coff, 2*coff) grid indices, more than the reference's -n..2n; a body
  // outside that range is clamped instead of read out of bounds.
  int t = min(max(idx + A.coff, 0), A.clen - 1);
  if (dir == 0) return sel == 0 ? A.xc[t] : A.xm[t];
  if (dir == 1) return sel == 0 ? A.yc[t] : A.ym[t];
  return sel == 0 ? A.zc[t] : A.zm[t];
}

// Gaussian weight and its radial derivative (geom.f90:24-53).  exp is the
// written-out mls_exp (mls_exp.h), shared with the oracle, so that the
// plain form's MLS construction gives the oracle's bits.
__device__ __forceinline__ double mls_gaussian(double r, double rcoef) { return (r > 1.0) ? 0.0 : mls_exp(-sqd(r / rcoef)); }
__device__ __forceinline__ double mls_gauss_deriv(double r, double rcoef) {
  return (r > 1.0) ? 0.0 : -2.0 * r / sqd(rcoef) * mls_exp(-sqd(r / rcoef));
}

// In-place inverse of a 4x4 column-major matrix: LU with partial pivoting
// (dgetrf semantics, first maximal pivot) and inversion from the factors
// (dgetri).  Returns false if a pivot is exactly zero.
__device__ bool inv4(double* a) {
  const int n = 4;
  int ipiv[4];
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(a[j + n * j]);
    for (int i = j + 1; i < n; ++i)
      if (fabs(a[i + n * j]) > amax) { amax = fabs(a[i + n * j]); p = i; }
    ipiv[j] = p;
    if (a[p + n * j] == 0.0) return false;
    if (p != j)
      for (int cc = 0; cc < n; ++cc) { double t = a[j + n * cc]; a[j + n * cc] = a[p + n * cc]; a[p + n * cc] = t; }
    double r = 1.0 / a[j + n * j];
    for (int i = j + 1; i < n; ++i) a[i + n * j] *= r;
    for (int cc = j + 1; cc < n; ++cc) {
      double t = a[j + n * cc];
      for (int i = j + 1; i < n; ++i) a[i + n * cc] -= t * a[i + n * j];
    }
  }
  for (int j = 0; j < n; ++j) {
    a[j + n * j] = 1.0 / a[j + n * j];
    double ajj = -a[j + n * j];
    for (int i = 0; i < j; ++i) {
      double s = 0;
      for (int k = i; k < j; ++k) s += a[i + n * k] * a[k + n * j];
      a[i + n * j] = s;
    }
    for (int i = 0; i < j; ++i) a[i + n * j] *= ajj;
  }
  double work[4];
  for (int j = n - 1; j >= 0; --j) {
    for (int i = j + 1; i < n; ++i) { work[i] = a[i + n * j]; a[i + n * j] = 0.0; }
    if (j < n - 1)
      for (int i = 0; i < n; ++i) {
        double s = 0;
        for (int k = j + 1; k < n; ++k) s += a[i + n * k] * work[k];
        a[i + n * j] -= s;
      }
  }
  for (int j = n - 2; j >= 0; --j) {
    int jp = ipiv[j];
    if (jp != j)
      for (int i = 0; i < n; ++i) { double t = a[i + n * j]; a[i + n * j] = a[i + n * jp]; a[i + n * jp] = t; }
  }
  return true;
}

// ---------------------------------------------------------------------
// findCentroidIndices / findProbeIndices
// ---------------------------------------------------------------------
__global__ void centroid_idx_kernel(LagArgs A, const double* __restrict__ tri_bar, const int* __restrict__ ghost,
                                    int* __restrict__ pind) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nf || ghost[t]) return;
  const Grid& g = A.g;
  double px = tri_bar[3 * t], py = tri_bar[3 * t + 1], pz = tri_bar[3 * t + 2];
  int i1 = ffloor(px * g.dx1) + 1, ist = fnint(px * g.dx1) + 1;
  int j1 = ffloor(py * g.dx2) + 1, jst = fnint(py * g.dx2) + 1;
  int k1 = ffloor(pz * g.dx3) + 1, kst = fnint(pz * g.dx3) + 1;
  k1 = fmod_pos(k1 - 1, g.n3m) + 1;
  kst = fmod_pos(kst - 1, g.n3m) + 1;
  int* p = pind + 6 * t;
  p[0] = i1; p[1] = j1; p[2] = k1; p[3] = ist; p[4] = jst; p[5] = kst;
}

__global__ void probe_idx_kernel(LagArgs A, const double* __restrict__ tri_bar, const double* __restrict__ tri_nor,
                                 const int* __restrict__ ghost, double h, int* __restrict__ pind) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nf || ghost[t]) return;
  const Grid& g = A.g;
  double n0 = tri_nor[3 * t], n1 = tri_nor[3 * t + 1], n2 = tri_nor[3 * t + 2];
  double s = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  for (int side = 0; side < 2; ++side) {
    double pos[3];
    for (int d = 0; d < 3; ++d) {
      double nd = tri_nor[3 * t + d];
      pos[d] = side == 0 ? tri_bar[3 * t + d] + h * nd / s : tri_bar[3 * t + d] - h * nd / s;
    }
    int i1 = ffloor(pos[0] * g.dx1) + 1, j1 = ffloor(pos[1] * g.dx2) + 1, k1 = ffloor(pos[2] * g.dx3) + 1;
    k1 = fmod_pos(k1 - 1, g.n3m) + 1;
    pind[6 * t + 3 * side + 0] = i1; pind[6 * t + 3 * side + 1] = j1; pind[6 * t + 3 * side + 2] = k1;
  }
}

// ---------------------------------------------------------------------
// mlsWeight: one thread per (triangle, component)
// component 0 = wght1 (vx), 1 = wght2 (vy), 2 = wght3 (vz), 3 = wghttemp
// ---------------------------------------------------------------------
struct CageSpec {
  int ix, iy;      // pind slot (0-based) of the x and y cage centre
  int sx, sy, sz;  // coordinate selector per axis (0 = c, 1 = m)
  bool znint;      // z centre from nint (wght3) or floor
};
__device__ __forceinline__ CageSpec cage_spec(int comp) {
  switch (comp) {
    case 0: return CageSpec{3, 1, 0, 1, 1, false};   // xc, ym, zm ; pind(4), pind(2)
    case 1: return CageSpec{0, 4, 1, 0, 1, false};   // xm, yc, zm ; pind(1), pind(5)
    case 2: return CageSpec{0, 1, 1, 1, 0, true};    // xm, ym, zc ; pind(1), pind(2)
  }
  return CageSpec{0, 1, 1, 1, 1, false};             // xm, ym, zm ; pind(1), pind(2)
}

// The reference's MLS shape functions at pos for the 27-point cage centred on
// (i0, j0, k0) with per-axis staggering sx, sy, sz (mls_shape of wght1/2/3/
// temp, mlsWeight.f90:48-412, and of wght_press, mls_structLoads.f90:271-
// 404): basis [1, x, y, z] in absolute coordinates, A = sum W p p^T by
// rank-one updates in cage order, A^-1 by LU with partial pivoting, then
// phi = (p(x)^T A^-1) B.  IEEE operations in the oracle's order (this file is
// compiled without FMA contraction): the same bits.  Returns false on a
// singular A.
__device__ bool shape_lit(const LagArgs& A, const double pos[3], int i0, int j0, int k0, int sx, int sy, int sz,
                          double out[27]) {
  const Grid& g = A.g;
  const double ptx[4] = {1.0, pos[0], pos[1], pos[2]};
  // separable Gaussian weights (the reference evaluates the same 9 values)
  double wz[3], wy[3], wx[3], cz[3], cy[3], cx[3];
  for (int q = 0; q < 3; ++q) {
    cz[q] = coord(A, 2, sz, k0 - 1 + q);
    cy[q] = coord(A, 1, sy, j0 - 1 + q);
    cx[q] = coord(A, 0, sx, i0 - 1 + q);
    wz[q] = mls_gaussian(fabs(cz[q] - pos[2]) / (A.wscl / g.dx3), A.wcon);
    wy[q] = mls_gaussian(fabs(cy[q] - pos[1]) / (A.wscl / g.dx2), A.wcon);
    wx[q] = mls_gaussian(fabs(cx[q] - pos[0]) / (A.wscl / g.dx1), A.wcon);
  }
  double Am[16];
  for (int q = 0; q < 16; ++q) Am[q] = 0.0;
  for (int kk = 0; kk < 3; ++kk)
    for (int jj = 0; jj < 3; ++jj) {
      double w23 = wy[jj] * wz[kk];
      for (int ii = 0; ii < 3; ++ii) {
        double wtx = wx[ii] * w23;
        double pk[4] = {1.0, cx[ii], cy[jj], cz[kk]};
        for (int cc = 0; cc < 4; ++cc) {
          double tt = wtx * pk[cc];
          for (int r = 0; r < 4; ++r) Am[r + 4 * cc] = Am[r + 4 * cc] + tt * pk[r];
        }
      }
    }
  if (!inv4(Am)) return false;
  double ptxA[4];
  for (int cc = 0; cc < 4; ++cc) {
    double s = 0;
    for (int r = 0; r < 4; ++r) s += ptx[r] * Am[r + 4 * cc];
    ptxA[cc] = s;
  }
  for (int kk = 0; kk < 3; ++kk)
    for (int jj = 0; jj < 3; ++jj) {
      double w23 = wy[jj] * wz[kk];
      for (int ii = 0; ii < 3; ++ii) {
        double wtx = wx[ii] * w23;
        // B(:,n) = wtx * [1, x, y, z]
        out[ii + 3 * jj + 9 * kk] =
            ptxA[0] * (wtx * 1.0) + ptxA[1] * (wtx * cx[ii]) + ptxA[2] * (wtx * cy[jj]) + ptxA[3] * (wtx * cz[kk]);
      }
    }
  return true;
}

// One thread per (triangle, component): the serial order of the reference,
// and the fewest FP64 operations (the part's scarce resource).
__global__ void mls_weight_kernel(LagArgs A, const double* __restrict__ tri_bar, const int* __restrict__ ghost,
                                  const int* __restrict__ pind, double* __restrict__ p1, double* __restrict__ p2,
                                  double* __restrict__ p3, double* __restrict__ pt, int* __restrict__ flag) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  int t = gid >> 2, comp = gid & 3;
  if (t >= A.nf || ghost[t]) return;
  const Grid& g = A.g;
  double pos[3] = {tri_bar[3 * t], tri_bar[3 * t + 1], tri_bar[3 * t + 2]};
  CageSpec cs = cage_spec(comp);
  int i0 = pind[6 * t + cs.ix], j0 = pind[6 * t + cs.iy];
  int k0 = cs.znint ? fnint(pos[2] * g.dx3) + 1 : ffloor(pos[2] * g.dx3) + 1;
  double* out = (comp == 0) ? p1 : (comp == 1) ? p2 : (comp == 2) ? p3 : pt;
  double phi[27];
  if (!shape_lit(A, pos, i0, j0, k0, cs.sx, cs.sy, cs.sz, phi)) { atomicOr(flag, 1); return; }
  out += 27 * (size_t)t;
  for (int n = 0; n < 27; ++n) out[n] = phi[n];
}

// Weight and weight derivative of one cage coordinate for the literal
// gradient, as wght_grad_field evaluates them (mls_heatFlux.f90:166-185):
// norp = |pos - pc| / (wscl/dx); W = gaussian(norp); dW = 0 at norp < eps,
// else gauss_deriv(norp) * ((pos - pc) / |pos - pc| / (wscl/dx)).  The
// Gaussian's exp is evaluated once for both (the same value either way).
__device__ __forceinline__ void lit_axis_weight(const LagArgs& A, double pos, double pc, double dx, double eps,
                                                double& W, double& dW) {
  const double diff = pos - pc;
  const double norp = fabs(diff) / (A.wscl / dx);
  if (norp > 1.0) {
    W = 0.0;
    dW = 0.0;
    return;
  }
  const double e = mls_exp(-sqd(norp / A.wcon));
  W = e;
  dW = (norp < eps) ? 0.0 : (-2.0 * norp / sqd(A.wcon) * e) * (diff / fabs(diff) / (A.wscl / dx));
}

// The reference's MLS gradient at a probe, literally (wght_gradT,
// mls_heatFlux.f90:161-376; wght_gradP/U/V/W, mls_structLoads.f90:406-1298):
// basis [1, x, y, z] in absolute coordinates; A, dA/dx_d, B, dB/dx_d
// accumulated point by point in cage order (z layer, y, x) as the reference's
// rank-one DGEMM updates; A^-1 by LU with partial pivoting; gamma = A^-1 p(x);
//   d phi / dx_d = (A^-1 (e_d - dA_d gamma))^T B + gamma^T dB_d,
// contracted with the field over the cage.  Cage i, j around (pi1, pi2);
// z layers [k1-1, k1, k1] (the repeated layer of mls_heatFlux.f90:213) with
// k1 = floor(z*dx3)+1, or nint for the w-velocity; coordinates per axis from
// the field's staggering (sel 0 = face, 1 = centre); field values at the
// wrapped cage, z from [k1w-1, k1w, k1w+1].  Every operation is the oracle's
// (wght_grad_field) in its order, so the two agree bit for bit.  B and dB are
// not stored: each entry is a product of per-axis weight factors and a basis
// entry, recomputed where it is used from the same factors in the same order
// (the same bits); dA_d is accumulated in its own pass per direction.
// Returns false on a singular A.
__device__ bool probe_grad_lit(const LagArgs& A, const double pos[3], int pi1, int pi2, int sx, int sy, int sz,
                               bool knint, const double* __restrict__ q, double grad[3]) {
  const Grid& g = A.g;
  const double eps = 2.220446049250313e-16;       // EPSILON(1.0d0)
  const double ptx[4] = {1.0, pos[0], pos[1], pos[2]};
  const int k1 = knint ? fnint(pos[2] * g.dx3) + 1 : ffloor(pos[2] * g.dx3) + 1;
  const int kin[3] = {k1 - 1, k1, k1};
  const int k1w = fmod_pos(k1 - 1, g.n3m) + 1;
  const int keul[3] = {k1w - 1, k1w, k1w + 1};
  double pc[3][3], W[3][3], dW[3][3];             // [axis][point]
  for (int r = 0; r < 3; ++r) {
    pc[0][r] = coord(A, 0, sx, pi1 - 1 + r);
    pc[1][r] = coord(A, 1, sy, pi2 - 1 + r);
    pc[2][r] = coord(A, 2, sz, kin[r]);
  }
  const double dxa[3] = {g.dx1, g.dx2, g.dx3};
  for (int a = 0; a < 3; ++a)
    for (int r = 0; r < 3; ++r) lit_axis_weight(A, pos[a], pc[a][r], dxa[a], eps, W[a][r], dW[a][r]);
  double Am[16];
  for (int e = 0; e < 16; ++e) Am[e] = 0.0;
  for (int nk = 0; nk < 3; ++nk)
    for (int j = 0; j < 3; ++j) {
      const double w23 = W[1][j] * W[2][nk];
      for (int i = 0; i < 3; ++i) {
        const double wtx = W[0][i] * w23;
        const double pk[4] = {1.0, pc[0][i], pc[1][j], pc[2][nk]};
        for (int cc = 0; cc < 4; ++cc) {
          const double t = wtx * pk[cc];
          for (int r = 0; r < 4; ++r) Am[r + 4 * cc] = Am[r + 4 * cc] + t * pk[r];
        }
      }
    }
  if (!inv4(Am)) return false;
  double gam[4];
  for (int r = 0; r < 4; ++r) {                   // DGEMV('N', invA, ptx)
    double t = 0;
    for (int cc = 0; cc < 4; ++cc) t += Am[r + 4 * cc] * ptx[cc];
    gam[r] = t;
  }
  const int kk_[3] = {wrap(keul[0] - 1, g.n3m), wrap(keul[1] - 1, g.n3m), wrap(keul[2] - 1, g.n3m)};
  for (int d = 0; d < 3; ++d) {
    double dA[16];
    for (int e = 0; e < 16; ++e) dA[e] = 0.0;
    for (int nk = 0; nk < 3; ++nk)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          const double dwd = d == 0 ? (dW[0][i] * W[1][j]) * W[2][nk]
                           : d == 1 ? (W[0][i] * dW[1][j]) * W[2][nk]
                                    : (W[0][i] * W[1][j]) * dW[2][nk];
          const double pk[4] = {1.0, pc[0][i], pc[1][j], pc[2][nk]};
          for (int cc = 0; cc < 4; ++cc) {
            const double t = dwd * pk[cc];
            for (int r = 0; r < 4; ++r) dA[r + 4 * cc] = dA[r + 4 * cc] + t * pk[r];
          }
        }
    double pk_d[4] = {0.0, 0.0, 0.0, 0.0};
    pk_d[d + 1] = 1.0;
    for (int r = 0; r < 4; ++r) {                 // pk = -dA gamma + pk
      double t = 0;
      for (int cc = 0; cc < 4; ++cc) t += dA[r + 4 * cc] * gam[cc];
      pk_d[r] = pk_d[r] - t;
    }
    double dgam[4];
    for (int r = 0; r < 4; ++r) {
      double t = 0;
      for (int cc = 0; cc < 4; ++cc) t += Am[r + 4 * cc] * pk_d[cc];
      dgam[r] = t;
    }
    double gsum = 0;
    for (int nk = 0; nk < 3; ++nk)
      for (int j = 0; j < 3; ++j) {
        const int jj = fmod_pos(pi2 - 1 + j - 1, g.n2m);
        const double w23 = W[1][j] * W[2][nk];
        for (int i = 0; i < 3; ++i) {
          const double wtx = W[0][i] * w23;
          const double dwd = d == 0 ? (dW[0][i] * W[1][j]) * W[2][nk]
                           : d == 1 ? (W[0][i] * dW[1][j]) * W[2][nk]
                                    : (W[0][i] * W[1][j]) * dW[2][nk];
          const double pk[4] = {1.0, pc[0][i], pc[1][j], pc[2][nk]};
          double t1 = 0, t2 = 0;
          for (int r = 0; r < 4; ++r) t1 += dgam[r] * (wtx * pk[r]);
          for (int r = 0; r < 4; ++r) t2 += gam[r] * (dwd * pk[r]);
          const double T = q[cidx(g, fmod_pos(pi1 - 1 + i - 1, g.n1m), jj, kk_[nk])];
          gsum += (t1 + t2) * T;
        }
      }
    grad[d] = gsum;
  }
  return true;
}

// The reference's MLS value at a probe, literally (wght_press,
// mls_structLoads.f90:271-404): shape functions of the cell-centred cage
// around (i0, j0), z layers k1-1, k1, k1+1 with k1 = floor(z*dx3)+1, summed
// against the field in cage order as the oracle does.
__device__ bool probe_value_lit(const LagArgs& A, const double pos[3], int i0, int j0, const double* __restrict__ q,
                                double& val) {
  const Grid& g = A.g;
  const int k1 = ffloor(pos[2] * g.dx3) + 1;
  double phi[27];
  if (!shape_lit(A, pos, i0, j0, k1, 1, 1, 1, phi)) return false;
  const int k1w = fmod_pos(k1 - 1, g.n3m) + 1;
  double v = 0.0;
  int inw = 0;
  for (int kk = 0; kk < 3; ++kk) {
    const int kc = wrap(k1w - 1 + kk - 1, g.n3m);
    for (int j = 0; j < 3; ++j) {
      const int jj = fmod_pos(j0 - 1 + j - 1, g.n2m);
      for (int i = 0; i < 3; ++i) {
        v = v + q[cidx(g, fmod_pos(i0 - 1 + i - 1, g.n1m), jj, kc)] * phi[inw];
        ++inw;
      }
    }
  }
  val = v;
  return true;
}

// ---------------------------------------------------------------------
// mlsForce: interpolation Um per (triangle, component) and coefficient
// cfac*(target - Um); the spread goes through the sorted scatter plan.
// ---------------------------------------------------------------------
struct ForceArgs {
  const double* q[4];       // vx, vy, vz, temp (compact)
  const double* ptx[4];
  const double* vel_tri;
  const double* cfac;
  const int* pind;
  const int* ghost;
};

__device__ __forceinline__ void cage_center(int comp, const int* p, int& i0, int& j0, int& k0) {
  // forc1: pind(4), pind(2), pind(3); forc2: pind(1), pind(5), pind(3)
  // forc3: pind(1), pind(2), pind(6); forctemp: pind(1), pind(2), pind(3)
  switch (comp) {
    case 0: i0 = p[3]; j0 = p[1]; k0 = p[2]; return;
    case 1: i0 = p[0]; j0 = p[4]; k0 = p[2]; return;
    case 2: i0 = p[0]; j0 = p[1]; k0 = p[5]; return;
  }
  i0 = p[0]; j0 = p[1]; k0 = p[2];
}

__device__ __forceinline__ size_t cage_cell(const Grid& g, int i0, int j0, int k0, int slot) {
  int ii = fmod_pos(i0 - 2 + slot % 3, g.n1m);
  int jj = fmod_pos(j0 - 2 + (slot / 3) % 3, g.n2m);
  int kk = fmod_pos(k0 - 2 + slot / 9, g.n3m);
  return cidx(g, ii, jj, kk);
}

__global__ void force_coef_kernel(Grid g, int nf, ForceArgs F, double tmelt, double* __restrict__ coef) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  int t = gid >> 2, comp = gid & 3;
  if (t >= nf) return;
  if (F.ghost[t]) { coef[comp * (size_t)nf + t] = 0.0; return; }
  int i0, j0, k0;
  cage_center(comp, F.pind + 6 * t, i0, j0, k0);
  const double* phi = F.ptx[comp] + 27 * (size_t)t;
  const double* q = F.q[comp];
  double Um = 0.0;
  for (int s = 0; s < 27; ++s) Um = Um + q[cage_cell(g, i0, j0, k0, s)] * phi[s];
  double target = (comp == 3) ? tmelt : F.vel_tri[3 * t + comp];
  coef[comp * (size_t)nf + t] = F.cfac[t] * (target - Um);
}

// ---------------------------------------------------------------------
// Stable LSD radix sort of (key, value) pairs, 8-bit digits.
// ---------------------------------------------------------------------
constexpr int kSortChunk = 4096;

// The four cage sets (x, y, z staggered, cell-centred) are merged into one
// plan: entry e = comp*27*nf + 27*t + slot, key = comp*cells + cage cell
// (4*cells, after every cell, for ghost faces).  The plan depends only on the cage centres
// (pind) and the ghost flags; `plan_check` compares them with the values the
// plan was built from and every kernel of the rebuild returns at once when
// nothing changed, so a rebuild costs nothing on a stationary cage.
__global__ void plan_check_kernel(int nf, const int* __restrict__ pind, const int* __restrict__ ghost,
                                  const int* __restrict__ saved, int* __restrict__ dirty,
                                  const StepParams* __restrict__ pp) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0 && pp && pp->force_plan) atomicOr(dirty, 1);   // rebuild requested by the host
  if (t >= nf) return;
  const int* sv = saved + 7 * (size_t)t;
  bool diff = (sv[6] != ghost[t]);
  if (!ghost[t])
    for (int q = 0; q < 6; ++q) diff = diff || (sv[q] != pind[6 * t + q]);
  if (diff) atomicOr(dirty, 1);
}

__global__ void plan_commit_kernel(int nf, const int* __restrict__ pind, const int* __restrict__ ghost,
                                   int* __restrict__ saved, const int* __restrict__ dirty) {
  if (!*dirty) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  for (int q = 0; q < 6; ++q) saved[7 * (size_t)t + q] = pind[6 * t + q];
  saved[7 * (size_t)t + 6] = ghost[t];
}

__global__ void plan_keys_kernel(Grid g, int nf, const int* __restrict__ pind, const int* __restrict__ ghost,
                                 const int* __restrict__ dirty, int* __restrict__ key, int* __restrict__ src) {
  if (!*dirty) return;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  int per = 27 * nf;
  if (e >= 4 * per) return;
  int comp = e / per, r = e % per, t = r / 27, sl = r % 27;
  if (ghost[t]) { key[e] = (int)(4 * g.cells); src[e] = e; return; }   // sorts after every cell
  int i0, j0, k0;
  cage_center(comp, pind + 6 * t, i0, j0, k0);
  key[e] = (int)((size_t)comp * g.cells + cage_cell(g, i0, j0, k0, sl));
  src[e] = e;
}

__global__ void radix_hist_kernel(const int* __restrict__ key, int n, int shift, int nblk,
                                  const int* __restrict__ dirty, int* __restrict__ hist) {
  if (!*dirty) return;
  __shared__ int h[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
  __syncthreads();
  int b = blockIdx.x;
  int end = min(n, (b + 1) * kSortChunk);
  for (int e = b * kSortChunk + threadIdx.x; e < end; e += blockDim.x) atomicAdd(&h[(key[e] >> shift) & 255], 1);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * nblk + b] = h[d];
}

// exclusive scan of one tile of 1024 ints in place (warp-shuffle scans,
// then a scan of the 32 warp totals); the tile total goes to tsum[tile]
__device__ __forceinline__ int block_exclusive_scan(int v, int* wsum, int& total) {
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int off = 1; off < 32; off <<= 1) {
    int u = __shfl_up_sync(FULL, x, off);
    if (lane >= off) x += u;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int y = (lane < (int)(blockDim.x >> 5)) ? wsum[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      int u = __shfl_up_sync(FULL, y, off);
      if (lane >= off) y += u;
    }
    wsum[lane] = y;                         // inclusive warp totals
  }
  __syncthreads();
  total = wsum[(blockDim.x >> 5) - 1];
  return x - v + (w > 0 ? wsum[w - 1] : 0);
}

__global__ void scan_tile_kernel(int* __restrict__ a, int m, int* __restrict__ tsum, const int* __restrict__ dirty) {
  if (!*dirty) return;
  __shared__ int wsum[32];
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  int v = (idx < m) ? a[idx] : 0;
  int total;
  int ex = block_exclusive_scan(v, wsum, total);
  if (idx < m) a[idx] = ex;
  if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

__global__ void scan_add_kernel(int* __restrict__ a, int m, const int* __restrict__ tsum, const int* __restrict__ dirty) {
  if (!*dirty) return;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < m && blockIdx.x > 0) a[idx] += tsum[blockIdx.x];
}

// exclusive scan of m ints by one block of 1024 threads: coalesced tiles
// of 1024, warp-shuffle scans inside a tile, a running carry across tiles
// (used on the tile totals of the multi-block scan)
__global__ void scan_kernel(int* __restrict__ a, int m, const int* __restrict__ dirty) {
  if (!*dirty) return;
  __shared__ int wsum[32];
  __shared__ int carry;
  const unsigned FULL = 0xffffffffu;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < m; base += blockDim.x) {
    int idx = base + threadIdx.x;
    int v = (idx < m) ? a[idx] : 0;
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
      int u = __shfl_up_sync(FULL, x, off);
      if (lane >= off) x += u;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int y = wsum[lane];
      for (int off = 1; off < 32; off <<= 1) {
        int u = __shfl_up_sync(FULL, y, off);
        if (lane >= off) y += u;
      }
      wsum[lane] = y;                       // inclusive warp totals
    }
    __syncthreads();
    int incl = x + (w > 0 ? wsum[w - 1] : 0);
    if (idx < m) a[idx] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += incl;
    __syncthreads();
  }
}

// stable scatter: chunk order, then warp order, then lane order
__global__ void radix_scatter_kernel(const int* __restrict__ kin, const int* __restrict__ vin, int* __restrict__ kout,
                                     int* __restrict__ vout, int n, int shift, int nblk, const int* __restrict__ offs,
                                     const int* __restrict__ dirty) {
  if (!*dirty) return;
  __shared__ int base[256];
  __shared__ int wcnt[8][256];
  int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int d = tid; d < 256; d += 256) base[d] = offs[d * nblk + b];
  __syncthreads();
  int end = min(n, (b + 1) * kSortChunk);
  for (int start = b * kSortChunk; start < end; start += 256) {
    int idx = start + tid;
    bool valid = idx < end;
    int key = valid ? kin[idx] : 0;
    int dig = valid ? ((key >> shift) & 255) : 256;
    for (int q = tid; q < 8 * 256; q += 256) (&wcnt[0][0])[q] = 0;
    __syncthreads();
    unsigned peers = __match_any_sync(0xffffffffu, dig);
    int rank = __popc(peers & ((1u << lane) - 1u));
    int leader = __ffs(peers) - 1;
    if (valid && lane == leader) wcnt[w][dig] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int q = 0; q < w; ++q) pre += wcnt[q][dig];
      int pos = base[dig] + pre + rank;
      kout[pos] = key;
      vout[pos] = vin[idx];
    }
    __syncthreads();
    for (int d = tid; d < 256; d += 256) {
      int tot = 0;
      for (int q = 0; q < 8; ++q) tot += wcnt[q][d];
      base[d] += tot;
    }
    __syncthreads();
  }
}

// Heads of the runs of equal keys (one cell of one component) sum their run
// in triangle order and add the sum to that component's target field; with
// `segval` the head also records the sum (for the mean force).
struct ScatterOut {
  double* f[4];
  const double* phi[4];
  float* m32[4];   // FP32 mirrors of f (precision form), null where none
};

__device__ __forceinline__ int key_comp(int k, size_t cells) {
  size_t u = (size_t)k;
  return (u >= cells) + (u >= 2 * cells) + (u >= 3 * cells) + (u >= 4 * cells);   // 4 = ghost face
}

// Heads of the sorted plan (the first entry of each run of one real key),
// in key order, built with the plan: flag, exclusive scan, compaction.
__device__ __forceinline__ bool plan_head(const int* __restrict__ key, int e, size_t cells) {
  const int k = key[e];
  return key_comp(k, cells) < 4 && (e == 0 || key[e - 1] != k);
}

__global__ void head_flag_kernel(int n, size_t cells, const int* __restrict__ key, const int* __restrict__ dirty,
                                 int* __restrict__ hidx) {
  if (!*dirty) return;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) hidx[e] = plan_head(key, e, cells) ? 1 : 0;
}

__global__ void head_compact_kernel(int n, size_t cells, const int* __restrict__ key, const int* __restrict__ hidx,
                                    const int* __restrict__ dirty, int* __restrict__ heads, int* __restrict__ nheads) {
  if (!*dirty) return;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const bool head = plan_head(key, e, cells);
  if (head) heads[hidx[e]] = e;
  if (e == n - 1) *nheads = hidx[e] + (head ? 1 : 0);
}

// One warp per run (a cell of one component): the lanes take every 32nd
// entry of the run (face order), a fixed shuffle tree adds the 32 partial
// sums, lane 0 adds the total to the target field.  A warp instruction costs
// the same with 1 or 32 active lanes, and FP64 ones issue at a small fraction
// of the FP32 rate, so the runs (tens of entries each) are not summed by one
// thread.  With `segval` the run sum is also recorded at the run's index
// (for the mean force).
constexpr int kScatterBlocks = 1216;     // 8 blocks of 8 warps per SM on 152 SMs; the warps loop over runs
__global__ void __launch_bounds__(256) scatter_apply_kernel(int n, int nf, size_t cells, const int* __restrict__ key,
                                     const int* __restrict__ src, const double* __restrict__ coef, ScatterOut O,
                                     int comp_lo, int comp_hi, const int* __restrict__ heads,
                                     const int* __restrict__ nheads, double* __restrict__ segval) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int nh = *nheads;
  const int per = 27 * nf;
  for (int h = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); h < nh; h += nw) {
    const int e0 = heads[h];
    const int k = key[e0];
    const int comp = key_comp(k, cells);
    if (comp < comp_lo || comp >= comp_hi) continue;            // uniform over the warp
    const int e1 = h + 1 < nh ? heads[h + 1] : n;               // the last run ends before the ghost entries
    const double* __restrict__ phi = O.phi[comp];
    const double* __restrict__ cf = coef + (size_t)comp * nf;
    double sum = 0.0;
    for (int q = e0 + lane; q < e1 && key[q] == k; q += 32) {
      const int sr = src[q] - comp * per;
      if (!MIBM_IDX_OK(sr, per)) continue;
      sum = fma(cf[sr / 27], phi[sr], sum);
    }
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(FULL, sum, off);
    if (lane == 0 && MIBM_IDX_OK((size_t)k - (size_t)comp * cells, cells)) {
      const size_t cell = (size_t)k - (size_t)comp * cells;
      const double v = O.f[comp][cell] + sum;
      O.f[comp][cell] = v;
      if (O.m32[comp]) O.m32[comp][cell] = (float)v;
      if (segval) segval[h] = sum;
    }
  }
}

// fixed-order sum of the recorded run sums per velocity component: 256
// blocks over contiguous ranges of runs (shuffle trees, then the 8 warps in
// order); the last block to finish (a ticket in mean3's slot 7, reset by that
// block) adds the 256 block sums, one component per warp: lane l sums blocks
// l, l+32, l+64, ... in that order, then a fixed shuffle tree adds the 32
// lane sums (a fixed order, so the result is deterministic); it writes the
// means divided by the cell count (FP64 at mean3[0..2], an FP32
// copy for the precision form at float offset 8)
constexpr int kMeanBlocks = 256;
__global__ void __launch_bounds__(256) seg_mean_kernel(const int* __restrict__ nheads, const int* __restrict__ heads,
                                                      size_t cells, const int* __restrict__ key,
                                                      const double* __restrict__ segval, double* __restrict__ part,
                                                      double ncell, double* __restrict__ mean3) {
  const unsigned FULL = 0xffffffffu;
  __shared__ double ws[8][3];
  __shared__ bool last;
  const int n = *nheads;
  int per = (n + gridDim.x - 1) / gridDim.x;
  int lo = blockIdx.x * per, hi = min(n, lo + per);
  double s[3] = {0, 0, 0};
  for (int h = lo + threadIdx.x; h < hi; h += blockDim.x) {
    int comp = key_comp(key[heads[h]], cells);
    if (comp < 3) s[comp] += segval[h];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < 3; ++q) {
    double v = s[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (lane == 0) ws[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double v = ws[0][threadIdx.x];
    for (int w = 1; w < 8; ++w) v += ws[w][threadIdx.x];
    part[3 * (size_t)blockIdx.x + threadIdx.x] = v;
  }
  unsigned* ticket = reinterpret_cast<unsigned*>(mean3 + 7);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (warp < 3) {
    double v = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) v += __ldcg(part + 3 * (size_t)b + warp);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (lane == 0) {
      double m = v / ncell;
      mean3[warp] = m;
      reinterpret_cast<float*>(mean3 + 4)[warp] = (float)m;   // FP32 copy for the precision form
    }
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// ---------------------------------------------------------------------
// deterministic sums
// ---------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// per-block partial sums of up to 3 fields over the owned cells, fixed order
__global__ void field_sum_kernel(Grid g, const double* __restrict__ a, const double* __restrict__ b,
                                 const double* __restrict__ cc, double* __restrict__ part) {
  int j = blockIdx.x, k = blockIdx.y;
  double s[3] = {0, 0, 0};
  for (int i = threadIdx.x; i < g.n1m; i += blockDim.x) {
    size_t c0 = cidx(g, i, j, k);
    s[0] += a[c0]; s[1] += b[c0]; s[2] += cc[c0];
  }
  __shared__ double sm[3][32];
  for (int q = 0; q < 3; ++q) {
    double v = warp_sum(s[q]);
    if ((threadIdx.x & 31) == 0) sm[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int nw = blockDim.x >> 5;
    for (int q = 0; q < 3; ++q) {
      double v = (threadIdx.x < nw) ? sm[q][threadIdx.x] : 0.0;
      v = warp_sum(v);
      if (threadIdx.x == 0) part[3 * ((size_t)j + (size_t)g.n2m * k) + q] = v;
    }
  }
}

// sum m triples in fixed order, divide by the cell count -> mean3
__global__ void mean3_kernel(const double* __restrict__ part, int m, double ncell, double* __restrict__ out) {
  __shared__ double sm[3][1024];
  double s[3] = {0, 0, 0};
  for (int t = threadIdx.x; t < m; t += blockDim.x)
    for (int q = 0; q < 3; ++q) s[q] += part[3 * (size_t)t + q];
  for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] = s[q];
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off)
      for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out[q] = sm[q][0] / ncell;
}

__device__ __forceinline__ void cross3(double r[3], const double x[3], const double y[3]) {
  r[0] = x[1] * y[2] - y[1] * x[2];
  r[1] = x[2] * y[0] - y[2] * x[0];
  r[2] = x[0] * y[1] - y[0] * x[1];
}

// Per-face loads in the reference's order (mls_structLoads.f90:52-202):
// c[0..3) pressure force, [3..6) viscous force, [6..9) pressure torque,
// [9..12) viscous torque.
__device__ void face_loads(const double* __restrict__ e, const double nrm[3], const double rad[3], double sur,
                           double h, double ren, double c[12]) {
  double press_tri = e[0] - h * (e[1] * nrm[0] + e[2] * nrm[1] + e[3] * nrm[2]);
  double pn[3], buf[3];
  for (int d = 0; d < 3; ++d) { c[d] = press_tri * sur * nrm[d]; pn[d] = press_tri * nrm[d]; }
  cross3(buf, rad, pn);
  for (int d = 0; d < 3; ++d) c[6 + d] = buf[d] * sur;
  double S11 = e[4], S12 = e[5], S13 = e[6], S21 = e[7], S22 = e[8], S23 = e[9];
  double S31 = e[10], S32 = e[11], S33 = e[12];
  double sr = sur / ren;
  double tv[3];
  tv[0] = sr * (2.0 * S11 * nrm[0] + (S12 + S21) * nrm[1] + S13 * nrm[2]);
  tv[1] = sr * ((S21 + S12) * nrm[0] + 2.0 * S22 * nrm[1] + S23 * nrm[2]);
  tv[2] = sr * (S13 * nrm[0] + S23 * nrm[1]);
  double tn[3], rt[3];
  for (int d = 0; d < 3; ++d) tn[d] = 0.0 + tv[d];
  cross3(buf, rad, tv);
  for (int d = 0; d < 3; ++d) rt[d] = 0.0 + buf[d];
  tv[0] = sr * (S31 * nrm[2]);
  tv[1] = sr * (S32 * nrm[2]);
  tv[2] = sr * (S31 * nrm[0] + S32 * nrm[1] + 2.0 * S33 * nrm[2]);
  for (int d = 0; d < 3; ++d) tn[d] = tn[d] + tv[d];
  cross3(buf, rad, tv);
  for (int d = 0; d < 3; ++d) rt[d] = rt[d] + buf[d];
  for (int d = 0; d < 3; ++d) { c[3 + d] = tn[d]; c[9 + d] = rt[d]; }
}

// ---------------------------------------------------------------------
// Precision form of mlsWeight and mls_heatFlux.  MLS with the complete
// linear basis is invariant under an affine change of basis, so the shape
// functions (and their gradients) can be built from the basis
// p = (1, x - x0, y - y0, z - z0) shifted to the interpolation point x0,
// where p(x0) = e0.  With separable Gaussian weights w_n = wx_i wy_j wz_k
// every moment sum factorises into 1-D moments S_m = sum_q w_q d_q^m
// (m = 0, 1, 2) and the derivative weights likewise (D_m), so the 4x4
// moment matrix and its three derivatives take a few dozen FP64 operations
// instead of 27 rank-one updates each, and are far better conditioned than
// with absolute coordinates.  The 4x4 inversion is the FP64 LU of the plain
// form.  The values agree with the reference construction to its round-off
// (amplified by its conditioning), not bit for bit.
// ---------------------------------------------------------------------
__device__ __forceinline__ void moments3(const double w[3], const double d[3], double S[3]) {
  S[0] = w[0] + w[1] + w[2];
  S[1] = fma(w[0], d[0], fma(w[1], d[1], w[2] * d[2]));
  S[2] = fma(w[0] * d[0], d[0], fma(w[1] * d[1], d[1], (w[2] * d[2]) * d[2]));
}

// symmetric moment matrix (column-major) of the shifted linear basis from
// 1-D moments X, Y, Z (each S0, S1, S2)
__device__ __forceinline__ void moment_matrix(const double X[3], const double Y[3], const double Z[3], double M[16]) {
  double a00 = X[0] * Y[0] * Z[0];
  double a01 = X[1] * Y[0] * Z[0], a02 = X[0] * Y[1] * Z[0], a03 = X[0] * Y[0] * Z[1];
  double a11 = X[2] * Y[0] * Z[0], a22 = X[0] * Y[2] * Z[0], a33 = X[0] * Y[0] * Z[2];
  double a12 = X[1] * Y[1] * Z[0], a13 = X[1] * Y[0] * Z[1], a23 = X[0] * Y[1] * Z[1];
  M[0] = a00; M[1] = a01; M[2] = a02; M[3] = a03;
  M[4] = a01; M[5] = a11; M[6] = a12; M[7] = a13;
  M[8] = a02; M[9] = a12; M[10] = a22; M[11] = a23;
  M[12] = a03; M[13] = a13; M[14] = a23; M[15] = a33;
}

__global__ void mls_weight_sep_kernel(LagArgs A, const double* __restrict__ tri_bar, const int* __restrict__ ghost,
                                      const int* __restrict__ pind, double* __restrict__ p1, double* __restrict__ p2,
                                      double* __restrict__ p3, double* __restrict__ pt, int* __restrict__ flag) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  int t = gid >> 2, comp = gid & 3;
  if (t >= A.nf || ghost[t]) return;
  const Grid& g = A.g;
  double pos[3] = {tri_bar[3 * t], tri_bar[3 * t + 1], tri_bar[3 * t + 2]};
  CageSpec cs = cage_spec(comp);
  int i0 = pind[6 * t + cs.ix], j0 = pind[6 * t + cs.iy];
  int k0 = cs.znint ? fnint(pos[2] * g.dx3) + 1 : ffloor(pos[2] * g.dx3) + 1;
  double wx[3], wy[3], wz[3], dx[3], dy[3], dz[3];
  for (int q = 0; q < 3; ++q) {
    double cz = coord(A, 2, cs.sz, k0 - 1 + q), cy = coord(A, 1, cs.sy, j0 - 1 + q), cx = coord(A, 0, cs.sx, i0 - 1 + q);
    wz[q] = mls_gaussian(fabs(cz - pos[2]) / (A.wscl / g.dx3), A.wcon);
    wy[q] = mls_gaussian(fabs(cy - pos[1]) / (A.wscl / g.dx2), A.wcon);
    wx[q] = mls_gaussian(fabs(cx - pos[0]) / (A.wscl / g.dx1), A.wcon);
    dx[q] = cx - pos[0]; dy[q] = cy - pos[1]; dz[q] = cz - pos[2];
  }
  double X[3], Y[3], Z[3], M[16];
  moments3(wx, dx, X); moments3(wy, dy, Y); moments3(wz, dz, Z);
  moment_matrix(X, Y, Z, M);
  if (!inv4(M)) { atomicOr(flag, 1); return; }
  const double c0 = M[0], c1 = M[1], c2 = M[2], c3 = M[3];   // A^{-1} e0
  double* out = (comp == 0) ? p1 : (comp == 1) ? p2 : (comp == 2) ? p3 : pt;
  out += 27 * (size_t)t;
  for (int kk = 0; kk < 3; ++kk)
    for (int jj = 0; jj < 3; ++jj) {
      double wyz = wy[jj] * wz[kk], base = fma(c2, dy[jj], fma(c3, dz[kk], c0));
      for (int ii = 0; ii < 3; ++ii) out[ii + 3 * jj + 9 * kk] = (wx[ii] * wyz) * fma(c1, dx[ii], base);
    }
}

// Gaussian weight of one cage coordinate and its derivative along the axis
// (geom.f90:24-53 with the chain-rule factor of mls_heatFlux.f90:176-180).
// The cut-off decision r > 1 uses r = |x - x_c| / (wscl/dx) rounded as the
// reference rounds it; the rest uses precomputed reciprocals (the separable
// construction is insensitive to last-ulp changes of the weights).
struct AxisScale {
  double c, inv_c, inv_wcon, dcoef;   // wscl/dx, its reciprocal, 1/wcon, -2/wcon^2
};
__device__ __forceinline__ AxisScale axis_scale(const LagArgs& A, double dx) {
  AxisScale a;
  a.c = A.wscl / dx;
  a.inv_c = 1.0 / a.c;
  a.inv_wcon = 1.0 / A.wcon;
  a.dcoef = -2.0 / (A.wcon * A.wcon);
  return a;
}
__device__ __forceinline__ void axis_weight(const AxisScale& a, double pos, double pc, double& w, double& dw) {
  const double eps = 2.220446049250313e-16;
  double rr = pos - pc;
  double np = fabs(rr) / a.c;
  if (np > 1.0) { w = 0.0; dw = 0.0; return; }
  double e = exp(-sqd(np * a.inv_wcon));
  w = e;
  dw = (np < eps) ? 0.0 : (a.dcoef * np) * e * copysign(a.inv_c, rr);
}

// Separable MLS gradient at a probe: the gradient of wght_gradT (mls_heatFlux
// .f90:161-376) and wght_gradP/U/V/W (mls_structLoads.f90:406-1298).  Cage
// i, j centred on (pi1, pi2); z layers [k1-1, k1, k1] (the repeated layer of
// the reference) with k1 = floor(z*dx3)+1, or nint for the w-velocity;
// coordinates per axis from the field's staggering (sel 0 = face, 1 =
// centre); field values at the wrapped cage, z from [k1w-1, k1w, k1w+1].
// Returns false on a singular moment matrix.
__device__ bool probe_grad_sep(const LagArgs& A, const double pos[3], int pi1, int pi2, int sx, int sy, int sz,
                               bool knint, const double* __restrict__ q, double grad[3]) {
  const Grid& g = A.g;
  int k1 = knint ? fnint(pos[2] * g.dx3) + 1 : ffloor(pos[2] * g.dx3) + 1;
  int kin[3] = {k1 - 1, k1, k1};                  // mls_heatFlux.f90:213 (third layer repeats k1)
  int k1w = fmod_pos(k1 - 1, g.n3m) + 1;
  int keul[3] = {k1w - 1, k1w, k1w + 1};
  const int sel[3] = {sx, sy, sz};
  const AxisScale sc[3] = {axis_scale(A, g.dx1), axis_scale(A, g.dx2), axis_scale(A, g.dx3)};
  double w[3][3], dw[3][3], dd[3][3];             // [axis][point]
  for (int r = 0; r < 3; ++r) {
    double pc[3] = {coord(A, 0, sel[0], pi1 - 1 + r), coord(A, 1, sel[1], pi2 - 1 + r), coord(A, 2, sel[2], kin[r])};
    for (int a = 0; a < 3; ++a) {
      axis_weight(sc[a], pos[a], pc[a], w[a][r], dw[a][r]);
      dd[a][r] = pc[a] - pos[a];
    }
  }
  double S[3][3], D[3][3];
  for (int a = 0; a < 3; ++a) { moments3(w[a], dd[a], S[a]); moments3(dw[a], dd[a], D[a]); }
  double Ai[16];
  moment_matrix(S[0], S[1], S[2], Ai);
  if (!inv4(Ai)) return false;
  const double gam[4] = {Ai[0], Ai[1], Ai[2], Ai[3]};     // A^{-1} p(x0), p(x0) = e0
  // sums over the cage of the field times the weighted basis p = (1, d0, d1,
  // d2): MT (weights), MD[d] (derivative of the weights along d).  Weights
  // and basis factor by axis, so the sums are contracted one axis at a time
  // (x, then y, then z): about 250 FP64 operations instead of 675.
  double wd[3][3], dwd[3][3];
  for (int a = 0; a < 3; ++a)
    for (int r = 0; r < 3; ++r) { wd[a][r] = w[a][r] * dd[a][r]; dwd[a][r] = dw[a][r] * dd[a][r]; }
  double MT[4] = {0, 0, 0, 0}, MD[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
  for (int kk = 0; kk < 3; ++kk) {
    const int kk_ = wrap(keul[kk] - 1, g.n3m);
    // y sums of the x sums A = sum w0 q, B = sum w0 d0 q, C = sum dw0 q, D = sum dw0 d0 q
    double SA = 0, SAd = 0, SAw = 0, SAwd = 0, SB = 0, SBw = 0, SC = 0, SCd = 0, SD = 0;
    for (int jj = 0; jj < 3; ++jj) {
      const int jj_ = fmod_pos(pi2 - 1 + jj - 1, g.n2m);
      double qa = 0, qb = 0, qc = 0, qd = 0;
      for (int ii = 0; ii < 3; ++ii) {
        const double T = q[cidx(g, fmod_pos(pi1 - 1 + ii - 1, g.n1m), jj_, kk_)];
        qa = fma(w[0][ii], T, qa); qb = fma(wd[0][ii], T, qb);
        qc = fma(dw[0][ii], T, qc); qd = fma(dwd[0][ii], T, qd);
      }
      SA = fma(w[1][jj], qa, SA); SAd = fma(wd[1][jj], qa, SAd);
      SAw = fma(dw[1][jj], qa, SAw); SAwd = fma(dwd[1][jj], qa, SAwd);
      SB = fma(w[1][jj], qb, SB); SBw = fma(dw[1][jj], qb, SBw);
      SC = fma(w[1][jj], qc, SC); SCd = fma(wd[1][jj], qc, SCd);
      SD = fma(w[1][jj], qd, SD);
    }
    const double z = w[2][kk], zd = wd[2][kk], dz = dw[2][kk], dzd = dwd[2][kk];
    MT[0] = fma(z, SA, MT[0]); MT[1] = fma(z, SB, MT[1]); MT[2] = fma(z, SAd, MT[2]); MT[3] = fma(zd, SA, MT[3]);
    MD[0][0] = fma(z, SC, MD[0][0]); MD[0][1] = fma(z, SD, MD[0][1]);
    MD[0][2] = fma(z, SCd, MD[0][2]); MD[0][3] = fma(zd, SC, MD[0][3]);
    MD[1][0] = fma(z, SAw, MD[1][0]); MD[1][1] = fma(z, SBw, MD[1][1]);
    MD[1][2] = fma(z, SAwd, MD[1][2]); MD[1][3] = fma(zd, SAw, MD[1][3]);
    MD[2][0] = fma(dz, SA, MD[2][0]); MD[2][1] = fma(dz, SB, MD[2][1]);
    MD[2][2] = fma(dz, SAd, MD[2][2]); MD[2][3] = fma(dzd, SA, MD[2][3]);
  }
  for (int d = 0; d < 3; ++d) {
    double dA[16];
    double X[3], Y[3], Z[3];
    for (int m = 0; m < 3; ++m) {
      X[m] = d == 0 ? D[0][m] : S[0][m];
      Y[m] = d == 1 ? D[1][m] : S[1][m];
      Z[m] = d == 2 ? D[2][m] : S[2][m];
    }
    moment_matrix(X, Y, Z, dA);
    double pk[4];
    for (int r = 0; r < 4; ++r) {
      double a = 0;
      for (int cc = 0; cc < 4; ++cc) a = fma(dA[r + 4 * cc], gam[cc], a);
      pk[r] = (r == d + 1 ? 1.0 : 0.0) - a;
    }
    double acc = 0;
    for (int r = 0; r < 4; ++r) {
      double dg = 0;
      for (int cc = 0; cc < 4; ++cc) dg = fma(Ai[r + 4 * cc], pk[cc], dg);
      acc = fma(dg, MT[r], fma(gam[r], MD[d][r], acc));
    }
    grad[d] = acc;
  }
  return true;
}

// Separable MLS value at a probe (wght_press, mls_structLoads.f90:271-404):
// cell-centred cage around (i0, j0), z layers k1-1, k1, k1+1 (no repeated
// layer).  value = A^{-1} e0 . sum_n w_n p_n q_n in the shifted basis.
__device__ bool probe_value_sep(const LagArgs& A, const double pos[3], int i0, int j0, const double* __restrict__ q,
                                double& val) {
  const Grid& g = A.g;
  int k1 = ffloor(pos[2] * g.dx3) + 1;
  int k1w = fmod_pos(k1 - 1, g.n3m) + 1;
  const AxisScale sc[3] = {axis_scale(A, g.dx1), axis_scale(A, g.dx2), axis_scale(A, g.dx3)};
  double w[3][3], dd[3][3];
  for (int r = 0; r < 3; ++r) {
    double pc[3] = {coord(A, 0, 1, i0 - 1 + r), coord(A, 1, 1, j0 - 1 + r), coord(A, 2, 1, k1 - 1 + r)};
    for (int a = 0; a < 3; ++a) {
      double dwu;
      axis_weight(sc[a], pos[a], pc[a], w[a][r], dwu);
      dd[a][r] = pc[a] - pos[a];
    }
  }
  double S[3][3];
  for (int a = 0; a < 3; ++a) moments3(w[a], dd[a], S[a]);
  double Ai[16];
  moment_matrix(S[0], S[1], S[2], Ai);
  if (!inv4(Ai)) return false;
  // sum over the cage of q w p, contracted one axis at a time (as in
  // probe_grad_sep)
  double MT[4] = {0, 0, 0, 0};
  for (int kk = 0; kk < 3; ++kk) {
    const int kk_ = wrap(k1w - 1 + kk - 1, g.n3m);
    double SA = 0, SAd = 0, SB = 0;
    for (int jj = 0; jj < 3; ++jj) {
      const int jj_ = fmod_pos(j0 - 1 + jj - 1, g.n2m);
      double qa = 0, qb = 0;
      for (int ii = 0; ii < 3; ++ii) {
        const double T = q[cidx(g, fmod_pos(i0 - 1 + ii - 1, g.n1m), jj_, kk_)];
        qa = fma(w[0][ii], T, qa); qb = fma(w[0][ii] * dd[0][ii], T, qb);
      }
      SA = fma(w[1][jj], qa, SA); SAd = fma(w[1][jj] * dd[1][jj], qa, SAd); SB = fma(w[1][jj], qb, SB);
    }
    MT[0] = fma(w[2][kk], SA, MT[0]); MT[1] = fma(w[2][kk], SB, MT[1]);
    MT[2] = fma(w[2][kk], SAd, MT[2]); MT[3] = fma(w[2][kk] * dd[2][kk], SA, MT[3]);
  }
  double v = 0;
  for (int r = 0; r < 4; ++r) v = fma(Ai[r], MT[r], v);
  val = v;
  return true;
}

// mls_heatFlux.f90:77-158 at both probes of every face with the separable
// construction (precision form, moving body): one thread per (face, side).
__global__ void heat_flux_sep_kernel(LagArgs A, const double* __restrict__ temp, const double* __restrict__ tri_bar,
                                 const double* __restrict__ tri_nor, const int* __restrict__ ghost,
                                 const int* __restrict__ pind, double h, double pec, double* __restrict__ qw_o,
                                 double* __restrict__ qw_i, int* __restrict__ flag) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  int t = gid >> 1, side = gid & 1;
  if (t >= A.nf) return;
  double* qout = side == 0 ? qw_o : qw_i;
  if (ghost[t]) { qout[t] = 0.0; return; }
  double n0 = tri_nor[3 * t], n1 = tri_nor[3 * t + 1], n2 = tri_nor[3 * t + 2];
  double s = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  double pos[3];
  for (int d = 0; d < 3; ++d) {
    double nd = tri_nor[3 * t + d];
    pos[d] = side == 0 ? tri_bar[3 * t + d] + h * nd / s : tri_bar[3 * t + d] - h * nd / s;
  }
  int pi1 = pind[6 * t + 3 * side + 0], pi2 = pind[6 * t + 3 * side + 1];
  double grad[3];
  if (!probe_grad_sep(A, pos, pi1, pi2, 1, 1, 1, false, temp, grad)) { atomicOr(flag, 1); qout[t] = 0.0; return; }
  double qv = n0 * grad[0] + n1 * grad[1] + n2 * grad[2];
  qout[t] = qv / pec;
}

// The literal heat flux of the plain form (mls_heatFlux.f90:77-158 with
// wght_gradT), spread over a block of 4 warps for 32 probes (lane = probe,
// probe q = face q/2, side q%2): warp 0 forms the probe's per-axis weights
// (shared), then the moment matrix A by the reference's rank-one updates, its
// inverse and gamma; warp w = 1..3 forms dA_d (d = w - 1) meanwhile and, once
// A^-1 and gamma are published, the direction-d gradient.  Every value comes
// from exactly the operations of probe_grad_lit in its order (the oracle's
// bits); the split only gives the device four times the independent work per
// probe that one thread would have.
constexpr int kHfProbes = 32;
__global__ void __launch_bounds__(4 * kHfProbes)
heat_flux_lit_kernel(LagArgs A, const double* __restrict__ temp, const double* __restrict__ tri_bar,
                     const double* __restrict__ tri_nor, const int* __restrict__ ghost,
                     const int* __restrict__ pind, double h, double pec, double* __restrict__ qw_o,
                     double* __restrict__ qw_i, int* __restrict__ flag) {
  __shared__ double sW[3][3][kHfProbes], sdW[3][3][kHfProbes], spc[3][3][kHfProbes];
  __shared__ double sAi[16][kHfProbes], sgam[4][kHfProbes], sgrad[3][kHfProbes];
  __shared__ int sok[kHfProbes];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gid = blockIdx.x * kHfProbes + lane;
  const int t = gid >> 1, side = gid & 1;
  const bool valid = t < A.nf;
  const bool live = valid && !ghost[t];
  const Grid& g = A.g;
  const double eps = 2.220446049250313e-16;       // EPSILON(1.0d0)
  double pos[3] = {0.0, 0.0, 0.0};
  int pi1 = 0, pi2 = 0, k1 = 0;
  if (live) {
    const double n0 = tri_nor[3 * t], n1 = tri_nor[3 * t + 1], n2 = tri_nor[3 * t + 2];
    const double s = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    for (int d = 0; d < 3; ++d) {
      const double nd = tri_nor[3 * t + d];
      pos[d] = side == 0 ? tri_bar[3 * t + d] + h * nd / s : tri_bar[3 * t + d] - h * nd / s;
    }
    pi1 = pind[6 * t + 3 * side + 0];
    pi2 = pind[6 * t + 3 * side + 1];
    k1 = ffloor(pos[2] * g.dx3) + 1;
  }
  if (w == 0 && live) {
    const int kin[3] = {k1 - 1, k1, k1};          // the repeated layer of mls_heatFlux.f90:213
    const double dxa[3] = {g.dx1, g.dx2, g.dx3};
    for (int r = 0; r < 3; ++r) {
      const double pc[3] = {coord(A, 0, 1, pi1 - 1 + r), coord(A, 1, 1, pi2 - 1 + r), coord(A, 2, 1, kin[r])};
      for (int a = 0; a < 3; ++a) {
        double W, dW;
        lit_axis_weight(A, pos[a], pc[a], dxa[a], eps, W, dW);
        spc[a][r][lane] = pc[a];
        sW[a][r][lane] = W;
        sdW[a][r][lane] = dW;
      }
    }
  }
  __syncthreads();
  double dA[16];
  const int d = w - 1;
  if (w == 0) {
    int ok = 0;
    if (live) {
      double Am[16];
      for (int e = 0; e < 16; ++e) Am[e] = 0.0;
      for (int nk = 0; nk < 3; ++nk)
        for (int j = 0; j < 3; ++j) {
          const double w23 = sW[1][j][lane] * sW[2][nk][lane];
          for (int i = 0; i < 3; ++i) {
            const double wtx = sW[0][i][lane] * w23;
            const double pk[4] = {1.0, spc[0][i][lane], spc[1][j][lane], spc[2][nk][lane]};
            for (int cc = 0; cc < 4; ++cc) {
              const double tt = wtx * pk[cc];
              for (int r = 0; r < 4; ++r) Am[r + 4 * cc] = Am[r + 4 * cc] + tt * pk[r];
            }
          }
        }
      if (inv4(Am)) {
        ok = 1;
        const double ptx[4] = {1.0, pos[0], pos[1], pos[2]};
        for (int r = 0; r < 4; ++r) {               // DGEMV('N', invA, ptx)
          double tt = 0;
          for (int cc = 0; cc < 4; ++cc) tt += Am[r + 4 * cc] * ptx[cc];
          sgam[r][lane] = tt;
        }
        for (int e = 0; e < 16; ++e) sAi[e][lane] = Am[e];
      }
    }
    sok[lane] = ok;
  } else if (live) {
    for (int e = 0; e < 16; ++e) dA[e] = 0.0;
    for (int nk = 0; nk < 3; ++nk)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          const double dwd = d == 0 ? (sdW[0][i][lane] * sW[1][j][lane]) * sW[2][nk][lane]
                           : d == 1 ? (sW[0][i][lane] * sdW[1][j][lane]) * sW[2][nk][lane]
                                    : (sW[0][i][lane] * sW[1][j][lane]) * sdW[2][nk][lane];
          const double pk[4] = {1.0, spc[0][i][lane], spc[1][j][lane], spc[2][nk][lane]};
          for (int cc = 0; cc < 4; ++cc) {
            const double tt = dwd * pk[cc];
            for (int r = 0; r < 4; ++r) dA[r + 4 * cc] = dA[r + 4 * cc] + tt * pk[r];
          }
        }
  }
  __syncthreads();
  if (w > 0 && live && sok[lane]) {
    double gam[4];
    for (int r = 0; r < 4; ++r) gam[r] = sgam[r][lane];
    double pk_d[4] = {0.0, 0.0, 0.0, 0.0};
    pk_d[d + 1] = 1.0;
    for (int r = 0; r < 4; ++r) {                   // pk = -dA gamma + pk
      double tt = 0;
      for (int cc = 0; cc < 4; ++cc) tt += dA[r + 4 * cc] * gam[cc];
      pk_d[r] = pk_d[r] - tt;
    }
    double dgam[4];
    for (int r = 0; r < 4; ++r) {
      double tt = 0;
      for (int cc = 0; cc < 4; ++cc) tt += sAi[r + 4 * cc][lane] * pk_d[cc];
      dgam[r] = tt;
    }
    const int k1w = fmod_pos(k1 - 1, g.n3m) + 1;
    const int kk_[3] = {wrap(k1w - 2, g.n3m), wrap(k1w - 1, g.n3m), wrap(k1w, g.n3m)};
    double gsum = 0;
    for (int nk = 0; nk < 3; ++nk)
      for (int j = 0; j < 3; ++j) {
        const int jj = fmod_pos(pi2 - 1 + j - 1, g.n2m);
        const double w23 = sW[1][j][lane] * sW[2][nk][lane];
        for (int i = 0; i < 3; ++i) {
          const double wtx = sW[0][i][lane] * w23;
          const double dwd = d == 0 ? (sdW[0][i][lane] * sW[1][j][lane]) * sW[2][nk][lane]
                           : d == 1 ? (sW[0][i][lane] * sdW[1][j][lane]) * sW[2][nk][lane]
                                    : (sW[0][i][lane] * sW[1][j][lane]) * sdW[2][nk][lane];
          const double pk[4] = {1.0, spc[0][i][lane], spc[1][j][lane], spc[2][nk][lane]};
          double t1 = 0, t2 = 0;
          for (int r = 0; r < 4; ++r) t1 += dgam[r] * (wtx * pk[r]);
          for (int r = 0; r < 4; ++r) t2 += gam[r] * (dwd * pk[r]);
          const double T = temp[cidx(g, fmod_pos(pi1 - 1 + i - 1, g.n1m), jj, kk_[nk])];
          gsum += (t1 + t2) * T;
        }
      }
    sgrad[d][lane] = gsum;
  }
  __syncthreads();
  if (w == 0 && valid) {
    double* qout = side == 0 ? qw_o : qw_i;
    if (!live) {
      qout[t] = 0.0;
    } else if (!sok[lane]) {
      atomicOr(flag, 1);
      qout[t] = 0.0;
    } else {
      const double qv = tri_nor[3 * t] * sgrad[0][lane] + tri_nor[3 * t + 1] * sgrad[1][lane] +
                        tri_nor[3 * t + 2] * sgrad[2][lane];
      qout[t] = qv / pec;
    }
  }
}

// ---------------------------------------------------------------------
// Structural loads (mls_structLoads.f90:1-269).  Faces go in groups of 32
// (lane = face); each group is five one-warp blocks, and warp e evaluates, at
// each face's positive probe x_p = X + h n/|n|,
//   e = 0  the pressure (wght_press: cell-centred cage, z layers k1-1..k1+1
//          without the repeated layer, mls_structLoads.f90:271-404)
//   e = 1  grad p   (wght_gradP, cage (icent, jcent))
//   e = 2  grad u   (wght_gradU, x at faces, cage (istag, jcent))
//   e = 3  grad v   (wght_gradV, y at faces, cage (icent, jstag))
//   e = 4  grad w   (wght_gradW, z at faces with nint, cage (icent, jcent))
// so every warp runs one kind of evaluation, and stores it in the group's
// slots.  One-warp blocks spread over the SMs evenly (five-warp blocks of 32
// faces left a few SMs with two blocks of the FP64-bound evaluations).  The
// last of the five warps to finish (a group ticket) forms each face's
// pressure force, viscous normal stress and their moments about pos_CM in
// the reference's operation order (face_loads) and sums the 32 faces' 12
// values with fixed shuffle trees; the last group to finish (the global
// ticket) adds the group sums (lane l takes groups l, l+32, ... in order, then
// a fixed shuffle tree) and updates the loads.  Tickets are reset by the
// warps that close them.
// Lit (the plain form): the reference's MLS construction (probe_value_lit,
// probe_grad_lit), the oracle's bits per face.  Otherwise (the precision
// form) the separable construction, which agrees with the reference's
// rank-one accumulation in absolute coordinates to that construction's
// round-off (amplified by its ~1e8 conditioning) at a fifth of the cost.
// scratch: [groups][13][32] evaluations, then [groups][12] group sums;
// tickets: [0] groups done, [1 + g] warps of group g done.
// ---------------------------------------------------------------------
constexpr int kLoadFaces = 32;

__device__ __forceinline__ void struct_probe(const double* __restrict__ tri_bar, const double* __restrict__ tri_nor,
                                             int t, double h, double pos[3], double nrm[3]) {
  for (int d = 0; d < 3; ++d) nrm[d] = tri_nor[3 * t + d];
  double s = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  for (int d = 0; d < 3; ++d) pos[d] = tri_bar[3 * t + d] + h * nrm[d] / s;
}

template <bool Lit>
__global__ void __launch_bounds__(kLoadFaces)
loads_face_kernel(LagArgs A, const double* __restrict__ pr, const double* __restrict__ vx,
                  const double* __restrict__ vy, const double* __restrict__ vz, const double* __restrict__ tri_bar,
                  const double* __restrict__ tri_nor, const double* __restrict__ sur, const int* __restrict__ ghost,
                  const StepParams* __restrict__ pp, double h, double ren, double* __restrict__ scratch,
                  int* __restrict__ flag, unsigned* __restrict__ tickets, RigidDev* __restrict__ r) {
  const unsigned FULL = 0xffffffffu;
  const int lf = threadIdx.x;
  const int grp = blockIdx.x / 5, e = blockIdx.x % 5, ngrp = gridDim.x / 5;
  double* evg = scratch + (size_t)grp * 13 * kLoadFaces;
  double* part = scratch + (size_t)ngrp * 13 * kLoadFaces;
  const int t = grp * kLoadFaces + lf;
  const bool live = t < A.nf && !ghost[t];
  const Grid& g = A.g;
  double pos[3], nrm[3];
  if (live) {
    struct_probe(tri_bar, tri_nor, t, h, pos, nrm);
    int icent = ffloor(pos[0] * g.dx1) + 1, istag = fnint(pos[0] * g.dx1) + 1;
    int jcent = ffloor(pos[1] * g.dx2) + 1, jstag = fnint(pos[1] * g.dx2) + 1;
    bool ok;
    if (e == 0) {
      double v = 0.0;
      ok = Lit ? probe_value_lit(A, pos, icent, jcent, pr, v) : probe_value_sep(A, pos, icent, jcent, pr, v);
      evg[lf] = ok ? v : 0.0;
    } else {
      double gr[3] = {0, 0, 0};
      const double* q = e == 1 ? pr : e == 2 ? vx : e == 3 ? vy : vz;
      const int pi1 = e == 2 ? istag : icent, pi2 = e == 3 ? jstag : jcent;
      const int sx = e == 2 ? 0 : 1, sy = e == 3 ? 0 : 1, sz = e == 4 ? 0 : 1;
      ok = Lit ? probe_grad_lit(A, pos, pi1, pi2, sx, sy, sz, e == 4, q, gr)
               : probe_grad_sep(A, pos, pi1, pi2, sx, sy, sz, e == 4, q, gr);
      for (int d = 0; d < 3; ++d) evg[(1 + 3 * (e - 1) + d) * kLoadFaces + lf] = ok ? gr[d] : 0.0;
    }
    if (!ok) atomicOr(flag, 1);
  }
  // the last of the group's five warps forms the loads of its 32 faces
  __threadfence();
  __syncwarp();
  unsigned done = 0;
  if (lf == 0) done = atomicAdd(&tickets[1 + grp], 1u);
  if (__shfl_sync(FULL, done, 0) != 4u) return;
  __threadfence();
  double cf[12];
  for (int q = 0; q < 12; ++q) cf[q] = 0.0;
  if (live) {
    double e13[13], rad[3];
    for (int q = 0; q < 13; ++q) e13[q] = __ldcg(evg + q * kLoadFaces + lf);
    for (int d = 0; d < 3; ++d) rad[d] = tri_bar[3 * t + d] - pp->pos[d];
    face_loads(e13, nrm, rad, sur[t], h, ren, cf);
  }
  // group sums (a shuffle tree over the group's faces per quantity)
  for (int q = 0; q < 12; ++q) {
    double v = cf[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (lf == 0) part[12 * (size_t)grp + q] = v;
  }
  if (lf == 0) tickets[1 + grp] = 0u;
  __threadfence();
  __syncwarp();
  unsigned gdone = 0;
  if (lf == 0) gdone = atomicAdd(&tickets[0], 1u);
  if (__shfl_sync(FULL, gdone, 0) != (unsigned)ngrp - 1u) return;
  __threadfence();
  // the last group: the loads (lane l takes groups l, l+32, ... in order, then
  // a fixed shuffle tree), the previous loads to the _m1 slots, the new ones
  // stored and added to the running sums (mls_structLoads.f90:21-24, 207-262)
  double tot[12];
  for (int q = 0; q < 12; ++q) {
    double v = 0.0;
    for (int b = lf; b < ngrp; b += 32) v += __ldcg(part + 12 * (size_t)b + q);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    tot[q] = v;
  }
  if (lf == 0) {
    for (int q = 0; q < 12; ++q) {        // packed [prn, tau, rprn, rtau]
      r->load1[q] = r->load[q];
      r->load[q] = tot[q];
      r->acc[q] = r->acc[q] + tot[q];
    }
    tickets[0] = 0u;
  }
}

// face -> vertex: qw_v(v) = sum over adjacent faces (ascending) of q_f*(A_f/3/A_v)
__global__ void face_to_vert_kernel(int nv, const int* __restrict__ adj_off, const int* __restrict__ adj_face,
                                    const double* __restrict__ sur, const double* __restrict__ avert,
                                    const double* __restrict__ qf_o, const double* __restrict__ qf_i,
                                    double* __restrict__ qv_o, double* __restrict__ qv_i) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double so = 0.0, si = 0.0, av = avert[v];
  for (int q = adj_off[v]; q < adj_off[v + 1]; ++q) {
    int f = adj_face[q];
    double w = sur[f] / 3.0 / av;
    so = so + qf_o[f] * w;
    si = si + qf_i[f] * w;
  }
  qv_o[v] = so;
  qv_i[v] = si;
}

__global__ void stefan_kernel(int nv, const int* __restrict__ ghostv, const double* __restrict__ vert_nor,
                              const double* __restrict__ qv_o, const double* __restrict__ qv_i, double cp_over_L,
                              const StepParams* __restrict__ pp, double* __restrict__ vmelt,
                              double* __restrict__ vmelt_m1, double* __restrict__ xyzv) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double dt = pp->dt, ga = pp->ga, ro = pp->ro;
  for (int d = 0; d < 3; ++d) vmelt_m1[3 * v + d] = vmelt[3 * v + d];
  if (ghostv[v]) return;
  double dq = qv_i[v] - qv_o[v];
  for (int d = 0; d < 3; ++d) {
    double vm = cp_over_L * dq * vert_nor[3 * v + d];
    vmelt[3 * v + d] = vm;
    xyzv[3 * v + d] = xyzv[3 * v + d] + dt * (ga * vm + ro * vmelt_m1[3 * v + d]);
  }
}

// ---------------------------------------------------------------------
// geometry refresh (particle.f90:165-193)
// ---------------------------------------------------------------------
// calculate_area, update_tri_normal, calc_centroids_from_vert of face t and
// its summands of calculate_volume and calc_rigidBody_params
__device__ __forceinline__ void face_geom_one(int t, const int* __restrict__ vof, const double* __restrict__ x,
                                              double* __restrict__ sur, double* __restrict__ nor,
                                              double* __restrict__ bar, double pp[12]) {
  int a = vof[3 * t] - 1, b = vof[3 * t + 1] - 1, d = vof[3 * t + 2] - 1;
  double x1 = x[3 * a], y1 = x[3 * a + 1], z1 = x[3 * a + 2];
  double x2 = x[3 * b], y2 = x[3 * b + 1], z2 = x[3 * b + 2];
  double x3 = x[3 * d], y3 = x[3 * d + 1], z3 = x[3 * d + 2];
  // calculate_area (triaux.f90:82-119)
  double d12 = sqrt(sqd(x1 - x2) + sqd(y1 - y2) + sqd(z1 - z2));
  double d23 = sqrt(sqd(x2 - x3) + sqd(y2 - y3) + sqd(z2 - z3));
  double d31 = sqrt(sqd(x3 - x1) + sqd(y3 - y1) + sqd(z3 - z1));
  double sp = (d12 + d23 + d31) / 2.0;
  double ar = sqrt(sp * (sp - d12) * (sp - d23) * (sp - d31));
  sur[t] = ar;
  // update_tri_normal (triaux.f90:183-232)
  double e1x = x2 - x1, e1y = y2 - y1, e1z = z2 - z1, e2x = x3 - x1, e2y = y3 - y1, e2z = z3 - z1;
  double n0 = e1y * e2z - e1z * e2y, n1 = e1z * e2x - e1x * e2z, n2 = e1x * e2y - e1y * e2x;
  double m = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  nor[3 * t] = n0 / m; nor[3 * t + 1] = n1 / m; nor[3 * t + 2] = n2 / m;
  // calc_centroids_from_vert (triaux.f90:308-323)
  bar[3 * t] = (x1 + x2 + x3) / 3.0; bar[3 * t + 1] = (y1 + y2 + y3) / 3.0; bar[3 * t + 2] = (z1 + z2 + z3) / 3.0;
  // calculate_volume summand (triaux.f90:53-80)
  double vol = x1 * (y2 * z3 - z2 * y3) + x2 * (y3 * z1 - z3 * y1) + x3 * (y1 * z2 - z1 * y2);
  // calc_rigidBody_params summands (RigidAuxRoutines.f90:704-733)
  double v = x1 * y2 * z3 + y1 * z2 * x3 + x2 * y3 * z1 - (x3 * y2 * z1 + x2 * y1 * z3 + y3 * z2 * x1);
  double x4 = x1 + x2 + x3, y4 = y1 + y2 + y3, z4 = z1 + z2 + z3;
  pp[0] = ar; pp[1] = vol; pp[2] = v; pp[3] = v * x4; pp[4] = v * y4; pp[5] = v * z4;
  pp[6] = v * (x1 * x1 + x2 * x2 + x3 * x3 + x4 * x4);
  pp[7] = v * (y1 * y1 + y2 * y2 + y3 * y3 + y4 * y4);
  pp[8] = v * (z1 * z1 + z2 * z2 + z3 * z3 + z4 * z4);
  pp[9] = v * (y1 * x1 + y2 * x2 + y3 * x3 + y4 * x4);
  pp[10] = v * (z1 * x1 + z2 * x2 + z3 * x3 + z4 * x4);
  pp[11] = v * (z1 * y1 + z2 * y2 + z3 * y3 + z4 * y4);
}

// the post-processing of calc_rigidBody_params (RigidAuxRoutines.f90:736-775)
// from the 12 body sums: [Surface, Volume1, Volume, pos_CM(3), InertTensor(9)]
__device__ void geom_finish(const double* sm, double dens_ratio, double* __restrict__ out) {
  double Surface = sm[0], Volume1 = sm[1] / 6.0;
  double Vol = sm[2], Cx = sm[3], Cy = sm[4], Cz = sm[5];
  double r = 1.0 / (4.0 * Vol);
  Cx = Cx * r; Cy = Cy * r; Cz = Cz * r;
  Vol = Vol / 6.0;
  out[0] = Surface; out[1] = Volume1; out[2] = Vol;
  out[3] = Cx; out[4] = Cy; out[5] = Cz;
  r = 1.0 / 120.0;
  double Ixy = sm[9] * r - Vol * Cy * Cx;
  double Ixz = sm[10] * r - Vol * Cz * Cx;
  double Iyz = sm[11] * r - Vol * Cz * Cy;
  double xx = sm[6] * r - Vol * Cx * Cx, yy = sm[7] * r - Vol * Cy * Cy, zz = sm[8] * r - Vol * Cz * Cz;
  double Ixx = yy + zz, Iyy = zz + xx, Izz = xx + yy;
  double I[9] = {Ixx, -Ixy, -Ixz, -Ixy, Iyy, -Iyz, -Ixz, -Iyz, Izz};
  for (int q = 0; q < 9; ++q) out[6 + q] = I[q] * dens_ratio;
}

// One thread per face.  The 12 per-face sums are added over the block (one
// quantity per warp: four values per lane in thread order, then a shuffle
// tree) into part[12 * block + q]; the last block to finish (a ticket
// counter, reset by that block) adds the block sums the same way (lane l
// takes blocks l, l+32, ... in order, then a fixed shuffle tree over the
// lanes) and writes the body's scalars to out.  Each warp's dependent FP64
// chain is a few additions per quantity: on this part an FP64 warp
// instruction holds the pipe for about 64 cycles however few lanes run.
constexpr int kGeomBlock = 128;
static_assert(kGeomBlock == 128, "four values per lane in the block sums");
__global__ void __launch_bounds__(kGeomBlock)
face_geom_kernel(int nf, const int* __restrict__ vof, const int* __restrict__ ghost, const double* __restrict__ x,
                 double* __restrict__ sur, double* __restrict__ nor, double* __restrict__ bar,
                 double* __restrict__ part /* 12 per block */, unsigned* __restrict__ ticket, double dens_ratio,
                 double* __restrict__ out) {
  const unsigned FULL = 0xffffffffu;
  __shared__ double ws[12][kGeomBlock];
  __shared__ double tot[12];
  __shared__ bool last;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  double pp[12];
  for (int q = 0; q < 12; ++q) pp[q] = 0.0;
  if (t < nf && !ghost[t]) face_geom_one(t, vof, x, sur, nor, bar, pp);
  for (int q = 0; q < 12; ++q) ws[q][threadIdx.x] = pp[q];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = warp; q < 12; q += kGeomBlock / 32) {
    double v = ws[q][lane] + ws[q][lane + 32] + ws[q][lane + 64] + ws[q][lane + 96];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (lane == 0) part[12 * (size_t)blockIdx.x + q] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int q = warp; q < 12; q += kGeomBlock / 32) {
    double v = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) v += __ldcg(part + 12 * (size_t)b + q);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
    if (lane == 0) tot[q] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    geom_finish(tot, dens_ratio, out);
    *ticket = 0u;
  }
}


__global__ void vert_geom_kernel(int nv, const int* __restrict__ adj_off, const int* __restrict__ adj_face,
                                 const int* __restrict__ ghostv, const double* __restrict__ sur,
                                 const double* __restrict__ nor, double* __restrict__ avert,
                                 double* __restrict__ vnor) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double av = 0, a0 = 0, a1 = 0, a2 = 0;
  for (int q = adj_off[v]; q < adj_off[v + 1]; ++q) {
    int f = adj_face[q];
    double s = sur[f];
    av = av + s / 3.0;
    a0 = a0 + s * nor[3 * f]; a1 = a1 + s * nor[3 * f + 1]; a2 = a2 + s * nor[3 * f + 2];
  }
  avert[v] = av;
  if (ghostv[v]) { vnor[3 * v] = a0; vnor[3 * v + 1] = a1; vnor[3 * v + 2] = a2; return; }
  double m = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
  vnor[3 * v] = a0 / m; vnor[3 * v + 1] = a1 / m; vnor[3 * v + 2] = a2 / m;
}

// calculate_eLengths (triaux.f90:277-306); flag bit 0 set when a live edge
// is shorter than thresh (the remesh trigger rm_flag)
__global__ void elength_kernel(int ne, const int* __restrict__ voe, const int* __restrict__ ghoste,
                               const double* __restrict__ x, double thresh, double* __restrict__ el,
                               int* __restrict__ flag) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne || ghoste[e]) return;
  int v1 = voe[2 * e] - 1, v2 = voe[2 * e + 1] - 1;
  double len = sqrt(sqd(x[3 * v1] - x[3 * v2]) + sqd(x[3 * v1 + 1] - x[3 * v2 + 1]) + sqd(x[3 * v1 + 2] - x[3 * v2 + 2]));
  el[e] = len;
  if (flag && len < thresh) atomicOr(flag, 1);
}

// calculate_skewness (triaux.f90:325-358)
__global__ void skewness_kernel(int nf, const int* __restrict__ eof, const int* __restrict__ ghost,
                                const double* __restrict__ el, const double* __restrict__ sur,
                                double* __restrict__ skew) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf || ghost[t]) return;
  double perim = el[eof[3 * t] - 1] + el[eof[3 * t + 1] - 1] + el[eof[3 * t + 2] - 1];
  double sur_opt = sqrt(3.0) / 4.0 * sqd(perim / 3.0);
  skew[t] = (sur_opt - sur[t]) / sur_opt;
}

// update_tri_velocity (RigidAuxRoutines.f90:902-928) after a remesh:
// vel_tri = vel_CM + omega x (tri_bar - pos_CM), pos_CM of the refreshed
// geometry (geom + 3)
__global__ void tri_velocity_kernel(int nf, const int* __restrict__ ghost, const double* __restrict__ bar,
                                    const double* __restrict__ geom, const double* __restrict__ vel,
                                    const double* __restrict__ om, double* __restrict__ vel_tri) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf || ghost[t]) return;
  double r[3];
  for (int d = 0; d < 3; ++d) r[d] = bar[3 * t + d] - geom[3 + d];
  double c0 = om[1] * r[2] - r[1] * om[2];
  double c1 = om[2] * r[0] - r[2] * om[0];
  double c2 = om[0] * r[1] - r[0] * om[1];
  vel_tri[3 * t] = vel[0] + c0;
  vel_tri[3 * t + 1] = vel[1] + c1;
  vel_tri[3 * t + 2] = vel[2] + c2;
}

__global__ void cfac_kernel(int nf, const double* __restrict__ sur, double h, double celvol, double* __restrict__ cfac) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nf) cfac[t] = (sur[t] * h) / celvol;
}

// ---------------------------------------------------------------------
// narrow-band tagging (genSDF.f90:120-192)
// ---------------------------------------------------------------------
__device__ double point_tri_dist(const double P[3], const double V0[3], const double V1[3], const double V2[3]) {
  double E0[3], E1[3], DE[3];
  for (int d = 0; d < 3; ++d) { E0[d] = V1[d] - V0[d]; E1[d] = V2[d] - V0[d]; DE[d] = V0[d] - P[d]; }
  double a = E0[0] * E0[0] + E0[1] * E0[1] + E0[2] * E0[2];
  double b = E0[0] * E1[0] + E0[1] * E1[1] + E0[2] * E1[2];
  double cc = E1[0] * E1[0] + E1[1] * E1[1] + E1[2] * E1[2];
  double d = E0[0] * DE[0] + E0[1] * DE[1] + E0[2] * DE[2];
  double e = E1[0] * DE[0] + E1[1] * DE[1] + E1[2] * DE[2];
  double det = a * cc - b * b, s = b * e - cc * d, t = b * d - a * e;
  if (s + t <= det) {
    if (s < 0.0) {
      if (t < 0.0) {
        if (d < 0.0) { t = 0.0; s = (-d >= a) ? 1.0 : -d / a; }
        else { s = 0.0; if (e >= 0.0) t = 0.0; else if (-e >= cc) t = 1.0; else t = -e / cc; }
      } else {
        s = 0.0; if (e >= 0.0) t = 0.0; else if (-e >= cc) t = 1.0; else t = -e / cc;
      }
    } else if (t < 0.0) {
      t = 0.0; if (d >= 0.0) s = 0.0; else if (-d >= a) s = 1.0; else s = -d / a;
    } else {
      double invDet = 1.0 / det; s = s * invDet; t = t * invDet;
    }
  } else {
    if (s < 0.0) {
      double tmp0 = b + d, tmp1 = cc + e;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a - 2.0 * b + cc;
        if (numer >= denom) { s = 1.0; t = 0.0; } else { s = numer / denom; t = 1.0 - s; }
      } else {
        s = 0.0; if (tmp1 <= 0.0) t = 1.0; else if (e >= 0.0) t = 0.0; else t = -e / cc;
      }
    } else if (t < 0.0) {
      double tmp0 = b + e, tmp1 = a + d;
      if (tmp1 > tmp0) {
        double numer = tmp1 - tmp0, denom = a - 2.0 * b + cc;
        if (numer >= denom) { t = 1.0; s = 0.0; } else { t = numer / denom; s = 1.0 - t; }
      } else {
        t = 0.0; if (tmp1 <= 0.0) s = 1.0; else if (d >= 0.0) s = 0.0; else s = -d / a;
      }
    } else {
      double numer = cc + e - b - d, denom = a - 2.0 * b + cc;
      if (numer <= 0.0) s = 0.0; else if (numer >= denom) s = 1.0; else s = numer / denom;
      t = 1.0 - s;
    }
  }
  double D0 = (V0[0] + s * E0[0] + t * E1[0]) - P[0];
  double D1 = (V0[1] + s * E0[1] + t * E1[1]) - P[1];
  double D2 = (V0[2] + s * E0[2] + t * E1[2]) - P[2];
  return sqrt(D0 * D0 + D1 * D1 + D2 * D2);
}

struct TagArgs {
  LagArgs L;
  const double* x; const int* vof; const int* ghost; const double* bar; const double* nor;
};

__device__ __forceinline__ void tri_verts(const TagArgs& T, int f, double V0[3], double V1[3], double V2[3]) {
  int a = T.vof[3 * f] - 1, b = T.vof[3 * f + 1] - 1, c = T.vof[3 * f + 2] - 1;
  if (!(MIBM_IDX_OK(a, T.L.nv) & MIBM_IDX_OK(b, T.L.nv) & MIBM_IDX_OK(c, T.L.nv))) a = b = c = 0;
  for (int d = 0; d < 3; ++d) { V0[d] = T.x[3 * a + d]; V1[d] = T.x[3 * b + d]; V2[d] = T.x[3 * c + d]; }
}

__global__ void sdf_reset_kernel(Grid g, unsigned long long* __restrict__ sdf_bits, int* __restrict__ winner,
                                 unsigned* __restrict__ band_ub) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.cells) return;
  sdf_bits[t] = (unsigned long long)__double_as_longlong(999.0);   // genSDF.f90:138
  winner[t] = INT_MAX;
  if (band_ub) band_ub[t] = 0x7f800000u;                           // +inf
}

// Culling of the narrow-band distance pass.  With c the face centroid and
// R >= the largest centroid-vertex distance, every point of the face lies
// within R of c, so for a cell centre P
//   |P - c| - R  <=  dist(P, face)  <=  |P - c|.
// Pass U takes the minimum of the upper bounds over the candidate faces of a
// cell; the exact pass skips a face whose lower bound exceeds that minimum:
// such a face is strictly farther than the nearest one, so the minimum, the
// set of faces tied at it and hence the earliest-face winner are unchanged.
// The bounds are evaluated in FP32 from FP32 copies of the coordinates
// (|x| < 13, rounding error < 1e-6 per coordinate, < 3e-6 on |P - c|), and
// kBandMargin covers that error on both sides.
constexpr float kBandMargin = 8e-6f;

__global__ void cm32_kernel(LagArgs A, float* __restrict__ cm32) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.clen) return;
  cm32[t] = (float)A.xm[t];
  cm32[A.clen + t] = (float)A.ym[t];
  cm32[2 * A.clen + t] = (float)A.zm[t];
}

__global__ void band_prep_kernel(TagArgs T, float4* __restrict__ face4, int4* __restrict__ face_cell) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  const LagArgs& A = T.L;
  if (f >= A.nf) return;
  const Grid& g = A.g;
  double pos[3] = {T.bar[3 * f], T.bar[3 * f + 1], T.bar[3 * f + 2]};
  double V[3][3];
  tri_verts(T, f, V[0], V[1], V[2]);
  double r2 = 0.0;
  for (int v = 0; v < 3; ++v) {
    double dx = V[v][0] - pos[0], dy = V[v][1] - pos[1], dz = V[v][2] - pos[2];
    r2 = fmax(r2, dx * dx + dy * dy + dz * dz);
  }
  float R = (float)sqrt(r2);
  R = R * 1.000001f + 1e-30f;                                        // round the radius up
  face4[f] = make_float4((float)pos[0], (float)pos[1], (float)pos[2], R);
  // base cell of the band, as band_kernel derives it (genSDF.f90:151-153)
  face_cell[f] = make_int4(ffloor(pos[0] * g.dx1) + 1, ffloor(pos[1] * g.dx2) + 1, ffloor(pos[2] * g.dx3) + 1, 0);
}

__device__ __forceinline__ float band_center_dist(const float* __restrict__ cm32, int clen, int coff, int ii, int jj,
                                                  int kk, float4 c) {
  float px = cm32[min(max(ii + coff, 0), clen - 1)];
  float py = cm32[clen + min(max(jj + coff, 0), clen - 1)];
  float pz = cm32[2 * clen + min(max(kk + coff, 0), clen - 1)];
  float dx = px - c.x, dy = py - c.y, dz = pz - c.z;
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// after pass U: pairs whose lower bound does not exceed the cell's bound go
// to a compact list (warp-aggregated append), the others get the "far"
// distance 1e300 so that they never match the cell minimum
__global__ void band_select_kernel(TagArgs T, const float4* __restrict__ face4, const int4* __restrict__ face_cell,
                                   const float* __restrict__ cm32, const unsigned* __restrict__ band_ub,
                                   double* __restrict__ dist_buf, int* __restrict__ list, int* __restrict__ count) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int f = (int)(gid / 125), q = (int)(gid % 125);
  const LagArgs& A = T.L;
  bool keep = false;
  if (f < A.nf && !T.ghost[f]) {
    const Grid& g = A.g;
    int4 b = face_cell[f];
    int ii = b.x - 2 + q % 5, jj = b.y - 2 + (q / 5) % 5, kk = b.z - 2 + q / 25;
    int im = fmod_pos(ii - 1, g.n1m), jm = fmod_pos(jj - 1, g.n1m), km = fmod_pos(kk - 1, g.n3m);
    float4 fc = face4[f];
    float lb = band_center_dist(cm32, A.clen, A.coff, ii, jj, kk, fc) - fc.w - kBandMargin;
    keep = !(lb > __uint_as_float(band_ub[cidx(g, im, jm, km)]));
    if (!keep) dist_buf[gid] = 1e300;
  }
  unsigned m = __ballot_sync(0xffffffffu, keep);
  if (!m) return;
  int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (keep) list[base + __popc(m & ((1u << lane) - 1u))] = (int)gid;
}

// pass U: per (face, band cell) the upper bound |P - c| + margin, min per cell
__global__ void band_ub_kernel(TagArgs T, const float4* __restrict__ face4, const int4* __restrict__ face_cell,
                               const float* __restrict__ cm32, unsigned* __restrict__ band_ub) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int f = (int)(gid / 125), q = (int)(gid % 125);
  const LagArgs& A = T.L;
  if (f >= A.nf || T.ghost[f]) return;
  const Grid& g = A.g;
  int4 b = face_cell[f];
  int ii = b.x - 2 + q % 5, jj = b.y - 2 + (q / 5) % 5, kk = b.z - 2 + q / 25;
  int im = fmod_pos(ii - 1, g.n1m), jm = fmod_pos(jj - 1, g.n1m), km = fmod_pos(kk - 1, g.n3m);
  float ub = band_center_dist(cm32, A.clen, A.coff, ii, jj, kk, face4[f]) + kBandMargin;
  atomicMin(&band_ub[cidx(g, im, jm, km)], __float_as_uint(ub));
}

// one thread per (triangle, band cell) of the compact list of
// band_select_kernel (entry t < *count; the pairs it culls can neither hold
// a cell's minimum nor win it); pass 0: distance (stored) and the minimum
// per cell, pass 1: the earliest triangle at that distance, pass 2: the
// winner writes the signed distance and the VOF
__global__ void band_kernel(TagArgs T, int pass, unsigned long long* __restrict__ sdf_bits, int* __restrict__ winner,
                            double* __restrict__ vofp, double* __restrict__ dist_buf, const int4* __restrict__ face_cell,
                            const int* __restrict__ list, const int* __restrict__ count) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= *count) return;
  gid = list[gid];
  int f = (int)(gid / 125), q = (int)(gid % 125);
  const LagArgs& A = T.L;
  if (f >= A.nf || T.ghost[f]) return;
  const Grid& g = A.g;
  int4 b = face_cell[f];
  int ii = b.x - 2 + q % 5, jj = b.y - 2 + (q / 5) % 5, kk = b.z - 2 + q / 25;
  int im = fmod_pos(ii - 1, g.n1m), jm = fmod_pos(jj - 1, g.n1m), km = fmod_pos(kk - 1, g.n3m);
  size_t c0 = cidx(g, im, jm, km);
  double dist;
  if (pass == 0) {
    double P[3] = {coord(A, 0, 1, ii), coord(A, 1, 1, jj), coord(A, 2, 1, kk)};
    double V0[3], V1[3], V2[3];
    tri_verts(T, f, V0, V1, V2);
    dist = point_tri_dist(P, V0, V1, V2);
    dist_buf[gid] = dist;
    atomicMin(&sdf_bits[c0], (unsigned long long)__double_as_longlong(dist));
    return;
  }
  dist = dist_buf[gid];
  unsigned long long bits = (unsigned long long)__double_as_longlong(dist);
  if (pass == 1) {
    if (sdf_bits[c0] == bits && dist < 999.0) atomicMin(&winner[c0], f);
    return;
  }
  if (winner[c0] != f || sdf_bits[c0] != bits) return;
  double pos[3] = {T.bar[3 * f], T.bar[3 * f + 1], T.bar[3 * f + 2]};
  double P[3] = {coord(A, 0, 1, ii), coord(A, 1, 1, jj), coord(A, 2, 1, kk)};
  double Q0 = pos[0] - P[0], Q1 = pos[1] - P[1], Q2 = pos[2] - P[2];
  double dotval = T.nor[3 * f] * Q0 + T.nor[3 * f + 1] * Q1 + T.nor[3 * f + 2] * Q2;
  double sgnd = dist * (-copysign(1.0, dotval));
  double eps = 1.0 / g.dx1, vof;
  const double pi = 3.141592653589793238462643;
  if (sgnd <= -eps) vof = 0.0;
  else if (sgnd >= eps) vof = 1.0;
  else vof = 0.5 * (1.0 + sgnd * g.dx1 + (1.0 / pi) * sin(pi * sgnd * g.dx1));
  vofp[c0] = vof;
  sdf_bits[c0] = (unsigned long long)__double_as_longlong(sgnd);
}

// initial full tagging: one thread per cell of the bounding box
__device__ bool ray_tri(const double C[3], const double Q[3], const double V0[3], const double V1[3],
                        const double V2[3], double ip[3]) {
  const double EPS = 1e-12;
  double dir[3] = {Q[0] - C[0], Q[1] - C[1], Q[2] - C[2]};
  double e1[3], e2[3], h[3], s[3], q[3];
  for (int d = 0; d < 3; ++d) { e1[d] = V1[d] - V0[d]; e2[d] = V2[d] - V0[d]; }
  h[0] = dir[1] * e2[2] - dir[2] * e2[1]; h[1] = dir[2] * e2[0] - dir[0] * e2[2]; h[2] = dir[0] * e2[1] - dir[1] * e2[0];
  double a = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
  if (fabs(a) < EPS) return false;
  double f = 1.0 / a;
  for (int d = 0; d < 3; ++d) s[d] = C[d] - V0[d];
  double u = f * (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
  if (u < 0.0 || u > 1.0) return false;
  q[0] = s[1] * e1[2] - s[2] * e1[1]; q[1] = s[2] * e1[0] - s[0] * e1[2]; q[2] = s[0] * e1[1] - s[1] * e1[0];
  double v = f * (dir[0] * q[0] + dir[1] * q[1] + dir[2] * q[2]);
  if (v < 0.0 || u + v > 1.0) return false;
  double t = f * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
  if (t < 0.0 || t > 1.0) return false;
  for (int d = 0; d < 3; ++d) ip[d] = C[d] + t * dir[d];
  return true;
}

// pass A: ray parity / interface rule per bounding-box cell (rayTagQ_pencil,
// pencil_rayTag.f90:381-460) -> tmp[gid]
__global__ void initial_tag_kernel(TagArgs T, int bx0, int by0, int bz0, int nbx, int nby, int nbz,
                                   double* __restrict__ tmp) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)nbx * nby * nbz) return;
  const LagArgs& A = T.L;
  const Grid& g = A.g;
  int i = bx0 + (int)(gid % nbx), j = by0 + (int)((gid / nbx) % nby), kk = bz0 + (int)(gid / ((long long)nbx * nby));
  double Q[3] = {coord(A, 0, 1, i), coord(A, 1, 1, j), coord(A, 2, 1, kk)};
  double C[3] = {-g.xlen * 10.0, Q[1], Q[2]};
  double ymin = Q[1] - 0.5 / g.dx2, ymax = Q[1] + 0.5 / g.dx2, zmin = Q[2] - 0.5 / g.dx3, zmax = Q[2] + 0.5 / g.dx3;
  double xmin = Q[0] - 0.5 / g.dx1, xmax = Q[0] + 0.5 / g.dx1;
  int count = 0;
  double vof = -1.0;
  for (int f = 0; f < A.nf; ++f) {
    if (T.ghost[f]) continue;
    double V0[3], V1[3], V2[3];
    tri_verts(T, f, V0, V1, V2);
    double ylo = fmin(V0[1], fmin(V1[1], V2[1])), yhi = fmax(V0[1], fmax(V1[1], V2[1]));
    double zlo = fmin(V0[2], fmin(V1[2], V2[2])), zhi = fmax(V0[2], fmax(V1[2], V2[2]));
    if (yhi < ymin || ylo > ymax || zhi < zmin || zlo > zmax) continue;
    double xlo = fmin(V0[0], fmin(V1[0], V2[0])), xhi = fmax(V0[0], fmax(V1[0], V2[0]));
    if (!(xhi < xmin || xlo > xmax)) { vof = 0.5; break; }
    double ip[3];
    if (ray_tri(C, Q, V0, V1, V2, ip)) {
      if (ip[0] >= xmin && ip[0] <= xmax && ip[1] >= ymin && ip[1] <= ymax && ip[2] >= zmin && ip[2] <= zmax) {
        vof = 0.5;
        break;
      }
      ++count;
    }
  }
  if (vof < 0) vof = (count % 2 == 0) ? 1.0 : 0.0;
  tmp[gid] = vof;
}

// reference loop order (i outermost, kk innermost) as an integer key
__device__ __forceinline__ int box_order(long long gid, int nbx, int nby, int nbz) {
  int io = (int)(gid % nbx), jo = (int)((gid / nbx) % nby), ko = (int)(gid / ((long long)nbx * nby));
  return (io * nby + jo) * nbz + ko;
}

// pass B/C: a cell reached through several periodic images keeps the first
// value below 1 in loop order (pencil_rayTag.f90:298-302)
__global__ void initial_claim_kernel(Grid g, int bx0, int by0, int bz0, int nbx, int nby, int nbz,
                                     const double* __restrict__ tmp, int* __restrict__ claim, double* __restrict__ vofp,
                                     int pass) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)nbx * nby * nbz) return;
  double v = tmp[gid];
  if (!(v < 1.0)) return;
  int i = bx0 + (int)(gid % nbx), j = by0 + (int)((gid / nbx) % nby), kk = bz0 + (int)(gid / ((long long)nbx * nby));
  size_t c0 = cidx(g, fmod_pos(i - 1, g.n1m), fmod_pos(j - 1, g.n2m), fmod_pos(kk - 1, g.n3m));
  int key = box_order(gid, nbx, nby, nbz);
  if (pass == 0) atomicMin(&claim[c0], key);
  else if (claim[c0] == key) vofp[c0] = v;
}

__global__ void fill_kernel(Grid g, double* __restrict__ a, double v) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.cells) a[t] = v;
}

// ---------------------------------------------------------------------
// per-context Lagrangian state
// ---------------------------------------------------------------------
struct LagState {
  Ctx* c = nullptr;
  int* adj_off = nullptr;
  int* adj_face = nullptr;
  int adj_nf = -1, adj_nv = -1;
  double* face_part = nullptr;
  double* geom_out = nullptr;   // device [Surface, Volume1, Vol, Cx, Cy, Cz, InertTensor(9)]
  unsigned* geom_ticket = nullptr;   // blocks of face_geom_kernel done (0 between launches)
  double* loads_ev = nullptr;   // structural loads: per 32-face group 13 x 32 evaluations, then 12 group sums
  unsigned* loads_ticket = nullptr;   // groups done, then warps done per group (0 between launches)
  int* rm_flag = nullptr;       // remesh trigger (device)
  double* mean3 = nullptr;
  int* winner = nullptr;
  double* dist_buf = nullptr;
  // narrow-band culling: per cell an FP32 upper bound of the nearest face
  // distance (float bits), per face its FP32 centroid and circumradius and
  // the base cell of its 5^3 band, FP32 cell-centre coordinates
  unsigned* band_ub = nullptr;
  int* band_list = nullptr;      // (face, cell) pairs that survive the bound, and their count
  int* band_count = nullptr;
  float4* face4 = nullptr;
  int4* face_cell = nullptr;
  float* cm32 = nullptr;
  // merged scatter plan
  int plan_n = 0, plan_cap = 0, nblk = 0;
  int *key = nullptr, *src = nullptr, *tmp_key = nullptr, *tmp_src = nullptr, *hist = nullptr;
  int* tsum = nullptr;   // tile totals of the histogram scan
  int *hidx = nullptr, *heads = nullptr, *nheads = nullptr, *htsum = nullptr;   // run heads of the plan
  int *res_key = nullptr, *res_src = nullptr;   // buffers holding the sorted result
  int* saved = nullptr;                          // 7 ints per face: pind(1:6), ghost
  int* dirty = nullptr;
  double* segval = nullptr;
  bool force_rebuild = true;
  bool weights_valid = false;                    // stationary cages: weights kept
};
static std::vector<LagState*> g_lag;

static LagState* lag_of(Ctx* c) {
  for (auto* s : g_lag)
    if (s->c == c) return s;
  LagState* s = new LagState();
  s->c = c;
  g_lag.push_back(s);
  return s;
}

// The mesh changed on the host side: the scatter plan is rebuilt from
// scratch and the MLS weights recomputed.  The step graph stays valid (the
// rebuild is requested through pinned memory read at replay) unless the
// weights of a stationary body were being reused, which changes the launch
// sequence.
void lagr_invalidate(Ctx* c) {
  ++c->geom_gen;
  LagState* s = lag_of(c);
  s->force_rebuild = true;
  if (c->I(MIBM_I_STATIONARY) && s->weights_valid) ++c->lag_gen;
  s->weights_valid = false;
}

// Per step, while its parameter blocks are filled: a pending request to
// rebuild the scatter plan from scratch goes into substep 0's block, which
// the step reads on the device (so a step graph stays valid across uploads).
int lagr_take_plan_request(Ctx* c) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return 0;
  LagState* s = lag_of(c);
  int r = s->force_rebuild ? 1 : 0;
  s->force_rebuild = false;
  return r;
}

// the face/vertex/edge relations changed (a remesh or a host upload of the
// connectivity): rebuild the vertex->face lists too
void lagr_topology_changed(Ctx* c) {
  lagr_invalidate(c);
  lag_of(c)->adj_nf = -1;
}

static bool ensure_adjacency(Ctx* c) {
  LagState* s = lag_of(c);
  if (s->adj_off && s->adj_nf == c->maxnf && s->adj_nv == c->maxnv) return true;
  std::vector<int> vof(3 * (size_t)c->maxnf), ghost(c->maxnf);
  cudaMemcpy(vof.data(), c->dm[MIBM_M_VERT_OF_FACE], vof.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(ghost.data(), c->dm[MIBM_M_GHOST_FACE], ghost.size() * 4, cudaMemcpyDeviceToHost);
  std::vector<int> cnt(c->maxnv + 1, 0);
  for (int f = 0; f < c->maxnf; ++f) {
    if (ghost[f]) continue;
    for (int q = 0; q < 3; ++q) {
      int v = vof[3 * f + q] - 1;
      if (v < 0 || v >= c->maxnv) { fail(c, MIBM_EINVAL, "vert_of_face out of range"); return false; }
      cnt[v + 1]++;
    }
  }
  for (int v = 0; v < c->maxnv; ++v) cnt[v + 1] += cnt[v];
  std::vector<int> face(cnt[c->maxnv]), fill(cnt.begin(), cnt.end() - 1);
  for (int f = 0; f < c->maxnf; ++f) {      // ascending face order per vertex
    if (ghost[f]) continue;
    for (int q = 0; q < 3; ++q) face[fill[vof[3 * f + q] - 1]++] = f;
  }
  cudaFree(s->adj_off); cudaFree(s->adj_face);
  if (!cuda_ok(c, cudaMalloc(&s->adj_off, cnt.size() * 4), "adj")) return false;
  if (!cuda_ok(c, cudaMalloc(&s->adj_face, std::max<size_t>(1, face.size()) * 4), "adj")) return false;
  cudaMemcpy(s->adj_off, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->adj_face, face.data(), face.size() * 4, cudaMemcpyHostToDevice);
  s->adj_nf = c->maxnf; s->adj_nv = c->maxnv;
  return true;
}

static bool ensure_lag_buffers(Ctx* c) {
  LagState* s = lag_of(c);
  if (!s->face_part) {
    if (!cuda_ok(c, cudaMalloc(&s->face_part, sizeof(double) * 12 * std::max(1, c->maxnf)), "lag")) return false;
    if (!cuda_ok(c, cudaMalloc(&s->geom_out, sizeof(double) * 16), "lag")) return false;
    if (!cuda_ok(c, cudaMalloc(&s->geom_ticket, sizeof(unsigned)), "lag")) return false;
    cudaMemsetAsync(s->geom_out, 0, sizeof(double) * 16, c->stream);
    cudaMemsetAsync(s->geom_ticket, 0, sizeof(unsigned), c->stream);
    // [0..3) FP64 mean force, [4..6) the same rounded to FP32 (3 floats)
    // [0..2] the means, [4..5] their FP32 copies, [7] seg_mean_kernel's ticket
    if (!cuda_ok(c, cudaMalloc(&s->mean3, sizeof(double) * 8), "lag")) return false;
    cudaMemsetAsync(s->mean3, 0, sizeof(double) * 8, c->stream);
  }
  if (!c->tri_coef)
    if (!cuda_ok(c, cudaMalloc(&c->tri_coef, sizeof(double) * 4 * std::max(1, c->maxnf)), "lag")) return false;
  if (!s->key) {
    int n = 4 * 27 * std::max(1, c->maxnf);
    s->nblk = (n + kSortChunk - 1) / kSortChunk;
    bool ok = cuda_ok(c, cudaMalloc(&s->key, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->src, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->tmp_key, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->tmp_src, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->hist, sizeof(int) * 256 * (size_t)s->nblk), "plan") &&
              cuda_ok(c, cudaMalloc(&s->tsum, sizeof(int) * (size_t)div_up(256 * (size_t)s->nblk, 1024)), "plan") &&
              cuda_ok(c, cudaMalloc(&s->saved, sizeof(int) * 7 * (size_t)std::max(1, c->maxnf)), "plan") &&
              cuda_ok(c, cudaMalloc(&s->dirty, sizeof(int)), "plan") &&
              cuda_ok(c, cudaMalloc(&s->segval, sizeof(double) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->hidx, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->heads, sizeof(int) * n), "plan") &&
              cuda_ok(c, cudaMalloc(&s->nheads, sizeof(int)), "plan") &&
              cuda_ok(c, cudaMalloc(&s->htsum, sizeof(int) * (size_t)div_up(n, 1024)), "plan");
    if (!ok) return false;
    s->plan_n = n;
    cudaMemsetAsync(s->saved, 0xff, sizeof(int) * 7 * (size_t)std::max(1, c->maxnf), c->stream);
    cudaMemsetAsync(s->nheads, 0, sizeof(int), c->stream);
  }
  return true;
}

// Flags raised by device kernels (singular MLS matrix).  In the fused step
// they are read once at the end of the step.
static bool check_flag(Ctx* c, const char* what) {
  cudaMemcpyAsync(c->hflag, c->dflag, 4, cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), what)) return false;
  if (c->hflag[0]) {
    fail(c, MIBM_ENUMERIC, std::string(what) + ((c->hflag[0] & 2) ? ": singular inertia tensor (dgetrf info /= 0)"
                                                                  : ": singular MLS moment matrix (dgetrf info /= 0)"));
    cudaMemsetAsync(c->dflag, 0, 4, c->stream);
    return false;
  }
  return true;
}

// Host check of the connectivity every Lagrangian kernel dereferences
// (vertex indices in 1..maxnv); also builds the vertex->face lists.
bool validate_mesh(Ctx* c) {
  LagState* s = lag_of(c);
  s->adj_nf = -1;   // force a rebuild from the current device copy
  return ensure_adjacency(c);
}

// (Re)build the merged scatter plan when the cage centres changed.
// dp: inside the fused step, the substep's parameter block, whose
// force_plan carries a rebuild request (lagr_take_plan_request); nullptr
// (drop-ins): the pending request is applied now.  A request raised inside
// a step (a remesh, which runs without a step graph) is applied now too.
static void update_plan(Ctx* c, const StepParams* dp) {
  LagState* s = lag_of(c);
  int nf = c->maxnf, n = s->plan_n;
  cudaMemsetAsync(s->dirty, s->force_rebuild ? 1 : 0, sizeof(int), c->stream);   // non-zero: dirty
  s->force_rebuild = false;
  const int* pind = M<int>(c, MIBM_M_PIND);
  const int* ghost = M<int>(c, MIBM_M_GHOST_FACE);
  { MIBM_PROF(c, "plan_check");
    plan_check_kernel<<<div_up(nf, 256), 256, 0, c->stream>>>(nf, pind, ghost, s->saved, s->dirty, dp); }
  { MIBM_PROF(c, "plan_keys");
    plan_keys_kernel<<<div_up(n, 256), 256, 0, c->stream>>>(c->g, nf, pind, ghost, s->dirty, s->tmp_key, s->tmp_src); }
  int* kin = s->tmp_key; int* vin = s->tmp_src; int* kout = s->key; int* vout = s->src;
  int bits = 1;
  while ((size_t(1) << bits) <= 4 * c->g.cells) ++bits;
  int passes = (bits + 7) / 8;
  for (int ps = 0; ps < passes; ++ps) {
    int shift = 8 * ps;
    { MIBM_PROF(c, "radix_hist");
      radix_hist_kernel<<<s->nblk, 256, 0, c->stream>>>(kin, n, shift, s->nblk, s->dirty, s->hist); }
    { MIBM_PROF(c, "radix_scan");
      int m = 256 * s->nblk;
      unsigned tiles = div_up(m, 1024);
      scan_tile_kernel<<<tiles, 1024, 0, c->stream>>>(s->hist, m, s->tsum, s->dirty);
      scan_kernel<<<1, 1024, 0, c->stream>>>(s->tsum, (int)tiles, s->dirty);
      scan_add_kernel<<<tiles, 1024, 0, c->stream>>>(s->hist, m, s->tsum, s->dirty); }
    { MIBM_PROF(c, "radix_scatter");
      radix_scatter_kernel<<<s->nblk, 256, 0, c->stream>>>(kin, vin, kout, vout, n, shift, s->nblk, s->hist, s->dirty); }
    std::swap(kin, kout); std::swap(vin, vout);
  }
  s->res_key = kin; s->res_src = vin;         // fixed per grid: the buffers of the last pass
  { MIBM_PROF(c, "plan_heads");
    const unsigned tiles = div_up(n, 1024);
    head_flag_kernel<<<tiles, 1024, 0, c->stream>>>(n, c->g.cells, s->res_key, s->dirty, s->hidx);
    scan_tile_kernel<<<tiles, 1024, 0, c->stream>>>(s->hidx, n, s->htsum, s->dirty);
    scan_kernel<<<1, 1024, 0, c->stream>>>(s->htsum, (int)tiles, s->dirty);
    scan_add_kernel<<<tiles, 1024, 0, c->stream>>>(s->hidx, n, s->htsum, s->dirty);
    head_compact_kernel<<<tiles, 1024, 0, c->stream>>>(n, c->g.cells, s->res_key, s->hidx, s->dirty, s->heads,
                                                       s->nheads); }
  c->launches += 5;
  { MIBM_PROF(c, "plan_commit");
    plan_commit_kernel<<<div_up(nf, 256), 256, 0, c->stream>>>(nf, pind, ghost, s->saved, s->dirty); }
  c->launches += 3 + 5 * passes;
  MIBM_LAUNCH_CHECK(c, "scatter plan");
}

// m32: base of the FP32 mirrors (u, v, w, T at 0, cells, 2 cells, 3 cells)
// that the scatter keeps equal to the forced fields, or null
static ScatterOut scatter_out(Ctx* c, bool into_fields, float* m32) {
  ScatterOut O;
  for (int q = 0; q < 4; ++q) O.m32[q] = (into_fields && m32) ? m32 + (size_t)q * c->g.cells : nullptr;
  static const int fo[4] = {MIBM_F_FORXC, MIBM_F_FORYC, MIBM_F_FORZC, MIBM_F_FORTEMP};
  static const int fq[4] = {MIBM_F_VX, MIBM_F_VY, MIBM_F_VZ, MIBM_F_TEMP};
  for (int q = 0; q < 4; ++q) O.f[q] = c->df[into_fields ? fq[q] : fo[q]];
  O.phi[0] = M<double>(c, MIBM_M_PTXAB_Q1); O.phi[1] = M<double>(c, MIBM_M_PTXAB_Q2);
  O.phi[2] = M<double>(c, MIBM_M_PTXAB_Q3); O.phi[3] = M<double>(c, MIBM_M_PTXAB_TEMP);
  return O;
}

static void force_coefficients(Ctx* c) {
  ForceArgs F;
  F.q[0] = c->df[MIBM_F_VX]; F.q[1] = c->df[MIBM_F_VY]; F.q[2] = c->df[MIBM_F_VZ]; F.q[3] = c->df[MIBM_F_TEMP];
  F.ptx[0] = M<double>(c, MIBM_M_PTXAB_Q1); F.ptx[1] = M<double>(c, MIBM_M_PTXAB_Q2);
  F.ptx[2] = M<double>(c, MIBM_M_PTXAB_Q3); F.ptx[3] = M<double>(c, MIBM_M_PTXAB_TEMP);
  F.vel_tri = M<double>(c, MIBM_M_VEL_TRI); F.cfac = M<double>(c, MIBM_M_CFAC);
  F.pind = M<int>(c, MIBM_M_PIND); F.ghost = M<int>(c, MIBM_M_GHOST_FACE);
  { MIBM_PROF(c, "force_coef");
    force_coef_kernel<<<div_up(4 * (size_t)c->maxnf, 128), 128, 0, c->stream>>>(c->g, c->maxnf, F, c->S(MIBM_S_TMELT),
                                                                                  c->tri_coef); }
  ++c->launches;
}

static void scatter(Ctx* c, bool into_fields, int lo, int hi, bool record, float* m32 = nullptr) {
  LagState* s = lag_of(c);
  { MIBM_PROF(c, "scatter_apply");
    scatter_apply_kernel<<<(unsigned)std::min<size_t>(kScatterBlocks, div_up(s->plan_n, 256)), 256, 0, c->stream>>>(
        s->plan_n, c->maxnf, c->g.cells, s->res_key, s->res_src, c->tri_coef, scatter_out(c, into_fields, m32), lo, hi,
        s->heads, s->nheads, record ? s->segval : nullptr); }
  ++c->launches;
}

// ---------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------
void lagr_find_centroid_indices(Ctx* c) {
  if (c->maxnf == 0) return;
  { MIBM_PROF(c, "centroid_idx");
    centroid_idx_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(
        lag_args(c), M<double>(c, MIBM_M_TRI_BAR), M<int>(c, MIBM_M_GHOST_FACE), M<int>(c, MIBM_M_PIND)); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "findCentroidIndices");
}

static void mls_weight_launch(Ctx* c) {
  if (c->precision == 1) {
    { MIBM_PROF(c, "mls_weight_sep");
      mls_weight_sep_kernel<<<div_up(4 * (size_t)c->maxnf, 128), 128, 0, c->stream>>>(
          lag_args(c), M<double>(c, MIBM_M_TRI_BAR), M<int>(c, MIBM_M_GHOST_FACE), M<int>(c, MIBM_M_PIND),
          M<double>(c, MIBM_M_PTXAB_Q1), M<double>(c, MIBM_M_PTXAB_Q2), M<double>(c, MIBM_M_PTXAB_Q3),
          M<double>(c, MIBM_M_PTXAB_TEMP), c->dflag); }
    ++c->launches;
    return;
  }
  { MIBM_PROF(c, "mls_weight");
    mls_weight_kernel<<<div_up(4 * (size_t)c->maxnf, 64), 64, 0, c->stream>>>(
        lag_args(c), M<double>(c, MIBM_M_TRI_BAR), M<int>(c, MIBM_M_GHOST_FACE), M<int>(c, MIBM_M_PIND),
        M<double>(c, MIBM_M_PTXAB_Q1), M<double>(c, MIBM_M_PTXAB_Q2), M<double>(c, MIBM_M_PTXAB_Q3),
        M<double>(c, MIBM_M_PTXAB_TEMP), c->dflag); }
  ++c->launches;
}

void lagr_mls_weight(Ctx* c) {
  if (c->maxnf == 0) return;
  mls_weight_launch(c);
  if (MIBM_LAUNCH_CHECK(c, "mlsWeight")) check_flag(c, "mlsWeight");
}

// mlsforce_ drop-in: spreads into the dense for_* fields
void lagr_mls_force(Ctx* c, const StepParams*, bool) {
  if (c->maxnf == 0) return;
  if (!ensure_lag_buffers(c)) return;
  force_coefficients(c);
  update_plan(c, nullptr);
  scatter(c, false, 0, 4, false);
  MIBM_LAUNCH_CHECK(c, "mlsForce");
}

void lagr_velforce(Ctx* c) {
  if (!ensure_lag_buffers(c)) return;
  LagState* s = lag_of(c);
  dim3 grid(c->g.n2m, c->g.n3m);
  { MIBM_PROF(c, "field_sum");
    field_sum_kernel<<<grid, 128, 0, c->stream>>>(c->g, c->df[MIBM_F_FORXC], c->df[MIBM_F_FORYC],
                                                  c->df[MIBM_F_FORZC], c->red + kRedPart); }
  double ncell = (double)c->g.n1m * (double)c->g.n2m * (double)c->g.n3m;
  { MIBM_PROF(c, "mean3");
    mean3_kernel<<<1, 1024, 0, c->stream>>>(c->red + kRedPart, c->g.n2m * c->g.n3m, ncell, s->mean3); }
  c->launches += 2;
  k_velforce_apply(c, s->mean3);
}

void lagr_tempforce(Ctx* c) { k_tempforce_apply(c); }

void lagr_find_probe_indices(Ctx* c) {
  if (c->maxnf == 0) return;
  { MIBM_PROF(c, "probe_idx");
    probe_idx_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(
        lag_args(c), M<double>(c, MIBM_M_TRI_BAR), M<double>(c, MIBM_M_TRI_NOR), M<int>(c, MIBM_M_GHOST_FACE),
        c->S(MIBM_S_H_EULERIAN), M<int>(c, MIBM_M_PIND)); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "findProbeIndices");
}

// Which MLS construction evaluates gradients and values at the probes.  The
// reference's (absolute coordinates, condition numbers 1e7-1e8) returns the
// oracle's bits only when its inputs are the oracle's bits: the plain form
// uses it for a body that does not move (fixed, melting or not: the
// geometry follows the Stefan update, which is bit-exact) and for the
// drop-in calls.  Once a body moves, its position carries the fluid solver's
// round-off from the first step on, and the reference's construction turns
// any last-bit difference of the geometry into ~1e-9 noise (its conditioning
// times the rounding unit); there, and in the precision form, the separable
// construction is used, which has none of that noise and agrees with the
// reference's to it, at a quarter of its FP64 operations.
static bool literal_mls(Ctx* c) { return c->precision == 0 && c->I(MIBM_I_IMLSSTR) != 1; }

static void heat_flux_launch(Ctx* c) {
  LagState* s = lag_of(c);
  { MIBM_PROF(c, "heat_flux");
    if (literal_mls(c))
      heat_flux_lit_kernel<<<div_up(2 * (size_t)c->maxnf, kHfProbes), 4 * kHfProbes, 0, c->stream>>>(
          lag_args(c), c->df[MIBM_F_TEMP], M<double>(c, MIBM_M_TRI_BAR), M<double>(c, MIBM_M_TRI_NOR),
          M<int>(c, MIBM_M_GHOST_FACE), M<int>(c, MIBM_M_PIND), c->S(MIBM_S_H_EULERIAN), c->S(MIBM_S_PEC),
          M<double>(c, MIBM_M_QW_O), M<double>(c, MIBM_M_QW_I), c->dflag);
    else
      heat_flux_sep_kernel<<<div_up(2 * (size_t)c->maxnf, 128), 128, 0, c->stream>>>(
          lag_args(c), c->df[MIBM_F_TEMP], M<double>(c, MIBM_M_TRI_BAR), M<double>(c, MIBM_M_TRI_NOR),
          M<int>(c, MIBM_M_GHOST_FACE), M<int>(c, MIBM_M_PIND), c->S(MIBM_S_H_EULERIAN), c->S(MIBM_S_PEC),
          M<double>(c, MIBM_M_QW_O), M<double>(c, MIBM_M_QW_I), c->dflag); }
  { MIBM_PROF(c, "face_to_vert");
    face_to_vert_kernel<<<div_up(c->maxnv, 128), 128, 0, c->stream>>>(
        c->maxnv, s->adj_off, s->adj_face, M<double>(c, MIBM_M_SUR), M<double>(c, MIBM_M_AVERT),
        M<double>(c, MIBM_M_QW_O), M<double>(c, MIBM_M_QW_I), M<double>(c, MIBM_M_QW_OVERT),
        M<double>(c, MIBM_M_QW_IVERT)); }
  c->launches += 2;
}

void lagr_heat_flux(Ctx* c) {
  if (c->maxnf == 0) return;
  if (!ensure_adjacency(c)) return;
  heat_flux_launch(c);
  if (MIBM_LAUNCH_CHECK(c, "mls_heatFlux")) check_flag(c, "mls_heatFlux");
}

void lagr_stefan(Ctx* c, const StepParams* dp) {
  if (c->maxnv == 0) return;
  { MIBM_PROF(c, "stefan");
    stefan_kernel<<<div_up(c->maxnv, 128), 128, 0, c->stream>>>(
        c->maxnv, M<int>(c, MIBM_M_GHOST_VERT), M<double>(c, MIBM_M_VERT_NOR), M<double>(c, MIBM_M_QW_OVERT),
        M<double>(c, MIBM_M_QW_IVERT), c->S(MIBM_S_CPLIQUID) / c->S(MIBM_S_LATHEAT), dp, M<double>(c, MIBM_M_VMELT),
        M<double>(c, MIBM_M_VMELT_M1), M<double>(c, MIBM_M_XYZV)); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "stefan");
  lag_of(c)->weights_valid = false;
}

// Geometry refresh (particle.f90:165-193): kernels only; the scalars stay
// in the device buffer until geometry_to_host.  body_only: the pass before
// the Newton-Euler update (particle.f90:108-117: centroids, normals,
// volume, centre of mass and inertia tensor of the melted body); it also
// rewrites `sur`, which nothing reads before the full refresh recomputes it.
// kGeomFaces: the per-face pass alone (areas, normals, centroids and the
// block sums); kGeomRest: what follows it (vertex areas and normals, the
// body's sums, edge lengths, skewness, cfac)
enum GeomPart { kGeomAll, kGeomFaces, kGeomRest };

static void geometry_launch(Ctx* c, bool imelt, bool body_only = false, GeomPart part = kGeomAll) {
  LagState* s = lag_of(c);
  if (part != kGeomRest) {
    { MIBM_PROF(c, "face_geom");
      face_geom_kernel<<<div_up(c->maxnf, kGeomBlock), kGeomBlock, 0, c->stream>>>(
          c->maxnf, M<int>(c, MIBM_M_VERT_OF_FACE), M<int>(c, MIBM_M_GHOST_FACE), M<double>(c, MIBM_M_XYZV),
          M<double>(c, MIBM_M_SUR), M<double>(c, MIBM_M_TRI_NOR), M<double>(c, MIBM_M_TRI_BAR), s->face_part,
          s->geom_ticket, c->S(MIBM_S_DENS_RATIO), s->geom_out); }
    ++c->launches;
  }
  if (body_only || part == kGeomFaces) return;
  { MIBM_PROF(c, "vert_geom");
    vert_geom_kernel<<<div_up(c->maxnv, 128), 128, 0, c->stream>>>(
        c->maxnv, s->adj_off, s->adj_face, M<int>(c, MIBM_M_GHOST_VERT), M<double>(c, MIBM_M_SUR),
        M<double>(c, MIBM_M_TRI_NOR), M<double>(c, MIBM_M_AVERT), M<double>(c, MIBM_M_VERT_NOR)); }
  c->launches += 1;
  if (c->maxne > 0) {           // calculate_eLengths, calculate_skewness (particle.f90:173-176)
    MIBM_PROF(c, "edges");
    elength_kernel<<<div_up(c->maxne, 128), 128, 0, c->stream>>>(
        c->maxne, M<int>(c, MIBM_M_VERT_OF_EDGE), M<int>(c, MIBM_M_GHOST_EDGE), M<double>(c, MIBM_M_XYZV), 0.0,
        M<double>(c, MIBM_M_ELENGTHS), nullptr);
    skewness_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(
        c->maxnf, M<int>(c, MIBM_M_EDGE_OF_FACE), M<int>(c, MIBM_M_GHOST_FACE), M<double>(c, MIBM_M_ELENGTHS),
        M<double>(c, MIBM_M_SUR), M<double>(c, MIBM_M_SKEWNESS));
    c->launches += 2;
  }
  if (imelt) {
    { MIBM_PROF(c, "cfac");
      cfac_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(c->maxnf, M<double>(c, MIBM_M_SUR),
                                                                c->S(MIBM_S_H_EULERIAN), c->S(MIBM_S_CELVOL),
                                                                M<double>(c, MIBM_M_CFAC)); }
    ++c->launches;
  }
}

// Surface, Volume and centre of mass to the registered host scalars
// (calc_rigidBody_params writes Volume last, RigidAuxRoutines.f90:738).
void lagr_geometry_to_host(Ctx* c) {
  if (c->maxnf == 0) return;
  LagState* s = lag_of(c);
  if (!s->geom_out) return;
  cudaMemcpyAsync(c->red_host, s->geom_out, sizeof(double) * 15, cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "geometry")) return;
  *c->hs[MIBM_S_SURFACE] = c->red_host[0];
  *c->hs[MIBM_S_VOLUME] = c->red_host[2];
  for (int d = 0; d < 3; ++d) c->hs[MIBM_S_POS_CM][d] = c->red_host[3 + d];
  for (int q = 0; q < 9; ++q) c->hs[MIBM_S_INERT_TENSOR][q] = c->red_host[6 + q];
}

// literal: the reference's MLS construction (the drop-in mls_structloads_
// of the plain form); the fused step of a moving body uses the separable one
// (see literal_mls).
static void struct_loads_launch(Ctx* c, const StepParams* dp, bool literal) {
  LagState* s = lag_of(c);
  const int nb = (int)div_up(std::max(1, c->maxnf), kLoadFaces);   // groups of 32 faces
  if (!s->loads_ev) {
    if (!cuda_ok(c, cudaMalloc(&s->loads_ev, sizeof(double) * (13 * kLoadFaces + 12) * (size_t)nb), "structLoads") ||
        !cuda_ok(c, cudaMalloc(&s->loads_ticket, sizeof(unsigned) * (size_t)(nb + 1)), "structLoads"))
      return;
    cudaMemsetAsync(s->loads_ticket, 0, sizeof(unsigned) * (size_t)(nb + 1), c->stream);
  }
  double h = c->S(MIBM_S_H_EULERIAN);
  { MIBM_PROF(c, "loads_face");
    auto kern = literal ? loads_face_kernel<true> : loads_face_kernel<false>;
    kern<<<5 * nb, kLoadFaces, 0, c->stream>>>(
        lag_args(c), c->df[MIBM_F_PR], c->df[MIBM_F_VX], c->df[MIBM_F_VY], c->df[MIBM_F_VZ],
        M<double>(c, MIBM_M_TRI_BAR), M<double>(c, MIBM_M_TRI_NOR), M<double>(c, MIBM_M_SUR),
        M<int>(c, MIBM_M_GHOST_FACE), dp, h, c->S(MIBM_S_REN), s->loads_ev, c->dflag, s->loads_ticket,
        c->drigid); }
  c->launches += 1;
}

// mls_structLoads on the device state; the loads stay in c->drigid.
void lagr_struct_loads(Ctx* c, const StepParams* dp) {
  if (c->maxnf == 0) return;
  if (!ensure_lag_buffers(c) || !rigid_ensure(c)) return;
  struct_loads_launch(c, dp, c->precision == 0);
  if (MIBM_LAUNCH_CHECK(c, "mls_structLoads")) check_flag(c, "mls_structLoads");
}

// particle.f90:108-129: geometry of the melted body, then update_part_pos
// (newton_euler, update_xyz) on the device.
static void motion_launch(Ctx* c, const StepParams* dp) {
  LagState* s = lag_of(c);
  geometry_launch(c, false, true);
  k_newton_euler(c, dp, s->geom_out);
  k_update_xyz(c, false);
}

void lagr_geometry_refresh(Ctx* c, bool imelt) {
  if (c->maxnf == 0) return;
  if (!ensure_adjacency(c) || !ensure_lag_buffers(c)) return;
  geometry_launch(c, imelt);
  lagr_geometry_to_host(c);
}

// the narrow band keeps its minimum distances as integer bit patterns in the
// signed-distance field's own memory (non-negative doubles order as their
// bits) and leaves the signed distances there: no copy pass
static unsigned long long* sdf_bits_of(Ctx* c) { return reinterpret_cast<unsigned long long*>(c->df[MIBM_F_SDF]); }

void lagr_tag_narrow_band(Ctx* c) {
  if (c->maxnf == 0) return;
  LagState* s = lag_of(c);
  if (!s->winner && !cuda_ok(c, cudaMalloc(&s->winner, sizeof(int) * c->g.cells), "band")) return;
  unsigned long long* const sdf_bits = sdf_bits_of(c);
  TagArgs T;
  T.L = lag_args(c);
  if (!s->dist_buf) {
    bool ok = cuda_ok(c, cudaMalloc(&s->dist_buf, sizeof(double) * 125 * (size_t)c->maxnf), "band") &&
              cuda_ok(c, cudaMalloc(&s->band_ub, sizeof(unsigned) * c->g.cells), "band") &&
              cuda_ok(c, cudaMalloc(&s->band_list, sizeof(int) * 125 * (size_t)c->maxnf), "band") &&
              cuda_ok(c, cudaMalloc(&s->band_count, sizeof(int)), "band") &&
              cuda_ok(c, cudaMalloc(&s->face4, sizeof(float4) * (size_t)c->maxnf), "band") &&
              cuda_ok(c, cudaMalloc(&s->face_cell, sizeof(int4) * (size_t)c->maxnf), "band") &&
              cuda_ok(c, cudaMalloc(&s->cm32, sizeof(float) * 3 * (size_t)T.L.clen), "band");
    if (!ok) return;
    cm32_kernel<<<div_up(T.L.clen, 256), 256, 0, c->stream>>>(T.L, s->cm32);
    ++c->launches;
  }
  T.x = M<double>(c, MIBM_M_XYZV); T.vof = M<int>(c, MIBM_M_VERT_OF_FACE); T.ghost = M<int>(c, MIBM_M_GHOST_FACE);
  T.bar = M<double>(c, MIBM_M_TRI_BAR); T.nor = M<double>(c, MIBM_M_TRI_NOR);
  { MIBM_PROF(c, "sdf_reset");
    sdf_reset_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g, sdf_bits, s->winner, s->band_ub); }
  size_t nthr = (size_t)c->maxnf * 125;
  { MIBM_PROF(c, "band_bound");
    band_prep_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(T, s->face4, s->face_cell);
    band_ub_kernel<<<div_up(nthr, 128), 128, 0, c->stream>>>(T, s->face4, s->face_cell, s->cm32, s->band_ub);
    cudaMemsetAsync(s->band_count, 0, sizeof(int), c->stream);
    band_select_kernel<<<div_up(nthr, 128), 128, 0, c->stream>>>(T, s->face4, s->face_cell, s->cm32, s->band_ub,
                                                                  s->dist_buf, s->band_list, s->band_count); }
  for (int pass = 0; pass < 3; ++pass) {
    MIBM_PROF(c, "band");
    band_kernel<<<div_up(nthr, 128), 128, 0, c->stream>>>(T, pass, sdf_bits, s->winner, c->df[MIBM_F_VOFP],
                                                           s->dist_buf, s->face_cell, s->band_list, s->band_count);
  }
  c->launches += 7;
  k_interp_vof(c);
  MIBM_LAUNCH_CHECK(c, "narrowBandTagging");
}

void lagr_tag_initial(Ctx* c) {
  if (c->maxnf == 0) return;
  // bounding box (tagCells.f90:32-66, dx1 on all axes as in the reference)
  std::vector<double> x(3 * (size_t)c->maxnv);
  std::vector<int> gv(c->maxnv);
  cudaMemcpy(x.data(), c->dm[MIBM_M_XYZV], x.size() * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(gv.data(), c->dm[MIBM_M_GHOST_VERT], gv.size() * 4, cudaMemcpyDeviceToHost);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int v = 0; v < c->maxnv; ++v) {
    if (gv[v]) continue;
    for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], x[3 * v + d]); hi[d] = std::max(hi[d], x[3 * v + d]); }
  }
  int b0[3], nb[3];
  for (int d = 0; d < 3; ++d) {
    b0[d] = (int)std::floor(lo[d] * c->g.dx1) + 1 - 2;
    int b1 = (int)std::floor(hi[d] * c->g.dx1) + 1 + 2;
    nb[d] = b1 - b0[d] + 1;
  }
  int vids[4] = {MIBM_F_VOFP, MIBM_F_VOFX, MIBM_F_VOFY, MIBM_F_VOFZ};
  for (int q = 0; q < 4; ++q) {
    fill_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g, c->df[vids[q]], 1.0);
    ++c->launches;
  }
  TagArgs T;
  T.L = lag_args(c);
  T.x = M<double>(c, MIBM_M_XYZV); T.vof = M<int>(c, MIBM_M_VERT_OF_FACE); T.ghost = M<int>(c, MIBM_M_GHOST_FACE);
  T.bar = M<double>(c, MIBM_M_TRI_BAR); T.nor = M<double>(c, MIBM_M_TRI_NOR);
  size_t ncell = (size_t)nb[0] * nb[1] * nb[2];
  LagState* s = lag_of(c);
  if (!s->winner && !cuda_ok(c, cudaMalloc(&s->winner, sizeof(int) * c->g.cells), "band")) return;
  double* tmp = nullptr;
  if (!cuda_ok(c, cudaMalloc(&tmp, sizeof(double) * std::max<size_t>(1, ncell)), "initial tag")) return;
  sdf_reset_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g, sdf_bits_of(c), s->winner, nullptr);
  initial_tag_kernel<<<div_up(ncell, 128), 128, 0, c->stream>>>(T, b0[0], b0[1], b0[2], nb[0], nb[1], nb[2], tmp);
  for (int pass = 0; pass < 2; ++pass)
    initial_claim_kernel<<<div_up(ncell, 256), 256, 0, c->stream>>>(c->g, b0[0], b0[1], b0[2], nb[0], nb[1], nb[2], tmp,
                                                                    s->winner, c->df[MIBM_F_VOFP], pass);
  c->launches += 4;
  bool ok = MIBM_LAUNCH_CHECK(c, "initial tag");
  cudaStreamSynchronize(c->stream);
  cudaFree(tmp);
  if (!ok) return;
  lagr_tag_narrow_band(c);
}

bool lagr_remesh_active(Ctx* c) {
  return c->I(MIBM_I_IREMESH) == 1 && c->I(MIBM_I_IMLSFOR) == 1 && c->maxnf > 0 && c->maxne > 0;
}

// particle.f90:119-160: the trigger (calculate_eLengths of the moved mesh)
// read on the host, and when it fires the hand-off to the host's remesher.
// Returns true if the mesh was remeshed.  Synchronises the stream.
static bool remesh_check(Ctx* c) {
  LagState* s = lag_of(c);
  if (!s->rm_flag && !cuda_ok(c, cudaMalloc(&s->rm_flag, sizeof(int)), "remesh")) return false;
  cudaMemsetAsync(s->rm_flag, 0, sizeof(int), c->stream);
  { MIBM_PROF(c, "edges");
    elength_kernel<<<div_up(c->maxne, 128), 128, 0, c->stream>>>(
        c->maxne, M<int>(c, MIBM_M_VERT_OF_EDGE), M<int>(c, MIBM_M_GHOST_EDGE), M<double>(c, MIBM_M_XYZV),
        c->S(MIBM_S_E_THRESH), M<double>(c, MIBM_M_ELENGTHS), s->rm_flag); }
  ++c->launches;
  cudaMemcpyAsync(c->hflag + 1, s->rm_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "remesh trigger")) return false;
  if (!c->hflag[1]) return false;
  if (!c->remesh_fn) {
    fail(c, MIBM_ESTATE, "remeshing triggered (an edge is shorter than E_thresh) but no remesher is set "
                         "(mibm_set_remesh_callback_)");
    return false;
  }
  // update_tri_normal of the moved mesh and its volume, then every mesh
  // array to the host
  geometry_launch(c, false, true);
  cudaMemcpyAsync(c->red_host, s->geom_out, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->stream);
  for (int i = 0; i < MIBM_NMESH; ++i)
    cudaMemcpyAsync(c->hm[i], c->dm[i], mesh_bytes(c, i), cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "remesh download")) return false;
  *c->hs[MIBM_S_VOLUME] = c->red_host[1];          // calculate_volume
  int st = c->remesh_fn(c->remesh_user);
  if (st != 0) {
    fail(c, MIBM_EABORT, "remesher returned " + std::to_string(st));
    return false;
  }
  for (int i = 0; i < MIBM_NMESH; ++i)
    cudaMemcpyAsync(c->dm[i], c->hm[i], mesh_bytes(c, i), cudaMemcpyHostToDevice, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "remesh upload")) return false;
  lagr_topology_changed(c);
  ++c->remesh_count;
  return ensure_adjacency(c);
}

static void tri_velocity_launch(Ctx* c, const double* vel, const double* om) {
  MIBM_PROF(c, "tri_velocity");
  tri_velocity_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(
      c->maxnf, M<int>(c, MIBM_M_GHOST_FACE), M<double>(c, MIBM_M_TRI_BAR), lag_of(c)->geom_out, vel, om,
      M<double>(c, MIBM_M_VEL_TRI));
  ++c->launches;
}

// device addresses of vel_CM and omega_c for update_tri_velocity: the moving
// body's state, else the values the substep was given
static void body_velocity(Ctx* c, const StepParams* dp, const double** vel, const double** om) {
  if (c->I(MIBM_I_IMLSSTR) == 1 && c->drigid) {
    *vel = (const double*)((const char*)c->drigid + offsetof(RigidDev, vel));
    *om = (const double*)((const char*)c->drigid + offsetof(RigidDev, om));
  } else {
    *vel = (const double*)((const char*)dp + offsetof(StepParams, vel));
    *om = (const double*)((const char*)dp + offsetof(StepParams, om));
  }
}

// particle.f90:38-193 (drop-in particle_): dense force fields, host checks
void lagr_particle(Ctx* c, const StepParams* dp) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return;
  lagr_find_centroid_indices(c);
  lagr_mls_weight(c);
  if (c->status != MIBM_OK) return;
  static const int fo[4] = {MIBM_F_FORXC, MIBM_F_FORYC, MIBM_F_FORZC, MIBM_F_FORTEMP};
  for (int q = 0; q < 4; ++q) cudaMemsetAsync(c->df[fo[q]], 0, c->g.cells * sizeof(double), c->stream);
  lagr_mls_force(c, dp, true);
  bool imelt = c->I(MIBM_I_IMELT) == 1;
  if (imelt) {
    lagr_find_probe_indices(c);
    lagr_heat_flux(c);
    if (c->status != MIBM_OK) return;
  }
  bool str = c->I(MIBM_I_IMLSSTR) == 1;
  if (str) {
    if (!ensure_lag_buffers(c) || !rigid_ensure(c)) return;
    rigid_pack(c, c->hrigid_in, false);
    rigid_upload(c);
    lagr_struct_loads(c, dp);
    if (c->status != MIBM_OK) return;
  }
  lagr_velforce(c);
  lagr_tempforce(c);
  if (imelt) lagr_stefan(c, dp);
  if (!ensure_adjacency(c) || !ensure_lag_buffers(c)) return;
  if (str) motion_launch(c, dp);
  bool remeshed = lagr_remesh_active(c) && remesh_check(c);
  if (c->status != MIBM_OK) return;
  geometry_launch(c, imelt);
  if (remeshed) {
    const double *vel, *om;
    body_velocity(c, dp, &vel, &om);
    tri_velocity_launch(c, vel, om);
  }
  if (str) {
    k_rigid_publish(c, lag_of(c)->geom_out, nullptr);
    rigid_download(c);
  }
  lagr_geometry_to_host(c);
  if (str) {
    if (!check_flag(c, "update_part_pos")) return;
    rigid_unpack(c, c->hrigid_out, false);
  }
  if (c->S(MIBM_S_VOLUME) < c->S(MIBM_S_V_THRESH)) fail(c, MIBM_EABORT, "Geometry V/VE smaller than threshold");
}

// particle.f90:38-193 inside the fused step: no host synchronisation.  The
// forces are added straight into u, v, w (the mean force is left in
// `mean3` for the projection update to subtract) and, after the heat flux
// has read the unforced temperature, into T.  MLS weights of a stationary
// cage are reused.  Flags and geometry scalars are read by the caller at the
// end of the step.
// The work of a substep that depends on the geometry alone: narrow-band
// tagging (tagCells at the start of the substep, tsch.f90:45-47) and, from
// particle, the cage indices, the MLS weights and the scatter plan.  The fused
// step runs it on the side stream of the substep before (the geometry is
// final once that substep's particle is done): for substeps 1 and 2, and for
// substep 0 of the next step (slot 3: no parameter block, the host's plan
// rebuild requests invalidate it instead).
void lagr_substep_prologue(Ctx* c, int slot) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return;
  // the tagging (VOF fields) and the cage indices, weights and plan read the
  // same geometry and write disjoint buffers: the tagging goes to a stream of
  // its own and is joined back before the prologue ends
  const bool split = !c->I(MIBM_I_STATIONARY) && c->side2 && lagr_fork_enabled(c);
  c->geom_join_tag = split;
  if (split) {
    cudaEventRecord(c->ev_tfork, c->stream);
    cudaStreamWaitEvent(c->side2, c->ev_tfork, 0);
    std::swap(c->stream, c->side2);
    lagr_tag_narrow_band(c);
    cudaEventRecord(c->ev_tjoin, c->stream);
    std::swap(c->stream, c->side2);
  } else if (!c->I(MIBM_I_STATIONARY)) {
    lagr_tag_narrow_band(c);
  }
  if (!ensure_adjacency(c) || !ensure_lag_buffers(c)) {
    if (split) cudaStreamWaitEvent(c->stream, c->ev_tjoin, 0);
    return;
  }
  LagState* s = lag_of(c);
  bool stationary = c->I(MIBM_I_STATIONARY) != 0;
  lagr_find_centroid_indices(c);
  // the MLS weights and the scatter plan both read the cage indices and
  // nothing the other writes: the weights go to a third stream
  const bool wsplit = split && c->side3;
  if (wsplit) {
    cudaEventRecord(c->ev_wfork, c->stream);
    cudaStreamWaitEvent(c->side3, c->ev_wfork, 0);
    std::swap(c->stream, c->side3);
  }
  if (!(stationary && s->weights_valid)) {
    mls_weight_launch(c);
    s->weights_valid = stationary;
    if (stationary) ++c->lag_gen;     // later steps skip the weights: another launch sequence
  }
  if (wsplit) {
    cudaEventRecord(c->ev_wjoin, c->stream);
    std::swap(c->stream, c->side3);
  }
  update_plan(c, slot < 3 ? c->dparams + slot : nullptr);
  if (wsplit) cudaStreamWaitEvent(c->stream, c->ev_wjoin, 0);
  if (split) cudaStreamWaitEvent(c->stream, c->ev_tjoin, 0);
}

// The side stream takes the second half of particle (and the work that
// follows it) unless the host's remesher may be needed mid-way or kernels
// are timed one by one (mibm_profile_: serial, so each time is its own).
bool lagr_fork_enabled(Ctx* c) {
  return c->side && !lagr_remesh_active(c) && !c->profiling && c->I(MIBM_I_IMLSFOR) == 1 && c->maxnf > 0;
}

// The structural loads read u, v, w after their line solves, p, and the
// geometry, nothing that the temperature's line solves write: the fused step
// starts them on the side stream once w is solved, so that they run beside
// the temperature solves; the velocity scatter, which changes u, v, w, waits
// for them (lagr_particle_fused).  Same conditions as the particle fork.
void lagr_loads_early(Ctx* c, const StepParams* dp) {
  c->loads_pending = false;
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0 || c->I(MIBM_I_IMLSSTR) != 1) return;
  if (!lagr_fork_enabled(c)) return;
  if (!ensure_adjacency(c) || !ensure_lag_buffers(c)) return;
  cudaEventRecord(c->ev_lfork, c->stream);
  cudaStreamWaitEvent(c->side, c->ev_lfork, 0);
  std::swap(c->stream, c->side);
  struct_loads_launch(c, dp, false);
  cudaEventRecord(c->ev_ldone, c->stream);
  std::swap(c->stream, c->side);
  c->loads_pending = true;
}

const double* lagr_particle_fused(Ctx* c, const StepParams* dp, float* m32, StepParams* next,
                                  int next_prologue) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return nullptr;
  if (!ensure_adjacency(c) || !ensure_lag_buffers(c)) return nullptr;
  LagState* s = lag_of(c);
  lagr_join(c);                   // cage indices, MLS weights, scatter plan of this substep
  force_coefficients(c);
  bool str = c->I(MIBM_I_IMLSSTR) == 1;
  if (str) {                                 // reads the unforced u, v, w and p
    if (c->loads_pending) {
      cudaStreamWaitEvent(c->stream, c->ev_ldone, 0);
      c->loads_pending = false;
    } else {
      struct_loads_launch(c, dp, false);
    }
  }
  scatter(c, true, 0, 3, true);
  double ncell = (double)c->g.n1m * (double)c->g.n2m * (double)c->g.n3m;
  { MIBM_PROF(c, "seg_mean");
    seg_mean_kernel<<<kMeanBlocks, 256, 0, c->stream>>>(s->nheads, s->heads, c->g.cells, s->res_key, s->segval,
                                                        c->red + kRedPart, ncell, s->mean3); }
  c->launches += 1;
  // Fork: the rest of particle (heat flux, temperature forcing, Stefan
  // front, motion, geometry) reads and writes none of the buffers of the
  // pressure projection that the caller enqueues next, so it runs on the
  // side stream; lagr_join makes the main stream wait for it before the next
  // substep.
  const bool fork = lagr_fork_enabled(c);
  if (fork) {
    cudaEventRecord(c->ev_fork, c->stream);
    cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    std::swap(c->stream, c->side);
  }
  bool imelt = c->I(MIBM_I_IMELT) == 1;
  if (imelt) {
    lagr_find_probe_indices(c);
    heat_flux_launch(c);
  }
  scatter(c, true, 3, 4, false, m32);
  if (imelt) lagr_stefan(c, dp);
  if (str) motion_launch(c, dp);
  bool remeshed = !fork && lagr_remesh_active(c) && remesh_check(c);
  if (c->status == MIBM_OK && fork && next_prologue >= 0 && c->side3) {
    // the next substep's geometry-only work needs the new face centroids and
    // normals alone: it starts after the per-face pass, while a third stream
    // finishes the refresh and publishes the moved body (ev_pub)
    geometry_launch(c, imelt, false, kGeomFaces);
    cudaEventRecord(c->ev_gfork, c->stream);
    cudaStreamWaitEvent(c->side3, c->ev_gfork, 0);
    std::swap(c->stream, c->side3);
    geometry_launch(c, imelt, false, kGeomRest);
    if (str) k_rigid_publish(c, s->geom_out, next);
    cudaEventRecord(c->ev_pub, c->stream);
    std::swap(c->stream, c->side3);
    c->geom_join_tag = false;
    lagr_substep_prologue(c, next_prologue);
    c->prologue_done = true;
    cudaStreamWaitEvent(c->stream, c->ev_pub, 0);     // the full join covers the refresh
    MIBM_LAUNCH_CHECK(c, "particle");
  } else if (c->status == MIBM_OK) {
    geometry_launch(c, imelt);
    if (remeshed) {
      const double *vel, *om;
      body_velocity(c, dp, &vel, &om);
      tri_velocity_launch(c, vel, om);
    }
    if (str) k_rigid_publish(c, s->geom_out, next);
    if (fork) cudaEventRecord(c->ev_pub, c->stream);
    c->geom_join_tag = false;
    if (fork && next_prologue >= 0) {
      lagr_substep_prologue(c, next_prologue);
      c->prologue_done = true;
    }
    MIBM_LAUNCH_CHECK(c, "particle");
  }
  if (fork) {
    cudaEventRecord(c->ev_join, c->stream);
    std::swap(c->stream, c->side);
    c->join_pending = true;
    c->geom_join_pending = true;
  }
  return c->status == MIBM_OK ? s->mean3 : nullptr;
}

// the main stream waits for the side-stream half of the last particle
void lagr_join(Ctx* c) {
  if (!c->join_pending) return;
  cudaStreamWaitEvent(c->stream, c->ev_join, 0);
  c->join_pending = false;
  c->geom_join_pending = false;
}

// the main stream waits for what the next substep's explicit terms read
// from the side branch: the moved body (published state, geometry) and,
// when the tagging ran on its own stream, the VOF fields
void lagr_join_geom(Ctx* c) {
  if (!c->geom_join_pending) return;
  cudaStreamWaitEvent(c->stream, c->ev_pub, 0);
  if (c->geom_join_tag) cudaStreamWaitEvent(c->stream, c->ev_tjoin, 0);
  c->geom_join_pending = false;
}

// End of the fused step, in two halves so that the device half can sit in
// a captured step graph: lagr_step_readback enqueues the copies of the MLS
// flag and the geometry scalars into pinned host memory; after the stream
// has completed, lagr_step_host_finish reads them (MLS failure status,
// Surface, Volume, centre of mass, V_thresh abort of particle.f90:218-224).
void lagr_step_readback(Ctx* c) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return;
  LagState* s = lag_of(c);
  cudaMemcpyAsync(c->hflag, c->dflag, 4, cudaMemcpyDeviceToHost, c->stream);
  if (s->geom_out) cudaMemcpyAsync(c->step_host, s->geom_out, sizeof(double) * 15, cudaMemcpyDeviceToHost, c->stream);
  if (c->I(MIBM_I_IMLSSTR) == 1 && c->drigid) rigid_download(c);
}

void lagr_step_host_finish(Ctx* c) {
  if (c->I(MIBM_I_IMLSFOR) != 1 || c->maxnf == 0) return;
  if (c->hflag[0]) {
    fail(c, MIBM_ENUMERIC, (c->hflag[0] & 2) ? "particle: singular inertia tensor (dgetrf info /= 0)"
                                             : "particle: singular MLS moment matrix (dgetrf info /= 0)");
    c->hflag[0] = 0;
    cudaMemsetAsync(c->dflag, 0, 4, c->stream);
    return;
  }
  if (!lag_of(c)->geom_out) return;
  if (c->I(MIBM_I_IMLSSTR) == 1 && c->drigid) rigid_unpack(c, c->hrigid_out, false);
  *c->hs[MIBM_S_SURFACE] = c->step_host[0];
  *c->hs[MIBM_S_VOLUME] = c->step_host[2];
  for (int d = 0; d < 3; ++d) c->hs[MIBM_S_POS_CM][d] = c->step_host[3 + d];
  for (int q = 0; q < 9; ++q) c->hs[MIBM_S_INERT_TENSOR][q] = c->step_host[6 + q];
  if (c->S(MIBM_S_VOLUME) < c->S(MIBM_S_V_THRESH)) fail(c, MIBM_EABORT, "Geometry V/VE smaller than threshold");
}

void lagr_free(Ctx* c) {
  for (size_t q = 0; q < g_lag.size(); ++q)
    if (g_lag[q]->c == c) {
      LagState* s = g_lag[q];
      cudaFree(s->adj_off); cudaFree(s->adj_face); cudaFree(s->face_part); cudaFree(s->geom_out); cudaFree(s->geom_ticket);
      cudaFree(s->loads_ev); cudaFree(s->loads_ticket); cudaFree(s->rm_flag);
      cudaFree(s->mean3); cudaFree(s->winner); cudaFree(s->dist_buf);
      cudaFree(s->band_ub); cudaFree(s->face4); cudaFree(s->face_cell); cudaFree(s->cm32);
      cudaFree(s->band_list); cudaFree(s->band_count);
      cudaFree(s->key); cudaFree(s->src); cudaFree(s->tmp_key); cudaFree(s->tmp_src); cudaFree(s->hist);
      cudaFree(s->tsum);
      cudaFree(s->saved); cudaFree(s->dirty); cudaFree(s->segval);
      cudaFree(s->hidx); cudaFree(s->heads); cudaFree(s->nheads); cudaFree(s->htsum);
      delete s;
      g_lag.erase(g_lag.begin() + q);
      break;
    }
}

}  // namespace mibm
