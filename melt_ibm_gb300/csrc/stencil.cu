// stencil.cu -- staggered second-order stencils of the RK3 substep.
//
// Kernels restate, per cell:
//   hdnl1.f90:15-77, hdnl2.f90:16-78, hdnl3.f90:16-88, hdnlte.f90:45-158
//   invtr1.f90:25-64, invtr2.f90:22-59, invtr3.f90:20-58, invtrte.f90:17-59
//   divg.f90:9-23, updvp.f90:16-31, prcalc.f90:17-33, cfl.f90:1-77,
//   velforce.f90:44-52, tempforce.f90:32-40, interp_vof tagCells.f90:85-111
// on the compact device layout (common.cuh) with periodic index wraps in
// place of the Fortran ghost planes.  One thread per cell, x fastest; the
// grid covers (x/32, y/8, z).  The FP64 form of these kernels is bounded by
// the FP64 FMA rate of the part, not by HBM, so the code avoids divisions
// (reciprocals are taken once on the host) and skips terms that are zero by
// configuration (HIT forcing off).
#include <algorithm>

#include "common.cuh"
#include "fpconv.cuh"

namespace mibm {

typedef int idx_t;

struct StencilArgs {
  Grid g;
  const double* __restrict__ vx;
  const double* __restrict__ vy;
  const double* __restrict__ vz;
  const double* __restrict__ temp;
  const double* __restrict__ pr;
  const double* __restrict__ vofx;
  const double* __restrict__ vofy;
  const double* __restrict__ vofz;
  const double* __restrict__ vofp;
  const double* __restrict__ forcx;
  const double* __restrict__ forcy;
  const double* __restrict__ forcz;
  const double* __restrict__ xc;   // coordinate tables, offset coord_off
  const double* __restrict__ xm;
  const double* __restrict__ yc;
  const double* __restrict__ ym;
  const double* __restrict__ zc;
  const double* __restrict__ zm;
  const float* __restrict__ u32;   // FP32 mirrors (precision form only)
  const float* __restrict__ v32;
  const float* __restrict__ w32;
  const float* __restrict__ t32;
  const float* __restrict__ p32;
  // advection products of the fused step (6 fields, adv_products_kernel) in
  // the FP64 form and in the precision form
  const double* __restrict__ prod;
  const float* __restrict__ prod32;
  int coff;
  int forcing;
};

// the five prognostic fields as read by the stencils of compute type R: the
// FP64 fields themselves, or their FP32 mirrors in the precision form
template <typename R>
struct Prog {
  const R* u; const R* v; const R* w; const R* t; const R* p; const R* pd;
};
template <typename R> __device__ __forceinline__ Prog<R> prog(const StencilArgs& A);
template <> __device__ __forceinline__ Prog<double> prog<double>(const StencilArgs& A) {
  return Prog<double>{A.vx, A.vy, A.vz, A.temp, A.pr, A.prod};
}
template <> __device__ __forceinline__ Prog<float> prog<float>(const StencilArgs& A) {
  return Prog<float>{A.u32, A.v32, A.w32, A.t32, A.p32, A.prod32};
}

static StencilArgs make_args(Ctx* c) {
  StencilArgs a;
  a.g = c->g;
  a.vx = c->df[MIBM_F_VX]; a.vy = c->df[MIBM_F_VY]; a.vz = c->df[MIBM_F_VZ];
  a.temp = c->df[MIBM_F_TEMP]; a.pr = c->df[MIBM_F_PR];
  a.vofx = c->df[MIBM_F_VOFX]; a.vofy = c->df[MIBM_F_VOFY]; a.vofz = c->df[MIBM_F_VOFZ]; a.vofp = c->df[MIBM_F_VOFP];
  a.forcx = c->df[MIBM_F_FORCX]; a.forcy = c->df[MIBM_F_FORCY]; a.forcz = c->df[MIBM_F_FORCZ];
  a.xc = c->xc; a.xm = c->xm; a.yc = c->yc; a.ym = c->ym; a.zc = c->zc; a.zm = c->zm;
  const float* m = c->q32;
  size_t n = c->g.cells;
  a.u32 = m; a.v32 = m ? m + n : nullptr; a.w32 = m ? m + 2 * n : nullptr;
  a.t32 = m ? m + 3 * n : nullptr; a.p32 = m ? m + 4 * n : nullptr;
  a.prod = c->prod; a.prod32 = c->prod32;
  a.coff = c->coord_off;
  a.forcing = c->I(MIBM_I_FORCING);
  return a;
}

// NaN or +-Inf, and the max of two non-negative values, on the bit patterns:
// integer operations instead of FP64 ones (which issue at the FP64 rate)
__device__ __forceinline__ bool bits_nonfinite(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
}
__device__ __forceinline__ bool bits_nonfinite(float x) { return ((__float_as_int(x) >> 23) & 0xff) == 0xff; }
__device__ __forceinline__ double max_nonneg(double a, double b) {
  return __longlong_as_double(max(__double_as_longlong(a), __double_as_longlong(b)));
}
__device__ __forceinline__ float max_nonneg(float a, float b) {
  return __int_as_float(max(__float_as_int(a), __float_as_int(b)));
}

// VOF == 1 (a fully fluid cell) tested on the bit pattern: an integer
// compare instead of an FP64 one (FP64 compares issue at the FP64 rate).
__device__ __forceinline__ bool vof_is_one(double v) {
  return __double_as_longlong(v) == 0x3FF0000000000000LL;
}

// The forcing term VOF*forc/len of hdnl1/2/3 (hdnl1.f90:74) added to h, as
// (VOF*forc)*(1/len) with 1/len formed once on the host: a multiply instead
// of an FP64 division (a long sequence of FP64 operations), the value within
// one rounding of the quotient.  In a fluid cell (VOF = 1) it is one FMA, and
// the precision form converts a single FP64 value there.
template <typename R>
__device__ __forceinline__ R add_forcing(R h, const double* __restrict__ vof, const double* __restrict__ forc,
                                         idx_t c0, R rlen) {
  const double v = vof[c0];
  if constexpr (sizeof(R) == 8) {
    if (vof_is_one(v)) return forc[c0] * rlen + h;
    return (v * forc[c0]) * rlen + h;
  } else {
    if (vof_is_one(v)) return d2f_bits(forc[c0]) * rlen + h;
    return d2f_bits(v * forc[c0]) * rlen + h;
  }
}

// Cell index and the six periodic neighbour offsets in 32-bit arithmetic
// (the largest supported grid, 512^3 with pitch 512, has < 2^31 cells).
#define CELL_INDEX                                                   \
  const Grid& g = A.g;                                               \
  int i = blockIdx.x * blockDim.x + threadIdx.x;                     \
  int j = blockIdx.y * blockDim.y + threadIdx.y;                     \
  int k = blockIdx.z;                                                \
  if (i >= g.n1m || j >= g.n2m) return;                              \
  const int P = g.P;                                                 \
  const int PL = (int)g.plane;                                       \
  const idx_t c0 = i + P * (j + g.n2m * k);                          \
  const idx_t dip = (i + 1 == g.n1m) ? 1 - g.n1m : 1;                \
  const idx_t dim = (i == 0) ? g.n1m - 1 : -1;                       \
  const idx_t djp = (j + 1 == g.n2m) ? -(g.n2m - 1) * P : P;         \
  const idx_t djm = (j == 0) ? (g.n2m - 1) * P : -P;                 \
  const idx_t dkp = (k + 1 == g.n3m) ? -(g.n3m - 1) * PL : PL;       \
  const idx_t dkm = (k == 0) ? (g.n3m - 1) * PL : -PL;               \
  if (!(MIBM_IDX_OK(k, g.n3m) & MIBM_IDX_OK(c0 + dip, g.cells) &     \
        MIBM_IDX_OK(c0 + dim, g.cells) & MIBM_IDX_OK(c0 + djp, g.cells) & \
        MIBM_IDX_OK(c0 + djm, g.cells) & MIBM_IDX_OK(c0 + dkp, g.cells) & \
        MIBM_IDX_OK(c0 + dkm, g.cells)))                              \
    return;                                                          \
  (void)dip; (void)dim; (void)djp; (void)djm; (void)dkp; (void)dkm; (void)P;

// ---------------------------------------------------------------------
// explicit terms, templated on the compute type R: R = double is the plain
// FP64 form (bit-identical to a double-only build), R = float the precision
// form, which reads the FP32 mirrors of the fields and the FP32 coefficients
// so that no FP64 operation is left in the cell loop (on this part FP64
// arithmetic and FP64<->FP32 conversions share the low FP64 issue rate).
// ---------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R h_x(const StencilArgs& A, idx_t c0, idx_t dip, idx_t dim, idx_t djp,
                                 idx_t djm, idx_t dkp, idx_t dkm, const StepParams& p) {
  const Prog<R> F = prog<R>(A);
  const R* vx = F.u; const R* vy = F.v; const R* vz = F.w;
  R udx1 = coef<R>(p, kQ1), udx2 = coef<R>(p, kQ2), udx3 = coef<R>(p, kQ3);
  R vxc = vx[c0];
  R a = vx[c0 + dip] + vxc, b = vx[c0 + dim] + vxc;
  R x11 = a * a - b * b;
  R x12 = (vy[c0 + djp] + vy[c0 + dim + djp]) * (vx[c0 + djp] + vxc) -
          (vy[c0] + vy[c0 + dim]) * (vxc + vx[c0 + djm]);
  R x13 = (vz[c0 + dkp] + vz[c0 + dim + dkp]) * (vx[c0 + dkp] + vxc) -
          (vz[c0] + vz[c0 + dim]) * (vxc + vx[c0 + dkm]);
  R h = -(udx1 * x11 + udx2 * x12 + udx3 * x13);   // -(h11 + h12 + h13), each h1d = x1d * udx_d
  if (A.forcing) h = add_forcing<R>(h, A.vofx, A.forcx, c0, coef<R>(p, kRXLEN));
  return h;
}

template <typename R>
__device__ __forceinline__ R h_y(const StencilArgs& A, idx_t c0, idx_t dip, idx_t dim, idx_t djp,
                                 idx_t djm, idx_t dkp, idx_t dkm, const StepParams& p) {
  const Prog<R> F = prog<R>(A);
  const R* vx = F.u; const R* vy = F.v; const R* vz = F.w;
  R udx1 = coef<R>(p, kQ1), udx2 = coef<R>(p, kQ2), udx3 = coef<R>(p, kQ3);
  R vyc = vy[c0];
  R x21 = (vy[c0 + dip] + vyc) * (vx[c0 + dip] + vx[c0 + dip + djm]) -
          (vyc + vy[c0 + dim]) * (vx[c0] + vx[c0 + djm]);
  R a = vy[c0 + djp] + vyc, b = vy[c0 + djm] + vyc;
  R x22 = a * a - b * b;
  R x23 = (vz[c0 + dkp] + vz[c0 + djm + dkp]) * (vy[c0 + dkp] + vyc) -
          (vz[c0] + vz[c0 + djm]) * (vyc + vy[c0 + dkm]);
  R h = -(udx1 * x21 + udx2 * x22 + udx3 * x23);
  if (A.forcing) h = add_forcing<R>(h, A.vofy, A.forcy, c0, coef<R>(p, kRYLEN));
  return h;
}

template <typename R>
__device__ __forceinline__ R h_z(const StencilArgs& A, idx_t c0, idx_t dip, idx_t dim, idx_t djp,
                                 idx_t djm, idx_t dkp, idx_t dkm, const StepParams& p) {
  const Prog<R> F = prog<R>(A);
  const R* vx = F.u; const R* vy = F.v; const R* vz = F.w;
  R udx1 = coef<R>(p, kQ1), udx2 = coef<R>(p, kQ2), udx3 = coef<R>(p, kQ3);
  R vzc = vz[c0];
  R x31 = (vx[c0 + dip] + vx[c0 + dip + dkm]) * (vz[c0 + dip] + vzc) -
          (vx[c0] + vx[c0 + dkm]) * (vzc + vz[c0 + dim]);
  R x32 = (vy[c0 + djp] + vy[c0 + djp + dkm]) * (vz[c0 + djp] + vzc) -
          (vy[c0] + vy[c0 + dkm]) * (vzc + vz[c0 + djm]);
  R a = vz[c0 + dkp] + vzc, b = vzc + vz[c0 + dkm];
  R x33 = a * a - b * b;
  R h = -(udx1 * x31 + udx2 * x32 + udx3 * x33);
  if (p.betagz != 0.0) {
    R T_interp = (F.t[c0] + F.t[c0 + dkm]) * R(0.5);
    h = h + coef<R>(p, kBETAGZ) * (T_interp - coef<R>(p, kTLIQ));
  }
  if (A.forcing) h = add_forcing<R>(h, A.vofz, A.forcz, c0, coef<R>(p, kRZLEN));
  return h;
}

// ---------------------------------------------------------------------
// The advection terms of hdnl1-3 are differences of products at cell faces
// and edges that neighbouring cells and the three momentum components share:
//   h11 = Pc - Pc[i-1], h12 = E[j+1] - E, h13 = F[k+1] - F,
//   h21 = E[i+1] - E,   h22 = Qc - Qc[j-1], h23 = H[k+1] - H,
//   h31 = F[i+1] - F,   h32 = H[j+1] - H,   h33 = Rc - Rc[k-1]
// with, at cell (i,j,k),
//   Pc = (u[i+1]+u)^2, Qc = (v[j+1]+v)^2, Rc = (w[k+1]+w)^2,
//   E = (v+v[i-1]) (u+u[j-1]), F = (w+w[i-1]) (u+u[k-1]), H = (w+w[j-1]) (v+v[k-1])
// (hdnl1.f90:40-72, hdnl2.f90:40-73, hdnl3.f90:40-80 regrouped).  The fused
// step forms the six products once per cell (15 FP64 operations) instead of
// inside each component's stencil (39 for the three), the same values up to
// the rounding of the products.
// ---------------------------------------------------------------------
template <typename R>
__global__ void adv_products_kernel(StencilArgs A, R* __restrict__ out) {
  CELL_INDEX
  const Prog<R> F = prog<R>(A);
  const R* u = F.u; const R* v = F.v; const R* w = F.w;
  const size_t n = g.cells;
  const R uc = u[c0], vc = v[c0], wc = w[c0];
  const R a = u[c0 + dip] + uc, b = v[c0 + djp] + vc, d = w[c0 + dkp] + wc;
  out[c0] = a * a;
  out[n + c0] = b * b;
  out[2 * n + c0] = d * d;
  out[3 * n + c0] = (vc + v[c0 + dim]) * (uc + u[c0 + djm]);
  out[4 * n + c0] = (wc + w[c0 + dim]) * (uc + u[c0 + dkm]);
  out[5 * n + c0] = (wc + w[c0 + djm]) * (vc + v[c0 + dkm]);
}

// ISO (FP64, equal grid spacings, udx1 = udx2 = udx3): the three
// differences summed in 64-bit integers on the integer pipe and rounded once
// (sum3_diff_f64), one FP64 operation instead of six, within FP64 round-off
// of the reference's order
template <typename R, bool ISO = false>
__device__ __forceinline__ R h_prod(const StencilArgs& A, int W, idx_t c0, idx_t dip, idx_t dim, idx_t djp,
                                    idx_t djm, idx_t dkp, idx_t dkm, const StepParams& p) {
  const Prog<R> F = prog<R>(A);
  const size_t n = A.g.cells;
  const R* Pc = F.pd; const R* Qc = F.pd + n; const R* Rc = F.pd + 2 * n;
  const R* E = F.pd + 3 * n; const R* Fx = F.pd + 4 * n; const R* H = F.pd + 5 * n;
  const R udx1 = coef<R>(p, kQ1), udx2 = coef<R>(p, kQ2), udx3 = coef<R>(p, kQ3);
  R h;
  if constexpr (ISO && sizeof(R) == 8) {
    if (W == 0) h = -(udx1 * sum3_diff_f64(Pc[c0], Pc[c0 + dim], E[c0 + djp], E[c0], Fx[c0 + dkp], Fx[c0]));
    else if (W == 1) h = -(udx1 * sum3_diff_f64(E[c0 + dip], E[c0], Qc[c0], Qc[c0 + djm], H[c0 + dkp], H[c0]));
    else h = -(udx1 * sum3_diff_f64(Fx[c0 + dip], Fx[c0], H[c0 + djp], H[c0], Rc[c0], Rc[c0 + dkm]));
    if (W == 2 && p.betagz != 0.0) {
      R T_interp = (F.t[c0] + F.t[c0 + dkm]) * R(0.5);
      h = h + coef<R>(p, kBETAGZ) * (T_interp - coef<R>(p, kTLIQ));
    }
    if (A.forcing) {
      if (W == 0) h = add_forcing<R>(h, A.vofx, A.forcx, c0, coef<R>(p, kRXLEN));
      else if (W == 1) h = add_forcing<R>(h, A.vofy, A.forcy, c0, coef<R>(p, kRYLEN));
      else h = add_forcing<R>(h, A.vofz, A.forcz, c0, coef<R>(p, kRZLEN));
    }
    return h;
  }
  if (W == 0) {
    h = -(udx1 * (Pc[c0] - Pc[c0 + dim]) + udx2 * (E[c0 + djp] - E[c0]) + udx3 * (Fx[c0 + dkp] - Fx[c0]));
    if (A.forcing) h = add_forcing<R>(h, A.vofx, A.forcx, c0, coef<R>(p, kRXLEN));
  } else if (W == 1) {
    h = -(udx1 * (E[c0 + dip] - E[c0]) + udx2 * (Qc[c0] - Qc[c0 + djm]) + udx3 * (H[c0 + dkp] - H[c0]));
    if (A.forcing) h = add_forcing<R>(h, A.vofy, A.forcy, c0, coef<R>(p, kRYLEN));
  } else {
    h = -(udx1 * (Fx[c0 + dip] - Fx[c0]) + udx2 * (H[c0 + djp] - H[c0]) + udx3 * (Rc[c0] - Rc[c0 + dkm]));
    if (p.betagz != 0.0) {
      R T_interp = (F.t[c0] + F.t[c0 + dkm]) * R(0.5);
      h = h + coef<R>(p, kBETAGZ) * (T_interp - coef<R>(p, kTLIQ));
    }
    if (A.forcing) h = add_forcing<R>(h, A.vofz, A.forcz, c0, coef<R>(p, kRZLEN));
  }
  return h;
}

__device__ __forceinline__ double nint_d(double x) { return round(x); }   // Fortran NINT semantics

template <typename R>
__device__ __forceinline__ R h_t(const StencilArgs& A, int i, int j, int k, idx_t c0, idx_t dip, idx_t dim,
                                 idx_t djp, idx_t djm, idx_t dkp, idx_t dkm, const StepParams& p) {
  const Grid& g = A.g;
  const Prog<R> F = prog<R>(A);
  const R* vx = F.u; const R* vy = F.v; const R* vz = F.w; const R* T = F.t;
  R udx1 = coef<R>(p, kH1), udx2 = coef<R>(p, kH2), udx3 = coef<R>(p, kH3);
  R tc = T[c0], tip = T[c0 + dip], tim = T[c0 + dim], tjp = T[c0 + djp], tjm = T[c0 + djm];
  R tkp = T[c0 + dkp], tkm = T[c0 + dkm];
  R x31 = vx[c0 + dip] * (tip + tc) - vx[c0] * (tc + tim);
  R x32 = vy[c0 + djp] * (tjp + tc) - vy[c0] * (tc + tjm);
  R x33 = vz[c0 + dkp] * (tkp + tc) - vz[c0] * (tc + tkm);
  R hs = udx1 * x31 + udx2 * x32 + udx3 * x33;     // h31 + h32 + h33
  const double vpd = A.vofp[c0];
  if (vof_is_one(vpd)) return -hs;                 // fluid cell: VOFp = 1, no solid term
  R vp = narrow<R>(vpd);
  R ht = -hs * vp;
  R sv = R(1.0) - vp;
  R h31, h32, h33;
  if (sv != R(0.0)) {
    // solid-body advection, hdnlte.f90:94-153 (Fortran indices i+1, j+1, k+1);
    // positions and the rigid-body velocity in FP64
    int fi = i + 1, fj = j + 1, fk = k + 1;
    double r0 = A.xc[fi + A.coff] - p.pos[0], r1 = A.ym[fj + A.coff] - p.pos[1], r2 = A.zm[fk + A.coff] - p.pos[2];
    r0 = r0 - g.xlen * nint_d(r0 / g.xlen); r1 = r1 - g.ylen * nint_d(r1 / g.ylen); r2 = r2 - g.zlen * nint_d(r2 / g.zlen);
    double u_imh = p.vel[0] + p.om[1] * r2 - p.om[2] * r1;
    h31 = R(u_imh) * (tip - tim) * udx1;
    r0 = A.xm[fi + A.coff] - p.pos[0]; r1 = A.yc[fj + A.coff] - p.pos[1]; r2 = A.zm[fk + A.coff] - p.pos[2];
    r0 = r0 - g.xlen * nint_d(r0 / g.xlen); r1 = r1 - g.ylen * nint_d(r1 / g.ylen); r2 = r2 - g.zlen * nint_d(r2 / g.zlen);
    double v_jmh = p.vel[1] + p.om[2] * r0 - p.om[0] * r2;
    h32 = R(v_jmh) * (tjp - tjm) * udx2;
    r0 = A.xm[fi + A.coff] - p.pos[0]; r1 = A.ym[fj + A.coff] - p.pos[1]; r2 = A.zc[fk + A.coff] - p.pos[2];
    double w_kmh = p.vel[2] + p.om[0] * r1 - p.om[1] * r0;
    h33 = R(w_kmh) * (tkp - tkm) * udx3;
    ht = ht - (h31 + h32 + h33) * sv;
  }
  return ht;
}

__global__ void hdnl_kernel(StencilArgs A, int which, const StepParams* __restrict__ pp, double* __restrict__ out) {
  CELL_INDEX
  StepParams p = *pp;
  double h;
  if (which == 0) h = h_x<double>(A, c0, dip, dim, djp, djm, dkp, dkm, p);
  else if (which == 1) h = h_y<double>(A, c0, dip, dim, djp, djm, dkp, dkm, p);
  else if (which == 2) h = h_z<double>(A, c0, dip, dim, djp, djm, dkp, dkm, p);
  else h = h_t<double>(A, i, j, k, c0, dip, dim, djp, djm, dkp, dkm, p);
  out[c0] = h;
}

// ---------------------------------------------------------------------
// RHS of the factored implicit step
// ---------------------------------------------------------------------
// Diffusion term of the RHS with its factor folded into the coefficients:
// sum_d L_d*(q[+d] - 2 q + q[-d]) = sum_d L_d*(q[+d] + q[-d]) - LC*q,
// L_d = al/ren*dt*dxq_d (or al/pec*dt*dxq_d) and LC = 2*(L1 + L2 + L3).
// ISO (FP64, equal grid spacings, L1 = L2 = L3): the six neighbours summed in
// 64-bit integers on the integer pipe and rounded once (sum6_f64), two FP64
// operations per cell instead of seven, within FP64 round-off of the
// reference's order.
template <typename R, bool ISO = false>
__device__ __forceinline__ R lap_dt(const R* q, idx_t c0, idx_t dip, idx_t dim, idx_t djp, idx_t djm,
                                    idx_t dkp, idx_t dkm, R L1, R L2, R L3, R LC) {
  if constexpr (ISO && sizeof(R) == 8) {
    const R s = L1 * sum6_f64(q[c0 + dip], q[c0 + dim], q[c0 + djp], q[c0 + djm], q[c0 + dkp], q[c0 + dkm]);
    return s - LC * q[c0];
  } else {
    R s = L1 * (q[c0 + dip] + q[c0 + dim]) + L2 * (q[c0 + djp] + q[c0 + djm]) + L3 * (q[c0 + dkp] + q[c0 + dkm]);
    return s - LC * q[c0];
  }
}

// rhs = dt*(ga*H + ro*ru + al/ren*lap(u) - al*grad p) (invtr1.f90:57-60 and
// invtr2/3) and rhs = dt*(ga*H + ro*ru) + al/pec*dt*lap(T) (invtrte.f90),
// evaluated as GDT*H + RDT*ru + lap_dt - PD*(p - p[-1]) with the products of
// dt and the substep coefficients formed once per substep on the host: the
// same value up to rounding, with 11 (velocity) or 9 (temperature) FP64
// operations per cell instead of 18 and 17.
template <typename R, bool ISO = false>
__device__ __forceinline__ R rhs_value(const StencilArgs& A, int which, R h, R ru, idx_t c0, idx_t dip,
                                       idx_t dim, idx_t djp, idx_t djm, idx_t dkp, idx_t dkm,
                                       const StepParams& p) {
  const Prog<R> F = prog<R>(A);
  const R gdt = coef<R>(p, kGDT), rdt = coef<R>(p, kRDT);
  if (which == 3) {
    R d = lap_dt<R, ISO>(F.t, c0, dip, dim, djp, djm, dkp, dkm, coef<R>(p, kLT1), coef<R>(p, kLT2),
                    coef<R>(p, kLT3), coef<R>(p, kLTC));
    return gdt * h + (rdt * ru + d);
  }
  const R* q = which == 0 ? F.u : (which == 1 ? F.v : F.w);
  const idx_t dpm = which == 0 ? dim : (which == 1 ? djm : dkm);
  const R pd = coef<R>(p, which == 0 ? kPD1 : (which == 1 ? kPD2 : kPD3));
  R d = lap_dt<R, ISO>(q, c0, dip, dim, djp, djm, dkp, dkm, coef<R>(p, kLV1), coef<R>(p, kLV2), coef<R>(p, kLV3),
                  coef<R>(p, kLVC));
  return gdt * h + (rdt * ru + (d - pd * (F.p[c0] - F.p[c0 + dpm])));
}

// invtr drop-in: reads H from the explicit-term array, writes rhs, ru = H
__global__ void invtr_rhs_kernel(StencilArgs A, int which, const StepParams* __restrict__ pp,
                                 const double* __restrict__ H, double* __restrict__ ru, double* __restrict__ rhs) {
  CELL_INDEX
  StepParams p = *pp;
  double h = H[c0];
  rhs[c0] = rhs_value<double>(A, which, h, ru[c0], c0, dip, dim, djp, djm, dkp, dkm, p);
  ru[c0] = h;
}

// fused path: explicit term computed in registers (hdnl + invtr RHS); R is
// the compute type, ru and rhs are stored in R
// (one instance per component W, so each carries only its own stencil; ISO:
// the FP64 advection differences of h_prod and the diffusion sum of lap_dt
// on the integer pipe)
template <typename R, int W, bool ISO = false>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 3)
fused_rhs_kernel(StencilArgs A, const StepParams* __restrict__ pp, R* __restrict__ ru, R* __restrict__ rhs) {
  CELL_INDEX
  const StepParams& p = *pp;
  R h;
  if (W < 3) h = h_prod<R, ISO>(A, W, c0, dip, dim, djp, djm, dkp, dkm, p);   // products of adv_products_kernel
  else h = h_t<R>(A, i, j, k, c0, dip, dim, djp, djm, dkp, dkm, p);
  rhs[c0] = rhs_value<R, ISO>(A, W, h, ru[c0], c0, dip, dim, djp, djm, dkp, dkm, p);
  ru[c0] = h;
}

// Precision form: the explicit terms and RHS of u, v and w in one pass over
// the FP32 mirrors.  The advection products that adv_products_kernel writes
// for the FP64 form (Pc, Qc, Rc, E, Fx, H at a cell and at its neighbours)
// are formed here from the velocities by the same operations in the same
// order -- the products rounded on their own (__fmul_rn), so that none is
// fused into the difference that follows -- and the rest is h_prod's and
// rhs_value's: the same bits as the products kernel followed by
// fused_rhs_kernel<float, 0..2>, with about 100 instead of 180 bytes of
// traffic per cell and one launch instead of four.
__global__ void __launch_bounds__(256, 2)
fused_uvw_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp, float* __restrict__ ru3,
                     float* __restrict__ rhs3) {
  CELL_INDEX
  const StepParams& p = *pp;
  const float* __restrict__ u = A.u32;
  const float* __restrict__ v = A.v32;
  const float* __restrict__ w = A.w32;
  const float* __restrict__ pr = A.p32;
  const size_t n = g.cells;
  // every value the cell needs, loaded before any is used: the loads are
  // independent, so they are all in flight at once (the kernel is bound by
  // their latency)
  const double vfx = A.forcing ? A.vofx[c0] : 1.0, vfy = A.forcing ? A.vofy[c0] : 1.0;
  const double vfz = A.forcing ? A.vofz[c0] : 1.0;
  const double fcx = A.forcing ? A.forcx[c0] : 0.0, fcy = A.forcing ? A.forcy[c0] : 0.0;
  const double fcz = A.forcing ? A.forcz[c0] : 0.0;
  const float ru0 = ru3[c0], ru1 = ru3[n + c0], ru2 = ru3[2 * n + c0];
  const float uc = u[c0], uip = u[c0 + dip], um = u[c0 + dim], ujp = u[c0 + djp], ujm = u[c0 + djm];
  const float ukp = u[c0 + dkp], ukm = u[c0 + dkm], uipjm = u[c0 + dip + djm], uipkm = u[c0 + dip + dkm];
  const float vc = v[c0], vip = v[c0 + dip], vim = v[c0 + dim], vjp = v[c0 + djp], vm = v[c0 + djm];
  const float vkp = v[c0 + dkp], vkm = v[c0 + dkm], vjpim = v[c0 + djp + dim], vjpkm = v[c0 + djp + dkm];
  const float wc = w[c0], wip = w[c0 + dip], wim = w[c0 + dim], wjp = w[c0 + djp], wjm = w[c0 + djm];
  const float wkp = w[c0 + dkp], wm = w[c0 + dkm], wkpim = w[c0 + dkp + dim], wkpjm = w[c0 + dkp + djm];
  const float pc = pr[c0], pim = pr[c0 + dim], pjm = pr[c0 + djm], pkm = pr[c0 + dkm];
  const float tc = p.betagz != 0.0 ? A.t32[c0] : 0.f, tkm = p.betagz != 0.0 ? A.t32[c0 + dkm] : 0.f;
  // products at c0
  const float Pc0 = __fmul_rn(uip + uc, uip + uc);
  const float Qc0 = __fmul_rn(vjp + vc, vjp + vc);
  const float Rc0 = __fmul_rn(wkp + wc, wkp + wc);
  const float E0 = __fmul_rn(vc + vim, uc + ujm);
  const float F0 = __fmul_rn(wc + wim, uc + ukm);
  const float H0 = __fmul_rn(wc + wjm, vc + vkm);
  // products at the neighbours the differences need (each the product of
  // the cell it belongs to: Pc(c) = (u[c+i] + u[c])^2, E(c) = (v[c] +
  // v[c-i]) (u[c] + u[c-j]), Fx(c) = (w[c] + w[c-i]) (u[c] + u[c-k]),
  // H(c) = (w[c] + w[c-j]) (v[c] + v[c-k]))
  const float Pcm = __fmul_rn(uc + um, uc + um);
  const float Qcm = __fmul_rn(vc + vm, vc + vm);
  const float Rcm = __fmul_rn(wc + wm, wc + wm);
  const float Ejp = __fmul_rn(vjp + vjpim, ujp + uc);
  const float Eip = __fmul_rn(vip + vc, uip + uipjm);
  const float Fkp = __fmul_rn(wkp + wkpim, ukp + uc);
  const float Fip = __fmul_rn(wip + wc, uip + uipkm);
  const float Hkp = __fmul_rn(wkp + wkpjm, vkp + vc);
  const float Hjp = __fmul_rn(wjp + wc, vjp + vjpkm);
  const float udx1 = p.cf[kQ1], udx2 = p.cf[kQ2], udx3 = p.cf[kQ3];
  // h_prod's expressions, add_forcing's forcing term
  auto forced = [&](float h, double vf, double fc, float rlen) {
    if (!A.forcing) return h;
    return (vof_is_one(vf) ? d2f_bits(fc) : d2f_bits(vf * fc)) * rlen + h;
  };
  float hu = -(udx1 * (Pc0 - Pcm) + udx2 * (Ejp - E0) + udx3 * (Fkp - F0));
  hu = forced(hu, vfx, fcx, p.cf[kRXLEN]);
  float hv = -(udx1 * (Eip - E0) + udx2 * (Qc0 - Qcm) + udx3 * (Hkp - H0));
  hv = forced(hv, vfy, fcy, p.cf[kRYLEN]);
  float hw = -(udx1 * (Fip - F0) + udx2 * (Hjp - H0) + udx3 * (Rc0 - Rcm));
  if (p.betagz != 0.0) {
    const float T_interp = (tc + tkm) * 0.5f;
    hw = hw + p.cf[kBETAGZ] * (T_interp - p.cf[kTLIQ]);
  }
  hw = forced(hw, vfz, fcz, p.cf[kRZLEN]);
  // rhs_value's expressions (lap_dt, pressure gradient, RK combination)
  const float gdt = p.cf[kGDT], rdt = p.cf[kRDT];
  const float L1 = p.cf[kLV1], L2 = p.cf[kLV2], L3 = p.cf[kLV3], LC = p.cf[kLVC];
  const float du = (L1 * (uip + um) + L2 * (ujp + ujm) + L3 * (ukp + ukm)) - LC * uc;
  const float dv = (L1 * (vip + vim) + L2 * (vjp + vm) + L3 * (vkp + vkm)) - LC * vc;
  const float dw = (L1 * (wip + wim) + L2 * (wjp + wjm) + L3 * (wkp + wm)) - LC * wc;
  rhs3[c0] = gdt * hu + (rdt * ru0 + (du - p.cf[kPD1] * (pc - pim)));
  rhs3[n + c0] = gdt * hv + (rdt * ru1 + (dv - p.cf[kPD2] * (pc - pjm)));
  rhs3[2 * n + c0] = gdt * hw + (rdt * ru2 + (dw - p.cf[kPD3] * (pc - pkm)));
  ru3[c0] = hu;
  ru3[n + c0] = hv;
  ru3[2 * n + c0] = hw;
}

// Precision form: the temperature's explicit term and RHS (hdnlte + invtrte)
// as fused_rhs_kernel<float, 3> computes them, with every value of a fluid
// cell loaded before any is used (the kernel is bound by load latency); a
// cell that is not fully fluid takes h_t's solid-advection branch.  The
// same bits as fused_rhs_kernel<float, 3>.
__global__ void __launch_bounds__(256, 3)
fused_t_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp, float* __restrict__ ru,
                   float* __restrict__ rhs) {
  CELL_INDEX
  const StepParams& p = *pp;
  const float* __restrict__ T = A.t32;
  const double vpd = A.vofp[c0];
  const float ruc = ru[c0];
  const float tc = T[c0], tip = T[c0 + dip], tim = T[c0 + dim], tjp = T[c0 + djp], tjm = T[c0 + djm];
  const float tkp = T[c0 + dkp], tkm = T[c0 + dkm];
  const float uip = A.u32[c0 + dip], uc = A.u32[c0], vjp = A.v32[c0 + djp], vc = A.v32[c0];
  const float wkp = A.w32[c0 + dkp], wc = A.w32[c0];
  float h;
  if (vof_is_one(vpd)) {
    const float udx1 = p.cf[kH1], udx2 = p.cf[kH2], udx3 = p.cf[kH3];
    const float x31 = uip * (tip + tc) - uc * (tc + tim);
    const float x32 = vjp * (tjp + tc) - vc * (tc + tjm);
    const float x33 = wkp * (tkp + tc) - wc * (tc + tkm);
    const float hs = udx1 * x31 + udx2 * x32 + udx3 * x33;
    h = -hs;
  } else {
    h = h_t<float>(A, i, j, k, c0, dip, dim, djp, djm, dkp, dkm, p);
  }
  const float d = (p.cf[kLT1] * (tip + tim) + p.cf[kLT2] * (tjp + tjm) + p.cf[kLT3] * (tkp + tkm)) - p.cf[kLTC] * tc;
  rhs[c0] = p.cf[kGDT] * h + (p.cf[kRDT] * ruc + d);
  ru[c0] = h;
}

static bool equal_spacings(const Grid& g) { return g.dx1 == g.dx2 && g.dx1 == g.dx3; }

template <typename R, bool ISO>
static void fused_rhs_launch_by(Ctx* c, const StepParams* dp, int w, R* ru, R* rhs) {
  const int by = (c->tune_by == 2 || c->tune_by == 4) ? c->tune_by : 8;   // autotuned block height
  dim3 grid(div_up(c->g.n1m, 32), div_up(c->g.n2m, by), c->g.n3m), block(32, by);
  StencilArgs a = make_args(c);
  switch (w) {
    case 0: fused_rhs_kernel<R, 0, ISO><<<grid, block, 0, c->stream>>>(a, dp, ru, rhs); break;
    case 1: fused_rhs_kernel<R, 1, ISO><<<grid, block, 0, c->stream>>>(a, dp, ru, rhs); break;
    case 2: fused_rhs_kernel<R, 2, ISO><<<grid, block, 0, c->stream>>>(a, dp, ru, rhs); break;
    default: fused_rhs_kernel<R, 3, ISO><<<grid, block, 0, c->stream>>>(a, dp, ru, rhs); break;
  }
}

// FP64 with equal spacings: the advection and diffusion sums on the integer
// pipe; the FP32
// instances keep the FP32 arithmetic (one-pass kernels give their bits)
template <typename R>
static void fused_rhs_launch(Ctx* c, const StepParams* dp, int w, R* ru, R* rhs) {
  if (sizeof(R) == 8 && equal_spacings(c->g)) fused_rhs_launch_by<R, true>(c, dp, w, ru, rhs);
  else fused_rhs_launch_by<R, false>(c, dp, w, ru, rhs);
}

static void fused_uvw_launch(Ctx* c, const StepParams* dp, float* ru4, float* rhs4) {
  const int by = (c->tune_by == 2 || c->tune_by == 4) ? c->tune_by : 8;   // autotuned block height
  dim3 grid(div_up(c->g.n1m, 32), div_up(c->g.n2m, by), c->g.n3m), block(32, by);
  fused_uvw_f32_kernel<<<grid, block, 0, c->stream>>>(make_args(c), dp, ru4, rhs4);
}

static void fused_t_launch(Ctx* c, const StepParams* dp, float* ru, float* rhs) {
  const int by = (c->tune_by == 2 || c->tune_by == 4) ? c->tune_by : 8;   // autotuned block height
  dim3 grid(div_up(c->g.n1m, 32), div_up(c->g.n2m, by), c->g.n3m), block(32, by);
  fused_t_f32_kernel<<<grid, block, 0, c->stream>>>(make_args(c), dp, ru, rhs);
}

// ---------------------------------------------------------------------
// projection stencils
// ---------------------------------------------------------------------
// divg.f90: dph = div(u) / (dt al).  ISO (equal grid spacings): the sum of
// the three face differences formed in 64-bit integers on the integer pipe
// and rounded once (sum3_diff_f64), times dx1/(dt al): one FP64 operation
// per cell instead of six, within FP64 round-off of the reference's order.
template <bool ISO>
__global__ void divg_kernel(StencilArgs A, const StepParams* __restrict__ pp, double* __restrict__ dph) {
  CELL_INDEX
  if constexpr (ISO) {
    dph[c0] = sum3_diff_f64(A.vx[c0 + dip], A.vx[c0], A.vy[c0 + djp], A.vy[c0], A.vz[c0 + dkp], A.vz[c0]) *
              pp->cd[kDVI];
  } else {
    double usdtal = pp->cd[kUSDTAL];
    double dq = (A.vx[c0 + dip] - A.vx[c0]) * g.dx1 + (A.vy[c0 + djp] - A.vy[c0]) * g.dx2 +
                (A.vz[c0 + dkp] - A.vz[c0]) * g.dx3;
    dph[c0] = dq * usdtal;
  }
}

// precision form: the divergence residual of the FP64 velocity, formed at
// FP64 accuracy (the face differences cancel to round-off of u), then rounded
// once to FP32 as the right-hand side of the FP32 Poisson solve.  ISO (equal
// grid spacings in the three directions): the sum of the three differences is
// formed in 64-bit integers on the integer pipe (sum3_diff_f32: FP64
// accuracy, no FP64 instruction; five FP64 operations per cell bounded the
// kernel at 2.4 times its memory time) and the spacing is folded into the
// FP32 factor; otherwise the differences are scaled in FP64.
template <bool ISO>
__global__ void divg_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp, float* __restrict__ res) {
  CELL_INDEX
  if constexpr (ISO) {
    res[c0] = sum3_diff_f32(A.vx[c0 + dip], A.vx[c0], A.vy[c0 + djp], A.vy[c0], A.vz[c0 + dkp], A.vz[c0]) *
              pp->cf[kDVI];
  } else {
    double du = A.vx[c0 + dip] - A.vx[c0], dv = A.vy[c0 + djp] - A.vy[c0], dw = A.vz[c0 + dkp] - A.vz[c0];
    double dq = fma(dw, g.dx3, fma(dv, g.dx2, du * g.dx1));
    res[c0] = d2f_bits(dq) * pp->cf[kUSDTAL];
  }
}

// mean3 (fused step only): the mean IBM force of velforce.f90:21-50, removed
// here instead of in a separate pass (a constant does not change divg)
__global__ void updvp_kernel(StencilArgs A, const StepParams* __restrict__ pp, const double* __restrict__ dph,
                             double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                             const double* __restrict__ mean3) {
  CELL_INDEX
  double udx1 = pp->cd[kUP1], udx2 = pp->cd[kUP2], udx3 = pp->cd[kUP3];
  double loc = dph[c0];
  double mx = 0.0, my = 0.0, mz = 0.0;
  if (mean3) { mx = mean3[0]; my = mean3[1]; mz = mean3[2]; }
  vx[c0] = (vx[c0] - mx) - (loc - dph[c0 + dim]) * udx1;
  vy[c0] = (vy[c0] - my) - (loc - dph[c0 + djm]) * udx2;
  vz[c0] = (vz[c0] - mz) - (loc - dph[c0 + dkm]) * udx3;
}

// precision form: u -= al dt grad(phi) with phi from the FP32 Poisson solve;
// the increment is formed in FP32 (with the FP32 mean force mean3f folded
// in when given) and added to the FP64 velocity; optional FP32 mirror m32
// (u, v, w at 0, cells, 2 cells)
__global__ void updvp_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp, const float* __restrict__ phi,
                                 double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                                 const float* __restrict__ mean3f, float* __restrict__ m32) {
  CELL_INDEX
  float loc = phi[c0];
  float ix = (loc - phi[c0 + dim]) * pp->cf[kUP1];
  float iy = (loc - phi[c0 + djm]) * pp->cf[kUP2];
  float iz = (loc - phi[c0 + dkm]) * pp->cf[kUP3];
  if (mean3f) { ix += mean3f[0]; iy += mean3f[1]; iz += mean3f[2]; }
  double x = vx[c0] - f2d_bits(ix), y = vy[c0] - f2d_bits(iy), z = vz[c0] - f2d_bits(iz);
  vx[c0] = x; vy[c0] = y; vz[c0] = z;
  if (m32) { m32[c0] = d2f_bits(x); m32[c0 + g.cells] = d2f_bits(y); m32[c0 + 2 * g.cells] = d2f_bits(z); }
}

// precision form: p += phi - al beta lap(phi), increment in FP32, optional
// FP32 mirror of p
__global__ void prcalc_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp, const float* __restrict__ phi,
                                  double* __restrict__ pr, float* __restrict__ m32) {
  CELL_INDEX
  float be = pp->cf[kBE];
  float d = phi[c0];
  float inc = d - be * ((phi[c0 + dip] - 2.0f * d + phi[c0 + dim]) * pp->cf[kDQ1] +
                        (phi[c0 + djp] - 2.0f * d + phi[c0 + djm]) * pp->cf[kDQ2] +
                        (phi[c0 + dkp] - 2.0f * d + phi[c0 + dkm]) * pp->cf[kDQ3]);
  double q = pr[c0] + f2d_bits(inc);
  pr[c0] = q;
  if (m32) m32[c0] = d2f_bits(q);
}

// precision form: updvp_f32_kernel and prcalc_f32_kernel in one pass (they
// read the same phi), every load issued before the first use; the same
// expressions, so the same bits.  m32: the mirrors' base (u, v, w at 0,
// cells, 2 cells; p at 4 cells), or null
// OOP: u, v, w read from (ux, uy, uz) and written to (vx, vy, vz) (after a
// sweep of updvp_prcalc_divg_f32_kernel); otherwise in place in (vx, vy, vz)
template <bool OOP>
__global__ void updvp_prcalc_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp,
                                        const float* __restrict__ phi, const double* __restrict__ ux,
                                        const double* __restrict__ uy, const double* __restrict__ uz,
                                        double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                                        double* __restrict__ pr, const float* __restrict__ mean3f,
                                        float* __restrict__ m32) {
  CELL_INDEX
  const float loc = phi[c0], fim = phi[c0 + dim], fjm = phi[c0 + djm], fkm = phi[c0 + dkm];
  const float fip = phi[c0 + dip], fjp = phi[c0 + djp], fkp = phi[c0 + dkp];
  const double u0 = (OOP ? ux : vx)[c0], v0 = (OOP ? uy : vy)[c0], w0 = (OOP ? uz : vz)[c0], p0 = pr[c0];
  float ix = (loc - fim) * pp->cf[kUP1];
  float iy = (loc - fjm) * pp->cf[kUP2];
  float iz = (loc - fkm) * pp->cf[kUP3];
  if (mean3f) { ix += mean3f[0]; iy += mean3f[1]; iz += mean3f[2]; }
  const double x = u0 - f2d_bits(ix), y = v0 - f2d_bits(iy), z = w0 - f2d_bits(iz);
  vx[c0] = x; vy[c0] = y; vz[c0] = z;
  const float be = pp->cf[kBE];
  const float inc = loc - be * ((fip - 2.0f * loc + fim) * pp->cf[kDQ1] +
                                (fjp - 2.0f * loc + fjm) * pp->cf[kDQ2] +
                                (fkp - 2.0f * loc + fkm) * pp->cf[kDQ3]);
  const double q = p0 + f2d_bits(inc);
  pr[c0] = q;
  if (m32) {
    m32[c0] = d2f_bits(x); m32[c0 + g.cells] = d2f_bits(y); m32[c0 + 2 * g.cells] = d2f_bits(z);
    m32[c0 + 4 * g.cells] = d2f_bits(q);
  }
}

// precision form, a projection sweep that is not the last: the update of
// updvp_prcalc_f32_kernel with u, v, w written out of place (from (ux, uy,
// uz) to (vx, vy, vz); p in place; no mirrors), together with the next
// sweep's divergence residual of the updated velocity (divg_f32_kernel).
// The updates of the three upwind neighbours (i+1, j+1, k+1) are formed
// again here by the same operations, so they have the bits that their own
// threads write: the residual equals divg_f32_kernel's on the written
// fields, and the sweep reads the velocity once instead of twice.
template <bool ISO>
__global__ void updvp_prcalc_divg_f32_kernel(StencilArgs A, const StepParams* __restrict__ pp,
                                             const float* __restrict__ phi, const double* __restrict__ ux,
                                             const double* __restrict__ uy, const double* __restrict__ uz,
                                             double* __restrict__ vx, double* __restrict__ vy,
                                             double* __restrict__ vz, double* __restrict__ pr,
                                             const float* __restrict__ mean3f, float* __restrict__ res) {
  CELL_INDEX
  const float loc = phi[c0], fim = phi[c0 + dim], fjm = phi[c0 + djm], fkm = phi[c0 + dkm];
  const float fip = phi[c0 + dip], fjp = phi[c0 + djp], fkp = phi[c0 + dkp];
  const double u0 = ux[c0], v0 = uy[c0], w0 = uz[c0], p0 = pr[c0];
  const double un = ux[c0 + dip], vn = uy[c0 + djp], wn = uz[c0 + dkp];
  float ix = (loc - fim) * pp->cf[kUP1], iy = (loc - fjm) * pp->cf[kUP2], iz = (loc - fkm) * pp->cf[kUP3];
  float jx = (fip - loc) * pp->cf[kUP1], jy = (fjp - loc) * pp->cf[kUP2], jz = (fkp - loc) * pp->cf[kUP3];
  if (mean3f) {
    ix += mean3f[0]; iy += mean3f[1]; iz += mean3f[2];
    jx += mean3f[0]; jy += mean3f[1]; jz += mean3f[2];
  }
  const double x = u0 - f2d_bits(ix), y = v0 - f2d_bits(iy), z = w0 - f2d_bits(iz);
  const double xn = un - f2d_bits(jx), yn = vn - f2d_bits(jy), zn = wn - f2d_bits(jz);
  vx[c0] = x; vy[c0] = y; vz[c0] = z;
  const float be = pp->cf[kBE];
  const float inc = loc - be * ((fip - 2.0f * loc + fim) * pp->cf[kDQ1] +
                                (fjp - 2.0f * loc + fjm) * pp->cf[kDQ2] +
                                (fkp - 2.0f * loc + fkm) * pp->cf[kDQ3]);
  pr[c0] = p0 + f2d_bits(inc);
  if constexpr (ISO) {
    res[c0] = sum3_diff_f32(xn, x, yn, y, zn, z) * pp->cf[kDVI];
  } else {
    const double du = xn - x, dv = yn - y, dw = zn - z;
    const double dq = fma(dw, g.dx3, fma(dv, g.dx2, du * g.dx1));
    res[c0] = d2f_bits(dq) * pp->cf[kUSDTAL];
  }
}

// FP32 mirrors of u, v, w, T, p (field f at m32 + f*cells)
__global__ void mirror_kernel(size_t n, const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, const double* __restrict__ t,
                              const double* __restrict__ p, float* __restrict__ m32) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  m32[e] = d2f_bits(u[e]); m32[e + n] = d2f_bits(v[e]); m32[e + 2 * n] = d2f_bits(w[e]);
  m32[e + 3 * n] = d2f_bits(t[e]); m32[e + 4 * n] = d2f_bits(p[e]);
}

__global__ void cast_d2f_kernel(size_t n, const double* __restrict__ a, float* __restrict__ b) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) b[e] = d2f_bits(a[e]);
}

__global__ void cast_f2d_kernel(size_t n, const float* __restrict__ a, double* __restrict__ b) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) b[e] = f2d_bits(a[e]);
}

// max |div u| (divgck semantics, divg.f90:26-56) into bits of `out`
__global__ void divmax_kernel(StencilArgs A, unsigned long long* __restrict__ out) {
  CELL_INDEX
  double dq = (A.vx[c0 + dip] - A.vx[c0]) * g.dx1 + (A.vy[c0 + djp] - A.vy[c0]) * g.dx2 +
              (A.vz[c0 + dkp] - A.vz[c0]) * g.dx3;
  double v = fabs(dq);
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

__global__ void prcalc_kernel(StencilArgs A, const StepParams* __restrict__ pp, const double* __restrict__ dph,
                              double* __restrict__ pr) {
  CELL_INDEX
  // p + phi - al*beta*lap(phi) (prcalc.f90:17-33) as
  // p + (1 + 2 al beta sum dxq) phi - sum (al beta dxq)(phi[+] + phi[-]):
  // the coefficients formed on the host, 8 FP64 operations instead of 14
  const double d = dph[c0];
  const double t = pp->cd[kPB1] * (dph[c0 + dip] + dph[c0 + dim]) + pp->cd[kPB2] * (dph[c0 + djp] + dph[c0 + djm]) +
                   pp->cd[kPB3] * (dph[c0 + dkp] + dph[c0 + dkm]);
  pr[c0] = (pr[c0] + pp->cd[kPBC] * d) - t;
}

// updvp then prcalc of the same substep in one pass (the fused step): both
// read phi and write disjoint fields; each keeps its own operation order
// ISO (equal grid spacings): the six neighbours of the pressure update's
// Laplacian summed in 64-bit integers on the integer pipe (sum6_f64) and
// scaled once: three FP64 operations for the pressure instead of eight,
// within FP64 round-off of the reference's order (prcalc.f90)
template <bool ISO>
__global__ void updvp_prcalc_kernel(StencilArgs A, const StepParams* __restrict__ pp, const double* __restrict__ dph,
                                    double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                                    const double* __restrict__ mean3, double* __restrict__ pr) {
  CELL_INDEX
  const double udx1 = pp->cd[kUP1], udx2 = pp->cd[kUP2], udx3 = pp->cd[kUP3];
  const double d = dph[c0];
  const double pim = dph[c0 + dim], pjm = dph[c0 + djm], pkm = dph[c0 + dkm];
  const double pip = dph[c0 + dip], pjp = dph[c0 + djp], pkp = dph[c0 + dkp];
  double mx = 0.0, my = 0.0, mz = 0.0;
  if (mean3) { mx = mean3[0]; my = mean3[1]; mz = mean3[2]; }
  vx[c0] = (vx[c0] - mx) - (d - pim) * udx1;
  vy[c0] = (vy[c0] - my) - (d - pjm) * udx2;
  vz[c0] = (vz[c0] - mz) - (d - pkm) * udx3;
  double t;
  if constexpr (ISO) t = pp->cd[kPB1] * sum6_f64(pip, pim, pjp, pjm, pkp, pkm);
  else t = pp->cd[kPB1] * (pip + pim) + pp->cd[kPB2] * (pjp + pjm) + pp->cd[kPB3] * (pkp + pkm);
  pr[c0] = (pr[c0] + pp->cd[kPBC] * d) - t;
}

__global__ void add_kernel(Grid g, double* __restrict__ q, const double* __restrict__ r) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.cells) q[t] = q[t] + r[t];
}

__global__ void interp_vof_kernel(StencilArgs A, double* __restrict__ vofx, double* __restrict__ vofy,
                                  double* __restrict__ vofz) {
  CELL_INDEX
  const double* vp = A.vofp;
  double c = vp[c0];
  // 0.5*(a + c) == c exactly when a and c are the same double (a + c = 2c
  // and the halving are exact), which holds everywhere but at the
  // interface; testing the bits keeps those cells off the FP64 pipe
  const long long cb = __double_as_longlong(c);
  double a = vp[c0 + dim], b = vp[c0 + djm], d = vp[c0 + dkm];
  bool same = __double_as_longlong(a) == cb && __double_as_longlong(b) == cb && __double_as_longlong(d) == cb;
  if (__all_sync(__activemask(), same)) {   // warp-uniform branch: no FP64 issue at all
    vofx[c0] = c; vofy[c0] = c; vofz[c0] = c;
    return;
  }
  vofx[c0] = 0.5 * (a + c);
  vofy[c0] = 0.5 * (b + c);
  vofz[c0] = 0.5 * (d + c);
}

__global__ void velforce_apply_kernel(Grid g, const double* __restrict__ mean3, const double* __restrict__ fx,
                                      const double* __restrict__ fy, const double* __restrict__ fz,
                                      double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.cells) return;
  vx[t] = vx[t] + fx[t] - mean3[0];
  vy[t] = vy[t] + fy[t] - mean3[1];
  vz[t] = vz[t] + fz[t] - mean3[2];
}

__global__ void tempforce_apply_kernel(Grid g, const double* __restrict__ ft, double* __restrict__ T) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.cells) return;
  T[t] = T[t] + ft[t];
}

// ---------------------------------------------------------------------
// CFL reductions (max is order independent: bitwise deterministic)
// ---------------------------------------------------------------------
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// cfl.f90:11-26: i+1, j+1, k+1 are not wrapped -- column n1 / row n2 are the
// stored padding values, plane n3m+1 is the periodic ghost.
// R = float: the precision form on the FP32 mirrors (dt only sets the step
// size; the FP32 maximum is rounded up to double unchanged).  ISO (FP64,
// equal spacings): the three magnitudes summed on the integer pipe
// (sum3_abs_pair_f64) and scaled once, within FP64 round-off of cfl.f90's
// order, one FP64 operation per cell instead of eight.
template <typename R, bool ISO = false>
__global__ void cfl_kernel(StencilArgs A, const double* __restrict__ padx, const double* __restrict__ pady,
                           double* __restrict__ part, int* __restrict__ nonfinite) {
  const Grid& g = A.g;
  const Prog<R> F = prog<R>(A);
  const R h1 = R(0.5 * g.dx1), h2 = R(0.5 * g.dx2), h3 = R(0.5 * g.dx3);
  R mr = R(0);
  const int rows = g.n2m * g.n3m;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * g.n1m; t += gridDim.x * blockDim.x) {
    int i = t % g.n1m, row = t / g.n1m;
    int j = row % g.n2m, k = row / g.n2m;
    size_t c0 = cidx(g, i, j, k);
    R vxp = (i + 1 < g.n1m) ? F.u[c0 + 1] : R(padx[j + (size_t)g.n2m * k]);
    R vyp = (j + 1 < g.n2m) ? F.v[c0 + g.P] : R(pady[i + (size_t)g.n1m * k]);
    R vzp = F.w[cidx(g, i, j, (k + 1 == g.n3m) ? 0 : k + 1)];
    // (x*0.5)*dx of cfl.f90 equals x*(0.5*dx) bit for bit (scaling by 0.5 is
    // exact), so the FP64 value is the reference's with one multiply less
    R qcf;
    if constexpr (ISO && sizeof(R) == 8) qcf = sum3_abs_pair_f64(F.u[c0], vxp, F.v[c0], vyp, F.w[c0], vzp) * h1;
    else qcf = fabs((F.u[c0] + vxp) * h1) + fabs((F.v[c0] + vyp) * h2) + fabs((F.w[c0] + vzp) * h3);
    // a max would drop a NaN: a non-finite velocity or temperature raises the guard
    if (bits_nonfinite(qcf) || bits_nonfinite(F.t[c0])) atomicOr(nonfinite, 1);
    mr = max_nonneg(mr, qcf);
  }
  double m = warp_max((double)mr);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    v = warp_max(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// get_dt advective term: max(|u| dt dx1 + |v| dt dx2 + |w| dt dx3); ISO
// (FP64, equal spacings): (|u| + |v| + |w|) on the integer pipe
// (sum3_abs_f64) times dt dx1, within FP64 round-off of the reference's order
template <typename R, bool ISO = false>
__global__ void getdt_kernel(StencilArgs A, double dt, double* __restrict__ part) {
  const Grid& g = A.g;
  const Prog<R> F = prog<R>(A);
  const R d1 = R(dt * g.dx1), d2 = R(dt * g.dx2), d3 = R(dt * g.dx3);
  R mr = R(0);
  const int rows = g.n2m * g.n3m;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rows * g.n1m; t += gridDim.x * blockDim.x) {
    int i = t % g.n1m, row = t / g.n1m;
    size_t c0 = cidx(g, i, row % g.n2m, row / g.n2m);
    R v;
    if constexpr (ISO && sizeof(R) == 8)
      v = sum3_abs_f64(F.u[c0], F.v[c0], F.w[c0]) * d1;
    else if (sizeof(R) == 8)   // FP64 form: the reference's operation order
      v = fabs(F.u[c0]) * R(dt) * R(g.dx1) + fabs(F.v[c0]) * R(dt) * R(g.dx2) + fabs(F.w[c0]) * R(dt) * R(g.dx3);
    else
      v = fabs(F.u[c0]) * d1 + fabs(F.v[c0]) * d2 + fabs(F.w[c0]) * d3;
    mr = fmax(mr, v);
  }
  double m = warp_max((double)mr);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    v = warp_max(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

__global__ void max_reduce_kernel(const double* __restrict__ part, size_t n, double* __restrict__ out) {
  double m = 0.0;
  for (size_t t = threadIdx.x; t < n; t += blockDim.x) m = fmax(m, part[t]);
  m = warp_max(m);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    v = warp_max(v);
    if (threadIdx.x == 0) out[0] = v;
  }
}

// ---------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------
static dim3 cell_grid(const Grid& g) { return dim3(div_up(g.n1m, 32), div_up(g.n2m, 8), g.n3m); }
static const dim3 kCellBlock(32, 8);

static double* hdnl_out(Ctx* c, int which) {
  switch (which) {
    case 0: return c->df[MIBM_F_DQ];
    case 1: return c->df[MIBM_F_DPH];
    case 2: return c->df[MIBM_F_QCAP];
  }
  return c->df[MIBM_F_HTEMP];
}
static double* ru_of(Ctx* c, int which) {
  switch (which) {
    case 0: return c->df[MIBM_F_RU1];
    case 1: return c->df[MIBM_F_RU2];
    case 2: return c->df[MIBM_F_RU3];
  }
  return c->df[MIBM_F_RUT];
}

void k_hdnl(Ctx* c, int which, const StepParams* dp) {
  { MIBM_PROF(c, "hdnl"); hdnl_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), which, dp, hdnl_out(c, which)); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "hdnl");
}

void k_invtr_rhs(Ctx* c, int which, const StepParams* dp, double* rhs_out) {
  { MIBM_PROF(c, "invtr_rhs"); invtr_rhs_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), which, dp, hdnl_out(c, which),
                                                                   ru_of(c, which), rhs_out); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "invtr_rhs");
}

template <typename R>
static void adv_products_launch(Ctx* c, R* out) {
  { MIBM_PROF(c, sizeof(R) == 8 ? "adv_products" : "adv_products_f32");
    adv_products_kernel<R><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), out); }
  ++c->launches;
}

void k_fused_rhs(Ctx* c, const StepParams* dp) {
  adv_products_launch<double>(c, c->prod);
  for (int w = 0; w < 4; ++w) {
    { MIBM_PROF(c, "fused_rhs");
      fused_rhs_launch<double>(c, dp, w, ru_of(c, w), c->rhs4 + (size_t)w * c->g.cells); }
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, "fused_rhs");
}

// Autotuner support: time the explicit-term kernel (components u and T; in
// the precision form u, v, w and T) with block height `by`, best of `reps`
// runs after one warm-up, in ms.  The RK
// history it overwrites is saved first and restored, so the context's state
// is unchanged.  ru4/rhs4: the form's history and RHS buffers.
template <typename R>
static float time_fused_by(Ctx* c, const StepParams* dp, int by, int reps, R* ru4, R* rhs4, R* const* ru_fields) {
  const size_t n = c->g.cells;
  R* save = nullptr;
  if (!cuda_ok(c, cudaMalloc(&save, 4 * n * sizeof(R)), "tune")) return -1.f;
  for (int w = 0; w < 4; ++w)
    cudaMemcpyAsync(save + (size_t)w * n, ru_fields[w], n * sizeof(R), cudaMemcpyDeviceToDevice, c->stream);
  const int old = c->tune_by;
  c->tune_by = by;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const bool uvw = sizeof(R) == 4 && c->fused_uvw;
  if (sizeof(R) == 8) adv_products_launch<double>(c, c->prod);   // read by the u component
  else if (!uvw) adv_products_launch<float>(c, c->prod32);
  auto run = [&]() {
    if constexpr (sizeof(R) == 4) {
      if (uvw) {
        fused_uvw_launch(c, dp, ru_fields[0], rhs4);
        fused_t_launch(c, dp, ru_fields[3], rhs4 + 3 * n);
      } else {
        fused_rhs_launch<R>(c, dp, 0, ru_fields[0], rhs4);
        fused_rhs_launch<R>(c, dp, 3, ru_fields[3], rhs4 + 3 * n);
      }
    } else {
      fused_rhs_launch<R>(c, dp, 0, ru_fields[0], rhs4);
      fused_rhs_launch<R>(c, dp, 3, ru_fields[3], rhs4 + 3 * n);
    }
  };
  float best = -1.f;
  run();
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0, c->stream);
    run();
    cudaEventRecord(e1, c->stream);
    if (!cuda_ok(c, cudaEventSynchronize(e1), "tune")) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (best < 0.f || ms < best) best = ms;
  }
  for (int w = 0; w < 4; ++w)
    cudaMemcpyAsync(ru_fields[w], save + (size_t)w * n, n * sizeof(R), cudaMemcpyDeviceToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(save);
  c->tune_by = old;
  (void)ru4;
  return best;
}

float stencil_time_by(Ctx* c, const StepParams* dp, int by, int reps) {
  if (c->precision == 1) {
    float* ru[4];
    for (int w = 0; w < 4; ++w) ru[w] = c->ru32 + (size_t)w * c->g.cells;
    return time_fused_by<float>(c, dp, by, reps, c->ru32, c->rhs32, ru);
  }
  double* ru[4];
  for (int w = 0; w < 4; ++w) ru[w] = ru_of(c, w);
  return time_fused_by<double>(c, dp, by, reps, nullptr, c->rhs4, ru);
}

// precision form: FP32 explicit terms and RHS into FP32 ru / rhs buffers
// the precision form's explicit terms: u, v, w in one kernel (or, with the
// one-pass kernel switched off, through the products as in the FP64 form),
// then T
void k_fused_rhs_f32(Ctx* c, const StepParams* dp, float* ru4, float* rhs4) {
  if (c->fused_uvw) {
    { MIBM_PROF(c, "fused_uvw_f32"); fused_uvw_launch(c, dp, ru4, rhs4); }
    ++c->launches;
  } else {
    adv_products_launch<float>(c, c->prod32);
    for (int w = 0; w < 3; ++w) {
      { MIBM_PROF(c, "fused_rhs_f32");
        fused_rhs_launch<float>(c, dp, w, ru4 + (size_t)w * c->g.cells, rhs4 + (size_t)w * c->g.cells); }
      ++c->launches;
    }
  }
  { MIBM_PROF(c, "fused_rhs_f32");
    if (c->fused_uvw) fused_t_launch(c, dp, ru4 + 3 * c->g.cells, rhs4 + 3 * c->g.cells);
    else fused_rhs_launch<float>(c, dp, 3, ru4 + 3 * c->g.cells, rhs4 + 3 * c->g.cells); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "fused_rhs_f32");
}

void k_divg(Ctx* c, const StepParams* dp) {
  { MIBM_PROF(c, "divg");
    if (equal_spacings(c->g))
      divg_kernel<true><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, c->df[MIBM_F_DPH]);
    else
      divg_kernel<false><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, c->df[MIBM_F_DPH]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "divg");
}

void k_updvp(Ctx* c, const StepParams* dp, const double* mean3) {
  { MIBM_PROF(c, "updvp"); updvp_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, c->df[MIBM_F_DPH], c->df[MIBM_F_VX],
                                                               c->df[MIBM_F_VY], c->df[MIBM_F_VZ], mean3); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "updvp");
}

void k_updvp_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool mirror) {
  { MIBM_PROF(c, "updvp_f32");
    const float* mean3f = mean3 ? reinterpret_cast<const float*>(mean3 + 4) : nullptr;
    updvp_f32_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, phi, c->df[MIBM_F_VX],
                                                                     c->df[MIBM_F_VY], c->df[MIBM_F_VZ], mean3f,
                                                                     mirror ? c->q32 : nullptr); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "updvp_f32");
}

void k_updvp_prcalc_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool mirror,
                        bool from_vel1) {
  { MIBM_PROF(c, "updvp_prcalc_f32");
    const float* mean3f = mean3 ? reinterpret_cast<const float*>(mean3 + 4) : nullptr;
    double* const* f = c->df;
    if (from_vel1) {
      const double* u = c->vel1;
      updvp_prcalc_f32_kernel<true><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(
          make_args(c), dp, phi, u, u + c->g.cells, u + 2 * c->g.cells, f[MIBM_F_VX], f[MIBM_F_VY], f[MIBM_F_VZ],
          f[MIBM_F_PR], mean3f, mirror ? c->q32 : nullptr);
    } else {
      updvp_prcalc_f32_kernel<false><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(
          make_args(c), dp, phi, nullptr, nullptr, nullptr, f[MIBM_F_VX], f[MIBM_F_VY], f[MIBM_F_VZ], f[MIBM_F_PR],
          mean3f, mirror ? c->q32 : nullptr);
    } }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "updvp_prcalc_f32");
}

// a projection sweep that is not the last, fused with the next sweep's
// divergence residual (res): u, v, w move between the fields and vel1
// (from_vel1: from vel1 to the fields, else the other way); false when the
// scratch cannot be allocated (the caller takes the unfused sweep)
bool k_updvp_prcalc_divg_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool from_vel1,
                             float* res) {
  if (!c->vel1 && cudaMalloc(&c->vel1, 3 * c->g.cells * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    c->vel1 = nullptr;
    return false;
  }
  { MIBM_PROF(c, "updvp_prcalc_divg_f32");
    const float* mean3f = mean3 ? reinterpret_cast<const float*>(mean3 + 4) : nullptr;
    const size_t n = c->g.cells;
    double* const* f = c->df;
    const double* s[3] = {f[MIBM_F_VX], f[MIBM_F_VY], f[MIBM_F_VZ]};
    double* d[3] = {c->vel1, c->vel1 + n, c->vel1 + 2 * n};
    if (from_vel1)
      for (int q = 0; q < 3; ++q) { s[q] = d[q]; d[q] = f[MIBM_F_VX + q]; }
    if (c->g.dx1 == c->g.dx2 && c->g.dx1 == c->g.dx3)
      updvp_prcalc_divg_f32_kernel<true><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(
          make_args(c), dp, phi, s[0], s[1], s[2], d[0], d[1], d[2], f[MIBM_F_PR], mean3f, res);
    else
      updvp_prcalc_divg_f32_kernel<false><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(
          make_args(c), dp, phi, s[0], s[1], s[2], d[0], d[1], d[2], f[MIBM_F_PR], mean3f, res); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "updvp_prcalc_divg_f32");
  return true;
}

void k_prcalc_f32(Ctx* c, const StepParams* dp, const float* phi, bool mirror) {
  { MIBM_PROF(c, "prcalc_f32");
    prcalc_f32_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, phi, c->df[MIBM_F_PR],
                                                                      mirror ? c->q32 + 4 * c->g.cells : nullptr); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "prcalc_f32");
}

void k_divg_f32(Ctx* c, const StepParams* dp, float* res) {
  { MIBM_PROF(c, "divg_f32");
    if (c->g.dx1 == c->g.dx2 && c->g.dx1 == c->g.dx3)
      divg_f32_kernel<true><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, res);
    else
      divg_f32_kernel<false><<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, res); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "divg_f32");
}

void k_mirror_fields(Ctx* c) {
  { MIBM_PROF(c, "mirror");
    mirror_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g.cells, c->df[MIBM_F_VX], c->df[MIBM_F_VY],
                                                                  c->df[MIBM_F_VZ], c->df[MIBM_F_TEMP],
                                                                  c->df[MIBM_F_PR], c->q32); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "mirror");
}

void k_cast_d2f(Ctx* c, size_t n, const double* a, float* b) {
  cast_d2f_kernel<<<div_up(n, 256), 256, 0, c->stream>>>(n, a, b);
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "cast");
}

void k_cast_f2d(Ctx* c, size_t n, const float* a, double* b) {
  cast_f2d_kernel<<<div_up(n, 256), 256, 0, c->stream>>>(n, a, b);
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "cast");
}

// max |div u| over the owned cells (device), cleared first
void k_divmax(Ctx* c, unsigned long long* out) {
  cudaMemsetAsync(out, 0, sizeof(unsigned long long), c->stream);
  { MIBM_PROF(c, "divmax");
    divmax_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), out); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "divmax");
}

void k_updvp_prcalc(Ctx* c, const StepParams* dp, const double* mean3) {
  { MIBM_PROF(c, "updvp_prcalc");
    auto kern = equal_spacings(c->g) ? updvp_prcalc_kernel<true> : updvp_prcalc_kernel<false>;
    kern<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, c->df[MIBM_F_DPH], c->df[MIBM_F_VX],
                                                         c->df[MIBM_F_VY], c->df[MIBM_F_VZ], mean3,
                                                         c->df[MIBM_F_PR]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "updvp_prcalc");
}

void k_prcalc(Ctx* c, const StepParams* dp) {
  { MIBM_PROF(c, "prcalc"); prcalc_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), dp, c->df[MIBM_F_DPH], c->df[MIBM_F_PR]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "prcalc");
}

void k_add_field(Ctx* c, double* q, const double* r) {
  { MIBM_PROF(c, "add"); add_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g, q, r); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "add");
}

void k_interp_vof(Ctx* c) {
  { MIBM_PROF(c, "interp_vof"); interp_vof_kernel<<<cell_grid(c->g), kCellBlock, 0, c->stream>>>(make_args(c), c->df[MIBM_F_VOFX],
                                                                    c->df[MIBM_F_VOFY], c->df[MIBM_F_VOFZ]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "interp_vof");
}

void k_velforce_apply(Ctx* c, const double* mean3) {
  { MIBM_PROF(c, "velforce_apply"); velforce_apply_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(
      c->g, mean3, c->df[MIBM_F_FORXC], c->df[MIBM_F_FORYC], c->df[MIBM_F_FORZC], c->df[MIBM_F_VX], c->df[MIBM_F_VY],
      c->df[MIBM_F_VZ]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "velforce");
}

void k_tempforce_apply(Ctx* c) {
  { MIBM_PROF(c, "tempforce_apply"); tempforce_apply_kernel<<<div_up(c->g.cells, 256), 256, 0, c->stream>>>(c->g, c->df[MIBM_F_FORTEMP],
                                                                          c->df[MIBM_F_TEMP]); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "tempforce");
}

// blocks of the two max reductions: a few waves over the SMs, never more
// than the rows (the partials area of the reduction buffer holds one per row)
static unsigned reduce_blocks(const Grid& g) {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  size_t want = (size_t)std::max(1, sms) * 8;
  return (unsigned)std::min(want, (size_t)g.n2m * g.n3m);
}

// CFL maximum (cfl.f90:11-26) reduced on the device and copied to the
// pinned host slot `out`; read it after the stream has completed.
void k_cfl_async(Ctx* c, double* out) {
  unsigned nb = reduce_blocks(c->g);
  bool f32 = c->precision == 1 && c->q32_valid;
  { MIBM_PROF(c, "cfl");
    if (f32) cfl_kernel<float><<<nb, 256, 0, c->stream>>>(make_args(c), c->pad_vx, c->pad_vy, c->red + kRedPart, c->dflag + 2);
    else if (equal_spacings(c->g))
      cfl_kernel<double, true><<<nb, 256, 0, c->stream>>>(make_args(c), c->pad_vx, c->pad_vy, c->red + kRedPart,
                                                         c->dflag + 2);
    else cfl_kernel<double><<<nb, 256, 0, c->stream>>>(make_args(c), c->pad_vx, c->pad_vy, c->red + kRedPart, c->dflag + 2); }
  max_reduce_kernel<<<1, 1024, 0, c->stream>>>(c->red + kRedPart, nb, c->red + kRedOut);
  c->launches += 2;
  cudaMemcpyAsync(out, c->red + kRedOut, 8, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(c->hflag + 2, c->dflag + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
}

// After the stream has completed a k_cfl_async: the non-finite guard.
// Bit 1 of the same word: a bounded wait of the staged line solves ran out
// in the step before (tridiag.cu).
bool cfl_finite(Ctx* c) {
  const int f = c->hflag[2];
  if (!f) return true;
  c->hflag[2] = 0;
  cudaMemsetAsync(c->dflag + 2, 0, sizeof(int), c->stream);
  if (f & 2) fail(c, MIBM_ETIMEOUT, "line solve: a staged tile copy did not complete within its wait limit");
  else fail(c, MIBM_ENONFINITE, "cfl: non-finite velocity or temperature");
  return false;
}

// get_dt advective maximum for time step dt (cfl.f90:33-77), as k_cfl_async
void k_getdt_async(Ctx* c, double dt, double* out) {
  unsigned nb = reduce_blocks(c->g);
  bool f32 = c->precision == 1 && c->q32_valid;
  { MIBM_PROF(c, "getdt");
    if (f32) getdt_kernel<float><<<nb, 256, 0, c->stream>>>(make_args(c), dt, c->red + kRedPart + c->red_elems / 2);
    else if (equal_spacings(c->g))
      getdt_kernel<double, true><<<nb, 256, 0, c->stream>>>(make_args(c), dt, c->red + kRedPart + c->red_elems / 2);
    else getdt_kernel<double><<<nb, 256, 0, c->stream>>>(make_args(c), dt, c->red + kRedPart + c->red_elems / 2); }
  max_reduce_kernel<<<1, 1024, 0, c->stream>>>(c->red + kRedPart + c->red_elems / 2, nb, c->red + kRedOut + 1);
  c->launches += 2;
  cudaMemcpyAsync(out, c->red + kRedOut + 1, 8, cudaMemcpyDeviceToHost, c->stream);
}

// cfl.f90:448 starts the max at 1e-8
double cfl_value(double reduced) { return fmax(0.00000001, reduced); }

// viscous restriction 6/ren*dt*dx1**2 (cfl.f90:499), the same for every cell
double getdt_buffer(const Grid& g, double reduced, double dt, double ren) {
  return fmax(reduced, 6.0 / ren * dt * (g.dx1 * g.dx1));
}

double k_cfl(Ctx* c) {
  k_cfl_async(c, c->red_host);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "cfl")) return 0.0;
  cfl_finite(c);
  return cfl_value(c->red_host[0]);
}

double k_get_dt_buffer(Ctx* c, double dt, double ren) {
  k_getdt_async(c, dt, c->red_host + 1);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "get_dt")) return 0.0;
  return getdt_buffer(c->g, c->red_host[1], dt, ren);
}

}  // namespace mibm
