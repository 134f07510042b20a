// rigid.cu -- moving body: newton_euler, calc_rot_matrix, update_part_pos /
// update_xyz (RigidAuxRoutines.f90:1-306, 556-582, 818-868).
//
// The rigid-body state is a few dozen doubles, so the Newton-Euler update is
// one device thread: it stays in the stream between the structural loads
// and the geometry refresh of the same substep, and in a captured step graph,
// with no host round trip.  Its inputs are the loads summed on the device
// (lagr.cu), the geometry of the melted body (volume, centre of mass,
// inertia tensor) and the state of the previous substep; its outputs feed
// update_xyz (one thread per vertex / face) and the next substep's explicit
// terms (pos_CM, vel_CM, omega_c in the substep parameters).
//
// Single particle and no collisions: update_substepping (RigidAuxRoutines.
// f90:310-418) moves nothing unless `collision` flags a pair, which needs two
// particles.  Compiled without FMA contraction, like the oracle.
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace mibm {

// calc_rot_matrix (RigidAuxRoutines.f90:556-582): normalises q, AA column-major
__device__ void rot_matrix(double q[4], double AA[9]) {
  double norm = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int i = 0; i < 4; ++i) q[i] = q[i] / norm;
  AA[0] = q[0] * q[0] + q[1] * q[1] - q[2] * q[2] - q[3] * q[3];
  AA[3] = 2.0 * (q[1] * q[2] + q[0] * q[3]);
  AA[6] = 2.0 * (q[1] * q[3] - q[0] * q[2]);
  AA[1] = 2.0 * (q[1] * q[2] - q[0] * q[3]);
  AA[4] = q[0] * q[0] - q[1] * q[1] + q[2] * q[2] - q[3] * q[3];
  AA[7] = 2.0 * (q[2] * q[3] + q[0] * q[1]);
  AA[2] = 2.0 * (q[1] * q[3] + q[0] * q[2]);
  AA[5] = 2.0 * (q[2] * q[3] - q[0] * q[1]);
  AA[8] = q[0] * q[0] - q[1] * q[1] - q[2] * q[2] + q[3] * q[3];
}

// newton_euler + the periodic wrap of update_part_pos.  geom: [.., .., Volume,
// pos_CM(3), InertTensor(9)] of the body before the move.
//
// One warp.  On this part an FP64 instruction occupies a sub-partition's FP64
// unit for the same time whether one lane or all 32 are active, so the
// independent entries of each phase (the 3 components, the 4 quaternion
// entries, the 9 matrix entries, sine beside cosine) are computed by as many
// lanes at once; each entry keeps the operation sequence of the one-thread
// version (no FMA contraction), so the values are the same.  The LU inverse
// stays on lane 0.  Phases meet in shared memory after a __syncwarp().
__global__ void newton_euler_kernel(const StepParams* __restrict__ pp, const double* __restrict__ geom,
                                    double dens_ratio, double xlen, double ylen, double zlen, RigidDev* r,
                                    int* __restrict__ flag) {
  if (blockIdx.x != 0) return;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x;
  __shared__ double I[9], I_LHS[9], I_inv[9], AA[9], buf[9], om1[3], vel1[3], rhs[3], om[3], ob[3], quat[4];
  __shared__ double sc[4];          // magOM, angle, ch, sh
  __shared__ double qn_s;
  const double al = pp->al, ga = pp->ga, ro = pp->ro, dt = pp->dt;
  const double* prn = r->load; const double* tau = r->load + 3;
  const double* rprn = r->load + 6; const double* rtau = r->load + 9;
  const double* prn1 = r->load1; const double* tau1 = r->load1 + 3;
  const double* rprn1 = r->load1 + 6; const double* rtau1 = r->load1 + 9;
  if (lane < 9) { I[lane] = geom[6 + lane]; I_LHS[lane] = geom[6 + lane]; }
  if (lane < 3) { vel1[lane] = r->vel[lane]; om1[lane] = r->om[lane]; }
  if (lane < 4) quat[lane] = 0.0;
  __syncwarp();
  // translation, RigidAuxRoutines.f90:218-225 (lane i: component i)
  double vel = 0.0, pos = 0.0;
  if (lane < 3) {
    const double e_z = lane == 2 ? -1.0 : 0.0;
    const double pre_fac = 1.0 / geom[2] / dens_ratio;
    vel = vel1[lane] + ga * dt * pre_fac * (-prn[lane] + tau[lane]) + ro * dt * pre_fac * (-prn1[lane] + tau1[lane]) +
          al * dt * (1.0 - (1.0 / dens_ratio)) * e_z;
    pos = geom[3 + lane] + 0.5 * al * dt * (vel + vel1[lane]);
  }
  // rotation: iterative inertia-tensor update, RigidAuxRoutines.f90:243-296
  const double tolerance = 1.e-15;
  const int max_iter = 10000;
  double Iresidual = 1.0;
  int n_iter = 1;
  while (n_iter <= max_iter && Iresidual > tolerance) {
    // the inverse of I_LHS (dgetrf + dgetri in the reference) by cofactors,
    // entry (i, j) on lane i + 3j: a dependent FP64 chain of one cofactor, a
    // 3-term determinant and one reciprocal instead of an LU's six
    // reciprocals and eliminations on one thread; the same matrix up to
    // rounding.  Singular (flag 2) when the determinant is exactly zero.
    {
      double cof = 0.0;
      if (lane < 9) {
        const int i = lane % 3, j = lane / 3;
        const int r0 = (j + 1) % 3, r1 = (j + 2) % 3, c0 = (i + 1) % 3, c1 = (i + 2) % 3;
        cof = I_LHS[r0 + 3 * c0] * I_LHS[r1 + 3 * c1] - I_LHS[r0 + 3 * c1] * I_LHS[r1 + 3 * c0];
      }
      const double c00 = __shfl_sync(FULL, cof, 0), c01 = __shfl_sync(FULL, cof, 1), c02 = __shfl_sync(FULL, cof, 2);
      const double det = I_LHS[0] * c00 + I_LHS[3] * c01 + I_LHS[6] * c02;
      if (det == 0.0) { if (lane == 0) atomicOr(flag, 2); return; }
      const double rdet = 1.0 / det;
      if (lane < 9) I_inv[lane] = cof * rdet;
    }
    __syncwarp();
    if (lane < 3) {
      double m = 0.0;
      for (int j = 0; j < 3; ++j) m += I[lane + 3 * j] * om1[j];
      rhs[lane] = m + ga * dt * (-rprn[lane] + rtau[lane]) + ro * dt * (-rprn1[lane] + rtau1[lane]);
    }
    __syncwarp();
    if (lane < 3) {
      double m = 0.0;
      for (int j = 0; j < 3; ++j) m += I_inv[lane + 3 * j] * rhs[j];
      om[lane] = m;
      ob[lane] = 0.5 * (m + om1[lane]);
    }
    __syncwarp();
    if (lane == 0) {
      const double magOM = sqrt(ob[0] * ob[0] + ob[1] * ob[1] + ob[2] * ob[2]);
      sc[0] = magOM;
      sc[1] = magOM * al * dt;
    }
    __syncwarp();
    const double magOM = sc[0], angle = sc[1];
    if (lane < 3) ob[lane] = magOM < tolerance ? 0.0 : ob[lane] / magOM;
    if (lane == 3) sincos(0.5 * angle, &sc[3], &sc[2]);
    __syncwarp();
    if (lane < 4) quat[lane] = lane == 0 ? sc[2] : sc[3] * ob[lane - 1];
    __syncwarp();
    // two normalisations, as the reference: quat / |quat|, then calc_rot_matrix's own
    for (int pass = 0; pass < 2; ++pass) {
      if (lane == 0) qn_s = sqrt(quat[0] * quat[0] + quat[1] * quat[1] + quat[2] * quat[2] + quat[3] * quat[3]);
      __syncwarp();
      const double qn = qn_s;
      __syncwarp();
      if (lane < 4) quat[lane] = quat[lane] / qn;
      __syncwarp();
    }
    if (lane < 9) {
      const double q0 = quat[0], q1 = quat[1], q2 = quat[2], q3 = quat[3];
      double v;
      switch (lane) {
        case 0: v = q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3; break;
        case 3: v = 2.0 * (q1 * q2 + q0 * q3); break;
        case 6: v = 2.0 * (q1 * q3 - q0 * q2); break;
        case 1: v = 2.0 * (q1 * q2 - q0 * q3); break;
        case 4: v = q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3; break;
        case 7: v = 2.0 * (q2 * q3 + q0 * q1); break;
        case 2: v = 2.0 * (q1 * q3 + q0 * q2); break;
        case 5: v = 2.0 * (q2 * q3 - q0 * q1); break;
        default: v = q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3; break;
      }
      AA[lane] = v;
    }
    __syncwarp();
    const int i = lane % 3, j = lane / 3;
    double prev = 0.0;
    if (lane < 9) {
      prev = I_LHS[lane];
      double m = 0.0;
      for (int k = 0; k < 3; ++k) m += I[i + 3 * k] * AA[j + 3 * k];
      buf[lane] = m;
    }
    __syncwarp();
    double d = 0.0;
    if (lane < 9) {        // each lane reads and writes only its own entry of I_LHS here
      double m = 0.0;
      for (int k = 0; k < 3; ++k) m += AA[i + 3 * k] * buf[k + 3 * j];
      d = fabs(m - prev);
      I_LHS[lane] = m;
    }
    // residual: the maximum of the nine |changes| (fmax is exact, so the order is immaterial)
    for (int off = 16; off > 0; off >>= 1) d = fmax(d, __shfl_xor_sync(FULL, d, off));
    Iresidual = d;
    ++n_iter;
    __syncwarp();
  }
  // periodicity corrections, RigidAuxRoutines.f90:40-51
  if (lane < 3) {
    const double L = lane == 0 ? xlen : (lane == 1 ? ylen : zlen);
    if (pos < 0.) pos = pos + L;
    if (pos > L) pos = pos - L;
    r->vel[lane] = vel;
    r->om[lane] = om[lane];
    r->xf[9 + lane] = pos;
    r->xf[12 + lane] = geom[3 + lane];
  }
  // update_xyz re-derives AA from the stored quaternion, which that call
  // normalises once more in place
  if (lane == 0) {
    double q[4] = {quat[0], quat[1], quat[2], quat[3]}, A[9];
    rot_matrix(q, A);
    for (int k = 0; k < 4; ++k) r->quat[k] = q[k];
    for (int k = 0; k < 9; ++k) { r->inert[k] = I_LHS[k]; r->xf[k] = A[k]; }
    r->iters = n_iter - 1;
  }
}

// update_xyz (RigidAuxRoutines.f90:818-868): vertices turned by AA^T about
// the old centre and moved to the new one; face velocities vel_CM +
// omega x (centroid - old centre) from the centroids before the move.
__global__ void update_xyz_kernel(int nv, int nf, const int* __restrict__ ghostv, const int* __restrict__ ghostf,
                                  const RigidDev* __restrict__ r, double* __restrict__ x,
                                  const double* __restrict__ bar, double* __restrict__ vel_tri) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double* AA = r->xf;
  const double* pos = r->xf + 9;
  const double* pos1 = r->xf + 12;
  if (t < nv && !ghostv[t]) {
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = x[3 * t + k] - pos1[k];
    for (int q = 0; q < 3; ++q) {
      double m = 0.0;
      for (int k = 0; k < 3; ++k) m += AA[k + 3 * q] * d[k];
      x[3 * t + q] = m + pos[q];
    }
  }
  if (t < nf && !ghostf[t]) {
    double ds[3];
    for (int k = 0; k < 3; ++k) ds[k] = bar[3 * t + k] - pos1[k];
    const double* om = r->om;
    double c0 = om[1] * ds[2] - ds[1] * om[2];
    double c1 = om[2] * ds[0] - ds[2] * om[0];
    double c2 = om[0] * ds[1] - ds[0] * om[1];
    vel_tri[3 * t] = r->vel[0] + c0;
    vel_tri[3 * t + 1] = r->vel[1] + c1;
    vel_tri[3 * t + 2] = r->vel[2] + c2;
  }
}

// calc_centroids_from_vert (triaux.f90:308-323)
__global__ void centroid_kernel(int nf, const int* __restrict__ vof, const int* __restrict__ ghost,
                                const double* __restrict__ x, double* __restrict__ bar) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf || ghost[t]) return;
  int a = vof[3 * t] - 1, b = vof[3 * t + 1] - 1, d = vof[3 * t + 2] - 1;
  for (int k = 0; k < 3; ++k) bar[3 * t + k] = (x[3 * a + k] + x[3 * b + k] + x[3 * d + k]) / 3.0;
}

// After the geometry refresh: the inertia tensor of the moved body
// (calc_rigidBody_params of the primitive geometry, particle.f90:189) and
// the centre of mass / velocities the next substep's explicit terms read.
__global__ void publish_kernel(const double* __restrict__ geom, RigidDev* r, StepParams* next) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int q = 0; q < 9; ++q) r->inert[q] = geom[6 + q];
  if (next) {
    for (int d = 0; d < 3; ++d) {
      next->pos[d] = geom[3 + d];
      next->vel[d] = r->vel[d];
      next->om[d] = r->om[d];
    }
  }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
bool rigid_ensure(Ctx* c) {
  if (c->drigid) return true;
  if (!cuda_ok(c, cudaMalloc(&c->drigid, sizeof(RigidDev)), "rigid")) return false;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->hrigid_in, sizeof(RigidDev)), "rigid")) return false;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->hrigid_out, sizeof(RigidDev)), "rigid")) return false;
  memset(c->hrigid_in, 0, sizeof(RigidDev));
  memset(c->hrigid_out, 0, sizeof(RigidDev));
  return true;
}

static const int kLoadIds[4] = {MIBM_S_INT_PRN_DA, MIBM_S_INT_TAU_DA, MIBM_S_INT_R_X_PRN_DA, MIBM_S_INT_R_X_TAU_DA};
static const int kLoad1Ids[4] = {MIBM_S_INT_PRN_DA_M1, MIBM_S_INT_TAU_DA_M1, MIBM_S_INT_R_X_PRN_DA_M1,
                                 MIBM_S_INT_R_X_TAU_DA_M1};
static const int kAccIds[4] = {MIBM_S_FP, MIBM_S_FTAU, MIBM_S_TORQ_P, MIBM_S_TORQ_TAU};

// registered module state -> h.  geom_from_scalars: Volume, pos_CM and
// InertTensor as the drop-in update_part_pos_ reads them.
void rigid_pack(Ctx* c, RigidDev* h, bool geom_from_scalars) {
  for (int d = 0; d < 3; ++d) { h->vel[d] = c->hs[MIBM_S_VEL_CM][d]; h->om[d] = c->hs[MIBM_S_OMEGA_C][d]; }
  for (int q = 0; q < 4; ++q) h->quat[q] = c->hs[MIBM_S_QUAT][q];
  for (int b = 0; b < 4; ++b)
    for (int d = 0; d < 3; ++d) {
      h->load[3 * b + d] = c->hs[kLoadIds[b]][d];
      h->load1[3 * b + d] = c->hs[kLoad1Ids[b]][d];
      h->acc[3 * b + d] = c->hs[kAccIds[b]][d];
    }
  for (int q = 0; q < 9; ++q) h->inert[q] = c->hs[MIBM_S_INERT_TENSOR][q];
  if (geom_from_scalars) {
    for (int q = 0; q < 16; ++q) h->geom_in[q] = 0.0;
    h->geom_in[2] = c->S(MIBM_S_VOLUME);
    for (int d = 0; d < 3; ++d) h->geom_in[3 + d] = c->hs[MIBM_S_POS_CM][d];
    for (int q = 0; q < 9; ++q) h->geom_in[6 + q] = c->hs[MIBM_S_INERT_TENSOR][q];
  }
}

// h -> registered module state.  pos_from_motion: pos_CM is the
// Newton-Euler result (the drop-in update_part_pos_); otherwise the caller
// sets it from the refreshed geometry.
void rigid_unpack(Ctx* c, const RigidDev* h, bool pos_from_motion) {
  for (int d = 0; d < 3; ++d) { c->hs[MIBM_S_VEL_CM][d] = h->vel[d]; c->hs[MIBM_S_OMEGA_C][d] = h->om[d]; }
  for (int q = 0; q < 4; ++q) c->hs[MIBM_S_QUAT][q] = h->quat[q];
  for (int b = 0; b < 4; ++b)
    for (int d = 0; d < 3; ++d) {
      c->hs[kLoadIds[b]][d] = h->load[3 * b + d];
      c->hs[kLoad1Ids[b]][d] = h->load1[3 * b + d];
      c->hs[kAccIds[b]][d] = h->acc[3 * b + d];
    }
  for (int q = 0; q < 9; ++q) c->hs[MIBM_S_INERT_TENSOR][q] = h->inert[q];
  if (pos_from_motion)
    for (int d = 0; d < 3; ++d) c->hs[MIBM_S_POS_CM][d] = h->xf[9 + d];
}

// stream-ordered copies through the pinned blocks (captured into step graphs)
void rigid_upload(Ctx* c) {
  cudaMemcpyAsync(c->drigid, c->hrigid_in, sizeof(RigidDev), cudaMemcpyHostToDevice, c->stream);
}
void rigid_download(Ctx* c) {
  cudaMemcpyAsync(c->hrigid_out, c->drigid, sizeof(RigidDev), cudaMemcpyDeviceToHost, c->stream);
}

void k_newton_euler(Ctx* c, const StepParams* dp, const double* geom) {
  { MIBM_PROF(c, "newton_euler");
    newton_euler_kernel<<<1, 32, 0, c->stream>>>(dp, geom, c->S(MIBM_S_DENS_RATIO), c->g.xlen, c->g.ylen,
                                                 c->g.zlen, c->drigid, c->dflag); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "newton_euler");
}

void k_update_xyz(Ctx* c, bool centroids) {
  int n = std::max(c->maxnv, c->maxnf);
  if (n == 0) return;
  { MIBM_PROF(c, "update_xyz");
    update_xyz_kernel<<<div_up(n, 128), 128, 0, c->stream>>>(
        c->maxnv, c->maxnf, (const int*)c->dm[MIBM_M_GHOST_VERT], (const int*)c->dm[MIBM_M_GHOST_FACE], c->drigid,
        (double*)c->dm[MIBM_M_XYZV], (const double*)c->dm[MIBM_M_TRI_BAR], (double*)c->dm[MIBM_M_VEL_TRI]); }
  ++c->launches;
  if (centroids && c->maxnf > 0) {
    MIBM_PROF(c, "centroids");
    centroid_kernel<<<div_up(c->maxnf, 128), 128, 0, c->stream>>>(
        c->maxnf, (const int*)c->dm[MIBM_M_VERT_OF_FACE], (const int*)c->dm[MIBM_M_GHOST_FACE],
        (const double*)c->dm[MIBM_M_XYZV], (double*)c->dm[MIBM_M_TRI_BAR]);
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, "update_xyz");
}

void k_rigid_publish(Ctx* c, const double* geom, StepParams* next) {
  { MIBM_PROF(c, "rigid_publish");
    publish_kernel<<<1, 32, 0, c->stream>>>(geom, c->drigid, next); }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, "rigid_publish");
}

void rigid_free(Ctx* c) {
  cudaFree(c->drigid);
  if (c->hrigid_in) cudaFreeHost(c->hrigid_in);
  if (c->hrigid_out) cudaFreeHost(c->hrigid_out);
  c->drigid = nullptr; c->hrigid_in = nullptr; c->hrigid_out = nullptr;
}

}  // namespace mibm
