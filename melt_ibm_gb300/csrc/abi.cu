// abi.cu -- drop-in entry points of include/mibm.h and the fused RK3 step.
//
// Every routine keeps the reference's name, argument list and side effects on
// the registered arrays (with the device copy authoritative until
// mibm_sync_to_host_).  `tschem_` replays tsch.f90:32-97 with two fusions
// that leave the results unchanged up to rounding:
//   * the explicit term of each component is computed inside its RHS kernel
//     (hdnl* + invtr* RHS), so dq/dph/qcap/htemp are not materialised;
//   * the four RHS fields are separate buffers, so all explicit terms are
//     formed from the substep's initial fields exactly as tsch.f90:49-57
//     orders them (every invtr only advances its own component).
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace mibm {

void tri_free(Ctx* c);
void fft_free(Ctx* c);

// Copy the current host scalars to device slot `slot` (stream ordered; the
// source is pageable, so the host may reuse it as soon as the call returns).
static const StepParams* push_params(Ctx* c, int slot) {
  StepParams p = host_params(c);
  cudaMemcpyAsync(c->dparams + slot, &p, sizeof(StepParams), cudaMemcpyHostToDevice, c->stream);
  return c->dparams + slot;
}

static int field_of_plane1(Ctx* c, const double* q) {
  size_t n1 = c->g.n1m + 1;
  for (int id = 0; id < MIBM_NFIELDS; ++id) {
    int ny, klo, nk;
    field_host_shape(c, id, ny, klo, nk);
    const double* p1 = c->hf[id] + (klo == 0 ? n1 * (size_t)ny : 0);
    if (p1 == q) return id;
  }
  return -1;
}

static void invtr(Ctx* c, int which) {
  const StepParams* dp = push_params(c, 3);
  double* rhs = c->df[MIBM_F_RHS];
  k_invtr_rhs(c, which, dp, rhs);
  static const int fid[4] = {MIBM_F_VX, MIBM_F_VY, MIBM_F_VZ, MIBM_F_TEMP};
  double al = c->S(MIBM_S_AL), dt = c->S(MIBM_S_DT);
  double b1, b2, b3;
  if (which < 3) {
    double beta = c->S(MIBM_S_BETA);
    b1 = beta * al * c->g.dx1q; b2 = beta * al * c->g.dx2q; b3 = beta * al * c->g.dx3q;
  } else {
    double pec = c->S(MIBM_S_PEC);
    b1 = dt / pec * 0.5 * al * c->g.dx1q; b2 = dt / pec * 0.5 * al * c->g.dx2q; b3 = dt / pec * 0.5 * al * c->g.dx3q;
  }
  k_solve_x(c, rhs, b1);
  k_solve_y(c, rhs, b2);
  k_solve_z(c, rhs, b3, c->df[fid[which]]);
}

static const int kRuFields[4] = {MIBM_F_RU1, MIBM_F_RU2, MIBM_F_RU3, MIBM_F_RUT};

static bool ensure_f32(Ctx* c) {
  const Grid& g = c->g;
  if (!c->ru32) {
    if (!cuda_ok(c, cudaMalloc(&c->ru32, 4 * g.cells * sizeof(float)), "ru32")) return false;
    if (!cuda_ok(c, cudaMalloc(&c->rhs32, 4 * g.cells * sizeof(float)), "rhs32")) return false;
    if (!cuda_ok(c, cudaMalloc(&c->phi32, g.cells * sizeof(float)), "phi32")) return false;
    if (!cuda_ok(c, cudaMalloc(&c->res32, g.cells * sizeof(float)), "res32")) return false;
    if (!cuda_ok(c, cudaMalloc(&c->q32, 5 * g.cells * sizeof(float)), "q32")) return false;
    if (!cuda_ok(c, cudaMalloc(&c->prod32, 6 * g.cells * sizeof(float)), "prod32")) return false;
    for (int q = 0; q < 4; ++q) k_cast_d2f(c, g.cells, c->df[kRuFields[q]], c->ru32 + (size_t)q * g.cells);
    c->q32_valid = false;
  }
  if (!c->q32_valid) {
    k_mirror_fields(c);
    c->q32_valid = true;
  }
  return MIBM_LAUNCH_CHECK(c, "precision buffers");
}

void precision_before_download(Ctx* c, unsigned long long mask) {
  if (c->precision != 1 || !c->ru32) return;
  for (int q = 0; q < 4; ++q)
    if (mask & (1ull << kRuFields[q])) k_cast_f2d(c, c->g.cells, c->ru32 + (size_t)q * c->g.cells, c->df[kRuFields[q]]);
}

void precision_after_upload(Ctx* c, unsigned long long mask) {
  static const int prog[5] = {MIBM_F_VX, MIBM_F_VY, MIBM_F_VZ, MIBM_F_TEMP, MIBM_F_PR};
  for (int q = 0; q < 5; ++q)
    if (mask & (1ull << prog[q])) c->q32_valid = false;
  if (c->precision != 1 || !c->ru32) return;
  for (int q = 0; q < 4; ++q)
    if (mask & (1ull << kRuFields[q])) k_cast_d2f(c, c->g.cells, c->df[kRuFields[q]], c->ru32 + (size_t)q * c->g.cells);
}

static const double kGam[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0};     // papero.f90:118-137
// the body moves (particle.f90:108-129): its state rides with the step
static bool moving_body(Ctx* c) {
  return c->I(MIBM_I_IMLSFOR) == 1 && c->I(MIBM_I_IMLSSTR) == 1 && c->maxnf > 0;
}
static const double kRom[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
static const int kStepFid[4] = {MIBM_F_VX, MIBM_F_VY, MIBM_F_VZ, MIBM_F_TEMP};

// tsch.f90:18-97 in three phases.  step_prepare (host): beta, the factor
// tables of the 18 line solves (invtr*.f90 betadx) and the three substeps'
// scalars, written to pinned buffers; buffers the form needs.  step_enqueue
// (device, no host synchronisation): every copy and kernel of the step --
// this is what a step graph captures.  step_finish (host): wait, then the
// MLS / geometry checks.
static bool step_prepare(Ctx* c) {
  const Grid& g = c->g;
  *c->hs[MIBM_S_BETA] = c->S(MIBM_S_DT) / c->S(MIBM_S_REN) * 0.5;
  double bd[3][2][3];
  double dt = c->S(MIBM_S_DT), beta = c->S(MIBM_S_BETA), pec = c->S(MIBM_S_PEC);
  const double dq[3] = {g.dx1q, g.dx2q, g.dx3q};
  for (int ns = 0; ns < 3; ++ns) {
    double al = kGam[ns] + kRom[ns];
    for (int d = 0; d < 3; ++d) {
      bd[ns][0][d] = beta * al * dq[d];
      bd[ns][1][d] = dt / pec * 0.5 * al * dq[d];
    }
  }
  bool f32 = c->precision == 1;
  if (f32) {
    if (!ensure_f32(c)) return false;
  } else {
    c->q32_valid = false;
    if (!c->rhs4 && !cuda_ok(c, cudaMalloc(&c->rhs4, 4 * g.cells * sizeof(double)), "rhs4")) return false;
    if (!c->prod && !cuda_ok(c, cudaMalloc(&c->prod, 6 * g.cells * sizeof(double)), "advection products"))
      return false;
  }
  if (!tri_step_fill(c, bd, f32)) return false;
  if (!fft_prepare(c, false) || (f32 && !fft_prepare(c, true))) return false;
  if (moving_body(c)) {
    if (!rigid_ensure(c)) return false;
    rigid_pack(c, c->hrigid_in, false);
  }
  for (int ns = 0; ns < 3; ++ns) {
    *c->hs[MIBM_S_AL] = kGam[ns] + kRom[ns];
    *c->hs[MIBM_S_GA] = kGam[ns];
    *c->hs[MIBM_S_RO] = kRom[ns];
    c->hparams[ns] = host_params(c);
  }
  c->hparams[0].force_plan = lagr_take_plan_request(c);
  return c->status == MIBM_OK;
}

// FP64 form: the temperature's line solves run on their own stream beside
// the velocity's (they read and write only the temperature's RHS and T,
// which the velocity solves do not touch), so that each kernel's last wave is
// filled by the other's blocks; joined before the forcing, which reads T.
// Not while kernels are timed one by one, and not in the precision form,
// whose staged z solves hold every SM (measured: 30.19 -> 30.10 ms per 256^3
// FP64 step, 4.43 -> 4.35 ms at 128^3; no gain in the precision form).
static bool tsolve_fork(Ctx* c) { return c->tsolve && !c->profiling && c->precision == 0; }

static void tsolve_begin(Ctx* c) {
  if (!tsolve_fork(c)) return;
  cudaEventRecord(c->ev_sfork, c->stream);
  cudaStreamWaitEvent(c->tsolve, c->ev_sfork, 0);
  std::swap(c->stream, c->tsolve);
}

static void tsolve_end(Ctx* c) {
  if (!tsolve_fork(c)) return;
  std::swap(c->stream, c->tsolve);
  cudaEventRecord(c->ev_sjoin, c->tsolve);
}

static void tsolve_join(Ctx* c) {
  if (tsolve_fork(c)) cudaStreamWaitEvent(c->stream, c->ev_sjoin, 0);
}

// Precision form: FP32 explicit terms, RHS, line solves and FFTs; u, v, w,
// T, p stay FP64 and every FP32 kernel reads their FP32 mirrors.  The
// projection is repeated `nproj` times, each on the divergence residual of
// the FP64 velocity (iterative refinement), so the final divergence is at
// FP64 round-off.  MLS inversions, the Stefan front and the geometry stay
// FP64.  Mirrors: T is written by the z solve and the temperature forcing,
// u, v, w by the last velocity update, p by the last pressure update of the
// substep.
static void step_enqueue_f32(Ctx* c) {
  const Grid& g = c->g;
  int tlen = 0;
  const float* tf = nullptr;
  if (!tri_step_enqueue(c, true, &tlen, &tf)) return;
  float* t_mirror = c->q32 + 3 * g.cells;
  for (int ns = 0; ns < 3; ++ns) {
    const StepParams* dp = c->dparams + ns;
    lagr_join_geom(c);            // the rest of the side branch is waited for before the forcing
    if (!c->prologue_done) { lagr_join(c); lagr_substep_prologue(c, ns); }
    c->prologue_done = false;
    k_fused_rhs_f32(c, dp, c->ru32, c->rhs32);
    {
      // T on its own stream, then u, v, w: one launch per direction (they
      // share the velocity tables)
      tsolve_begin(c);
      const float* Tt = tf + (size_t)((ns * 2 + 1) * 3) * tlen;
      float* r = c->rhs32 + 3 * g.cells;
      double* qt[1] = {c->df[kStepFid[3]]};
      k_solve_x_f32(c, r, Tt, 1);
      k_solve_y_f32(c, r, Tt + tlen, 1);
      k_solve_z_f32(c, r, Tt + 2 * tlen, qt, 1, t_mirror);
      tsolve_end(c);
      const float* Tv = tf + (size_t)((ns * 2 + 0) * 3) * tlen;
      double* qv[3] = {c->df[kStepFid[0]], c->df[kStepFid[1]], c->df[kStepFid[2]]};
      k_solve_x_f32(c, c->rhs32, Tv, 3);
      k_solve_y_f32(c, c->rhs32, Tv + tlen, 3);
      k_solve_z_f32(c, c->rhs32, Tv + 2 * tlen, qv, 3, nullptr);
      lagr_loads_early(c, dp);                  // u, v, w solved: loads beside the forcing's preparation
      tsolve_join(c);
    }
    const double* mean3 = lagr_particle_fused(c, dp, c->q32, ns < 2 ? c->dparams + ns + 1 : nullptr, ns + 1);
    if (c->status != MIBM_OK) return;
    // one-pass form: each sweep but the last also forms the next sweep's
    // residual, with u, v, w moved between the fields and vel1 (the same bits)
    bool in_vel1 = false, have_res = false;
    for (int it = 0; it < c->nproj; ++it) {
      bool last = it + 1 == c->nproj;
      if (!have_res) k_divg_f32(c, dp, c->res32);      // FP64 residual, rounded once
      have_res = false;
      k_phcalc_f32(c, c->res32, c->phi32);             // FP32 Poisson solve
      if (c->fused_uvw) {
        const double* m = it == 0 ? mean3 : nullptr;
        if (!last && k_updvp_prcalc_divg_f32(c, dp, c->phi32, m, in_vel1, c->res32)) {
          in_vel1 = !in_vel1;
          have_res = true;
        } else {
          k_updvp_prcalc_f32(c, dp, c->phi32, m, last, in_vel1);
          in_vel1 = false;
        }
      } else {
        k_updvp_f32(c, dp, c->phi32, it == 0 ? mean3 : nullptr, last);
        k_prcalc_f32(c, dp, c->phi32, last);
      }
    }
    if (c->status != MIBM_OK) return;
  }
}

static void step_enqueue_f64(Ctx* c) {
  const Grid& g = c->g;
  int tlen = 0;
  const double* tables = tri_step_enqueue(c, false, &tlen, nullptr);
  if (!tables) return;
  for (int ns = 0; ns < 3; ++ns) {
    const StepParams* dp = c->dparams + ns;
    lagr_join_geom(c);            // the rest of the side branch is waited for before the forcing
    if (!c->prologue_done) { lagr_join(c); lagr_substep_prologue(c, ns); }
    c->prologue_done = false;
    k_fused_rhs(c, dp);
    {
      // T on its own stream, then u, v, w: one launch per direction (they
      // share the velocity tables)
      tsolve_begin(c);
      const double* Tt = tables + (size_t)((ns * 2 + 1) * 3) * tlen;
      double* r = c->rhs4 + 3 * g.cells;
      double* qt[1] = {c->df[kStepFid[3]]};
      k_solve_x_T(c, r, Tt, 1);
      k_solve_y_T(c, r, Tt + tlen, 1);
      k_solve_z_T(c, r, Tt + 2 * tlen, qt, 1, 0);
      tsolve_end(c);
      const double* Tv = tables + (size_t)((ns * 2 + 0) * 3) * tlen;
      double* qv[3] = {c->df[kStepFid[0]], c->df[kStepFid[1]], c->df[kStepFid[2]]};
      k_solve_x_T(c, c->rhs4, Tv, 3);
      k_solve_y_T(c, c->rhs4, Tv + tlen, 3);
      k_solve_z_T(c, c->rhs4, Tv + 2 * tlen, qv, 3, 0);
      lagr_loads_early(c, dp);                  // u, v, w solved: loads beside the forcing's preparation
      tsolve_join(c);
    }
    const double* mean3 = lagr_particle_fused(c, dp, nullptr, ns < 2 ? c->dparams + ns + 1 : nullptr, ns + 1);
    if (c->status != MIBM_OK) return;
    k_divg(c, dp);
    k_phcalc(c);
    k_updvp_prcalc(c, dp, mean3);
    if (c->status != MIBM_OK) return;
  }
}

// device address of vel_CM at the end of a step: the moving body's state,
// else the value the step was given
static const double* step_vel_cm(Ctx* c) {
  if (moving_body(c)) return (const double*)((const char*)c->drigid + offsetof(RigidDev, vel));
  return (const double*)((const char*)(c->dparams + 2) + offsetof(StepParams, vel));
}

static void step_enqueue(Ctx* c) {
  cudaMemcpyAsync(c->dparams, c->hparams, 3 * sizeof(StepParams), cudaMemcpyHostToDevice, c->stream);
  if (moving_body(c)) rigid_upload(c);
  if (c->precision == 1) step_enqueue_f32(c);
  else step_enqueue_f64(c);
  lagr_join(c);
  if (c->status == MIBM_OK && c->diag_on) diag_enqueue(c, step_vel_cm(c));
  if (c->status == MIBM_OK) lagr_step_readback(c);
}

static uint64_t step_key(Ctx* c);

static void step_finish(Ctx* c) {
  lagr_join(c);
  c->early_prologue = false;
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "tschem")) return;
  if (c->status != MIBM_OK) return;
  lagr_step_host_finish(c);
  if (c->diag_on && c->status == MIBM_OK) diag_finish(c);
  if (c->precision == 1 && c->status == MIBM_OK) c->q32_valid = true;
  ++c->steps_done;
  // the last substep enqueued the next step's substep-0 geometry work
  if (c->status == MIBM_OK && lagr_fork_enabled(c)) {
    c->early_prologue = true;
    c->early_gen = c->geom_gen;
    c->early_key = step_key(c);
  }
}

// Substep 0's geometry-only work (tagging, cage indices, MLS weights,
// scatter plan): the previous step enqueued it at the end of its last
// substep, on the side stream, unless a host call since may have changed its
// inputs (geom_gen) or the step's configuration changed (step key); then it
// runs here, ahead of the step and outside any step graph, after the
// parameter blocks (substep 0's carries the host's plan rebuild request).
static void step_head(Ctx* c) {
  const bool early = c->early_prologue && c->early_gen == c->geom_gen && c->early_key == step_key(c);
  c->early_prologue = false;
  if (!early) {
    cudaMemcpyAsync(c->dparams, c->hparams, 3 * sizeof(StepParams), cudaMemcpyHostToDevice, c->stream);
    lagr_substep_prologue(c, 0);
  }
  c->prologue_done = true;
}

// Everything a step reads by value from the host besides the per-step
// scalars (dt, al, ga, ro, beta, the rigid-body state: those go through the
// pinned parameter and rigid-body blocks): the integer flags, the constant
// scalars passed to kernels, the form, and the Lagrangian launch sequence
// generation.
static uint64_t step_key(Ctx* c) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) { h ^= v; h *= 1099511628211ull; };
  for (int i = 0; i < MIBM_NINTS; ++i)
    if (i != MIBM_I_NTIME) mix((uint64_t)(uint32_t)c->I(i));
  static const int per_step[] = {MIBM_S_DT, MIBM_S_AL, MIBM_S_GA, MIBM_S_RO, MIBM_S_BETA, MIBM_S_TIME,
                                 MIBM_S_CFLM, MIBM_S_VOLUME, MIBM_S_SURFACE, MIBM_S_POS_CM, MIBM_S_VEL_CM,
                                 MIBM_S_OMEGA_C, MIBM_S_DTMAX, MIBM_S_QUAT, MIBM_S_INERT_TENSOR,
                                 MIBM_S_INT_PRN_DA, MIBM_S_INT_TAU_DA, MIBM_S_INT_R_X_PRN_DA,
                                 MIBM_S_INT_R_X_TAU_DA, MIBM_S_INT_PRN_DA_M1, MIBM_S_INT_TAU_DA_M1,
                                 MIBM_S_INT_R_X_PRN_DA_M1, MIBM_S_INT_R_X_TAU_DA_M1, MIBM_S_FP, MIBM_S_FTAU,
                                 MIBM_S_TORQ_P, MIBM_S_TORQ_TAU};
  for (int i = 0; i < MIBM_NSCALARS; ++i) {
    bool skip = false;
    for (int p : per_step) skip |= (p == i);
    if (skip) continue;
    uint64_t b;
    double v = c->S(i);
    memcpy(&b, &v, 8);
    mix(b);
  }
  mix((uint64_t)c->precision); mix((uint64_t)c->nproj); mix(c->lag_gen); mix(c->q32 ? 1 : 0);
  mix(c->tune_gen); mix(c->diag_on ? 1 : 0);
  return h;
}

// A step becomes a graph from its second call, unless kernels are being
// profiled one by one or the step may stop for the host's remesher.
static bool graphs_allowed(Ctx* c) {
  return c->use_graph && c->steps_done >= 1 && !c->profiling && !lagr_remesh_active(c);
}

static void drop_graph(Ctx* c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
  c->graph_key = 0;
}

// Capture step_enqueue into a graph; false (and graphs off for this
// context) if the capture or the instantiation fails.
static bool capture_step(Ctx* c, uint64_t key) {
  drop_graph(c);
  uint64_t gen = c->lag_gen, before = c->launches;
  if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    c->use_graph = false;
    return false;
  }
  step_enqueue(c);
  cudaGraph_t gr = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
  uint64_t kernels = c->launches - before;
  c->launches = before;                         // counted again at every replay
  if (e != cudaSuccess || !gr || c->status != MIBM_OK || gen != c->lag_gen) {
    if (gr) cudaGraphDestroy(gr);
    cudaGetLastError();
    if (e != cudaSuccess) c->use_graph = false;
    return false;
  }
  cudaGraphExec_t ex = nullptr;
  if (cudaGraphInstantiate(&ex, gr, cudaGraphInstantiateFlagUseNodePriority) != cudaSuccess) {
    cudaGraphDestroy(gr);
    cudaGetLastError();
    c->use_graph = false;
    return false;
  }
  c->graph = gr;
  c->graph_exec = ex;
  c->graph_key = key;
  c->graph_kernels = kernels;
  return true;
}

// tsch.f90:18-97 on the device.  From the second call on, the device part
// runs as a captured graph (one launch per step) while its key holds.
static void tschem(Ctx* c) {
  if (!step_prepare(c)) return;
  step_head(c);
  if (c->status != MIBM_OK) return;
  bool graph = graphs_allowed(c);
  if (graph) {
    uint64_t key = step_key(c);
    if (!c->graph_exec || key != c->graph_key) graph = capture_step(c, key);
  }
  if (graph) {
    if (!cuda_ok(c, cudaGraphLaunch(c->graph_exec, c->stream), "step graph")) return;
    c->launches += c->graph_kernels;
  } else {
    step_enqueue(c);
  }
  step_finish(c);
}

// ---------------------------------------------------------------------
// Autotuner.  Per shape (grid n1m x n2m x n3m, form) it times, with CUDA
// events on the case's own stream, every feasible chunk length of the x-,
// y- and z-line solves (scratch lines) and the block heights 2, 4, 8 of the
// explicit-term kernel (RK history saved and restored), and keeps the
// fastest of each.  Results live in a process-wide table, so every later
// case of the same shape reuses them, and can be saved to / loaded from a
// text file.  A context picks them up by mibm_autotune_; its step graph is
// re-captured (the tuning generation is part of the step key).
// ---------------------------------------------------------------------
struct TuneResult {
  int m[3] = {0, 0, 0};
  int by = 8;
  float ms_m[3] = {0, 0, 0};
  float ms_by = 0;
};
static std::mutex g_tune_mu;
static std::map<std::vector<int>, TuneResult> g_tune;

static std::vector<int> tune_key(Ctx* c) { return {c->g.n1m, c->g.n2m, c->g.n3m, c->precision}; }

static void tune_apply(Ctx* c, const TuneResult& r) {
  for (int d = 0; d < 3; ++d) c->tune_m[d] = r.m[d];
  c->tune_by = r.by;
  ++c->tune_gen;
}

static int autotune(Ctx* c) {
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(tune_key(c));
    if (it != g_tune.end()) { tune_apply(c, it->second); return MIBM_OK; }
  }
  // the form's buffers and parameters must exist for the explicit-term timing
  if (!step_prepare(c)) return c->status;
  cudaMemcpyAsync(c->dparams, c->hparams, 3 * sizeof(StepParams), cudaMemcpyHostToDevice, c->stream);
  const bool f32 = c->precision == 1;
  TuneResult r;
  for (int d = 0; d < 3; ++d) {
    std::vector<int> cand = tri_chunk_candidates(c, d);
    r.m[d] = tri_chunk(c, d);
    r.ms_m[d] = -1.f;
    for (int m : cand) {
      float ms = tri_time_direction(c, d, m, f32, 5);
      if (c->status != MIBM_OK) return c->status;
      if (ms >= 0.f && (r.ms_m[d] < 0.f || ms < r.ms_m[d])) { r.ms_m[d] = ms; r.m[d] = m; }
    }
  }
  r.ms_by = -1.f;
  for (int by : {2, 4, 8}) {
    float ms = stencil_time_by(c, c->dparams, by, 5);
    if (c->status != MIBM_OK) return c->status;
    if (ms >= 0.f && (r.ms_by < 0.f || ms < r.ms_by)) { r.ms_by = ms; r.by = by; }
  }
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune[tune_key(c)] = r;
  }
  tune_apply(c, r);
  // the preparation above built the FP32 mirrors ahead of the case's first
  // step; leave them stale so that the case's own sequence (CFL of step 1
  // from the FP64 fields) is exactly that of an untuned case
  c->q32_valid = false;
  return MIBM_OK;
}

// ---------------------------------------------------------------------
// Batched form: many independent cases (contexts, any grid size, either
// form) advanced by one reference time-loop iteration together
// (gcurv.f90:151-172 for each case).  Per batch step: every case's CFL and
// dt reductions are enqueued on its own stream and read back with one wait
// per case; dt, forcing and the step's host preparation follow; then the
// step graphs of all cases run as one batch graph (one child-graph node per
// case, no edges between them, so the device overlaps the cases), or, for
// cases without a graph yet, as direct launches on their own streams.  The
// per-case host checks close the step.  Each case computes exactly what
// stepping it alone computes.
// ---------------------------------------------------------------------
struct Batch {
  std::vector<int> ids;
  int launch = 0;                            // 0: one batch graph; 1: each case's graph on its own stream
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaGraphExec_t> built_from;   // the case graphs the batch graph holds
};
static std::mutex g_batch_mu;
static std::map<int, Batch*> g_batch;
static int g_batch_next = 1;

static Batch* batch_of(int h) {
  std::lock_guard<std::mutex> g(g_batch_mu);
  auto it = g_batch.find(h);
  return it == g_batch.end() ? nullptr : it->second;
}

static void batch_drop_graph(Batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->built_from.clear();
}

// One batch step.  A case that fails (non-finite field, allocation or CUDA
// error in its own work) is left out of the rest of the step with its status
// kept in its context; the other cases complete the step exactly as they
// would alone.  Returns MIBM_OK, or the first failing case's status (the host
// finds the failed cases with mibm_context_bind_ + mibm_last_status_).
static int batch_step(Batch* b, int ntime) {
  std::vector<Ctx*> all;
  {
    std::lock_guard<std::mutex> g(g_batch_mu);
    for (int id : b->ids) {
      Ctx* c = context_by_id(id);
      if (!c || !ready(c)) { fail(c, MIBM_ESTATE, "batch: context " + std::to_string(id) + " is gone or not initialised"); return MIBM_ESTATE; }
      all.push_back(c);
    }
  }
  int first_bad = MIBM_OK;
  auto drop_failed = [&](std::vector<Ctx*>& v) {
    std::vector<Ctx*> keep;
    for (Ctx* c : v) {
      if (c->status == MIBM_OK) keep.push_back(c);
      else if (first_bad == MIBM_OK) first_bad = c->status;
    }
    v.swap(keep);
  };
  std::vector<Ctx*> cs = all;
  drop_failed(cs);
  // (A) CFL and dt reductions of every case, gcurv.f90:153-160; ntime <= 0:
  // every case counts its own steps (cases that joined at different times)
  for (Ctx* c : cs) {
    const int nt = ntime > 0 ? ntime : (int)c->steps_done + 1;
    *c->hi[MIBM_I_NTIME] = nt;
    if (c->I(MIBM_I_IDTV) == 1 && nt != 1) *c->hs[MIBM_S_DT] = c->S(MIBM_S_DTMAX);
    k_cfl_async(c, c->red_host);
    if (c->I(MIBM_I_IDTV) == 1) k_getdt_async(c, c->S(MIBM_S_DT), c->red_host + 1);
  }
  for (Ctx* c : cs) {
    if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "batch cfl")) continue;
    if (!cfl_finite(c)) continue;
    *c->hs[MIBM_S_CFLM] = cfl_value(c->red_host[0]);
    if (c->I(MIBM_I_IDTV) == 1) {
      double dt = c->S(MIBM_S_DT);
      double buf = getdt_buffer(c->g, c->red_host[1], dt, c->S(MIBM_S_REN));
      if (buf > 0.0) *c->hs[MIBM_S_DT] = dt * c->S(MIBM_S_CFLFIX) / buf;
    }
  }
  drop_failed(cs);
  // (B) forcing (gcurv.f90:164-170) and the host part of each step
  for (Ctx* c : cs) {
    if (c->I(MIBM_I_FORCING) == 1) {
      int which = c->I(MIBM_I_WHICH_HIT);
      if (which == 1) k_hit_random_force(c);
      else if (which == 2) k_hit_abc_force(c);
      else if (which == 3) k_hit_linear_force(c);
    }
    if (c->status != MIBM_OK) continue;
    if (!step_prepare(c)) { if (c->status == MIBM_OK) fail(c, MIBM_ESTATE, "batch: step preparation"); continue; }
    step_head(c);
  }
  drop_failed(cs);
  // (C) device work: step graphs (captured where missing or stale)
  bool all_graphs = b->launch == 0;
  for (Ctx* c : cs) {
    bool graph = graphs_allowed(c);
    if (graph) {
      uint64_t key = step_key(c);
      if (!c->graph_exec || key != c->graph_key) graph = capture_step(c, key);
    }
    all_graphs = all_graphs && graph && c->status == MIBM_OK;
  }
  drop_failed(cs);
  if (cs.empty()) return first_bad;
  if (all_graphs) {
    std::vector<cudaGraphExec_t> now;
    for (Ctx* c : cs) now.push_back(c->graph_exec);
    if (!b->exec || now != b->built_from) {
      batch_drop_graph(b);
      bool ok = cudaGraphCreate(&b->graph, 0) == cudaSuccess;
      for (size_t q = 0; ok && q < cs.size(); ++q) {
        cudaGraphNode_t node;
        ok = cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, cs[q]->graph) == cudaSuccess;
      }
      ok = ok && cudaGraphInstantiate(&b->exec, b->graph, cudaGraphInstantiateFlagUseNodePriority) == cudaSuccess;
      if (!ok) { cudaGetLastError(); batch_drop_graph(b); all_graphs = false; }
      else b->built_from = now;
    }
  }
  if (all_graphs) {
    for (Ctx* c : cs)   // forcing and buffer work enqueued on the case streams comes first
      if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "batch")) return c->status;
    if (!cuda_ok(cs[0], cudaGraphLaunch(b->exec, b->stream), "batch graph")) return cs[0]->status;
    for (Ctx* c : cs) c->launches += c->graph_kernels;
    if (!cuda_ok(cs[0], cudaStreamSynchronize(b->stream), "batch graph")) return cs[0]->status;
  } else {
    for (Ctx* c : cs) {
      if (c->graph_exec && graphs_allowed(c)) {
        if (cuda_ok(c, cudaGraphLaunch(c->graph_exec, c->stream), "step graph")) c->launches += c->graph_kernels;
      } else {
        step_enqueue(c);
      }
    }
  }
  // (D) per-case host checks, time
  for (Ctx* c : cs) {
    step_finish(c);
    if (c->status != MIBM_OK) {
      if (first_bad == MIBM_OK) first_bad = c->status;
      continue;
    }
    *c->hs[MIBM_S_TIME] = c->S(MIBM_S_TIME) + c->S(MIBM_S_DT);
  }
  return first_bad;
}

}  // namespace mibm

using namespace mibm;

// Every drop-in routine is one NVTX range named after the routine (the
// per-routine tracing of the reference's TIMED build, tsch.f90:26-84, for
// Nsight tools).  NVTX v3 is header-only: without a tool attached a range
// costs a branch.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define DROPIN_BEGIN                          \
  NvtxRange mibm_nvtx_range_(__func__);       \
  Ctx* c = current();                         \
  if (!ready(c)) return;
// drop-in routines that write u, v, w, T or p: the FP32 mirrors of the
// precision form are rebuilt before its next step
#define DROPIN_WRITES         \
  DROPIN_BEGIN                \
  c->q32_valid = false;
#define DROPIN_END cuda_ok(c, cudaGetLastError(), __func__);
// drop-in routines that write the geometry, the VOF fields, the cage
// indices, the MLS weights or the scatter plan: the next step redoes its
// substep-0 geometry work instead of taking the one its predecessor enqueued
#define DROPIN_GEOM           \
  DROPIN_BEGIN                \
  ++c->geom_gen;

extern "C" {

void tschem_(void) { DROPIN_BEGIN tschem(c); DROPIN_END }
void hdnl1_(void) { DROPIN_BEGIN k_hdnl(c, 0, push_params(c, 3)); DROPIN_END }
void hdnl2_(void) { DROPIN_BEGIN k_hdnl(c, 1, push_params(c, 3)); DROPIN_END }
void hdnl3_(void) { DROPIN_BEGIN k_hdnl(c, 2, push_params(c, 3)); DROPIN_END }
void hdnlte_(void) { DROPIN_BEGIN k_hdnl(c, 3, push_params(c, 3)); DROPIN_END }
void invtr1_(void) { DROPIN_WRITES invtr(c, 0); DROPIN_END }
void invtr2_(void) { DROPIN_WRITES invtr(c, 1); DROPIN_END }
void invtr3_(void) { DROPIN_WRITES invtr(c, 2); DROPIN_END }
void invtrte_(void) { DROPIN_WRITES invtr(c, 3); DROPIN_END }
void solxi_(const double* betadx) { DROPIN_BEGIN k_solve_x(c, c->df[MIBM_F_RHS], *betadx); DROPIN_END }
void solxj_(const double* betadx) { DROPIN_BEGIN k_solve_y(c, c->df[MIBM_F_RHS], *betadx); DROPIN_END }
void solxk_(double* q, const double* betadx) {
  DROPIN_WRITES
  int id = field_of_plane1(c, q);
  if (id < 0) { fail(c, MIBM_EINVAL, "solxk_: q is not element (1,1,kstart) of a registered field"); return; }
  k_solve_z(c, c->df[MIBM_F_RHS], *betadx, c->df[id]);
  DROPIN_END
}
void divg_(void) { DROPIN_BEGIN k_divg(c, push_params(c, 3)); DROPIN_END }
void phcalc_(void) { DROPIN_BEGIN k_phcalc(c); DROPIN_END }
void updvp_(void) { DROPIN_WRITES k_updvp(c, push_params(c, 3)); DROPIN_END }
void prcalc_(void) { DROPIN_WRITES k_prcalc(c, push_params(c, 3)); DROPIN_END }
void findcentroidindices_(void) { DROPIN_GEOM lagr_find_centroid_indices(c); DROPIN_END }
void mlsweight_(void) { DROPIN_GEOM lagr_mls_weight(c); DROPIN_END }
void mlsforce_(void) { DROPIN_WRITES ++c->geom_gen; lagr_mls_force(c, push_params(c, 3), true); DROPIN_END }
void velforce_(void) { DROPIN_WRITES lagr_velforce(c); DROPIN_END }
void tempforce_(void) { DROPIN_WRITES lagr_tempforce(c); DROPIN_END }
void findprobeindices_(void) { DROPIN_GEOM lagr_find_probe_indices(c); DROPIN_END }
void mls_heatflux_(void) { DROPIN_GEOM lagr_heat_flux(c); DROPIN_END }
void apply_stefancondition_(void) { DROPIN_WRITES ++c->geom_gen; lagr_stefan(c, push_params(c, 3)); DROPIN_END }
void tagcells_(void) { DROPIN_GEOM lagr_tag_narrow_band(c); DROPIN_END }
void tagcells_initial_(void) { DROPIN_GEOM lagr_tag_initial(c); DROPIN_END }
void particle_(void) { DROPIN_WRITES ++c->geom_gen; lagr_particle(c, push_params(c, 3)); DROPIN_END }

// mls_structLoads: the loads of the registered fields and mesh into the
// registered int_*_dA (previous values to the _m1 slots, sums to Fp, ...).
void mls_structloads_(void) {
  DROPIN_BEGIN
  if (c->maxnf == 0 || !rigid_ensure(c)) return;
  rigid_pack(c, c->hrigid_in, false);
  rigid_upload(c);
  lagr_struct_loads(c, push_params(c, 3));
  if (c->status != MIBM_OK) return;
  rigid_download(c);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "mls_structloads")) return;
  rigid_unpack(c, c->hrigid_out, false);
  DROPIN_END
}

// update_part_pos: Newton-Euler from the registered loads, Volume, pos_CM
// and InertTensor; moves the device mesh (xyzv, tri_bar, vel_tri) and
// updates pos_CM, vel_CM, omega_c, quat and InertTensor.
void update_part_pos_(void) {
  DROPIN_BEGIN
  if (c->maxnf == 0 || !rigid_ensure(c)) return;
  rigid_pack(c, c->hrigid_in, true);
  rigid_upload(c);
  const double* geom = (const double*)((const char*)c->drigid + offsetof(RigidDev, geom_in));
  k_newton_euler(c, push_params(c, 3), geom);
  k_update_xyz(c, true);
  rigid_download(c);
  cudaMemcpyAsync(c->hflag, c->dflag, 4, cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "update_part_pos")) return;
  if (c->hflag[0]) {
    fail(c, MIBM_ENUMERIC, "update_part_pos: singular inertia tensor (dgetrf info /= 0)");
    c->hflag[0] = 0;
    cudaMemsetAsync(c->dflag, 0, 4, c->stream);
    return;
  }
  rigid_unpack(c, c->hrigid_out, true);
  lagr_invalidate(c);
  DROPIN_END
}

// forcx, forcy, forcz are read by the stencils as FP64 in both forms (no
// FP32 mirror), so the HIT drop-ins leave the mirrors valid
void calchitrandomforce_(void) { DROPIN_BEGIN k_hit_random_force(c); DROPIN_END }
void calcabc_hitforce_(void) { DROPIN_BEGIN k_hit_abc_force(c); DROPIN_END }
void mibm_linear_hit_force_(void) { DROPIN_BEGIN k_hit_linear_force(c); DROPIN_END }
int mibm_hit_modes_(void) {
  Ctx* c = current(); if (!ready(c)) return 0;
  return hit_modes(c);
}
void mibm_hit_bhat_(double* bhat, const int* dir) {
  Ctx* c = current(); if (!ready(c)) return;
  if (!bhat || (*dir != 0 && *dir != 1)) { fail(c, MIBM_EINVAL, "hit_bhat: dir 0 (get) or 1 (set)"); return; }
  hit_bhat(c, bhat, *dir);
}
void mibm_hit_rng_(unsigned long long* state, const int* dir) {
  Ctx* c = current(); if (!ready(c)) return;
  if (!state || (*dir != 0 && *dir != 1)) { fail(c, MIBM_EINVAL, "hit_rng: dir 0 (get) or 1 (set)"); return; }
  hit_rng(c, state, *dir);
}

void cfl_(void) {
  DROPIN_BEGIN
  *c->hs[MIBM_S_CFLM] = k_cfl(c);
  DROPIN_END
}

void get_dt_(void) {
  DROPIN_BEGIN
  double dt = c->S(MIBM_S_DT);
  double buf = k_get_dt_buffer(c, dt, c->S(MIBM_S_REN));
  if (buf > 0.0) *c->hs[MIBM_S_DT] = dt * c->S(MIBM_S_CFLFIX) / buf;
  DROPIN_END
}

// Select the form of tschem_: 0 = plain FP64 (default), 1 = FP32 compute
// with FP64 fields and refined projection; nproj = Poisson solves per
// substep in the precision form (>= 1).
void mibm_set_precision_(const int* mode, const int* nproj) {
  Ctx* c = current(); if (!ready(c)) return;
  if (*mode < 0 || *mode > 1 || *nproj < 1 || *nproj > 8) { fail(c, MIBM_EINVAL, "set_precision: mode 0|1, nproj 1..8"); return; }
  // the explicit-term histories live in ru32 while the precision form runs:
  // hand them over in the direction of the switch
  if (*mode == 1 && c->precision == 0 && c->ru32)
    for (int q = 0; q < 4; ++q) k_cast_d2f(c, c->g.cells, c->df[kRuFields[q]], c->ru32 + (size_t)q * c->g.cells);
  if (*mode == 0 && c->precision == 1 && c->ru32)
    for (int q = 0; q < 4; ++q) k_cast_f2d(c, c->g.cells, c->ru32 + (size_t)q * c->g.cells, c->df[kRuFields[q]]);
  c->q32_valid = false;
  c->precision = *mode;
  c->nproj = *nproj;
  ++c->geom_gen;                       // the MLS weights of the two forms differ
}

// Staged FP32 line solves on (1, default) or off (0): bit-identical results
// either way; the switch exists to compare the two data paths.
void mibm_set_tma_(const int* on) {
  Ctx* c = current(); if (!ready(c)) return;
  if (*on != 0 && *on != 1) { fail(c, MIBM_EINVAL, "set_tma: 0|1"); return; }
  if (c->tma != *on) ++c->tune_gen;    // the step graph holds the other kernels
  c->tma = *on;
}

// The precision form's one-pass kernels (u, v, w explicit terms in one
// kernel, velocity and pressure updates in one kernel; 1, default) or the
// products path and separate updates as in the FP64 form (0): the same
// bits; the switch exists to compare the two.
void mibm_set_fused_uvw_(const int* on) {
  Ctx* c = current(); if (!ready(c)) return;
  if (*on != 0 && *on != 1) { fail(c, MIBM_EINVAL, "set_fused_uvw: 0|1"); return; }
  if (c->fused_uvw != *on) ++c->tune_gen;
  c->fused_uvw = *on;
}

// Batched form (see Batch above).  ids: contexts after mibm_init_ (and the
// initial tagging); returns a handle > 0, or 0 with the status in
// mibm_last_status_.
int mibm_batch_create_(const int* ids, const int* n) {
  if (*n < 0 || (!ids && *n > 0)) { fail(nullptr, MIBM_EINVAL, "batch_create: bad member list"); return 0; }
  Batch* b = new Batch();
  for (int q = 0; q < *n; ++q) {
    Ctx* c = context_by_id(ids[q]);
    if (!c || !ready(c)) { delete b; fail(nullptr, MIBM_EINVAL, "batch_create: context not initialised"); return 0; }
    for (int id : b->ids)
      if (id == ids[q]) { delete b; fail(nullptr, MIBM_EINVAL, "batch_create: context listed twice"); return 0; }
    b->ids.push_back(ids[q]);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    fail(nullptr, MIBM_ECUDA, "batch_create: stream");
    return 0;
  }
  std::lock_guard<std::mutex> g(g_batch_mu);
  int h = g_batch_next++;
  g_batch[h] = b;
  return h;
}

// One iteration of the time loop (cfl, dt, forcing, tschem) for every case
// of the batch; ntime as in gcurv.f90:151, or <= 0 for each case's own step
// count + 1.  Returns a status.
int mibm_batch_step_(const int* handle, const int* ntime) {
  NvtxRange range("mibm_batch_step_");
  Batch* b = batch_of(*handle);
  if (!b) { fail(nullptr, MIBM_EINVAL, "batch_step: unknown batch"); return MIBM_EINVAL; }
  return batch_step(b, *ntime);
}

// Membership of a batch between steps: add a context (initialised, not yet a
// member) or remove one.  Returns a status.  Removing the last member leaves
// an empty batch whose steps do nothing.
int mibm_batch_add_(const int* handle, const int* id) {
  Batch* b = batch_of(*handle);
  if (!b) { fail(nullptr, MIBM_EINVAL, "batch_add: unknown batch"); return MIBM_EINVAL; }
  Ctx* c = context_by_id(*id);
  if (!c || !ready(c)) { fail(nullptr, MIBM_EINVAL, "batch_add: context not initialised"); return MIBM_EINVAL; }
  std::lock_guard<std::mutex> g(g_batch_mu);
  for (int q : b->ids)
    if (q == *id) { fail(nullptr, MIBM_EINVAL, "batch_add: context already a member"); return MIBM_EINVAL; }
  b->ids.push_back(*id);
  return MIBM_OK;
}

int mibm_batch_remove_(const int* handle, const int* id) {
  Batch* b = batch_of(*handle);
  if (!b) { fail(nullptr, MIBM_EINVAL, "batch_remove: unknown batch"); return MIBM_EINVAL; }
  std::lock_guard<std::mutex> g(g_batch_mu);
  for (size_t q = 0; q < b->ids.size(); ++q)
    if (b->ids[q] == *id) {
      b->ids.erase(b->ids.begin() + q);
      return MIBM_OK;
    }
  fail(nullptr, MIBM_EINVAL, "batch_remove: not a member");
  return MIBM_EINVAL;
}

// How a batch step launches its cases' step graphs: 0 = one batch graph of
// child-graph nodes (rebuilt when the members or their graphs change), 1 =
// each case's own step graph on its own stream (nothing to rebuild when cases
// join or leave).  The results are the same either way.
int mibm_batch_set_launch_(const int* handle, const int* mode) {
  Batch* b = batch_of(*handle);
  if (!b) { fail(nullptr, MIBM_EINVAL, "batch_set_launch: unknown batch"); return MIBM_EINVAL; }
  if (*mode != 0 && *mode != 1) { fail(nullptr, MIBM_EINVAL, "batch_set_launch: mode 0|1"); return MIBM_EINVAL; }
  b->launch = *mode;
  if (b->launch == 1) batch_drop_graph(b);
  return MIBM_OK;
}

int mibm_batch_destroy_(const int* handle) {
  Batch* b = nullptr;
  {
    std::lock_guard<std::mutex> g(g_batch_mu);
    auto it = g_batch.find(*handle);
    if (it == g_batch.end()) return MIBM_EINVAL;
    b = it->second;
    g_batch.erase(it);
  }
  batch_drop_graph(b);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MIBM_OK;
}

// Autotune the bound context's shapes (cached per grid and form); returns a
// status.  get: out[0..3] = x, y, z chunk lengths and the block height in
// use.  save / load: the process-wide table as text, one shape per line.
int mibm_autotune_(void) {
  Ctx* c = current(); if (!ready(c)) return MIBM_ESTATE;
  return autotune(c);
}

int mibm_autotune_get_(int* out) {
  Ctx* c = current(); if (!ready(c)) return MIBM_ESTATE;
  for (int d = 0; d < 3; ++d) out[d] = tri_chunk(c, d);
  out[3] = c->tune_by;
  return MIBM_OK;
}

int mibm_autotune_save_(const char* path) {
  FILE* f = fopen(path, "w");
  if (!f) return MIBM_EINVAL;
  std::lock_guard<std::mutex> g(g_tune_mu);
  fprintf(f, "# n1m n2m n3m form  m_x m_y m_z by  ms_x ms_y ms_z ms_by\n");
  for (auto& e : g_tune)
    fprintf(f, "%d %d %d %d  %d %d %d %d  %.5f %.5f %.5f %.5f\n", e.first[0], e.first[1], e.first[2], e.first[3],
            e.second.m[0], e.second.m[1], e.second.m[2], e.second.by, e.second.ms_m[0], e.second.ms_m[1],
            e.second.ms_m[2], e.second.ms_by);
  fclose(f);
  return MIBM_OK;
}

int mibm_autotune_load_(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return MIBM_EINVAL;
  char line[512];
  std::lock_guard<std::mutex> g(g_tune_mu);
  while (fgets(line, sizeof(line), f)) {
    if (line[0] == '#') continue;
    int k[4];
    TuneResult r;
    if (sscanf(line, "%d %d %d %d %d %d %d %d %f %f %f %f", &k[0], &k[1], &k[2], &k[3], &r.m[0], &r.m[1], &r.m[2],
               &r.by, &r.ms_m[0], &r.ms_m[1], &r.ms_m[2], &r.ms_by) == 12)
      g_tune[{k[0], k[1], k[2], k[3]}] = r;
  }
  fclose(f);
  return MIBM_OK;
}

void mibm_set_graphs_(const int* on) {
  Ctx* c = current(); if (!ready(c)) return;
  c->use_graph = *on != 0;
  if (!c->use_graph) drop_graph(c);
}

// The host's remesher (see include/mibm.h); fn = NULL removes it.
void mibm_set_remesh_callback_(mibm_remesh_fn fn, void* user) {
  Ctx* c = current(); if (!ready(c)) return;
  c->remesh_fn = fn;
  c->remesh_user = user;
}

int mibm_remesh_count_(void) {
  Ctx* c = current(); if (!c) return 0;
  return c->remesh_count;
}

// statistics of the library remesher's last call on the bound context
int mibm_remesh_stats_(double* out) {
  Ctx* c = current(); if (!c || !out) return MIBM_EINVAL;
  for (int q = 0; q < 8; ++q) out[q] = c->remesh_stats[q];
  return MIBM_OK;
}

// Diagnostics (diag.cu): computed now, or per step inside tschem_.
int mibm_diagnostics_(double* out) {
  Ctx* c = current(); if (!ready(c)) return c ? c->status : MIBM_ESTATE;
  if (!out) { fail(c, MIBM_EINVAL, "diagnostics: null output"); return MIBM_EINVAL; }
  const StepParams* dp = push_params(c, 3);
  diag_enqueue(c, (const double*)((const char*)dp + offsetof(StepParams, vel)));
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "diagnostics")) return c->status;
  if (c->status != MIBM_OK) return c->status;
  diag_finish(c);
  memcpy(out, c->diag_last, sizeof(double) * MIBM_NDIAG);
  return MIBM_OK;
}

void mibm_set_diagnostics_(const int* on) {
  Ctx* c = current(); if (!ready(c)) return;
  c->diag_on = *on != 0;
}

int mibm_diagnostics_get_(double* out) {
  Ctx* c = current(); if (!ready(c)) return c ? c->status : MIBM_ESTATE;
  if (!c->diag_valid) { fail(c, MIBM_ESTATE, "diagnostics: no step computed them"); return MIBM_ESTATE; }
  memcpy(out, c->diag_last, sizeof(double) * MIBM_NDIAG);
  return MIBM_OK;
}

// max over owned cells of |div u| (divgck, divg.f90:26-56); synchronises
double mibm_divergence_max_(void) {
  Ctx* c = current(); if (!ready(c)) return -1.0;
  if (!c->divmax && !cuda_ok(c, cudaMalloc(&c->divmax, sizeof(unsigned long long)), "divmax")) return -1.0;
  k_divmax(c, c->divmax);
  unsigned long long bits = 0;
  cudaMemcpyAsync(&bits, c->divmax, sizeof(bits), cudaMemcpyDeviceToHost, c->stream);
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "divergence")) return -1.0;
  double v;
  memcpy(&v, &bits, sizeof(v));
  return v;
}

void interp_(double* arrold, double* arrnew, const int* n1o, const int* n2o, const int* n3o, const int* intvar,
             const int* kstarto, const int* kendo) {
  DROPIN_BEGIN
  if (!arrold || !arrnew) { fail(c, MIBM_EINVAL, "interp_: null array"); return; }
  k_interp_restart(c, arrold, arrnew, *n1o, *n2o, *n3o, *intvar, *kstarto, *kendo);
  DROPIN_END
}

}  // extern "C"
