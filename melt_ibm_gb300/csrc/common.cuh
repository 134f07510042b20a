// common.cuh -- shared context, device layout and helpers of libmibm.so.
//
// Device layout of a cell field (compact, no ghost planes):
//   q(i, j, k), 0-based i < n1m, j < n2m, k < n3m  ->  q[i + P*(j + n2m*k)]
// with row pitch P = n1m rounded up to a multiple of 4 elements (32-byte rows
// in FP64, 16-byte rows in FP32).  The Fortran ghost planes k = 0, n3m+1 of
// the host arrays are periodic copies (mpi_routines.f90:139-210 on one rank),
// so kernels wrap k instead of storing them; they are rebuilt on the host
// copy at mibm_sync_to_host_.  The Fortran padding column i = n1 of vx and row
// j = n2 of vy are read only by `cfl` (cfl.f90:19-26); their values are kept
// in two small device planes (pad_vx, pad_vy).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mibm.h"

namespace mibm {

constexpr int kMaxCtx = 4096;

// Per-substep products of grid and step scalars used by the stencils.  Each
// is one IEEE operation (or the left-to-right product the reference writes)
// evaluated on the host in FP64, so the FP64 kernels read the same value they
// would compute per cell; `cf` holds the same values rounded once to FP32.
// Taking them off the device matters because FP64 multiplies, divisions and
// FP64<->FP32 conversions all issue at the low FP64 rate.
enum Coef {
  kQ1, kQ2, kQ3,          // dx1*0.25, dx2*0.25, dx3*0.25   (hdnl1-3 udx)
  kH1, kH2, kH3,          // dx1*0.5,  dx2*0.5,  dx3*0.5    (hdnlte udx)
  kDQ1, kDQ2, kDQ3,       // dx1q, dx2q, dx3q
  kGA, kRO, kALRE, kDT,
  kPX1, kPX2, kPX3,       // dx1*al, dx2*al, al*dx3          (invtr pressure gradient)
  kALPEC,                 // al/pec                          (invtrte)
  kBETAGZ, kTLIQ,
  kXLEN, kYLEN, kZLEN,
  kUP1, kUP2, kUP3,       // al*dt*dx1, al*dt*dx2, al*dt*dx3 (updvp)
  kBE,                    // al*beta                         (prcalc)
  kUSDTAL,                // 1/(dt*al)                       (divg)
  // the RHS of invtr1-3 / invtrte with dt folded in (one multiply per term)
  kGDT, kRDT,             // ga*dt, ro*dt
  kLV1, kLV2, kLV3, kLVC, // al/ren*dt*dxq (per direction), 2*(kLV1+kLV2+kLV3)
  kLT1, kLT2, kLT3, kLTC, // al/pec*dt*dxq, 2*(kLT1+kLT2+kLT3)
  kPD1, kPD2, kPD3,       // dt*kPX1, dt*kPX2, dt*kPX3
  kRXLEN, kRYLEN, kRZLEN, // 1/xlen, 1/ylen, 1/zlen           (hdnl1-3 forcing term)
  kPB1, kPB2, kPB3, kPBC, // al*beta*dxq per direction, 1 + 2*(kPB1+kPB2+kPB3)  (prcalc)
  kDVI,                   // dx1/(dt*al)                     (precision-form divg, equal spacings)
  kNCoef
};

// Per-substep scalars read by the kernels.  The fused RK3 path keeps one
// copy per substep on the device so that a captured graph reads the values
// of the current step (dt changes every step in CFL mode).
struct StepParams {
  double al, ga, ro, dt, beta;
  double alre;      // al / ren
  double pec, ren;
  double betagz, tliq, tmelt;
  double pos[3], vel[3], om[3];
  double cd[kNCoef];
  float cf[kNCoef];
  int force_plan;   // rebuild the scatter plan from scratch this substep (a host mesh upload)
};

template <typename R> __host__ __device__ __forceinline__ R coef(const StepParams& p, int i);
template <> __host__ __device__ __forceinline__ double coef<double>(const StepParams& p, int i) { return p.cd[i]; }
template <> __host__ __device__ __forceinline__ float coef<float>(const StepParams& p, int i) { return p.cf[i]; }

// Moving-body state (imlsstr = 1) kept on the device while a step runs:
// rigid velocities, orientation, the structural loads of this and the
// previous substep (mls_structLoads.f90:21-24), their running sums, and the
// products of the Newton-Euler update that update_xyz applies.  Loads are
// packed [int_prn_dA, int_tau_dA, int_r_x_prn_dA, int_r_x_tau_dA] and the
// sums [Fp, Ftau, Torq_p, Torq_tau].  `geom_in` mirrors the geometry buffer
// layout [Surface, Volume1, Volume, pos_CM(3), InertTensor(9)] for the
// drop-in update_part_pos_, which takes them from the registered scalars.
struct RigidDev {
  double vel[3], om[3], quat[4];
  double load[12], load1[12], acc[12];
  double inert[9];
  double xf[15];        // AA (column-major), new pos_CM, pos_CM before the move
  double geom_in[16];
  int iters, pad;
};

struct Grid {
  int n1m, n2m, n3m;         // cells per direction
  int P;                     // row pitch (elements)
  size_t plane, cells;       // P*n2m, plane*n3m
  double xlen, ylen, zlen;
  double dx1, dx2, dx3, dx1q, dx2q, dx3q;
  int H, HP;                 // n1m/2+1 complex columns, padded pitch
};

// Device pointer bundle passed by value to kernels.
struct DevFields {
  double* f[MIBM_NFIELDS];
};

struct Ctx {
  int id = 0;
  int status = MIBM_OK;
  std::string msg;
  int device = 0;
  bool grid_set = false, inited = false;
  Grid g{};
  // host registration
  double* hf[MIBM_NFIELDS] = {nullptr};
  void* hm[MIBM_NMESH] = {nullptr};
  double* hs[MIBM_NSCALARS] = {nullptr};
  int* hi[MIBM_NINTS] = {nullptr};
  int maxnv = 0, maxne = 0, maxnf = 0;
  // device storage
  double* df[MIBM_NFIELDS] = {nullptr};   // compact fields
  double* pad_vx = nullptr;               // vx(n1, j, k), j<n2m, k<n3m
  double* pad_vy = nullptr;               // vy(i, n2, k), i<n1m, k<n3m
  void* dm[MIBM_NMESH] = {nullptr};       // mesh mirrors
  double* stage = nullptr;                // host<->device staging (one Fortran field)
  void* mesh_stage = nullptr;             // one uploaded mesh array, compared with the device copy
  size_t stage_bytes = 0;
  // spectral work for phcalc: complex [k][j][kx], kx pitch HP
  double2* spec = nullptr;
  // modified wavenumbers (phini.f90:28-56) and coordinates (cordin.f90)
  double *ak1 = nullptr, *ak2 = nullptr, *ak3 = nullptr;
  double *xc = nullptr, *xm = nullptr, *yc = nullptr, *ym = nullptr, *zc = nullptr, *zm = nullptr;
  int coord_off = 0;                      // coordinate arrays cover [-coord_off, ...)
  // scratch for reductions / Lagrangian work
  double* red = nullptr;                  // reduction scratch: [0,64) results, [64,...) partials
  size_t red_elems = 0;
  double* red_host = nullptr;             // pinned
  int* dflag = nullptr;                   // device error flags
  int* hflag = nullptr;                   // pinned copy
  double* tri_coef = nullptr;             // per triangle & component: cfac*(target-Um)
  double* lag_red = nullptr;              // per-triangle partial sums
  cudaStream_t stream = nullptr;
  // second stream of the fused step: the Lagrangian work after the velocity
  // forcing runs on it beside the pressure projection (fork / join events)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool join_pending = false;
  // the part of the side branch the next substep's explicit terms need: the
  // published rigid-body state (ev_pub) and the VOF fields (ev_tjoin when the
  // tagging ran on its own stream); the cage indices, MLS weights and scatter
  // plan (ev_join) are waited for only before the forcing
  cudaEvent_t ev_pub = nullptr, ev_gfork = nullptr;
  bool geom_join_pending = false, geom_join_tag = false;
  cudaEvent_t ev_lfork = nullptr, ev_ldone = nullptr;   // structural loads on the side stream
  cudaStream_t side2 = nullptr;                         // narrow-band tagging beside the MLS weights and plan
  cudaEvent_t ev_tfork = nullptr, ev_tjoin = nullptr;
  cudaStream_t side3 = nullptr;                         // MLS weights beside the scatter plan
  cudaEvent_t ev_wfork = nullptr, ev_wjoin = nullptr;
  cudaStream_t tsolve = nullptr;                        // the temperature's line solves beside the velocity's
  cudaEvent_t ev_sfork = nullptr, ev_sjoin = nullptr;
  bool loads_pending = false;
  std::vector<void*> pinned;              // host arrays page-locked by mibm_pin_host_
  // device-accessible addresses of page-locked host fields: the pack and
  // unpack kernels read and write them directly over the CPU-GPU link
  double* hf_dev[MIBM_NFIELDS] = {nullptr};
  bool prologue_done = false;             // the next substep's geometry-only work is enqueued
  // substep 0's geometry-only work, enqueued by the previous step's last
  // substep: valid while geom_gen (bumped by every host call that may change
  // the geometry, the VOF fields or the MLS state) and the step key hold
  bool early_prologue = false;
  uint64_t geom_gen = 0, early_gen = 0, early_key = 0;
  // fused-step state
  StepParams* dparams = nullptr;          // [3] device copies (one per substep)
  StepParams* hparams = nullptr;          // pinned
  double* rhs4 = nullptr;                 // 4 RHS fields for the fused path
  double* prod = nullptr;                 // 6 advection products (fused FP64 path)
  float* prod32 = nullptr;                // the same in the precision form
  // precision form (FP32 compute, FP64 fields, refined projection)
  int precision = 0;                      // 0 = plain FP64, 1 = FP32 + refinement
  int nproj = 2;                          // Poisson solves per substep in precision form
  float* ru32 = nullptr;                  // 4 explicit-term histories (FP32)
  float* rhs32 = nullptr;                 // 4 RHS / line-solve fields (FP32)
  float* phi32 = nullptr;                 // FP32 pressure correction
  float* res32 = nullptr;                 // FP32 copy of the FP64 divergence residual
  double* vel1 = nullptr;                 // u, v, w after a projection sweep that is not the last (3 fields)
  // FP32 mirrors of u, v, w, T, p (5 fields, field order of the Stencil
  // kernels) read by the FP32 stencils.  The kernels that write the FP64
  // fields in the precision form also write the mirror; anything else that
  // writes a field (drop-in routines, mibm_sync_from_host_, the FP64 form)
  // clears q32_valid and the next precision step rebuilds the mirrors.
  float* q32 = nullptr;
  bool q32_valid = false;
  unsigned long long* divmax = nullptr;   // device max|div u| (IEEE bits)
  // captured step graph (tschem_ from its second call): replayed while the
  // key of everything a step reads by value from the host is unchanged
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool use_graph = true;
  uint64_t graph_key = 0;
  uint64_t graph_kernels = 0;             // kernel launches recorded in the graph
  uint64_t steps_done = 0;
  uint64_t lag_gen = 0;                   // bumped when the Lagrangian launch sequence changes
  bool profiling = false;                 // per-kernel event profiling on (no graphs then)
  // shapes chosen by the autotuner (tune.cu); -1 / 8 = the default rules
  int tune_m[3] = {-1, -1, -1};           // line-solve chunk length per direction
  int tune_by = 2;                        // block height of the explicit-term kernels (32 x 2 threads: the
                                          // autotuner's choice at 48^3, 128^3 and 256^3)
  uint64_t tune_gen = 0;
  int tma = 1;                            // FP32 y/z line solves staged by bulk tensor copies
  int fused_uvw = 1;                      // FP32 one-pass kernels (u, v, w explicit terms; projection update)
  double* step_host = nullptr;            // pinned: geometry scalars read back at step end
  // remeshing hand-off: the host's remesher and the hand-offs done
  mibm_remesh_fn remesh_fn = nullptr;
  void* remesh_user = nullptr;
  int remesh_count = 0;
  // the library's remesher (remesh.cu): statistics of its last call on this
  // context [edge collapses, vertex deletions, edge relaxations, vol_melt,
  // vol_coarse, vol_smooth, largest vertex drift, extra volume passes]
  double remesh_stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // per-step diagnostics (diag.cu): requested, last values, device state
  bool diag_on = false, diag_valid = false;
  double diag_last[MIBM_NDIAG] = {0};
  void* diag = nullptr;
  RigidDev* drigid = nullptr;             // moving-body state (device)
  RigidDev* hrigid_in = nullptr;          // pinned: uploaded at the start of a step
  RigidDev* hrigid_out = nullptr;         // pinned: read back at its end
  uint64_t launches = 0;                  // kernels launched through this context
  cudaEvent_t timers[64] = {nullptr};

  double S(int id) const { return *hs[id]; }
  int I(int id) const { return *hi[id]; }
};

Ctx* current();
void fail(Ctx* c, int st, const std::string& m);
Ctx* context_by_id(int id);
bool cuda_ok(Ctx* c, cudaError_t e, const char* what);
bool ready(Ctx* c);
StepParams host_params(Ctx* c);

#define MIBM_LAUNCH_CHECK(c, what) cuda_ok((c), cudaGetLastError(), (what))

// Brackets the launches in its scope with CUDA events when profiling is on
// (prof.cu); a no-op otherwise.
class ProfScope {
 public:
  ProfScope(Ctx* c, const char* name);
  ~ProfScope();
 private:
  Ctx* c_;
  int idx_;
};
#define MIBM_PROF(c, name) ::mibm::ProfScope _mibm_prof_scope_((c), (name))
void prof_release(Ctx* c);
void prof_flush_if_full(Ctx* c);

// ---------------------------------------------------------------------
// Bounds build (compiled with -DMIBM_BOUNDS): checked indices that fall
// outside their array are counted in a device word of the translation unit
// and the access is skipped or redirected to element 0 -- no trap, the
// context stays usable.  mibm_bounds_check_() collects the counts of every
// unit.  In the normal build the checks compile to nothing.
// ---------------------------------------------------------------------
#ifdef MIBM_BOUNDS
static __device__ unsigned g_bounds_hits;
__device__ __forceinline__ bool bounds_ok(size_t i, size_t n) {
  if (i < n) return true;
  atomicAdd(&g_bounds_hits, 1u);
  return false;
}
void bounds_register(unsigned (*take)());
namespace {
unsigned bounds_take_unit() {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_bounds_hits, sizeof v) != cudaSuccess) return 0;
  cudaMemcpyToSymbol(g_bounds_hits, &z, sizeof z);
  return v;
}
struct BoundsUnit { BoundsUnit() { bounds_register(&bounds_take_unit); } };
static BoundsUnit g_bounds_unit;
}  // namespace
#define MIBM_IDX_OK(i, n) ::mibm::bounds_ok((size_t)(i), (size_t)(n))
#else
#define MIBM_IDX_OK(i, n) true
#endif

inline __host__ __device__ size_t cidx(const Grid& g, int i, int j, int k) {
#if defined(MIBM_BOUNDS) && defined(__CUDA_ARCH__)
  // the whole allocation: pitch columns, rows, planes
  if (!(bounds_ok((size_t)i, (size_t)g.P) & bounds_ok((size_t)j, (size_t)g.n2m) & bounds_ok((size_t)k, (size_t)g.n3m)))
    return 0;
#endif
  return (size_t)i + (size_t)g.P * ((size_t)j + (size_t)g.n2m * (size_t)k);
}
inline __host__ __device__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }
inline __host__ __device__ int fmod_pos(int a, int n) { int r = a % n; return r < 0 ? r + n : r; }

inline unsigned div_up(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// layout of Ctx::red
constexpr size_t kRedOut = 0;        // small results
constexpr size_t kRedPart = 64;      // per-block partials (up to 3 * n2m * n3m)

// mesh helpers
inline size_t mesh_elems(Ctx* c, int id) {
  switch (id) {
    case MIBM_M_XYZV: case MIBM_M_VERT_NOR: case MIBM_M_VMELT: case MIBM_M_VMELT_M1: return 3 * (size_t)c->maxnv;
    case MIBM_M_VERT_OF_FACE: case MIBM_M_TRI_BAR: case MIBM_M_TRI_NOR: case MIBM_M_VEL_TRI:
    case MIBM_M_EDGE_OF_FACE: return 3 * (size_t)c->maxnf;
    case MIBM_M_SUR: case MIBM_M_CFAC: case MIBM_M_GHOST_FACE: case MIBM_M_QW_O: case MIBM_M_QW_I:
    case MIBM_M_SKEWNESS: return (size_t)c->maxnf;
    case MIBM_M_AVERT: case MIBM_M_GHOST_VERT: case MIBM_M_QW_OVERT: case MIBM_M_QW_IVERT: return (size_t)c->maxnv;
    case MIBM_M_PIND: return 6 * (size_t)c->maxnf;
    case MIBM_M_PTXAB_Q1: case MIBM_M_PTXAB_Q2: case MIBM_M_PTXAB_Q3: case MIBM_M_PTXAB_TEMP: return 27 * (size_t)c->maxnf;
    case MIBM_M_VERT_OF_EDGE: return 2 * (size_t)c->maxne;
    case MIBM_M_GHOST_EDGE: return (size_t)c->maxne;
    case MIBM_M_ELENGTHS: return (size_t)c->maxne;
  }
  return 0;
}
inline bool mesh_is_int(int id) {
  return id == MIBM_M_VERT_OF_FACE || id == MIBM_M_GHOST_FACE || id == MIBM_M_GHOST_VERT || id == MIBM_M_PIND ||
         id == MIBM_M_VERT_OF_EDGE || id == MIBM_M_EDGE_OF_FACE || id == MIBM_M_GHOST_EDGE;
}
inline size_t mesh_bytes(Ctx* c, int id) { return mesh_elems(c, id) * (mesh_is_int(id) ? 4 : 8); }

// Fortran host shape of a registered field
inline void field_host_shape(const Ctx* c, int id, int& ny, int& klo, int& nk) {
  ny = (id == MIBM_F_DPH) ? c->g.n2m + 2 : c->g.n2m + 1;
  bool plain = (id >= MIBM_F_RHS && id <= MIBM_F_RUT) || id == MIBM_F_SDF;
  klo = plain ? 1 : 0;
  nk = plain ? c->g.n3m : c->g.n3m + 2;
}

// ---------------------------------------------------------------------
// kernel-launch entry points implemented in the .cu files
// ---------------------------------------------------------------------
// stencil.cu
void k_hdnl(Ctx* c, int which, const StepParams* dp);
void k_invtr_rhs(Ctx* c, int which, const StepParams* dp, double* rhs_out);
void k_fused_rhs(Ctx* c, const StepParams* dp);
void k_fused_rhs_f32(Ctx* c, const StepParams* dp, float* ru4, float* rhs4);
void k_updvp_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool mirror);
void k_prcalc_f32(Ctx* c, const StepParams* dp, const float* phi, bool mirror);
void k_divg_f32(Ctx* c, const StepParams* dp, float* res);
void k_updvp_prcalc_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool mirror,
                        bool from_vel1 = false);
bool k_updvp_prcalc_divg_f32(Ctx* c, const StepParams* dp, const float* phi, const double* mean3, bool from_vel1,
                             float* res);
void k_mirror_fields(Ctx* c);
// HIT forcing (hit.cu)
void k_hit_random_force(Ctx* c);
void k_hit_abc_force(Ctx* c);
void k_hit_linear_force(Ctx* c);
int hit_modes(Ctx* c);
void hit_bhat(Ctx* c, double* buf, int dir);
void hit_rng(Ctx* c, unsigned long long* state, int dir);
void hit_free(Ctx* c);
// autotuner support (tridiag.cu, stencil.cu)
float tri_time_direction(Ctx* c, int dir, int m, bool f32, int reps);
std::vector<int> tri_chunk_candidates(Ctx* c, int dir);
int tri_chunk(Ctx* c, int dir);
float stencil_time_by(Ctx* c, const StepParams* dp, int by, int reps);
// restart regrid (interp.cu): host arrays in, host array out
void k_interp_restart(Ctx* c, double* arrold, double* arrnew, int n1o, int n2o, int n3o, int intvar, int kstarto,
                      int kendo);
// precision form around host transfers: the explicit-term histories ru* are
// carried in FP32 on the device; uploads of u, v, w, T, p invalidate the mirrors
void precision_before_download(Ctx* c, unsigned long long mask);
void precision_after_upload(Ctx* c, unsigned long long mask);
void k_cast_f2d(Ctx* c, size_t n, const float* a, double* b);
void k_cast_d2f(Ctx* c, size_t n, const double* a, float* b);
void k_divmax(Ctx* c, unsigned long long* out);
void k_divg(Ctx* c, const StepParams* dp);
void k_updvp(Ctx* c, const StepParams* dp, const double* mean3 = nullptr);
void k_prcalc(Ctx* c, const StepParams* dp);
void k_updvp_prcalc(Ctx* c, const StepParams* dp, const double* mean3);
void k_add_field(Ctx* c, double* q, const double* r);
double k_cfl(Ctx* c);
void k_cfl_async(Ctx* c, double* out);
bool fft_prepare(Ctx* c, bool f32);
void tri_build_table(int n, double betadx, std::vector<double>& t);
size_t tri_ext_len(int n, int m);
void tri_build_ext_table(int n, int m, double betadx, std::vector<double>& out);
bool cfl_finite(Ctx* c);
void k_getdt_async(Ctx* c, double dt, double* out);
double cfl_value(double reduced);
double getdt_buffer(const Grid& g, double reduced, double dt, double ren);
double k_get_dt_buffer(Ctx* c, double dt, double ren);
void k_interp_vof(Ctx* c);
void k_velforce_apply(Ctx* c, const double* mean3);
void k_tempforce_apply(Ctx* c);
// tridiag.cu
void k_solve_x(Ctx* c, double* rhs, double betadx);
void k_solve_y(Ctx* c, double* rhs, double betadx);
void k_solve_z(Ctx* c, double* rhs, double betadx, double* q);
void k_solve_x_T(Ctx* c, double* rhs, const double* T, int nfield);
void k_solve_y_T(Ctx* c, double* rhs, const double* T, int nfield);
void k_solve_z_T(Ctx* c, double* rhs, const double* T, double* const* q, int nfield, int write_rhs);
bool tri_step_fill(Ctx* c, const double betadx[3][2][3], bool f32);
const double* tri_step_enqueue(Ctx* c, bool f32, int* len_out, const float** f32_out);
void k_solve_x_f32(Ctx* c, float* rhs, const float* T, int nfield);
void k_solve_y_f32(Ctx* c, float* rhs, const float* T, int nfield);
// mirror: FP32 copies of the q fields written beside them (field f at mirror + f*cells), or null
void k_solve_z_f32(Ctx* c, float* rhs, const float* T, double* const* q, int nfield, float* mirror);
// fft.cu
void k_phcalc(Ctx* c);
void k_phcalc_f32(Ctx* c, const float* src, float* phi);
// lagr.cu
void lagr_find_centroid_indices(Ctx* c);
void lagr_mls_weight(Ctx* c);
void lagr_mls_force(Ctx* c, const StepParams* dp, bool dense_forces);
void lagr_velforce(Ctx* c);
void lagr_tempforce(Ctx* c);
void lagr_find_probe_indices(Ctx* c);
void lagr_heat_flux(Ctx* c);
void lagr_stefan(Ctx* c, const StepParams* dp);
void lagr_geometry_refresh(Ctx* c, bool imelt);
void lagr_tag_narrow_band(Ctx* c);
void lagr_tag_initial(Ctx* c);
void lagr_particle(Ctx* c, const StepParams* dp);
// m32: base of the FP32 mirrors (precision form; the temperature forcing
// keeps T's mirror equal to the forced field), or null
const double* lagr_particle_fused(Ctx* c, const StepParams* dp, float* m32, StepParams* next,
                                  int next_prologue);
void lagr_substep_prologue(Ctx* c, int slot);
int lagr_take_plan_request(Ctx* c);
void lagr_struct_loads(Ctx* c, const StepParams* dp);
// diag.cu (CalcDissipation, vorticity, calcFluidVelAvgs)
void diag_enqueue(Ctx* c, const double* vcm);
void diag_finish(Ctx* c);
void diag_free(Ctx* c);
// rigid.cu (moving body)
bool rigid_ensure(Ctx* c);
void rigid_pack(Ctx* c, RigidDev* h, bool geom_from_scalars);
void rigid_unpack(Ctx* c, const RigidDev* h, bool pos_from_motion);
void rigid_upload(Ctx* c);
void rigid_download(Ctx* c);
void k_newton_euler(Ctx* c, const StepParams* dp, const double* geom);
void k_update_xyz(Ctx* c, bool centroids);
void k_rigid_publish(Ctx* c, const double* geom, StepParams* next);
void rigid_free(Ctx* c);
void lagr_step_readback(Ctx* c);
void lagr_join(Ctx* c);
void lagr_join_geom(Ctx* c);
void lagr_loads_early(Ctx* c, const StepParams* dp);
bool lagr_fork_enabled(Ctx* c);
void lagr_step_host_finish(Ctx* c);
void lagr_geometry_to_host(Ctx* c);
void lagr_invalidate(Ctx* c);
void lagr_topology_changed(Ctx* c);
bool lagr_remesh_active(Ctx* c);
void lagr_free(Ctx* c);
// ctx.cu
bool ensure_params(Ctx* c);
bool validate_mesh(Ctx* c);
void release(Ctx* c);

}  // namespace mibm
