/*
 * mibm.h -- C-ABI of the GB300 melt_IBM fluid RK3 substep.
 *
 * The reference (kevzhong/melt_IBM, Fortran 90) implements the substep as
 * argument-less *external* subroutines that read and write module globals
 * (param.f90:4-266).  gfortran exports external subroutines as lowercase
 * symbols with a trailing underscore and passes every argument by reference,
 * so the drop-in entry points below keep exactly that shape: a Fortran host
 * that links libmibm.so instead of the reference objects calls the same
 * names with the same arguments.
 *
 * Because the routines take no arguments, the module globals they read are
 * handed over once through a registration layer (mibm_register_*): the host
 * passes the address of each Fortran array (with its bounds) and of each
 * scalar.  The library keeps device mirrors of every registered array;
 * between mibm_sync_from_host_ / mibm_sync_to_host_ calls the device copy is
 * authoritative.  Scalars (al, ga, ro, dt, ...) are read through their
 * registered host address at every call, as the Fortran routines read the
 * module variable.
 *
 * Errors: the reference routines return nothing and `stop` / MPI_Abort on
 * failure (mlsWeight.f90:121-124, particle.f90:206-224).  The drop-ins keep
 * void signatures; failures are recorded and read with mibm_last_status_()
 * and mibm_last_message().  No device trap is ever raised: device-side
 * failures (singular MLS matrix, non-finite field, wait limit) set a flag
 * that the host reads after the launch sequence.  The non-finite guard is
 * the library's own: cfl_ (and mibm_batch_step_, which runs it) reports
 * MIBM_ENONFINITE when an owned cell's velocity or temperature is NaN or
 * Inf, where the reference's max would drop the NaN.
 *
 * Threading: one context per case.  A context is bound to the calling host
 * thread (mibm_context_bind_); every drop-in acts on the bound context.
 */
#ifndef MIBM_H
#define MIBM_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes                                                        */
/* ------------------------------------------------------------------ */
enum {
  MIBM_OK = 0,
  MIBM_EINVAL = 1,     /* bad dimension / argument                        */
  MIBM_ENOTREG = 2,    /* a required array or scalar was not registered   */
  MIBM_ECUDA = 3,      /* CUDA runtime error                              */
  MIBM_ENOMEM = 4,     /* device allocation failed                        */
  MIBM_ESTATE = 5,     /* call out of order (e.g. before mibm_init_)      */
  MIBM_ETIMEOUT = 6,   /* bounded device wait ran out                     */
  MIBM_ENUMERIC = 7,   /* singular MLS matrix (the reference `stop`s)     */
  MIBM_EBUDGET = 8,    /* serving layer: HBM budget refused the case      */
  MIBM_EABORT = 9,     /* body volume below threshold (particle.f90:218)  */
  MIBM_ENONFINITE = 10 /* cfl_ met a non-finite velocity or temperature   */
};

/* ------------------------------------------------------------------ */
/* Registered 3-D fields.  Shapes are the reference's (init.f90:15-83): */
/*   GHOSTED  : (n1, n2,   0:n3m+1)  n1 = n1m+1, n2 = n2m+1             */
/*   DPH      : (n1, n2+1, 0:n3m+1)                                     */
/*   PLAIN    : (n1, n2,   1:n3m)                                       */
/* `base` is the address of element (1,1,klo).                          */
/* ------------------------------------------------------------------ */
enum {
  MIBM_F_VX = 0, MIBM_F_VY = 1, MIBM_F_VZ = 2, MIBM_F_TEMP = 3, MIBM_F_PR = 4,
  MIBM_F_DPH = 5,
  MIBM_F_RHS = 6, MIBM_F_DQ = 7, MIBM_F_QCAP = 8, MIBM_F_HTEMP = 9,
  MIBM_F_RU1 = 10, MIBM_F_RU2 = 11, MIBM_F_RU3 = 12, MIBM_F_RUT = 13,
  MIBM_F_FORCX = 14, MIBM_F_FORCY = 15, MIBM_F_FORCZ = 16,
  MIBM_F_VOFX = 17, MIBM_F_VOFY = 18, MIBM_F_VOFZ = 19, MIBM_F_VOFP = 20,
  MIBM_F_FORXC = 21, MIBM_F_FORYC = 22, MIBM_F_FORZC = 23, MIBM_F_FORTEMP = 24,
  MIBM_F_SDF = 25,
  MIBM_NFIELDS = 26
};

/* Lagrangian mesh arrays (allotri.f90:1-88), single particle.            */
/* Element type is double unless marked (i32) = Fortran default integer /  */
/* logical (4 bytes, .true. = nonzero).                                    */
enum {
  MIBM_M_XYZV = 0,        /* (3, maxnv)                                  */
  MIBM_M_VERT_OF_FACE = 1,/* (3, maxnf)  i32, 1-based                    */
  MIBM_M_TRI_BAR = 2,     /* (3, maxnf)                                  */
  MIBM_M_TRI_NOR = 3,     /* (3, maxnf)                                  */
  MIBM_M_VERT_NOR = 4,    /* (3, maxnv)                                  */
  MIBM_M_SUR = 5,         /* (maxnf)                                     */
  MIBM_M_AVERT = 6,       /* (maxnv)                                     */
  MIBM_M_VEL_TRI = 7,     /* (3, maxnf)                                  */
  MIBM_M_CFAC = 8,        /* (maxnf)                                     */
  MIBM_M_GHOST_FACE = 9,  /* (maxnf)  i32 logical                        */
  MIBM_M_GHOST_VERT = 10, /* (maxnv)  i32 logical                        */
  MIBM_M_PIND = 11,       /* (6, maxnf) i32                              */
  MIBM_M_PTXAB_Q1 = 12,   /* (27, maxnf)                                 */
  MIBM_M_PTXAB_Q2 = 13,
  MIBM_M_PTXAB_Q3 = 14,
  MIBM_M_PTXAB_TEMP = 15,
  MIBM_M_QW_O = 16,       /* (maxnf)                                     */
  MIBM_M_QW_I = 17,
  MIBM_M_QW_OVERT = 18,   /* (maxnv)                                     */
  MIBM_M_QW_IVERT = 19,
  MIBM_M_VMELT = 20,      /* (3, maxnv)                                  */
  MIBM_M_VMELT_M1 = 21,
  MIBM_M_VERT_OF_EDGE = 22,  /* (2, maxne) i32                           */
  MIBM_M_EDGE_OF_FACE = 23,  /* (3, maxnf) i32                           */
  MIBM_M_GHOST_EDGE = 24,    /* (maxne) i32 logical                      */
  MIBM_M_ELENGTHS = 25,      /* (maxne)                                  */
  MIBM_M_SKEWNESS = 26,      /* (maxnf)                                  */
  MIBM_NMESH = 27
};

/* Scalars (double), registered by address.  Vectors take 3 consecutive  */
/* doubles at the registered address; QUAT takes 4 and INERT_TENSOR 9    */
/* (InertTensor(3,3), column-major).                                     */
enum {
  MIBM_S_DT = 0, MIBM_S_AL, MIBM_S_GA, MIBM_S_RO, MIBM_S_BETA,
  MIBM_S_REN, MIBM_S_PEC, MIBM_S_BETAGZ, MIBM_S_TMELT, MIBM_S_TLIQ,
  MIBM_S_TSOL, MIBM_S_LATHEAT, MIBM_S_CPLIQUID, MIBM_S_DTMAX, MIBM_S_CFLFIX,
  MIBM_S_CFLM, MIBM_S_H_EULERIAN, MIBM_S_CELVOL, MIBM_S_VOLUME, MIBM_S_SURFACE,
  MIBM_S_POS_CM, MIBM_S_VEL_CM, MIBM_S_OMEGA_C, MIBM_S_WCON, MIBM_S_WSCL,
  MIBM_S_E_THRESH, MIBM_S_V_THRESH, MIBM_S_DENS_RATIO, MIBM_S_TIME,
  /* HIT forcing parameters (param.f90:16, read from HITForcing.in at    */
  /* papero.f90:52-56): tl, epsstar, kf_on_kmin, C_HIT                   */
  MIBM_S_TL, MIBM_S_EPSSTAR, MIBM_S_KF_ON_KMIN, MIBM_S_C_HIT,
  /* Moving body (imlsstr = 1; param.f90:229-257, allotri.f90:62-83):    */
  /* orientation quaternion, inertia tensor, the surface-integrated       */
  /* pressure / viscous forces and torques of mls_structLoads and their   */
  /* values one substep back, and the load sums kept for output           */
  /* (Fp, Ftau, Torq_p, Torq_tau).                                        */
  MIBM_S_QUAT, MIBM_S_INERT_TENSOR,
  MIBM_S_INT_PRN_DA, MIBM_S_INT_TAU_DA, MIBM_S_INT_R_X_PRN_DA, MIBM_S_INT_R_X_TAU_DA,
  MIBM_S_INT_PRN_DA_M1, MIBM_S_INT_TAU_DA_M1, MIBM_S_INT_R_X_PRN_DA_M1, MIBM_S_INT_R_X_TAU_DA_M1,
  MIBM_S_FP, MIBM_S_FTAU, MIBM_S_TORQ_P, MIBM_S_TORQ_TAU,
  MIBM_NSCALARS
};

/* Integer flags (Fortran default integer / logical), registered by address. */
enum {
  MIBM_I_IMLSFOR = 0, MIBM_I_IMLSSTR, MIBM_I_IMELT, MIBM_I_IREMESH,
  MIBM_I_TAGTYPE, MIBM_I_FORCING, MIBM_I_IDTV, MIBM_I_NTIME,
  MIBM_I_STATIONARY, MIBM_I_NSST,
  MIBM_I_WHICH_HIT,   /* param.f90:17: 1 Eswaran-Pope, 2 ABC                  */
  MIBM_I_HIT_SEED,    /* seed of the forcing's random stream (see below)       */
  MIBM_NINTS
};

/* ------------------------------------------------------------------ */
/* Context, registration, synchronisation                              */
/* ------------------------------------------------------------------ */
int  mibm_context_create_(void);               /* returns id > 0 (bound) */
int  mibm_context_bind_(const int* id);
int  mibm_context_destroy_(const int* id);
int  mibm_last_status_(void);
const char* mibm_last_message(void);

/* Grid of the case: replaces the bou.in read (papero.f90:289-306) and    */
/* cordin (cordin.f90:1-99).  n1m must equal n2m (phcalc.f90:24-33).      */
void mibm_set_grid_(const int* n1m, const int* n2m, const int* n3m,
                    const double* xlen, const double* ylen, const double* zlen);
void mibm_set_mesh_sizes_(const int* maxnv, const int* maxne, const int* maxnf);
void mibm_register_field_(const int* id, double* base);
void mibm_register_mesh_(const int* id, void* base);
void mibm_register_scalar_(const int* id, double* addr);
void mibm_register_int_(const int* id, int* addr);
/* After registration: allocate device mirrors, wavenumbers (phini.f90:4-59),
 * coordinates; copies every registered array host -> device. */
void mibm_init_(void);
/* mask bit b (0..25) selects field b; bit 32+m selects mesh array m.     */
/* An uploaded mesh array is compared word by word with the device copy;   */
/* what the library derived from the mesh (scatter plan, MLS weights, the  */
/* next step's geometry work) is redone only for arrays that changed, and */
/* for uploads of the VOF fields or the signed distance.                   */
void mibm_sync_from_host_(const long long* mask);
void mibm_sync_to_host_(const long long* mask);
/* Page-lock (on = 1) or release (on = 0) the registered host arrays of   */
/* the bound context with cudaHostRegister (mapped), so that mibm_sync_*_  */
/* move them at the host link's speed: the repacking kernels read and     */
/* write the fields in place, the mesh arrays are copied by DMA (no        */
/* counterpart in the reference).  While pinned, the arrays                */
/* must outlive the context or be released first; destroying the context   */
/* releases them.  Arrays the host has already page-locked are left as they */
/* are.  Returns a status.                                                  */
int  mibm_pin_host_(const int* on);
/* Visible CUDA devices (0 without a GPU); kernels launched by the bound
 * context so far (libmibm.so only). */
int  mibm_device_count_(void);
unsigned long long mibm_launch_count_(void);
/* Select the CUDA device for contexts created afterwards by this thread. */
int  mibm_select_device_(const int* dev);
/* Phase timers (the reference's TIMED clocks, tsch.f90:26-84): record CUDA
 * event `slot` (0..63) on the bound context's stream; elapsed milliseconds
 * between two recorded slots (waits for the later one). */
void mibm_timer_mark_(const int* slot);
double mibm_timer_ms_(const int* a, const int* b);
/* Per-kernel profile of the bound context: on = 1 starts (and clears),
 * 0 stops; entries give kernel name, summed event time and launch count. */
void mibm_profile_(const int* on);
int  mibm_profile_count_(void);
int  mibm_profile_get_(const int* idx, char* name, const int* cap, double* total_ms,
                       long long* launches);

/* ------------------------------------------------------------------ */
/* Drop-in routines (reference file:line of the routine each replaces) */
/* ------------------------------------------------------------------ */
void tschem_(void);       /* tsch.f90:1-99  (3 RK3 substeps, fused path)   */
void hdnl1_(void);        /* hdnl1.f90:1-80                                 */
void hdnl2_(void);        /* hdnl2.f90:1-81                                 */
void hdnl3_(void);        /* hdnl3.f90:1-91                                 */
void hdnlte_(void);       /* hdnlte.f90:1-161                               */
void invtr1_(void);       /* invtr1.f90:1-77                                */
void invtr2_(void);       /* invtr2.f90:1-71                                */
void invtr3_(void);       /* invtr3.f90:1-65                                */
void invtrte_(void);      /* invtrte.f90:1-67                               */
void solxi_(const double* betadx);             /* solxi.f90:1-52        */
void solxj_(const double* betadx);             /* solxj.f90:1-40        */
void solxk_(double* q, const double* betadx);  /* solxk.f90:1-60; q =
                              address of vx/vy/vz/temp(1,1,kstart)     */
void divg_(void);         /* divg.f90:1-24                                  */
void phcalc_(void);       /* phcalc.f90:11-97                               */
void updvp_(void);        /* updvp.f90:8-34                                 */
void prcalc_(void);       /* prcalc.f90:5-35                                */
void findcentroidindices_(void);  /* findCentroidIndices.f90:6-53           */
void mlsweight_(void);    /* mlsWeight.f90:1-45 (wght1/2/3/temp)            */
void mlsforce_(void);     /* mlsForce.f90:1-36 (forc1/2/3/forctemp)         */
void velforce_(void);     /* velforce.f90:1-59                              */
void tempforce_(void);    /* tempforce.f90:1-46                             */
void findprobeindices_(void);     /* findProbeIndices.f90:9-76              */
void mls_heatflux_(void); /* mls_heatFlux.f90:1-158 (wght_gradT, faceToVert) */
void apply_stefancondition_(void);/* stefanCondition.f90:1-61               */
void tagcells_(void);     /* tagCells.f90:4-27 (narrow band + interp_vof)   */
void particle_(void);     /* particle.f90:1-230 (forcing, melt, motion,
                             geometry)                                     */
void mls_structloads_(void);  /* mls_structLoads.f90:1-269 (wght_press,
                             wght_gradP/U/V/W): pressure and viscous loads */
void update_part_pos_(void);  /* RigidAuxRoutines.f90:1-54 (newton_euler,
                             calc_rot_matrix, update_xyz; no collisions)   */
void cfl_(void);          /* cfl.f90:1-31                                   */
void get_dt_(void);       /* cfl.f90:33-77                                  */
void interp_(double* arrold, double* arrnew, const int* n1o, const int* n2o,
             const int* n3o, const int* intvar, const int* kstarto,
             const int* kendo);                  /* interp.f90:1-221    */
/* Form of tschem_ (no counterpart in the reference, which is FP64 only):
 * mode 0 = plain FP64 (default); mode 1 = precision form -- FP32 explicit
 * terms, RHS, line solves and FFTs on FP64 fields, with the pressure
 * projection repeated `nproj` times on the FP64 divergence residual. */
void mibm_set_precision_(const int* mode, const int* nproj);
/* mibm_set_tma_: the precision form's y- and z-line solves and the y and z */
/* passes of its 256-point transforms read their lines through bulk tensor  */
/* copies (TMA) into shared memory (1, default) or straight from global     */
/* memory (0).  Both give the same bits; lines longer than 256 cells or     */
/* grids narrower than 32 cells always take the second path.  A staged copy */
/* that does not complete within about a second is reported as             */
/* MIBM_ETIMEOUT by the next cfl_.                                          */
void mibm_set_tma_(const int* on);
/* mibm_set_fused_uvw_: the precision form's one-pass kernels (1, default): */
/* the explicit terms and RHS of u, v, w in one kernel that forms the       */
/* advection products from the velocity mirrors itself, and the velocity   */
/* and pressure updates of each projection in one kernel; 0: the products  */
/* kernel, one RHS kernel per component and separate updates, as in the    */
/* FP64 form.  Both give the same bits.                                     */
void mibm_set_fused_uvw_(const int* on);
/* Step graphs (no counterpart in the reference): from its second call on,  */
/* tschem_ captures its device work into a CUDA graph and replays it while */
/* nothing it reads by value from the host changes (flags, constants, the */
/* form, the mesh's launch sequence); on = 0 launches every kernel         */
/* directly instead.  Results are identical either way.                    */
void mibm_set_graphs_(const int* on);
/* Batched form (no counterpart in the reference, which runs one case per  */
/* MPI job): independent cases -- each its own context after mibm_init_,   */
/* any grid size, either form -- advanced by one iteration of the time     */
/* loop (cfl, get_dt, forcing, tschem; gcurv.f90:151-172) together.  Their  */
/* reductions overlap, their step graphs run as one batch graph (one child */
/* node per case, no edges: the device interleaves them), and each case    */
/* gets exactly the result of stepping it alone.  create returns a handle  */
/* > 0 (0 on error; an empty member list is allowed); step returns a     */
/* status (ntime <= 0: each case uses its own completed-step count + 1).   */
/* A case that fails during a batch step (non-finite field, allocation or  */
/* CUDA error in its own work) is left out of the rest of that step with    */
/* its status kept in its context, and the step returns that status; the  */
/* other cases complete the step exactly as they would alone.  add/remove */
/* change the members between steps (serving: cases join and leave);       */
/* set_launch chooses 0 = one batch graph (default, rebuilt when members   */
/* change) or 1 = each case's own step graph on its own stream (no rebuild */
/* when members change).  Destroy the batch before its contexts.           */
/* Autotuner (no counterpart in the reference): times the feasible chunk    */
/* lengths of the x-, y- and z-line solves and the block heights of the    */
/* explicit-term kernel on the bound context (scratch data; its state is   */
/* unchanged) and keeps the fastest; results are cached per (grid, form)   */
/* for the process and can be saved to / loaded from a text file.  get     */
/* writes the chunk lengths (x, y, z) and block height in use to out[0..3]. */
int  mibm_autotune_(void);
int  mibm_autotune_get_(int* out);
int  mibm_autotune_save_(const char* path);
int  mibm_autotune_load_(const char* path);
int mibm_batch_create_(const int* ids, const int* n);
int mibm_batch_step_(const int* handle, const int* ntime);
int mibm_batch_destroy_(const int* handle);
int mibm_batch_add_(const int* handle, const int* id);
int mibm_batch_remove_(const int* handle, const int* id);
int mibm_batch_set_launch_(const int* handle, const int* mode);
/* max over the owned cells of |div u| as divgck computes it
 * (divg.f90:26-56); synchronises with the device. */
double mibm_divergence_max_(void);
/* Initial full cell tagging at t = 0 (pencil_rayTag.f90:37-165 with the  */
/* narrow band, tagCells.f90:17-23 with initial_tag = .true.).            */
void tagcells_initial_(void);

/* HIT forcing into forcx, forcy, forcz (called once per step before      */
/* tschem_ when forcing = 1, gcurv.f90:164-170).                          */
/* calchitrandomforce_: Eswaran & Pope stochastic forcing, hit.f90:1-126.  */
/*   The Ornstein-Uhlenbeck update of bhat(3,nmodes,nmodes,nmodes) and    */
/*   the solenoidal projection run on the host in the reference's loop    */
/*   order; the DFT sums run on the device.  gfortran's random_number      */
/*   cannot be reproduced, so the Gaussian increments come from this       */
/*   library's stream: splitmix64 seeded with the HIT_SEED integer at the */
/*   first call, u = ((x >> 11) + 1) * 2^-53 in (0, 1], Box-Muller as in   */
/*   hit.f90:40-42 (two draws per direction, modes in l, m, n order).      */
/*   bhat lives in the context; nmodes = 2*floor(kf_on_kmin) + 1.         */
void calchitrandomforce_(void);
/* calcabc_hitforce_: ABC forcing, hit.f90:224-254 (CalcABC_HITForce).    */
void calcabc_hitforce_(void);
/* mibm_hit_modes_: nmodes of the current parameters (InitRandomForce,    */
/* hit.f90:128-150).  mibm_hit_bhat_: copy bhat out of (dir = 0) or into  */
/* (dir = 1) the context, as 2*3*nmodes^3 doubles (re, im) in Fortran     */
/* order bhat(ndir,l,m,n) -- the state WriteRandForcCoef / hdf_read_bhat  */
/* save and restore (hit.f90:256-356).                                    */
int  mibm_hit_modes_(void);
void mibm_hit_bhat_(double* bhat, const int* dir);
/* mibm_hit_rng_: position of the Gaussian-increment stream (the splitmix64 */
/* counter), read (dir = 0; before the first draw: the seed it would take)  */
/* or set (dir = 1).  Saved beside bhat in a continuation so that a        */
/* restarted run draws the increments the uninterrupted run would (the      */
/* reference reseeds at restart, hit.f90:39-42; exact continuation needs    */
/* the stream position).                                                    */
void mibm_hit_rng_(unsigned long long* state, const int* dir);
/* Bounds build (the library compiled with -DMIBM_BOUNDS, a debug build):    */
/* kernels check cell, line, mesh and scatter indices against their arrays;  */
/* an index out of range skips the access and is counted on the device (no  */
/* trap).  mibm_bounds_check_: synchronises, returns the accesses skipped    */
/* since the last call and resets the count (-1: not a bounds build).       */
/* mibm_bounds_selftest_: one planted out-of-range index in a kernel of its */
/* own, checked before the access: 0 when the check caught it, 1 when not, */
/* -1 when not a bounds build.                                              */
int  mibm_bounds_check_(void);
int  mibm_bounds_selftest_(void);
/* mibm_selftest_: checks the library's integer-pipe FP64<->FP32 conversions  */
/* (used by the precision form) against the hardware conversions, bit for  */
/* bit, on edge cases and 2^26 random patterns, and the line-solve factor   */
/* table built on the device (by mibm_solxi_noalloc) against the host's     */
/* build, bit for bit.  Returns the number of mismatches (0 = pass), -1     */
/* without a usable GPU.                                                    */
int  mibm_selftest_(void);
/* Linear forcing (no counterpart in the reference, which offers only the */
/* two forcings above): forc = C_HIT * u at each velocity's own staggered */
/* position, stored as xlen * C_HIT * u so that the reference's explicit  */
/* term adds VOF * C_HIT * u (hdnl1.f90:74 divides forcx by xlen).         */
void mibm_linear_hit_force_(void);

/* Remeshing hand-off (particle.f90:119-160, 196-200).  The remesher edits  */
/* the mesh topology (edge collapses, vertex smoothing: remesh_coarsen.f90,  */
/* remesh_smooth.f90) and stays with the host.  With iremesh = 1 the device  */
/* computes the edge lengths every substep after the body has moved        */
/* (calculate_eLengths, triaux.f90:277-306); when a live edge is shorter    */
/* than E_thresh the library writes the current mesh to the registered     */
/* host arrays (every mesh array; tri_nor from update_tri_normal, and the   */
/* registered Volume set to calculate_volume of that mesh) and calls the    */
/* host's remesher `fn(user)`, which edits those arrays in place and        */
/* returns 0, or nonzero to abort the run (the volume-residual check of     */
/* particle.f90:205-216) -- the library then reports MIBM_EABORT.  The       */
/* library uploads the mesh, rebuilds what depends on its topology, and     */
/* continues the substep: primitive geometry, then update_tri_velocity      */
/* (RigidAuxRoutines.f90:902-928).  A step with iremesh = 1 runs without a  */
/* step graph and reads the trigger once per substep (one host              */
/* synchronisation).  A trigger with no remesher set stops the step with    */
/* MIBM_ESTATE.  mibm_remesh_count_: hand-offs done by the bound context.   */
typedef int (*mibm_remesh_fn)(void* user);
void mibm_set_remesh_callback_(mibm_remesh_fn fn, void* user);
int  mibm_remesh_count_(void);
/* The reference's remesher as host code of the library (remesh.cu): QEM    */
/* edge collapses and vertex deletions (remesh_coarsen.f90:2-760), then     */
/* volume-conserving edge relaxation (remesh_smooth.f90:3-474).  Arrays in */
/* the reference's layouts with 1-based indices: xyzv, vmelt (3, nv),       */
/* tri_nor (3, nf), elengths (ne), vert_of_face, edge_of_face (3, nf),      */
/* vert_of_edge (2, ne), ghost flags (0/1), and face_of_edge (2, ne), which */
/* the caller keeps between calls (rebuilt as partaux.f90:221-245 builds it */
/* when it does not describe the mesh, e.g. all zero).  Returns 0; 1       */
/* topology not preserved, 2 reduced to a tetrahedron, 3 volume residual    */
/* above 1e-14 (the reference's aborts), 4 singular QEM system, 5 a         */
/* neighbour walk failed, 6 bad arguments.  stats (8 doubles, may be NULL): */
/* edge collapses, vertex deletions, edge relaxations, vol_melt,            */
/* vol_coarse, vol_smooth, largest drift, extra volume passes.              */
/* mibm_remesh_builtin_ is the same remesher in the form of a remesh        */
/* callback, on the bound context's registered host arrays (face_of_edge    */
/* kept per context): mibm_set_remesh_callback_(mibm_remesh_builtin_, NULL). */
/* mibm_remesh_stats_: the statistics of its last call on the bound context. */
int mibm_remesh_mesh(int nv, int ne, int nf, double* xyzv, double* tri_nor, double* vmelt, double* elengths,
                     int* vert_of_face, int* edge_of_face, int* vert_of_edge, int* face_of_edge,
                     int* ghost_face, int* ghost_edge, int* ghost_vert, double e_thresh, double* stats);
int  mibm_remesh_builtin_(void* user);
int  mibm_remesh_stats_(double* out);

/* Per-step diagnostics.  The reference's CalcDissipation (diss.f90:11-201), */
/* vorticity (vorticity.f90:1-109) and calcFluidVelAvgs (calcSlipVels.f90:   */
/* 17-181), called after every tschem (gcurv.f90:194-203), sum over the     */
/* fully fluid cells (VOFp = 1) and append the results to text files; here  */
/* they return the same numbers in out[MIBM_NDIAG] (layout below, the       */
/* files' columns after `time`).  As CalcDissipation does, a body that is   */
/* not stationary is re-tagged first (tagCells).                            */
/*   mibm_diagnostics_: computes them now (synchronises with the device).   */
/*   mibm_set_diagnostics_(on): with on = 1 every tschem_ appends the same   */
/*   computation to its device work (and step graph) and reads the results  */
/*   back with the step's own end-of-step copies: no extra synchronisation. */
/*   mibm_diagnostics_get_: the values of the last such step (or of the     */
/*   last mibm_diagnostics_ call).  Status codes returned; MIBM_ESTATE if     */
/*   nothing has computed them yet.                                         */
enum {
  MIBM_D_DISS = 0, MIBM_D_KENERG, MIBM_D_URMS, MIBM_D_ETA, MIBM_D_LAMBDA_T,
  MIBM_D_RE_L, MIBM_D_RE_LAMBDA, MIBM_D_L_INT, MIBM_D_CHI,   /* diss.txt        */
  MIBM_D_ENSTROPHY,                                           /* enstrophy.txt   */
  MIBM_D_NFLUID, MIBM_D_U, MIBM_D_V, MIBM_D_W,
  MIBM_D_UU, MIBM_D_VV, MIBM_D_WW,                            /* fluidAvgVels    */
  MIBM_D_UREL, MIBM_D_VREL, MIBM_D_WREL,
  MIBM_D_UUREL, MIBM_D_VVREL, MIBM_D_WWREL,                   /* rel_velBox.txt  */
  MIBM_D_T, MIBM_D_DT, MIBM_D_DT2,                            /* fluidAvgTemps   */
  MIBM_NDIAG
};
int  mibm_diagnostics_(double* out);
void mibm_set_diagnostics_(const int* on);
int  mibm_diagnostics_get_(double* out);

/* ------------------------------------------------------------------ */
/* Allocation-free x-line solve.  No counterpart in the reference: it is  */
/* for callers whose device memory belongs to someone else -- a CUDA      */
/* Fortran or OpenACC host that passes its own device arrays, or a        */
/* process that has handed all free HBM to a case pool -- and that cannot */
/* let a library call cudaMalloc (it would exceed their budget or fail).  */
/* It runs the same periodic tridiagonal solve as solxi_ in place on       */
/* `rhs`, a device array in the compact layout x fastest with row pitch    */
/* `pitch` (elements), n2m rows and n3m planes, on `stream` (NULL = the   */
/* legacy default stream).  Its only scratch, the line-factor table, is a  */
/* file-scope device array sized for lines up to 512 cells (16.4 KB, held */
/* by every GPU that loads the library until exit); n1m > 512 (or n3m >    */
/* 65535) returns MIBM_EINVAL without launching.  The first call on a      */
/* device looks up that array's device address (once per device, with the */
/* device current): make that first call before any stream capture.  Each */
/* call writes the whole table on `stream` with a one-thread kernel and   */
/* then solves; no host buffer is read.  All calls share the one table:    */
/* calls whose work can overlap on the GPU race on it.  That includes two  */
/* calls made one after the other from the host on DIFFERENT streams: the  */
/* second call's table write can run while the first call's solve still   */
/* reads the table.  Order such calls yourself (an event recorded after   */
/* the first call and waited on by the second stream, or one stream).     */
/* Nothing is allocated: no cudaMalloc, cudaFree or allocating library    */
/* routine.  Returns a status.                                            */
/* ------------------------------------------------------------------ */
int mibm_solxi_noalloc(double* rhs, int n1m, int n2m, int n3m, int pitch, double betadx,
                       void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MIBM_H */
