// ctx.cu -- contexts, registration, device mirrors and host synchronisation.
//
// Replaces the reference's module-global state (param.f90:4-266) and its
// allocation (init.f90:2-88, allotri.f90:1-88, cordin.f90:1-99,
// phini.f90:4-59) with one device context per case.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "common.cuh"

namespace mibm {

void tri_free(Ctx* c);
void fft_free(Ctx* c);

static std::mutex g_mu;
static std::map<int, Ctx*> g_ctx;
static int g_next = 1;
static thread_local Ctx* t_cur = nullptr;
static thread_local int t_status = MIBM_OK;
static thread_local std::string t_msg;

Ctx* current() {
  if (!t_cur) { t_status = MIBM_ESTATE; t_msg = "no context bound"; }
  return t_cur;
}

// registered context of an id, or null (also for destroyed contexts)
Ctx* context_by_id(int id) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_ctx.find(id);
  return it == g_ctx.end() ? nullptr : it->second;
}

int last_status_of_thread() { return t_status; }

void fail(Ctx* c, int st, const std::string& m) {
  t_status = st; t_msg = m;
  if (c && c->status == MIBM_OK) { c->status = st; c->msg = m; }
}

bool cuda_ok(Ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  fail(c, MIBM_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

bool ready(Ctx* c) {
  if (!c) return false;
  if (!c->inited) { fail(c, MIBM_ESTATE, "mibm_init_ not called"); return false; }
  if (c->status != MIBM_OK) return false;
  cudaSetDevice(c->device);
  return true;
}

StepParams host_params(Ctx* c) {
  StepParams p{};
  p.al = c->S(MIBM_S_AL); p.ga = c->S(MIBM_S_GA); p.ro = c->S(MIBM_S_RO);
  p.dt = c->S(MIBM_S_DT); p.beta = c->S(MIBM_S_BETA);
  p.ren = c->S(MIBM_S_REN); p.alre = p.al / p.ren; p.pec = c->S(MIBM_S_PEC);
  p.betagz = c->S(MIBM_S_BETAGZ); p.tliq = c->S(MIBM_S_TLIQ); p.tmelt = c->S(MIBM_S_TMELT);
  for (int d = 0; d < 3; ++d) {
    p.pos[d] = c->hs[MIBM_S_POS_CM][d];
    p.vel[d] = c->hs[MIBM_S_VEL_CM][d];
    p.om[d] = c->hs[MIBM_S_OMEGA_C][d];
  }
  const Grid& g = c->g;
  double* q = p.cd;
  q[kQ1] = g.dx1 * 0.25; q[kQ2] = g.dx2 * 0.25; q[kQ3] = g.dx3 * 0.25;
  q[kH1] = g.dx1 * 0.5; q[kH2] = g.dx2 * 0.5; q[kH3] = g.dx3 * 0.5;
  q[kDQ1] = g.dx1q; q[kDQ2] = g.dx2q; q[kDQ3] = g.dx3q;
  q[kGA] = p.ga; q[kRO] = p.ro; q[kALRE] = p.alre; q[kDT] = p.dt;
  q[kPX1] = g.dx1 * p.al; q[kPX2] = g.dx2 * p.al; q[kPX3] = p.al * g.dx3;
  q[kALPEC] = p.al / p.pec;
  q[kBETAGZ] = p.betagz; q[kTLIQ] = p.tliq;
  q[kXLEN] = g.xlen; q[kYLEN] = g.ylen; q[kZLEN] = g.zlen;
  q[kUP1] = p.al * p.dt * g.dx1; q[kUP2] = p.al * p.dt * g.dx2; q[kUP3] = p.al * p.dt * g.dx3;
  q[kBE] = p.al * p.beta;
  q[kUSDTAL] = 1.0 / (p.dt * p.al);
  q[kGDT] = p.ga * p.dt; q[kRDT] = p.ro * p.dt;
  q[kLV1] = p.alre * p.dt * g.dx1q; q[kLV2] = p.alre * p.dt * g.dx2q; q[kLV3] = p.alre * p.dt * g.dx3q;
  q[kLVC] = 2.0 * (q[kLV1] + q[kLV2] + q[kLV3]);
  const double alpec = p.al / p.pec;
  q[kLT1] = alpec * p.dt * g.dx1q; q[kLT2] = alpec * p.dt * g.dx2q; q[kLT3] = alpec * p.dt * g.dx3q;
  q[kLTC] = 2.0 * (q[kLT1] + q[kLT2] + q[kLT3]);
  q[kPD1] = p.dt * q[kPX1]; q[kPD2] = p.dt * q[kPX2]; q[kPD3] = p.dt * q[kPX3];
  q[kRXLEN] = 1.0 / g.xlen; q[kRYLEN] = 1.0 / g.ylen; q[kRZLEN] = 1.0 / g.zlen;
  q[kPB1] = q[kBE] * g.dx1q; q[kPB2] = q[kBE] * g.dx2q; q[kPB3] = q[kBE] * g.dx3q;
  q[kPBC] = 1.0 + 2.0 * (q[kPB1] + q[kPB2] + q[kPB3]);
  q[kDVI] = g.dx1 * q[kUSDTAL];
  for (int i = 0; i < kNCoef; ++i) p.cf[i] = (float)q[i];
  return p;
}

// ---------------------------------------------------------------------
// host <-> device repacking
// ---------------------------------------------------------------------
// Fortran-layout staging (n1 x ny x nk, klo) -> compact device field.
__global__ void pack_kernel(Grid g, const double* __restrict__ st, int n1, int ny, int koff,
                            double* __restrict__ d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, k = blockIdx.z;
  if (i >= g.n1m) return;
  d[cidx(g, i, j, k)] = st[(size_t)i + (size_t)n1 * ((size_t)j + (size_t)ny * (size_t)(k + koff))];
}

// compact device field -> Fortran staging, rebuilding periodic ghost planes
__global__ void unpack_kernel(Grid g, const double* __restrict__ d, int n1, int ny, int nk, int koff,
                              double* __restrict__ st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, kh = blockIdx.z;          // host plane index 0..nk-1
  if (i >= g.n1m) return;
  int k = kh - koff;                            // compact plane
  k = wrap(k, g.n3m);
  st[(size_t)i + (size_t)n1 * ((size_t)j + (size_t)ny * (size_t)kh)] = d[cidx(g, i, j, k)];
}

__global__ void pad_pack(Grid g, const double* __restrict__ st, int n1, int ny, int koff, int which,
                         double* __restrict__ pad) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (which == 0) {   // vx(n1, j, k)
    if (t >= g.n2m) return;
    pad[t + (size_t)g.n2m * k] = st[(size_t)(n1 - 1) + (size_t)n1 * ((size_t)t + (size_t)ny * (size_t)(k + koff))];
  } else {            // vy(i, n2, k)
    if (t >= g.n1m) return;
    pad[t + (size_t)g.n1m * k] = st[(size_t)t + (size_t)n1 * ((size_t)(g.n2m) + (size_t)ny * (size_t)(k + koff))];
  }
}

__global__ void pad_unpack(Grid g, const double* __restrict__ pad, int n1, int ny, int nk, int koff, int which,
                           double* __restrict__ st) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int kh = blockIdx.y;
  int k = wrap(kh - koff, g.n3m);
  if (which == 0) {
    if (t >= g.n2m) return;
    st[(size_t)(n1 - 1) + (size_t)n1 * ((size_t)t + (size_t)ny * (size_t)kh)] = pad[t + (size_t)g.n2m * k];
  } else {
    if (t >= g.n1m) return;
    st[(size_t)t + (size_t)n1 * ((size_t)(g.n2m) + (size_t)ny * (size_t)kh)] = pad[t + (size_t)g.n1m * k];
  }
}

// Takes an uploaded mesh array into the device copy, word by word, and sets
// bit `id` of *changed when any word differs (bitwise: NaNs compare by
// payload), so that an upload that changes nothing keeps what was derived
// from the mesh.
__global__ void mesh_take_kernel(const unsigned* __restrict__ src, unsigned* __restrict__ dst, size_t n, int id,
                                 int* changed) {
  bool diff = false;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    unsigned v = src[t];
    diff |= v != dst[t];
    dst[t] = v;
  }
  if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(changed, 1 << id);
}

// A page-locked host field (mibm_pin_host_) is read or written by the
// pack/unpack kernels in place over the CPU-GPU link, which moves it faster
// than a staged copy followed by a repacking kernel; otherwise it goes
// through the staging buffer with one contiguous copy.
static void sync_field_from_host(Ctx* c, int id) {
  int ny, klo, nk;
  field_host_shape(c, id, ny, klo, nk);
  int n1 = c->g.n1m + 1;
  size_t bytes = (size_t)n1 * ny * nk * sizeof(double);
  const double* src = c->hf_dev[id];
  if (!src) {
    if (!cuda_ok(c, cudaMemcpyAsync(c->stage, c->hf[id], bytes, cudaMemcpyHostToDevice, c->stream), "H2D field")) return;
    src = c->stage;
  }
  int koff = (klo == 0) ? 1 : 0;   // compact k=0 is host plane index koff
  dim3 grid(div_up(c->g.n1m, 128), c->g.n2m, c->g.n3m);
  pack_kernel<<<grid, 128, 0, c->stream>>>(c->g, src, n1, ny, koff, c->df[id]);
  ++c->launches;
  if (id == MIBM_F_VX || id == MIBM_F_VY) {
    int which = id == MIBM_F_VX ? 0 : 1;
    dim3 pg(div_up(which == 0 ? c->g.n2m : c->g.n1m, 128), c->g.n3m);
    pad_pack<<<pg, 128, 0, c->stream>>>(c->g, src, n1, ny, koff, which, which == 0 ? c->pad_vx : c->pad_vy);
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, "pack");
}

static void sync_field_to_host(Ctx* c, int id) {
  int ny, klo, nk;
  field_host_shape(c, id, ny, klo, nk);
  int n1 = c->g.n1m + 1;
  int koff = (klo == 0) ? 1 : 0;
  // in place into a page-locked host field, else into the staging buffer;
  // either way only the owned cells, the ghost planes and the padding that
  // cfl reads (vx column n1, vy row n2) are written
  double* dst = c->hf_dev[id] ? c->hf_dev[id] : c->stage;
  dim3 grid(div_up(c->g.n1m, 128), c->g.n2m, nk);
  unpack_kernel<<<grid, 128, 0, c->stream>>>(c->g, c->df[id], n1, ny, nk, koff, dst);
  ++c->launches;
  size_t wx = (size_t)c->g.n1m, hy = (size_t)c->g.n2m;
  if (id == MIBM_F_VX || id == MIBM_F_VY) {
    int which = id == MIBM_F_VX ? 0 : 1;
    dim3 pg(div_up(which == 0 ? c->g.n2m : c->g.n1m, 128), nk);
    pad_unpack<<<pg, 128, 0, c->stream>>>(c->g, which == 0 ? c->pad_vx : c->pad_vy, n1, ny, nk, koff, which, dst);
    ++c->launches;
    if (which == 0) wx = n1; else hy = c->g.n2m + 1;
  }
  if (!MIBM_LAUNCH_CHECK(c, "unpack")) return;
  if (c->hf_dev[id]) return;
  cudaMemcpy3DParms p{};
  p.srcPtr = make_cudaPitchedPtr(c->stage, (size_t)n1 * sizeof(double), n1, ny);
  p.dstPtr = make_cudaPitchedPtr(c->hf[id], (size_t)n1 * sizeof(double), n1, ny);
  p.extent = make_cudaExtent(wx * sizeof(double), hy, nk);
  p.kind = cudaMemcpyDeviceToHost;
  cuda_ok(c, cudaMemcpy3DAsync(&p, c->stream), "D2H field");
}

static bool dev_alloc(Ctx* c, void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) { fail(c, MIBM_ENOMEM, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e)); return false; }
  cudaMemsetAsync(*p, 0, bytes, c->stream);
  return true;
}

static void upload_coords(Ctx* c) {
  // cordin.f90:74-97 on extended ranges; index t <-> coordinate index t - off
  const Grid& g = c->g;
  int off = 2 * std::max(g.n1m, g.n3m) + 4;
  c->coord_off = off;
  int len = 3 * off;
  std::vector<double> xc(len), xm(len), yc(len), ym(len), zc(len), zm(len);
  for (int t = 0; t < len; ++t) {
    int i = t - off;
    xc[t] = g.xlen * ((double)(i - 1) / (double)g.n1m);
    yc[t] = g.ylen * ((double)(i - 1) / (double)g.n2m);
    zc[t] = g.zlen * ((double)(i - 1) / (double)g.n3m);
    xm[t] = (g.xlen * ((double)(i - 1) / (double)g.n1m) + g.xlen * ((double)i / (double)g.n1m)) * 0.5;
    ym[t] = (g.ylen * ((double)(i - 1) / (double)g.n2m) + g.ylen * ((double)i / (double)g.n2m)) * 0.5;
    zm[t] = (g.zlen * ((double)(i - 1) / (double)g.n3m) + g.zlen * ((double)i / (double)g.n3m)) * 0.5;
  }
  double** dst[6] = {&c->xc, &c->xm, &c->yc, &c->ym, &c->zc, &c->zm};
  std::vector<double>* src[6] = {&xc, &xm, &yc, &ym, &zc, &zm};
  for (int q = 0; q < 6; ++q) {
    if (!dev_alloc(c, (void**)dst[q], len * sizeof(double), "coords")) return;
    cudaMemcpyAsync(*dst[q], src[q]->data(), len * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  }
  cudaStreamSynchronize(c->stream);
}

static void upload_wavenumbers(Ctx* c) {
  // phini.f90:28-56, evaluated exactly as the reference orders the operations
  const Grid& g = c->g;
  double pi = 2.0 * std::asin(1.0);
  auto mk = [&](int n, double len, std::vector<double>& ak) {
    int nh = n / 2 + 1, np = nh + 1;
    std::vector<double> a(n + 1);
    for (int i = 1; i <= nh; ++i) a[i] = (double)(i - 1) * 2.0 * pi;
    for (int i = np; i <= n; ++i) a[i] = (double)(-(n - i + 1)) * 2.0 * pi;
    ak.resize(n);
    double f = (double)n / len;
    for (int i = 1; i <= n; ++i) ak[i - 1] = 2.0 * (1.0 - std::cos(a[i] / n)) * (f * f);
  };
  std::vector<double> a1, a2, a3;
  mk(g.n1m, g.xlen, a1); mk(g.n2m, g.ylen, a2); mk(g.n3m, g.zlen, a3);
  if (!dev_alloc(c, (void**)&c->ak1, a1.size() * 8, "ak1")) return;
  if (!dev_alloc(c, (void**)&c->ak2, a2.size() * 8, "ak2")) return;
  if (!dev_alloc(c, (void**)&c->ak3, a3.size() * 8, "ak3")) return;
  cudaMemcpyAsync(c->ak1, a1.data(), a1.size() * 8, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->ak2, a2.data(), a2.size() * 8, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->ak3, a3.data(), a3.size() * 8, cudaMemcpyHostToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
}

bool ensure_params(Ctx* c) {
  if (c->dparams) return true;
  if (!dev_alloc(c, (void**)&c->dparams, 4 * sizeof(StepParams), "params")) return false;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->hparams, 4 * sizeof(StepParams)), "pinned params")) return false;
  return true;
}

static void unpin_host(Ctx* c) {
  if (c->stream) cudaStreamSynchronize(c->stream);      // no kernel still reads or writes them
  for (void* p : c->pinned) cudaHostUnregister(p);
  c->pinned.clear();
  for (int i = 0; i < MIBM_NFIELDS; ++i) c->hf_dev[i] = nullptr;
  cudaGetLastError();
}

void release(Ctx* c) {
  cudaSetDevice(c->device);
  unpin_host(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  for (int i = 0; i < MIBM_NFIELDS; ++i) cudaFree(c->df[i]);
  for (int i = 0; i < MIBM_NMESH; ++i) cudaFree(c->dm[i]);
  cudaFree(c->pad_vx); cudaFree(c->pad_vy); cudaFree(c->stage); cudaFree(c->spec); cudaFree(c->mesh_stage);
  cudaFree(c->ak1); cudaFree(c->ak2); cudaFree(c->ak3);
  cudaFree(c->xc); cudaFree(c->xm); cudaFree(c->yc); cudaFree(c->ym); cudaFree(c->zc); cudaFree(c->zm);
  cudaFree(c->red); cudaFree(c->dflag); cudaFree(c->dparams); cudaFree(c->rhs4);
  cudaFree(c->ru32); cudaFree(c->rhs32); cudaFree(c->phi32); cudaFree(c->divmax);
  cudaFree(c->res32); cudaFree(c->vel1); cudaFree(c->q32); cudaFree(c->prod); cudaFree(c->prod32);
  cudaFree(c->tri_coef); cudaFree(c->lag_red);
  if (c->red_host) cudaFreeHost(c->red_host);
  if (c->hflag) cudaFreeHost(c->hflag);
  if (c->step_host) cudaFreeHost(c->step_host);
  if (c->hparams) cudaFreeHost(c->hparams);
  for (int q = 0; q < 64; ++q)
    if (c->timers[q]) cudaEventDestroy(c->timers[q]);
  prof_release(c);
  lagr_free(c);
  tri_free(c);
  fft_free(c);
  hit_free(c);
  rigid_free(c);
  diag_free(c);
  if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
  if (c->side2) { cudaStreamSynchronize(c->side2); cudaStreamDestroy(c->side2); }
  if (c->side3) { cudaStreamSynchronize(c->side3); cudaStreamDestroy(c->side3); }
  if (c->tsolve) { cudaStreamSynchronize(c->tsolve); cudaStreamDestroy(c->tsolve); }
  if (c->ev_sfork) cudaEventDestroy(c->ev_sfork);
  if (c->ev_sjoin) cudaEventDestroy(c->ev_sjoin);
  if (c->ev_wfork) cudaEventDestroy(c->ev_wfork);
  if (c->ev_wjoin) cudaEventDestroy(c->ev_wjoin);
  if (c->ev_tfork) cudaEventDestroy(c->ev_tfork);
  if (c->ev_tjoin) cudaEventDestroy(c->ev_tjoin);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_pub) cudaEventDestroy(c->ev_pub);
  if (c->ev_gfork) cudaEventDestroy(c->ev_gfork);
  if (c->ev_lfork) cudaEventDestroy(c->ev_lfork);
  if (c->ev_ldone) cudaEventDestroy(c->ev_ldone);
  if (c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace mibm

using namespace mibm;

extern "C" {

int mibm_context_create_(void) {
  Ctx* c = new Ctx();
  {
    std::lock_guard<std::mutex> g(g_mu);
    c->id = g_next++;
    g_ctx[c->id] = c;
  }
  cudaGetDevice(&c->device);
  // The IBM streams (side, side2, side3) carry chains of small latency-bound
  // kernels that the main stream waits for at its joins; at the greatest
  // priority their blocks take SM slots as soon as they free up, beside the
  // main stream's large grids (256^3 FP64 step 26.48 -> 26.12 ms, 128^3 free
  // body 3.94 -> 3.87 ms FP64 and 2.21 -> 2.12 ms precision form; the main
  // stream at the greatest priority instead: slower).  The step graphs keep
  // these priorities per node (cudaGraphInstantiateFlagUseNodePriority).
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  const int p_main = prio_least, p_side = prio_greatest;
  if (!cuda_ok(c, cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, p_main), "stream") ||
      !cuda_ok(c, cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, p_side), "stream") ||
      !cuda_ok(c, cudaStreamCreateWithPriority(&c->side2, cudaStreamNonBlocking, p_side), "stream") ||
      !cuda_ok(c, cudaStreamCreateWithPriority(&c->side3, cudaStreamNonBlocking, p_side), "stream") ||
      !cuda_ok(c, cudaStreamCreateWithPriority(&c->tsolve, cudaStreamNonBlocking, p_main), "stream") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_sfork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_sjoin, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_wfork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_wjoin, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_tfork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_tjoin, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_pub, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_gfork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_lfork, cudaEventDisableTiming), "event") ||
      !cuda_ok(c, cudaEventCreateWithFlags(&c->ev_ldone, cudaEventDisableTiming), "event")) {
    t_cur = c;
    return -MIBM_ECUDA;
  }
  t_cur = c;
  return c->id;
}

int mibm_context_bind_(const int* id) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_ctx.find(*id);
  if (it == g_ctx.end()) { t_status = MIBM_EINVAL; t_msg = "unknown context"; return MIBM_EINVAL; }
  t_cur = it->second;
  cudaSetDevice(t_cur->device);
  return MIBM_OK;
}

int mibm_context_destroy_(const int* id) {
  Ctx* c = nullptr;
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_ctx.find(*id);
    if (it == g_ctx.end()) return MIBM_EINVAL;
    c = it->second;
    g_ctx.erase(it);
  }
  if (t_cur == c) t_cur = nullptr;
  release(c);
  delete c;
  return MIBM_OK;
}

int mibm_last_status_(void) { return t_cur ? t_cur->status : t_status; }
const char* mibm_last_message(void) { return t_cur ? t_cur->msg.c_str() : t_msg.c_str(); }

void mibm_set_grid_(const int* n1m, const int* n2m, const int* n3m, const double* xlen, const double* ylen,
                    const double* zlen) {
  Ctx* c = current(); if (!c) return;
  if (*n1m < 8 || *n2m < 8 || *n3m < 8 || *n1m != *n2m || (*n1m % 2) || (*n3m % 2)) {
    fail(c, MIBM_EINVAL, "grid: need n1m == n2m, even, >= 8 and n3m even >= 8");
    return;
  }
  auto radix_ok = [](int n) { while (n % 2 == 0) n /= 2; while (n % 3 == 0) n /= 3; return n == 1; };
  if (!radix_ok(*n1m) || !radix_ok(*n3m) || *n1m > 512 || *n3m > 512) {
    fail(c, MIBM_EINVAL, "grid: sizes must be 2^a 3^b and <= 512 (phcalc FFT)");
    return;
  }
  Grid& g = c->g;
  g.n1m = *n1m; g.n2m = *n2m; g.n3m = *n3m;
  g.P = (g.n1m + 3) / 4 * 4;
  g.plane = (size_t)g.P * g.n2m; g.cells = g.plane * g.n3m;
  g.xlen = *xlen; g.ylen = *ylen; g.zlen = *zlen;
  g.dx1 = (double)g.n1m / g.xlen; g.dx2 = (double)g.n2m / g.ylen; g.dx3 = (double)g.n3m / g.zlen;
  g.dx1q = g.dx1 * g.dx1; g.dx2q = g.dx2 * g.dx2; g.dx3q = g.dx3 * g.dx3;
  g.H = g.n1m / 2 + 1; g.HP = (g.H + 7) / 8 * 8;
  c->grid_set = true;
}

void mibm_set_mesh_sizes_(const int* maxnv, const int* maxne, const int* maxnf) {
  Ctx* c = current(); if (!c) return;
  if (*maxnv < 0 || *maxne < 0 || *maxnf < 0 || *maxnf > (1 << 24)) { fail(c, MIBM_EINVAL, "mesh sizes"); return; }
  c->maxnv = *maxnv; c->maxne = *maxne; c->maxnf = *maxnf;
}

void mibm_register_field_(const int* id, double* base) {
  Ctx* c = current(); if (!c) return;
  if (*id < 0 || *id >= MIBM_NFIELDS) { fail(c, MIBM_EINVAL, "register_field: bad id"); return; }
  c->hf[*id] = base;
  c->hf_dev[*id] = nullptr;          // a new array is not the page-locked one
}
void mibm_register_mesh_(const int* id, void* base) {
  Ctx* c = current(); if (!c) return;
  if (*id < 0 || *id >= MIBM_NMESH) { fail(c, MIBM_EINVAL, "register_mesh: bad id"); return; }
  c->hm[*id] = base;
}
void mibm_register_scalar_(const int* id, double* addr) {
  Ctx* c = current(); if (!c) return;
  if (*id < 0 || *id >= MIBM_NSCALARS) { fail(c, MIBM_EINVAL, "register_scalar: bad id"); return; }
  c->hs[*id] = addr;
}
void mibm_register_int_(const int* id, int* addr) {
  Ctx* c = current(); if (!c) return;
  if (*id < 0 || *id >= MIBM_NINTS) { fail(c, MIBM_EINVAL, "register_int: bad id"); return; }
  c->hi[*id] = addr;
}

void mibm_init_(void) {
  Ctx* c = current(); if (!c) return;
  if (!c->grid_set) { fail(c, MIBM_ESTATE, "mibm_set_grid_ not called"); return; }
  for (int i = 0; i < MIBM_NFIELDS; ++i)
    if (!c->hf[i]) { fail(c, MIBM_ENOTREG, "field " + std::to_string(i) + " not registered"); return; }
  for (int i = 0; i < MIBM_NSCALARS; ++i)
    if (!c->hs[i]) { fail(c, MIBM_ENOTREG, "scalar " + std::to_string(i) + " not registered"); return; }
  for (int i = 0; i < MIBM_NINTS; ++i)
    if (!c->hi[i]) { fail(c, MIBM_ENOTREG, "int " + std::to_string(i) + " not registered"); return; }
  if (c->maxnf > 0)
    for (int i = 0; i < MIBM_NMESH; ++i)
      if (!c->hm[i]) { fail(c, MIBM_ENOTREG, "mesh array " + std::to_string(i) + " not registered"); return; }
  cudaSetDevice(c->device);
  const Grid& g = c->g;
  for (int i = 0; i < MIBM_NFIELDS; ++i)
    if (!dev_alloc(c, (void**)&c->df[i], g.cells * sizeof(double), "field")) return;
  if (!dev_alloc(c, (void**)&c->pad_vx, (size_t)g.n2m * g.n3m * 8, "pad")) return;
  if (!dev_alloc(c, (void**)&c->pad_vy, (size_t)g.n1m * g.n3m * 8, "pad")) return;
  c->stage_bytes = (size_t)(g.n1m + 1) * (g.n2m + 2) * (g.n3m + 2) * sizeof(double);
  if (!dev_alloc(c, (void**)&c->stage, c->stage_bytes, "staging")) return;
  if (!dev_alloc(c, (void**)&c->spec, (size_t)g.HP * g.n2m * g.n3m * sizeof(double2), "spectrum")) return;
  c->red_elems = kRedPart + 3 * (size_t)g.n2m * g.n3m + 1024;
  if (!dev_alloc(c, (void**)&c->red, c->red_elems * sizeof(double), "reduction")) return;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->red_host, 4096), "pinned")) return;
  if (!dev_alloc(c, (void**)&c->dflag, 64, "flags")) return;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->hflag, 64), "pinned")) return;
  if (!cuda_ok(c, cudaMallocHost((void**)&c->step_host, 32 * sizeof(double)), "pinned")) return;
  memset(c->hflag, 0, 64);
  size_t mesh_max = 0;
  for (int i = 0; i < MIBM_NMESH; ++i) {
    size_t b = mesh_bytes(c, i);
    if (b == 0) continue;
    if (!dev_alloc(c, &c->dm[i], b, "mesh")) return;
    mesh_max = std::max(mesh_max, b);
  }
  if (mesh_max && !dev_alloc(c, &c->mesh_stage, mesh_max, "mesh staging")) return;
  if (!ensure_params(c)) return;
  upload_coords(c);
  if (c->status != MIBM_OK) return;
  upload_wavenumbers(c);
  c->inited = true;
  long long all = -1;
  mibm_sync_from_host_(&all);
  cudaStreamSynchronize(c->stream);
  lagr_topology_changed(c);            // nothing derived from the mesh exists yet
  if (c->maxnf > 0 && !validate_mesh(c)) c->inited = false;
}

void mibm_sync_from_host_(const long long* mask) {
  Ctx* c = current(); if (!ready(c)) return;
  unsigned long long m = (unsigned long long)*mask;
  for (int i = 0; i < MIBM_NFIELDS; ++i)
    if (m & (1ull << i)) sync_field_from_host(c, i);
  precision_after_upload(c, m);
  const bool mesh_up = c->maxnf > 0 && (m >> 32) != 0;
  int* changed = c->dflag + 4;         // bit i: mesh array i differs from the device copy
  if (mesh_up) cudaMemsetAsync(changed, 0, sizeof(int), c->stream);
  for (int i = 0; i < MIBM_NMESH && mesh_up; ++i) {
    size_t bytes = mesh_bytes(c, i);
    if (!((m >> 32) & (1ull << i)) || bytes == 0) continue;
    if (!cuda_ok(c, cudaMemcpyAsync(c->mesh_stage, c->hm[i], bytes, cudaMemcpyHostToDevice, c->stream), "H2D mesh"))
      return;
    size_t words = bytes / 4;
    mesh_take_kernel<<<std::min<size_t>(div_up(words, 256), 1024), 256, 0, c->stream>>>(
        (const unsigned*)c->mesh_stage, (unsigned*)c->dm[i], words, i, changed);
    ++c->launches;
  }
  if (mesh_up) {
    MIBM_LAUNCH_CHECK(c, "mesh upload");
    cudaMemcpyAsync(c->hflag + 4, changed, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  }
  if (!cuda_ok(c, cudaStreamSynchronize(c->stream), "sync_from_host")) return;
  const unsigned long long mchg = mesh_up ? (unsigned long long)(unsigned)c->hflag[4] : 0ull;
  // what the next step's geometry-only work reads from the fields: the
  // volume fractions (narrow-band tagging updates VOFp in place) and the
  // signed distance; the scatter plan and the MLS weights depend on the
  // mesh, the vertex->face lists on its connectivity
  const unsigned long long geom_fields = (1ull << MIBM_F_VOFX) | (1ull << MIBM_F_VOFY) | (1ull << MIBM_F_VOFZ) |
                                         (1ull << MIBM_F_VOFP) | (1ull << MIBM_F_SDF);
  const unsigned long long topo = (1ull << MIBM_M_VERT_OF_FACE) | (1ull << MIBM_M_GHOST_FACE);
  if (m & geom_fields) ++c->geom_gen;
  if (mchg & topo) lagr_topology_changed(c);
  else if (mchg) lagr_invalidate(c);
  if (c->maxnf > 0 && (mchg & topo)) validate_mesh(c);
}

void mibm_sync_to_host_(const long long* mask) {
  Ctx* c = current(); if (!ready(c)) return;
  unsigned long long m = (unsigned long long)*mask;
  precision_before_download(c, m);
  for (int i = 0; i < MIBM_NFIELDS; ++i)
    if (m & (1ull << i)) sync_field_to_host(c, i);
  for (int i = 0; i < MIBM_NMESH && c->maxnf > 0; ++i)
    if ((m >> 32) & (1ull << i))
      cuda_ok(c, cudaMemcpyAsync(c->hm[i], c->dm[i], mesh_bytes(c, i), cudaMemcpyDeviceToHost, c->stream), "D2H mesh");
  cuda_ok(c, cudaStreamSynchronize(c->stream), "sync_to_host");
}

int mibm_pin_host_(const int* on) {
  Ctx* c = current(); if (!ready(c)) return c ? c->status : MIBM_ESTATE;
  if (!*on) { unpin_host(c); return MIBM_OK; }
  if (!c->pinned.empty()) return MIBM_OK;
  auto pin = [&](void* p, size_t bytes) {
    if (!p || bytes == 0) return false;
    cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped);
    if (e == cudaSuccess) { c->pinned.push_back(p); return true; }
    cudaGetLastError();                    // already page-locked, or not registrable: copies stay pageable
    return false;
  };
  for (int id = 0; id < MIBM_NFIELDS; ++id) {
    int ny, klo, nk;
    field_host_shape(c, id, ny, klo, nk);
    if (pin(c->hf[id], (size_t)(c->g.n1m + 1) * ny * nk * sizeof(double))) {
      void* dp = nullptr;
      if (cudaHostGetDevicePointer(&dp, c->hf[id], 0) == cudaSuccess) c->hf_dev[id] = (double*)dp;
      else cudaGetLastError();
    }
  }
  for (int i = 0; i < MIBM_NMESH && c->maxnf > 0; ++i) pin(c->hm[i], mesh_bytes(c, i));
  return MIBM_OK;
}

// Number of CUDA devices visible to this process (0 on a host without a
// GPU or driver); lets a caller choose its path before creating a context.
int mibm_device_count_(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

int mibm_select_device_(const int* dev) {
  cudaError_t e = cudaSetDevice(*dev);
  if (e != cudaSuccess) { t_status = MIBM_ECUDA; t_msg = cudaGetErrorString(e); return MIBM_ECUDA; }
  return MIBM_OK;
}

void mibm_timer_mark_(const int* slot) {
  Ctx* c = current(); if (!c || *slot < 0 || *slot >= 64) return;
  if (!c->timers[*slot] && !cuda_ok(c, cudaEventCreate(&c->timers[*slot]), "event")) return;
  cuda_ok(c, cudaEventRecord(c->timers[*slot], c->stream), "event record");
}

double mibm_timer_ms_(const int* a, const int* b) {
  Ctx* c = current();
  if (!c || *a < 0 || *a >= 64 || *b < 0 || *b >= 64 || !c->timers[*a] || !c->timers[*b]) return -1.0;
  if (!cuda_ok(c, cudaEventSynchronize(c->timers[*b]), "event sync")) return -1.0;
  float ms = 0.f;
  if (!cuda_ok(c, cudaEventElapsedTime(&ms, c->timers[*a], c->timers[*b]), "event elapsed")) return -1.0;
  return (double)ms;
}

// Number of kernels launched through the bound context (for the benchmark's
// launch count).
unsigned long long mibm_launch_count_(void) {
  Ctx* c = current();
  return c ? c->launches : 0;
}

}  // extern "C"
