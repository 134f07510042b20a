// tridiag.cu -- periodic tridiagonal line solves of the approximate
// factorisation (solxi.f90:30-44, solxj.f90:17-31, solxk.f90:20-50).
//
// The reference assembles, for every line, the constant-coefficient system
//   -G/(1+2G) x_{i-1} + x_i - G/(1+2G) x_{i+1} = rhs_i/(1+2G)   (periodic)
// and solves it with tridiag_periodic.f90:1-60 (Thomas sweep plus a
// periodic closure).  Every quantity of that algorithm that does not involve
// the right-hand side (q, s, the pivots p and the closure denominator) is the
// same for all N^2 lines, so it is evaluated once on the host, in the same
// operation order as the reference, and the device only runs the three
// data-dependent recurrences:
//   forward   y_i = a_i r_i - b_i y_{i-1}      (a_i = p_i/(1+2G), b_i = ami p_i)
//   backward  f_i = y_i + q_i f_{i+1}
//   closure   x_n = (r_n/(1+2G) - api f_1 - ami f_{n-1}) / den
//             x_i = x_n s_i + f_i
// = 4 FP64 operations per element, one read and one write of the line.
//
// Main path (chunked solves): a line of n cells is cut into G chunks of M
// cells and each thread keeps one chunk in registers.  The two recurrences
// are linear, so a chunk runs them from a zero entry value and corrects
// afterwards with its true entry value times a factor that depends on the
// table only (prefix products of -b, suffix products of q):
//   forward   C_e = a_e r_e - b_e C_{e-1}          y_e = C_e + P_e y_in
//   backward  D_e = C_e + q_e D_{e+1}              f_e = D_e + DP_e y_in + Q_e f_in
// with P_e = prod(-b) from the chunk start to e, Q_e = prod(q) from e to the
// chunk end and DP_e = P_e + q_e DP_{e+1}.  The entry values y_in, f_in of
// the chunks are a scan over the chunk end values: warp shuffles for
// x-lines (one warp per line, lane = chunk, contiguous vector loads), shared
// memory for y- and z-lines (lane = adjacent i, warp = chunk, coalesced
// rows).  The last cell of the line joins the last chunk through zero
// coefficients (a = b = q = 0, s = 1), so every chunk is alike.  Rounding
// differs from the sequential sweep only in summation order.
//
// Fallback (line lengths the chunking does not split, and the allocation-
// free entry point): lines staged through shared memory in tiles of 32
// lines, one thread running one line's sequential sweep.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fpconv.cuh"
#include "tma.cuh"

namespace mibm {

struct TriTable {
  int n = 0;
  double betadx = -1.0;
  std::vector<double> h;      // [a | b | q | s] * n, then ackl_b, api, ami, inv_den
};

// IEEE round-to-nearest operations in source order on both sides.  The host
// side is compiled without floating-point contraction; the device side uses
// the explicitly rounded intrinsics, which are never fused into FMAs.  The
// two evaluations of tri_factors are therefore bit-identical.
__host__ __device__ __forceinline__ double tf_mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ __forceinline__ double tf_add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ __forceinline__ double tf_div(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// The line-independent part of tridiag_periodic.f90:22-49 for the system of
// solxi.f90:30-44 (diagonal 1, off-diagonals -G/(1+2G), rhs scaled by
// 1/(1+2G)), written into t[0 .. 4n+3] without any other storage:
//   t[0..n)    a_i = (1/(1+2G)) p_i   (a_1 = (1/(1+2G)) / aci)
//   t[n..2n)   b_i = ami p_i          (b_1 = 0)
//   t[2n..3n)  q_i,  t[3n..4n)  s_i (after the backward pass of :45-46)
//   t[4n..4n+3] 1/(1+2G), api, ami, 1/den (den of :47-49)
// with the pivots p_i = 1/(aci + ami q_{i-1}) formed and used in place.
__host__ __device__ inline void tri_factors(int n, double betadx, double* t) {
  const double ackl_b = tf_div(1.0, tf_add(1.0, tf_mul(2.0, betadx)));
  const double api = tf_mul(-betadx, ackl_b), ami = tf_mul(-betadx, ackl_b), aci = 1.0;
  double* a = t;
  double* b = t + n;
  double* q = t + 2 * n;
  double* s = t + 3 * n;
  q[0] = tf_div(-api, aci);
  s[0] = tf_div(-ami, aci);
  a[0] = tf_div(ackl_b, aci);
  b[0] = 0.0;
  for (int i = 1; i < n; ++i) {
    const double p = tf_div(1.0, tf_add(aci, tf_mul(ami, q[i - 1])));
    q[i] = tf_mul(-api, p);
    s[i] = tf_mul(tf_mul(-ami, s[i - 1]), p);
    a[i] = tf_mul(ackl_b, p);
    b[i] = tf_mul(ami, p);
  }
  s[n - 1] = 1.0;
  for (int i = n - 2; i >= 0; --i) s[i] = tf_add(s[i], tf_mul(q[i], s[i + 1]));
  const double den = tf_add(tf_add(tf_mul(api, s[0]), tf_mul(ami, s[n - 2])), aci);
  t[4 * n + 0] = ackl_b;
  t[4 * n + 1] = api;
  t[4 * n + 2] = ami;
  t[4 * n + 3] = tf_div(1.0, den);
}

// Host evaluation of the factor table.
static void build_table(int n, double betadx, std::vector<double>& t) {
  t.assign(4 * (size_t)n + 4, 0.0);
  tri_factors(n, betadx, t.data());
}

// the factor table of build_table for callers outside this file (the z-line
// Poisson solve of fft.cu)
void tri_build_table(int n, double betadx, std::vector<double>& t) { build_table(n, betadx, t); }

static size_t slot_len(int nmax);
static void fill_slot(int n, int m, double betadx, double* out);
int tri_chunk(Ctx* c, int dir);

// Device table cache: small ring of slots, refilled when (n, betadx) changes.
struct TriCache {
  double* dev = nullptr;
  double* pinned = nullptr;
  int slots = 0, len = 0, next = 0;
  std::vector<int> n, m;
  std::vector<double> bd;
};

struct CtxTri {
  TriCache cache;
};

static std::vector<std::pair<Ctx*, CtxTri*>> g_tri;

static CtxTri* tri_of(Ctx* c) {
  for (auto& e : g_tri)
    if (e.first == c) return e.second;
  CtxTri* t = new CtxTri();
  g_tri.emplace_back(c, t);
  return t;
}

// Returns a device pointer to the table of (n, betadx).  The table is
// written to a pinned slot and copied on the context stream, so the value is
// stream-ordered with the solve that uses it.
static const double* table_for(Ctx* c, int dir, double betadx) {
  const int n = dir == 0 ? c->g.n1m : (dir == 1 ? c->g.n2m : c->g.n3m);
  const int m = tri_chunk(c, dir);
  TriCache& tc = tri_of(c)->cache;
  int nmax = std::max(c->g.n1m, c->g.n3m);
  if (!tc.dev) {
    tc.slots = 64;
    tc.len = (int)slot_len(nmax);
    if (!cuda_ok(c, cudaMalloc(&tc.dev, sizeof(double) * tc.len * tc.slots), "tri table")) return nullptr;
    if (!cuda_ok(c, cudaMallocHost(&tc.pinned, sizeof(double) * tc.len * tc.slots), "tri table")) return nullptr;
    tc.n.assign(tc.slots, -1);
    tc.m.assign(tc.slots, -1);
    tc.bd.assign(tc.slots, -1.0);
  }
  for (int s = 0; s < tc.slots; ++s)
    if (tc.n[s] == n && tc.m[s] == m && tc.bd[s] == betadx) return tc.dev + (size_t)s * tc.len;
  int s = tc.next;
  tc.next = (tc.next + 1) % tc.slots;
  // a slot may still be read by an in-flight kernel: order the refill on the stream
  cudaStreamSynchronize(c->stream);
  fill_slot(n, m, betadx, tc.pinned + (size_t)s * tc.len);
  cudaMemcpyAsync(tc.dev + (size_t)s * tc.len, tc.pinned + (size_t)s * tc.len, sizeof(double) * tc.len,
                  cudaMemcpyHostToDevice, c->stream);
  tc.n[s] = n;
  tc.m[s] = m;
  tc.bd[s] = betadx;
  return tc.dev + (size_t)s * tc.len;
}

static void steptab_free(Ctx* c);

static void tmaps_free(Ctx* c);

void tri_free(Ctx* c) {
  steptab_free(c);
  tmaps_free(c);
  for (size_t q = 0; q < g_tri.size(); ++q)
    if (g_tri[q].first == c) {
      cudaFree(g_tri[q].second->cache.dev);
      cudaFreeHost(g_tri[q].second->cache.pinned);
      delete g_tri[q].second;
      g_tri.erase(g_tri.begin() + q);
      return;
    }
}

// One thread: solve the line held in shared memory at base[e*stride],
// e = 0..n-1, with the factor table T (also in shared memory).  The loops
// are unrolled by 4 with the independent loads (line values and factors)
// issued ahead of the dependent FMA chain.
template <typename V>
__device__ __forceinline__ void solve_line(V* base, int stride, int n, const V* __restrict__ T) {
  const V* a = T;
  const V* b = T + n;
  const V* q = T + 2 * n;
  const V* s = T + 3 * n;
  V ackl_b = T[4 * n + 0], api = T[4 * n + 1], ami = T[4 * n + 2], inv_den = T[4 * n + 3];
  V rn = base[(size_t)(n - 1) * stride];
  V y = a[0] * base[0];
  base[0] = y;
  int e = 1;
  for (; e + 4 <= n - 1; e += 4) {
    V r0 = base[(size_t)e * stride], r1 = base[(size_t)(e + 1) * stride];
    V r2 = base[(size_t)(e + 2) * stride], r3 = base[(size_t)(e + 3) * stride];
    V a0 = a[e] * r0, a1 = a[e + 1] * r1, a2 = a[e + 2] * r2, a3 = a[e + 3] * r3;
    y = a0 - b[e] * y;     base[(size_t)e * stride] = y;
    y = a1 - b[e + 1] * y; base[(size_t)(e + 1) * stride] = y;
    y = a2 - b[e + 2] * y; base[(size_t)(e + 2) * stride] = y;
    y = a3 - b[e + 3] * y; base[(size_t)(e + 3) * stride] = y;
  }
  for (; e < n - 1; ++e) {
    y = a[e] * base[(size_t)e * stride] - b[e] * y;
    base[(size_t)e * stride] = y;
  }
  V f = V(0.0);   // f_n = 0
  e = n - 2;
  for (; e - 3 >= 0; e -= 4) {
    V y0 = base[(size_t)e * stride], y1 = base[(size_t)(e - 1) * stride];
    V y2 = base[(size_t)(e - 2) * stride], y3 = base[(size_t)(e - 3) * stride];
    f = y0 + q[e] * f;     base[(size_t)e * stride] = f;
    f = y1 + q[e - 1] * f; base[(size_t)(e - 1) * stride] = f;
    f = y2 + q[e - 2] * f; base[(size_t)(e - 2) * stride] = f;
    f = y3 + q[e - 3] * f; base[(size_t)(e - 3) * stride] = f;
  }
  for (; e >= 0; --e) {
    f = base[(size_t)e * stride] + q[e] * f;
    base[(size_t)e * stride] = f;
  }
  V f1 = base[0], fnm1 = base[(size_t)(n - 2) * stride];
  V xn = (rn * ackl_b - api * f1 - ami * fnm1) * inv_den;
  for (e = 0; e < n - 1; ++e) base[(size_t)e * stride] = xn * s[e] + base[(size_t)e * stride];
  base[(size_t)(n - 1) * stride] = xn;
}

// copy the factor table (4n + 4 doubles) into shared memory
template <typename V>
__device__ __forceinline__ const V* stage_table(V* sT, const V* __restrict__ T, int n) {
  for (int q = threadIdx.x; q < 4 * n + 4; q += blockDim.x) sT[q] = T[q];
  return sT;
}

constexpr int kLines = 32;

// x-lines: tile = up to 32 rows (j) of one plane k.
template <typename V>
__global__ void solve_x_kernel(Grid g, V* __restrict__ rhs, const V* __restrict__ T) {
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = (V*)smraw;
  int n = g.n1m, pitch = n + 1;
  int j0 = blockIdx.x * kLines, k = blockIdx.y;
  int nl = min(kLines, g.n2m - j0);
  const V* sT = stage_table(sm + kLines * pitch, T, n);
  int total = nl * n;
  for (int t0 = threadIdx.x; t0 < total; t0 += 8 * blockDim.x) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      v[u] = (t < total) ? rhs[cidx(g, t % n, j0 + t / n, k)] : V(0.0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      if (t < total) sm[(t / n) * pitch + t % n] = v[u];
    }
  }
  __syncthreads();
  if (threadIdx.x < nl) solve_line(sm + threadIdx.x * pitch, 1, n, sT);
  __syncthreads();
  for (int t = threadIdx.x; t < total; t += blockDim.x) rhs[cidx(g, t % n, j0 + t / n, k)] = sm[(t / n) * pitch + t % n];
}

// y-lines: tile = up to 32 adjacent i of one plane k; smem[j][l]
template <typename V>
__global__ void solve_y_kernel(Grid g, V* __restrict__ rhs, const V* __restrict__ T) {
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = (V*)smraw;
  int n = g.n2m;
  int i0 = blockIdx.x * kLines, k = blockIdx.y;
  int nl = min(kLines, g.n1m - i0);
  const V* sT = stage_table(sm + n * kLines, T, n);
  for (int t0 = threadIdx.x; t0 < n * kLines; t0 += 8 * blockDim.x) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      int j = t / kLines, l = t % kLines;
      v[u] = (t < n * kLines && l < nl) ? rhs[cidx(g, i0 + l, j, k)] : V(0.0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      if (t < n * kLines) sm[t] = v[u];
    }
  }
  __syncthreads();
  if (threadIdx.x < nl) solve_line(sm + threadIdx.x, kLines, n, sT);
  __syncthreads();
  for (int t = threadIdx.x; t < n * kLines; t += blockDim.x) {
    int j = t / kLines, l = t % kLines;
    if (l < nl) rhs[cidx(g, i0 + l, j, k)] = sm[t];
  }
}

// z-lines: tile = up to 32 adjacent i of one row j; smem[k][l]; then q += x
// (solxk.f90:44-50), optionally leaving rhs holding the increment and, in
// the precision form, writing the FP32 mirror m32 of the updated q.
template <typename V>
__global__ void solve_z_kernel(Grid g, V* __restrict__ rhs, const V* __restrict__ T, double* __restrict__ q,
                               int write_rhs, float* __restrict__ m32) {
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = (V*)smraw;
  int n = g.n3m;
  int i0 = blockIdx.x * kLines, j = blockIdx.y;
  int nl = min(kLines, g.n1m - i0);
  const V* sT = stage_table(sm + n * kLines, T, n);
  for (int t0 = threadIdx.x; t0 < n * kLines; t0 += 8 * blockDim.x) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      int k = t / kLines, l = t % kLines;
      v[u] = (t < n * kLines && l < nl) ? rhs[cidx(g, i0 + l, j, k)] : V(0.0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int t = t0 + u * blockDim.x;
      if (t < n * kLines) sm[t] = v[u];
    }
  }
  __syncthreads();
  if (threadIdx.x < nl) solve_line(sm + threadIdx.x, kLines, n, sT);
  __syncthreads();
  for (int t = threadIdx.x; t < n * kLines; t += blockDim.x) {
    int k = t / kLines, l = t % kLines;
    if (l < nl) {
      size_t c0 = cidx(g, i0 + l, j, k);
      V x = sm[t];
      if (write_rhs) rhs[c0] = x;
      double qn = q[c0] + widen(x);
      q[c0] = qn;
      if (m32) m32[c0] = d2f_bits(qn);
    }
  }
}


// ---------------------------------------------------------------------
// chunked solves
// ---------------------------------------------------------------------
// Chunk lengths with a kernel instance.  x-lines: G = n/M lanes of one warp
// (largest G <= 32); y/z-lines: G = n/M warps of one block (M as large as
// possible, G <= 32).  0 = not split, use the tile kernels.
static const int kChunkM[] = {2, 3, 4, 6, 8, 12, 16};

static bool chunk_ok(int m) {
  for (int v : kChunkM)
    if (v == m) return true;
  return false;
}

// lanes a line occupies in the x-line kernel: G = n/M rounded up to a power
// of two (shuffle segments); a warp solves 32/that lines
__host__ __device__ constexpr int line_lanes(int G) {
  return G <= 1 ? 1 : (G <= 2 ? 2 : (G <= 4 ? 4 : (G <= 8 ? 8 : (G <= 16 ? 16 : 32))));
}
static int ilog2(int v) { int l = 0; while ((1 << l) < v) ++l; return l; }

// x-lines: the chunk length with the fewest FP64 warp instructions per line.
// A warp instruction costs the same however many of its lanes are active,
// and on this part FP64 ones issue at a small fraction of the FP32 rate: per
// line, 6 per element of a chunk (forward, backward, fix-up, closure) plus 4
// per round of the two shuffle scans, shared by the 32/Gp lines of a warp.
// Segments of at least 16 lanes are preferred: with 8 (M = 16 at 128) the
// longer per-thread chains and fewer warps lose what the model saves
// (measured at 128^3: M = 8 0.475 ms, M = 16 0.523 ms per step of x-solves;
// at 256^3 M = 16 with 16 lanes is the best).
int tri_chunk_line(int n) {
  int best = 0, best_wide = 0;
  double best_cost = 1e300, best_wide_cost = 1e300;
  for (int m : kChunkM) {
    if (n % m != 0 || n / m > 32) continue;
    const int gp = line_lanes(n / m);
    const double cost = (6.0 * m + 4.0 * ilog2(gp) + 8.0) * gp / 32.0;
    if (cost < best_cost) { best_cost = cost; best = m; }
    if (gp >= 16 && cost < best_wide_cost) { best_wide_cost = cost; best_wide = m; }
  }
  return best_wide ? best_wide : best;
}

// y/z blocks: up to 32 chunks (warps) of M <= 8 cells, or 16 chunks of the
// longer M (register budget of a 1024- or 512-thread block)
constexpr int kColMaxChunks = 32;
__host__ __device__ constexpr int col_max_chunks(int m) { return m >= 12 ? 16 : 32; }

int tri_chunk_col(int n) {
  static const int pref[] = {16, 12, 8, 6, 4, 3, 2};
  for (int m : pref)
    if (n % m == 0 && n / m <= col_max_chunks(m)) return m;
  return 0;
}

// extended table of (n, M): element arrays a, b, q, s, P, Q, DP at offsets
// 0, n, .., 6n, element e stored at (e % M) * G + e / M (a warp reads one
// word per lane, or one broadcast word); then PL (P at each chunk end), QF (Q
// at each chunk start), DPF (DP at each chunk start), the four scalars
// ackl_b, api, ami, 1/den of the base table, and the chunk coefficients AC,
// BC (G each) of the one-pass correction:
//   x_e = D_e + DP'_e (y_in + AC_h xn) + Q'_e (f_in + BC_h xn).
// The periodic correction s (tridiag_periodic.f90:47-49) obeys the
// homogeneous recurrences inside a chunk that holds none of its two source
// rows, so there s = AC_h DP + BC_h Q with AC_h the forward-only value of s
// before the chunk and BC_h the final s after it; the first chunk (y_in = 0)
// keeps s in its DP' slots (AC = 1, BC = 0) and the last (f_in = 0) in its Q'
// slots (AC = 0, BC = 1).  Two FMAs per element instead of three.
__host__ __device__ constexpr size_t ext_len(int n, int m) { return m ? 7 * (size_t)n + 5 * (size_t)(n / m) + 4 : 0; }

// x-line scan factors after the extended table (line-solve slots only).
// The chunk entry values of an x-line are exclusive scans of the affine
// chunk maps y -> C + PL y (forward) and f -> U + QF f (backward, lanes in
// descending order), by warp shuffles in rounds of offset 2^r.  Round r
// multiplies by the composite factor of the 2^r lanes a lane already
// covers; the FP64 kernel reads it from W_r[h] instead of forming it with
// a second shuffle and an FP64 multiply per round (the products are those
// the shuffle scan forms, in its order, so the result is the same).
// Layout at ext_len(n, m): WF[5][G] (lanes h - 2^r + 1 .. h), WB[5][G]
// (lanes h .. h + 2^r - 1).
constexpr int kScanRounds = 5;
static size_t scan_len(int n, int m) { return m ? 2 * kScanRounds * (size_t)(n / m) : 0; }

// W[r][h] for the factors f in scan order (position h)
static void build_scan(const std::vector<double>& f, double* W) {
  const int G = (int)f.size();
  std::vector<double> cur(f);
  for (int r = 0; r < kScanRounds; ++r) {
    const int off = 1 << r;
    for (int h = 0; h < G; ++h) W[r * G + h] = cur[h];
    std::vector<double> nxt(cur);
    for (int h = off; h < G; ++h) nxt[h] = cur[h] * cur[h - off];
    cur.swap(nxt);
  }
}

static void build_ext(const std::vector<double>& t, int n, int m, double* out, bool scans = false) {
  int G = n / m;
  std::vector<double> a(t.begin(), t.begin() + n), b(t.begin() + n, t.begin() + 2 * n);
  std::vector<double> q(t.begin() + 2 * n, t.begin() + 3 * n), s(t.begin() + 3 * n, t.begin() + 4 * n);
  a[n - 1] = 0.0; b[n - 1] = 0.0; q[n - 1] = 0.0; b[0] = 0.0; s[n - 1] = 1.0;
  auto pos = [&](int e) { return (size_t)(e % m) * G + e / m; };
  std::vector<double> P(n);
  for (int e = 0; e < n; ++e) {
    out[pos(e)] = a[e];
    out[n + pos(e)] = b[e];
    out[2 * (size_t)n + pos(e)] = q[e];
    out[3 * (size_t)n + pos(e)] = s[e];
  }
  // forward-only part of s (the first loop of tridiag_periodic's s)
  std::vector<double> sf(n);
  sf[0] = -t[4 * (size_t)n + 2];
  for (int e = 1; e < n; ++e) sf[e] = -t[n + e] * sf[e - 1];
  double* AC = out + 7 * (size_t)n + 3 * G + 4;
  double* BC = AC + G;
  for (int h = 0; h < G; ++h) {
    int st = h * m, en = st + m - 1;
    if (h == 0) { AC[h] = 1.0; BC[h] = 0.0; }
    else if (h == G - 1) { AC[h] = 0.0; BC[h] = 1.0; }
    else { AC[h] = sf[st - 1]; BC[h] = s[en + 1]; }
    double pv = 1.0;
    for (int e = st; e <= en; ++e) { pv = -b[e] * pv; P[e] = pv; out[4 * (size_t)n + pos(e)] = pv; }
    out[7 * (size_t)n + h] = pv;
    double qv = 1.0, dv = 0.0;
    for (int e = en; e >= st; --e) {
      qv = q[e] * qv;
      dv = P[e] + q[e] * dv;
      out[5 * (size_t)n + pos(e)] = (h == G - 1 && G > 1) ? s[e] : qv;
      out[6 * (size_t)n + pos(e)] = h == 0 ? s[e] : dv;
    }
    out[7 * (size_t)n + G + h] = qv;
    out[7 * (size_t)n + 2 * G + h] = dv;
  }
  for (int w = 0; w < 4; ++w) out[7 * (size_t)n + 3 * G + w] = t[4 * (size_t)n + w];
  if (!scans) return;
  // forward: PL in lane order; backward: QF of lanes G-1 .. 0, whose scan
  // entry at position G-1-h is the composite of lanes h .. h + 2^r - 1
  double* WF = out + ext_len(n, m);
  double* WB = WF + kScanRounds * G;
  std::vector<double> fF(G), fB(G), Wtmp(kScanRounds * (size_t)G);
  for (int h = 0; h < G; ++h) {
    fF[h] = out[7 * (size_t)n + h];
    fB[h] = out[7 * (size_t)n + G + (G - 1 - h)];
  }
  build_scan(fF, WF);
  build_scan(fB, Wtmp.data());
  for (int r = 0; r < kScanRounds; ++r)
    for (int h = 0; h < G; ++h) WB[r * G + h] = Wtmp[r * (size_t)G + (G - 1 - h)];
}

// one table slot: base table (tile kernels) and the extended table of the
// chunk length M chosen for the direction the slot serves (0 = none)
struct TriLayout {
  int n, m;
  size_t off_ext, len;
};

static TriLayout tri_layout(int n, int m) {
  TriLayout L;
  L.n = n;
  L.m = m;
  L.off_ext = 4 * (size_t)n + 4;
  L.len = L.off_ext + ext_len(n, m) + scan_len(n, m);
  return L;
}

static bool chunk_feasible(int n, int m, bool line) {
  if (!chunk_ok(m) || n % m != 0) return false;
  return line ? n / m <= 32 : n / m <= col_max_chunks(m);
}

// chunk length of direction dir (0 x, 1 y, 2 z) for context c: the
// autotuner's choice when one is set and feasible, else the default rule
int tri_chunk(Ctx* c, int dir) {
  const int n = dir == 0 ? c->g.n1m : (dir == 1 ? c->g.n2m : c->g.n3m);
  int m = c->tune_m[dir];
  if (m > 0 && chunk_feasible(n, m, dir == 0)) return m;
  return dir == 0 ? tri_chunk_line(n) : tri_chunk_col(n);
}

// candidate chunk lengths of direction dir (for the autotuner)
std::vector<int> tri_chunk_candidates(Ctx* c, int dir) {
  const int n = dir == 0 ? c->g.n1m : (dir == 1 ? c->g.n2m : c->g.n3m);
  std::vector<int> out;
  for (int m : kChunkM)
    if (chunk_feasible(n, m, dir == 0)) out.push_back(m);
  return out;
}

// fills one slot (base + the extended table of chunk m) for (n, betadx)
static void fill_slot(int n, int m, double betadx, double* out) {
  std::vector<double> t;
  build_table(n, betadx, t);
  TriLayout L = tri_layout(n, m);
  std::copy(t.begin(), t.end(), out);
  if (m) build_ext(t, n, m, out + L.off_ext, true);
}

// the extended table of chunk length m for one line of n cells (ext_len(n, m)
// values), for callers outside this file (the z-line Poisson solve of fft.cu)
size_t tri_ext_len(int n, int m) { return ext_len(n, m); }
void tri_build_ext_table(int n, int m, double betadx, std::vector<double>& out) {
  std::vector<double> t;
  build_table(n, betadx, t);
  out.assign(ext_len(n, m), 0.0);
  build_ext(t, n, m, out.data());
}

// slot length for lines up to nmax and any chunk (ext_len + scan_len <=
// 7n + 5*32 + 4 + 2*5*32)
static size_t slot_len(int nmax) {
  return 4 * (size_t)nmax + 4 + 7 * (size_t)nmax + 5 * 32 + 4 + 2 * kScanRounds * 32;
}

template <typename V, int M>
__device__ __forceinline__ void load_chunk(const V* __restrict__ p, V (&r)[M]) {
  if constexpr (sizeof(V) == 4 && M % 4 == 0) {
#pragma unroll
    for (int v = 0; v < M / 4; ++v) {
      float4 t = reinterpret_cast<const float4*>(p)[v];
      r[4 * v] = t.x; r[4 * v + 1] = t.y; r[4 * v + 2] = t.z; r[4 * v + 3] = t.w;
    }
  } else if constexpr (sizeof(V) == 8 && M % 2 == 0) {
#pragma unroll
    for (int v = 0; v < M / 2; ++v) {
      double2 t = reinterpret_cast<const double2*>(p)[v];
      r[2 * v] = t.x; r[2 * v + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < M; ++i) r[i] = p[i];
  }
}

template <typename V, int M>
__device__ __forceinline__ void store_chunk(V* __restrict__ p, const V (&r)[M]) {
  if constexpr (sizeof(V) == 4 && M % 4 == 0) {
#pragma unroll
    for (int v = 0; v < M / 4; ++v)
      reinterpret_cast<float4*>(p)[v] = make_float4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]);
  } else if constexpr (sizeof(V) == 8 && M % 2 == 0) {
#pragma unroll
    for (int v = 0; v < M / 2; ++v) reinterpret_cast<double2*>(p)[v] = make_double2(r[2 * v], r[2 * v + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < M; ++i) p[i] = r[i];
  }
}

// x-lines: a line (row j of plane k) occupies a segment of GP = line_lanes(G)
// lanes, lane h < G of it holding cells [h*M, h*M + M); a warp solves 32/GP
// lines.  Rows start on 16-byte boundaries (pitch multiple of 4).
template <typename V, int M>
__global__ void __launch_bounds__(256) solve_xc_kernel(Grid g, V* __restrict__ rhs, const V* __restrict__ X,
                                                       int nfield) {
  const unsigned FULL = 0xffffffffu;
  const int n = g.n1m, G = n / M, GP = line_lanes(G), LPW = 32 / GP;
  const int lane = threadIdx.x & 31, hl = lane % GP;
  const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int per = g.n2m * g.n3m, lines = per * nfield;   // nfield fields at stride cells
  if (warp * LPW >= lines) return;                   // whole warp
  const int line = warp * LPW + lane / GP;
  const bool act = line < lines && hl < G;
  const int f = line / per, l = line - f * per;
  const int j = l % g.n2m, k = l / g.n2m;
  V* row = act ? rhs + (size_t)f * g.cells + cidx(g, 0, j, k) + (size_t)hl * M : rhs;
  // the bounds build: a row outside the field is neither read nor written
  const bool inb = !act || MIBM_IDX_OK(cidx(g, 0, j, k) + (size_t)hl * M + M - 1, g.cells);
  V r[M];
  if (act && inb) load_chunk<V, M>(row, r);
  else {
#pragma unroll
    for (int i = 0; i < M; ++i) r[i] = V(0);
  }
  const V rlast = r[M - 1];
  const int h = hl < G ? hl : 0;
  // forward, zero entry
  V C = V(0);
#pragma unroll
  for (int i = 0; i < M; ++i) {
    int t = i * G + h;
    C = X[t] * r[i] - X[n + t] * C;
    r[i] = C;
  }
  // y_in: exclusive scan of the affine chunk maps y -> C + PL y.  FP64: each
  // round multiplies by the composite factor the table holds for it
  // (build_scan); FP32 forms it with a second shuffle (cheaper than a load).
  const V* WF = X + ext_len(n, M);
  const V* WB = WF + kScanRounds * G;
  V Cv = act ? C : V(0), Pv = act ? X[7 * n + h] : V(1);
  for (int off = 1, r = 0; off < GP; off <<= 1, ++r) {
    V Co = __shfl_up_sync(FULL, Cv, off, GP);
    if constexpr (sizeof(V) == 8) {
      if (hl >= off) Cv = Cv + WF[r * G + h] * Co;
    } else {
      V Po = __shfl_up_sync(FULL, Pv, off, GP);
      if (hl >= off) { Cv = Cv + Pv * Co; Pv = Pv * Po; }
    }
  }
  V y_in = __shfl_up_sync(FULL, Cv, 1, GP);
  if (hl == 0) y_in = V(0);
  // backward, zero entry
  V D = V(0);
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    D = r[i] + X[2 * n + i * G + h] * D;
    r[i] = D;
  }
  // f_in: exclusive suffix scan of f -> u + QF f, u = D_first + DPF y_in
  V Uv = act ? r[0] + X[7 * n + 2 * G + h] * y_in : V(0), Qv = act ? X[7 * n + G + h] : V(1);
  for (int off = 1, r = 0; off < GP; off <<= 1, ++r) {
    V Uo = __shfl_down_sync(FULL, Uv, off, GP);
    if constexpr (sizeof(V) == 8) {
      if (hl + off < G) Uv = Uv + WB[r * G + h] * Uo;
    } else {
      V Qo = __shfl_down_sync(FULL, Qv, off, GP);
      if (hl + off < G) { Uv = Uv + Qv * Uo; Qv = Qv * Qo; }
    }
  }
  V f_in = __shfl_down_sync(FULL, Uv, 1, GP);
  if (hl + 1 >= G) f_in = V(0);
  // periodic closure from the reduced solution at element 0 (first chunk,
  // y_in = 0) and element n-2 (last chunk, f_in = 0), then the one-pass
  // correction (build_ext)
  const V* S = X + 7 * n + 3 * G;
  const V x0 = r[0] + X[5 * n + h] * f_in;
  const V xm = r[M - 2] + X[6 * n + (M - 2) * G + h] * y_in;
  V f1 = __shfl_sync(FULL, x0, 0, GP);
  V fnm1 = __shfl_sync(FULL, xm, G - 1, GP);
  V rn = __shfl_sync(FULL, rlast, G - 1, GP);
  V xn = (rn * S[0] - S[1] * f1 - S[2] * fnm1) * S[3];
  const V al = y_in + S[4 + h] * xn, be = f_in + S[4 + G + h] * xn;
#pragma unroll
  for (int i = 0; i < M; ++i) {
    int t = i * G + h;
    r[i] = r[i] + X[6 * n + t] * al + X[5 * n + t] * be;
  }
  if (act && inb) store_chunk<V, M>(row, r);
}

// y- and z-lines: block = 32 adjacent i (lanes) x G chunks (warps) of one
// plane k (y-lines) or one row j (z-lines).  For z-lines the result is added
// to q (solxk.f90:44-50), optionally also left in rhs, and in the precision
// form copied to the FP32 mirror m32.
struct QSet { double* p[3]; };   // fields the z-line increments are added to, per field of the launch

template <typename V, int M, bool ZL>
__global__ void __launch_bounds__(32 * col_max_chunks(M)) solve_cc_kernel(Grid g, V* __restrict__ rhs_base, const V* __restrict__ X,
                                                        QSet qs, int write_rhs, float* __restrict__ m32) {
  __shared__ V sC[kColMaxChunks][32];
  __shared__ V sU[kColMaxChunks][32];
  __shared__ V sF[3][32];
  const int n = ZL ? g.n3m : g.n2m, G = n / M;
  const int lane = threadIdx.x, w = threadIdx.y;
  const int x = blockIdx.x * 32 + lane;
  const bool act0 = x < g.n1m;
  // field of the launch (blockIdx.y runs over the planes of each field in turn)
  const int planes = ZL ? g.n2m : g.n3m;
  const int f = blockIdx.y / planes, pl = blockIdx.y - f * planes;
  V* __restrict__ rhs = rhs_base + (size_t)f * g.cells;
  double* __restrict__ q = ZL ? qs.p[f] : nullptr;
  // element stride of the line (< 2^31 for every supported grid) and the
  // first cell of this thread's chunk
  const int stride = ZL ? (int)g.plane : g.P;
  const int e0 = w * M;
  const size_t first = (ZL ? cidx(g, act0 ? x : 0, pl, 0) : cidx(g, act0 ? x : 0, 0, pl)) +
                       (size_t)e0 * stride;
  V* __restrict__ rp = rhs + first;
  V r[M];
  double qv[ZL ? M : 1];
  // the bounds build treats a line outside the field as inactive (loads
  // and stores skipped; the thread still takes part in the barriers)
  const bool act = act0 && MIBM_IDX_OK(first + (size_t)(M - 1) * stride, g.cells);
#pragma unroll
  for (int i = 0; i < M; ++i) r[i] = act ? rp[i * stride] : V(0);
  if (ZL) {   // the field the increment is added to, fetched with the line (more loads in flight)
    const double* __restrict__ qp = q + first;
#pragma unroll
    for (int i = 0; i < M; ++i) qv[ZL ? i : 0] = act ? qp[i * stride] : 0.0;
  }
  const V rlast = r[M - 1];
  V C = V(0);
#pragma unroll
  for (int i = 0; i < M; ++i) {
    int t = i * G + w;
    C = X[t] * r[i] - X[n + t] * C;
    r[i] = C;
  }
  sC[w][lane] = C;
  __syncthreads();
  V y_in = V(0);
  for (int hh = 0; hh < w; ++hh) y_in = sC[hh][lane] + X[7 * n + hh] * y_in;
  V D = V(0);
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    D = r[i] + X[2 * n + i * G + w] * D;
    r[i] = D;
  }
  sU[w][lane] = r[0] + X[7 * n + 2 * G + w] * y_in;
  __syncthreads();
  V f_in = V(0);
  for (int hh = G - 1; hh > w; --hh) f_in = sU[hh][lane] + X[7 * n + G + hh] * f_in;
  // periodic closure from the reduced solution at element 0 (first chunk,
  // y_in = 0) and element n-2 (last chunk, f_in = 0), then the one-pass
  // correction (build_ext)
  if (w == 0) sF[0][lane] = r[0] + X[5 * n + w] * f_in;
  if (w == G - 1) { sF[1][lane] = r[M - 2] + X[6 * n + (M - 2) * G + w] * y_in; sF[2][lane] = rlast; }
  __syncthreads();
  const V* S = X + 7 * n + 3 * G;
  V xn = (sF[2][lane] * S[0] - S[1] * sF[0][lane] - S[2] * sF[1][lane]) * S[3];
  if (!act) return;
  const V al = y_in + S[4 + w] * xn, be = f_in + S[4 + G + w] * xn;
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const int t = i * G + w;
    V xv = r[i] + X[6 * n + t] * al + X[5 * n + t] * be;
    int o = i * stride;
    if (ZL) {
      if (write_rhs) rp[o] = xv;
      double qn = qv[ZL ? i : 0] + widen(xv);
      q[first + o] = qn;
      if (m32) m32[(size_t)f * g.cells + first + o] = d2f_bits(qn);
    } else {
      rp[o] = xv;
    }
  }
}

// ---------------------------------------------------------------------
// y- and z-lines in FP32 with the lines staged by bulk tensor copies
// ---------------------------------------------------------------------
// The same arithmetic as solve_cc_kernel<float, M, ZL>, bit for bit, in a
// persistent kernel: each block walks tiles t = blockIdx.x, + gridDim.x, ...
// of 32 adjacent x times one whole line (a plane j for z-lines, k for
// y-lines) of one field.  One thread copies the next tiles' lines (and, for
// z-lines, the FP64 field the increment is added to) into a ring of `nstage`
// shared-memory stages with cp.async.bulk.tensor while the block solves the
// current one, so the loads of several tiles are always in flight and the
// registers hold only the chunk (the FP64 field waits in shared memory).
// The factor table is copied to shared memory once per block.  Results are
// written with coalesced stores (32 consecutive x per warp instruction).
// A stage wait that runs out of time (about a second: a copy that never
// completes) sets bit 2 of `err` and the block leaves after its other copies
// have landed or timed out; the host reports MIBM_ETIMEOUT.
struct ColMaps {
  CUtensorMap rhs;    // nfield rhs fields; box (32, 1, n3m, 1) for z-lines, (32, n2m, 1, 1) for y-lines
  CUtensorMap q[3];   // z-lines: per field, the FP64 field the increment is added to; box (32, 1, n3m, 1)
};

template <int M, bool ZL>
__global__ void __launch_bounds__(32 * col_max_chunks(M), 1) solve_cc_tma_kernel(
    const __grid_constant__ ColMaps maps, Grid g, float* __restrict__ rhs_base, const float* __restrict__ Xg,
    int xlen, QSet qs, float* __restrict__ m32, int nfield, int nstage, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ float sC[kColMaxChunks][32];
  __shared__ float sU[kColMaxChunks][32];
  __shared__ float sF[3][32];
  const int n = ZL ? g.n3m : g.n2m, G = n / M;
  const int lane = threadIdx.x, w = threadIdx.y, tid = w * 32 + lane, nthr = 32 * G;
  const int planes = ZL ? g.n2m : g.n3m, nxt = (g.n1m + 31) / 32;
  const int ntiles = nxt * planes * nfield;
  const uint32_t stage_bytes = (uint32_t)n * 32u * (ZL ? 12u : 4u);
  // barriers at a 1024-byte boundary (the launch adds that much slack), the
  // stages from 128 bytes after it: every copy destination 128-byte aligned
  unsigned char* smem = smem_raw + ((1024u - (tma::smem_addr(smem_raw) & 1023u)) & 1023u);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* stage0 = smem + 128;
  float* X = reinterpret_cast<float*>(stage0 + (size_t)nstage * stage_bytes);
  auto sR = [&](int s) { return reinterpret_cast<float*>(stage0 + (size_t)s * stage_bytes); };
  auto sQ = [&](int s) { return reinterpret_cast<double*>(stage0 + (size_t)s * stage_bytes + (size_t)n * 128); };
  auto issue = [&](int tile, int s) {
    const int xt = tile % nxt, rest = tile / nxt, pl = rest % planes, f = rest / planes;
    tma::mbar_arrive_expect_tx(bars + s, stage_bytes);
    if (ZL) {
      tma::load_4d(sR(s), &maps.rhs, bars + s, xt * 32, pl, 0, f);
      tma::load_4d(sQ(s), &maps.q[f], bars + s, xt * 32, pl, 0, 0);
    } else {
      tma::load_4d(sR(s), &maps.rhs, bars + s, xt * 32, 0, pl, f);
    }
  };
  if (tid == 0) {
    for (int s = 0; s < nstage; ++s) tma::mbar_init(bars + s, 1);
    tma::fence_proxy_async();
    for (int s = 0; s < nstage; ++s) {
      const int tile = blockIdx.x + s * gridDim.x;
      if (tile < ntiles) issue(tile, s);
    }
  }
  for (int q = tid; q < xlen; q += nthr) X[q] = Xg[q];
  __syncthreads();
  const int stride = ZL ? (int)g.plane : g.P;
  const int e0 = w * M;
  for (int li = 0;; ++li) {
    const int tile = blockIdx.x + li * gridDim.x;
    if (tile >= ntiles) break;
    const int s = li % nstage;
    const bool ok = tma::mbar_wait(bars + s, (uint32_t)((li / nstage) & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0) {
        atomicOr(err, 2);
        for (int k = 1; k < nstage; ++k) {   // the copies still in flight
          const int L = li + k;
          if (blockIdx.x + L * gridDim.x < ntiles) tma::mbar_wait(bars + L % nstage, (uint32_t)((L / nstage) & 1));
        }
      }
      return;
    }
    const int xt = tile % nxt, rest = tile / nxt, pl = rest % planes, f = rest / planes;
    const int x = xt * 32 + lane;
    const bool act = x < g.n1m;
    const float* R = sR(s);
    float r[M];
#pragma unroll
    for (int i = 0; i < M; ++i) r[i] = R[(e0 + i) * 32 + lane];
    const float rlast = r[M - 1];
    float C = 0.f;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      int t = i * G + w;
      C = X[t] * r[i] - X[n + t] * C;
      r[i] = C;
    }
    sC[w][lane] = C;
    __syncthreads();
    float y_in = 0.f;
    for (int hh = 0; hh < w; ++hh) y_in = sC[hh][lane] + X[7 * n + hh] * y_in;
    float D = 0.f;
#pragma unroll
    for (int i = M - 1; i >= 0; --i) {
      D = r[i] + X[2 * n + i * G + w] * D;
      r[i] = D;
    }
    sU[w][lane] = r[0] + X[7 * n + 2 * G + w] * y_in;
    __syncthreads();
    float f_in = 0.f;
    for (int hh = G - 1; hh > w; --hh) f_in = sU[hh][lane] + X[7 * n + G + hh] * f_in;
    if (w == 0) sF[0][lane] = r[0] + X[5 * n + w] * f_in;
    if (w == G - 1) { sF[1][lane] = r[M - 2] + X[6 * n + (M - 2) * G + w] * y_in; sF[2][lane] = rlast; }
    __syncthreads();
    const float* S = X + 7 * n + 3 * G;
    const float xn = (sF[2][lane] * S[0] - S[1] * sF[0][lane] - S[2] * sF[1][lane]) * S[3];
    if (act) {
      const float al = y_in + S[4 + w] * xn, be = f_in + S[4 + G + w] * xn;
      const size_t first = (ZL ? cidx(g, x, pl, 0) : cidx(g, x, 0, pl)) + (size_t)e0 * stride;
      if (!MIBM_IDX_OK(first + (size_t)(M - 1) * stride, g.cells)) {
        // the bounds build skips the stores; the block still reaches the barrier below
      } else if (ZL) {
        double* __restrict__ q = qs.p[f];
        float* __restrict__ mf = m32 ? m32 + (size_t)f * g.cells : nullptr;
        const double* Q = sQ(s);
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const int t = i * G + w;
          const float xv = r[i] + X[6 * n + t] * al + X[5 * n + t] * be;
          const double qn = Q[(e0 + i) * 32 + lane] + widen(xv);
          q[first + (size_t)i * stride] = qn;
          if (mf) mf[first + (size_t)i * stride] = d2f_bits(qn);
        }
      } else {
        float* __restrict__ rp = rhs_base + (size_t)f * g.cells + first;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const int t = i * G + w;
          rp[(size_t)i * stride] = r[i] + X[6 * n + t] * al + X[5 * n + t] * be;
        }
      }
    }
    __syncthreads();   // stage s, sC, sU, sF are free again
    if (tid == 0) {
      const int next = tile + nstage * gridDim.x;
      if (next < ntiles) {
        tma::fence_proxy_async();
        issue(next, s);
      }
    }
  }
}

// Tables of one fused RK3 step: [substep][velocity|temperature][x|y|z].
// Built on the host into one pinned buffer (`tri_step_fill`) and copied in
// stream order (`tri_step_enqueue`); the copy is part of a captured step
// graph, so the buffer address is fixed.  The step ends with a stream
// synchronisation (tschem_ reads the geometry back), so the host never
// refills the buffer while a copy from it is pending.
struct StepTables {
  double* dev = nullptr;
  float* devf = nullptr;                 // FP32 copy for the precision form
  double* pinned = nullptr;              // 18 double tables, then 18 float tables
  int len = 0;
};
static std::vector<std::pair<Ctx*, StepTables*>> g_steptab;

static StepTables* steptab_of(Ctx* c) {
  for (auto& e : g_steptab)
    if (e.first == c) return e.second;
  StepTables* t = new StepTables();
  g_steptab.emplace_back(c, t);
  return t;
}

bool tri_step_fill(Ctx* c, const double betadx[3][2][3], bool f32) {
  StepTables* st = steptab_of(c);
  int nmax = std::max(c->g.n1m, c->g.n3m);
  if (!st->dev) {
    st->len = (int)slot_len(nmax);
    size_t bytes = sizeof(double) * 18 * (size_t)st->len;
    if (!cuda_ok(c, cudaMalloc(&st->dev, bytes), "step tables")) return false;
    if (!cuda_ok(c, cudaMalloc(&st->devf, bytes / 2), "step tables")) return false;
    if (!cuda_ok(c, cudaMallocHost(&st->pinned, bytes + bytes / 2), "step tables")) return false;
  }
  const int n[3] = {c->g.n1m, c->g.n2m, c->g.n3m};
  for (int ns = 0; ns < 3; ++ns)
    for (int f = 0; f < 2; ++f)
      for (int d = 0; d < 3; ++d)
        fill_slot(n[d], tri_chunk(c, d), betadx[ns][f][d], st->pinned + (size_t)((ns * 2 + f) * 3 + d) * st->len);
  if (f32) {
    float* hf = (float*)(st->pinned + 18 * (size_t)st->len);
    for (size_t q = 0; q < 18 * (size_t)st->len; ++q) hf[q] = (float)st->pinned[q];
  }
  return true;
}

// device tables of the step (FP64, and FP32 when f32) after tri_step_fill
const double* tri_step_enqueue(Ctx* c, bool f32, int* len_out, const float** f32_out) {
  StepTables* st = steptab_of(c);
  if (!st->dev) return nullptr;
  if (f32) {
    float* hf = (float*)(st->pinned + 18 * (size_t)st->len);
    cudaMemcpyAsync(st->devf, hf, sizeof(float) * 18 * (size_t)st->len, cudaMemcpyHostToDevice, c->stream);
    if (f32_out) *f32_out = st->devf;
  } else {
    cudaMemcpyAsync(st->dev, st->pinned, sizeof(double) * 18 * (size_t)st->len, cudaMemcpyHostToDevice, c->stream);
  }
  *len_out = st->len;
  return st->dev;
}

static void steptab_free(Ctx* c) {
  for (size_t q = 0; q < g_steptab.size(); ++q)
    if (g_steptab[q].first == c) {
      StepTables* t = g_steptab[q].second;
      cudaFree(t->dev);
      cudaFree(t->devf);
      if (t->pinned) cudaFreeHost(t->pinned);
      delete t;
      g_steptab.erase(g_steptab.begin() + q);
      return;
    }
}

static bool smem_ok(Ctx* c, const void* fn, size_t bytes) {
  if (bytes > 48 * 1024)
    return cuda_ok(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes), "smem attr");
  return true;
}

#define MIBM_CHUNK_CASES(M_, CALL) \
  switch (M_) {                       \
    case 2: CALL(2); break;           \
    case 3: CALL(3); break;           \
    case 4: CALL(4); break;           \
    case 6: CALL(6); break;           \
    case 8: CALL(8); break;           \
    case 12: CALL(12); break;         \
    case 16: CALL(16); break;         \
  }

// Tensor maps of the TMA line solves, cached per context by (address, box)
// so that a captured step graph replays with identical parameters.
struct TmapEntry {
  const void* base;
  int elem, nfield, box[4];
  CUtensorMap map;
};
static std::vector<std::pair<Ctx*, std::vector<TmapEntry>*>> g_tmaps;
static std::mutex g_tmaps_mu;

static bool tmap_of(Ctx* c, const void* base, int elem, int nfield, const int box[4], CUtensorMap* out) {
  std::lock_guard<std::mutex> lk(g_tmaps_mu);
  std::vector<TmapEntry>* v = nullptr;
  for (auto& e : g_tmaps)
    if (e.first == c) v = e.second;
  if (!v) {
    v = new std::vector<TmapEntry>();
    g_tmaps.emplace_back(c, v);
  }
  for (const TmapEntry& e : *v)
    if (e.base == base && e.elem == elem && e.nfield == nfield && !memcmp(e.box, box, sizeof(e.box))) {
      *out = e.map;
      return true;
    }
  TmapEntry e{};
  e.base = base; e.elem = elem; e.nfield = nfield;
  memcpy(e.box, box, sizeof(e.box));
  if (!tma::encode_fields(&e.map, base, elem, c->g.n1m, c->g.n2m, c->g.n3m, c->g.P, c->g.cells, nfield, box))
    return false;
  if (v->size() > 64) v->clear();
  v->push_back(e);
  *out = e.map;
  return true;
}

static void tmaps_free(Ctx* c) {
  std::lock_guard<std::mutex> lk(g_tmaps_mu);
  for (size_t q = 0; q < g_tmaps.size(); ++q)
    if (g_tmaps[q].first == c) {
      delete g_tmaps[q].second;
      g_tmaps.erase(g_tmaps.begin() + q);
      return;
    }
}

// stages of the TMA line solve: two, the copies issued two tiles ahead
// (z-lines: the FP32 line and the FP64 field, 96 KB per stage at 256 cells;
// y-lines: 32 KB -- four stages measured the same as two); one block per SM
static int tma_stages(bool) { return 2; }

template <bool ZL>
static bool solve_cc_tma_launch(Ctx* c, float* rhs, const float* X, int M, const QSet& q, int nfield,
                                float* m32, const char* name) {
  const int n = ZL ? c->g.n3m : c->g.n2m;
  if (!c->tma || n > 256 || c->g.n1m < 32 || nfield < 1 || nfield > 3) return false;
  const int G = n / M;
  const int xlen = (int)ext_len(n, M);
  const int nstage = tma_stages(ZL);
  const size_t stage_bytes = (size_t)n * 32 * (ZL ? 12 : 4);
  const size_t smem = 1024 + 128 + nstage * stage_bytes + sizeof(float) * (size_t)xlen;
  int dev = 0, optin = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t static_smem = sizeof(float) * (2 * kColMaxChunks * 32 + 3 * 32);
  if (smem + static_smem > (size_t)optin) return false;
  ColMaps maps{};
  const int box_r[4] = {32, ZL ? 1 : n, ZL ? n : 1, 1};
  if (!tmap_of(c, rhs, 4, nfield, box_r, &maps.rhs)) return false;
  if (ZL)
    for (int f = 0; f < nfield; ++f) {
      const int box_q[4] = {32, 1, n, 1};
      if (!tmap_of(c, q.p[f], 8, 1, box_q, &maps.q[f])) return false;
    }
  const void* fn = nullptr;
#define TMA_FN(MM) fn = (const void*)solve_cc_tma_kernel<MM, ZL>
  MIBM_CHUNK_CASES(M, TMA_FN)
#undef TMA_FN
  if (!fn) return false;
  if (!cuda_ok(c, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "tma smem"))
    return false;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * G, smem);
  const int ntiles = ((c->g.n1m + 31) / 32) * (ZL ? c->g.n2m : c->g.n3m) * nfield;
  const int grid = std::max(1, std::min(ntiles, std::max(1, per_sm) * std::max(1, sms)));
  dim3 block(32, G);
  {
    MIBM_PROF(c, name);
#define TMA_CC(MM)                                                                                          \
  solve_cc_tma_kernel<MM, ZL><<<grid, block, smem, c->stream>>>(maps, c->g, rhs, X, xlen, q, m32, nfield, \
                                                                 nstage, c->dflag + 2)
    MIBM_CHUNK_CASES(M, TMA_CC)
#undef TMA_CC
  }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, name);
  return true;
}

template <typename V>
static bool solve_xc_launch(Ctx* c, V* rhs, const V* T, const char* name, int nfield) {
  TriLayout L = tri_layout(c->g.n1m, tri_chunk(c, 0));
  if (!L.m) return false;
  const V* X = T + L.off_ext;
  const int lpw = 32 / line_lanes(c->g.n1m / L.m);           // lines per warp
  dim3 grid(div_up((size_t)c->g.n2m * c->g.n3m * nfield, 8 * (size_t)lpw));
  {
    MIBM_PROF(c, name);
#define XC(M) solve_xc_kernel<V, M><<<grid, 256, 0, c->stream>>>(c->g, rhs, X, nfield)
    MIBM_CHUNK_CASES(L.m, XC)
#undef XC
  }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, name);
  return true;
}

template <typename V, bool ZL>
static bool solve_cc_launch(Ctx* c, V* rhs, const V* T, const QSet& q, int nfield, int write_rhs, float* m32,
                            const char* name) {
  TriLayout L = tri_layout(ZL ? c->g.n3m : c->g.n2m, tri_chunk(c, ZL ? 2 : 1));
  if (!L.m) return false;
  const V* X = T + L.off_ext;
  if constexpr (sizeof(V) == 4)
    if (!write_rhs && solve_cc_tma_launch<ZL>(c, rhs, X, L.m, q, nfield, m32, name)) return true;
  dim3 block(32, L.n / L.m);
  dim3 grid(div_up(c->g.n1m, 32), (ZL ? c->g.n2m : c->g.n3m) * nfield);
  {
    MIBM_PROF(c, name);
#define CC(M) solve_cc_kernel<V, M, ZL><<<grid, block, 0, c->stream>>>(c->g, rhs, X, q, write_rhs, m32)
    MIBM_CHUNK_CASES(L.m, CC)
#undef CC
  }
  ++c->launches;
  MIBM_LAUNCH_CHECK(c, name);
  return true;
}

// nfield consecutive fields at stride cells in rhs share the table T: one
// launch for all of them (the three velocity components of the fused step),
// so that the grid holds enough blocks to keep every SM busy to the end.
// Lengths without a chunked instance fall back to the tile kernels, one
// launch per field.
template <typename V>
static void solve_x_launch(Ctx* c, V* rhs, const V* T, const char* name, int nfield) {
  if (solve_xc_launch<V>(c, rhs, T, name, nfield)) return;
  size_t sm = ((size_t)kLines * (c->g.n1m + 1) + 4 * (size_t)c->g.n1m + 4) * sizeof(V);
  if (!smem_ok(c, (const void*)solve_x_kernel<V>, sm)) return;
  dim3 grid(div_up(c->g.n2m, kLines), c->g.n3m);
  for (int f = 0; f < nfield; ++f) {
    { MIBM_PROF(c, name); solve_x_kernel<V><<<grid, 128, sm, c->stream>>>(c->g, rhs + (size_t)f * c->g.cells, T); }
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, name);
}

template <typename V>
static void solve_y_launch(Ctx* c, V* rhs, const V* T, const char* name, int nfield) {
  if (solve_cc_launch<V, false>(c, rhs, T, QSet{}, nfield, 0, nullptr, name)) return;
  size_t sm = ((size_t)kLines * c->g.n2m + 4 * (size_t)c->g.n2m + 4) * sizeof(V);
  if (!smem_ok(c, (const void*)solve_y_kernel<V>, sm)) return;
  dim3 grid(div_up(c->g.n1m, kLines), c->g.n3m);
  for (int f = 0; f < nfield; ++f) {
    { MIBM_PROF(c, name); solve_y_kernel<V><<<grid, 128, sm, c->stream>>>(c->g, rhs + (size_t)f * c->g.cells, T); }
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, name);
}

template <typename V>
static void solve_z_launch(Ctx* c, V* rhs, const V* T, const QSet& q, int nfield, int write_rhs, float* m32,
                           const char* name) {
  if (solve_cc_launch<V, true>(c, rhs, T, q, nfield, write_rhs, m32, name)) return;
  size_t sm = ((size_t)kLines * c->g.n3m + 4 * (size_t)c->g.n3m + 4) * sizeof(V);
  if (!smem_ok(c, (const void*)solve_z_kernel<V>, sm)) return;
  dim3 grid(div_up(c->g.n1m, kLines), c->g.n2m);
  for (int f = 0; f < nfield; ++f) {
    { MIBM_PROF(c, name);
      solve_z_kernel<V><<<grid, 128, sm, c->stream>>>(c->g, rhs + (size_t)f * c->g.cells, T, q.p[f], write_rhs, m32); }
    ++c->launches;
  }
  MIBM_LAUNCH_CHECK(c, name);
}

static QSet qset(double* const* q, int nfield) {
  QSet s{};
  for (int f = 0; f < nfield && f < 3; ++f) s.p[f] = q[f];
  return s;
}

void k_solve_x_T(Ctx* c, double* rhs, const double* T, int nfield) {
  solve_x_launch<double>(c, rhs, T, "solve_x", nfield);
}
void k_solve_y_T(Ctx* c, double* rhs, const double* T, int nfield) {
  solve_y_launch<double>(c, rhs, T, "solve_y", nfield);
}
void k_solve_z_T(Ctx* c, double* rhs, const double* T, double* const* q, int nfield, int write_rhs) {
  solve_z_launch<double>(c, rhs, T, qset(q, nfield), nfield, write_rhs, nullptr, "solve_z");
}
void k_solve_x_f32(Ctx* c, float* rhs, const float* T, int nfield) {
  solve_x_launch<float>(c, rhs, T, "solve_x_f32", nfield);
}
void k_solve_y_f32(Ctx* c, float* rhs, const float* T, int nfield) {
  solve_y_launch<float>(c, rhs, T, "solve_y_f32", nfield);
}
void k_solve_z_f32(Ctx* c, float* rhs, const float* T, double* const* q, int nfield, float* mirror) {
  solve_z_launch<float>(c, rhs, T, qset(q, nfield), nfield, 0, mirror, "solve_z_f32");
}

void k_solve_x(Ctx* c, double* rhs, double betadx) {
  const double* T = table_for(c, 0, betadx);
  if (T) k_solve_x_T(c, rhs, T, 1);
}

void k_solve_y(Ctx* c, double* rhs, double betadx) {
  const double* T = table_for(c, 1, betadx);
  if (T) k_solve_y_T(c, rhs, T, 1);
}

void k_solve_z(Ctx* c, double* rhs, double betadx, double* q) {
  const double* T = table_for(c, 2, betadx);
  if (T) k_solve_z_T(c, rhs, T, &q, 1, 1);
}

// ---------------------------------------------------------------------
// Autotuner support: time the solve of direction dir with chunk length m
// (0 = tile kernel) on scratch lines (betadx 0.9), best of `reps` runs after
// one warm-up, in ms.  The context's own state is not touched.
// ---------------------------------------------------------------------
float tri_time_direction(Ctx* c, int dir, int m, bool f32, int reps) {
  const int n = dir == 0 ? c->g.n1m : (dir == 1 ? c->g.n2m : c->g.n3m);
  const int saved = c->tune_m[dir];
  c->tune_m[dir] = m;
  std::vector<double> slot(slot_len(std::max(c->g.n1m, c->g.n3m)), 0.0);
  fill_slot(n, m, 0.9, slot.data());
  std::vector<float> slotf(slot.begin(), slot.end());
  void* tab = nullptr;
  void* rhs = nullptr;
  double* q = nullptr;
  float best = -1.f;
  size_t vs = f32 ? sizeof(float) : sizeof(double);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool ok = cuda_ok(c, cudaMalloc(&tab, sizeof(double) * slot.size()), "tune") &&
            cuda_ok(c, cudaMalloc(&rhs, vs * c->g.cells), "tune") &&
            cuda_ok(c, cudaMalloc((void**)&q, sizeof(double) * c->g.cells), "tune") &&
            cuda_ok(c, cudaEventCreate(&e0), "tune") && cuda_ok(c, cudaEventCreate(&e1), "tune");
  if (ok) {
    if (f32) cudaMemcpyAsync(tab, slotf.data(), sizeof(float) * slotf.size(), cudaMemcpyHostToDevice, c->stream);
    else cudaMemcpyAsync(tab, slot.data(), sizeof(double) * slot.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(rhs, 0, vs * c->g.cells, c->stream);
    cudaMemsetAsync(q, 0, sizeof(double) * c->g.cells, c->stream);
    auto run = [&]() {
      if (f32) {
        float* r = (float*)rhs;
        const float* T = (const float*)tab;
        if (dir == 0) solve_x_launch<float>(c, r, T, "tune", 1);
        else if (dir == 1) solve_y_launch<float>(c, r, T, "tune", 1);
        else solve_z_launch<float>(c, r, T, qset(&q, 1), 1, 0, nullptr, "tune");
      } else {
        double* r = (double*)rhs;
        const double* T = (const double*)tab;
        if (dir == 0) solve_x_launch<double>(c, r, T, "tune", 1);
        else if (dir == 1) solve_y_launch<double>(c, r, T, "tune", 1);
        else solve_z_launch<double>(c, r, T, qset(&q, 1), 1, 0, nullptr, "tune");
      }
    };
    run();
    for (int r = 0; r < reps && c->status == MIBM_OK; ++r) {
      cudaEventRecord(e0, c->stream);
      run();
      cudaEventRecord(e1, c->stream);
      if (!cuda_ok(c, cudaEventSynchronize(e1), "tune")) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (best < 0.f || ms < best) best = ms;
    }
  }
  cudaStreamSynchronize(c->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(tab); cudaFree(rhs); cudaFree(q);
  c->tune_m[dir] = saved;
  return best;
}

// ---------------------------------------------------------------------
// Allocation-free x-line solve (mibm_solxi_noalloc, see include/mibm.h).
//
// Same kernel and same factor table as the library's x-line solves, but the
// table lives in a file-scope device array instead of memory the library
// allocates.  Every GPU that loads the library holds this array until the
// process exits.  The table is written on the device by a one-thread kernel
// on the caller's stream (tri_factors, the function build_table runs on the
// host, bit for bit), so the call touches no host buffer.
// ---------------------------------------------------------------------
constexpr int kNoAllocMaxN = 512;                      // longest x-line
constexpr int kNoAllocTable = 4 * kNoAllocMaxN + 4;    // [a|b|q|s]*n + 4 scalars
static __device__ __align__(256) double g_noalloc_table[kNoAllocTable];

// The factor table of (n, betadx) written by one thread into `out`.
__global__ void tri_factors_kernel(int n, double betadx, double* __restrict__ out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) tri_factors(n, betadx, out);
}

// Host-side stand-in of g_noalloc_table is not a device address: the device
// address is looked up once per device with that device current.
static std::mutex g_noalloc_mu;
static double* g_noalloc_addr[64] = {nullptr};

static cudaError_t noalloc_table_address(int dev, double** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!g_noalloc_addr[dev]) {
    double* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_table);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

// Self-test (mibm_selftest_): the device evaluation of the factor table must
// equal the host's build_table bit for bit.  Returns the number of differing
// entries, or -1 on a CUDA error.
long long tri_factors_selftest() {
  const int ns[] = {2, 3, 16, 24, 127, 200, 256, 512};
  const double bds[] = {1e-6, 0.004, 0.37, 0.9, 6.5, 40.0, 3.3e3};
  double* dev = nullptr;
  if (cudaMalloc(&dev, sizeof(double) * kNoAllocTable) != cudaSuccess) { cudaGetLastError(); return -1; }
  long long bad = 0;
  std::vector<double> ref, got(kNoAllocTable);
  for (int n : ns)
    for (double bd : bds) {
      build_table(n, bd, ref);
      tri_factors_kernel<<<1, 1>>>(n, bd, dev);
      if (cudaMemcpy(got.data(), dev, sizeof(double) * ref.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaFree(dev);
        cudaGetLastError();
        return -1;
      }
      for (size_t q = 0; q < ref.size(); ++q)
        if (memcmp(&ref[q], &got[q], sizeof(double)) != 0) ++bad;
    }
  cudaFree(dev);
  return bad;
}

}  // namespace mibm

extern "C" int mibm_solxi_noalloc(double* rhs, int n1m, int n2m, int n3m, int pitch, double betadx,
                                  void* stream) {
  using namespace mibm;
  if (!rhs || n1m < 2 || n2m < 1 || n3m < 1 || pitch < n1m) return MIBM_EINVAL;
  if (n1m > kNoAllocMaxN) return MIBM_EINVAL;      // table would not fit the static scratch
  if (n3m > 65535) return MIBM_EINVAL;             // one grid row of blocks per plane
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MIBM_ECUDA;
  double* table = nullptr;
  if (noalloc_table_address(dev, &table) != cudaSuccess) return MIBM_ECUDA;
  Grid g{};
  g.n1m = n1m; g.n2m = n2m; g.n3m = n3m; g.P = pitch;
  g.plane = (size_t)pitch * n2m; g.cells = g.plane * n3m;
  size_t sm = ((size_t)kLines * (n1m + 1) + 4 * (size_t)n1m + 4) * sizeof(double);
  if (sm > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)solve_x_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
          cudaSuccess)
    return MIBM_ECUDA;
  cudaStream_t st = (cudaStream_t)stream;
  // the line-independent factors, in stream order ahead of the solve
  tri_factors_kernel<<<1, 1, 0, st>>>(n1m, betadx, table);
  if (cudaGetLastError() != cudaSuccess) return MIBM_ECUDA;
  dim3 grid(div_up(n2m, kLines), n3m);
  solve_x_kernel<double><<<grid, 128, sm, st>>>(g, rhs, table);
  return cudaGetLastError() == cudaSuccess ? MIBM_OK : MIBM_ECUDA;
}
