// fft_fast.cuh -- Poisson-solve FFT passes specialised for one line length N
// at compile time (phcalc.f90:11-97, same chain and conventions as fft.cu).
//
// A block transforms L lines of length N held in one shared buffer, element
// e of line l at buf[e*(L+1) + l] (the padding keeps both the column loads
// of the y/z passes and the row loads of the x passes free of bank
// conflicts).  Each Stockham stage reads every butterfly's inputs into
// registers, synchronises, applies the twiddles and the radix-4/2/3
// butterfly and writes the outputs in place; stage radices, strides and
// twiddle steps are compile-time constants, so no index division is left
// at run time.  Twiddles e^{-2 pi i m/N} are the FP64-tabulated table of
// fft.cu, staged in shared memory.  L (a power of two) is chosen so that a
// block moves at least 128 contiguous bytes per spectrum row and a thread
// holds at most 16 (FP32) or 8 (FP64) complex values per stage.
#pragma once

#include "fft_common.cuh"
#include "tma.cuh"

namespace mibm {
namespace fastfft {

__host__ __device__ constexpr int nstages(int n) {
  int s = 0;
  while (n % 4 == 0) { n /= 4; ++s; }
  while (n % 2 == 0) { n /= 2; ++s; }
  while (n % 3 == 0) { n /= 3; ++s; }
  return s;
}

__host__ __device__ constexpr int radix_at(int n, int st) {
  int s = 0;
  while (n % 4 == 0) { if (s == st) return 4; n /= 4; ++s; }
  while (n % 2 == 0) { if (s == st) return 2; n /= 2; ++s; }
  while (n % 3 == 0) { if (s == st) return 3; n /= 3; ++s; }
  return 1;
}

// lines per block and threads per block for length N and complex type C
// LONE = 1: the one-line shape of the y/z passes for the columns left over
// after whole tiles of L (the Nyquist column kx = n1m/2 for even n1m), so that
// a last tile of one real column does not transform L - 1 padding lines
template <typename C, int N, int LONE = 0>
struct Shape {
  // values per block: small tiles, so that a pass has many blocks and the
  // last wave leaves few SMs idle (these passes are FP64-issue bound), but
  // at least 8 (FP64) or 16 (FP32) lines so that a block still moves 128
  // contiguous bytes per spectrum row
  static constexpr int kWork = sizeof(C) == 16 ? 1024 : 2048;
  static constexpr int kMinL = sizeof(C) == 16 ? 8 : 16;
  // lines per block: the largest power of two <= min(32, max(kMinL, kWork / N))
  static constexpr int pow2_floor(int v) { int p = 1; while (2 * p <= v) p *= 2; return p; }
  static constexpr int Lw = (kWork / N) < kMinL ? kMinL : ((kWork / N) > 32 ? 32 : kWork / N);
  static constexpr int L = LONE ? 1 : pow2_floor(Lw);
  static constexpr int T = LONE ? 64 : 256;
  // resident blocks per SM asked of ptxas: four for the 256-point FP32 x and
  // z passes (latency-bound; measured faster, though the z pass spills a
  // little), three elsewhere (the y pass at four spills more and runs slower)
  static constexpr int kMinBlocks = LONE ? 8 : (sizeof(C) == 8 && N == 256 ? 4 : 3);
  static constexpr int kMinBlocksY = LONE ? 8 : 3;
  static constexpr int ES = L + 1;
  static constexpr size_t smem = sizeof(C) * ((size_t)N + (size_t)N * ES);
};

template <typename C, int R, bool INV>
__device__ __forceinline__ void butterfly(C (&v)[R]) {
  typedef typename Real<C>::T Rt;
  if constexpr (R == 4) {
    C a02p = cadd(v[0], v[2]), a02m = csub(v[0], v[2]);
    C a13p = cadd(v[1], v[3]), a13m = csub(v[1], v[3]);
    // -i*(a1-a3) for the forward sign, +i*(a1-a3) for the inverse
    C rot = INV ? mk<C>(-a13m.y, a13m.x) : mk<C>(a13m.y, -a13m.x);
    v[0] = cadd(a02p, a13p);
    v[2] = csub(a02p, a13p);
    v[1] = cadd(a02m, rot);
    v[3] = csub(a02m, rot);
  } else if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else {
    const Rt s3 = Rt(0.86602540378443864676);   // sqrt(3)/2
    C t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    C m = mk<C>(v[0].x - Rt(0.5) * t1.x, v[0].y - Rt(0.5) * t1.y);
    // forward: -i*s3*t2 ; inverse: +i*s3*t2
    C sv = INV ? mk<C>(-s3 * t2.y, s3 * t2.x) : mk<C>(s3 * t2.y, -s3 * t2.x);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(m, sv);
    v[2] = csub(m, sv);
  }
}

// one Stockham stage of radix R after NS points have been combined
template <typename C, int N, int L, int T, int R, int NS, bool INV>
__device__ __forceinline__ void stage(C* buf, const C* tw) {
  constexpr int ES = L + 1, NB = N / R, TOT = NB * L, PER = (TOT + T - 1) / T, TS = N / (NS * R);
  C v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * T;
    if (TOT % T == 0 || b < TOT) {
      const int l = b % L, j = b / L;
#pragma unroll
      for (int r = 0; r < R; ++r) v[p][r] = buf[(j + r * NB) * ES + l];
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * T;
    if (TOT % T == 0 || b < TOT) {
      const int l = b % L, j = b / L, kk = j % NS;
      if constexpr (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = tw[kk * r * TS];
          if (INV) w.y = -w.y;
          v[p][r] = cmul(v[p][r], w);
        }
      }
      butterfly<C, R, INV>(v[p]);
      const int o = (j / NS) * NS * R + kk;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[(o + r * NS) * ES + l] = v[p][r];
    }
  }
  __syncthreads();
}

template <typename C, int N, int L, int T, bool INV, int S = 0, int NS = 1>
__device__ __forceinline__ void run(C* buf, const C* tw) {
  if constexpr (S < nstages(N)) {
    constexpr int R = radix_at(N, S);
    stage<C, N, L, T, R, NS, INV>(buf, tw);
    run<C, N, L, T, INV, S + 1, NS * R>(buf, tw);
  }
}

// 16-point DFT in registers, x[k] := sum_n x[n] W16^{nk} (forward sign, or
// the conjugate for INV), as 4 x 4: DFT4 over a of x[4a + b] for each b,
// the twiddles W16^{bc}, DFT4 over b for each c (output k = c + 4d).  The
// W16 powers are the table's entries W_N^{(N/16) m}.
template <typename C, int N, bool INV>
__device__ __forceinline__ void dft16(C (&x)[16], const C* tw) {
  C z[4][4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    C v[4] = {x[b], x[4 + b], x[8 + b], x[12 + b]};
    butterfly<C, 4, INV>(v);
#pragma unroll
    for (int c = 0; c < 4; ++c) z[b][c] = v[c];
  }
#pragma unroll
  for (int b = 1; b < 4; ++b)
#pragma unroll
    for (int c = 1; c < 4; ++c) {
      C w = tw[(N / 16) * b * c];
      if (INV) w.y = -w.y;
      z[b][c] = cmul(z[b][c], w);
    }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    C v[4] = {z[0][c], z[1][c], z[2][c], z[3][c]};
    butterfly<C, 4, INV>(v);
#pragma unroll
    for (int d = 0; d < 4; ++d) x[c + 4 * d] = v[d];
  }
}

// The 256-point transform of L = 16 lines with 256 threads as 16 x 16
// (n = 16 n1 + n2, k = k1 + 16 k2): pass 1, thread (line tid/16, n2 =
// tid%16), the 16-point DFTs over n1 and the twiddles W256^{n2 k1}, written
// to element 16 k1 + n2 (each thread reads and writes only the elements of
// its own n2, so no barrier between); pass 2, thread (line tid%16, k1 =
// tid/16), the 16-point DFTs over n2, written to element k1 + 16 k2 after a
// barrier.  Two shared-memory round trips and three barriers instead of the
// four and eight of the radix-4 stages; the lane order of each pass keeps
// its 8-byte accesses free of bank conflicts with the padded layout
// (element e of line l at e*(L+1) + l).
template <typename C, int N, int L, int T, bool INV, bool DENSE = false>
__device__ __forceinline__ void run16x16(C* buf, const C* tw) {
  static_assert(N == 256 && L == 16 && T == 256, "16 x 16 engine: 256 points, 16 lines, 256 threads");
  // DENSE: element e of line l at e*L + l (the layout a bulk tensor copy
  // writes); lanes then take 16 lines of one n2 in pass 1 as in pass 2,
  // which keeps the accesses of both passes free of bank conflicts
  constexpr int ES = DENSE ? L : L + 1;
  C x[16];
  {
    const int l = DENSE ? (threadIdx.x & 15) : (threadIdx.x >> 4);
    const int n2 = DENSE ? (threadIdx.x >> 4) : (threadIdx.x & 15);
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) x[n1] = buf[(16 * n1 + n2) * ES + l];
    dft16<C, N, INV>(x, tw);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
      C w = tw[(n2 * k1) & (N - 1)];
      if (INV) w.y = -w.y;
      x[k1] = cmul(x[k1], w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) buf[(16 * k1 + n2) * ES + l] = x[k1];
  }
  __syncthreads();
  const int l = threadIdx.x & 15, k1 = threadIdx.x >> 4;
#pragma unroll
  for (int n2 = 0; n2 < 16; ++n2) x[n2] = buf[(16 * k1 + n2) * ES + l];
  dft16<C, N, INV>(x, tw);
  __syncthreads();
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) buf[(k1 + 16 * k2) * ES + l] = x[k2];
  __syncthreads();
}

// the transform of the block's L lines in buf: the 16 x 16 engine where it
// applies (FP32, 256 points, the 16-line tiles), else the radix-4/2/3 stages
template <typename C, int N, int L, int T, bool INV>
__device__ __forceinline__ void transform(C* buf, const C* tw) {
  if constexpr (sizeof(C) == 8 && N == 256 && L == 16 && T == 256) run16x16<C, N, L, T, INV>(buf, tw);
  else run<C, N, L, T, INV>(buf, tw);
}

template <typename C, int N, int T>
__device__ __forceinline__ void stage_twiddles(C* s, const C* __restrict__ tw) {
  for (int m = threadIdx.x; m < N; m += T) s[m] = tw[m];
}

// X forward: rows (j, j+1) of plane k packed as one complex line, r2c split
template <typename C, typename S, int N>
__global__ void __launch_bounds__(Shape<C, N>::T, Shape<C, N>::kMinBlocks) x_fwd(FftArgs<C> F, const S* __restrict__ src, C* __restrict__ spec) {
  typedef typename Real<C>::T R;
  constexpr int L = Shape<C, N>::L, T = Shape<C, N>::T, ES = Shape<C, N>::ES, PER = (N * L + T - 1) / T;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* tw = (C*)shraw;
  C* buf = tw + N;
  stage_twiddles<C, N, T>(tw, F.twx);
  const Grid& g = F.g;
  const int k = blockIdx.y, jp0 = blockIdx.x * L;
  const int npairs = min(L, g.n2m / 2 - jp0);
  C v[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    const int e = t % N, l = t / N;
    if ((N * L) % T == 0 || t < N * L) {
      if (l < npairs) {
        const int j = 2 * (jp0 + l);
        v[p] = mk<C>(R(src[cidx(g, e, j, k)]), R(src[cidx(g, e, j + 1, k)]));
      } else {
        v[p] = mk<C>(R(0), R(0));
      }
    }
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    if ((N * L) % T == 0 || t < N * L) buf[(t % N) * ES + t / N] = v[p];
  }
  __syncthreads();
  transform<C, N, L, T, false>(buf, tw);
  const int H = g.H;
  for (int t = threadIdx.x; t < H * L; t += T) {
    const int l = t / H, kx = t - l * H;
    if (l >= npairs) continue;
    C z = buf[kx * ES + l];
    C zc = conjc(buf[((N - kx) % N) * ES + l]);
    // X_a = (Z + conj Z_-)/2 ; X_b = (Z - conj Z_-)/(2i)
    C xa = mk<C>(R(0.5) * (z.x + zc.x), R(0.5) * (z.y + zc.y));
    C d = csub(z, zc);
    C xb = mk<C>(R(0.5) * d.y, R(-0.5) * d.x);
    const int j = 2 * (jp0 + l);
    spec[(size_t)kx + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)] = xa;
    spec[(size_t)kx + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)] = xb;
  }
}

// X inverse (c2r): half spectra of rows (j, j+1) -> real rows
template <typename C, int N>
__global__ void __launch_bounds__(Shape<C, N>::T, Shape<C, N>::kMinBlocks) x_inv(FftArgs<C> F, const C* __restrict__ spec,
                                                       typename Real<C>::T* __restrict__ dst) {
  typedef typename Real<C>::T R;
  constexpr int L = Shape<C, N>::L, T = Shape<C, N>::T, ES = Shape<C, N>::ES, PER = (N * L + T - 1) / T;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* tw = (C*)shraw;
  C* buf = tw + N;
  stage_twiddles<C, N, T>(tw, F.twx);
  const Grid& g = F.g;
  const int H = g.H;
  const int k = blockIdx.y, jp0 = blockIdx.x * L;
  const int npairs = min(L, g.n2m / 2 - jp0);
  C v[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    const int kx = t % N, l = t / N;
    if ((N * L) % T == 0 || t < N * L) {
      if (l < npairs) {
        const int j = 2 * (jp0 + l);
        const int sk = (kx < H) ? kx : N - kx;
        C xa = spec[(size_t)sk + (size_t)g.HP * ((size_t)j + (size_t)g.n2m * k)];
        C xb = spec[(size_t)sk + (size_t)g.HP * ((size_t)(j + 1) + (size_t)g.n2m * k)];
        if (sk == 0 || 2 * sk == N) { xa.y = R(0); xb.y = R(0); }
        if (kx >= H) { xa.y = -xa.y; xb.y = -xb.y; }
        v[p] = mk<C>(xa.x - xb.y, xa.y + xb.x);   // Z = Xa + i Xb
      } else {
        v[p] = mk<C>(R(0), R(0));
      }
    }
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    if ((N * L) % T == 0 || t < N * L) buf[(t % N) * ES + t / N] = v[p];
  }
  __syncthreads();
  transform<C, N, L, T, true>(buf, tw);
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    const int i = t % N, l = t / N;
    if (((N * L) % T == 0 || t < N * L) && l < npairs) {
      const int j = 2 * (jp0 + l);
      C z = buf[i * ES + l];
      dst[cidx(g, i, j, k)] = z.x;
      dst[cidx(g, i, j + 1, k)] = z.y;
    }
  }
}

// tile of L adjacent kx columns, line elements `step` apart in the spectrum
template <typename C, int N, int LONE>
__device__ __forceinline__ void load_cols(C* buf, const C* __restrict__ spec, size_t base, size_t step, int nc) {
  typedef Shape<C, N, LONE> Sh;
  constexpr int L = Sh::L, T = Sh::T, ES = Sh::ES, PER = (N * L + T - 1) / T;
  C v[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    const int l = t % L, e = t / L;
    if ((N * L) % T == 0 || t < N * L) v[p] = (l < nc) ? spec[base + l + step * e] : C{};
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    if ((N * L) % T == 0 || t < N * L) buf[(t / L) * ES + t % L] = v[p];
  }
}

template <typename C, int N, int LONE>
__device__ __forceinline__ void store_cols(const C* buf, C* __restrict__ spec, size_t base, size_t step, int nc) {
  typedef Shape<C, N, LONE> Sh;
  constexpr int L = Sh::L, T = Sh::T, ES = Sh::ES, PER = (N * L + T - 1) / T;
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * T;
    const int l = t % L, e = t / L;
    if (((N * L) % T == 0 || t < N * L) && l < nc) spec[base + l + step * e] = buf[e * ES + l];
  }
}

// Y pass (forward or inverse) on L kx columns from kx_base + L*blockIdx.x of plane k
template <typename C, int N, bool INV, int LONE = 0>
__global__ void __launch_bounds__(Shape<C, N, LONE>::T, Shape<C, N, LONE>::kMinBlocksY)
y_pass(FftArgs<C> F, C* __restrict__ spec, int kx_base) {
  typedef Shape<C, N, LONE> Sh;
  constexpr int L = Sh::L, T = Sh::T;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* tw = (C*)shraw;
  C* buf = tw + N;
  stage_twiddles<C, N, T>(tw, F.twy);
  const Grid& g = F.g;
  const int kx0 = kx_base + blockIdx.x * L, k = blockIdx.y;
  const int nc = min(L, g.H - kx0);
  const size_t base = (size_t)kx0 + (size_t)g.HP * (size_t)g.n2m * k;
  load_cols<C, N, LONE>(buf, spec, base, (size_t)g.HP, nc);
  __syncthreads();
  transform<C, N, L, T, INV>(buf, tw);
  store_cols<C, N, LONE>(buf, spec, base, (size_t)g.HP, nc);
}

// Z pass: forward, scale, eigenvalue division, zero mode, inverse
template <typename C, int N, int LONE = 0>
__global__ void __launch_bounds__(Shape<C, N, LONE>::T, Shape<C, N, LONE>::kMinBlocks)
z_solve(FftArgs<C> F, C* __restrict__ spec, int kx_base) {
  typedef typename Real<C>::T R;
  typedef Shape<C, N, LONE> Sh;
  constexpr int L = Sh::L, T = Sh::T, ES = Sh::ES;
  extern __shared__ __align__(16) unsigned char shraw[];
  C* tw = (C*)shraw;
  C* buf = tw + N;
  stage_twiddles<C, N, T>(tw, F.twz);
  const Grid& g = F.g;
  const int kx0 = kx_base + blockIdx.x * L, j = blockIdx.y;
  const int nc = min(L, g.H - kx0);
  const size_t zstride = (size_t)g.HP * g.n2m;
  const size_t base = (size_t)kx0 + (size_t)g.HP * j;
  load_cols<C, N, LONE>(buf, spec, base, zstride, nc);
  __syncthreads();
  transform<C, N, L, T, false>(buf, tw);
  const R* __restrict__ eig = F.eig + (size_t)g.H * j;
  const size_t eig_k = (size_t)g.H * g.n2m;
  for (int t = threadIdx.x; t < N * L; t += T) {
    const int l = t % L, k = t / L;
    C v = buf[k * ES + l];
    if (l < nc) {
      // buft / float(n1m*n2m*n3m) / (-ak3(k)-ak1(i)-ak2(j)), zero mode := 0
      if (k == 0 && kx0 + l == 0 && j == 0) v = mk<C>(R(0), R(0));
      else { const R f = eig[(size_t)(kx0 + l) + eig_k * k]; v.x *= f; v.y *= f; }
    } else {
      v = mk<C>(R(0), R(0));
    }
    buf[k * ES + l] = v;
  }
  __syncthreads();
  transform<C, N, L, T, true>(buf, tw);
  store_cols<C, N, LONE>(buf, spec, base, zstride, nc);
}

// Z pass as a periodic tridiagonal solve per (kx, ky) line (fft.cu
// make_ztri): one thread per line (lines numbered kx fastest, so that a
// warp's accesses are adjacent), real and imaginary parts together, the
// sweeps of tridiag_periodic.f90 with the line's factors, in place.  Each
// sweep moves kG elements and their factors into registers with independent
// loads before the kG dependent steps that use them.  The line kx = ky = 0 is
// left to the transform kernel.
template <typename C>
__global__ void __launch_bounds__(64) z_tri(FftArgs<C> F, C* __restrict__ spec) {
  typedef typename Real<C>::T R;
  constexpr int kG = 8;
  const Grid& g = F.g;
  const int n = g.n3m, H = g.H, NT = F.zt_lines;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= H * g.n2m) return;
  const int kx = l % H, ky = l / H;
  if (kx == 0 && ky == 0) return;
  const int lt = kx + H * (ky <= g.n2m - ky ? ky : g.n2m - ky);
  const size_t NS = (size_t)n * NT;
  const R* __restrict__ a = F.ztri + lt;
  const R* __restrict__ b = a + NS;
  const R* __restrict__ q = a + 2 * NS;
  const R* __restrict__ s = a + 3 * NS;
  const R* __restrict__ sc = F.ztri + 4 * NS + 4 * (size_t)lt;
  const R ackl = sc[0], api = sc[1], ami = sc[2], inv_den = sc[3];
  C* __restrict__ base = spec + kx + (size_t)g.HP * ky;
  const size_t st = (size_t)g.HP * g.n2m;
  const C rn = base[(size_t)(n - 1) * st];
  C y = mk<C>(R(0), R(0));
  for (int e0 = 0; e0 < n - 1; e0 += kG) {
    C r[kG];
    R ae[kG], be[kG];
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 + u;
      const bool ok = e < n - 1;
      r[u] = ok ? base[(size_t)e * st] : C{};
      ae[u] = ok ? a[(size_t)e * NT] : R(0);
      be[u] = (ok && e > 0) ? b[(size_t)e * NT] : R(0);
    }
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 + u;
      if (e < n - 1) {
        y = e == 0 ? mk<C>(ae[u] * r[u].x, ae[u] * r[u].y)
                   : mk<C>(ae[u] * r[u].x - be[u] * y.x, ae[u] * r[u].y - be[u] * y.y);
        base[(size_t)e * st] = y;
      }
    }
  }
  C f = mk<C>(R(0), R(0));
  C xnm1 = f;                                          // element n-2 after the backward sweep
  for (int e0 = n - 2; e0 >= 0; e0 -= kG) {
    C yy[kG];
    R qe[kG];
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 - u;
      yy[u] = e >= 0 ? base[(size_t)e * st] : C{};
      qe[u] = e >= 0 ? q[(size_t)e * NT] : R(0);
    }
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 - u;
      if (e >= 0) {
        f = mk<C>(yy[u].x + qe[u] * f.x, yy[u].y + qe[u] * f.y);
        base[(size_t)e * st] = f;
        if (e == n - 2) xnm1 = f;
      }
    }
  }
  const C f1 = f;                                      // element 0 after the backward sweep
  const C xn = mk<C>((rn.x * ackl - api * f1.x - ami * xnm1.x) * inv_den,
                     (rn.y * ackl - api * f1.y - ami * xnm1.y) * inv_den);
  for (int e0 = 0; e0 < n - 1; e0 += kG) {
    C v[kG];
    R se[kG];
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 + u;
      const bool ok = e < n - 1;
      v[u] = ok ? base[(size_t)e * st] : C{};
      se[u] = ok ? s[(size_t)e * NT] : R(0);
    }
#pragma unroll
    for (int u = 0; u < kG; ++u) {
      const int e = e0 + u;
      if (e < n - 1) base[(size_t)e * st] = mk<C>(xn.x * se[u] + v[u].x, xn.y * se[u] + v[u].y);
    }
  }
  base[(size_t)(n - 1) * st] = xn;
}

// shared-memory opt-in for the instances above the default 48 KB
template <typename K>
inline bool smem_attr(Ctx* c, K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return cuda_ok(c, cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                 "fft smem");
}

template <typename C, typename S, int N>
void launch_x_fwd(Ctx* c, const FftArgs<C>& F, const S* src, C* spec) {
  typedef Shape<C, N> Sh;
  auto k = x_fwd<C, S, N>;
  if (!smem_attr(c, k, Sh::smem)) return;
  dim3 grid(div_up(c->g.n2m / 2, Sh::L), c->g.n3m);
  k<<<grid, Sh::T, Sh::smem, c->stream>>>(F, src, spec);
}

template <typename C, int N>
void launch_x_inv(Ctx* c, const FftArgs<C>& F, const C* spec, typename Real<C>::T* dst) {
  typedef Shape<C, N> Sh;
  auto k = x_inv<C, N>;
  if (!smem_attr(c, k, Sh::smem)) return;
  dim3 grid(div_up(c->g.n2m / 2, Sh::L), c->g.n3m);
  k<<<grid, Sh::T, Sh::smem, c->stream>>>(F, spec, dst);
}

// whole tiles of L columns, then the columns left over one line per block
// (H = n1m/2 + 1 leaves the Nyquist column when L divides n1m/2)
// Y and Z passes of the precision form's 256-point transforms with the
// columns staged by bulk tensor copies: a persistent kernel over tiles of 16
// adjacent kx columns (128 bytes per row) -- of one plane k for the y pass
// (MODE 1 forward, 2 inverse), of one ky for the z pass (MODE 0: forward,
// the eigenvalue division, inverse) -- each copied into a ring of
// shared-memory stages ahead of the block; the transforms run in place on
// the stage in the dense layout (16 x 16 engine), the results go back with
// coalesced stores.  The same operations as y_pass / z_solve<float2, 256>
// on the whole tiles (the lone Nyquist column stays with the one-line
// kernels).  Stage waits are bounded (about a second); a timeout sets bit 2
// of `err` and the block leaves after its other copies have landed.
template <int MODE, int NSTAGE>
__global__ void __launch_bounds__(256, 2)
col_pass_tma(const __grid_constant__ CUtensorMap map, FftArgs<float2> F, float2* __restrict__ spec, int ntiles,
             int* __restrict__ err) {
  constexpr int N = 256, L = 16, T = 256;
  constexpr uint32_t kStage = N * L * sizeof(float2);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024u - (tma::smem_addr(smem_raw) & 1023u)) & 1023u);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  float2* tw = reinterpret_cast<float2*>(smem + 128);
  float2* stage0 = reinterpret_cast<float2*>(smem + 128 + N * sizeof(float2));
  const Grid& g = F.g;
  const int tiles_x = g.H / L;
  auto issue = [&](int tile, int s) {
    const int kt = tile % tiles_x, o = tile / tiles_x;     // o: ky (z pass) or k (y pass)
    tma::mbar_arrive_expect_tx(bars + s, kStage);
    if (MODE == 0) tma::load_4d(stage0 + (size_t)s * N * L, &map, bars + s, kt * L, o, 0, 0);
    else tma::load_4d(stage0 + (size_t)s * N * L, &map, bars + s, kt * L, 0, o, 0);
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) tma::mbar_init(bars + s, 1);
    tma::fence_proxy_async();
    for (int s = 0; s < NSTAGE; ++s) {
      const int tile = blockIdx.x + s * gridDim.x;
      if (tile < ntiles) issue(tile, s);
    }
  }
  stage_twiddles<float2, N, T>(tw, MODE == 0 ? F.twz : F.twy);
  __syncthreads();
  const size_t lstride = MODE == 0 ? (size_t)g.HP * g.n2m : (size_t)g.HP;   // element stride of a line
  const size_t eig_k = (size_t)g.H * g.n2m;
  for (int li = 0;; ++li) {
    const int tile = blockIdx.x + li * gridDim.x;
    if (tile >= ntiles) break;
    const int s = li % NSTAGE;
    const bool ok = tma::mbar_wait(bars + s, (uint32_t)((li / NSTAGE) & 1));
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) {
        atomicOr(err, 2);
        for (int kq = 1; kq < NSTAGE; ++kq) {
          const int Lq = li + kq;
          if (blockIdx.x + Lq * gridDim.x < ntiles) tma::mbar_wait(bars + Lq % NSTAGE, (uint32_t)((Lq / NSTAGE) & 1));
        }
      }
      return;
    }
    const int kt = tile % tiles_x, o = tile / tiles_x, kx0 = kt * L;
    float2* buf = stage0 + (size_t)s * N * L;
    if (MODE == 0) {
      const int j = o;
      run16x16<float2, N, L, T, false, true>(buf, tw);
      const float* __restrict__ eig = F.eig + (size_t)g.H * j;
      for (int t = threadIdx.x; t < N * L; t += T) {
        const int l = t % L, k = t / L;
        float2 v = buf[t];
        // buft / float(n1m*n2m*n3m) / (-ak3(k)-ak1(i)-ak2(j)), zero mode := 0
        if (k == 0 && kx0 + l == 0 && j == 0) v = mk<float2>(0.f, 0.f);
        else { const float f = eig[(size_t)(kx0 + l) + eig_k * k]; v.x *= f; v.y *= f; }
        buf[t] = v;
      }
      __syncthreads();
      run16x16<float2, N, L, T, true, true>(buf, tw);
    } else {
      run16x16<float2, N, L, T, MODE == 2, true>(buf, tw);
    }
    const size_t base = MODE == 0 ? (size_t)kx0 + (size_t)g.HP * o : (size_t)kx0 + (size_t)g.HP * g.n2m * o;
    for (int t = threadIdx.x; t < N * L; t += T) {
      const int l = t % L, e = t / L;
      spec[base + l + lstride * e] = buf[t];
    }
    __syncthreads();   // stage s is free again
    if (threadIdx.x == 0) {
      const int next = tile + NSTAGE * gridDim.x;
      if (next < ntiles) {
        tma::fence_proxy_async();
        issue(next, s);
      }
    }
  }
}

// the TMA y (MODE 1 forward, 2 inverse) or z (MODE 0) pass on the whole
// 16-column tiles of a 256-point FP32 transform; false when it does not
// apply (the caller then launches the shared-memory tile kernel)
template <typename C, int N, int MODE>
bool launch_col_tma(Ctx* c, const FftArgs<C>& F, C* spec) {
  if constexpr (!(sizeof(C) == 8 && N == 256)) {
    return false;
  } else {
    constexpr int kStages = 3;
    const Grid& g = c->g;
    const int tiles_x = g.H / 16;
    if (!c->tma || tiles_x < 1 || ((uintptr_t)spec & 15) != 0) return false;
    CUtensorMap map;
    const int box[4] = {16, MODE == 0 ? 1 : N, MODE == 0 ? N : 1, 1};
    if (!tma::encode_fields(&map, spec, 8, g.H, g.n2m, g.n3m, g.HP, (size_t)g.HP * g.n2m * g.n3m, 1, box))
      return false;
    const size_t smem = 1024 + 128 + N * sizeof(float2) + (size_t)kStages * N * 16 * sizeof(float2);
    auto k = col_pass_tma<MODE, kStages>;
    if (!smem_attr(c, k, smem)) return false;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem);
    const int ntiles = tiles_x * (MODE == 0 ? g.n2m : g.n3m);
    const int grid = std::max(1, std::min(ntiles, std::max(1, per_sm) * std::max(1, sms)));
    k<<<grid, 256, smem, c->stream>>>(map, F, spec, ntiles, c->dflag + 2);
    return true;
  }
}

template <typename C, int N>
void launch_y(Ctx* c, const FftArgs<C>& F, C* spec, int sign) {
  typedef Shape<C, N> Sh;
  typedef Shape<C, N, 1> S1;
  auto kf = y_pass<C, N, false>;
  auto ki = y_pass<C, N, true>;
  auto kf1 = y_pass<C, N, false, 1>;
  auto ki1 = y_pass<C, N, true, 1>;
  if (!smem_attr(c, kf, Sh::smem) || !smem_attr(c, ki, Sh::smem) || !smem_attr(c, kf1, S1::smem) ||
      !smem_attr(c, ki1, S1::smem))
    return;
  const int tiles = c->g.H / Sh::L, rest = c->g.H - tiles * Sh::L;
  if (tiles > 0 && !(sign < 0 ? launch_col_tma<C, N, 1>(c, F, spec) : launch_col_tma<C, N, 2>(c, F, spec))) {
    dim3 grid(tiles, c->g.n3m);
    if (sign < 0) kf<<<grid, Sh::T, Sh::smem, c->stream>>>(F, spec, 0);
    else ki<<<grid, Sh::T, Sh::smem, c->stream>>>(F, spec, 0);
  }
  if (rest > 0) {
    dim3 grid(rest, c->g.n3m);
    if (sign < 0) kf1<<<grid, S1::T, S1::smem, c->stream>>>(F, spec, tiles * Sh::L);
    else ki1<<<grid, S1::T, S1::smem, c->stream>>>(F, spec, tiles * Sh::L);
    if (tiles > 0) ++c->launches;      // the caller counts one launch per pass
  }
}

// The same lines chunked (the scheme of the chunked line solves of
// tridiag.cu, on complex values with one table per line): a block holds 32
// lines (lanes, consecutive in kx + H*ky) and the G = n/M chunks of M cells
// (warps, in registers); forward and backward sweeps per chunk from zero
// entries, the chunk entries by a serial scan over the lower chunks in
// shared memory, the periodic closure from elements 0 and n-2, then one
// correction pass.  Table entry q of line lt sits at q*NT + lt (32 lanes read
// consecutive words); lanes without a line (past the end, and the zero line,
// which the transform solves) use line 0's all-zero table and store nothing.
template <typename C, int M>
__global__ void __launch_bounds__(32 * kZtMaxChunks) z_tri_cc(FftArgs<C> F, C* __restrict__ spec) {
  typedef typename Real<C>::T R;
  __shared__ C sC[kZtMaxChunks][32];
  __shared__ C sU[kZtMaxChunks][32];
  __shared__ C sF[3][32];
  const Grid& g = F.g;
  const int n = g.n3m, G = n / M, H = g.H, NT = F.zt_lines;
  const int lane = threadIdx.x, w = threadIdx.y;
  const int l = blockIdx.x * 32 + lane;
  const bool act = l > 0 && l < H * g.n2m;
  const int kx = act ? l % H : 0, ky = act ? l / H : 0;
  const int lt = kx + H * (ky <= g.n2m - ky ? ky : g.n2m - ky);
  const R* __restrict__ X = F.ztri + lt;
  auto T = [&](int q) { return X[(size_t)q * NT]; };
  const size_t st = (size_t)g.HP * g.n2m;
  C* __restrict__ rp = spec + kx + (size_t)g.HP * ky + (size_t)(w * M) * st;
  C r[M];
#pragma unroll
  for (int i = 0; i < M; ++i) r[i] = act ? rp[(size_t)i * st] : mk<C>(R(0), R(0));
  const C rlast = r[M - 1];
  C cf = mk<C>(R(0), R(0));
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const int t = i * G + w;
    const R a = T(t), b = T(n + t);
    cf = mk<C>(a * r[i].x - b * cf.x, a * r[i].y - b * cf.y);
    r[i] = cf;
  }
  sC[w][lane] = cf;
  __syncthreads();
  C y_in = mk<C>(R(0), R(0));
  for (int hh = 0; hh < w; ++hh) {
    const R pl = T(7 * n + hh);
    const C v = sC[hh][lane];
    y_in = mk<C>(v.x + pl * y_in.x, v.y + pl * y_in.y);
  }
  C d = mk<C>(R(0), R(0));
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    const R q = T(2 * n + i * G + w);
    d = mk<C>(r[i].x + q * d.x, r[i].y + q * d.y);
    r[i] = d;
  }
  {
    const R dpf = T(7 * n + 2 * G + w);
    sU[w][lane] = mk<C>(r[0].x + dpf * y_in.x, r[0].y + dpf * y_in.y);
  }
  __syncthreads();
  C f_in = mk<C>(R(0), R(0));
  for (int hh = G - 1; hh > w; --hh) {
    const R qf = T(7 * n + G + hh);
    const C v = sU[hh][lane];
    f_in = mk<C>(v.x + qf * f_in.x, v.y + qf * f_in.y);
  }
  if (w == 0) {
    const R q0 = T(5 * n);
    sF[0][lane] = mk<C>(r[0].x + q0 * f_in.x, r[0].y + q0 * f_in.y);
  }
  if (w == G - 1) {
    const R dp = T(6 * n + (M - 2) * G + w);
    sF[1][lane] = mk<C>(r[M - 2].x + dp * y_in.x, r[M - 2].y + dp * y_in.y);
    sF[2][lane] = rlast;
  }
  __syncthreads();
  const int S = 7 * n + 3 * G;
  const R ackl = T(S), api = T(S + 1), ami = T(S + 2), inv_den = T(S + 3);
  const C f0 = sF[0][lane], f1 = sF[1][lane], rn = sF[2][lane];
  const C xn = mk<C>((rn.x * ackl - api * f0.x - ami * f1.x) * inv_den,
                     (rn.y * ackl - api * f0.y - ami * f1.y) * inv_den);
  if (!act) return;
  const R ac = T(S + 4 + w), bc = T(S + 4 + G + w);
  const C al = mk<C>(y_in.x + ac * xn.x, y_in.y + ac * xn.y);
  const C be = mk<C>(f_in.x + bc * xn.x, f_in.y + bc * xn.y);
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const int t = i * G + w;
    const R dp = T(6 * n + t), qq = T(5 * n + t);
    rp[(size_t)i * st] = mk<C>(r[i].x + dp * al.x + qq * be.x, r[i].y + dp * al.y + qq * be.y);
  }
}

template <typename C, int N>
void launch_z(Ctx* c, const FftArgs<C>& F, C* spec) {
  typedef Shape<C, N> Sh;
  typedef Shape<C, N, 1> S1;
  auto k = z_solve<C, N>;
  auto k1 = z_solve<C, N, 1>;
  if (!smem_attr(c, k, Sh::smem) || !smem_attr(c, k1, S1::smem)) return;
  if (F.ztri && N >= 3) {
    // tridiagonal lines, and the zero line by transform
    const size_t lines = (size_t)c->g.H * c->g.n2m;
    if (F.zt_m == 16) z_tri_cc<C, 16><<<div_up(lines, 32), dim3(32, c->g.n3m / 16), 0, c->stream>>>(F, spec);
    else if (F.zt_m == 8) z_tri_cc<C, 8><<<div_up(lines, 32), dim3(32, c->g.n3m / 8), 0, c->stream>>>(F, spec);
    else z_tri<C><<<div_up(lines, 64), 64, 0, c->stream>>>(F, spec);
    k1<<<dim3(1, 1), S1::T, S1::smem, c->stream>>>(F, spec, 0);
    ++c->launches;                 // the caller counts one launch per pass
    return;
  }
  const int tiles = c->g.H / Sh::L, rest = c->g.H - tiles * Sh::L;
  if (tiles > 0 && !launch_col_tma<C, N, 0>(c, F, spec))
    k<<<dim3(tiles, c->g.n2m), Sh::T, Sh::smem, c->stream>>>(F, spec, 0);
  if (rest > 0) {
    k1<<<dim3(rest, c->g.n2m), S1::T, S1::smem, c->stream>>>(F, spec, tiles * Sh::L);
    if (tiles > 0) ++c->launches;      // the caller counts one launch per pass
  }
}

}  // namespace fastfft

// line lengths with an instance
#define MIBM_FFT_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512)

}  // namespace mibm
