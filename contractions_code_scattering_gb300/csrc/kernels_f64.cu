// Plain FP64 engine kernels: batched complex block GEMM, fused Hadamard traces,
// deterministic row sums and the source-time average.
//
// On GB300 the FP64 pipe delivers about 2 DFMA per clock per SM, so these
// kernels are bound by that pipe, not by memory.  A warp's DFMA occupies the
// pipe for all 32 lanes, also where lanes are masked off, so the design goal is
// tiles that cover the Nev x Nev block without padded lanes (the tile edge is
// an autotuner choice: 32, 50 or 20) while keeping the summation order of the
// reference (k ascending for every matrix element).
#include <algorithm>
#include <cmath>

#include "kernels.h"

namespace ctr {

// ----------------------------------------------------------------- GEMM
// C = sum_q w_q * op(A_q) * op(B_q) for Nev x Nev row-major blocks, where op is
// identity or conjugate transpose (flags bit q: A_q, bit 4+q: B_q).  One CTA
// computes a 32 x 32 output tile; 256 threads, 2 x 2 outputs each.
constexpr int GT = 32;   // output tile edge
constexpr int GK = 16;   // K chunk staged in shared memory

__global__ void __launch_bounds__(256) zgemm_f64_kernel(const ZTask* __restrict__ tasks, int ntask, int N,
                                                        int tiles_per_dim) {
  __shared__ double2 As[GT][GK + 1];
  __shared__ double2 Bs[GK][GT + 1];
  const int tiles = tiles_per_dim * tiles_per_dim;
  const int task_id = blockIdx.x / tiles;
  if (task_id >= ntask) return;
  const int tile = blockIdx.x % tiles;
  const int i0 = (tile / tiles_per_dim) * GT, j0 = (tile % tiles_per_dim) * GT;
  const ZTask& T = tasks[task_id];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;

  double2 acc[2][2];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) acc[a][b] = make_double2(0.0, 0.0);

  for (int q = 0; q < T.nterm; q++) {
    const double2* A = T.A[q];
    const double2* B = T.B[q];
    const bool ca = (T.flags >> q) & 1, cb = (T.flags >> (4 + q)) & 1;
    double2 part[2][2];
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) part[a][b] = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < N; k0 += GK) {
      // stage A rows i0..i0+31, cols k0..k0+15 and B rows k0..k0+15, cols j0..j0+31
      for (int e = threadIdx.x; e < GT * GK; e += 256) {
        int r = e / GK, c = e % GK;
        int gi = i0 + r, gk = k0 + c;
        double2 v = make_double2(0.0, 0.0);
        if (gi < N && gk < N) {
          if (!ca) v = A[(size_t)gi * N + gk];
          else { v = A[(size_t)gk * N + gi]; v.y = -v.y; }
        }
        As[r][c] = v;
        int rk = e / GT, cj = e % GT;
        int gk2 = k0 + rk, gj = j0 + cj;
        double2 u = make_double2(0.0, 0.0);
        if (gk2 < N && gj < N) {
          if (!cb) u = B[(size_t)gk2 * N + gj];
          else { u = B[(size_t)gj * N + gk2]; u.y = -u.y; }
        }
        Bs[rk][cj] = u;
      }
      __syncthreads();
      const int kmax = min(GK, N - k0);
      const bool r0 = i0 + ty < N, r1 = i0 + ty + 16 < N, c0 = j0 + tx < N, c1 = j0 + tx + 16 < N;
      if (r0 || r1) {
        for (int kk = 0; kk < kmax; kk++) {
          double2 a0 = As[ty][kk], a1 = As[ty + 16][kk];
          double2 b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
          if (r0 && c0) cmac(part[0][0], a0, b0);
          if (r0 && c1) cmac(part[0][1], a0, b1);
          if (r1 && c0) cmac(part[1][0], a1, b0);
          if (r1 && c1) cmac(part[1][1], a1, b1);
        }
      }
      __syncthreads();
    }
    const double2 w = make_double2((double)T.wre[q], (double)T.wim[q]);
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) {
        if (q == 0 && w.x == 1.0 && w.y == 0.0) acc[a][b] = part[a][b];
        else {
          double2 t = cmul(w, part[a][b]);
          acc[a][b].x += t.x;
          acc[a][b].y += t.y;
        }
      }
  }
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      int gi = i0 + ty + 16 * a, gj = j0 + tx + 16 * b;
      if (gi < N && gj < N) T.C[(size_t)gi * N + gj] = acc[a][b];
    }
}

// The same product with a T x T output tile: (T/TM) x (T/TN) threads, thread
// (ty, tx) computing rows ty + a T/TM (a < TM) and columns tx + b T/TN (b < TN),
// K staged KC at a time.  T = 50 covers Nev = 100 with 250 busy lanes of 256.
template <int T, int TM, int TN, int KC>
__global__ void __launch_bounds__((T / TM) * (T / TN), 2) zgemm_f64_tile_kernel(const ZTask* __restrict__ tasks,
                                                                             int ntask, int N, int tiles_per_dim) {
  constexpr int RY = T / TM, RX = T / TN, NT = RY * RX;
  static_assert(RY * TM == T && RX * TN == T, "tile split");
  __shared__ double2 As[T][KC + 1];
  __shared__ double2 Bs[KC][T + 1];
  const int tiles = tiles_per_dim * tiles_per_dim;
  const int task_id = blockIdx.x / tiles;
  if (task_id >= ntask) return;
  const int tile = blockIdx.x % tiles;
  const int i0 = (tile / tiles_per_dim) * T, j0 = (tile % tiles_per_dim) * T;
  const ZTask& Tk = tasks[task_id];
  const int ty = threadIdx.x / RX, tx = threadIdx.x % RX;
  bool rv[TM], cv[TN];
#pragma unroll
  for (int a = 0; a < TM; a++) rv[a] = i0 + ty + a * RY < N;
#pragma unroll
  for (int b = 0; b < TN; b++) cv[b] = j0 + tx + b * RX < N;

  double2 acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; a++)
#pragma unroll
    for (int b = 0; b < TN; b++) acc[a][b] = make_double2(0.0, 0.0);

  for (int q = 0; q < Tk.nterm; q++) {
    const double2* A = Tk.A[q];
    const double2* B = Tk.B[q];
    const bool ca = (Tk.flags >> q) & 1, cb = (Tk.flags >> (4 + q)) & 1;
    double2 part[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; a++)
#pragma unroll
      for (int b = 0; b < TN; b++) part[a][b] = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < N; k0 += KC) {
      for (int e = threadIdx.x; e < T * KC; e += NT) {
        const int r = e / KC, c = e % KC, gi = i0 + r, gk = k0 + c;
        double2 v = make_double2(0.0, 0.0);
        if (gi < N && gk < N) {
          if (!ca) v = A[(size_t)gi * N + gk];
          else { v = A[(size_t)gk * N + gi]; v.y = -v.y; }
        }
        As[r][c] = v;
        const int rk = e / T, cj = e % T, gk2 = k0 + rk, gj = j0 + cj;
        double2 u = make_double2(0.0, 0.0);
        if (gk2 < N && gj < N) {
          if (!cb) u = B[(size_t)gk2 * N + gj];
          else { u = B[(size_t)gj * N + gk2]; u.y = -u.y; }
        }
        Bs[rk][cj] = u;
      }
      __syncthreads();
      const int kmax = min(KC, N - k0);
      for (int kk = 0; kk < kmax; kk++) {
        double2 av[TM], bv[TN];
#pragma unroll
        for (int a = 0; a < TM; a++) av[a] = As[ty + a * RY][kk];
#pragma unroll
        for (int b = 0; b < TN; b++) bv[b] = Bs[kk][tx + b * RX];
#pragma unroll
        for (int a = 0; a < TM; a++)
#pragma unroll
          for (int b = 0; b < TN; b++)
            if (rv[a] && cv[b]) cmac(part[a][b], av[a], bv[b]);
      }
      __syncthreads();
    }
    const double2 w = make_double2((double)Tk.wre[q], (double)Tk.wim[q]);
#pragma unroll
    for (int a = 0; a < TM; a++)
#pragma unroll
      for (int b = 0; b < TN; b++) {
        if (q == 0 && w.x == 1.0 && w.y == 0.0) acc[a][b] = part[a][b];
        else {
          const double2 t = cmul(w, part[a][b]);
          acc[a][b].x += t.x;
          acc[a][b].y += t.y;
        }
      }
  }
#pragma unroll
  for (int a = 0; a < TM; a++)
#pragma unroll
    for (int b = 0; b < TN; b++)
      if (rv[a] && cv[b]) Tk.C[(size_t)(i0 + ty + a * RY) * N + (j0 + tx + b * RX)] = acc[a][b];
}

// FP64 matrix-instruction form (mma.sync m8n8k4 f64, the "DMMA" path of the
// FP64 pipe, which delivers more flops per pipe cycle than DFMA on GB300).
// CTA = one task x one block of NFC column fragments; warp w owns output rows
// 8w .. 8w+7 (NFR warps cover N <= 8 NFR rows); fragments past N are skipped.  Fragment layouts (PTX ISA,
// m8n8k4 .f64): A 8x4 row-major, lane holds A[lane/4][lane%4]; B 4x8
// column-major, lane holds B[lane%4][lane/4]; C 8x8, lane holds
// C[lane/4][2 (lane%4) + {0,1}].  Complex: Cr += Ar Br + (-Ai) Bi,
// Ci += Ar Bi + Ai Br.  The task weights must be exact multipliers (a real or
// an imaginary power of two, or zero), which the launcher checks: they scale
// A as it is staged, and all terms accumulate into one sum.
__device__ __forceinline__ void dmma884(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

template <int NFR, int NFC>
__global__ void __launch_bounds__(NFR * 32, 1) zgemm_f64_dmma_kernel(const ZTask* __restrict__ tasks, int ntask,
                                                                     int N, int ncb) {
  constexpr int KC = 8, RM = NFR * 8, CN = NFC * 8, NT = NFR * 32;
  __shared__ double2 As[RM][KC + 1];
  __shared__ double2 Bs[KC][CN + 1];
  const int task_id = blockIdx.x / ncb;
  if (task_id >= ntask) return;
  const int j0 = (blockIdx.x % ncb) * CN;
  const ZTask& Tk = tasks[task_id];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  double cr[NFC][2], ci[NFC][2];
#pragma unroll
  for (int f = 0; f < NFC; f++) cr[f][0] = cr[f][1] = ci[f][0] = ci[f][1] = 0.0;
  for (int q = 0; q < Tk.nterm; q++) {
    const double2* A = Tk.A[q];
    const double2* B = Tk.B[q];
    const bool ca = (Tk.flags >> q) & 1, cb = (Tk.flags >> (4 + q)) & 1;
    const double wr = (double)Tk.wre[q], wi = (double)Tk.wim[q];
    for (int k0 = 0; k0 < N; k0 += KC) {
      for (int e = threadIdx.x; e < RM * KC; e += NT) {
        const int r = e / KC, c = e % KC, gk = k0 + c;
        double2 v = make_double2(0.0, 0.0);
        if (r < N && gk < N) {
          if (!ca) v = A[(size_t)r * N + gk];
          else { v = A[(size_t)gk * N + r]; v.y = -v.y; }
          v = make_double2(wr * v.x - wi * v.y, wr * v.y + wi * v.x);  // exact: w is +-2^e or +-i 2^e
        }
        As[r][c] = v;
      }
      for (int e = threadIdx.x; e < KC * CN; e += NT) {
        const int rk = e / CN, cj = e % CN, gk = k0 + rk, gj = j0 + cj;
        double2 u = make_double2(0.0, 0.0);
        if (gk < N && gj < N) {
          if (!cb) u = B[(size_t)gk * N + gj];
          else { u = B[(size_t)gj * N + gk]; u.y = -u.y; }
        }
        Bs[rk][cj] = u;
      }
      __syncthreads();
#pragma unroll
      for (int ks = 0; ks < KC; ks += 4) {
        const double2 a = As[warp * 8 + g][ks + t];
        const double nai = -a.y;
#pragma unroll
        for (int f = 0; f < NFC; f++) {
          if (j0 + f * 8 >= N) break;  // fragments past the block (uniform across the CTA)
          const double2 b = Bs[ks + t][f * 8 + g];
          dmma884(cr[f][0], cr[f][1], a.x, b.x);
          dmma884(cr[f][0], cr[f][1], nai, b.y);
          dmma884(ci[f][0], ci[f][1], a.x, b.y);
          dmma884(ci[f][0], ci[f][1], a.y, b.x);
        }
      }
      __syncthreads();
    }
  }
  const int row = warp * 8 + g;
  if (row < N)
#pragma unroll
    for (int f = 0; f < NFC; f++)
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int col = j0 + f * 8 + 2 * t + i;
        if (col < N) Tk.C[(size_t)row * N + col] = make_double2(cr[f][i], ci[f][i]);
      }
}

// ---------------------------------------------------------------- trace
// The error scale sum (|Re x| + |Im x|)(|Re y| + |Im y|) of a trace needs a few
// significant bits, not FP64: it is accumulated in FP32 from the doubles' high
// words, scaled by 2^TRACE_ABS_SHIFT so that products from 2^-206 to 2^48 stay
// in FP32's range (smaller ones flush to zero, which the refinement checks
// treat as "flag if the value is not zero"), with integer operations only, so
// that the FP64 pipe, the bound of these kernels on GB300, does just the four
// FMAs of the complex product.
constexpr int TRACE_ABS_SHIFT = 40;

// |v| 2^TRACE_ABS_SHIFT as a float, the mantissa truncated to 20 bits; 0 below
// FP32's normal range, infinity above it
__device__ __forceinline__ float abs_scaled_f32(double v) {
  const int hi = __double2hiint(v) & 0x7FFFFFFF;
  const int e = (hi >> 20) - 1023 + 127 + TRACE_ABS_SHIFT;
  if (e <= 0) return 0.f;
  if (e >= 255) return __int_as_float(0x7F800000);
  return __int_as_float((e << 23) | ((hi & 0xFFFFF) << 3));
}

__device__ __forceinline__ float abs1_scaled_f32(double2 v) { return abs_scaled_f32(v.x) + abs_scaled_f32(v.y); }

// out = coef * sum_e X_e * conj(Y_e) over the Nev*Nev elements (mode 0), or
// coef * sum_ij X_ij * Y_ji = coef * Tr[X Y] (mode 1).  One CTA per task; the
// reduction tree is fixed, so results are bitwise reproducible.
__global__ void __launch_bounds__(256) trace_f64_kernel(const TraceTask* __restrict__ tasks, int ntask, int N) {
  const int t = blockIdx.x;
  if (t >= ntask) return;
  const TraceTask& T = tasks[t];
  const int n2 = N * N;
  const bool want_abs = T.absout != nullptr;
  double re = 0.0, im = 0.0;
  float abf = 0.f;
  // two FMAs into each accumulator per element (the FP64 pipe is the bound)
  if (T.mode == 0) {
    for (int e = threadIdx.x; e < n2; e += 256) {
      double2 x = T.X[e], y = T.Y[e];
      re = fma(x.x, y.x, re);
      re = fma(x.y, y.y, re);
      im = fma(x.y, y.x, im);
      im = fma(-x.x, y.y, im);
      if (want_abs) abf = fmaf(abs1_scaled_f32(x), abs1_scaled_f32(y), abf);
    }
  } else {
    for (int e = threadIdx.x; e < n2; e += 256) {
      int i = e / N, j = e % N;
      double2 x = T.X[e], y = T.Y[(size_t)j * N + i];
      re = fma(x.x, y.x, re);
      re = fma(-x.y, y.y, re);
      im = fma(x.x, y.y, im);
      im = fma(x.y, y.x, im);
      if (want_abs) abf = fmaf(abs1_scaled_f32(x), abs1_scaled_f32(y), abf);
    }
  }
  re = block_sum_256(re);
  im = block_sum_256(im);
  double ab = 0.0;
  if (want_abs) ab = block_sum_256((double)abf) * 0x1p-80;  // 2^(-2 TRACE_ABS_SHIFT)
  if (threadIdx.x == 0) {
    double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
    double2 s = make_double2(re, im);
    *T.out = cmul(c, s);
    if (want_abs) *T.absout = sqrt(c.x * c.x + c.y * c.y) * ab;
  }
}

// ------------------------------------------------------------- row sums
// out[p][o] = sum_{k in [off[o], off[o+1])} rows[p][idx[k]]  (ascending idx)
__global__ void rowsum_kernel(const double2* __restrict__ rows, int nrows, const int* __restrict__ off,
                              const int* __restrict__ idx, int nout, int npair, double2* __restrict__ out,
                              size_t out_pair_stride) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= npair * nout) return;
  int p = g / nout, o = g % nout;
  double re = 0.0, im = 0.0;
  for (int k = off[o]; k < off[o + 1]; k++) {
    double2 v = rows[(size_t)p * nrows + idx[k]];
    re += v.x;
    im += v.y;
  }
  out[(size_t)p * out_pair_stride + o] = make_double2(re, im);
}

__global__ void rowsum_refine_kernel(const double2* __restrict__ rows, const double* __restrict__ rabs, int nrows,
                                     const int* __restrict__ off, const int* __restrict__ idx, int nout, int npair,
                                     double2* __restrict__ out, double eps_over_tol, int* __restrict__ count,
                                     int* __restrict__ list, int pair_base) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= npair * nout) return;
  const int p = g / nout, o = g % nout;
  double re = 0.0, im = 0.0, sc = 0.0;
  for (int k = off[o]; k < off[o + 1]; k++) {
    const size_t r = (size_t)p * nrows + idx[k];
    re += rows[r].x;
    im += rows[r].y;
    sc += rabs[r];
  }
  out[(size_t)p * nout + o] = make_double2(re, im);
  // flagged: an error estimate above the tolerance (or not a number), or an
  // error scale that underflowed while the value did not
  const double mag = sqrt(re * re + im * im);
  if (eps_over_tol > 0.0 && (!(sc * eps_over_tol <= mag) || (sc == 0.0 && mag > 0.0))) {
    const int slot = atomicAdd(count, 1);
    list[slot] = (pair_base + p) * nout + o;
  }
}

// Smallest trusted error scale sum |coef| sum |A||B| of a float-float entry.
constexpr double FF_MIN_SCALE = 0x1p-90;

__global__ void rowsum_coef_refine_kernel(const double2* __restrict__ tr, const double* __restrict__ trabs, int ntr,
                                          const int* __restrict__ off, const int* __restrict__ idx,
                                          const int* __restrict__ tix, const float* __restrict__ coef, int nout,
                                          int npair, double2* __restrict__ out, double eps_over_tol,
                                          int* __restrict__ count, int* __restrict__ list, int pair_base) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= npair * nout) return;
  const int p = g / nout, o = g % nout;
  double re = 0.0, im = 0.0, sc = 0.0;
  for (int k = off[o]; k < off[o + 1]; k++) {
    const int r = idx[k];
    const size_t t = (size_t)p * ntr + tix[r];
    const double cr = coef[2 * r], ci = coef[2 * r + 1];
    const double2 v = tr[t];
    re += cr * v.x - ci * v.y;
    im += cr * v.y + ci * v.x;
    sc += sqrt(cr * cr + ci * ci) * trabs[t];
  }
  out[(size_t)p * nout + o] = make_double2(re, im);
  // flagged: an error estimate above the tolerance, a NaN (a product whose
  // scale left the float-float range), or an error scale so small that the
  // FP32 words of its traces may have underflowed
  if (eps_over_tol > 0.0 && (!(sc * eps_over_tol <= sqrt(re * re + im * im)) || sc < FF_MIN_SCALE)) {
    const int slot = atomicAdd(count, 1);
    list[slot] = (pair_base + p) * nout + o;
  }
}

__global__ void scatter_kernel(const int* __restrict__ where, const double2* __restrict__ vals, int n,
                               double2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[where[i]] = vals[i];
}

// -------------------------------------------------------- source average
__global__ void source_average_kernel(int Nt, int ncorr, const double2* __restrict__ corr, double scale,
                                      double2* __restrict__ avg) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= Nt * ncorr) return;
  int dt = g / ncorr, c = g % ncorr;
  double re = 0.0, im = 0.0;
  for (int ti = 0; ti < Nt; ti++) {
    int tf = (ti + dt) % Nt;
    double2 v = corr[((size_t)tf * Nt + ti) * ncorr + c];
    re += v.x;
    im += v.y;
  }
  avg[g] = make_double2(re / Nt * scale, im / Nt * scale);
}

// --------------------------------------------------------------- launchers
// Variants of the FP64 block GEMM (autotuner knob "zgemm_f64.tile"): DFMA
// tiles of edge 32, 50 and 20, and matrix-instruction (DMMA) forms for
// N <= 104 (13 row strips x 7 column fragments a CTA) and N <= 128 (16 x 8).
static const int kTileEdge[] = {32, 50, 20};
constexpr int kTileVariants = 5;

static bool dmma_fits(int v, int N) { return (v == 3 && N <= 104) || (v == 4 && N <= 128); }

static int launch_zgemm_variant(int v, const ZTask* d_tasks, int ntask, int N, cudaStream_t s) {
  if (v >= 3) {
    if (!dmma_fits(v, N)) return fail(CTR_ERR_ARG, "zgemm_f64: variant %d does not cover Nev = %d", v, N);
    const int nfc = v == 3 ? 7 : 8, ncb = ((N + 7) / 8 + nfc - 1) / nfc;
    const long long blocks = (long long)ntask * ncb;
    if (blocks > 0x7fffffffLL) return fail(CTR_ERR_ARG, "zgemm_f64: too many tasks (%d)", ntask);
    TimedLaunch tl(s, "zgemm_f64");
    if (v == 3)
      zgemm_f64_dmma_kernel<13, 7><<<(unsigned)blocks, 13 * 32, 0, s>>>(d_tasks, ntask, N, ncb);
    else
      zgemm_f64_dmma_kernel<16, 8><<<(unsigned)blocks, 16 * 32, 0, s>>>(d_tasks, ntask, N, ncb);
    CTR_CUDA(cudaGetLastError());
    return CTR_OK;
  }
  const int T = kTileEdge[v];
  const int tpd = (N + T - 1) / T;
  const long long blocks = (long long)ntask * tpd * tpd;
  if (blocks > 0x7fffffffLL) return fail(CTR_ERR_ARG, "zgemm_f64: too many tasks (%d)", ntask);
  TimedLaunch tl(s, "zgemm_f64");
  switch (v) {
    case 0: zgemm_f64_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_tasks, ntask, N, tpd); break;
    case 1: zgemm_f64_tile_kernel<50, 5, 2, 10><<<(unsigned)blocks, 250, 0, s>>>(d_tasks, ntask, N, tpd); break;
    default: zgemm_f64_tile_kernel<20, 2, 1, 10><<<(unsigned)blocks, 200, 0, s>>>(d_tasks, ntask, N, tpd); break;
  }
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

// A weight the DMMA form can fold into A exactly: zero, or a real or imaginary
// power of two (the gamma5 signs and dyadic factors of the diagram tables).
static bool exact_weight(float re, float im) {
  auto pow2 = [](float x) {
    int e;
    return std::fabs(std::frexp(x, &e)) == 0.5f;
  };
  return (re == 0.f && (im == 0.f || pow2(im))) || (im == 0.f && pow2(re));
}

int launch_zgemm_f64(const ZTask* d_tasks, int ntask, int N, cudaStream_t s, const ZTask* h_tasks) {
  if (ntask == 0) return CTR_OK;
  // DMMA forms need exact weights; without the host copy they are not offered
  bool exact = h_tasks != nullptr;
  for (int t = 0; exact && t < ntask; t++)
    for (int q = 0; q < h_tasks[t].nterm; q++)
      if (!exact_weight(h_tasks[t].wre[q], h_tasks[t].wim[q])) exact = false;
  // default: the DFMA edge that pads Nev least (ties to the larger tile).  With
  // the complex multiply-accumulate as four FMAs it beat the DMMA forms at every
  // Nev measured on GB300 (Nev = 100: 89 ms against 117 ms per batch of the rho
  // workload; Nev = 128: 112 ms against 127 ms); the DMMA forms stay candidates.
  int dflt = 0;
  long long best = -1;
  for (int v = 0; v < 3; v++) {
    const long long T = kTileEdge[v], cover = ((N + T - 1) / T) * T;
    if (best < 0 || cover < best) best = cover, dflt = v;
  }
  const int ncand = exact && N > 64 ? kTileVariants : 3;
  int v = dflt;
  CTR_TRY(tune_resolve("zgemm_f64.tile", "nev=" + std::to_string(N) + (exact ? ",exact" : ""), ncand, dflt, s,
                       [&](int c) {
                         if (c >= 3 && !dmma_fits(c, N)) return launch_zgemm_variant(dflt, d_tasks, ntask, N, s);
                         return launch_zgemm_variant(c, d_tasks, ntask, N, s);
                       },
                       &v));
  if (v >= 3 && !dmma_fits(v, N)) v = dflt;
  return launch_zgemm_variant(v, d_tasks, ntask, N, s);
}

int launch_trace_f64(const TraceTask* d_tasks, int ntask, int N, cudaStream_t s) {
  if (ntask == 0) return CTR_OK;
  TimedLaunch tl(s, "trace_f64");
  trace_f64_kernel<<<ntask, 256, 0, s>>>(d_tasks, ntask, N);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_rowsum(const double2* rows, int nrows, const int* off, const int* idx, int nout, int npair,
                  double2* out, size_t out_pair_stride, cudaStream_t s) {
  int n = npair * nout;
  if (n == 0) return CTR_OK;
  TimedLaunch tl(s, "rowsum");
  rowsum_kernel<<<(n + 255) / 256, 256, 0, s>>>(rows, nrows, off, idx, nout, npair, out, out_pair_stride);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_source_average(int Nt, int ncorr, const double2* corr, double scale, double2* avg, cudaStream_t s) {
  int n = Nt * ncorr;
  if (n == 0) return CTR_OK;
  TimedLaunch tl(s, "source_average");
  source_average_kernel<<<(n + 255) / 256, 256, 0, s>>>(Nt, ncorr, corr, scale, avg);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_rowsum_refine(const double2* rows, const double* rabs, int nrows, const int* off, const int* idx, int nout,
                         int npair, double2* out, double eps_over_tol, int* count, int* list, int pair_base,
                         cudaStream_t s) {
  const int n = npair * nout;
  if (n == 0) return CTR_OK;
  TimedLaunch tl(s, "rowsum_refine");
  rowsum_refine_kernel<<<(n + 255) / 256, 256, 0, s>>>(rows, rabs, nrows, off, idx, nout, npair, out, eps_over_tol,
                                                        count, list, pair_base);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_rowsum_coef_refine(const double2* tr, const double* trabs, int ntr, const int* off, const int* idx,
                              const int* tix, const float* coef, int nout, int npair, double2* out,
                              double eps_over_tol, int* count, int* list, int pair_base, cudaStream_t s) {
  const int n = npair * nout;
  if (n == 0) return CTR_OK;
  TimedLaunch tl(s, "rowsum_refine");
  rowsum_coef_refine_kernel<<<(n + 255) / 256, 256, 0, s>>>(tr, trabs, ntr, off, idx, tix, coef, nout, npair, out,
                                                             eps_over_tol, count, list, pair_base);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

__global__ void stage_copy_kernel(int4* __restrict__ dst, const int4* __restrict__ src, size_t n16,
                                  uint8_t* __restrict__ dtail, const uint8_t* __restrict__ stail, int ntail) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
  if (blockIdx.x == 0 && threadIdx.x < ntail) dtail[threadIdx.x] = stail[threadIdx.x];
}

int launch_stage_copy(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return CTR_OK;
  // both buffers are at least 16-byte aligned (cudaMalloc / cudaHostAlloc)
  const size_t n16 = bytes / 16;
  const int ntail = (int)(bytes % 16);
  const int grid = (int)std::min<size_t>(1024, std::max<size_t>(1, (n16 + 255) / 256));
  TimedLaunch tl(s, "stage_copy");
  stage_copy_kernel<<<grid, 256, 0, s>>>((int4*)dst, (const int4*)src, n16, (uint8_t*)dst + n16 * 16,
                                         (const uint8_t*)src + n16 * 16, ntail);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

__global__ void readback_kernel(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, size_t bytes, int words) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (words) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < bytes / 4; i += stride)
      ((uint32_t*)dst)[i] = ((const uint32_t*)src)[i];
  } else {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < bytes; i += stride) dst[i] = src[i];
  }
}

int launch_readback(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return CTR_OK;
  const int words = (((uintptr_t)dst | (uintptr_t)src | bytes) & 3) == 0;
  const size_t n = words ? bytes / 4 : bytes;
  const int grid = (int)std::min<size_t>(256, std::max<size_t>(1, (n + 255) / 256));
  TimedLaunch tl(s, "readback");
  readback_kernel<<<grid, 256, 0, s>>>((uint8_t*)dst, (const uint8_t*)src, bytes, words);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_scatter(const int* where, const double2* vals, int n, double2* out, cudaStream_t s) {
  if (n == 0) return CTR_OK;
  TimedLaunch tl(s, "refine_scatter");
  scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(where, vals, n, out);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

}  // namespace ctr
