// Split-precision tensor-core engine.
//
// A complex FP64 product C = X * Y (Nev <= 128) is computed on the tcgen05
// tensor cores as follows.
//  * Slicing.  Every row of the left operand X (every column of the right
//    operand Y) gets a power-of-two scale 2^E with all |entries| < 2^E.  The
//    scaled magnitude |x|/2^E is written in balanced base-512 digits,
//    |x|/2^E = sum_s d_s 2^{-8-9s}, d_0 in [0,256], d_s in [-256,255] (s >= 1),
//    taken straight from the FP64 bit pattern with integer operations (no FP64
//    arithmetic).  Every |d_s| <= 256 is an integer of at most 8 significant
//    bits, so each piece sign*d_s*2^{-8-9s} is exact in BF16 while carrying 9
//    bits.  The digits are rounded to nearest at the last one: with
//    NSLICE = 5 the residual is <= 2^-45 of 2^E and unbiased.
//  * MMA.  Slice pairs (i,j) with i+j <= 4 (15 pairs) are multiplied with
//    tcgen05.mma kind::f16 (BF16 in, FP32 accumulate in TMEM); the complex
//    product takes 4 real MMAs per pair (the -Xi*Yi term uses the A-negate bit).
//    Pairs accumulate in four levels, i+j = 0, 1, 2 and >= 3.  Levels 0-2 hold
//    integer multiples of 2^-16, 2^-25, 2^-34 below 2^24 units (level 0 for any
//    data with K <= 128, levels 1-2 for non-adversarial data), which the FP32
//    tensor-core accumulation keeps exactly; measured on GB300, an accumulator
//    mixing magnitudes loses low bits to truncation (~2^-17 of its size over a
//    full K loop), which the separate levels confine to level >= 3, i.e. to
//    ~2^-44 of the result.  Level values are combined in float-float (two FP32
//    words, ~48 bits) and scaled by 2^{E_row + E_col}.
//  * Data movement.  Slices are stored pre-tiled in the UMMA K-major
//    no-swizzle core-matrix layout, grouped by K-chunk of 16, so one pipeline
//    stage (all slices and both real/imag planes of one K-chunk) is one
//    contiguous bulk async copy per operand.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>

#include "kernels.h"
#include "sm100_ptx.cuh"
#include "split.h"

namespace ctr {

using namespace ptx;

// ----------------------------------------------------------- slicing math
__device__ __forceinline__ int f64_exp_bound(double x) {
  // e with |x| < 2^e for normal x; very small for zero / subnormal
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7FF);
  return be == 0 ? -30000 : be - 1022;
}

// f64_fixed of x * (+-2^k) without the FP64 product: a power-of-two factor
// only moves the exponent (and flips the sign when `flip`).  A product that
// would leave the normal range (|x 2^k| < 2^-1022) gives 0, as the subnormal
// FP64 product does in f64_fixed; the sign is the product's in every case.
__device__ __forceinline__ uint64_t f64_fixed_pow2(double x, int k, bool flip, int E, bool& neg) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  neg = ((b >> 63) != 0) != flip;
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0 || be + k <= 0) return 0;
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  const int sh = be + k - 1012 - E;
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0;
  return m >> (-sh);
}

// 63-bit fixed-point magnitude of x / 2^E (|x| < 2^E) and its sign.
__device__ __forceinline__ uint64_t f64_fixed(double x, int E, bool& neg) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  neg = (b >> 63) != 0;
  const int be = (int)((b >> 52) & 0x7FF);
  if (be == 0) return 0;
  const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  const int sh = be - 1012 - E;  // <= 10 because |x| < 2^E
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0;
  return m >> (-sh);
}

// Balanced digits of the magnitude U (63-bit fixed point, U < 2^63).  Digit s
// sits at bit slice_shift(s) = 55 - 9s.  Adding 256 at every digit position
// s >= 1 and half a unit of the last one turns the balanced digits into the
// plain base-512 digits of W = U + digit_offset():
//   d_0 = W >> 55 in [0, 256],  d_s = ((W >> (55 - 9s)) & 511) - 256,
// and sum_s d_s 2^{55-9s} is U rounded to nearest at the last digit
// (W < 2^63 + 2^55, no overflow).
__host__ __device__ constexpr int slice_shift(int s) { return 55 - 9 * s; }

__host__ __device__ constexpr uint64_t digit_offset(int nslice) {
  uint64_t o = 1ull << (slice_shift(nslice - 1) - 1);
  for (int s = 1; s < nslice; s++) o += 256ull << slice_shift(s);
  return o;
}

template <int NS = SPLIT_NSLICE>
__device__ __forceinline__ uint64_t round_fixed(uint64_t U) { return U + digit_offset(NS); }

// FP32 bits of digit s of W, d_s 2^{-8-9s} with its sign flipped when neg, built
// without an integer conversion: the 9-bit field f of the digit becomes the top
// of the significand of X = 2^q (1 + f/512), q = 1 - 9s, and X - 2^q (1 + o/512)
// = (f - o) 2^{q-9} exactly (the operands are within a factor 2), with o = 0
// for s = 0 (d_0 = f) and o = 256 otherwise (d_s = f - 256).  At most 9
// significant bits, so the value is exact in BF16 and its BF16 encoding is the
// high half of these bits.  A zero digit gives +0 (-0 when neg).
__device__ __forceinline__ uint32_t slice_bits(uint64_t W, int s, bool neg) {
  const int p = slice_shift(s);
  const uint32_t w = p >= 14 ? (uint32_t)(W >> (p - 14)) : (uint32_t)W << (14 - p);
  const uint32_t eb = (uint32_t)(128 - 9 * s) << 23;
  const float v = __uint_as_float((w & (511u << 14)) | eb) - __uint_as_float(eb | (s ? (1u << 22) : 0u));
  return __float_as_uint(v) ^ (neg ? 0x80000000u : 0u);
}

__device__ __forceinline__ __nv_bfloat16 slice_bf16(uint64_t W, int s, bool neg) {
  return __ushort_as_bfloat16((unsigned short)(slice_bits(W, s, neg) >> 16));
}

// The value of slice_bf16 before its conversion to BF16 (exact in BF16).
__device__ __forceinline__ float slice_f32(uint64_t W, int s, bool neg) { return __uint_as_float(slice_bits(W, s, neg)); }

// Two slices of adjacent k as one packed BF16 pair (k in the low half).
__device__ __forceinline__ uint32_t slice_pair(uint64_t W0, bool n0, uint64_t W1, bool n1, int s) {
  return __byte_perm(slice_bits(W0, s, n0), slice_bits(W1, s, n1), 0x7632);
}

// BF16 bits of -x for BF16 bits x (one value, or a packed pair).
__device__ __forceinline__ __nv_bfloat16 bf16_neg(__nv_bfloat16 x) {
  return __ushort_as_bfloat16((unsigned short)(__bfloat16_as_ushort(x) ^ 0x8000u));
}
constexpr uint32_t BF16X2_SIGNS = 0x80008000u;

// Byte offset of element (row, k) of one (slice, plane) sub-tile inside a
// K-chunk stage: core matrices of 8 rows x 8 elements, K-adjacent at +128 B,
// row-group-adjacent at +256 B.
__device__ __forceinline__ uint32_t core_offset(int row, int k) {
  return (uint32_t)((row >> 3) * 256 + ((k >> 3) & 1) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Left operand: one M tile (128 stacked rows) of one operand instance.
// Row r of the stack is row (r % nev) of block blk[r / nev]; element k of it
// is blk[r/nev][(r%nev)*nev + k].  Output: [nchunk][SPLIT_A_STAGE] bytes and
// 128 row exponents.
__global__ void __launch_bounds__(256) slice_left_kernel(const SliceLeftJob* __restrict__ jobs, int nev,
                                                         int nchunk, int mtiles) {
  extern __shared__ __align__(128) uint8_t sm[];
  int* sexp = (int*)sm;
  uint8_t* stage = sm + 512;
  const SliceLeftJob& J = jobs[blockIdx.x / mtiles];
  const int mt = blockIdx.x % mtiles;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // row exponents
  for (int rr = warp; rr < SPLIT_M; rr += 8) {
    const int r = mt * SPLIT_M + rr;
    int e = -30000;
    if (r < J.rows) {
      const double2* row = J.blk[r / nev] + (size_t)(r % nev) * nev;
      for (int k = lane; k < nev; k += 32) {
        double2 v = row[k];
        e = max(e, max(f64_exp_bound(v.x), f64_exp_bound(v.y)));
      }
    }
    for (int o = 16; o; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if (lane == 0) {
      const int E = e < -1000 ? 0 : e;
      sexp[rr] = E;
      J.exps[mt * SPLIT_M + rr] = E;
    }
  }
  __syncthreads();
  uint8_t* dst_tile = J.out + (size_t)mt * nchunk * SPLIT_A_STAGE;
  constexpr int PER = SPLIT_M * SPLIT_K / 256;
  for (int kc = 0; kc < nchunk; kc++) {
    // 128 rows x 16 k: 16 consecutive threads read one row segment (coalesced);
    // a thread's 8 loads are issued before any of them is sliced
    double2 vv[PER];
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u;
      const int r = mt * SPLIT_M + (e >> 4), k = kc * SPLIT_K + (e & 15);
      vv[u] = (r < J.rows && k < nev) ? J.blk[r / nev][(size_t)(r % nev) * nev + k] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u;
      const int rr = e >> 4, kk = e & 15;
      const double2 v = vv[u];
      const int E = sexp[rr];
      bool nr, ni;
      const uint64_t Ur = round_fixed(f64_fixed(v.x, E, nr)), Ui = round_fixed(f64_fixed(v.y, E, ni));
      const uint32_t off = core_offset(rr, kk);
#pragma unroll
      for (int s = 0; s < SPLIT_NSLICE; s++) {
        *(__nv_bfloat16*)(stage + (s * 2 + 0) * SPLIT_A_SUB + off) = slice_bf16(Ur, s, nr);
        *(__nv_bfloat16*)(stage + (s * 2 + 1) * SPLIT_A_SUB + off) = slice_bf16(Ui, s, ni);
      }
    }
    __syncthreads();
    int4* d = (int4*)(dst_tile + (size_t)kc * SPLIT_A_STAGE);
    const int4* src = (const int4*)stage;
    for (int i = threadIdx.x; i < SPLIT_A_STAGE / 16; i += 256) d[i] = src[i];
    __syncthreads();
  }
}

// Right operand (stored N x K, K-major): one N tile of SPLIT_N stacked columns.
// Column n of the stack is column (n % nev) of block blk[n / nev]; its element
// k is blk[n/nev][k*nev + n%nev].  Exponent per column.
__global__ void __launch_bounds__(256) slice_right_kernel(const SliceRightJob* __restrict__ jobs, int nev,
                                                          int nchunk, int ntiles) {
  extern __shared__ __align__(128) uint8_t sm[];
  int* sexp = (int*)sm;
  uint8_t* stage = sm + 512;
  const SliceRightJob& J = jobs[blockIdx.x / ntiles];
  const int nt = blockIdx.x % ntiles;
  // column exponents: 4 threads per column (rows k = kq mod 4; consecutive
  // threads read consecutive columns), partial maxima combined in shared memory
  __shared__ int part[256];
  {
    const int nn = threadIdx.x % SPLIT_N, kq = threadIdx.x / SPLIT_N;
    const int n = nt * SPLIT_N + nn;
    int e = -30000;
    if (n < J.cols) {
      const double2* col = J.blk[n / nev] + (n % nev);
#pragma unroll 5
      for (int k = kq; k < nev; k += 4) {
        const double2 v = col[(size_t)k * nev];
        e = max(e, max(f64_exp_bound(v.x), f64_exp_bound(v.y)));
      }
    }
    part[threadIdx.x] = e;
  }
  __syncthreads();
  if (threadIdx.x < SPLIT_N) {
    const int* q = part + threadIdx.x;
    const int e = max(max(q[0], q[SPLIT_N]), max(q[2 * SPLIT_N], q[3 * SPLIT_N]));
    const int E = e < -1000 ? 0 : e;
    sexp[threadIdx.x] = E;
    J.exps[nt * SPLIT_N + threadIdx.x] = E;  // exps sized ntiles * SPLIT_N (padding columns get 0)
  }
  __syncthreads();
  uint8_t* dst_tile = J.out + (size_t)nt * nchunk * SPLIT_B_STAGE;
  constexpr int PER = SPLIT_N * SPLIT_K / 256;
  for (int kc = 0; kc < nchunk; kc++) {
    double2 vv[PER];
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u;
      const int n = nt * SPLIT_N + e % SPLIT_N, k = kc * SPLIT_K + e / SPLIT_N;
      vv[u] = (n < J.cols && k < nev) ? J.blk[n / nev][(size_t)k * nev + (n % nev)] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u;
      const int nn = e % SPLIT_N, kk = e / SPLIT_N;
      const double2 v = vv[u];
      const int E = sexp[nn];
      bool nr, ni;
      const uint64_t Ur = round_fixed(f64_fixed(v.x, E, nr)), Ui = round_fixed(f64_fixed(v.y, E, ni));
      const uint32_t off = core_offset(nn, kk);
#pragma unroll
      for (int s = 0; s < SPLIT_NSLICE; s++) {
        // planes -im, re, im (packed complex MMAs)
        const __nv_bfloat16 bi = slice_bf16(Ui, s, ni);
        *(__nv_bfloat16*)(stage + (s * 3 + 0) * SPLIT_B_SUB + off) = bf16_neg(bi);
        *(__nv_bfloat16*)(stage + (s * 3 + 1) * SPLIT_B_SUB + off) = slice_bf16(Ur, s, nr);
        *(__nv_bfloat16*)(stage + (s * 3 + 2) * SPLIT_B_SUB + off) = bi;
      }
    }
    __syncthreads();
    int4* d = (int4*)(dst_tile + (size_t)kc * SPLIT_B_STAGE);
    const int4* src = (const int4*)stage;
    for (int i = threadIdx.x; i < SPLIT_B_STAGE / 16; i += 256) d[i] = src[i];
    __syncthreads();
  }
}

// Staged forms of slice_left / slice_right (same output bytes): one CTA per
// 32-row (left) or 32-column (right) quarter of an operand tile copies its
// quarter of the FP64 operand into shared memory once (cp.async, all loads in
// flight together), takes the scale exponents from there and slices every K
// chunk from there, so the operand is read from memory once.  A quarter covers
// 4 of the core-matrix row groups of each (slice, plane) sub-tile, i.e. 1 KB
// contiguous in each.  DIRECT = false stages each K chunk's output in shared
// memory and copies it out in 16-byte pieces; DIRECT = true stores every
// thread's packed BF16 pairs straight to memory (a warp's store covers whole
// 32-byte sectors: 4 rows x 16 contiguous bytes at two 128-byte-apart runs)
// and needs no barrier after the exponents.
constexpr int SLQ = 32;  // rows / columns of a quarter

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// shared memory of the staged slicers: the quarter (SLQ x nev complex), the
// staged output chunk (planes x 1 KB) and the exponents
inline size_t slice_staged_smem(int nev, int planes) { return (size_t)SLQ * nev * 16 + (size_t)planes * 1024 + 256; }

template <bool DIRECT>
__global__ void __launch_bounds__(256) slice_left_staged_kernel(const SliceLeftJob* __restrict__ jobs, int nev,
                                                                int nchunk, int mtiles) {
  extern __shared__ __align__(128) uint8_t sm[];
  double2* data = (double2*)sm;  // [SLQ][nev]
  uint8_t* stage = sm + (size_t)SLQ * nev * 16;
  int* sexp = (int*)(stage + (DIRECT ? 0 : SPLIT_NSLICE * 2 * 1024));
  const int quarters = SPLIT_M / SLQ;
  const int job = blockIdx.x / (mtiles * quarters), rem = blockIdx.x - job * mtiles * quarters;
  const int mt = rem / quarters, qt = rem - mt * quarters;
  const SliceLeftJob& J = jobs[job];
  const int r0 = mt * SPLIT_M + qt * SLQ;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // rows r0 .. r0 + SLQ - 1 (each row contiguous in its block); padding rows are zero
  for (int e = threadIdx.x; e < SLQ * nev; e += 256) {
    const int rr = e / nev, k = e - rr * nev, r = r0 + rr;
    if (r < J.rows)
      cp_async16(data + e, J.blk[r / nev] + (size_t)(r % nev) * nev + k);
    else
      data[e] = make_double2(0.0, 0.0);
  }
  cp_async_wait_all();
  __syncthreads();
  // row exponents
  for (int rr = warp; rr < SLQ; rr += 8) {
    int e = -30000;
    if (r0 + rr < J.rows)
      for (int k = lane; k < nev; k += 32) {
        const double2 v = data[rr * nev + k];
        e = max(e, max(f64_exp_bound(v.x), f64_exp_bound(v.y)));
      }
    for (int o = 16; o; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
    if (lane == 0) {
      const int E = e < -1000 ? 0 : e;
      sexp[rr] = E;
      J.exps[r0 + rr] = E;
    }
  }
  __syncthreads();
  uint8_t* dst_tile = J.out + (size_t)mt * nchunk * SPLIT_A_STAGE + qt * 1024;
  static_assert(SLQ * SPLIT_K == 2 * 256, "two adjacent k per thread");
  const int rr = threadIdx.x >> 3, kk = (threadIdx.x & 7) * 2;
  const uint32_t off = core_offset(rr, kk);  // k and k + 1 are adjacent
  const int E = sexp[rr];
  for (int kc = 0; kc < nchunk; kc++) {
    const int k = kc * SPLIT_K + kk;
    const double2 v0 = k < nev ? data[rr * nev + k] : make_double2(0.0, 0.0);
    const double2 v1 = k + 1 < nev ? data[rr * nev + k + 1] : make_double2(0.0, 0.0);
    bool nr0, ni0, nr1, ni1;
    const uint64_t Ur0 = round_fixed(f64_fixed(v0.x, E, nr0)), Ui0 = round_fixed(f64_fixed(v0.y, E, ni0));
    const uint64_t Ur1 = round_fixed(f64_fixed(v1.x, E, nr1)), Ui1 = round_fixed(f64_fixed(v1.y, E, ni1));
    if constexpr (DIRECT) {
      uint8_t* d = dst_tile + (size_t)kc * SPLIT_A_STAGE + off;
#pragma unroll
      for (int sl = 0; sl < SPLIT_NSLICE; sl++) {
        *(uint32_t*)(d + (size_t)(sl * 2 + 0) * SPLIT_A_SUB) = slice_pair(Ur0, nr0, Ur1, nr1, sl);
        *(uint32_t*)(d + (size_t)(sl * 2 + 1) * SPLIT_A_SUB) = slice_pair(Ui0, ni0, Ui1, ni1, sl);
      }
    } else {
#pragma unroll
      for (int sl = 0; sl < SPLIT_NSLICE; sl++) {
        *(uint32_t*)(stage + (sl * 2 + 0) * 1024 + off) = slice_pair(Ur0, nr0, Ur1, nr1, sl);
        *(uint32_t*)(stage + (sl * 2 + 1) * 1024 + off) = slice_pair(Ui0, ni0, Ui1, ni1, sl);
      }
      __syncthreads();
      uint8_t* d = dst_tile + (size_t)kc * SPLIT_A_STAGE;
      for (int i = threadIdx.x; i < SPLIT_NSLICE * 2 * 64; i += 256) {
        const int piece = i >> 6, w = i & 63;
        ((int4*)(d + (size_t)piece * SPLIT_A_SUB))[w] = ((const int4*)(stage + piece * 1024))[w];
      }
      __syncthreads();
    }
  }
}

template <bool DIRECT>
__global__ void __launch_bounds__(256) slice_right_staged_kernel(const SliceRightJob* __restrict__ jobs, int nev,
                                                                 int nchunk, int ntiles) {
  extern __shared__ __align__(128) uint8_t sm[];
  double2* data = (double2*)sm;  // [nev][SLQ]
  uint8_t* stage = sm + (size_t)SLQ * nev * 16;
  int* sexp = (int*)(stage + (DIRECT ? 0 : SPLIT_NSLICE * 3 * 1024));
  __shared__ int part[256];
  const int quarters = SPLIT_N / SLQ;
  const int job = blockIdx.x / (ntiles * quarters), rem = blockIdx.x - job * ntiles * quarters;
  const int nt = rem / quarters, qt = rem - nt * quarters;
  const SliceRightJob& J = jobs[job];
  const int n0 = nt * SPLIT_N + qt * SLQ;
  // columns n0 .. n0 + SLQ - 1: a warp reads one row k of them; padding columns are zero
  {
    const int c = threadIdx.x & 31, n = n0 + c;
    const double2* colp = n < J.cols ? J.blk[n / nev] + (n % nev) : nullptr;
    for (int k = threadIdx.x >> 5; k < nev; k += 8) {
      if (colp)
        cp_async16(data + k * SLQ + c, colp + (size_t)k * nev);
      else
        data[k * SLQ + c] = make_double2(0.0, 0.0);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // column exponents: 8 threads per column, partial maxima combined in shared memory
  {
    const int c = threadIdx.x & 31, kq = threadIdx.x >> 5;
    int e = -30000;
    if (n0 + c < J.cols)
      for (int k = kq; k < nev; k += 8) {
        const double2 v = data[k * SLQ + c];
        e = max(e, max(f64_exp_bound(v.x), f64_exp_bound(v.y)));
      }
    part[threadIdx.x] = e;
  }
  __syncthreads();
  if (threadIdx.x < SLQ) {
    int e = part[threadIdx.x];
    for (int w = 1; w < 8; w++) e = max(e, part[w * 32 + threadIdx.x]);
    const int E = e < -1000 ? 0 : e;
    sexp[threadIdx.x] = E;
    J.exps[n0 + threadIdx.x] = E;
  }
  __syncthreads();
  uint8_t* dst_tile = J.out + (size_t)nt * nchunk * SPLIT_B_STAGE + qt * 1024;
  static_assert(SLQ * SPLIT_K == 2 * 256, "two adjacent k per thread");
  // 8 consecutive lanes: 8 columns of one k pair (128 contiguous bytes of the
  // quarter, and 8 core-matrix rows); a warp: 8 columns x 4 k pairs, whose
  // packed pairs fill 128 contiguous output bytes
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nn = (warp & 3) * 8 + (lane & 7), kk = ((warp >> 2) * 4 + (lane >> 3)) * 2;
  const uint32_t off = core_offset(nn, kk);  // k and k + 1 are adjacent
  const int E = sexp[nn];
  for (int kc = 0; kc < nchunk; kc++) {
    const int k = kc * SPLIT_K + kk;
    const double2 v0 = k < nev ? data[k * SLQ + nn] : make_double2(0.0, 0.0);
    const double2 v1 = k + 1 < nev ? data[(k + 1) * SLQ + nn] : make_double2(0.0, 0.0);
    bool nr0, ni0, nr1, ni1;
    const uint64_t Ur0 = round_fixed(f64_fixed(v0.x, E, nr0)), Ui0 = round_fixed(f64_fixed(v0.y, E, ni0));
    const uint64_t Ur1 = round_fixed(f64_fixed(v1.x, E, nr1)), Ui1 = round_fixed(f64_fixed(v1.y, E, ni1));
    if constexpr (DIRECT) {
      uint8_t* d = dst_tile + (size_t)kc * SPLIT_B_STAGE + off;
#pragma unroll
      for (int sl = 0; sl < SPLIT_NSLICE; sl++) {
        const uint32_t pi = slice_pair(Ui0, ni0, Ui1, ni1, sl);
        *(uint32_t*)(d + (size_t)(sl * 3 + 0) * SPLIT_B_SUB) = pi ^ BF16X2_SIGNS;
        *(uint32_t*)(d + (size_t)(sl * 3 + 1) * SPLIT_B_SUB) = slice_pair(Ur0, nr0, Ur1, nr1, sl);
        *(uint32_t*)(d + (size_t)(sl * 3 + 2) * SPLIT_B_SUB) = pi;
      }
    } else {
#pragma unroll
      for (int sl = 0; sl < SPLIT_NSLICE; sl++) {
        // planes -im, re, im (packed complex MMAs)
        const uint32_t pi = slice_pair(Ui0, ni0, Ui1, ni1, sl);
        *(uint32_t*)(stage + (sl * 3 + 0) * 1024 + off) = pi ^ BF16X2_SIGNS;
        *(uint32_t*)(stage + (sl * 3 + 1) * 1024 + off) = slice_pair(Ur0, nr0, Ur1, nr1, sl);
        *(uint32_t*)(stage + (sl * 3 + 2) * 1024 + off) = pi;
      }
      __syncthreads();
      uint8_t* d = dst_tile + (size_t)kc * SPLIT_B_STAGE;
      for (int i = threadIdx.x; i < SPLIT_NSLICE * 3 * 64; i += 256) {
        const int piece = i >> 6, w = i & 63;
        ((int4*)(d + (size_t)piece * SPLIT_B_SUB))[w] = ((const int4*)(stage + piece * 1024))[w];
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------ task-form slicers
// Element (r, k) of a left task operand before its term's weight and
// conjugation, which the slicers apply as exponent and sign (the weights are
// real powers of two).
__device__ __forceinline__ double2 task_left_raw(const SliceTaskLJob& J, int nev, int r, int k) {
  const int q = k / nev, j = k - q * nev;
  if (r >= nev || q >= J.nterm) return make_double2(0.0, 0.0);
  return ((J.dag >> q) & 1) ? J.a[q][(size_t)j * nev + r] : J.a[q][(size_t)r * nev + j];
}

// Fixed-point magnitudes and signs of w_q op(x) for term q, with w_q = +-2^wexp_q
// and op the identity or the complex conjugate (dag): integer operations only.
__device__ __forceinline__ void weighted_fixed(double2 x, int wexp, bool wneg, bool dag, int E, uint64_t& Ur,
                                               bool& nr, uint64_t& Ui, bool& ni) {
  Ur = f64_fixed_pow2(x.x, wexp, wneg, E, nr);
  Ui = f64_fixed_pow2(x.y, wexp, wneg != dag, E, ni);
}

// Element (k, n) of a right task operand before its conjugation (applied as a
// sign by the slicer).
__device__ __forceinline__ double2 task_right_raw(const SliceTaskRJob& J, int nev, int k, int n) {
  const int q = k / nev, i = k - q * nev, jb = n / nev, c = n - jb * nev;
  if (q >= J.nterm || jb >= J.nb) return make_double2(0.0, 0.0);
  const double2* B = J.b[jb][q];
  return ((J.dag >> (4 * jb + q)) & 1) ? B[(size_t)c * nev + i] : B[(size_t)i * nev + c];
}

// Task-form slicing runs in two launches: the exponent bounds of every distinct
// block of the launch (one read of each block), then one CTA per (operand tile,
// K chunk), which combines the bounds of its operand's blocks into the row or
// column scale exponents, so that a stage with few operands still spreads over
// every SM.
//
// Block exponents: CTA b scans block blk[b] (nev x nev, row-major) once;
// bexp[b][0][r] = max_c bound(row r), bexp[b][1][c] = max_r bound(column c).
__global__ void __launch_bounds__(256) block_exp_kernel(const double2* const* __restrict__ blk, int nev,
                                                        int* __restrict__ bexp) {
  // warp w scans rows w, w + 8, ...: the row bound by a shuffle reduction, and
  // lane l keeps the bound of columns l, l + 32, ... over its warp's rows
  // (nev <= SPLIT_MAXK = 128, so 4 columns a lane); the warps' column bounds
  // are combined in shared memory at the end
  __shared__ int cpart[8][SPLIT_MAXK];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double2* B = blk[blockIdx.x];
  int* o = bexp + (size_t)blockIdx.x * 2 * nev;
  int cm[SPLIT_MAXK / 32];
#pragma unroll
  for (int u = 0; u < SPLIT_MAXK / 32; u++) cm[u] = -30000;
#pragma unroll 2
  for (int r = warp; r < nev; r += 8) {
    const double2* row = B + (size_t)r * nev;
    double2 v[SPLIT_MAXK / 32];
#pragma unroll
    for (int u = 0; u < SPLIT_MAXK / 32; u++) {
      const int c = lane + 32 * u;
      v[u] = c < nev ? row[c] : make_double2(0.0, 0.0);
    }
    int rm = -30000;
#pragma unroll
    for (int u = 0; u < SPLIT_MAXK / 32; u++) {
      if (lane + 32 * u >= nev) continue;
      const int x = max(f64_exp_bound(v[u].x), f64_exp_bound(v[u].y));
      rm = max(rm, x);
      cm[u] = max(cm[u], x);
    }
    for (int off = 16; off; off >>= 1) rm = max(rm, __shfl_xor_sync(0xffffffffu, rm, off));
    if (lane == 0) o[r] = rm;
  }
#pragma unroll
  for (int u = 0; u < SPLIT_MAXK / 32; u++) cpart[warp][lane + 32 * u] = cm[u];
  __syncthreads();
  for (int c = threadIdx.x; c < nev; c += 256) {
    int m = cpart[0][c];
    for (int w = 1; w < 8; w++) m = max(m, cpart[w][c]);
    o[nev + c] = m;
  }
}

// Left operand slices: CTA = (job, K chunk); 128 rows x 16 k, 8 elements a thread.
template <class C>
__global__ void __launch_bounds__(256) slice_task_left_kernel(const SliceTaskLJob* __restrict__ jobs, int nev,
                                                              int nchunk, const int* __restrict__ bexp) {
  extern __shared__ __align__(128) uint8_t sm[];
  int* sexp = (int*)sm;
  uint8_t* stage = sm + 512;
  const SliceTaskLJob& J = jobs[blockIdx.x / nchunk];
  const int kc = blockIdx.x % nchunk;
  const int K = J.nterm * nev;
  if (threadIdx.x < SPLIT_M) {
    // row r over all K: the row (column, for a conjugate-transposed term) bounds of
    // the terms' blocks, shifted by the weights' exponents
    const int r = threadIdx.x;
    int e = -30000;
    if (r < nev)
      for (int q = 0; q < J.nterm; q++) {
        const int b = bexp[((size_t)J.bi[q] * 2 + ((J.dag >> q) & 1)) * nev + r];
        if (b > -30000) e = max(e, b + J.wexp[q]);
      }
    const int E = (e < -1000 ? 0 : e) + J.eplus;
    sexp[r] = E;
    if (kc == 0) J.exps[r] = E;
  }
  // 16 consecutive threads along k: shared-memory stores without bank conflicts
  constexpr int PER = SPLIT_M * SPLIT_K / 256;
  double2 v[PER];
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 256;
    const int rr = e >> 4, k = kc * SPLIT_K + (e & 15);
    v[u] = k < K ? task_left_raw(J, nev, rr, k) : make_double2(0.0, 0.0);
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 256;
    const int rr = e >> 4, kk = e & 15;
    const int q = min((kc * SPLIT_K + kk) / nev, J.nterm - 1);
    const int E = sexp[rr];
    bool nr, ni;
    uint64_t Ur, Ui;
    weighted_fixed(v[u], J.wexp[q], J.w[q] < 0.f, (J.dag >> q) & 1, E, Ur, nr, Ui, ni);
    Ur = round_fixed<C::NS>(Ur);
    Ui = round_fixed<C::NS>(Ui);
    const uint32_t off = core_offset(rr, kk);
#pragma unroll
    for (int s = 0; s < C::NS; s++) {
      *(__nv_bfloat16*)(stage + (s * 2 + 0) * C::A_SUB + off) = slice_bf16(Ur, s, nr);
      *(__nv_bfloat16*)(stage + (s * 2 + 1) * C::A_SUB + off) = slice_bf16(Ui, s, ni);
    }
  }
  __syncthreads();
  int4* d = (int4*)(J.out + (size_t)kc * C::A_STAGE);
  const int4* src = (const int4*)stage;
  for (int i = threadIdx.x; i < C::A_STAGE / 16; i += 256) d[i] = src[i];
}

// Stacked left operand slices: CTA = (job, M tile, K chunk).  Row g of the stack
// is row g % nev of slab g / nev; 128 rows x 16 k.  A thread slices 4 pairs of
// adjacent k and stores each slice's pair as one packed BF16 word straight to
// the tiled operand: a warp covers 4 rows x 8 pairs, i.e. whole 32-byte
// sectors (two rows' 16-byte runs) of the core matrices.
template <class C>
__global__ void __launch_bounds__(256) slice_stack_left_kernel(const SliceStackLJob* __restrict__ jobs, int nev,
                                                               int nchunk, int mtiles, const int* __restrict__ bexp) {
  __shared__ int sexp[SPLIT_M];
  const int kc = blockIdx.x % nchunk, t = blockIdx.x / nchunk;
  const SliceStackLJob& J = jobs[t / mtiles];
  const int mt = t % mtiles;
  const int K = J.nterm * nev, rows = J.nslab * nev;
  if (threadIdx.x < SPLIT_M) {
    const int g = mt * SPLIT_M + threadIdx.x;
    int e = -30000;
    if (g < rows) {
      const int sl = g / nev, r = g - sl * nev;
      for (int q = 0; q < J.nterm; q++) {
        const int b = bexp[((size_t)J.bi[sl][q] * 2 + ((J.dag >> q) & 1)) * nev + r];
        if (b > -30000) e = max(e, b + J.wexp[q]);
      }
    }
    const int E = (e < -1000 ? 0 : e) + J.eplus;
    sexp[threadIdx.x] = E;
    if (kc == 0) J.exps[g] = E;
  }
  constexpr int PER = SPLIT_M * SPLIT_K / 2 / 256;
  double2 v[PER][2];
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 256;
    const int rr = e >> 3, g = mt * SPLIT_M + rr;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int k = kc * SPLIT_K + 2 * (e & 7) + h;
      v[u][h] = make_double2(0.0, 0.0);
      if (k < K && g < rows) {
        const int sl = g / nev, r = g - sl * nev, q = k / nev, j = k - q * nev;
        v[u][h] = ((J.dag >> q) & 1) ? J.a[sl][q][(size_t)j * nev + r] : J.a[sl][q][(size_t)r * nev + j];
      }
    }
  }
  __syncthreads();
  uint8_t* d0 = J.out + ((size_t)mt * nchunk + kc) * C::A_STAGE;
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 256;
    const int rr = e >> 3, kp = e & 7;
    const int E = sexp[rr];
    uint64_t Ur[2], Ui[2];
    bool nr[2], ni[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int q = min((kc * SPLIT_K + 2 * kp + h) / nev, J.nterm - 1);
      weighted_fixed(v[u][h], J.wexp[q], J.w[q] < 0.f, (J.dag >> q) & 1, E, Ur[h], nr[h], Ui[h], ni[h]);
      Ur[h] = round_fixed<C::NS>(Ur[h]);
      Ui[h] = round_fixed<C::NS>(Ui[h]);
    }
    uint8_t* d = d0 + core_offset(rr, 2 * kp);
#pragma unroll
    for (int s = 0; s < C::NS; s++) {
      *(uint32_t*)(d + (s * 2 + 0) * C::A_SUB) = slice_pair(Ur[0], nr[0], Ur[1], nr[1], s);
      *(uint32_t*)(d + (s * 2 + 1) * C::A_SUB) = slice_pair(Ui[0], ni[0], Ui[1], ni[1], s);
    }
  }
}

// Right operand slices: CTA = (job, N tile, K chunk); BN columns x 16 k.  A
// thread slices pairs of adjacent k of one column and stores each slice's pair
// as one packed BF16 word per plane straight to the tiled operand: a warp
// covers 4 adjacent columns x 8 pairs, i.e. whole 32-byte sectors (two
// columns' 16-byte runs) of the core matrices.
template <class C>
__global__ void __launch_bounds__(128) slice_task_right_kernel(const SliceTaskRJob* __restrict__ jobs, int nev,
                                                               int nchunk, int ntiles, const int* __restrict__ bexp) {
  __shared__ int sexp[C::BN];
  const int kc = blockIdx.x % nchunk, t = blockIdx.x / nchunk;
  const SliceTaskRJob& J = jobs[t / ntiles];
  const int nt = t % ntiles;
  const int K = J.nterm * nev, ncols = J.nb * nev;
  if (threadIdx.x < C::BN) {
    // column n = (block jb, column c) over all K: the column (row, for a
    // conjugate-transposed term) bounds of block jb's terms
    const int n = nt * C::BN + threadIdx.x;
    int e = -30000;
    if (n < ncols) {
      const int jb = n / nev, c = n - jb * nev;
      for (int q = 0; q < J.nterm; q++) {
        const int dag = (J.dag >> (4 * jb + q)) & 1;
        e = max(e, bexp[((size_t)J.bi[jb][q] * 2 + (dag ? 0 : 1)) * nev + c]);
      }
    }
    const int E = (e < -1000 ? 0 : e) + J.eplus;
    sexp[threadIdx.x] = E;
    if (kc == 0) J.exps[n] = E;  // exps sized ntiles * BN (padding columns get 0)
  }
  constexpr int PER = C::BN * SPLIT_K / 2 / 128;
  static_assert(C::BN * SPLIT_K / 2 % 128 == 0, "column pairs a thread");
  double2 v[PER][2];
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 128;
    const int n = nt * C::BN + (e >> 3);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int k = kc * SPLIT_K + 2 * (e & 7) + h;
      v[u][h] = (n < ncols && k < K) ? task_right_raw(J, nev, k, n) : make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  uint8_t* d0 = J.out + ((size_t)nt * nchunk + kc) * C::B_STAGE;
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int e = threadIdx.x + u * 128;
    const int nn = e >> 3, kp = e & 7, n = nt * C::BN + nn;
    const int jb = min(n / nev, J.nb - 1);
    const int E = sexp[nn];
    uint64_t Ur[2], Ui[2];
    bool nr[2], ni[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int q = min((kc * SPLIT_K + 2 * kp + h) / nev, J.nterm - 1);
      weighted_fixed(v[u][h], 0, false, (J.dag >> (4 * jb + q)) & 1, E, Ur[h], nr[h], Ui[h], ni[h]);
      Ur[h] = round_fixed<C::NS>(Ur[h]);
      Ui[h] = round_fixed<C::NS>(Ui[h]);
    }
    uint8_t* d = d0 + core_offset(nn, 2 * kp);
#pragma unroll
    for (int s = 0; s < C::NS; s++) {
      const uint32_t re = slice_pair(Ur[0], nr[0], Ur[1], nr[1], s), im = slice_pair(Ui[0], ni[0], Ui[1], ni[1], s);
      if (C::PACK) {
        *(uint32_t*)(d + (s * 3 + 0) * C::B_SUB) = im ^ BF16X2_SIGNS;
        *(uint32_t*)(d + (s * 3 + 1) * C::B_SUB) = re;
        *(uint32_t*)(d + (s * 3 + 2) * C::B_SUB) = im;
      } else {
        *(uint32_t*)(d + (s * 2 + 0) * C::B_SUB) = re;
        *(uint32_t*)(d + (s * 2 + 1) * C::B_SUB) = im;
      }
    }
  }
}

// ------------------------------------------------------------------ GEMM
// Persistent kernel: each CTA walks output tiles t = blockIdx.x, +gridDim.x, ...
// of 128 x SPLIT_N.  Warp 0: TMEM allocation and the bulk-copy producer, which
// runs ahead across tile boundaries through an NSTAGE ring; warp 1: MMA issue;
// warps 2 .. 2 + EPI_WARPS - 1: epilogue (TMEM lanes 32*(warp%4) .. +31).  The
// MMA warp and the epilogue hand the TMEM accumulators back and forth with two
// mbarriers (tmem_full after the last MMA of a tile, tmem_empty once the
// epilogue holds them in registers, before its global stores).
// Threads of a GEMM CTA: producer and MMA warps plus C::EPI_WARPS epilogue warps.
template <class C>
constexpr int gemm_threads() { return 64 + 32 * C::EPI_WARPS; }
constexpr int NSTAGE = 3;
constexpr uint32_t TMEM_COLS = 512;  // (re, im) x NL levels x BN columns fit in 512 for both configurations
constexpr uint64_t WAIT_NS = 2000000000ull;  // 2 s per wait

constexpr int GEMM_SMEM_TAIL = 1024;  // barriers, TMEM slot, column exponents and output pointers

template <class C>
constexpr size_t gemm_smem_bytes() {
  return (size_t)NSTAGE * (C::A_STAGE + C::B_STAGE) + GEMM_SMEM_TAIL;
}
static_assert(2 * CfgStd::NL * CfgStd::BN <= (int)TMEM_COLS && 2 * CfgHP::NL * CfgHP::BN <= (int)TMEM_COLS,
              "accumulators exceed TMEM");

// I * 2^e as a double, rounded to nearest even; integer operations only
// (normal results; magnitudes below 2^-1022 flush to zero).
__device__ __forceinline__ double i2d_scaled(long long I, int e) {
  if (I == 0) return 0.0;
  const unsigned long long sgn = I < 0 ? (1ull << 63) : 0ull;
  unsigned long long u = I < 0 ? 0ull - (unsigned long long)I : (unsigned long long)I;
  const int lz = __clzll((long long)u);
  u <<= lz;
  unsigned long long mant = u >> 11;
  const unsigned long long rem = u & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) mant++;
  int ex = 63 - lz + e;
  if (mant >> 53) {
    mant >>= 1;
    ex++;
  }
  const int biased = ex + 1023;
  if (biased <= 0) return 0.0;
  if (biased >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)biased << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// Smallest row + column scale exponent of a float-float product (below it the
// FP32 words of the products' traces would leave the normal range).
constexpr int FF_MIN_EXP = -100;

__device__ __forceinline__ float pow2f(int e) {
  e = max(-126, min(127, e));
  return __int_as_float((127 + e) << 23);
}

__device__ __forceinline__ double pow2d(int e) {
  e = max(-1022, min(1023, e));
  return __longlong_as_double((long long)(1023 + e) << 52);
}

template <int NTHR>
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(NTHR) : "memory"); }

// TMEM hand-back groups: the epilogue drains the level accumulators in groups,
// levels {0, 1} first, then each further level on its own, and hands every
// group back as soon as it holds it in registers.  The first K chunk of the
// next tile issues its MMAs group by group, each after that group's hand-back,
// so the MMAs of the early levels run while later levels are still drained.
template <class C>
constexpr int tmem_groups() { return C::NL - 1; }
__host__ __device__ constexpr int level_group(int l) { return l <= 1 ? 0 : l - 1; }

// The MMAs of one slice pair (i, j) of one K chunk into its level accumulator.
// adesc / bdesc describe sub-tile (slice 0, re) of the stage; the other
// sub-tiles are constant byte offsets (added as offset >> 4 to the
// start-address field, which cannot carry: shared addresses are < 2^18).
template <class C, int I, int J>
__device__ __forceinline__ void issue_pair(uint32_t tbase, uint64_t adesc, uint64_t bdesc, bool first_chunk) {
  constexpr uint32_t id_pos = idesc_bf16_f32(SPLIT_M, C::BN, false);
  constexpr uint32_t id_neg = idesc_bf16_f32(SPLIT_M, C::BN, true);
  constexpr uint32_t id_wide = idesc_bf16_f32(SPLIT_M, 2 * C::BN, false);
  constexpr int lvl = (I + J) < C::NL - 1 ? (I + J) : C::NL - 1;
  // in i-major order the first pair of level l is (0, l)
  const uint32_t accum = (!first_chunk || !(I == 0 && J <= C::NL - 1)) ? 1u : 0u;
  const uint64_t ar = adesc + (uint64_t)(((I * 2 + 0) * C::A_SUB) >> 4);
  const uint64_t ai = adesc + (uint64_t)(((I * 2 + 1) * C::A_SUB) >> 4);
  if constexpr (C::PACK) {
    // planes -Yi, Yr, Yi of slice j are adjacent along N (row groups 256 B apart)
    const uint64_t b_nr = bdesc + (uint64_t)(((J * 3 + 0) * C::B_SUB) >> 4);  // [-Yi | Yr]
    const uint64_t b_ri = bdesc + (uint64_t)(((J * 3 + 1) * C::B_SUB) >> 4);  // [Yr | Yi]
    const uint32_t d = tbase + (uint32_t)C::acc_col(0, lvl);
    umma_f16(d, ar, b_ri, id_wide, accum);  // [Re | Im] += Xr [Yr | Yi]
    umma_f16(d, ai, b_nr, id_wide, 1u);     // [Re | Im] += Xi [-Yi | Yr]
  } else {
    const uint64_t br = bdesc + (uint64_t)(((J * 2 + 0) * C::B_SUB) >> 4);
    const uint64_t bi = bdesc + (uint64_t)(((J * 2 + 1) * C::B_SUB) >> 4);
    const uint32_t dre = tbase + (uint32_t)C::acc_col(0, lvl);
    const uint32_t dim = tbase + (uint32_t)C::acc_col(1, lvl);
    umma_f16(dre, ar, br, id_pos, accum);  // Re += Xr Yr
    umma_f16(dre, ai, bi, id_neg, 1u);     // Re -= Xi Yi
    umma_f16(dim, ar, bi, id_pos, accum);  // Im += Xr Yi
    umma_f16(dim, ai, br, id_pos, 1u);     // Im += Xi Yr
  }
}

// The slice pairs (i, j), i + j < NS, whose level falls in hand-back group G
// (G < 0: all pairs), in i-major order.  Every level accumulator sees its
// pairs in the same order whatever the grouping, so the FP32 last level sums
// them in the same order and the results do not depend on it.
template <class C, int G, int I = 0, int J = 0>
__device__ __forceinline__ void issue_pairs(uint32_t tbase, uint64_t adesc, uint64_t bdesc, bool first_chunk) {
  if constexpr (I < C::NS) {
    if constexpr (I + J < C::NS) {
      constexpr int lvl = (I + J) < C::NL - 1 ? (I + J) : C::NL - 1;
      if constexpr (G < 0 || level_group(lvl) == G) issue_pair<C, I, J>(tbase, adesc, bdesc, first_chunk);
      issue_pairs<C, G, I, J + 1>(tbase, adesc, bdesc, first_chunk);
    } else {
      issue_pairs<C, G, I + 1, 0>(tbase, adesc, bdesc, first_chunk);
    }
  }
}

// All MMAs of one K chunk: NS(NS+1)/2 slice pairs (i + j < NS) into the NL
// level accumulators.
template <class C>
__device__ __forceinline__ void issue_chunk(uint32_t tbase, uint64_t adesc, uint64_t bdesc, bool first_chunk) {
  issue_pairs<C, -1>(tbase, adesc, bdesc, first_chunk);
}

// The MMAs of hand-back group g (runtime index) of one K chunk.
template <class C>
__device__ __forceinline__ void issue_group(int g, uint32_t tbase, uint64_t adesc, uint64_t bdesc, bool first_chunk) {
  static_assert(tmem_groups<C>() >= 2 && tmem_groups<C>() <= 4, "hand-back groups");
  if (g == 0)
    issue_pairs<C, 0>(tbase, adesc, bdesc, first_chunk);
  else if (g == 1)
    issue_pairs<C, 1>(tbase, adesc, bdesc, first_chunk);
  else if (g == 2)
    issue_pairs<C, 2>(tbase, adesc, bdesc, first_chunk);
  else if constexpr (tmem_groups<C>() > 3)
    issue_pairs<C, 3>(tbase, adesc, bdesc, first_chunk);
}

// NC consecutive TMEM columns of this warp's 32 lanes into v (NC = 16, 12, 8 or 4).
template <int NC>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float* v) {
  static_assert(NC % 4 == 0 && NC <= 16, "TMEM load width");
  if constexpr (NC == 16) {
    tmem_ld16(taddr, v);
  } else if constexpr (NC >= 8) {
    tmem_ld8(taddr, v);
    if constexpr (NC > 8) tmem_ld_cols<NC - 8>(taddr + 8, v + 8);
  } else {
    tmem_ld4(taddr, v);
    if constexpr (NC > 4) tmem_ld_cols<NC - 4>(taddr + 4, v + 4);
  }
}

// Output tile -> (instance, M tile, N tile).  order 0 walks the N tiles of one
// M tile first (consecutive CTAs share the left operand tile), order 1 the M
// tiles of one N tile first (they share the right operand tile).
__device__ __forceinline__ void tile_coords(const SplitGemmBatch& g, int tile, int& inst, int& mt, int& nt) {
  const int per_inst = g.mtiles * g.ntiles;
  inst = tile / per_inst;
  const int r = tile - inst * per_inst;
  if (g.order == 0) {
    mt = r / g.ntiles;
    nt = r - mt * g.ntiles;
  } else {
    nt = r / g.mtiles;
    mt = r - nt * g.mtiles;
  }
}

template <class C>
__global__ void __launch_bounds__(gemm_threads<C>(), 1)
    split_gemm_kernel(SplitGemmBatch g, int ntiles_total, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + NSTAGE * C::A_STAGE;
  uint64_t* full = (uint64_t*)(smem + NSTAGE * (C::A_STAGE + C::B_STAGE));
  uint64_t* empty = full + NSTAGE;
  uint64_t* tfull = empty + NSTAGE;
  uint64_t* tempty = tfull + 1;  // one per hand-back group
  uint64_t* drainb = tempty + tmem_groups<C>();
  uint32_t* tslot = (uint32_t*)(drainb + 1);
  int* sexp = (int*)(tslot + 4);  // C::BN column exponents of the current tile
  // complex128 output: destination of row 0 of each column of the current tile
  double2** colp = (double2**)(smem + NSTAGE * (C::A_STAGE + C::B_STAGE) + 512);
  static_assert(512 + 8 * C::BN <= GEMM_SMEM_TAIL && 16 * 8 + 16 + 4 * C::BN <= 512, "GEMM shared-memory tail");

  volatile int* status = (volatile int*)(tslot + 1);  // block-uniform decisions
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    for (int g = 0; g < tmem_groups<C>(); g++) mbar_init(&tempty[g], C::EPI_WARPS);  // one arrival per epilogue warp
    mbar_init(drainb, 1);
    fence_mbar_init();
    // A CTA that starts after another one recorded a failure does nothing.
    status[0] = *(volatile int*)err;
  }
  __syncthreads();
  if (status[0]) return;  // uniform: every thread read the same shared value
  if (warp == 0) {
    tmem_alloc(tslot, TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t g_chunk = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles_total && ok; tile += gridDim.x) {
        int inst, mt, nt;
        tile_coords(g, tile, inst, mt, nt);
        const SplitGemmInst* I = &g.inst[inst];
        const uint8_t* gA = I->left + (size_t)mt * g.nchunk * C::A_STAGE;
        const uint8_t* gB = I->right + (size_t)nt * g.nchunk * C::B_STAGE;
        for (int kc = 0; kc < g.nchunk; kc++, g_chunk++) {
          const int s = g_chunk % NSTAGE;
          if (g_chunk >= NSTAGE && !mbar_wait(&empty[s], ((g_chunk / NSTAGE) - 1) & 1, WAIT_NS, err)) {
            atomicExch(err, 1);
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], C::A_STAGE + C::B_STAGE);
          bulk_g2s(sA + s * C::A_STAGE, gA + (size_t)kc * C::A_STAGE, C::A_STAGE, &full[s]);
          bulk_g2s(sB + s * C::B_STAGE, gB + (size_t)kc * C::B_STAGE, C::B_STAGE, &full[s]);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t g_chunk = 0, local = 0;
      bool ok = true;
      const uint64_t adesc0 = sdesc_kmajor_noswz(smem_u32(sA), 128, 256);
      const uint64_t bdesc0 = sdesc_kmajor_noswz(smem_u32(sB), 128, 256);
      for (int tile = blockIdx.x; tile < ntiles_total && ok; tile += gridDim.x, local++) {
        for (int kc = 0; kc < g.nchunk; kc++, g_chunk++) {
          const int s = g_chunk % NSTAGE;
          if (!mbar_wait(&full[s], (g_chunk / NSTAGE) & 1, WAIT_NS, err)) {
            atomicExch(err, 2);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint64_t ad = adesc0 + (uint64_t)((s * C::A_STAGE) >> 4);
          const uint64_t bd = bdesc0 + (uint64_t)((s * C::B_STAGE) >> 4);
          if (kc == 0) {
            // first chunk: each group of levels once the epilogue handed it back
            for (int grp = 0; grp < tmem_groups<C>() && ok; grp++) {
              if (local > 0 && !mbar_wait(&tempty[grp], (local - 1) & 1, 2 * WAIT_NS, err)) {
                atomicExch(err, 4);
                ok = false;
                break;
              }
              tc_fence_after();
              issue_group<C>(grp, tbase, ad, bd, true);
            }
            if (!ok) break;
          } else {
            issue_chunk<C>(tbase, ad, bd, false);
          }
          umma_commit(&empty[s]);  // stage s free once these MMAs have read it
        }
        if (ok) umma_commit(tfull);
      }
      // wait for every issued MMA before the accumulators are released
      umma_commit(drainb);
      if (!mbar_wait(drainb, 0, WAIT_NS)) atomicExch(err, 5);
    }
  } else {
    // epilogue: warp w drains TMEM lane quadrant w % 4; the EPI_WARPS / 4
    // warps of a quadrant split the tile's columns between them
    constexpr int EPH = C::EPI_WARPS / 4, CPW = C::BN / EPH;
    const int q = warp & 3, half = (warp - 2) / 4;
    const int et = threadIdx.x - 64;  // 0 .. 32 * EPI_WARPS - 1 within the epilogue group
    const int row = q * 32 + lane;
    const uint32_t tl = tbase + ((uint32_t)(q * 32) << 16);
    uint32_t local = 0;
    for (int tile = blockIdx.x; tile < ntiles_total; tile += gridDim.x, local++) {
      int inst, mt, nt;
      tile_coords(g, tile, inst, mt, nt);
      const SplitGemmInst* I = &g.inst[inst];
      // stage this tile's column exponents; the barrier also keeps the previous
      // tile's values until every epilogue thread has used them
      epi_bar<32 * C::EPI_WARPS>();
      if (et < C::BN) {
        sexp[et] = I->rexp[nt * C::BN + et];
        if constexpr (C::INT_OUT) {
          const int gcol = nt * C::BN + et;
          colp[et] = gcol < g.ncols ? I->outs[gcol / g.blkn] + (gcol % g.blkn) : nullptr;
        }
      }
      const int grow = mt * SPLIT_M + row;
      const bool rvalid = grow < g.mrows;
      const int erow = I->lexp[grow];
      // one thread waits for the accumulators; the outcome is shared so that
      // all epilogue threads leave the loop together
      if (et == 0) {
        const bool done = mbar_wait(tfull, local & 1, 4 * WAIT_NS, err);
        if (!done) atomicExch(err, 3);
        status[1] = done ? 0 : 1;
      }
      epi_bar<32 * C::EPI_WARPS>();
      if (status[1]) break;
      tc_fence_after();
      // Each warp drains its CPW columns into registers and hands TMEM back to
      // the MMA warp before it writes anything to global memory, so the next
      // tile's MMAs run while this tile's products are stored.
      const int cbase = half * CPW;
      // hand TMEM group grp back to the MMA warp (after this warp's loads of it)
      auto hand_back = [&](int grp) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[grp]);
      };
      if constexpr (C::INT_OUT) {
        // complex128 output: the exact levels and the last one summed exactly
        // in 64-bit integers (units 2^-54 of the row/column scale; level 0 is
        // below 2^8, so no overflow), then rounded once to double.
        // Level l < NL-1 holds integer multiples of 2^-(16+9l) (products of
        // digits d_i 2^(-8-9i) with i+j = l), at most 2^28 of them, so one
        // FP32 -> int32 conversion of v 2^(16+9l) is exact; the last level is
        // rounded to 2^-54 (|v| < 2^-24 there, so it fits an int32 as well;
        // 64-bit conversions would go through GB300's slow FP64 pipe).
        // Integer sums do not depend on the order of the levels.
        auto level_units = [](float v, int l) -> long long {
          if (l < C::NL - 1) return (long long)__float2int_rn(v * __int_as_float((127 + 16 + 9 * l) << 23)) << (38 - 9 * l);
          // the last level holds pairs i+j >= NL-1: |v| 2^54 <= 5 K 2^16 2^-52 2^54 < 2^30
          return (long long)__float2int_rn(v * __int_as_float((127 + 54) << 23));
        };
        // (each group goes back as soon as its last load has landed, before
        // that load's values are folded in: the MMA warp waits on the loads only)
        long long acc[2][CPW];
#pragma unroll
        for (int part = 0; part < 2; part++) {  // group 0: levels 0 and 1
          float v0[CPW], v1[CPW];
          tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, 0) + cbase), v0);
          tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, 1) + cbase), v1);
          tmem_ld_wait();
          if (part == 1) hand_back(0);
#pragma unroll
          for (int c = 0; c < CPW; c++) acc[part][c] = level_units(v0[c], 0) + level_units(v1[c], 1);
        }
#pragma unroll
        for (int l = 2; l < C::NL; l++) {  // group l - 1: level l
#pragma unroll
          for (int part = 0; part < 2; part++) {
            float v[CPW];
            tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, l) + cbase), v);
            tmem_ld_wait();
            if (part == 1) hand_back(l - 1);
#pragma unroll
            for (int c = 0; c < CPW; c++) acc[part][c] += level_units(v[c], l);
          }
        }
        if (rvalid) {
          const int erow = I->lexp[grow];
#pragma unroll
          for (int c = 0; c < CPW; c++) {
            double2* dst = colp[cbase + c];
            if (!dst) continue;
            const int e = erow + sexp[cbase + c] - 54;
            dst[(size_t)grow * g.blkn] = make_double2(i2d_scaled(acc[0][c], e), i2d_scaled(acc[1][c], e));
          }
        }
      } else {
        // float-float output: levels 0 .. NL-2 exact, combined by exact two-sums;
        // the rounding errors and the last level go to the low word.
        // (s, e)[part][c]: running sum and error of column cbase + c; after
        // the last level, (hi, lo).
        const int ldo = g.ldo;
        if (g.levels) {
          // raw level values for the exactness tests, read before any hand-back
          // (the loads are warp-collective; rows past the end store nothing)
#pragma unroll 1
          for (int pl = 0; pl < 2 * C::NL; pl++) {
            const int part = pl / C::NL, l = pl % C::NL;
#pragma unroll
            for (int cc = 0; cc < CPW; cc += 4) {
              float v[4];
              tmem_ld4(tl + (uint32_t)(C::acc_col(part, l) + cbase + cc), v);
              tmem_ld_wait();
#pragma unroll
              for (int c = 0; c < 4; c++) {
                const int gcol = nt * C::BN + cbase + cc + c;
                if (rvalid && gcol < g.ncols) g.levels[((size_t)(part * C::NL + l) * g.ncols + gcol) * ldo + grow] = v[c];
              }
            }
          }
        }
        // (each group goes back as soon as its last load has landed, before
        // that load's values are folded in: the MMA warp waits on the loads only)
        float s[2][CPW], e[2][CPW];
#pragma unroll
        for (int part = 0; part < 2; part++) {  // group 0: levels 0 and 1
          tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, 0) + cbase), s[part]);
          tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, 1) + cbase), e[part]);
          tmem_ld_wait();
          if (part == 1) hand_back(0);
#pragma unroll
          for (int c = 0; c < CPW; c++) {
            float t, d;
            two_sum(s[part][c], e[part][c], t, d);
            s[part][c] = t;
            e[part][c] = 0.f + d;
          }
        }
#pragma unroll
        for (int l = 2; l < C::NL; l++) {  // group l - 1: level l
#pragma unroll
          for (int part = 0; part < 2; part++) {
            float v[CPW];
            tmem_ld_cols<CPW>(tl + (uint32_t)(C::acc_col(part, l) + cbase), v);
            tmem_ld_wait();
            if (part == 1) hand_back(l - 1);
#pragma unroll
            for (int c = 0; c < CPW; c++) {
              if (l < C::NL - 1) {
                float t, d;
                two_sum(s[part][c], v[c], t, d);
                s[part][c] = t;
                e[part][c] += d;
              } else {
                float h, lw;
                fast_two_sum(s[part][c], e[part][c] + v[c], h, lw);
                s[part][c] = h;
                e[part][c] = lw;
              }
            }
          }
        }
        if (rvalid && !g.levels) {
          float4* outp = I->out;
#pragma unroll
          for (int c = 0; c < CPW; c++) {
            const int gcol = nt * C::BN + cbase + c;
            if (gcol >= g.ncols) continue;
            // the float-float products and their traces stay accurate while the
            // scale stays well inside FP32's normal range; below 2^-100 the
            // product is written as NaN, which flags the entries that use it for
            // recomputation in FP64 range
            const int ex = erow + sexp[cbase + c];
            const float sc = ex < FF_MIN_EXP ? __int_as_float(0x7fc00000) : pow2f(ex);
            outp[(size_t)gcol * ldo + grow] =
                make_float4(s[0][c] * sc, e[0][c] * sc, s[1][c] * sc, e[1][c] * sc);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tbase, TMEM_COLS);
  }
}

// ----------------------------------------------------------- closing traces
// rows[q * nrows + r] = coef_r * sum_{i,j < nev} A(i,j) conj(B(i,j)) with
// A = abase[q] + rt[r].aoff, B = bbase[q] + rt[r].boff, element (i, j) at
// [j * ld + i] (float-float complex).  One CTA of 128 threads per (pair, row),
// rows of a pair adjacent so that the blocks they share are re-read from L2;
// thread i walks column elements i (and i + 128) over all j and keeps its sum
// in float-float.  The same pass accumulates |coef_r| sum |A|_1 |B|_1 (high
// words, FP32; |z|_1 = |Re z| + |Im z|, within a factor 2 of the product of
// moduli) into rabs.
__global__ void __launch_bounds__(128) trace_rows_kernel(const TraceRow* __restrict__ rt, int nrows,
                                                         const float4* const* __restrict__ abase,
                                                         const float4* const* __restrict__ bbase, int lda, int ldb,
                                                         int nev, double2* __restrict__ rows,
                                                         double* __restrict__ rabs) {
  const int q = blockIdx.x / nrows, r = blockIdx.x % nrows;
  const TraceRow T = rt[r];
  const float4* pa = abase[q] + T.aoff;
  const float4* pb = bbase[q] + T.boff;
  float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f, sa = 0.f;
  for (int i = threadIdx.x; i < nev; i += 128) {
    for (int j = 0; j < nev; j++) {
      const float4 a = pa[(size_t)j * lda + i];
      const float4 b = pb[(size_t)j * ldb + i];
      ff_mac(sr, er, a.x, a.y, b.x, b.y);    // + ar br
      ff_mac(sr, er, a.z, a.w, b.z, b.w);    // + ai bi
      ff_mac(si, ei, a.z, a.w, b.x, b.y);    // + ai br
      ff_mac(si, ei, -a.x, -a.y, b.z, b.w);  // - ar bi
      sa = fmaf(fabsf(a.x) + fabsf(a.z), fabsf(b.x) + fabsf(b.z), sa);
    }
  }
  double re = (double)sr + (double)er, im = (double)si + (double)ei, ab = (double)sa;
  __shared__ double red[3][4];
  for (int o = 16; o; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
    ab += __shfl_down_sync(0xffffffffu, ab, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = re;
    red[1][threadIdx.x >> 5] = im;
    red[2][threadIdx.x >> 5] = ab;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    re = red[0][0] + red[0][1] + red[0][2] + red[0][3];
    im = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    ab = red[2][0] + red[2][1] + red[2][2] + red[2][3];
    const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
    rows[blockIdx.x] = cmul(c, make_double2(re, im));
    rabs[blockIdx.x] = sqrt(c.x * c.x + c.y * c.y) * ab;
  }
}

// Flattened form of the same traces: the TPB threads of a CTA walk the nev*nev
// elements in column order (element e -> i = e % nev, j = e / nev), so every
// thread is busy whatever nev is, and each thread sums fewer terms.
template <int TPB>
__global__ void __launch_bounds__(TPB) trace_rows_flat_kernel(const TraceRow* __restrict__ rt, int nrows,
                                                              const float4* const* __restrict__ abase,
                                                              const float4* const* __restrict__ bbase, int lda,
                                                              int ldb, int nev, double2* __restrict__ rows,
                                                              double* __restrict__ rabs) {
  constexpr int NW = TPB / 32;
  const int q = blockIdx.x / nrows, r = blockIdx.x % nrows;
  const TraceRow T = rt[r];
  const float4* pa = abase[q] + T.aoff;
  const float4* pb = bbase[q] + T.boff;
  float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f, sa = 0.f;
  const int total = nev * nev, di = TPB % nev, dj = TPB / nev;
  int i = threadIdx.x % nev, j = threadIdx.x / nev;
  for (int e = threadIdx.x; e < total; e += TPB) {
    const float4 a = pa[(size_t)j * lda + i];
    const float4 b = pb[(size_t)j * ldb + i];
    ff_mac(sr, er, a.x, a.y, b.x, b.y);    // + ar br
    ff_mac(sr, er, a.z, a.w, b.z, b.w);    // + ai bi
    ff_mac(si, ei, a.z, a.w, b.x, b.y);    // + ai br
    ff_mac(si, ei, -a.x, -a.y, b.z, b.w);  // - ar bi
    sa = fmaf(fabsf(a.x) + fabsf(a.z), fabsf(b.x) + fabsf(b.z), sa);
    i += di;
    j += dj;
    if (i >= nev) {
      i -= nev;
      j++;
    }
  }
  double re = (double)sr + (double)er, im = (double)si + (double)ei, ab = (double)sa;
  __shared__ double red[3][NW];
  for (int o = 16; o; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
    ab += __shfl_down_sync(0xffffffffu, ab, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = re;
    red[1][threadIdx.x >> 5] = im;
    red[2][threadIdx.x >> 5] = ab;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    re = 0.0;
    im = 0.0;
    ab = 0.0;
    for (int w = 0; w < NW; w++) {
      re += red[0][w];
      im += red[1][w];
      ab += red[2][w];
    }
    const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
    rows[blockIdx.x] = cmul(c, make_double2(re, im));
    rabs[blockIdx.x] = sqrt(c.x * c.x + c.y * c.y) * ab;
  }
}

// Flattened walk with U independent element streams per thread: the U pairs of
// loads of one step are issued before their sums, so each thread keeps 2U
// 16-byte loads in flight (the traces are bound by memory latency otherwise).
template <int TPB, int U>
__global__ void __launch_bounds__(TPB) trace_rows_ilp_kernel(const TraceRow* __restrict__ rt, int nrows,
                                                             const float4* const* __restrict__ abase,
                                                             const float4* const* __restrict__ bbase, int lda,
                                                             int ldb, int nev, double2* __restrict__ rows,
                                                             double* __restrict__ rabs) {
  constexpr int NW = TPB / 32;
  const int q = blockIdx.x / nrows, r = blockIdx.x % nrows;
  const TraceRow T = rt[r];
  const float4* pa = abase[q] + T.aoff;
  const float4* pb = bbase[q] + T.boff;
  float sr = 0.f, er = 0.f, si = 0.f, ei = 0.f, sa = 0.f;
  const int total = nev * nev, step = TPB * U, di = step % nev, dj = step / nev;
  int iu[U], ju[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int e = threadIdx.x + u * TPB;
    iu[u] = e % nev;
    ju[u] = e / nev;
  }
  for (int e0 = threadIdx.x; e0 < total; e0 += step) {
    float4 a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (e0 + u * TPB < total) {
        a[u] = pa[(size_t)ju[u] * lda + iu[u]];
        b[u] = pb[(size_t)ju[u] * ldb + iu[u]];
      } else {
        a[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        b[u] = a[u];
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      ff_mac(sr, er, a[u].x, a[u].y, b[u].x, b[u].y);    // + ar br
      ff_mac(sr, er, a[u].z, a[u].w, b[u].z, b[u].w);    // + ai bi
      ff_mac(si, ei, a[u].z, a[u].w, b[u].x, b[u].y);    // + ai br
      ff_mac(si, ei, -a[u].x, -a[u].y, b[u].z, b[u].w);  // - ar bi
      sa = fmaf(fabsf(a[u].x) + fabsf(a[u].z), fabsf(b[u].x) + fabsf(b[u].z), sa);
      iu[u] += di;
      ju[u] += dj;
      if (iu[u] >= nev) {
        iu[u] -= nev;
        ju[u]++;
      }
    }
  }
  double re = (double)sr + (double)er, im = (double)si + (double)ei, ab = (double)sa;
  __shared__ double red[3][NW];
  for (int o = 16; o; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
    ab += __shfl_down_sync(0xffffffffu, ab, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = re;
    red[1][threadIdx.x >> 5] = im;
    red[2][threadIdx.x >> 5] = ab;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    re = 0.0;
    im = 0.0;
    ab = 0.0;
    for (int w = 0; w < NW; w++) {
      re += red[0][w];
      im += red[1][w];
      ab += red[2][w];
    }
    const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
    rows[blockIdx.x] = cmul(c, make_double2(re, im));
    rabs[blockIdx.x] = sqrt(c.x * c.x + c.y * c.y) * ab;
  }
}

// Grouped traces.  CTA (pair q, group g): warp TG_CWARPS is the producer, whose
// lane 0 copies column j of every block of the group (nev float-float complex
// values, 16 nev contiguous bytes) into stage j % TG_NSTAGE by cp.async.bulk;
// consumer warp w computes traces w and w + TG_CWARPS of the group, lane l over
// the elements i = l, l + 32, ... of each column.  The stage ring is handed over
// with full (transaction bytes) and empty (one arrival per consumer warp)
// mbarriers; every wait is bounded and a timeout records an error code.
constexpr int TG_NSTAGE = 4, TG_CWARPS = TG_MAXT / 2;
constexpr int TG_THREADS = 32 * (TG_CWARPS + 1);
constexpr size_t trace_groups_max_smem() { return (size_t)TG_NSTAGE * (TG_MAXA + TG_MAXB) * SPLIT_MAXK * 16; }

__global__ void __launch_bounds__(TG_THREADS) trace_groups_kernel(
    const TraceGroup* __restrict__ groups, int ngroups, int stage_bytes, const TraceRow* __restrict__ rt, int nrows,
    const float4* const* __restrict__ abase, const float4* const* __restrict__ bbase, int lda, int ldb, int nev,
    double2* __restrict__ rows, double* __restrict__ rabs, int* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t sm[];
  __shared__ TraceGroup G;
  __shared__ uint64_t full[TG_NSTAGE], empty[TG_NSTAGE];
  __shared__ int status;
  const int q = blockIdx.x / ngroups, gi = blockIdx.x - q * ngroups;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  static_assert(sizeof(TraceGroup) % 4 == 0 && sizeof(TraceGroup) / 4 <= TG_THREADS, "group copy");
  if (threadIdx.x < (int)(sizeof(TraceGroup) / 4))
    ((int*)&G)[threadIdx.x] = ((const int*)(groups + gi))[threadIdx.x];
  if (threadIdx.x == 0) {
    for (int s = 0; s < TG_NSTAGE; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TG_CWARPS);
    }
    fence_mbar_init();
    status = *(volatile int*)err;
  }
  __syncthreads();
  if (status) return;  // uniform: a failure was recorded before this CTA started
  const int na = G.na, nb = G.nb;
  const uint32_t colb = (uint32_t)nev * 16u;

  if (warp == TG_CWARPS) {
    if (lane == 0) {
      const float4* pa = abase[q];
      const float4* pb = bbase[q];
      const uint32_t tx = (uint32_t)(na + nb) * colb;
      int issued = 0;
      for (int j = 0; j < nev; j++) {
        const int s = j % TG_NSTAGE;
        if (j >= TG_NSTAGE && !mbar_wait(&empty[s], ((j / TG_NSTAGE) - 1) & 1, WAIT_NS, err)) {
          atomicExch(err, 6);
          break;
        }
        uint8_t* dst = sm + (size_t)s * stage_bytes;
        mbar_arrive_expect_tx(&full[s], tx);
        for (int a = 0; a < na; a++) bulk_g2s(dst + a * colb, pa + G.aoff[a] + (size_t)j * lda, colb, &full[s]);
        for (int b = 0; b < nb; b++)
          bulk_g2s(dst + (na + b) * colb, pb + G.boff[b] + (size_t)j * ldb, colb, &full[s]);
        issued++;
      }
      // copies still in flight (only after a failure): wait for them, bounded,
      // before the CTA's shared memory is released
      for (int j = issued - 1; j >= 0 && j >= issued - TG_NSTAGE; j--)
        mbar_wait(&full[j % TG_NSTAGE], (j / TG_NSTAGE) & 1, WAIT_NS);
    }
    return;
  }

  float sr[2] = {0.f, 0.f}, er[2] = {0.f, 0.f}, si[2] = {0.f, 0.f}, ei[2] = {0.f, 0.f}, sa[2] = {0.f, 0.f};
  bool ok = true;
  for (int j = 0; j < nev; j++) {
    const int s = j % TG_NSTAGE;
    // every lane observes the stage's completion; the outcome is made warp-uniform
    const bool got = mbar_wait(&full[s], (j / TG_NSTAGE) & 1, WAIT_NS, err);
    if (!__all_sync(0xffffffffu, got)) {
      if (lane == 0) atomicExch(err, 7);
      ok = false;
      break;
    }
    const float4* col = (const float4*)(sm + (size_t)s * stage_bytes);
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const int t = warp + u * TG_CWARPS;
      if (t >= G.nt) continue;
      const float4* A = col + G.ta[t] * nev;
      const float4* B = col + (na + G.tb[t]) * nev;
      for (int i = lane; i < nev; i += 32) {
        const float4 a = A[i], b = B[i];
        ff_mac(sr[u], er[u], a.x, a.y, b.x, b.y);    // + ar br
        ff_mac(sr[u], er[u], a.z, a.w, b.z, b.w);    // + ai bi
        ff_mac(si[u], ei[u], a.z, a.w, b.x, b.y);    // + ai br
        ff_mac(si[u], ei[u], -a.x, -a.y, b.z, b.w);  // - ar bi
        sa[u] = fmaf(fabsf(a.x) + fabsf(a.z), fabsf(b.x) + fabsf(b.z), sa[u]);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  if (!ok) return;
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int t = warp + u * TG_CWARPS;
    if (t >= G.nt) continue;
    double re = (double)sr[u] + (double)er[u], im = (double)si[u] + (double)ei[u], ab = (double)sa[u];
    for (int o = 16; o; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
      ab += __shfl_down_sync(0xffffffffu, ab, o);
    }
    if (lane == 0) {
      const int r = G.tr[t];
      const TraceRow T = rt[r];
      const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
      rows[(size_t)q * nrows + r] = cmul(c, make_double2(re, im));
      rabs[(size_t)q * nrows + r] = sqrt(c.x * c.x + c.y * c.y) * ab;
    }
  }
}

// Quad groups: at most 2 A blocks and 2 B blocks and the (up to 4) traces
// between them.  One CTA per (pair, group) walks the nev*nev elements with U
// independent streams a thread; each element of the group's (at most 4) blocks
// is loaded once and feeds every trace of the group, so a block shared by two
// traces is read once instead of twice.
template <int TPB, int U>
__global__ void __launch_bounds__(TPB) trace_quads_kernel(const TraceGroup* __restrict__ groups, int ngroups,
                                                          const TraceRow* __restrict__ rt, int nrows,
                                                          const float4* const* __restrict__ abase,
                                                          const float4* const* __restrict__ bbase, int lda, int ldb,
                                                          int nev, double2* __restrict__ rows,
                                                          double* __restrict__ rabs) {
  constexpr int NW = TPB / 32;
  const int q = blockIdx.x / ngroups, gi = blockIdx.x - q * ngroups;
  const TraceGroup& G = groups[gi];
  const int na = G.na, nb = G.nb, nt = G.nt;
  unsigned mask = 0;  // bit a * 2 + b: trace between A block a and B block b
  for (int t = 0; t < nt; t++) mask |= 1u << (G.ta[t] * 2 + G.tb[t]);
  const float4* pa0 = abase[q] + G.aoff[0];
  const float4* pa1 = abase[q] + G.aoff[na > 1 ? 1 : 0];
  const float4* pb0 = bbase[q] + G.boff[0];
  const float4* pb1 = bbase[q] + G.boff[nb > 1 ? 1 : 0];
  float sr[4], er[4], si[4], ei[4], sa[4];
#pragma unroll
  for (int k = 0; k < 4; k++) sr[k] = er[k] = si[k] = ei[k] = sa[k] = 0.f;
  const int total = nev * nev, step = TPB * U, di = step % nev, dj = step / nev;
  int iu[U], ju[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int e = threadIdx.x + u * TPB;
    iu[u] = e % nev;
    ju[u] = e / nev;
  }
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int e0 = threadIdx.x; e0 < total; e0 += step) {
    float4 a[U][2], b[U][2];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const bool in = e0 + u * TPB < total;
      const size_t oa = (size_t)ju[u] * lda + iu[u], ob = (size_t)ju[u] * ldb + iu[u];
      a[u][0] = in ? pa0[oa] : z;
      a[u][1] = (in && na > 1) ? pa1[oa] : z;
      b[u][0] = in ? pb0[ob] : z;
      b[u][1] = (in && nb > 1) ? pb1[ob] : z;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (!((mask >> k) & 1u)) continue;
        const float4 x = a[u][k >> 1], y = b[u][k & 1];
        ff_mac(sr[k], er[k], x.x, x.y, y.x, y.y);    // + ar br
        ff_mac(sr[k], er[k], x.z, x.w, y.z, y.w);    // + ai bi
        ff_mac(si[k], ei[k], x.z, x.w, y.x, y.y);    // + ai br
        ff_mac(si[k], ei[k], -x.x, -x.y, y.z, y.w);  // - ar bi
        sa[k] = fmaf(fabsf(x.x) + fabsf(x.z), fabsf(y.x) + fabsf(y.z), sa[k]);
      }
      iu[u] += di;
      ju[u] += dj;
      if (iu[u] >= nev) {
        iu[u] -= nev;
        ju[u]++;
      }
    }
  }
  __shared__ double red[4][3][NW];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (!((mask >> k) & 1u)) continue;
    double re = (double)sr[k] + (double)er[k], im = (double)si[k] + (double)ei[k], ab = (double)sa[k];
    for (int o = 16; o; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
      ab += __shfl_down_sync(0xffffffffu, ab, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[k][0][threadIdx.x >> 5] = re;
      red[k][1][threadIdx.x >> 5] = im;
      red[k][2][threadIdx.x >> 5] = ab;
    }
  }
  __syncthreads();
  if (threadIdx.x < nt) {
    const int t = threadIdx.x, k = G.ta[t] * 2 + G.tb[t];
    double re = 0.0, im = 0.0, ab = 0.0;
    for (int w = 0; w < NW; w++) {
      re += red[k][0][w];
      im += red[k][1][w];
      ab += red[k][2][w];
    }
    const int r = G.tr[t];
    const TraceRow T = rt[r];
    const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
    rows[(size_t)q * nrows + r] = cmul(c, make_double2(re, im));
    rabs[(size_t)q * nrows + r] = sqrt(c.x * c.x + c.y * c.y) * ab;
  }
}

// Failure detection check: one thread waits, through the same bounded wait as
// the GEMM pipeline, on an mbarrier that nothing arrives at; the wait gives up
// after timeout_ns and records error code 9.  Nothing hangs: the kernel returns.
__global__ void wait_probe_kernel(unsigned long long timeout_ns, int* __restrict__ err) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  if (!mbar_wait(&bar, 0, timeout_ns)) atomicExch(err, 9);
}

// ------------------------------------------------ closing traces as Gram products
// |v| / 2^E as a float from the double's high word (integer operations; the
// mantissa truncated to 20 bits, enough for a norm that bounds an error), 0
// below FP32's normal range.  |v| < 2^E, so the result is below 1.
__device__ __forceinline__ float abs_rel_f32(double v, int E) {
  const int hi = __double2hiint(v) & 0x7FFFFFFF;
  const int e = (hi >> 20) - 1023 - E + 127;
  return e <= 0 ? 0.f : __int_as_float((e << 23) | ((hi & 0xFFFFF) << 3));
}

// Gram operand slicing: CTA = (instance ip = group * npiece + piece, 8 rows of
// an operand tile).  Rows are blocks flattened to n2 elements (tiles of TR =
// 128 left rows or BN right columns); K is the piece.  The CTA stages its 8
// rows' pieces in shared memory (one read of each element); warp w then takes
// row w: its scale exponent is the largest bound (plus one: the leading digit
// halved), its norm the 2-norm of (|Re| + |Im|) / 2^E.  Last, warp w writes
// the digits of rows 2 (w % 4) and 2 (w % 4) + 1 (one per half warp, so that
// each store fills whole 32-byte sectors of the core matrices) over half of
// the piece, as packed BF16 pairs straight to the tiled operand.  Rows past
// nrows get their exponent and norm but no digits: their products land in
// padding rows or columns that are never stored.  Right tiles hold conj(Y) in
// the packed planes (-Im, Re, Im).
constexpr int GRAM_SLICE_SMEM = 8 * GRAM_PIECE * 16;
template <class C, bool RIGHT>
__global__ void __launch_bounds__(256) slice_gram_kernel(const double2* const* __restrict__ blk, int nrows, int ntile,
                                                         int n2, int npiece, int nchunk, uint8_t* __restrict__ out,
                                                         int* __restrict__ exps, float* __restrict__ norms) {
  constexpr int TR = RIGHT ? C::BN : SPLIT_M;
  constexpr int STAGE = RIGHT ? C::B_STAGE : C::A_STAGE;
  constexpr int SUB = RIGHT ? C::B_SUB : C::A_SUB;
  constexpr int RG = TR / 8;  // CTAs per tile
  static_assert(TR % 8 == 0, "8 rows a CTA");
  extern __shared__ __align__(16) double2 sv[];  // [8][GRAM_PIECE]
  __shared__ int sE[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ip = blockIdx.x / (ntile * RG), rest = blockIdx.x - ip * (ntile * RG);
  const int t = rest / RG, r0 = (rest - t * RG) * 8;  // first row of the CTA within the tile
  const int g = ip / npiece, p = ip - g * npiece;
  const int piece = nchunk * SPLIT_K, k0 = p * piece, kmax = min(piece, n2 - k0);
  // asynchronous copies (all of a thread's 16 in flight), zeros written directly
#pragma unroll
  for (int rr = 0; rr < 8; rr++) {
    const int row = t * TR + r0 + rr;
    const double2* b = row < nrows ? blk[(size_t)g * nrows + row] : nullptr;
#pragma unroll
    for (int u = 0; u < GRAM_PIECE / 256; u++) {
      const int k = threadIdx.x + 256 * u;
      if (k >= piece) continue;
      if (b && k < kmax)
        cp_async16(sv + rr * GRAM_PIECE + k, b + k0 + k);
      else
        sv[rr * GRAM_PIECE + k] = make_double2(0.0, 0.0);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  {
    const double2* x = sv + warp * GRAM_PIECE;
    int m = -30000;
    for (int k = lane; k < piece; k += 32) m = max(m, max(f64_exp_bound(x[k].x), f64_exp_bound(x[k].y)));
    for (int off = 16; off; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
    const int E = (m < -1000 ? 0 : m) + 1;
    float nn = 0.f;
    for (int k = lane; k < piece; k += 32) {
      const float a = abs_rel_f32(x[k].x, E) + abs_rel_f32(x[k].y, E);
      nn = fmaf(a, a, nn);
    }
    for (int off = 16; off; off >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, off);
    if (lane == 0) {
      const size_t orow = ((size_t)ip * ntile + t) * TR + r0 + warp;
      exps[orow] = E;
      norms[orow] = m < -1000 ? 0.f : sqrtf(nn);
      sE[warp] = E;
    }
  }
  __syncthreads();
  const int rr = 2 * (warp & 3) + (lane >> 4);
  if (t * TR + r0 + rr >= nrows) return;
  const int E = sE[rr];
  const double2* x = sv + rr * GRAM_PIECE;
  uint8_t* tile = out + ((size_t)ip * ntile + t) * nchunk * STAGE;
  for (int q = (warp >> 2) * (GRAM_PIECE / 4) + (lane & 15); q < (warp >> 2) * (GRAM_PIECE / 4) + GRAM_PIECE / 4;
       q += 16) {
    const int k = 2 * q;
    if (k >= piece) break;
    bool nr0, ni0, nr1, ni1;
    uint64_t Ur0, Ui0, Ur1, Ui1;
    weighted_fixed(x[k], 0, false, RIGHT, E, Ur0, nr0, Ui0, ni0);
    weighted_fixed(x[k + 1], 0, false, RIGHT, E, Ur1, nr1, Ui1, ni1);
    Ur0 = round_fixed<C::NS>(Ur0);
    Ui0 = round_fixed<C::NS>(Ui0);
    Ur1 = round_fixed<C::NS>(Ur1);
    Ui1 = round_fixed<C::NS>(Ui1);
    uint8_t* d = tile + (size_t)(k >> 4) * STAGE + core_offset(r0 + rr, k & 15);
#pragma unroll
    for (int s = 0; s < C::NS; s++) {
      const uint32_t re = slice_pair(Ur0, nr0, Ur1, nr1, s), im = slice_pair(Ui0, ni0, Ui1, ni1, s);
      if constexpr (RIGHT) {
        *(uint32_t*)(d + (s * 3 + 0) * SUB) = im ^ BF16X2_SIGNS;
        *(uint32_t*)(d + (s * 3 + 1) * SUB) = re;
        *(uint32_t*)(d + (s * 3 + 2) * SUB) = im;
      } else {
        *(uint32_t*)(d + (s * 2 + 0) * SUB) = re;
        *(uint32_t*)(d + (s * 2 + 1) * SUB) = im;
      }
    }
  }
}

// Trace values of a Gram launch, one thread per trace: the pieces' partial
// products summed in piece order, times the coefficient; the error scale
// sum_p (|x_p| |y_p| + 8) 2^(E_x + E_y) bounds sum |x|_1 |y|_1 (Cauchy-Schwarz
// over the piece) and the truncation of the slices (~2^-54 of the scales an
// element, 2^-48 over a piece's 512 of them with random signs); a piece whose
// row or column is all zeros adds neither.
__global__ void __launch_bounds__(128) gram_trace_sum_kernel(const GramTrace* __restrict__ tr, int ntr, int g0,
                                                             const double2* __restrict__ part, int npiece, int lrows,
                                                             int rcols, const int* __restrict__ lexp,
                                                             const int* __restrict__ rexp,
                                                             const float* __restrict__ lnorm,
                                                             const float* __restrict__ rnorm, double2* __restrict__ trv,
                                                             double* __restrict__ tra) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntr) return;
  const GramTrace T = tr[i];
  double re = 0.0, im = 0.0, ab = 0.0;
  for (int p = 0; p < npiece; p++) {
    const size_t ip = (size_t)(T.g - g0) * npiece + p;
    const double2 v = part[(ip * lrows + T.r) * rcols + T.c];
    re += v.x;
    im += v.y;
    if (tra) {
      const float nx = lnorm[ip * lrows + T.r], ny = rnorm[ip * rcols + T.c];
      if (nx > 0.f && ny > 0.f)
        ab += ((double)nx * (double)ny + 8.0) * pow2d(lexp[ip * lrows + T.r] + rexp[ip * rcols + T.c]);
    }
  }
  const double2 c = make_double2((double)T.coef[0], (double)T.coef[1]);
  trv[T.slot] = cmul(c, make_double2(re, im));
  if (tra) tra[T.slot] = sqrt(c.x * c.x + c.y * c.y) * ab;
}

// --------------------------------------------------------------- launchers
// Dynamic shared-memory limits are raised once per kernel (before any graph
// capture, through split_kernels_prepare, or at the first launch).
template <typename K>
static int ensure_smem(K kernel, size_t smem, bool& done) {
  if (!done) {
    CTR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    done = true;
  }
  return CTR_OK;
}
static bool g_attr_sls = false, g_attr_srs = false, g_attr_tg = false, g_attr_sld = false, g_attr_srd = false;
static bool g_attr_sl = false, g_attr_sr = false, g_attr_tl = false, g_attr_std = false,
            g_attr_hp = false;
static int g_nsm = 0;

template <class C>
static bool& gemm_attr_flag();
template <>
bool& gemm_attr_flag<CfgStd>() { return g_attr_std; }
template <>
bool& gemm_attr_flag<CfgHP>() { return g_attr_hp; }

static int sm_count(int* out) {
  if (!g_nsm) {
    int dev = 0;
    CTR_CUDA(cudaGetDevice(&dev));
    CTR_CUDA(cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  *out = g_nsm;
  return CTR_OK;
}

int split_kernels_prepare() {
  int nsm;
  CTR_TRY(sm_count(&nsm));
  CTR_TRY(ensure_smem(slice_left_kernel, 512 + SPLIT_A_STAGE, g_attr_sl));
  CTR_TRY(ensure_smem(slice_right_kernel, 512 + SPLIT_B_STAGE, g_attr_sr));
  CTR_TRY(ensure_smem(slice_left_staged_kernel<false>, slice_staged_smem(SPLIT_MAXK, SPLIT_NSLICE * 2), g_attr_sls));
  CTR_TRY(ensure_smem(slice_right_staged_kernel<false>, slice_staged_smem(SPLIT_MAXK, SPLIT_NSLICE * 3), g_attr_srs));
  CTR_TRY(ensure_smem(slice_left_staged_kernel<true>, slice_staged_smem(SPLIT_MAXK, 0), g_attr_sld));
  CTR_TRY(ensure_smem(slice_right_staged_kernel<true>, slice_staged_smem(SPLIT_MAXK, 0), g_attr_srd));
  CTR_TRY(ensure_smem(trace_groups_kernel, trace_groups_max_smem(), g_attr_tg));
  CTR_TRY(ensure_smem(slice_task_left_kernel<CfgHP>, 512 + CfgHP::A_STAGE, g_attr_tl));
  CTR_TRY(ensure_smem(split_gemm_kernel<CfgStd>, gemm_smem_bytes<CfgStd>(), g_attr_std));
  CTR_TRY(ensure_smem(split_gemm_kernel<CfgHP>, gemm_smem_bytes<CfgHP>(), g_attr_hp));
  return CTR_OK;
}

int launch_slice_left(const SliceLeftJob* d_jobs, int njobs, int nev, int nchunk, int mtiles, cudaStream_t s,
                      int form) {
  if (njobs == 0) return CTR_OK;
  if (form == 1 || form == 2) {
    if (nev > SPLIT_MAXK) return fail(CTR_ERR_ARG, "slicer: Nev %d above %d", nev, SPLIT_MAXK);
    const int grid = njobs * mtiles * (SPLIT_M / SLQ);
    TimedLaunch tl(s, "slice_left");
    if (form == 2) {
      CTR_TRY(ensure_smem(slice_left_staged_kernel<true>, slice_staged_smem(SPLIT_MAXK, 0), g_attr_sld));
      slice_left_staged_kernel<true><<<grid, 256, slice_staged_smem(nev, 0), s>>>(d_jobs, nev, nchunk, mtiles);
    } else {
      CTR_TRY(ensure_smem(slice_left_staged_kernel<false>, slice_staged_smem(SPLIT_MAXK, SPLIT_NSLICE * 2), g_attr_sls));
      slice_left_staged_kernel<false>
          <<<grid, 256, slice_staged_smem(nev, SPLIT_NSLICE * 2), s>>>(d_jobs, nev, nchunk, mtiles);
    }
    CTR_CUDA(cudaGetLastError());
    return CTR_OK;
  }
  const size_t smem = 512 + SPLIT_A_STAGE;
  CTR_TRY(ensure_smem(slice_left_kernel, smem, g_attr_sl));
  TimedLaunch tl(s, "slice_left");
  slice_left_kernel<<<njobs * mtiles, 256, smem, s>>>(d_jobs, nev, nchunk, mtiles);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_slice_right(const SliceRightJob* d_jobs, int njobs, int nev, int nchunk, int ntiles, cudaStream_t s,
                       int form) {
  if (njobs == 0) return CTR_OK;
  if (form == 1 || form == 2) {
    if (nev > SPLIT_MAXK) return fail(CTR_ERR_ARG, "slicer: Nev %d above %d", nev, SPLIT_MAXK);
    const int grid = njobs * ntiles * (SPLIT_N / SLQ);
    TimedLaunch tl(s, "slice_right");
    if (form == 2) {
      CTR_TRY(ensure_smem(slice_right_staged_kernel<true>, slice_staged_smem(SPLIT_MAXK, 0), g_attr_srd));
      slice_right_staged_kernel<true><<<grid, 256, slice_staged_smem(nev, 0), s>>>(d_jobs, nev, nchunk, ntiles);
    } else {
      CTR_TRY(ensure_smem(slice_right_staged_kernel<false>, slice_staged_smem(SPLIT_MAXK, SPLIT_NSLICE * 3), g_attr_srs));
      slice_right_staged_kernel<false>
          <<<grid, 256, slice_staged_smem(nev, SPLIT_NSLICE * 3), s>>>(d_jobs, nev, nchunk, ntiles);
    }
    CTR_CUDA(cudaGetLastError());
    return CTR_OK;
  }
  const size_t smem = 512 + SPLIT_B_STAGE;
  CTR_TRY(ensure_smem(slice_right_kernel, smem, g_attr_sr));
  TimedLaunch tl(s, "slice_right");
  slice_right_kernel<<<njobs * ntiles, 256, smem, s>>>(d_jobs, nev, nchunk, ntiles);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_slice_task_left(const SliceTaskLJob* d_jobs, int njobs, int nev, int nchunk, const int* bexp,
                           cudaStream_t s) {
  if (njobs == 0) return CTR_OK;
  const size_t smem = 512 + CfgHP::A_STAGE;
  CTR_TRY(ensure_smem(slice_task_left_kernel<CfgHP>, smem, g_attr_tl));
  TimedLaunch tl(s, "slice_task_left");
  slice_task_left_kernel<CfgHP><<<njobs * nchunk, 256, smem, s>>>(d_jobs, nev, nchunk, bexp);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_slice_stack_left(const SliceStackLJob* d_jobs, int njobs, int nev, int nchunk, int mtiles, const int* bexp,
                            cudaStream_t s) {
  if (njobs == 0) return CTR_OK;
  const long long grid = (long long)njobs * mtiles * nchunk;
  if (grid > 0x7fffffffLL) return fail(CTR_ERR_ARG, "stacked slicer: grid too large");
  TimedLaunch tl(s, "slice_stack_left");
  slice_stack_left_kernel<CfgHP><<<(unsigned)grid, 256, 0, s>>>(d_jobs, nev, nchunk, mtiles, bexp);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_slice_task_right(const SliceTaskRJob* d_jobs, int njobs, int nev, int nchunk, int ntiles, const int* bexp,
                            cudaStream_t s) {
  if (njobs == 0) return CTR_OK;
  TimedLaunch tl(s, "slice_task_right");
  slice_task_right_kernel<CfgHP><<<njobs * ntiles * nchunk, 128, 0, s>>>(d_jobs, nev, nchunk, ntiles, bexp);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

static bool g_attr_gl = false, g_attr_gr = false;

int launch_slice_gram(bool right, const double2* const* d_blk, int ngroup, int nrows, int ntile, int n2, int npiece,
                      int nchunk, uint8_t* out, int* exps, float* norms, cudaStream_t s) {
  if (ngroup == 0) return CTR_OK;
  if (nchunk < 1 || nchunk * SPLIT_K > GRAM_PIECE || (long long)npiece * nchunk * SPLIT_K < n2)
    return fail(CTR_ERR_ARG, "Gram slicer: %d chunks x %d pieces do not cover %d elements", nchunk, npiece, n2);
  const long long grid = (long long)ngroup * npiece * ntile;
  if (grid * (SPLIT_M / 8) > 0x7fffffffLL) return fail(CTR_ERR_ARG, "Gram slicer: grid too large");
  if (right) {
    CTR_TRY(ensure_smem(slice_gram_kernel<CfgHP, true>, GRAM_SLICE_SMEM, g_attr_gr));
    TimedLaunch tl(s, "slice_gram_right");
    slice_gram_kernel<CfgHP, true><<<(unsigned)(grid * (CfgHP::BN / 8)), 256, GRAM_SLICE_SMEM, s>>>(
        d_blk, nrows, ntile, n2, npiece, nchunk, out, exps, norms);
  } else {
    CTR_TRY(ensure_smem(slice_gram_kernel<CfgHP, false>, GRAM_SLICE_SMEM, g_attr_gl));
    TimedLaunch tl(s, "slice_gram_left");
    slice_gram_kernel<CfgHP, false><<<(unsigned)(grid * (SPLIT_M / 8)), 256, GRAM_SLICE_SMEM, s>>>(
        d_blk, nrows, ntile, n2, npiece, nchunk, out, exps, norms);
  }
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_gram_trace_sum(const GramTrace* d_tr, int ntr, int g0, const double2* part, int npiece, int lrows, int rcols,
                          const int* lexp, const int* rexp, const float* lnorm, const float* rnorm, double2* trv,
                          double* tra, cudaStream_t s) {
  if (ntr == 0) return CTR_OK;
  TimedLaunch tl(s, "gram_trace_sum");
  gram_trace_sum_kernel<<<(ntr + 127) / 128, 128, 0, s>>>(d_tr, ntr, g0, part, npiece, lrows, rcols, lexp, rexp,
                                                          lnorm, rnorm, trv, tra);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

// MMA schedule probe: the split GEMM's exact per-chunk MMA schedule (issue_chunk
// of configuration C, a commit per chunk, NSTAGE stage buffers) issued back to
// back by one thread per SM from shared-memory operands that stay put (hashed
// BF16 digits, magnitudes near 1), with no producer and no epilogue.  It
// measures what the tensor pipe gives this schedule by itself; the GEMM's own
// rate against it shows what its pipeline and tile hand-off cost.  cycles[0]
// accumulates the issuing thread's clock64 span over the CTAs.
template <class C>
__global__ void __launch_bounds__(128, 1) mma_schedule_probe_kernel(int nchunk, unsigned long long* __restrict__ cycles,
                                                                    int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + NSTAGE * C::A_STAGE;
  __shared__ uint64_t bar, ebar[NSTAGE];
  __shared__ uint32_t tslot;
  const int nwords = NSTAGE * (C::A_STAGE + C::B_STAGE) / 4;
  for (int i = threadIdx.x; i < nwords; i += blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u + blockIdx.x * 97u;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    ((uint32_t*)smem)[i] = (h & 0x807f807fu) | 0x3f003f00u;  // two BF16 of random sign, in [0.5, 1)
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    for (int st = 0; st < NSTAGE; st++) mbar_init(&ebar[st], 1);
    fence_mbar_init();
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes, then tensor-core reads
  __syncthreads();
  if (threadIdx.x < 32) {
    tmem_alloc(&tslot, TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tslot;
  if (threadIdx.x == 0) {
    const uint64_t adesc0 = sdesc_kmajor_noswz(smem_u32(sA), 128, 256);
    const uint64_t bdesc0 = sdesc_kmajor_noswz(smem_u32(sB), 128, 256);
    const unsigned long long t0 = clock64();
    for (int c = 0; c < nchunk; c++) {
      const int st = c % NSTAGE;
      issue_chunk<C>(tbase, adesc0 + (uint64_t)((st * C::A_STAGE) >> 4), bdesc0 + (uint64_t)((st * C::B_STAGE) >> 4),
                     c == 0);
      umma_commit(&ebar[st]);
    }
    umma_commit(&bar);
    if (!mbar_wait(&bar, 0, WAIT_NS)) atomicExch(err, 8);
    atomicAdd(cycles, clock64() - t0);
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    tmem_dealloc(tbase, TMEM_COLS);
  }
}

static bool g_attr_probe_std = false, g_attr_probe_hp = false;
template <class C>
static int launch_mma_probe_cfg(int nchunk, unsigned long long* d_cycles, int* d_err, bool& attr, int* nsm_out,
                                cudaStream_t s) {
  const size_t smem = (size_t)NSTAGE * (C::A_STAGE + C::B_STAGE);
  CTR_TRY(ensure_smem(mma_schedule_probe_kernel<C>, smem, attr));
  int nsm;
  CTR_TRY(sm_count(&nsm));
  TimedLaunch tl(s, "mma_schedule_probe");
  mma_schedule_probe_kernel<C><<<nsm, 128, smem, s>>>(nchunk, d_cycles, d_err);
  CTR_CUDA(cudaGetLastError());
  *nsm_out = nsm;
  return CTR_OK;
}

int launch_mma_schedule_probe(int hp, int nchunk, unsigned long long* d_cycles, int* d_err, int* nsm, int* mmas_per_chunk,
                              int* mma_n, cudaStream_t s) {
  if (hp) {
    *mmas_per_chunk = CfgHP::NS * (CfgHP::NS + 1);
    *mma_n = 2 * CfgHP::BN;
    return launch_mma_probe_cfg<CfgHP>(nchunk, d_cycles, d_err, g_attr_probe_hp, nsm, s);
  }
  *mmas_per_chunk = CfgStd::NS * (CfgStd::NS + 1);
  *mma_n = 2 * CfgStd::BN;
  return launch_mma_probe_cfg<CfgStd>(nchunk, d_cycles, d_err, g_attr_probe_std, nsm, s);
}

int launch_wait_probe(unsigned long long timeout_ns, int* d_err, cudaStream_t s) {
  TimedLaunch tl(s, "wait_probe");
  wait_probe_kernel<<<1, 32, 0, s>>>(timeout_ns, d_err);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_block_exp(const double2* const* d_blk, int nblk, int nev, int* bexp, cudaStream_t s) {
  if (nblk == 0) return CTR_OK;
  if (nev > SPLIT_MAXK) return fail(CTR_ERR_ARG, "block exponents: Nev %d above %d", nev, SPLIT_MAXK);
  TimedLaunch tl(s, "block_exp");
  block_exp_kernel<<<nblk, 256, 0, s>>>(d_blk, nev, bexp);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

template <class C>
static int launch_split_gemm_cfg(const SplitGemmBatch& g, int ninst, int* d_err, cudaStream_t s, const char* name,
                                 double* flops) {
  const size_t smem = gemm_smem_bytes<C>();
  CTR_TRY(ensure_smem(split_gemm_kernel<C>, smem, gemm_attr_flag<C>()));
  int nsm;
  CTR_TRY(sm_count(&nsm));
  const long long total = (long long)ninst * g.mtiles * g.ntiles;
  if (total > 0x7fffffffLL) return fail(CTR_ERR_ARG, "split GEMM: too many tiles");
  const int grid = (int)std::min<long long>(total, nsm);
  TimedLaunch tl(s, name);
  split_gemm_kernel<C><<<grid, gemm_threads<C>(), smem, s>>>(g, (int)total, d_err);
  CTR_CUDA(cudaGetLastError());
  // slice pairs i + j < NS, each two packed MMAs of M x 2BN x 16: 8 M BN 16 flops
  if (!capturing()) *flops += (double)total * (C::NS * (C::NS + 1) / 2) * 8.0 * SPLIT_M * C::BN * SPLIT_K * g.nchunk;
  return CTR_OK;
}

int launch_split_gemm(const SplitGemmBatch& g, int ninst, int* d_err, cudaStream_t s, bool gram) {
  if (ninst == 0) return CTR_OK;
  if (g.hp) {
    if (g.out_mode != 1 || g.levels) return fail(CTR_ERR_ARG, "split GEMM: the high-precision tiles write complex128");
    return gram ? launch_split_gemm_cfg<CfgHP>(g, ninst, d_err, s, "gram_gemm", &g_gram_mma_flops)
                : launch_split_gemm_cfg<CfgHP>(g, ninst, d_err, s, "split_gemm_hp", &g_split_mma_flops);
  }
  if (gram || g.out_mode != 0) return fail(CTR_ERR_ARG, "split GEMM: the standard tiles write float-float");
  return launch_split_gemm_cfg<CfgStd>(g, ninst, d_err, s, "split_gemm", &g_split_mma_flops);
}

int launch_trace_rows(const TraceRow* d_rows, int nrows, const float4* const* d_abase, const float4* const* d_bbase,
                      int lda, int ldb, int npair, int nev, double2* rows, double* rabs, int variant,
                      cudaStream_t s) {
  if (npair == 0 || nrows == 0) return CTR_OK;
  const long long nblk = (long long)npair * nrows;
  if (nblk > 0x7fffffffLL) return fail(CTR_ERR_ARG, "traces: grid too large");
  TimedLaunch tl(s, "trace_rows");
  switch (variant) {
    case 0:
      trace_rows_kernel<<<(unsigned)nblk, 128, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 1:
      trace_rows_flat_kernel<128>
          <<<(unsigned)nblk, 128, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 2:
      trace_rows_flat_kernel<256>
          <<<(unsigned)nblk, 256, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 3:
      trace_rows_flat_kernel<512>
          <<<(unsigned)nblk, 512, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 4:
      trace_rows_ilp_kernel<128, 4>
          <<<(unsigned)nblk, 128, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 5:
      trace_rows_ilp_kernel<256, 2>
          <<<(unsigned)nblk, 256, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 6:
      trace_rows_ilp_kernel<64, 4>
          <<<(unsigned)nblk, 64, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 7:
      trace_rows_ilp_kernel<64, 8>
          <<<(unsigned)nblk, 64, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    case 8:
      trace_rows_ilp_kernel<128, 8>
          <<<(unsigned)nblk, 128, 0, s>>>(d_rows, nrows, d_abase, d_bbase, lda, ldb, nev, rows, rabs);
      break;
    default: return fail(CTR_ERR_ARG, "traces: unknown variant %d", variant);
  }
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_trace_groups(const TraceGroup* d_groups, int ngroups, int maxcols, const TraceRow* d_rows, int nrows,
                        const float4* const* d_abase, const float4* const* d_bbase, int lda, int ldb, int npair,
                        int nev, double2* rows, double* rabs, int* d_err, cudaStream_t s) {
  if (npair == 0 || ngroups == 0) return CTR_OK;
  if (maxcols < 1 || maxcols > TG_MAXA + TG_MAXB) return fail(CTR_ERR_ARG, "trace groups: %d blocks per group", maxcols);
  const long long nblk = (long long)npair * ngroups;
  if (nblk > 0x7fffffffLL) return fail(CTR_ERR_ARG, "trace groups: grid too large");
  if (nev > SPLIT_MAXK) return fail(CTR_ERR_ARG, "trace groups: Nev %d above %d", nev, SPLIT_MAXK);
  const int stage_bytes = maxcols * nev * 16;
  const size_t smem = (size_t)TG_NSTAGE * stage_bytes;
  CTR_TRY(ensure_smem(trace_groups_kernel, trace_groups_max_smem(), g_attr_tg));
  TimedLaunch tl(s, "trace_groups");
  trace_groups_kernel<<<(unsigned)nblk, TG_THREADS, smem, s>>>(d_groups, ngroups, stage_bytes, d_rows, nrows,
                                                                d_abase, d_bbase, lda, ldb, nev, rows, rabs, d_err);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int launch_trace_quads(const TraceGroup* d_groups, int ngroups, const TraceRow* d_rows, int nrows,
                       const float4* const* d_abase, const float4* const* d_bbase, int lda, int ldb, int npair,
                       int nev, double2* rows, double* rabs, int variant, cudaStream_t s) {
  if (npair == 0 || ngroups == 0) return CTR_OK;
  const long long nblk = (long long)npair * ngroups;
  if (nblk > 0x7fffffffLL) return fail(CTR_ERR_ARG, "trace quads: grid too large");
  TimedLaunch tl(s, "trace_quads");
  if (variant == 0)
    trace_quads_kernel<128, 2><<<(unsigned)nblk, 128, 0, s>>>(d_groups, ngroups, d_rows, nrows, d_abase, d_bbase,
                                                                lda, ldb, nev, rows, rabs);
  else
    trace_quads_kernel<64, 4><<<(unsigned)nblk, 64, 0, s>>>(d_groups, ngroups, d_rows, nrows, d_abase, d_bbase,
                                                              lda, ldb, nev, rows, rabs);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int build_trace_groups(const TraceRow* rows, int nrows, int maxa, int maxb, int maxt,
                       std::vector<TraceGroup>& groups) {
  if (maxa > TG_MAXA || maxb > TG_MAXB || maxt > TG_MAXT) return -1;
  groups.clear();
  // connected components of the traces, linked by shared A or B blocks
  std::vector<int> parent(nrows);
  for (int r = 0; r < nrows; r++) parent[r] = r;
  auto find = [&](int x) {
    while (parent[x] != x) x = parent[x] = parent[parent[x]];
    return x;
  };
  {
    std::map<int, int> firsta, firstb;
    for (int r = 0; r < nrows; r++) {
      auto ia = firsta.emplace(rows[r].aoff, r).first;
      parent[find(r)] = find(ia->second);
      auto ib = firstb.emplace(rows[r].boff, r).first;
      parent[find(r)] = find(ib->second);
    }
  }
  std::vector<std::vector<int>> comps;
  {
    std::map<int, int> cix;
    for (int r = 0; r < nrows; r++) {
      auto it = cix.emplace(find(r), (int)comps.size()).first;
      if (it->second == (int)comps.size()) comps.emplace_back();
      comps[it->second].push_back(r);
    }
  }
  int maxcols = 0;
  TraceGroup cur;
  auto reset = [&]() { std::memset(&cur, 0, sizeof(cur)); };
  auto flush = [&]() {
    if (cur.nt > 0) {
      maxcols = std::max(maxcols, cur.na + cur.nb);
      groups.push_back(cur);
    }
    reset();
  };
  auto slot = [](const int* v, int n, int x) {
    for (int k = 0; k < n; k++)
      if (v[k] == x) return k;
    return -1;
  };
  // blocks of a trace list not yet in the current group
  auto need = [&](const std::vector<int>& tl, int& da, int& db) {
    std::vector<int> na_, nb_;
    for (int r : tl) {
      if (slot(cur.aoff, cur.na, rows[r].aoff) < 0 && std::find(na_.begin(), na_.end(), rows[r].aoff) == na_.end())
        na_.push_back(rows[r].aoff);
      if (slot(cur.boff, cur.nb, rows[r].boff) < 0 && std::find(nb_.begin(), nb_.end(), rows[r].boff) == nb_.end())
        nb_.push_back(rows[r].boff);
    }
    da = (int)na_.size();
    db = (int)nb_.size();
  };
  auto add = [&](int r) {
    int a = slot(cur.aoff, cur.na, rows[r].aoff);
    if (a < 0) {
      a = cur.na++;
      cur.aoff[a] = rows[r].aoff;
    }
    int b = slot(cur.boff, cur.nb, rows[r].boff);
    if (b < 0) {
      b = cur.nb++;
      cur.boff[b] = rows[r].boff;
    }
    cur.ta[cur.nt] = a;
    cur.tb[cur.nt] = b;
    cur.tr[cur.nt] = r;
    cur.nt++;
  };
  auto fits = [&](const std::vector<int>& tl) {
    int da, db;
    need(tl, da, db);
    return cur.na + da <= maxa && cur.nb + db <= maxb && cur.nt + (int)tl.size() <= maxt;
  };
  reset();
  for (const std::vector<int>& c : comps) {
    if (!fits(c)) flush();
    if (fits(c)) {
      for (int r : c) add(r);
      continue;
    }
    // a component larger than a group: trace by trace
    for (int r : c) {
      if (!fits({r})) flush();
      add(r);
    }
  }
  flush();
  return maxcols;
}

}  // namespace ctr

extern "C" int ctr_split_available(void) { return 1; }
