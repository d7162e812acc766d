// Shared definitions of the split-precision (BF16-slice tensor-core) engine.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "ctr_internal.h"

namespace ctr {

// Tile geometry (see kernels_split.cu).
constexpr int SPLIT_M = 128;     // rows of an output tile (TMEM lanes)
constexpr int SPLIT_N = 64;      // columns of an output tile (8 accumulators x 64 = 512 TMEM columns)
constexpr int SPLIT_K = 16;      // K of one MMA / one pipeline chunk
constexpr int SPLIT_NSLICE = 5;  // BF16 slices (balanced base-512 digits) per FP64 value
constexpr int SPLIT_MAXK = 128;  // largest Nev the engine takes (exactness bound of the leading level)
constexpr int SPLIT_A_SUB = SPLIT_M * SPLIT_K * 2;                  // one (slice, plane) sub-tile, bytes
constexpr int SPLIT_B_SUB = SPLIT_N * SPLIT_K * 2;
constexpr int SPLIT_B_PLANES = 3;                                   // -im, re, im (packed complex MMAs)
constexpr int SPLIT_A_STAGE = SPLIT_NSLICE * 2 * SPLIT_A_SUB;       // 40960 B: all slices, re+im, one K chunk
constexpr int SPLIT_B_STAGE = SPLIT_NSLICE * SPLIT_B_PLANES * SPLIT_B_SUB;  // 30720 B
constexpr int SPLIT_MAXBLK = 32;

// Kernel configurations: slices per value, TMEM accumulation levels, tile N.
//  * standard (two-sided form, float-float products): 5 slices (15 slice
//    pairs), levels 0, 1, 2 exact and >= 3 in FP32, N = 64 (8 x 64 = 512 TMEM columns);
//  * high precision (task form of the chain diagrams, complex128 products):
//    6 slices (21 slice pairs, 54 bits), levels 0-3 exact and >= 4 in FP32,
//    N = 48 (10 x 48 = 480 TMEM columns); the epilogue sums the levels exactly
//    in 64-bit integers, so products keep ~2^-53 of their row/column scales.
//
// Packed complex MMAs (PACK): the right operand keeps three planes per slice,
// -Yi, Yr, Yi, adjacent along N, so that the complex product takes two MMAs of
// width 2 BN per slice pair, Xr [Yr | Yi] and Xi [-Yi | Yr], into one [Re | Im]
// accumulator per level (instead of four MMAs of width BN); the left operand
// tile is then read from shared memory half as often per flop.
template <int NS_, int NL_, int BN_, bool PACK_, bool INT_OUT_>
struct SplitCfg {
  static constexpr int NS = NS_, NL = NL_, BN = BN_;
  static constexpr bool PACK = PACK_;
  static constexpr bool INT_OUT = INT_OUT_;  // epilogue: complex128 via exact integer sums (else float-float)
  static constexpr int EPI_WARPS = 16;             // 4 per TMEM lane quadrant, splitting the columns
  static constexpr int EPI_CW = 4;                 // columns per TMEM load in the epilogue
  static constexpr int B_PLANES = PACK ? 3 : 2;
  static constexpr int A_SUB = SPLIT_M * SPLIT_K * 2;
  static constexpr int B_SUB = BN * SPLIT_K * 2;
  static constexpr int A_STAGE = NS * 2 * A_SUB;
  static constexpr int B_STAGE = NS * B_PLANES * B_SUB;
  // TMEM column of accumulator (part 0 = Re / 1 = Im, level l)
  __host__ __device__ static constexpr int acc_col(int part, int l) { return PACK ? (l * 2 + part) * BN : (part * NL + l) * BN; }
};
using CfgStd = SplitCfg<SPLIT_NSLICE, 4, SPLIT_N, true, false>;
using CfgHP = SplitCfg<6, 5, 48, true, true>;
static_assert(CfgStd::B_STAGE == SPLIT_B_STAGE && CfgStd::A_STAGE == SPLIT_A_STAGE, "standard stage sizes");
static_assert(CfgStd::BN % (CfgStd::EPI_CW * (CfgStd::EPI_WARPS / 4)) == 0 &&
                  CfgHP::BN % (CfgHP::EPI_CW * (CfgHP::EPI_WARPS / 4)) == 0,
              "epilogue column split");

// Slicing of a stacked operand.  Left: rows r -> row r%nev of blk[r/nev].
struct SliceLeftJob {
  const double2* blk[SPLIT_MAXBLK];
  int rows;        // stacked rows (nblk * nev)
  int pad;
  uint8_t* out;    // [mtiles][nchunk][SPLIT_A_STAGE]
  int* exps;       // [mtiles * SPLIT_M]
};

// Right: columns n -> column n%nev of blk[n/nev].
struct SliceRightJob {
  const double2* blk[SPLIT_MAXBLK];
  int cols;
  int pad;
  uint8_t* out;    // [ntiles][nchunk][SPLIT_B_STAGE]
  int* exps;       // [ntiles * SPLIT_N]
};

struct SplitGemmInst {
  const uint8_t* left;   // sliced left operand (all M tiles)
  const uint8_t* right;  // sliced right operand (all N tiles)
  const int* lexp;       // row exponents
  const int* rexp;       // column exponents
  float4* out;           // out_mode 0: float-float complex, column-major: (r, c) at out[c * ldo + r]
  double2* const* outs;  // out_mode 1: complex128 row-major blocks; column c -> outs[c / blkn], (r, c % blkn)
};

struct SplitGemmBatch {
  const SplitGemmInst* inst;
  int mtiles, ntiles, nchunk;
  int mrows, ncols;  // valid rows / columns of every instance
  int ldo;           // column stride of the output (>= mtiles * SPLIT_M)
  float* levels;     // diagnostics only (NULL in production): raw accumulators
                     // [8][ncols][ldo] of instance 0 instead of the ff output
  int out_mode;      // 0: float-float column-major, 1: complex128 row-major blocks
  int blkn;          // out_mode 1: columns (and row stride) of one output block
  int hp;            // 0: CfgStd operands and tiles, 1: CfgHP (out_mode 1 only)
  int order;         // persistent tile walk: 0 N tiles innermost, 1 M tiles innermost
};

// Operands of the task form C = sum_q w_q op(A_q) op(B_q) (q < nterm <= 4),
// concatenated along K (term q occupies k in [q N, (q+1) N)).  Left: rows of
// the A side with the weights applied; right: up to SPLIT_TASK_NB output blocks
// stacked along N.  dag bit q (left) / bit 4j+q (right): conjugate transpose.
// eplus = 1 halves the leading digit (|d_0| <= 128) so that level 0 stays
// exact for K <= 512.
// The scale exponents come from per-block tables: bi indexes a table of
// [2][nev] ints per distinct block of the launch (row-wise and column-wise
// exponent bounds, launch_block_exp); wexp is the exponent of the power-of-two
// weight w.
constexpr int SPLIT_TASK_NB = 8;
struct SliceTaskLJob {
  const double2* a[4];
  float w[4];
  int bi[4], wexp[4];
  int nterm, dag, eplus, pad;
  uint8_t* out;  // [nchunk][CfgHP::A_STAGE]
  int* exps;     // [SPLIT_M]
};
struct SliceTaskRJob {
  const double2* b[SPLIT_TASK_NB][4];
  int bi[SPLIT_TASK_NB][4];
  int nb, nterm, dag, eplus;
  uint8_t* out;  // [ntiles][nchunk][CfgHP::B_STAGE]
  int* exps;     // [ntiles * CfgHP::BN]
};

// Stacked left operand of a block grid (the task form with M stacking): slab s
// (< nslab) contributes Nev rows of sum_q w_q op(a[s][q]) (terms along K as in
// SliceTaskLJob); the slabs follow one another along M, so an M tile may span
// several slabs.  The weights and transposes are the same for every slab.
constexpr int SPLIT_STACK = 32;
struct SliceStackLJob {
  const double2* a[SPLIT_STACK][4];
  int bi[SPLIT_STACK][4];
  float w[4];
  int wexp[4];
  int nslab, nterm, dag, eplus;
  uint8_t* out;  // [mtiles][nchunk][CfgHP::A_STAGE]
  int* exps;     // [mtiles * SPLIT_M]
};

// Closing trace of one two-sided row: element offsets of its A block (cd, L)
// and B block (ab, R) inside a pair's product matrices, and its coefficient.
struct TraceRow {
  int aoff, boff;
  float coef[2];
};

// A group of closing traces that share product blocks: TG_MAXA source-side (A)
// and TG_MAXB sink-side (B) blocks at most, TG_MAXT traces over them.  Trace k
// of the group is TraceRow tr[k] (also its output slot) and multiplies block
// ta[k] of the A list with block tb[k] of the B list.
constexpr int TG_MAXA = 8, TG_MAXB = 8, TG_MAXT = 16;
struct TraceGroup {
  int na, nb, nt, pad;
  int aoff[TG_MAXA], boff[TG_MAXB];
  int ta[TG_MAXT], tb[TG_MAXT], tr[TG_MAXT];
};

// Closing traces as Gram products.  A group of left blocks X_r (r < mrows) and
// right blocks Y_c (c < ncols) whose traces Tr-Had(X_r, Y_c) = sum_e X_r,e
// conj(Y_c,e) are many is one product G = X' Y'^dagger, X' and Y' the blocks
// flattened into rows of Nev^2 elements.  K runs in pieces of at most
// GRAM_PIECE elements, each an instance of the high-precision GEMM with its own
// row and column scales (the leading digit halved, so that level 0 stays exact
// up to K = 512); the pieces' complex128 partial products are summed per trace.
constexpr int GRAM_PIECE = 512;
struct GramTrace {
  int g, r, c;   // group (of the plan; the launch's first group is subtracted), left row, right column
  int slot;      // output slot: trv[slot], tra[slot]
  float coef[2]; // complex coefficient of the trace
};

// ------------------------------------------------------ float-float helpers
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

// (S, E) += (xh + xl) * (yh + yl), products kept to ~2^-47 relative.
__device__ __forceinline__ void ff_mac(float& S, float& E, float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  float s, t;
  two_sum(S, p, s, t);
  S = s;
  E += t + e;
}

// Slicing of stacked operands.  form 0: one CTA per operand tile, which reads
// the operand once for the scale exponents and once per K chunk; form 1: one
// CTA per quarter tile, which stages its quarter in shared memory (read once).
// Both write the same bytes.
int launch_slice_left(const SliceLeftJob* d_jobs, int njobs, int nev, int nchunk, int mtiles, cudaStream_t s,
                      int form = 0);
int launch_slice_right(const SliceRightJob* d_jobs, int njobs, int nev, int nchunk, int ntiles, cudaStream_t s,
                       int form = 0);
// gram: the launch computes Gram products of closing traces (timed as
// "gram_gemm" and counted apart from the block products' MMA flops).
int launch_split_gemm(const SplitGemmBatch& g, int ninst, int* d_err, cudaStream_t s, bool gram = false);
// Gram operands (high-precision tiles): for instance ip = g * npiece + p and
// tile t, the blocks blk[g * nrows + t * TR + r] (r < TR = 128 left / BN right;
// rows past nrows or null pointers are zero) over elements [p piece,
// (p + 1) piece) of their n2, as nchunk K chunks at out + ((ip * ntile + t) *
// nchunk + kc) * stage; the scale exponent (with the leading digit halved) and
// the 2-norm of (|Re| + |Im|) / 2^E of each row at exps / norms[ip * ntile * TR
// + t * TR + r].  right: the operand is conj(Y) as the right planes
// (-Im, Re, Im) of a K-major B.
int launch_slice_gram(bool right, const double2* const* d_blk, int ngroup, int nrows, int ntile, int n2, int npiece,
                      int nchunk, uint8_t* out, int* exps, float* norms, cudaStream_t s);
// Trace values of a Gram launch whose first group is g0: trv[slot] = coef * sum
// over the pieces of the partial product (r, c) of group g - g0 (instance ip's
// at part + ip * lrows * rcols, row-major
// rcols), tra[slot] (when not null) = |coef| * sum over the pieces of
// (|x_p| |y_p| + 8) 2^(E_x + E_y), a bound of sum |x|_1 |y|_1 and of the slices'
// truncation error (rows or columns of zeros add nothing).
int launch_gram_trace_sum(const GramTrace* d_tr, int ntr, int g0, const double2* part, int npiece, int lrows, int rcols,
                          const int* lexp, const int* rexp, const float* lnorm, const float* rnorm, double2* trv,
                          double* tra, cudaStream_t s);
// A bounded wait that runs out (timeout_ns) on an mbarrier nothing arrives at,
// recording error code 9 in *d_err (the failure-detection check).
int launch_wait_probe(unsigned long long timeout_ns, int* d_err, cudaStream_t s);
// The split GEMM's MMA schedule by itself (ctr_mma_schedule_probe): hp selects
// the high-precision configuration; returns the grid size, MMAs per K chunk and
// the MMAs' N.
int launch_mma_schedule_probe(int hp, int nchunk, unsigned long long* d_cycles, int* d_err, int* nsm, int* mmas_per_chunk,
                              int* mma_n, cudaStream_t s);
// Raises the shared-memory limits of the split kernels and caches the SM count.
int split_kernels_prepare();
// Closing traces over npair pairs: products of pair q at a_base[q] / b_base[q]
// (leading dimensions lda / ldb); rows[q * nrows + r] = coef_r * trace and
// rabs[q * nrows + r] = |coef_r| sum |A|_1 |B|_1.
// variant: 0 one thread per row i walking the columns (128 threads), 1/2/3 the
// flattened element walk with 128/256/512 threads, 4/5/6/7/8 the flattened walk
// with 4/2/4/8/8 independent streams a thread and 128/256/64/64/128 threads
// (TRACE_VARIANTS candidates).
constexpr int TRACE_VARIANTS = 9;
int launch_trace_rows(const TraceRow* d_rows, int nrows, const float4* const* d_abase, const float4* const* d_bbase,
                      int lda, int ldb, int npair, int nev, double2* rows, double* rabs, int variant,
                      cudaStream_t s);
// Grouped closing traces (same results as launch_trace_rows): one CTA per
// (pair, group) streams the columns of the group's blocks into shared memory by
// bulk copies and computes every trace of the group from them, so each block is
// read once per group.  maxcols = the largest na + nb of the groups.
int launch_trace_groups(const TraceGroup* d_groups, int ngroups, int maxcols, const TraceRow* d_rows, int nrows,
                        const float4* const* d_abase, const float4* const* d_bbase, int lda, int ldb, int npair,
                        int nev, double2* rows, double* rabs, int* d_err, cudaStream_t s);
// Quad groups (at most 2 A blocks, 2 B blocks, 4 traces; build_trace_groups
// with limits 2, 2, 4): one CTA per (pair, group) loads each element of the
// group's blocks once into registers for all its traces.  variant 0: 128
// threads x 2 element streams, 1: 64 threads x 4 streams.
int launch_trace_quads(const TraceGroup* d_groups, int ngroups, const TraceRow* d_rows, int nrows,
                       const float4* const* d_abase, const float4* const* d_bbase, int lda, int ldb, int npair,
                       int nev, double2* rows, double* rabs, int variant, cudaStream_t s);
// Builds the groups of a trace list: traces linked by a shared block go to the
// same group where the limits (maxa A blocks, maxb B blocks, maxt traces; at
// most TG_MAXA, TG_MAXB, TG_MAXT) allow.  Returns the largest na + nb.
int build_trace_groups(const TraceRow* rows, int nrows, int maxa, int maxb, int maxt,
                       std::vector<TraceGroup>& groups);
// Task-form slicing: the row and column exponent bounds of every distinct block
// of a launch first (bexp [nblk][2][nev]: bound of row r at [0][r], of column c at
// [1][c]), then the slices of each (operand tile, K chunk), whose scale exponents
// combine those bounds.
int launch_block_exp(const double2* const* d_blk, int nblk, int nev, int* bexp, cudaStream_t s);
int launch_slice_task_left(const SliceTaskLJob* d_jobs, int njobs, int nev, int nchunk, const int* bexp,
                           cudaStream_t s);
int launch_slice_task_right(const SliceTaskRJob* d_jobs, int njobs, int nev, int nchunk, int ntiles, const int* bexp,
                            cudaStream_t s);
// Stacked left operands of block grids: CTA = (job, M tile, K chunk), every job of
// the launch with mtiles M tiles.
int launch_slice_stack_left(const SliceStackLJob* d_jobs, int njobs, int nev, int nchunk, int mtiles, const int* bexp,
                            cudaStream_t s);

}  // namespace ctr
