// Device-side types and launchers shared by the engines.
#pragma once

#include <cuda_runtime.h>

#include "ctr_internal.h"

namespace ctr {

// One block GEMM task of the FP64 engine: C = sum_q w_q op(A_q) op(B_q).
struct ZTask {
  const double2* A[4];
  const double2* B[4];
  double2* C;
  float wre[4], wim[4];
  int nterm;
  int flags;  // bit q: conj-transpose A_q; bit 4+q: conj-transpose B_q
};

// One Hadamard trace: *out = coef * sum X (.) conj(Y)   (mode 0)
//                      *out = coef * Tr[X Y]            (mode 1)
// and, if absout is set, *absout = |coef| * sum |X_ij|_1 |Y_ij|_1 (mode 0) or
// |coef| * sum |X_ij|_1 |Y_ji|_1 (mode 1), |z|_1 = |Re z| + |Im z| (within a factor
// 2 of the product of moduli): the scale of the trace's rounding errors.
struct TraceTask {
  const double2* X;
  const double2* Y;
  double2* out;
  double* absout;
  float coef[2];
  int mode;
  int pad;
};

__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// c += a b as four FMAs into the accumulator (the FP64 pipe is the bound of
// every caller)
__device__ inline void cmac(double2& c, double2 a, double2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}

// Sum over a 256-thread block with a fixed reduction tree (deterministic).
__device__ inline double block_sum_256(double v) {
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; w++) r += red[w];
  return r;  // valid in thread 0
}

// h_tasks: the same tasks on the host (optional); it lets the launcher check
// that the weights allow the DMMA form.
int launch_zgemm_f64(const ZTask* d_tasks, int ntask, int N, cudaStream_t s, const ZTask* h_tasks = nullptr);
int launch_trace_f64(const TraceTask* d_tasks, int ntask, int N, cudaStream_t s);
int launch_rowsum(const double2* rows, int nrows, const int* off, const int* idx, int nout, int npair,
                  double2* out, size_t out_pair_stride, cudaStream_t s);
int launch_source_average(int Nt, int ncorr, const double2* corr, double scale, double2* avg, cudaStream_t s);
// Row sums as launch_rowsum (out stride nout) plus per-entry refinement flags:
// entries with eps_over_tol * sum(rabs) > |out| append (pair_base + p) * nout + o to list.
int launch_rowsum_refine(const double2* rows, const double* rabs, int nrows, const int* off, const int* idx, int nout,
                         int npair, double2* out, double eps_over_tol, int* count, int* list, int pair_base,
                         cudaStream_t s);
// Row sums over shared traces: out[p][o] = sum over rows r of output o (CSR off/idx) of
// coef[r] * tr[p][tix[r]]; the error scale sum |coef[r]| trabs[p][tix[r]] flags entries
// as launch_rowsum_refine does.
int launch_rowsum_coef_refine(const double2* tr, const double* trabs, int ntr, const int* off, const int* idx,
                              const int* tix, const float* coef, int nout, int npair, double2* out,
                              double eps_over_tol, int* count, int* list, int pair_base, cudaStream_t s);
// Scatter: out[where[i]] = vals[i].
int launch_scatter(const int* where, const double2* vals, int n, double2* out, cudaStream_t s);

}  // namespace ctr
