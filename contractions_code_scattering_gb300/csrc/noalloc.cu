// Allocation-free rho-rho entry point.
//
// Some callers cannot allocate device memory at the point where they want the
// contraction: code running while another component owns the device memory
// budget (a fixed pool or arena handed out at start-up), code that must not
// synchronise the device (cudaMalloc/cudaFree can), or hosts whose allocator is
// locked down.  ctr_rho_noalloc serves them: it computes the same correlators as
// ctr_rho with the plain FP64 engine for one t_sink row, and its only scratch is
// the file-scope device array below, of fixed size.  That array lives in this
// file's device module: a device reserves it when the module is loaded there,
// which under CUDA's default lazy module loading happens at the latest in the
// first call on that device, and keeps it until the process exits.
//
// Nothing is allocated and nothing is copied from the host: the call's plan
// (which blocks to multiply, which traces to take, how rows sum into outputs)
// is built once, when the library is loaded, into a host struct that every
// launch passes by value as a kernel parameter; a small kernel then writes the
// per-source-time task lists into the scratch array.
#include <cstring>

#include "kernels.h"

namespace ctr {

__global__ void zgemm_f64_kernel(const ZTask* __restrict__ tasks, int ntask, int N, int tiles_per_dim);
__global__ void trace_f64_kernel(const TraceTask* __restrict__ tasks, int ntask, int N);
__global__ void rowsum_kernel(const double2* __restrict__ rows, int nrows, const int* __restrict__ off,
                              const int* __restrict__ idx, int nout, int npair, double2* __restrict__ out,
                              size_t out_pair_stride);

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;  // 32 MiB: 160 products of Nev <= 114
constexpr int kHalf = 80;                             // distinct source-side (and sink-side) blocks of rho
constexpr int kProducts = 2 * kHalf;
constexpr int kRows = 768;
constexpr int kOut = 48;

// The scratch.  In host code this name is only a stand-in for the device
// symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The rho table in the form the task kernel reads: product keys, the products
// each row multiplies, its coefficient, and the rows of every output.  Output o
// of the reference's host reduction is rows 16*o .. 16*o+15 (the row index is
// (op pair*3 + direction)*16 + spin term, lib/contract_kernels_rho.cu:108-116),
// the same rule ctr_rho uses.  About 11 kB, passed by value to every launch.
struct Plan {
  int16_t a_key[kHalf];  // source-side product k: tau(tf,ti)_{cd} Phi_L(ti), key cd*5 + L
  int16_t b_key[kHalf];  // sink-side product k: Phi_R(tf) tau(tf,ti)_{ab}, key ab*5 + R
  int16_t row_a[kRows], row_b[kRows];
  float2 coef[kRows];
  int32_t csr[kOut + 1 + kRows];
  int nA, nB;
};

Plan make_plan(int* status) {
  Plan P;
  std::memset(&P, 0, sizeof(P));
  const Tables& T = tables();
  *status = CTR_OK;
  for (int r = 0; r < kRows; r++) {
    const int ka = (T.rho_spin[r][2] * 4 + T.rho_spin[r][3]) * 5 + T.rho_lprp[r][0];
    const int kb = (T.rho_spin[r][0] * 4 + T.rho_spin[r][1]) * 5 + T.rho_lprp[r][1];
    int ia = -1, ib = -1;
    for (int k = 0; k < P.nA; k++)
      if (P.a_key[k] == ka) ia = k;
    for (int k = 0; k < P.nB; k++)
      if (P.b_key[k] == kb) ib = k;
    if ((ia < 0 && P.nA == kHalf) || (ib < 0 && P.nB == kHalf)) {
      *status = CTR_ERR_UNSUPPORTED;
      return P;
    }
    if (ia < 0) {
      ia = P.nA;
      P.a_key[P.nA++] = (int16_t)ka;
    }
    if (ib < 0) {
      ib = P.nB;
      P.b_key[P.nB++] = (int16_t)kb;
    }
    P.row_a[r] = (int16_t)ia;
    P.row_b[r] = (int16_t)ib;
    P.coef[r] = make_float2(T.rho_coef[r][0], T.rho_coef[r][1]);
  }
  // Output r / 16 is the reference's rule; the table must agree with it: the 16
  // spin rows of an output share one operator pair (lp, rp).  A table that
  // breaks this is refused rather than summed into the wrong outputs.
  for (int r = 0; r < kRows; r++)
    if (T.rho_lprp[r][0] != T.rho_lprp[r & ~15][0] || T.rho_lprp[r][1] != T.rho_lprp[r & ~15][1]) {
      *status = CTR_ERR_UNSUPPORTED;
      return P;
    }
  // CSR of the outputs: counts by output index r / 16, then rows in ascending order
  int cnt[kOut] = {};
  for (int r = 0; r < kRows; r++) cnt[r / 16]++;
  P.csr[0] = 0;
  for (int o = 0; o < kOut; o++) P.csr[o + 1] = P.csr[o] + cnt[o];
  int fill[kOut];
  for (int o = 0; o < kOut; o++) fill[o] = P.csr[o];
  for (int r = 0; r < kRows; r++) P.csr[kOut + 1 + fill[r / 16]++] = r;
  return P;
}

// Built when the library is loaded, so that the entry point itself runs no
// host-side construction (and no allocation) of its own.
int g_plan_status = CTR_OK;
const Plan g_plan = make_plan(&g_plan_status);

// Byte layout of the scratch (all offsets 256-aligned).
constexpr size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffGemm = 0;
constexpr size_t kOffTrace = align_up(kOffGemm + sizeof(ZTask) * kProducts);
constexpr size_t kOffCsr = align_up(kOffTrace + sizeof(TraceTask) * kRows);
constexpr size_t kOffRows = align_up(kOffCsr + sizeof(int) * (kOut + 1 + kRows));
constexpr size_t kOffProducts = align_up(kOffRows + sizeof(double2) * kRows);

// Task lists of one (t_sink, t_source) pair, written into the scratch.
__global__ void noalloc_tasks_kernel(const Plan P, int N, int tf, int ti, const double2* __restrict__ tau_row,
                                     const double2* __restrict__ ph, unsigned char* __restrict__ S) {
  ZTask* gemm = (ZTask*)(S + kOffGemm);
  TraceTask* trace = (TraceTask*)(S + kOffTrace);
  int* csr = (int*)(S + kOffCsr);
  double2* rows = (double2*)(S + kOffRows);
  double2* prod = (double2*)(S + kOffProducts);
  const size_t N2 = (size_t)N * N;
  const double2* tblk = tau_row + (size_t)ti * 16 * N2;
  for (int i = threadIdx.x; i < P.nA + P.nB; i += blockDim.x) {
    ZTask z;
    for (int q = 0; q < 4; q++) {
      z.A[q] = nullptr;
      z.B[q] = nullptr;
      z.wre[q] = 0.f;
      z.wim[q] = 0.f;
    }
    if (i < P.nA) {  // tau_{cd} Phi_L(ti)
      const int cd = P.a_key[i] / 5, L = P.a_key[i] % 5;
      z.A[0] = tblk + (size_t)cd * N2;
      z.B[0] = ph + ((size_t)ti * 5 + L) * N2;
    } else {  // Phi_R(tf) tau_{ab}
      const int ab = P.b_key[i - P.nA] / 5, R = P.b_key[i - P.nA] % 5;
      z.A[0] = ph + ((size_t)tf * 5 + R) * N2;
      z.B[0] = tblk + (size_t)ab * N2;
    }
    z.C = prod + (size_t)i * N2;
    z.wre[0] = 1.f;
    z.nterm = 1;
    z.flags = 0;
    gemm[i] = z;
  }
  for (int r = threadIdx.x; r < kRows; r += blockDim.x) {
    TraceTask t;
    t.X = prod + (size_t)P.row_a[r] * N2;
    t.Y = prod + (size_t)(P.nA + P.row_b[r]) * N2;
    t.out = rows + r;
    t.absout = nullptr;
    t.coef[0] = P.coef[r].x;
    t.coef[1] = P.coef[r].y;
    t.mode = 0;
    t.pad = 0;
    trace[r] = t;
  }
  for (int k = threadIdx.x; k < kOut + 1 + kRows; k += blockDim.x) csr[k] = P.csr[k];
}

}  // namespace

size_t noalloc_scratch_bytes() { return kScratchBytes; }

int rho_noalloc(int N, int Nt, int tf, const double* prop_row, const double* mom5, double* corr,
                cudaStream_t stream) {
  const size_t N2 = (size_t)N * N;
  const size_t need = kOffProducts + (size_t)kProducts * N2 * sizeof(double2);
  if (need > kScratchBytes)
    return fail(CTR_ERR_ARG, "ctr_rho_noalloc: Nev=%d needs %zu bytes of scratch, the fixed maximum is %zu (Nev <= 114)",
                N, need, kScratchBytes);
  if (g_plan_status != CTR_OK) return fail(g_plan_status, "ctr_rho_noalloc: the rho table does not fit the fixed plan (too many blocks, or an output whose 16 rows mix operator pairs)");
  // Looked up on every call: cheap once the module is loaded, and never stale
  // after a cudaDeviceReset (which reloads the module elsewhere).
  void* base = nullptr;
  CTR_CUDA(cudaGetSymbolAddress(&base, g_noalloc_scratch));
  unsigned char* S = (unsigned char*)base;
  const ZTask* d_gemm = (const ZTask*)(S + kOffGemm);
  const TraceTask* d_trace = (const TraceTask*)(S + kOffTrace);
  const int* d_csr = (const int*)(S + kOffCsr);
  const double2* d_rows = (const double2*)(S + kOffRows);
  const double2* tau = (const double2*)prop_row;
  const double2* ph = (const double2*)mom5;
  const int nprod = g_plan.nA + g_plan.nB;
  const int tpd = (N + 31) / 32;
  for (int ti = 0; ti < Nt; ti++) {
    noalloc_tasks_kernel<<<1, 256, 0, stream>>>(g_plan, N, tf, ti, tau, ph, S);
    CTR_CUDA(cudaGetLastError());
    zgemm_f64_kernel<<<nprod * tpd * tpd, 256, 0, stream>>>(d_gemm, nprod, N, tpd);
    CTR_CUDA(cudaGetLastError());
    trace_f64_kernel<<<kRows, 256, 0, stream>>>(d_trace, kRows, N);
    CTR_CUDA(cudaGetLastError());
    rowsum_kernel<<<1, 64, 0, stream>>>(d_rows, kRows, d_csr, d_csr + kOut + 1, kOut, 1,
                                        (double2*)corr + (size_t)ti * kOut, kOut);
    CTR_CUDA(cudaGetLastError());
  }
  return CTR_OK;
}

}  // namespace ctr

extern "C" int ctr_rho_noalloc(int nev, int nt, int tf, const double* prop_row, const double* mom5, double* corr,
                               void* stream) {
  if (ctr::capturing())
    return ctr::fail(CTR_ERR_UNSUPPORTED, "ctr_rho_noalloc is not available while this thread records with "
                     "ctr_graph_begin/ctr_graph_end");
  if (nev < 1 || nt < 1 || tf < 0 || tf >= nt || !prop_row || !mom5 || !corr)
    return ctr::fail(CTR_ERR_ARG, "ctr_rho_noalloc: bad arguments");
  if (((uintptr_t)prop_row | (uintptr_t)mom5 | (uintptr_t)corr) & 15)
    return ctr::fail(CTR_ERR_ARG, "ctr_rho_noalloc: device pointers must be 16-byte aligned");
  return ctr::rho_noalloc(nev, nt, tf, prop_row, mom5, corr, (cudaStream_t)stream);
}

extern "C" size_t ctr_rho_noalloc_scratch_bytes(void) { return ctr::noalloc_scratch_bytes(); }
