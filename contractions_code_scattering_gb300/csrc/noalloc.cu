// Allocation-free rho-rho entry point.
//
// Some callers cannot allocate device memory at the point where they want the
// contraction: code running while another component owns the device memory
// budget (a fixed pool or arena handed out at start-up), code that must not
// synchronise the device (cudaMalloc/cudaFree can), or hosts whose allocator is
// locked down.  ctr_rho_noalloc serves them: it computes the same correlators as
// ctr_rho with the plain FP64 engine for one t_sink row, and its only scratch is
// the file-scope device array below, of fixed size, reserved when the library
// is loaded and held by every GPU that loads it until the process exits.  It
// calls no cudaMalloc, cudaFree, cudaMallocHost or any allocating routine; its
// host-side task lists live in fixed static arrays.
#include <cstring>
#include <mutex>

#include "kernels.h"

namespace ctr {

__global__ void zgemm_f64_kernel(const ZTask* __restrict__ tasks, int ntask, int N, int tiles_per_dim);
__global__ void trace_f64_kernel(const TraceTask* __restrict__ tasks, int ntask, int N);
__global__ void rowsum_kernel(const double2* __restrict__ rows, int nrows, const int* __restrict__ off,
                              const int* __restrict__ idx, int nout, int npair, double2* __restrict__ out,
                              size_t out_pair_stride);

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;  // 32 MiB: 160 products of Nev <= 114
constexpr int kProducts = 160;                        // 80 source-side + 80 sink-side blocks of rho
constexpr int kRows = 768;
constexpr int kOut = 48;
constexpr int kMaxDevices = 64;

// The scratch.  In host code this name is only a stand-in for the device
// symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// The diagram tables are built when the library is loaded, so that the entry
// point itself never triggers their (host) construction.
const Tables& g_tables_at_load = tables();

// Fixed host-side staging of one t_source's task lists.
struct HostTasks {
  ZTask gemm[kProducts];
  TraceTask trace[kRows];
  int csr[kOut + 1 + kRows];
};
HostTasks g_host;
std::mutex g_host_mutex;

// Byte layout of the scratch (all offsets 256-aligned).
constexpr size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffGemm = 0;
constexpr size_t kOffTrace = align_up(kOffGemm + sizeof(ZTask) * kProducts);
constexpr size_t kOffCsr = align_up(kOffTrace + sizeof(TraceTask) * kRows);
constexpr size_t kOffRows = align_up(kOffCsr + sizeof(int) * (kOut + 1 + kRows));
constexpr size_t kOffProducts = align_up(kOffRows + sizeof(double2) * kRows);

int scratch_address(void** out) {
  int dev = 0;
  CTR_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(CTR_ERR_UNSUPPORTED, "device index %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lk(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    CTR_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return CTR_OK;
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
  void* base;
  CTR_TRY(scratch_address(&base));
  uint8_t* S = (uint8_t*)base;
  ZTask* d_gemm = (ZTask*)(S + kOffGemm);
  TraceTask* d_trace = (TraceTask*)(S + kOffTrace);
  int* d_csr = (int*)(S + kOffCsr);
  double2* d_rows = (double2*)(S + kOffRows);
  double2* d_prod = (double2*)(S + kOffProducts);

  // distinct source-side (s3,s4,lp) and sink-side (s1,s2,rp) blocks of the rho table
  const Tables& T = tables();
  int keyA[kRows], keyB[kRows];
  int listA[kProducts / 2], listB[kProducts / 2];
  int nA = 0, nB = 0;
  for (int r = 0; r < kRows; r++) {
    const int ka = (T.rho_spin[r][2] * 4 + T.rho_spin[r][3]) * 5 + T.rho_lprp[r][0];
    const int kb = (T.rho_spin[r][0] * 4 + T.rho_spin[r][1]) * 5 + T.rho_lprp[r][1];
    int ia = -1, ib = -1;
    for (int k = 0; k < nA; k++)
      if (listA[k] == ka) ia = k;
    for (int k = 0; k < nB; k++)
      if (listB[k] == kb) ib = k;
    if (ia < 0) {
      if (nA == kProducts / 2) return fail(CTR_ERR_ARG, "ctr_rho_noalloc: table has too many blocks");
      ia = nA;
      listA[nA++] = ka;
    }
    if (ib < 0) {
      if (nB == kProducts / 2) return fail(CTR_ERR_ARG, "ctr_rho_noalloc: table has too many blocks");
      ib = nB;
      listB[nB++] = kb;
    }
    keyA[r] = ia;
    keyB[r] = ib;
  }

  std::lock_guard<std::mutex> lk(g_host_mutex);
  HostTasks& H = g_host;
  for (int o = 0; o <= kOut; o++) H.csr[o] = 16 * o;  // rows of output o: 16*o .. 16*o+15 (table order)
  for (int r = 0; r < kRows; r++) H.csr[kOut + 1 + r] = r;
  CTR_CUDA(cudaMemcpyAsync(d_csr, H.csr, sizeof(H.csr), cudaMemcpyHostToDevice, stream));

  const double2* tau = (const double2*)prop_row;
  const double2* ph = (const double2*)mom5;
  const int tpd = (N + 31) / 32;
  for (int ti = 0; ti < Nt; ti++) {
    const double2* tblk = tau + (size_t)ti * 16 * N2;
    for (int k = 0; k < nA; k++) {
      const int cd = listA[k] / 5, L = listA[k] % 5;
      ZTask& z = H.gemm[k];
      std::memset(&z, 0, sizeof(z));
      z.A[0] = tblk + (size_t)cd * N2;
      z.B[0] = ph + ((size_t)ti * 5 + L) * N2;
      z.C = d_prod + (size_t)k * N2;
      z.wre[0] = 1.f;
      z.nterm = 1;
    }
    for (int k = 0; k < nB; k++) {
      const int ab = listB[k] / 5, R = listB[k] % 5;
      ZTask& z = H.gemm[nA + k];
      std::memset(&z, 0, sizeof(z));
      z.A[0] = ph + ((size_t)tf * 5 + R) * N2;
      z.B[0] = tblk + (size_t)ab * N2;
      z.C = d_prod + (size_t)(nA + k) * N2;
      z.wre[0] = 1.f;
      z.nterm = 1;
    }
    for (int r = 0; r < kRows; r++) {
      TraceTask& t = H.trace[r];
      std::memset(&t, 0, sizeof(t));
      t.X = d_prod + (size_t)keyA[r] * N2;
      t.Y = d_prod + (size_t)(nA + keyB[r]) * N2;
      t.out = d_rows + r;
      t.coef[0] = T.rho_coef[r][0];
      t.coef[1] = T.rho_coef[r][1];
      t.mode = 0;
    }
    // Pageable-source copies: the runtime stages the host data before returning,
    // so the static host arrays can be refilled for the next t_source at once.
    CTR_CUDA(cudaMemcpyAsync(d_gemm, H.gemm, sizeof(ZTask) * (nA + nB), cudaMemcpyHostToDevice, stream));
    CTR_CUDA(cudaMemcpyAsync(d_trace, H.trace, sizeof(TraceTask) * kRows, cudaMemcpyHostToDevice, stream));
    zgemm_f64_kernel<<<(nA + nB) * tpd * tpd, 256, 0, stream>>>(d_gemm, nA + nB, N, tpd);
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
  CTR_NO_CAPTURE("ctr_rho_noalloc");
  if (nev < 1 || nt < 1 || tf < 0 || tf >= nt || !prop_row || !mom5 || !corr)
    return ctr::fail(CTR_ERR_ARG, "ctr_rho_noalloc: bad arguments");
  if (((uintptr_t)prop_row | (uintptr_t)mom5 | (uintptr_t)corr) & 15)
    return ctr::fail(CTR_ERR_ARG, "ctr_rho_noalloc: device pointers must be 16-byte aligned");
  return ctr::rho_noalloc(nev, nt, tf, prop_row, mom5, corr, (cudaStream_t)stream);
}

extern "C" size_t ctr_rho_noalloc_scratch_bytes(void) { return ctr::noalloc_scratch_bytes(); }
