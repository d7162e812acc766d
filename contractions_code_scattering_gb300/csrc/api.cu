// Reference-compatible C++ API (include/interface.h, include/contract.h) over
// the C ABI, plus the host-level C entry points it is built on
// (ctr_read_prop, ctr_read_momenta, ctr_calculate_*), which return status
// codes instead of terminating.
//
// Each calculate* call: uploads the host perambulator (widening float data on
// the device for SINGLE), re-lays the elementals from the caller's [op][t]
// order into [t][op] (lib/interface.cpp:20-26), runs the engine over all
// (t_sink, t_src) pairs, averages over source times on the device and appends
// the reference's text blocks to the output file.
#include <cuda_runtime.h>
#include <sys/time.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "contract.h"
#include "ctr_internal.h"
#include "interface.h"

namespace contract {
int i_dir = 0;
}

namespace ctr {
namespace {

bool g_on = false;
int g_nev = 0, g_nt = 0, g_dev = 0;

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t bytes) {
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    return CTR_OK;
  }
  double* d() const { return (double*)p; }
};

// File order [s1][v1][t1][s2][v2][t2] -> library order [t1][t2][s1][s2][v1][v2]
// (lib/contract.cpp:524-534).  For fixed (s1, v1, t1, s2) this is a transpose of
// the [v2][t2] plane; 32x32 tiles through shared memory keep both sides coalesced.
template <typename OutT>
__global__ void reorder_prop_kernel(const double2* __restrict__ in, OutT* __restrict__ out, int N, int Nt) {
  __shared__ double2 tile[32][33];
  const int tiles_t = (Nt + 31) / 32;
  const int t0 = (blockIdx.y % tiles_t) * 32, v0 = (blockIdx.y / tiles_t) * 32;
  int rest = blockIdx.x;  // ((s1*N + v1)*Nt + t1)*4 + s2
  const int s2 = rest % 4;
  rest /= 4;
  const int t1 = rest % Nt;
  rest /= Nt;
  const int v1 = rest % N;
  const int s1 = rest / N;
  const size_t in_base = (size_t)blockIdx.x * N * Nt;  // + v2*Nt + t2
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int v2 = v0 + r, t2 = t0 + threadIdx.x;
    if (v2 < N && t2 < Nt) tile[r][threadIdx.x] = in[in_base + (size_t)v2 * Nt + t2];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int t2 = t0 + r, v2 = v0 + threadIdx.x;
    if (v2 < N && t2 < Nt) {
      const size_t o = (((((size_t)t1 * Nt + t2) * 4 + s1) * 4 + s2) * N + v1) * N + v2;
      const double2 v = tile[threadIdx.x][r];
      out[2 * o] = (OutT)v.x;
      out[2 * o + 1] = (OutT)v.y;
    }
  }
}

__global__ void widen_kernel(const float* __restrict__ src, double* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// Upload the host perambulator [Nt][Nt][16][N][N] complex (float or double) as complex128.
int upload_prop(const void* prop, bool single, int N, int Nt, DevBuf& out) {
  const size_t n = (size_t)Nt * Nt * 16 * N * N * 2;  // reals
  CTR_TRY(out.alloc(n * sizeof(double)));
  if (!single) {
    CTR_CUDA(cudaMemcpy(out.p, prop, n * sizeof(double), cudaMemcpyHostToDevice));
    return CTR_OK;
  }
  DevBuf tmp;
  CTR_TRY(tmp.alloc(n * sizeof(float)));
  CTR_CUDA(cudaMemcpy(tmp.p, prop, n * sizeof(float), cudaMemcpyHostToDevice));
  widen_kernel<<<1024, 256>>>((const float*)tmp.p, out.d(), n);
  CTR_CUDA(cudaGetLastError());
  CTR_CUDA(cudaDeviceSynchronize());
  return CTR_OK;
}

// Host elementals [nop][Nt][N][N] (caller order) -> device [Nt][nop][N][N].
int upload_moms(const double* mom, int nop, const int* op_sel, int N, int Nt, DevBuf& out) {
  const size_t blk = (size_t)N * N * 2;
  std::vector<double> h((size_t)Nt * nop * blk);
  for (int t = 0; t < Nt; t++)
    for (int k = 0; k < nop; k++)
      std::memcpy(&h[((size_t)t * nop + k) * blk], mom + ((size_t)op_sel[k] * Nt + t) * blk, blk * sizeof(double));
  CTR_TRY(out.alloc(h.size() * sizeof(double)));
  CTR_CUDA(cudaMemcpy(out.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
  return CTR_OK;
}

int upload_plain(const double* mom, int N, int Nt, DevBuf& out) {
  const size_t n = (size_t)Nt * N * N * 2;
  CTR_TRY(out.alloc(n * sizeof(double)));
  CTR_CUDA(cudaMemcpy(out.p, mom, n * sizeof(double), cudaMemcpyHostToDevice));
  return CTR_OK;
}

int prop_diag(const DevBuf& prop, int N, int Nt, DevBuf& diag) {
  const size_t blk = (size_t)16 * N * N * 2 * sizeof(double);
  CTR_TRY(diag.alloc(Nt * blk));
  for (int t = 0; t < Nt; t++)
    CTR_CUDA(cudaMemcpy((char*)diag.p + t * blk, (const char*)prop.p + ((size_t)t * Nt + t) * blk, blk,
                        cudaMemcpyDeviceToDevice));
  return CTR_OK;
}

// Source-time average on the device, returned on the host: [Nt][ncorr] complex.
int averaged(const DevBuf& corr, int Nt, int ncorr, std::vector<double>& avg) {
  DevBuf d;
  CTR_TRY(d.alloc((size_t)Nt * ncorr * 16));
  CTR_TRY(ctr_source_average(Nt, ncorr, corr.d(), 1.0, d.d(), nullptr));
  avg.resize((size_t)Nt * ncorr * 2);
  CTR_CUDA(cudaMemcpy(avg.data(), d.p, avg.size() * sizeof(double), cudaMemcpyDeviceToHost));
  return CTR_OK;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

int open_out(const char* path, File& F) {
  F.f = std::fopen(path, "a");
  if (!F.f) return fail(CTR_ERR_IO, "cannot open %s for writing results", path);
  return CTR_OK;
}

double now() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + tv.tv_usec * 1e-6;
}

void report(double t0, double flops, bool single) {
  const double dt = now() - t0;
  printf("Elapsed time is %lf sec, kernel performance is %lf GFlops in %s precision\n", dt, flops / dt / 1e9,
         single ? "single" : "double");
}

int check_on(int nev, int nt) {
  if (!g_on) return fail(CTR_ERR_ARG, "the contraction library is not initialised (call initContract)");
  if (nev != g_nev || nt != g_nt)
    return fail(CTR_ERR_ARG, "call sizes (Nev=%d, Nt=%d) differ from initContract (%d, %d)", nev, nt, g_nev, g_nt);
  return CTR_OK;
}

inline int engine_of(int single) { return single ? CTR_ENGINE_SPLIT : CTR_ENGINE_FP64; }

// Reference per-call flop accounting: spin rows x (products x 8 N^3 + trace 8 N^2), Nt^2 pairs
// (lib/interface.cpp:33-39 and the other calculate* bodies).
double flops_rows(double rows, double nprod, int N, int Nt) {
  const double n = N;
  return rows * (nprod * 8.0 * n * n * n + 8.0 * n * n) * Nt * Nt;
}

}  // namespace

bool contract_state(int* nev, int* nt) {
  if (nev) *nev = g_nev;
  if (nt) *nt = g_nt;
  return g_on;
}

// lib/contract.cpp:633-638
void dump_rho(FILE* f, const double* a, int nt) {
  for (int iop = 0; iop < 16; iop++)
    for (int it = 0; it < nt; it++) {
      const double* c = &a[((size_t)it * 48 + iop * 3) * 2];
      fprintf(f, "%d %d \t %+e %+e \t %+e %+e \t %+e %+e\n", iop, it, c[0], c[1], c[2], c[3], c[4], c[5]);
    }
  fprintf(f, "\n");
  fflush(f);
}

// lib/contract.cpp:720-722 (printed x2; the label is the option parser's i_dir)
void dump_rhopi(FILE* f, const double* a, int nt) {
  for (int iop = 0; iop < 4; iop++)
    for (int it = 0; it < nt; it++)
      fprintf(f, "%d %d %d \t %+e %+e\n", iop, contract::i_dir, it, 2 * a[(it * 4 + iop) * 2], 2 * a[(it * 4 + iop) * 2 + 1]);
  fprintf(f, "\n");
  fflush(f);
}

// lib/contract.cpp:815-835
void dump_pipi(FILE* f, const double* a, int nt, int isospin) {
  const char* label[5] = {"Square", "DoubleTriangle", "Star", "Fish", "DoubleTriangle_Hor"};
  for (int k = 0; k < (isospin == 0 ? 5 : 4); k++) {
    for (int it = 0; it < nt; it++)
      fprintf(f, "%s: %d \t %+e %+e\n", label[k], it, a[(it * 5 + k) * 2], a[(it * 5 + k) * 2 + 1]);
    fprintf(f, "\n");
  }
  fflush(f);
}

// lib/contract.cpp:874-878
void dump_loop(FILE* f, const double* l, int nt) {
  for (int it = 0; it < nt; it++) fprintf(f, "loop: %d \t %+e %+e\n", it, l[it * 2], l[it * 2 + 1]);
  fprintf(f, "\n");
  fflush(f);
}

// lib/contract.cpp:940-944: printed as -C
void dump_sigma(FILE* f, const double* a, int nt) {
  for (int iop = 0; iop < 4; iop++)
    for (int it = 0; it < nt; it++)
      fprintf(f, "twop: %d %d \t %+e %+e\n", iop, it, -a[(it * 4 + iop) * 2], -a[(it * 4 + iop) * 2 + 1]);
  fprintf(f, "\n");
  fflush(f);
}

// lib/contract.cpp:1019-1025
void dump_fish_hor(FILE* f, const double* hf, int nt) {
  for (int it = 0; it < nt; it++) fprintf(f, "fish_hor: %d \t %+e %+e\n", it, hf[it * 2], hf[it * 2 + 1]);
  fprintf(f, "\n");
  fflush(f);
}

// lib/contract.cpp:1043-1048: scaled by -2/sqrt(6)
void dump_triangle(FILE* f, const double* a, int nt) {
  const double w = -2. / std::sqrt(6.);
  for (int iop = 0; iop < 2; iop++)
    for (int it = 0; it < nt; it++)
      fprintf(f, "triangle: %d %d \t %+e %+e\n", iop, it, w * a[(it * 2 + iop) * 2], w * a[(it * 2 + iop) * 2 + 1]);
  fprintf(f, "\n");
  fflush(f);
}

// File payload (host, complex128, file order) -> host_out in the library layout,
// transposed on the device.
int reorder_prop_device(int N, int Nt, const double* file_payload, int single, void* host_out) {
  const size_t n = (size_t)Nt * Nt * 16 * N * N;
  DevBuf din, dout;
  CTR_TRY(din.alloc(n * 16));
  CTR_TRY(dout.alloc(n * (single ? 8 : 16)));
  CTR_CUDA(cudaMemcpy(din.p, file_payload, n * 16, cudaMemcpyHostToDevice));
  const long long planes = 4LL * N * Nt * 4;
  const long long tiles = (long long)((Nt + 31) / 32) * ((N + 31) / 32);
  if (planes > 0x7fffffffLL || tiles > 65535) return fail(CTR_ERR_ARG, "perambulator too large for the reorder grid");
  dim3 grid((unsigned)planes, (unsigned)tiles);
  {
    TimedLaunch tl(nullptr, "reorder_prop");
    if (single)
      reorder_prop_kernel<float><<<grid, dim3(32, 8)>>>((const double2*)din.p, (float*)dout.p, N, Nt);
    else
      reorder_prop_kernel<double><<<grid, dim3(32, 8)>>>((const double2*)din.p, (double*)dout.p, N, Nt);
    CTR_CUDA(cudaGetLastError());
  }
  CTR_CUDA(cudaMemcpy(host_out, dout.p, n * (single ? 8 : 16), cudaMemcpyDeviceToHost));
  return CTR_OK;
}

}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_contract_init(int nev, int nt, int dev) {
  CTR_NO_CAPTURE("ctr_contract_init");
  if (g_on) return fail(CTR_ERR_ARG, "initContract can be called once only");
  if (nev < 1 || nt < 1) return fail(CTR_ERR_ARG, "Nev=%d, Nt=%d invalid", nev, nt);
  CTR_TRY(ctr_device_init(dev));
  g_nev = nev;
  g_nt = nt;
  g_dev = dev;
  g_on = true;
  return CTR_OK;
}

int ctr_contract_destroy(void) {
  CTR_NO_CAPTURE("ctr_contract_destroy");
  if (!g_on) return fail(CTR_ERR_ARG, "cannot destroy contract library because is not on");
  ctr_release_workspace();
  compat_release();
  g_on = false;
  return CTR_OK;
}

// Perambulator file -> host buffer [t1][t2][s1][s2][v1][v2] complex (lib/contract.cpp:91-160).
int ctr_read_prop(const char* path, int nev, int nt, int single, void* host_out) {
  CTR_NO_CAPTURE("ctr_read_prop");
  if (!path || !host_out || nev < 1 || nt < 1) return fail(CTR_ERR_ARG, "ctr_read_prop: bad arguments");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(CTR_ERR_IO, "cannot find file %s for reading the perambulator", path);
  char cfg[100];
  uint32_t hnt = 0, hnv = 0;
  size_t got = std::fread(cfg, 1, 100, f);
  got += std::fread(&hnt, 4, 1, f) * 4;
  got += std::fread(&hnv, 4, 1, f) * 4;
  if (got != 108) {
    std::fclose(f);
    return fail(CTR_ERR_IO, "%s: truncated header", path);
  }
  cfg[99] = 0;
  if ((int)hnv != nev) {
    std::fclose(f);
    return fail(CTR_ERR_IO, "NeV given (%d) is not equal with what the file holds (%u)", nev, hnv);
  }
  if ((int)hnt != nt) {
    std::fclose(f);
    return fail(CTR_ERR_IO, "Nt given (%d) is not equal with what the file holds (%u)", nt, hnt);
  }
  const size_t n = (size_t)nt * nt * 16 * nev * nev;  // complex elements
  std::vector<double> buf(n * 2);
  const size_t r = std::fread(buf.data(), 16, n, f);
  std::fclose(f);
  if (r != n) return fail(CTR_ERR_IO, "%s: did not read the expected size (%zu of %zu elements)", path, r, n);
  CTR_TRY(reorder_prop_device(nev, nt, buf.data(), single, host_out));
  return CTR_OK;
}

// Momentum list (lib/catchOpts.cpp:108-233): momcomb lines of nmom*3 integers.
// For nmom = 2 the third momentum is p1 + p2.  p: [4][3][momcomb] (momentum, component, line).
int ctr_read_momenta(const char* path, int nmom, int momcomb, int* p) {
  if (!path || !p) return fail(CTR_ERR_ARG, "ctr_read_momenta: null argument");
  if (nmom != 1 && nmom != 2 && nmom != 4) return fail(CTR_ERR_ARG, "Only 1,2,4 momenta are allowed");
  if (momcomb < 1) return fail(CTR_ERR_ARG, "At least one momentum combination is needed");
  std::ifstream fp(path);
  if (!fp) return fail(CTR_ERR_IO, "cannot open momentum list %s", path);
  std::vector<std::string> lines;
  std::string line;
  while (std::getline(fp, line)) lines.push_back(line);
  // a final line without a newline still counts; an empty last line does not
  if (!lines.empty() && lines.back().empty()) lines.pop_back();
  if ((int)lines.size() != momcomb)
    return fail(CTR_ERR_IO, "Number of lines in the file (%zu) is not in agreement with the number of momentum "
                "combinations (%d)", lines.size(), momcomb);
  {
    std::stringstream is(lines[0]);
    int v, nc = 0;
    while (is >> v) nc++;
    if (nc != nmom * 3)
      return fail(CTR_ERR_IO, "Number of columns in the file (%d) is not in agreement with the number of momenta (%d)",
                  nc, nmom);
  }
  std::memset(p, 0, sizeof(int) * 12 * momcomb);
  for (int i = 0; i < momcomb; i++) {
    std::stringstream is(lines[i]);
    const int nread = nmom == 2 ? 2 : nmom;
    for (int m = 0; m < nread; m++)
      for (int c = 0; c < 3; c++)
        if (!(is >> p[(m * 3 + c) * momcomb + i]))
          return fail(CTR_ERR_IO, "line %d of %s: expected %d integers", i + 1, path, nmom * 3);
    if (nmom == 2)
      for (int c = 0; c < 3; c++) p[(2 * 3 + c) * momcomb + i] = p[(0 * 3 + c) * momcomb + i] + p[(1 * 3 + c) * momcomb + i];
  }
  return CTR_OK;
}

int ctr_calculate_rho(int nev, int nt, const void* prop, const double* mom, int single, const char* outfile) {
  CTR_NO_CAPTURE("ctr_calculate_rho");
  CTR_TRY(check_on(nev, nt));
  File F;
  CTR_TRY(open_out(outfile, F));
  const double t0 = now();
  DevBuf dp, dm, dc;
  CTR_TRY(upload_prop(prop, single, nev, nt, dp));
  const int ops[5] = {0, 1, 2, 3, 4};
  CTR_TRY(upload_moms(mom, 5, ops, nev, nt, dm));
  CTR_TRY(dc.alloc((size_t)nt * nt * 48 * 16));
  CTR_TRY(ctr_rho(engine_of(single), nev, nt, 0, nt, dp.d(), dm.d(), dc.d(), nullptr));
  CTR_TRY(ctr_sync(nullptr));
  std::vector<double> a;
  CTR_TRY(averaged(dc, nt, 48, a));
  dump_rho(F.f, a.data(), nt);
  report(t0, flops_rows(768, 2, nev, nt), single);
  return CTR_OK;
}

int ctr_calculate_rhopi(int idir, int nev, int nt, const void* prop, const double* p1, const double* p2,
                        const double* p1p2, int single, const char* outfile) {
  CTR_NO_CAPTURE("ctr_calculate_rhopi");
  CTR_TRY(check_on(nev, nt));
  File F;
  CTR_TRY(open_out(outfile, F));
  const double t0 = now();
  DevBuf dp, dd, d1, d2, d12, dc;
  CTR_TRY(upload_prop(prop, single, nev, nt, dp));
  CTR_TRY(prop_diag(dp, nev, nt, dd));
  CTR_TRY(upload_plain(p1, nev, nt, d1));
  CTR_TRY(upload_plain(p2, nev, nt, d2));
  const int ops[5] = {0, 1, 2, 3, 4};
  CTR_TRY(upload_moms(p1p2, 5, ops, nev, nt, d12));
  CTR_TRY(dc.alloc((size_t)nt * nt * 4 * 16));
  CTR_TRY(ctr_rhopi(CTR_ENGINE_FP64, nev, nt, 0, nt, idir, dp.d(), dd.d(), d1.d(), d2.d(), d12.d(), dc.d(), nullptr));
  CTR_TRY(ctr_sync(nullptr));
  std::vector<double> a;
  CTR_TRY(averaged(dc, nt, 4, a));
  dump_rhopi(F.f, a.data(), nt);
  report(t0, flops_rows(256, 4, nev, nt), single);
  return CTR_OK;
}

int ctr_calculate_pipi(int nev, int nt, const void* prop, const double* p1, const double* p2, const double* p3,
                       const double* p4, int single, const char* outfile, int isospin) {
  CTR_NO_CAPTURE("ctr_calculate_pipi");
  CTR_TRY(check_on(nev, nt));
  if (isospin != 0 && isospin != 1) return fail(CTR_ERR_ARG, "This Isospin is not implemeted");
  File F;
  CTR_TRY(open_out(outfile, F));
  const double t0 = now();
  DevBuf dp, dd, d[4], dc;
  CTR_TRY(upload_prop(prop, single, nev, nt, dp));
  CTR_TRY(prop_diag(dp, nev, nt, dd));
  const double* ps[4] = {p1, p2, p3, p4};
  for (int k = 0; k < 4; k++) CTR_TRY(upload_plain(ps[k], nev, nt, d[k]));
  CTR_TRY(dc.alloc((size_t)nt * nt * 5 * 16));
  CTR_TRY(ctr_pipi(CTR_ENGINE_FP64, nev, nt, 0, nt, isospin, dp.d(), dd.d(), d[0].d(), d[1].d(), d[2].d(), d[3].d(),
                   dc.d(), nullptr));
  CTR_TRY(ctr_sync(nullptr));
  std::vector<double> a;
  CTR_TRY(averaged(dc, nt, 5, a));
  dump_pipi(F.f, a.data(), nt, isospin);
  const double n3 = 8.0 * nev * (double)nev * nev, n2 = 8.0 * nev * (double)nev;
  const double sq = 256 * (6 * n3 + n2), sf = 16 * (2 * n3 + n2);
  report(t0, (isospin == 0 ? 3 * sq + 2 * sf : 2 * sq + 2 * sf) * nt * (double)nt, single);
  return CTR_OK;
}

int ctr_calculate_sigma(int nev, int nt, const void* prop, const double* mom, int single, const char* outfile) {
  CTR_NO_CAPTURE("ctr_calculate_sigma");
  CTR_TRY(check_on(nev, nt));
  File F;
  CTR_TRY(open_out(outfile, F));
  DevBuf dp, dd, dl, dx2, dc;
  CTR_TRY(upload_prop(prop, single, nev, nt, dp));
  CTR_TRY(prop_diag(dp, nev, nt, dd));
  CTR_TRY(dl.alloc((size_t)nt * 16));
  for (int i = 0; i < 4; i++) {  // lib/interface.cpp:219-249: e^{+ip}, e^{-ip} and the smeared pair
    const double t0 = now();
    DevBuf dm;
    CTR_TRY(upload_plain(mom + (size_t)i * nt * nev * nev * 2, nev, nt, dm));
    CTR_TRY(ctr_loop_unity(CTR_ENGINE_FP64, nev, nt, dd.d(), dm.d(), dl.d(), nullptr));
    std::vector<double> l((size_t)nt * 2);
    CTR_CUDA(cudaMemcpy(l.data(), dl.p, l.size() * sizeof(double), cudaMemcpyDeviceToHost));
    dump_loop(F.f, l.data(), nt);
    report(t0, 320000.0 * nt * (nev / 100.0) * (nev / 100.0), single);
  }
  const double t0 = now();
  const int ops[2] = {1, 3};  // e^{-ip} and smeared e^{-ip} (lib/interface.cpp:253-259)
  CTR_TRY(upload_moms(mom, 2, ops, nev, nt, dx2));
  CTR_TRY(dc.alloc((size_t)nt * nt * 4 * 16));
  CTR_TRY(ctr_sigma(engine_of(single), nev, nt, 0, nt, dp.d(), dx2.d(), dc.d(), nullptr));
  CTR_TRY(ctr_sync(nullptr));
  std::vector<double> a;
  CTR_TRY(averaged(dc, nt, 4, a));
  dump_sigma(F.f, a.data(), nt);
  report(t0, flops_rows(64, 2, nev, nt), single);
  return CTR_OK;
}

int ctr_calculate_sigmapi(int nev, int nt, const void* prop, const double* p1, const double* p2,
                          const double* p1p2, int single, const char* outfile) {
  CTR_NO_CAPTURE("ctr_calculate_sigmapi");
  CTR_TRY(check_on(nev, nt));
  File F;
  CTR_TRY(open_out(outfile, F));
  DevBuf dp, dd, dl, d1, d2, dx2, dhf, dtr;
  CTR_TRY(upload_prop(prop, single, nev, nt, dp));
  CTR_TRY(prop_diag(dp, nev, nt, dd));
  CTR_TRY(dl.alloc((size_t)nt * 16));
  for (int i = 0; i < 2; i++) {  // loops with e^{i(p1+p2)} and its smeared form (lib/interface.cpp:305-332)
    const double t0 = now();
    DevBuf dm;
    CTR_TRY(upload_plain(p1p2 + (size_t)i * nt * nev * nev * 2, nev, nt, dm));
    CTR_TRY(ctr_loop_unity(CTR_ENGINE_FP64, nev, nt, dd.d(), dm.d(), dl.d(), nullptr));
    std::vector<double> l((size_t)nt * 2);
    CTR_CUDA(cudaMemcpy(l.data(), dl.p, l.size() * sizeof(double), cudaMemcpyDeviceToHost));
    dump_loop(F.f, l.data(), nt);
    report(t0, 320000.0 * nt * (nev / 100.0) * (nev / 100.0), single);
  }
  const double t0 = now();
  CTR_TRY(upload_plain(p1, nev, nt, d1));
  CTR_TRY(upload_plain(p2, nev, nt, d2));
  const int ops[2] = {0, 1};
  CTR_TRY(upload_moms(p1p2, 2, ops, nev, nt, dx2));
  CTR_TRY(dhf.alloc((size_t)nt * 16));
  CTR_TRY(dtr.alloc((size_t)nt * nt * 2 * 16));
  CTR_TRY(ctr_sigmapi(CTR_ENGINE_FP64, nev, nt, 0, nt, dp.d(), dd.d(), d1.d(), d2.d(), dx2.d(), dhf.d(), dtr.d(),
                      nullptr));
  CTR_TRY(ctr_sync(nullptr));
  std::vector<double> hf((size_t)nt * 2);
  CTR_CUDA(cudaMemcpy(hf.data(), dhf.p, hf.size() * sizeof(double), cudaMemcpyDeviceToHost));
  dump_fish_hor(F.f, hf.data(), nt);
  std::vector<double> a;
  CTR_TRY(averaged(dtr, nt, 2, a));
  dump_triangle(F.f, a.data(), nt);
  const double n3 = 8.0 * nev * (double)nev * nev, n2 = 8.0 * nev * (double)nev;
  report(t0, 16 * (2 * n3 + n2) * nt + 128 * (4 * n3 + n2) * nt * (double)nt, single);
  return CTR_OK;
}

}  // extern "C"

// --------------------------------------------------------- C++ API (abort on error)
namespace {
[[noreturn]] void abort_with(const char* where) {
  fprintf(stderr, "%s\n", ctr_last_error());
  fprintf(stderr, "Error in %s\n", where);
  fflush(stderr);
  std::exit(EXIT_FAILURE);
}
inline void ok_or_abort(int rc, const char* where) {
  if (rc != CTR_OK) abort_with(where);
}
}  // namespace

void contract::initContract(contractInfo info) { ok_or_abort(ctr_contract_init(info.NeV, info.Nt, info.dev), "initContract"); }

void contract::destroyContract() { ok_or_abort(ctr_contract_destroy(), "destroyContract"); }

void* contract::readPropH(const std::string& fileName, PRECISION prec) {
  if (!g_on) {
    set_error("Need to initialize contract library before read propagator");
    abort_with("readPropH");
  }
  const size_t n = (size_t)g_nt * g_nt * 16 * g_nev * g_nev * 2;
  void* p = std::malloc(n * (prec == SINGLE ? sizeof(float) : sizeof(double)));
  if (!p) {
    set_error("Not enough memory to allocate");
    abort_with("readPropH");
  }
  ok_or_abort(ctr_read_prop(fileName.c_str(), g_nev, g_nt, prec == SINGLE, p), "readPropH");
  return p;
}

void calculateRho(contract::contractInfo info, void* prop, double* mom, contract::PRECISION prec, std::string outfile) {
  ok_or_abort(ctr_calculate_rho(info.NeV, info.Nt, prop, mom, prec == contract::SINGLE, outfile.c_str()),
              "calculateRho");
}

void calculateRhoPi(int idir, contract::contractInfo info, void* prop, double* p1, double* p2, double* p1p2,
                    contract::PRECISION prec, std::string outfile) {
  ok_or_abort(ctr_calculate_rhopi(idir, info.NeV, info.Nt, prop, p1, p2, p1p2, prec == contract::SINGLE,
                                  outfile.c_str()),
              "calculateRhoPi");
}

void calculatePiPi(contract::contractInfo info, void* prop, double* p1, double* p2, double* p3, double* p4,
                   contract::PRECISION prec, std::string outfile, contract::ISOSPIN iso) {
  ok_or_abort(ctr_calculate_pipi(info.NeV, info.Nt, prop, p1, p2, p3, p4, prec == contract::SINGLE, outfile.c_str(),
                                 iso == contract::I0 ? 0 : 1),
              "calculatePiPi");
}

void calculateSigma(contract::contractInfo info, void* prop, double* mom, contract::PRECISION prec,
                    std::string outfile) {
  ok_or_abort(ctr_calculate_sigma(info.NeV, info.Nt, prop, mom, prec == contract::SINGLE, outfile.c_str()),
              "calculateSigma");
}

void calculateSigmaPi(contract::contractInfo info, void* prop, double* p1, double* p2, double* p1p2,
                      contract::PRECISION prec, std::string outfile) {
  ok_or_abort(ctr_calculate_sigmapi(info.NeV, info.Nt, prop, p1, p2, p1p2, prec == contract::SINGLE,
                                    outfile.c_str()),
              "calculateSigmaPi");
}
