// The reference's launcher layer and classes (include/contract.h), over the C ABI.
//
// Launchers (lib/contract_kernels_*.cu, run_Contract* / run_CopyConstants*):
// each takes texture objects over linear device memory, as the reference's
// Base::createTexObject builds them (lib/contract.cpp:330-369: complex128 data
// read through an int4 channel, complex64 through float2).  The launcher
// recovers each operand's device pointer and size with
// cudaGetTextureObjectResourceDesc, checks them against initContract's Nev and
// Nt, runs the corresponding ctr_* entry point for the one t_sink row on the
// legacy default stream, and copies the row's correlators into the caller's
// host array -- where the reference's launchers leave their host reductions.
// SINGLE data are widened to complex128 on the device first and the results
// narrowed to float.  Errors terminate the process, as ABORT does.
//
// Classes (lib/contract.cpp:165-1053): Base and its subclasses keep host,
// device and "extra" device arrays sized by CLASS_ENUM; LapH_prop stages the
// perambulator row by row and its time diagonal; the Contract_* drivers call
// the launchers row by row into H_elem() and append the reference's text dumps.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "contract.h"
#include "ctr.h"
#include "ctr_internal.h"

using namespace contract;

namespace {

[[noreturn]] void die(const char* msg, const char* where) {
  fprintf(stderr, "%s", msg);
  fprintf(stderr, "Error in %s\n", where);
  fflush(stderr);
  std::exit(EXIT_FAILURE);
}

void warn(const char* msg, const char* where) {
  fprintf(stderr, "%s", msg);
  fprintf(stderr, "Warning in %s\n", where);
  fflush(stderr);
}

void ok(int rc, const char* where) {
  if (rc == CTR_OK) return;
  fprintf(stderr, "%s\n", ctr_last_error());
  die("", where);
}

void cuda_ok(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return;
  fprintf(stderr, "The last cuda error is %s\n", cudaGetErrorString(e));
  die("", where);
}

// Tables "copied to the device" (the library generates them itself; the flags
// keep the reference's order of calls: constants first, then launchers).
bool g_const_rho = false, g_const_rhopi = false, g_const_pipi = false, g_const_sigma = false,
     g_const_sigmapi = false;

void need(bool on, const char* where) {
  if (!on) die("Error: You need to initialize device constants before calling Kernels\n", where);
}

void copy_constants(bool& on, const char* what, const char* where) {
  if (on) {
    char msg[128];
    snprintf(msg, sizeof msg, "Warning: Copy constants for %s again will be skipped\n", what);
    warn(msg, where);
    return;
  }
  on = true;
}

int state_nev(int Nt, const char* where) {
  int nev = 0, nt = 0;
  if (!ctr::contract_state(&nev, &nt)) die("Error: contract library is not on\n", where);
  if (Nt != nt) die("Error: Nt differs from the one given to initContract\n", where);
  return nev;
}

// Grow-only device staging: widened SINGLE operands and the launchers' results.
struct Stage {
  void* p = nullptr;
  size_t bytes = 0;
  void* get(size_t need, const char* where) {
    if (need > bytes) {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      cuda_ok(cudaMalloc(&p, need), where);
      bytes = need;
    }
    return p;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};
constexpr int kStages = 8;  // 6 operands at most, the result
Stage g_stage[kStages];

__global__ void widen_kernel(const float* __restrict__ src, double* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// The device operand behind a texture: complex128 data of `count` complex elements.
const double* operand(int slot, cudaTextureObject_t tex, PRECISION prec, size_t count, const char* where) {
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof rd);
  cuda_ok(cudaGetTextureObjectResourceDesc(&rd, tex), where);
  if (rd.resType != cudaResourceTypeLinear) die("Error: the texture object is not over linear memory\n", where);
  const cudaChannelFormatDesc& d = rd.res.linear.desc;
  const bool as_double = d.f == cudaChannelFormatKindSigned && d.x == 32 && d.y == 32 && d.z == 32 && d.w == 32;
  const bool as_float = d.f == cudaChannelFormatKindFloat && d.x == 32 && d.y == 32 && d.z == 0 && d.w == 0;
  if (prec == DOUBLE && !as_double) die("Error: DOUBLE needs a texture of int4 over complex128 data\n", where);
  if (prec == SINGLE && !as_float) die("Error: SINGLE needs a texture of float2 over complex64 data\n", where);
  const size_t need = count * 2 * (prec == DOUBLE ? sizeof(double) : sizeof(float));
  if (rd.res.linear.sizeInBytes < need) die("Error: the texture object covers less data than the launcher reads\n", where);
  if (((uintptr_t)rd.res.linear.devPtr & 15) != 0) die("Error: texture memory is not 16-byte aligned\n", where);
  if (prec == DOUBLE) return (const double*)rd.res.linear.devPtr;
  double* w = (double*)g_stage[slot].get(need * 2, where);
  widen_kernel<<<1024, 256>>>((const float*)rd.res.linear.devPtr, w, count * 2);
  cuda_ok(cudaGetLastError(), where);
  return w;
}

double* result(size_t count, const char* where) {
  return (double*)g_stage[kStages - 1].get(count * 2 * sizeof(double), where);
}

// Wait for the row, then copy `count` complex results to the caller's host array.
void finish(const double* dres, size_t count, void* corr, PRECISION prec, const char* where) {
  ok(ctr_sync(nullptr), where);
  if (prec == DOUBLE) {
    cuda_ok(cudaMemcpy(corr, dres, count * 2 * sizeof(double), cudaMemcpyDeviceToHost), where);
    return;
  }
  std::vector<double> h(count * 2);
  cuda_ok(cudaMemcpy(h.data(), dres, h.size() * sizeof(double), cudaMemcpyDeviceToHost), where);
  float* f = (float*)corr;
  for (size_t i = 0; i < h.size(); i++) f[i] = (float)h[i];
}

void check_tf(int tf, int Nt, const char* where) {
  if (tf < 0 || tf >= Nt) die("Error: t_sink out of range\n", where);
}

// DOUBLE runs the plain FP64 engine; SINGLE runs the split engine where it covers
// the diagram (rho, sigma) and the FP64 engine on the widened data elsewhere.
int engine_for(PRECISION prec, bool split_covers) {
  return prec == SINGLE && split_covers ? CTR_ENGINE_SPLIT : CTR_ENGINE_FP64;
}

}  // namespace

namespace ctr {
void compat_release() {
  for (auto& s : g_stage) s.release();
  g_const_rho = g_const_rhopi = g_const_pipi = g_const_sigma = g_const_sigmapi = false;
}
}  // namespace ctr

// ------------------------------------------------------------------ launchers
void contract::run_CopyConstantsRho() { copy_constants(g_const_rho, "rho", "run_CopyConstantsRho"); }
void contract::run_CopyConstantsRhoPi() { copy_constants(g_const_rhopi, "rho-pi", "run_CopyConstantsRhoPi"); }
void contract::run_CopyConstantsPiPi() { copy_constants(g_const_pipi, "pi-pi", "run_CopyConstantsPiPi"); }
void contract::run_CopyConstantsSigma() { copy_constants(g_const_sigma, "sigma", "run_CopyConstantsSigma"); }
void contract::run_CopyConstantsSigmaPi() { copy_constants(g_const_sigmapi, "sigmapi", "run_CopyConstantsSigmaPi"); }

void contract::run_ContractRho(cudaTextureObject_t texProp, cudaTextureObject_t texMom, int tf, int Nt, void* corr,
                               PRECISION prec) {
  const char* W = "run_ContractRho";
  need(g_const_rho, W);
  const int N = state_nev(Nt, W);
  check_tf(tf, Nt, W);
  const size_t row = (size_t)Nt * 16 * N * N;
  const double* dp = operand(0, texProp, prec, row, W);
  const double* dm = operand(1, texMom, prec, (size_t)Nt * 5 * N * N, W);
  double* out = result((size_t)Nt * 48, W);
  ok(ctr_rho(engine_for(prec, true), N, Nt, tf, tf + 1, dp, dm, out, nullptr), W);
  finish(out, (size_t)Nt * 48, corr, prec, W);
}

void contract::run_ContractRhoPi(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                                 cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2,
                                 cudaTextureObject_t texMomP1P2, int tf, int Nt, int idir, void* corr, PRECISION prec) {
  const char* W = "run_ContractRhoPi";
  need(g_const_rhopi, W);
  const int N = state_nev(Nt, W);
  check_tf(tf, Nt, W);
  const size_t blk = (size_t)Nt * 16 * N * N, mat = (size_t)Nt * N * N;
  const double* dp = operand(0, texProp, prec, blk, W);
  const double* dd = operand(1, texPropDiag, prec, blk, W);
  const double* d1 = operand(2, texMomP1, prec, mat, W);
  const double* d2 = operand(3, texMomP2, prec, mat, W);
  const double* d12 = operand(4, texMomP1P2, prec, 5 * mat, W);
  double* out = result((size_t)Nt * 4, W);
  ok(ctr_rhopi(engine_for(prec, false), N, Nt, tf, tf + 1, idir, dp, dd, d1, d2, d12, out, nullptr), W);
  finish(out, (size_t)Nt * 4, corr, prec, W);
}

static void pipi_launch(int iso, cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                        cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2, cudaTextureObject_t texMomP3,
                        cudaTextureObject_t texMomP4, int tf, int Nt, void* corr, PRECISION prec, const char* W) {
  need(g_const_pipi, W);
  const int N = state_nev(Nt, W);
  check_tf(tf, Nt, W);
  const size_t blk = (size_t)Nt * 16 * N * N, mat = (size_t)Nt * N * N;
  const double* dp = operand(0, texProp, prec, blk, W);
  const double* dd = operand(1, texPropDiag, prec, blk, W);
  const double* d1 = operand(2, texMomP1, prec, mat, W);
  const double* d2 = operand(3, texMomP2, prec, mat, W);
  const double* d3 = operand(4, texMomP3, prec, mat, W);
  const double* d4 = operand(5, texMomP4, prec, mat, W);
  double* out = result((size_t)Nt * 5, W);
  ok(ctr_pipi(engine_for(prec, false), N, Nt, tf, tf + 1, iso, dp, dd, d1, d2, d3, d4, out, nullptr), W);
  finish(out, (size_t)Nt * 5, corr, prec, W);
}

void contract::run_ContractPiPi(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                                cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2,
                                cudaTextureObject_t texMomP3, cudaTextureObject_t texMomP4, int tf, int Nt, void* corr,
                                PRECISION prec) {
  pipi_launch(1, texProp, texPropDiag, texMomP1, texMomP2, texMomP3, texMomP4, tf, Nt, corr, prec, "run_ContractPiPi");
}

void contract::run_ContractPiPi_I0(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                                   cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2,
                                   cudaTextureObject_t texMomP3, cudaTextureObject_t texMomP4, int tf, int Nt,
                                   void* corr, PRECISION prec) {
  pipi_launch(0, texProp, texPropDiag, texMomP1, texMomP2, texMomP3, texMomP4, tf, Nt, corr, prec,
              "run_ContractPiPi_I0");
}

// The reference's loop kernel reads no diagram table, so it needs no constants.
void contract::run_ContractLoopUnity(cudaTextureObject_t texPropDiag, cudaTextureObject_t texMom, int Nt, void* loop,
                                     PRECISION prec) {
  const char* W = "run_ContractLoopUnity";
  const int N = state_nev(Nt, W);
  const double* dd = operand(0, texPropDiag, prec, (size_t)Nt * 16 * N * N, W);
  const double* dm = operand(1, texMom, prec, (size_t)Nt * N * N, W);
  double* out = result((size_t)Nt, W);
  ok(ctr_loop_unity(CTR_ENGINE_FP64, N, Nt, dd, dm, out, nullptr), W);
  finish(out, (size_t)Nt, loop, prec, W);
}

void contract::run_ContractSigma(cudaTextureObject_t texProp, cudaTextureObject_t texMom, int tf, int Nt, void* corr,
                                 PRECISION prec) {
  const char* W = "run_ContractSigma";
  need(g_const_sigma, W);
  const int N = state_nev(Nt, W);
  check_tf(tf, Nt, W);
  const double* dp = operand(0, texProp, prec, (size_t)Nt * 16 * N * N, W);
  const double* dm = operand(1, texMom, prec, (size_t)Nt * 2 * N * N, W);
  double* out = result((size_t)Nt * 4, W);
  ok(ctr_sigma(engine_for(prec, true), N, Nt, tf, tf + 1, dp, dm, out, nullptr), W);
  finish(out, (size_t)Nt * 4, corr, prec, W);
}

void contract::run_ContractSigmaPi_fish_hor(cudaTextureObject_t texPropDiag, cudaTextureObject_t texMomP1,
                                            cudaTextureObject_t texMomP2, int Nt, void* corr, PRECISION prec) {
  const char* W = "run_ContractSigmaPi_fish_hor";
  need(g_const_sigmapi, W);
  const int N = state_nev(Nt, W);
  const size_t mat = (size_t)Nt * N * N;
  const double* dd = operand(0, texPropDiag, prec, (size_t)Nt * 16 * N * N, W);
  const double* d1 = operand(1, texMomP1, prec, mat, W);
  const double* d2 = operand(2, texMomP2, prec, mat, W);
  double* out = result((size_t)Nt, W);
  ok(ctr_sigmapi(engine_for(prec, false), N, Nt, 0, Nt, nullptr, dd, d1, d2, nullptr, out, nullptr, nullptr), W);
  finish(out, (size_t)Nt, corr, prec, W);
}

void contract::run_ContractSigmaPi_triangle(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                                            cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2,
                                            cudaTextureObject_t texMomP1P2, int tf, int Nt, void* corr,
                                            PRECISION prec) {
  const char* W = "run_ContractSigmaPi_triangle";
  need(g_const_sigmapi, W);
  const int N = state_nev(Nt, W);
  check_tf(tf, Nt, W);
  const size_t blk = (size_t)Nt * 16 * N * N, mat = (size_t)Nt * N * N;
  const double* dp = operand(0, texProp, prec, blk, W);
  const double* dd = operand(1, texPropDiag, prec, blk, W);
  const double* d1 = operand(2, texMomP1, prec, mat, W);
  const double* d2 = operand(3, texMomP2, prec, mat, W);
  const double* d12 = operand(4, texMomP1P2, prec, 2 * mat, W);
  double* out = result((size_t)Nt * 2, W);
  ok(ctr_sigmapi(engine_for(prec, false), N, Nt, tf, tf + 1, dp, dd, d1, d2, d12, nullptr, out, nullptr), W);
  finish(out, (size_t)Nt * 2, corr, prec, W);
}

// -------------------------------------------------------------------- classes
namespace {

// Host and device lengths (complex elements) of each class (lib/contract.cpp:170-220).
void class_lengths(CLASS_ENUM c, long nev, long nt, long* host, long* dev) {
  const long m = nt * nev * nev;
  switch (c) {
    case BASE_CLASS: *host = *dev = 0; return;
    case LAPH_PROP_CLASS: *host = nt * 16 * m; *dev = 16 * m; return;  // the device holds one t_sink row
    case MOM_MATRICES_CLASS: *host = *dev = 5 * m; return;
    case MOM_MATRICES_CLASS_x2: *host = *dev = 2 * m; return;
    case MOM_MATRIX_CLASS: *host = *dev = m; return;
    case CONTRACT_RHO_RHO_CLASS: *host = *dev = nt * nt * 48; return;
    case CONTRACT_RHO_PION_PION_CLASS: *host = *dev = nt * nt * 4; return;
    case CONTRACT_PION_PION_PION_PION_CLASS: *host = *dev = nt * nt * 5; return;
    case CONTRACT_LOOP_UNITY: *host = *dev = nt; return;
    case CONTRACT_SIGMA_SIGMA_CLASS: *host = *dev = nt * nt * 4; return;
    case CONTRACT_SIGMA_PION_PION_CLASS: *host = *dev = nt + nt * nt * 2; return;
    default: die("Error: The class you ask is not implemented yet\n", "Base::Base");
  }
}

template <typename Float>
PRECISION prec_of() {
  return sizeof(Float) == sizeof(float) ? SINGLE : DOUBLE;
}

// avg[dt][c] = 1/Nt sum_ti h[(ti+dt)%Nt][ti][c] (the dumpData bodies' source average), as doubles.
template <typename Float>
std::vector<double> source_average(const Float* h, int nt, int ncorr) {
  std::vector<double> avg((size_t)nt * ncorr * 2, 0.0);
  for (int dt = 0; dt < nt; dt++)
    for (int c = 0; c < ncorr; c++) {
      double re = 0, im = 0;
      for (int ti = 0; ti < nt; ti++) {
        const Float* v = h + ((((size_t)((ti + dt) % nt) * nt + ti) * ncorr + c) * 2);
        re += (double)v[0];
        im += (double)v[1];
      }
      avg[((size_t)dt * ncorr + c) * 2] = re / nt;
      avg[((size_t)dt * ncorr + c) * 2 + 1] = im / nt;
    }
  return avg;
}

FILE* open_append(const std::string& outfile, const char* where) {
  FILE* f = std::fopen(outfile.c_str(), "a");
  if (!f) die("Error cannot open file for writting results\n", where);
  return f;
}

}  // namespace

namespace contract {

template <typename Float>
Base<Float>::Base(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT) {
  int nev = 0, nt = 0;
  if (!ctr::contract_state(&nev, &nt)) die("You need to initialize the library first\n", "Base::Base");
  NeV = nev;
  Nt = nt;
  class_lengths(classT, nev, nt, &totalLength_host, &totalLength_device);
  totalLength_host_bytes = (size_t)totalLength_host * 2 * sizeof(Float);
  totalLength_device_bytes = (size_t)totalLength_device * 2 * sizeof(Float);
  if (classT == BASE_CLASS) return;
  switch (alloc_flag) {
    case HOST: create_host(); break;
    case DEVICE: create_device(); break;
    case BOTH: create_host(); create_device(); break;
    case BOTH_EXTRA: create_host(); create_device(); create_device_extra(); break;
    case DEVICE_EXTRA: create_device(); create_device_extra(); break;
    case NONE: break;
  }
}

template <typename Float>
Base<Float>::~Base() {
  destroy_host();
  destroy_device();
  destroy_device_extra();
}

template <typename Float>
void Base<Float>::create_host() {
  h_elem = (Float*)std::malloc(totalLength_host_bytes ? totalLength_host_bytes : 1);
  if (!h_elem) die("Error: Allocating memory for host\n", "Base::create_host");
  isAllocHost = true;
  zero_host();
}

template <typename Float>
void Base<Float>::create_device() {
  cuda_ok(cudaMalloc((void**)&d_elem, totalLength_device_bytes), "Base::create_device");
  isAllocDevice = true;
  zero_device();
}

template <typename Float>
void Base<Float>::create_device_extra() {
  cuda_ok(cudaMalloc((void**)&d_elem_extra, totalLength_device_bytes), "Base::create_device_extra");
  isAllocDeviceExtra = true;
  zero_device_extra();
}

template <typename Float>
void Base<Float>::destroy_host() {
  if (isAllocHost) std::free(h_elem);
  isAllocHost = false;
}

template <typename Float>
void Base<Float>::destroy_device() {
  if (isAllocDevice) cudaFree(d_elem);
  isAllocDevice = false;
}

template <typename Float>
void Base<Float>::destroy_device_extra() {
  if (isAllocDeviceExtra) cudaFree(d_elem_extra);
  isAllocDeviceExtra = false;
}

template <typename Float>
void Base<Float>::zero_host() {
  if (!isAllocHost) die("Error: Try initialize memory not allocated in not permited\n", "Base::zero_host");
  std::memset(h_elem, 0, totalLength_host_bytes);
}

template <typename Float>
void Base<Float>::zero_device() {
  if (!isAllocDevice) die("Error: Try initialize memory not allocated in not permited\n", "Base::zero_device");
  cuda_ok(cudaMemset(d_elem, 0, totalLength_device_bytes), "Base::zero_device");
}

template <typename Float>
void Base<Float>::zero_device_extra() {
  if (!isAllocDeviceExtra)
    die("Error: Try initialize memory not allocated in not permited\n", "Base::zero_device_extra");
  cuda_ok(cudaMemset(d_elem_extra, 0, totalLength_device_bytes), "Base::zero_device_extra");
}

// Linear texture over complex data: int4 per complex128 element, float2 per complex64.
template <typename Float>
static void make_texture(cudaTextureObject_t* tex, void* ptr, size_t bytes, const char* where) {
  cudaChannelFormatDesc desc;
  std::memset(&desc, 0, sizeof desc);
  if (sizeof(Float) == sizeof(float)) {
    desc.f = cudaChannelFormatKindFloat;
    desc.x = desc.y = 32;
  } else {
    desc.f = cudaChannelFormatKindSigned;
    desc.x = desc.y = desc.z = desc.w = 32;
  }
  cudaResourceDesc res;
  std::memset(&res, 0, sizeof res);
  res.resType = cudaResourceTypeLinear;
  res.res.linear.devPtr = ptr;
  res.res.linear.desc = desc;
  res.res.linear.sizeInBytes = bytes;
  cudaTextureDesc td;
  std::memset(&td, 0, sizeof td);
  td.readMode = cudaReadModeElementType;
  cuda_ok(cudaCreateTextureObject(tex, &res, &td, nullptr), where);
}

template <typename Float>
void Base<Float>::createTexObject(cudaTextureObject_t* tex) {
  const char* W = "Base::createTexObject";
  if (!isAllocDevice) die("Error: Create texture object for memory not allocated is not allowed\n", W);
  if (isTextureOn) die("Error: Textures object is already on\n", W);
  make_texture<Float>(tex, d_elem, totalLength_device_bytes, W);
  isTextureOn = true;
}

template <typename Float>
void Base<Float>::destroyTexObject(cudaTextureObject_t tex) {
  cudaDestroyTextureObject(tex);
  isTextureOn = false;
}

template <typename Float>
void Base<Float>::createTexObjectExtra(cudaTextureObject_t* tex) {
  const char* W = "Base::createTexObjectExtra";
  if (!isAllocDeviceExtra) die("Error: Create texture object for memory not allocated is not allowed\n", W);
  if (isTextureExtraOn) die("Error: Textures object is already on\n", W);
  make_texture<Float>(tex, d_elem_extra, totalLength_device_bytes, W);
  isTextureExtraOn = true;
}

template <typename Float>
void Base<Float>::destroyTexObjectExtra(cudaTextureObject_t tex) {
  cudaDestroyTextureObject(tex);
  isTextureExtraOn = false;
}

template <typename Float>
void Base<Float>::printInfo() {
  printf("Nev=%d Nt=%d: host %zu bytes (%s), device %zu bytes (%s), extra (%s), %s precision\n", NeV, Nt,
         totalLength_host_bytes, isAllocHost ? "allocated" : "not allocated", totalLength_device_bytes,
         isAllocDevice ? "allocated" : "not allocated", isAllocDeviceExtra ? "allocated" : "not allocated",
         sizeof(Float) == sizeof(float) ? "single" : "double");
}

template <typename Float>
void Base<Float>::copyToDevice() {
  if (!h_elem || !isAllocDevice) die("Error: copyToDevice needs host and device memory\n", "Base::copyToDevice");
  cuda_ok(cudaMemcpy(d_elem, h_elem, totalLength_device_bytes, cudaMemcpyHostToDevice), "Base::copyToDevice");
}

// ------------------------------------------------------------------ LapH_prop
template <typename Float>
LapH_prop<Float>::LapH_prop(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT) : Base<Float>(alloc_flag, classT) {}

template <typename Float>
LapH_prop<Float>::LapH_prop(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, Float* h_elem_ref)
    : Base<Float>(alloc_flag == HOST || alloc_flag == BOTH_EXTRA ? NONE : alloc_flag, classT) {
  if (alloc_flag == HOST || alloc_flag == BOTH_EXTRA)
    die("The overloaded constructor for LapH_prop does not accept this alloc_flag\n", "LapH_prop::LapH_prop");
  this->destroy_host();  // BOTH: the borrowed array stands in for the host copy
  this->h_elem = h_elem_ref;
  isRefHost = true;
}

template <typename Float>
LapH_prop<Float>::~LapH_prop() {
  if (isRefHost) this->h_elem = nullptr;
}

template <typename Float>
void LapH_prop<Float>::readPropH(const std::string& fileName) {
  if (!this->isAllocHost) die("Error: Try read element without allocate memory\n", "LapH_prop::readPropH");
  ok(ctr_read_prop(fileName.c_str(), this->NeV, this->Nt, sizeof(Float) == sizeof(float), this->h_elem),
     "LapH_prop::readPropH");
}

template <typename Float>
void LapH_prop<Float>::copyToDeviceRowByRow(int it) {
  const char* W = "LapH_prop::copyToDeviceRowByRow";
  if (!this->isAllocHost && !isRefHost)
    die("Error: Cannot copy from host to device if host is not already allocated or has a refernence pointer\n", W);
  if (it < 0 || it >= this->Nt) die("Error: t_sink out of range\n", W);
  cuda_ok(cudaMemcpy(this->d_elem, this->h_elem + (size_t)it * this->totalLength_device * 2,
                     this->totalLength_device_bytes, cudaMemcpyHostToDevice), W);
}

template <typename Float>
void LapH_prop<Float>::copyToDeviceExtraDiag() {
  const char* W = "LapH_prop::copyToDeviceExtraDiag";
  if (!this->isAllocHost && !isRefHost)
    die("Error: Cannot copy from host to device if host is not already allocated or has a refernence pointer\n", W);
  if (!this->isAllocDeviceExtra) die("Error: Cannot copy to device extra is not allocated\n", W);
  const size_t blk = (size_t)16 * this->NeV * this->NeV * 2;  // Float values of one tau(t1, t2)
  for (int t = 0; t < this->Nt; t++)
    cuda_ok(cudaMemcpy(this->d_elem_extra + (size_t)t * blk, this->h_elem + ((size_t)t * this->Nt + t) * blk,
                       blk * sizeof(Float), cudaMemcpyHostToDevice), W);
}

// ------------------------------------------------------------ Contract_* drivers
template <typename Float>
Contract_rho_rho<Float>::Contract_rho_rho(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_rho_rho")) {}
template <typename Float>
Contract_rho_rho<Float>::~Contract_rho_rho() { fclose(pf); }
template <typename Float>
void Contract_rho_rho<Float>::copyConstantsRho() { run_CopyConstantsRho(); }
template <typename Float>
void Contract_rho_rho<Float>::contractRho(Mom_matrices<Float>& mom, LapH_prop<Float>& prop) {
  cudaTextureObject_t tm, tp;
  mom.copyToDevice();
  copyConstantsRho();
  mom.createTexObject(&tm);
  prop.createTexObject(&tp);
  const int nt = this->Nt;
  for (int it = 0; it < nt; it++) {
    prop.copyToDeviceRowByRow(it);
    run_ContractRho(tp, tm, it, nt, this->h_elem + (size_t)it * nt * 48 * 2, prec_of<Float>());
  }
  cuda_ok(cudaDeviceSynchronize(), "Contract_rho_rho::contractRho");
  dumpData();
  mom.destroyTexObject(tm);
  prop.destroyTexObject(tp);
}
template <typename Float>
void Contract_rho_rho<Float>::dumpData() {
  ctr::dump_rho(pf, source_average(this->h_elem, this->Nt, 48).data(), this->Nt);
}

template <typename Float>
Contract_rho_pipi<Float>::Contract_rho_pipi(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_rho_pipi")) {}
template <typename Float>
Contract_rho_pipi<Float>::~Contract_rho_pipi() { fclose(pf); }
template <typename Float>
void Contract_rho_pipi<Float>::copyConstantsRhoPi() { run_CopyConstantsRhoPi(); }
template <typename Float>
void Contract_rho_pipi<Float>::contractRhoPi(int idir, Mom_matrix<Float>& p1, Mom_matrix<Float>& p2,
                                             Mom_matrices<Float>& p12, LapH_prop<Float>& prop) {
  cudaTextureObject_t t1, t2, t12, tp, td;
  copyConstantsRhoPi();
  p1.copyToDevice();
  p2.copyToDevice();
  p12.copyToDevice();
  prop.copyToDeviceExtraDiag();
  p1.createTexObject(&t1);
  p2.createTexObject(&t2);
  p12.createTexObject(&t12);
  prop.createTexObject(&tp);
  prop.createTexObjectExtra(&td);
  const int nt = this->Nt;
  for (int it = 0; it < nt; it++) {
    prop.copyToDeviceRowByRow(it);
    run_ContractRhoPi(tp, td, t1, t2, t12, it, nt, idir, this->h_elem + (size_t)it * nt * 4 * 2, prec_of<Float>());
  }
  cuda_ok(cudaDeviceSynchronize(), "Contract_rho_pipi::contractRhoPi");
  dumpData();
  p1.destroyTexObject(t1);
  p2.destroyTexObject(t2);
  p12.destroyTexObject(t12);
  prop.destroyTexObject(tp);
  prop.destroyTexObjectExtra(td);
}
template <typename Float>
void Contract_rho_pipi<Float>::dumpData() {
  ctr::dump_rhopi(pf, source_average(this->h_elem, this->Nt, 4).data(), this->Nt);
}

template <typename Float>
Contract_pipi_pipi<Float>::Contract_pipi_pipi(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_pipi_pipi")) {}
template <typename Float>
Contract_pipi_pipi<Float>::~Contract_pipi_pipi() { fclose(pf); }
template <typename Float>
void Contract_pipi_pipi<Float>::copyConstantsPiPi() { run_CopyConstantsPiPi(); }
template <typename Float>
void Contract_pipi_pipi<Float>::contractPiPi(Mom_matrix<Float>& p1, Mom_matrix<Float>& p2, Mom_matrix<Float>& p3,
                                               Mom_matrix<Float>& p4, LapH_prop<Float>& prop, ISOSPIN Iso) {
  cudaTextureObject_t t1, t2, t3, t4, tp, td;
  copyConstantsPiPi();
  p1.copyToDevice();
  p2.copyToDevice();
  p3.copyToDevice();
  p4.copyToDevice();
  prop.copyToDeviceExtraDiag();
  p1.createTexObject(&t1);
  p2.createTexObject(&t2);
  p3.createTexObject(&t3);
  p4.createTexObject(&t4);
  prop.createTexObject(&tp);
  prop.createTexObjectExtra(&td);
  const int nt = this->Nt;
  for (int it = 0; it < nt; it++) {
    prop.copyToDeviceRowByRow(it);
    Float* row = this->h_elem + (size_t)it * nt * 5 * 2;
    if (Iso == I1) run_ContractPiPi(tp, td, t1, t2, t3, t4, it, nt, row, prec_of<Float>());
    if (Iso == I0) run_ContractPiPi_I0(tp, td, t1, t2, t3, t4, it, nt, row, prec_of<Float>());
  }
  cuda_ok(cudaDeviceSynchronize(), "Contract_pipi_pipi::contractPiPi");
  dumpData(Iso);
  p1.destroyTexObject(t1);
  p2.destroyTexObject(t2);
  p3.destroyTexObject(t3);
  p4.destroyTexObject(t4);
  prop.destroyTexObject(tp);
  prop.destroyTexObjectExtra(td);
}
template <typename Float>
void Contract_pipi_pipi<Float>::dumpData(ISOSPIN Iso) {
  ctr::dump_pipi(pf, source_average(this->h_elem, this->Nt, 5).data(), this->Nt, Iso == I0 ? 0 : 1);
}

template <typename Float>
Contract_loop_unity<Float>::Contract_loop_unity(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_loop_unity")) {}
template <typename Float>
Contract_loop_unity<Float>::~Contract_loop_unity() { fclose(pf); }
template <typename Float>
void Contract_loop_unity<Float>::contractLoopUnity(Mom_matrix<Float>& mom, LapH_prop<Float>& prop) {
  cudaTextureObject_t tm, td;
  mom.copyToDevice();
  mom.createTexObject(&tm);
  prop.copyToDeviceExtraDiag();
  prop.createTexObjectExtra(&td);
  run_ContractLoopUnity(td, tm, this->Nt, this->h_elem, prec_of<Float>());
  cuda_ok(cudaDeviceSynchronize(), "Contract_loop_unity::contractLoopUnity");
  dumpData();
  mom.destroyTexObject(tm);
  prop.destroyTexObjectExtra(td);
}
template <typename Float>
void Contract_loop_unity<Float>::dumpData() {
  std::vector<double> l((size_t)this->Nt * 2);
  for (size_t i = 0; i < l.size(); i++) l[i] = (double)this->h_elem[i];
  ctr::dump_loop(pf, l.data(), this->Nt);
}

template <typename Float>
Contract_sigma_sigma<Float>::Contract_sigma_sigma(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_sigma_sigma")) {}
template <typename Float>
Contract_sigma_sigma<Float>::~Contract_sigma_sigma() { fclose(pf); }
template <typename Float>
void Contract_sigma_sigma<Float>::copyConstantsSigma() { run_CopyConstantsSigma(); }
template <typename Float>
void Contract_sigma_sigma<Float>::contractSigma(Mom_matrices_x2<Float>& mom, LapH_prop<Float>& prop) {
  cudaTextureObject_t tm, tp;
  mom.copyToDevice();
  copyConstantsSigma();
  mom.createTexObject(&tm);
  prop.createTexObject(&tp);
  const int nt = this->Nt;
  for (int it = 0; it < nt; it++) {
    prop.copyToDeviceRowByRow(it);
    run_ContractSigma(tp, tm, it, nt, this->h_elem + (size_t)it * nt * 4 * 2, prec_of<Float>());
  }
  cuda_ok(cudaDeviceSynchronize(), "Contract_sigma_sigma::contractSigma");
  dumpData();
  mom.destroyTexObject(tm);
  prop.destroyTexObject(tp);
}
template <typename Float>
void Contract_sigma_sigma<Float>::dumpData() {
  ctr::dump_sigma(pf, source_average(this->h_elem, this->Nt, 4).data(), this->Nt);
}

template <typename Float>
Contract_sigma_pipi<Float>::Contract_sigma_pipi(ALLOCATION_FLAG a, CLASS_ENUM c, std::string outfile)
    : Base<Float>(a, c), pf(open_append(outfile, "Contract_sigma_pipi")) {}
template <typename Float>
Contract_sigma_pipi<Float>::~Contract_sigma_pipi() { fclose(pf); }
template <typename Float>
void Contract_sigma_pipi<Float>::copyConstantsSigmaPi() { run_CopyConstantsSigmaPi(); }
template <typename Float>
void Contract_sigma_pipi<Float>::contractSigmaPi(Mom_matrix<Float>& p1, Mom_matrix<Float>& p2,
                                                 Mom_matrices_x2<Float>& p12, LapH_prop<Float>& prop) {
  cudaTextureObject_t t1, t2, t12, tp, td;
  copyConstantsSigmaPi();
  p1.copyToDevice();
  p2.copyToDevice();
  p12.copyToDevice();
  prop.copyToDeviceExtraDiag();
  p1.createTexObject(&t1);
  p2.createTexObject(&t2);
  p12.createTexObject(&t12);
  prop.createTexObject(&tp);
  prop.createTexObjectExtra(&td);
  const int nt = this->Nt;
  run_ContractSigmaPi_fish_hor(td, t1, t2, nt, this->h_elem, prec_of<Float>());
  cuda_ok(cudaDeviceSynchronize(), "Contract_sigma_pipi::contractSigmaPi");
  dumpData_fish_hor();
  for (int it = 0; it < nt; it++) {
    prop.copyToDeviceRowByRow(it);
    run_ContractSigmaPi_triangle(tp, td, t1, t2, t12, it, nt, this->h_elem + (size_t)nt * 2 + (size_t)it * nt * 2 * 2,
                                 prec_of<Float>());
  }
  cuda_ok(cudaDeviceSynchronize(), "Contract_sigma_pipi::contractSigmaPi");
  dumpData_triangle();
  p1.destroyTexObject(t1);
  p2.destroyTexObject(t2);
  p12.destroyTexObject(t12);
  prop.destroyTexObject(tp);
  prop.destroyTexObjectExtra(td);
}
template <typename Float>
void Contract_sigma_pipi<Float>::dumpData_fish_hor() {
  std::vector<double> hf((size_t)this->Nt * 2);
  for (size_t i = 0; i < hf.size(); i++) hf[i] = (double)this->h_elem[i];
  ctr::dump_fish_hor(pf, hf.data(), this->Nt);
}
template <typename Float>
void Contract_sigma_pipi<Float>::dumpData_triangle() {
  ctr::dump_triangle(pf, source_average(this->h_elem + (size_t)this->Nt * 2, this->Nt, 2).data(), this->Nt);
}

}  // namespace contract

// Instantiations for both precisions, as the reference's contract.cpp provides.
namespace contract {
#define CTR_INSTANTIATE(T)                \
  template class Base<T>;                 \
  template class Mom_matrix<T>;           \
  template class Mom_matrices<T>;         \
  template class Mom_matrices_x2<T>;      \
  template class LapH_prop<T>;            \
  template class Contract_rho_rho<T>;     \
  template class Contract_rho_pipi<T>;    \
  template class Contract_pipi_pipi<T>;   \
  template class Contract_loop_unity<T>;  \
  template class Contract_sigma_sigma<T>; \
  template class Contract_sigma_pipi<T>;
CTR_INSTANTIATE(float)
CTR_INSTANTIATE(double)
#undef CTR_INSTANTIATE
}  // namespace contract
