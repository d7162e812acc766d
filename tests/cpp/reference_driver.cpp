// A reference-side caller of the C++ boundary (include/contract.h), as the
// reference's drivers and launchers use it, for tests/test_cpp_boundary.py.
//
//   reference_driver <dir> <nev> <nt>
//
// Reads complex128 inputs from <dir> (prop [Nt][Nt][4][4][N][N], mom5 [Nt][5][N][N],
// mom2 [Nt][2][N][N], p1..p4 [Nt][N][N]) and writes raw results there:
//  * launchers: texture objects built over linear device memory as the
//    reference's Base::createTexObject builds them (complex128 read as int4),
//    the perambulator staged row by row; every run_Contract* launcher, row by row
//    (launch_*.bin);
//  * classes: LapH_prop / Mom_* / Contract_* driving the same contractions,
//    H_elem() written out (class_*.bin), text dumps appended to class_*.txt;
//  * single precision: Contract_rho_rho<float> and Contract_pipi_pipi<float> on
//    the inputs rounded to float (single_*.bin).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "contract.h"

using namespace contract;

static std::string g_dir;

static std::vector<double> load(const char* name, size_t n) {
  std::vector<double> v(n * 2);
  FILE* f = fopen((g_dir + "/" + name).c_str(), "rb");
  if (!f || fread(v.data(), sizeof(double), v.size(), f) != v.size()) {
    fprintf(stderr, "cannot read %s\n", name);
    exit(2);
  }
  fclose(f);
  return v;
}

template <typename T>
static void save(const char* name, const T* p, size_t n) {
  FILE* f = fopen((g_dir + "/" + name).c_str(), "wb");
  if (!f || fwrite(p, sizeof(T), n, f) != n) {
    fprintf(stderr, "cannot write %s\n", name);
    exit(2);
  }
  fclose(f);
}

static void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    exit(3);
  }
}

// A device copy of n complex128 values with an int4 linear texture over it
// (the reference's Base::createTexObject for double data).
struct TexBuf {
  void* d = nullptr;
  cudaTextureObject_t tex = 0;
  size_t bytes = 0;
  explicit TexBuf(size_t ncomplex) : bytes(ncomplex * 16) {
    check(cudaMalloc(&d, bytes), "cudaMalloc");
    cudaChannelFormatDesc desc;
    memset(&desc, 0, sizeof desc);
    desc.f = cudaChannelFormatKindSigned;
    desc.x = desc.y = desc.z = desc.w = 32;
    cudaResourceDesc res;
    memset(&res, 0, sizeof res);
    res.resType = cudaResourceTypeLinear;
    res.res.linear.devPtr = d;
    res.res.linear.desc = desc;
    res.res.linear.sizeInBytes = bytes;
    cudaTextureDesc td;
    memset(&td, 0, sizeof td);
    td.readMode = cudaReadModeElementType;
    check(cudaCreateTextureObject(&tex, &res, &td, nullptr), "cudaCreateTextureObject");
  }
  void put(const double* h) { check(cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice), "cudaMemcpy"); }
  ~TexBuf() {
    cudaDestroyTextureObject(tex);
    cudaFree(d);
  }
};

template <typename Float>
static void fill(Base<Float>& b, const std::vector<double>& v) {
  for (size_t i = 0; i < v.size(); i++) b.H_elem()[i] = (Float)v[i];
}

template <typename Float>
static void run_classes(const char* prefix, int N, int Nt, const std::vector<double>& prop,
                        const std::vector<double>& mom5, const std::vector<double>& mom2,
                        const std::vector<double>* p, bool all) {
  std::vector<Float> hprop(prop.begin(), prop.end());
  LapH_prop<Float> lp(DEVICE_EXTRA, LAPH_PROP_CLASS, hprop.data());
  Mom_matrices<Float> m5(BOTH, MOM_MATRICES_CLASS);
  fill(m5, mom5);
  Mom_matrix<Float>* P[4];
  for (int k = 0; k < 4; k++) {
    P[k] = new Mom_matrix<Float>(BOTH, MOM_MATRIX_CLASS);
    fill(*P[k], p[k]);
  }
  const std::string base = g_dir + "/" + prefix;
  char name[128];
  {
    Contract_rho_rho<Float> c(HOST, CONTRACT_RHO_RHO_CLASS, base + "_rho.txt");
    c.contractRho(m5, lp);
    snprintf(name, sizeof name, "%s_rho.bin", prefix);
    save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
  }
  {
    Contract_pipi_pipi<Float> c(HOST, CONTRACT_PION_PION_PION_PION_CLASS, base + "_pipi.txt");
    c.contractPiPi(*P[0], *P[1], *P[2], *P[3], lp, I0);
    snprintf(name, sizeof name, "%s_pipi0.bin", prefix);
    save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
  }
  if (all) {
    {
      Contract_rho_pipi<Float> c(HOST, CONTRACT_RHO_PION_PION_CLASS, base + "_rhopi.txt");
      c.contractRhoPi(1, *P[0], *P[1], m5, lp);
      snprintf(name, sizeof name, "%s_rhopi1.bin", prefix);
      save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
    }
    {
      Contract_pipi_pipi<Float> c(HOST, CONTRACT_PION_PION_PION_PION_CLASS, base + "_pipi.txt");
      c.contractPiPi(*P[0], *P[1], *P[2], *P[3], lp, I1);
      snprintf(name, sizeof name, "%s_pipi1.bin", prefix);
      save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
    }
    Mom_matrices_x2<Float> m2(BOTH, MOM_MATRICES_CLASS_x2);
    fill(m2, mom2);
    {
      Contract_sigma_sigma<Float> c(HOST, CONTRACT_SIGMA_SIGMA_CLASS, base + "_sigma.txt");
      c.contractSigma(m2, lp);
      snprintf(name, sizeof name, "%s_sigma.bin", prefix);
      save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
    }
    {
      Contract_sigma_pipi<Float> c(HOST, CONTRACT_SIGMA_PION_PION_CLASS, base + "_sigmapi.txt");
      c.contractSigmaPi(*P[0], *P[1], m2, lp);
      snprintf(name, sizeof name, "%s_sigmapi.bin", prefix);
      save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
    }
    {
      Contract_loop_unity<Float> c(HOST, CONTRACT_LOOP_UNITY, base + "_loop.txt");
      c.contractLoopUnity(*P[0], lp);
      snprintf(name, sizeof name, "%s_loop.bin", prefix);
      save(name, c.H_elem(), c.Bytes_total_host() / sizeof(Float));
    }
  }
  for (int k = 0; k < 4; k++) delete P[k];
}

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s dir nev nt\n", argv[0]);
    return 1;
  }
  g_dir = argv[1];
  const int N = atoi(argv[2]), Nt = atoi(argv[3]);
  const size_t mat = (size_t)Nt * N * N, row = 16 * mat;
  std::vector<double> prop = load("prop.bin", (size_t)Nt * row);
  std::vector<double> mom5 = load("mom5.bin", 5 * mat), mom2 = load("mom2.bin", 2 * mat);
  std::vector<double> p[4] = {load("p1.bin", mat), load("p2.bin", mat), load("p3.bin", mat), load("p4.bin", mat)};

  contractInfo info;
  info.NeV = N;
  info.Nt = Nt;
  info.dev = 0;
  initContract(info);

  // ---- launchers on texture objects, the perambulator staged row by row
  {
    TexBuf trow(row), tdiag(row), t5(5 * mat), t2(2 * mat), tp[4] = {TexBuf(mat), TexBuf(mat), TexBuf(mat), TexBuf(mat)};
    std::vector<double> diag(row * 2);
    for (int t = 0; t < Nt; t++)
      memcpy(&diag[(size_t)t * 16 * N * N * 2], &prop[((size_t)t * Nt + t) * 16 * N * N * 2], 16 * (size_t)N * N * 16);
    tdiag.put(diag.data());
    t5.put(mom5.data());
    t2.put(mom2.data());
    for (int k = 0; k < 4; k++) tp[k].put(p[k].data());
    run_CopyConstantsRho();
    run_CopyConstantsRhoPi();
    run_CopyConstantsPiPi();
    run_CopyConstantsSigma();
    run_CopyConstantsSigmaPi();
    std::vector<double> rho((size_t)Nt * Nt * 48 * 2), rhopi[3], pipi0((size_t)Nt * Nt * 5 * 2),
        pipi1((size_t)Nt * Nt * 5 * 2), sig((size_t)Nt * Nt * 4 * 2), tri((size_t)Nt * Nt * 2 * 2);
    for (int d = 0; d < 3; d++) rhopi[d].resize((size_t)Nt * Nt * 4 * 2);
    for (int tf = 0; tf < Nt; tf++) {
      trow.put(&prop[(size_t)tf * row * 2]);
      run_ContractRho(trow.tex, t5.tex, tf, Nt, &rho[(size_t)tf * Nt * 48 * 2], DOUBLE);
      for (int d = 0; d < 3; d++)
        run_ContractRhoPi(trow.tex, tdiag.tex, tp[0].tex, tp[1].tex, t5.tex, tf, Nt, d,
                          &rhopi[d][(size_t)tf * Nt * 4 * 2], DOUBLE);
      run_ContractPiPi_I0(trow.tex, tdiag.tex, tp[0].tex, tp[1].tex, tp[2].tex, tp[3].tex, tf, Nt,
                          &pipi0[(size_t)tf * Nt * 5 * 2], DOUBLE);
      run_ContractPiPi(trow.tex, tdiag.tex, tp[0].tex, tp[1].tex, tp[2].tex, tp[3].tex, tf, Nt,
                       &pipi1[(size_t)tf * Nt * 5 * 2], DOUBLE);
      run_ContractSigma(trow.tex, t2.tex, tf, Nt, &sig[(size_t)tf * Nt * 4 * 2], DOUBLE);
      run_ContractSigmaPi_triangle(trow.tex, tdiag.tex, tp[0].tex, tp[1].tex, t2.tex, tf, Nt,
                                   &tri[(size_t)tf * Nt * 2 * 2], DOUBLE);
    }
    std::vector<double> hf((size_t)Nt * 2), loop((size_t)Nt * 2);
    run_ContractSigmaPi_fish_hor(tdiag.tex, tp[0].tex, tp[1].tex, Nt, hf.data(), DOUBLE);
    run_ContractLoopUnity(tdiag.tex, tp[0].tex, Nt, loop.data(), DOUBLE);
    save("launch_rho.bin", rho.data(), rho.size());
    for (int d = 0; d < 3; d++) {
      char name[64];
      snprintf(name, sizeof name, "launch_rhopi%d.bin", d);
      save(name, rhopi[d].data(), rhopi[d].size());
    }
    save("launch_pipi0.bin", pipi0.data(), pipi0.size());
    save("launch_pipi1.bin", pipi1.data(), pipi1.size());
    save("launch_sigma.bin", sig.data(), sig.size());
    save("launch_triangle.bin", tri.data(), tri.size());
    save("launch_hor_fish.bin", hf.data(), hf.size());
    save("launch_loop.bin", loop.data(), loop.size());
  }

  // ---- the classes, both precisions
  run_classes<double>("class", N, Nt, prop, mom5, mom2, p, true);
  run_classes<float>("single", N, Nt, prop, mom5, mom2, p, false);

  destroyContract();
  printf("reference driver: done\n");
  return 0;
}
