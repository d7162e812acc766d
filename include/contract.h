/*
 * contract.h -- reference-compatible C++ entry points of the GB300 engine.
 *
 * Declares the library-level API of the reference's include/contract.h with the
 * same names, argument meanings and error behaviour: invalid use prints a
 * message and terminates the process, as the reference's ABORT macro
 * (include/utils.h:12-17) does.  The work is done by libctr.so through the C
 * ABI of ctr.h.  Three layers, as in the reference:
 *
 *  - library state: contractInfo, initContract, destroyContract, readPropH
 *    (include/contract.h:17-48 of the reference);
 *  - the launchers run_Contract* / run_CopyConstants* on texture objects
 *    (include/contract.h:50-69).  They take the texture objects the reference's
 *    Base::createTexObject builds over linear device memory (lib/contract.cpp:
 *    330-369: complex128 read as int4, complex64 as float2), recover the device
 *    pointers from them, and fill the caller's HOST corr arrays for one t_sink
 *    row, as the reference's launchers do after their host reductions;
 *  - the classes Base, Mom_matrix, Mom_matrices, Mom_matrices_x2, LapH_prop and
 *    Contract_* (include/contract.h:71-247) with the same public methods:
 *    device staging row by row, texture objects, the contract*() drivers that
 *    call the launchers and append the reference's text dumps, and H_elem() for
 *    full-precision results.
 *
 * Differences from the reference, by design:
 *  - Nev is not restricted to 100 (the reference aborts otherwise,
 *    lib/contract.cpp:59); the tensor-core engine takes Nev <= 128, the FP64
 *    engine any Nev.
 *  - destroyContract() releases the library's device buffers instead of
 *    calling cudaDeviceReset(), so that it can run inside a process that keeps
 *    using the GPU.
 *  - PRECISION selects the engine: DOUBLE -> plain FP64 engine (the drop-in),
 *    SINGLE -> float data widened on the device and contracted by the
 *    split-precision tensor-core engine where it covers the diagram (rho,
 *    sigma), else the FP64 engine; results are narrowed to float.
 *  - The diagram tables are generated by the library; run_CopyConstants*
 *    only marks them as available (the launchers refuse to run before, as the
 *    reference's do).
 */
#ifndef CTR_CONTRACT_H
#define CTR_CONTRACT_H

#include <cuda_runtime.h>

#include <cstdio>
#include <string>

namespace contract {

typedef struct {
  int NeV;
  int Nt;
  std::string PropH_fileName;
  int dev;
} contractInfo;

// Allocation of a Base object: host array, device array, and the device
// "extra" array (the perambulator's time diagonal tau(t,t)).
enum ALLOCATION_FLAG { NONE, HOST, DEVICE, BOTH, BOTH_EXTRA, DEVICE_EXTRA };
// What a Base object holds; fixes its host and device sizes.
enum CLASS_ENUM {
  BASE_CLASS,
  GAUGE_CLASS,
  VECTOR_CLASS,
  COLOR_VECTOR_CLASS,
  LAPH_EIGENVECTORS_CLASS,
  LAPH_PROP_CLASS,
  MOM_MATRIX_CLASS,
  MOM_MATRICES_CLASS,
  CONTRACT_RHO_RHO_CLASS,
  CONTRACT_RHO_PION_PION_CLASS,
  CONTRACT_PION_PION_PION_PION_CLASS,
  CONTRACT_LOOP_UNITY,
  MOM_MATRICES_CLASS_x2,
  CONTRACT_SIGMA_SIGMA_CLASS,
  CONTRACT_SIGMA_PION_PION_CLASS
};
enum PRECISION { SINGLE, DOUBLE };
enum ISOSPIN { I0, I1 };

// Global of the reference's option parser, printed by the rho->pipi dump
// (include/catchOpts.h:35, lib/contract.cpp:722).
extern int i_dir;

void initContract(contractInfo info);
void destroyContract();
// Reads a perambulator file (100-byte configuration name, uint32 Nt, uint32 Nvec,
// complex128 payload in (s1,v1,t1,s2,v2,t2) order) into a malloc'ed host buffer
// in the library layout [t1][t2][s1][s2][v1][v2], as float or double complex.
void* readPropH(const std::string& fileName, PRECISION prec);

// ------------------------------------------------------------- launchers
// Device operands behind the texture objects (Nev, Nt from initContract):
//   texProp      tau(tf, .)  [Nt][4][4][Nev][Nev]     (LapH_prop device row)
//   texPropDiag  tau(t, t)   [Nt][4][4][Nev][Nev]     (LapH_prop device extra)
//   texMom       rho: [Nt][5][Nev][Nev]; sigma: [Nt][2][Nev][Nev]
//   texMomP*     [Nt][Nev][Nev]; texMomP1P2: rho->pipi [Nt][5][..], sigma->pipi [Nt][2][..]
// Host outputs for t_sink tf (complex, interleaved re/im of the precision's type):
//   rho [Nt][16][3], rho->pipi [Nt][4], pipi [Nt][5], sigma [Nt][4],
//   sigma->pipi horizontal fish [Nt] (all t), triangle [Nt][2], loop [Nt].
void run_ContractRho(cudaTextureObject_t texProp, cudaTextureObject_t texMom, int tf, int Nt, void* corr,
                     PRECISION prec);
void run_CopyConstantsRho();

void run_ContractRhoPi(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag, cudaTextureObject_t texMomP1,
                       cudaTextureObject_t texMomP2, cudaTextureObject_t texMomP1P2, int tf, int Nt, int idir,
                       void* corr, PRECISION prec);
void run_CopyConstantsRhoPi();

void run_ContractPiPi(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag, cudaTextureObject_t texMomP1,
                      cudaTextureObject_t texMomP2, cudaTextureObject_t texMomP3, cudaTextureObject_t texMomP4,
                      int tf, int Nt, void* corr, PRECISION prec);
void run_ContractLoopUnity(cudaTextureObject_t texPropDiag, cudaTextureObject_t texMom, int Nt, void* loop,
                           PRECISION prec);
void run_CopyConstantsPiPi();
void run_ContractPiPi_I0(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag, cudaTextureObject_t texMomP1,
                         cudaTextureObject_t texMomP2, cudaTextureObject_t texMomP3, cudaTextureObject_t texMomP4,
                         int tf, int Nt, void* corr, PRECISION prec);

void run_ContractSigma(cudaTextureObject_t texProp, cudaTextureObject_t texMom, int tf, int Nt, void* corr,
                       PRECISION prec);
void run_CopyConstantsSigma();

void run_CopyConstantsSigmaPi();
void run_ContractSigmaPi_fish_hor(cudaTextureObject_t texPropDiag, cudaTextureObject_t texMomP1,
                                  cudaTextureObject_t texMomP2, int Nt, void* corr, PRECISION prec);
void run_ContractSigmaPi_triangle(cudaTextureObject_t texProp, cudaTextureObject_t texPropDiag,
                                  cudaTextureObject_t texMomP1, cudaTextureObject_t texMomP2,
                                  cudaTextureObject_t texMomP1P2, int tf, int Nt, void* corr, PRECISION prec);

// --------------------------------------------------------------- classes
// Complex arrays of Float (interleaved re/im) on the host and the device.
// Sizes (complex elements) follow the class: LapH_prop host Nt^2*16*Nev^2,
// device one t_sink row Nt*16*Nev^2 (+ the same for the extra diagonal);
// Mom_matrix Nt*Nev^2; Mom_matrices 5x that; Mom_matrices_x2 2x; results
// rho Nt^2*48, rho->pipi Nt^2*4, pipi Nt^2*5, loop Nt, sigma Nt^2*4,
// sigma->pipi Nt + Nt^2*2.
template <typename Float>
class Base {
 protected:
  int NeV = 0, Nt = 0;
  long int totalLength_host = 0, totalLength_device = 0;
  size_t totalLength_host_bytes = 0, totalLength_device_bytes = 0;
  Float* h_elem = nullptr;
  Float* d_elem = nullptr;
  Float* d_elem_extra = nullptr;
  bool isAllocHost = false, isAllocDevice = false, isAllocDeviceExtra = false;
  bool isTextureOn = false, isTextureExtraOn = false;

  void create_host();
  void create_device();
  void create_device_extra();
  void destroy_host();
  void destroy_device();
  void destroy_device_extra();
  void zero_host();
  void zero_device();
  void zero_device_extra();

 public:
  Base(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT);
  virtual ~Base();
  Base(const Base&) = delete;
  Base& operator=(const Base&) = delete;

  void createTexObject(cudaTextureObject_t* tex);
  void destroyTexObject(cudaTextureObject_t tex);
  void createTexObjectExtra(cudaTextureObject_t* tex);
  void destroyTexObjectExtra(cudaTextureObject_t tex);

  size_t Bytes_total_host() const { return totalLength_host_bytes; }
  size_t Bytes_total_device() const { return totalLength_device_bytes; }
  Float* H_elem() const { return h_elem; }
  Float* D_elem() const { return d_elem; }
  Float* D_elem_extra() const { return d_elem_extra; }
  int Precision() const { return (int)sizeof(Float); }
  void printInfo();
  void copyToDevice();
};

template <typename Float>
class Mom_matrix : public Base<Float> {
 public:
  Mom_matrix(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT) : Base<Float>(alloc_flag, classT) {}
};

template <typename Float>
class Mom_matrices : public Base<Float> {
 public:
  Mom_matrices(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT) : Base<Float>(alloc_flag, classT) {}
};

template <typename Float>
class Mom_matrices_x2 : public Base<Float> {
 public:
  Mom_matrices_x2(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT) : Base<Float>(alloc_flag, classT) {}
};

template <typename Float>
class LapH_prop : public Base<Float> {
 private:
  bool isRefHost = false;

 public:
  LapH_prop(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT);
  // Borrows the caller's host perambulator (not freed by the object).
  LapH_prop(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, Float* h_elem_ref);
  ~LapH_prop();
  void readPropH(const std::string& fileName);
  void copyToDeviceRowByRow(int it);  // tau(it, .) -> device row
  void copyToDeviceExtraDiag();       // tau(t, t) for every t -> device extra
};

template <typename Float>
class Contract_rho_rho : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void copyConstantsRho();
  void dumpData();

 public:
  Contract_rho_rho(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_rho_rho();
  void contractRho(Mom_matrices<Float>&, LapH_prop<Float>&);
};

template <typename Float>
class Contract_rho_pipi : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void copyConstantsRhoPi();
  void dumpData();

 public:
  Contract_rho_pipi(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_rho_pipi();
  void contractRhoPi(int idir, Mom_matrix<Float>&, Mom_matrix<Float>&, Mom_matrices<Float>&, LapH_prop<Float>&);
};

template <typename Float>
class Contract_pipi_pipi : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void copyConstantsPiPi();
  void dumpData(ISOSPIN Iso);

 public:
  Contract_pipi_pipi(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_pipi_pipi();
  void contractPiPi(Mom_matrix<Float>&, Mom_matrix<Float>&, Mom_matrix<Float>&, Mom_matrix<Float>&,
                    LapH_prop<Float>&, ISOSPIN Iso);
};

template <typename Float>
class Contract_loop_unity : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void dumpData();

 public:
  Contract_loop_unity(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_loop_unity();
  void contractLoopUnity(Mom_matrix<Float>&, LapH_prop<Float>&);
};

template <typename Float>
class Contract_sigma_sigma : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void copyConstantsSigma();
  void dumpData();

 public:
  Contract_sigma_sigma(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_sigma_sigma();
  void contractSigma(Mom_matrices_x2<Float>&, LapH_prop<Float>&);
};

template <typename Float>
class Contract_sigma_pipi : public Base<Float> {
 private:
  FILE* pf = nullptr;
  void copyConstantsSigmaPi();
  void dumpData_fish_hor();
  void dumpData_triangle();

 public:
  Contract_sigma_pipi(ALLOCATION_FLAG alloc_flag, CLASS_ENUM classT, std::string outfile);
  ~Contract_sigma_pipi();
  void contractSigmaPi(Mom_matrix<Float>&, Mom_matrix<Float>&, Mom_matrices_x2<Float>&, LapH_prop<Float>&);
};

}  // namespace contract

#endif
