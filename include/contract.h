/*
 * contract.h -- reference-compatible C++ entry points of the GB300 engine.
 *
 * Declares the library-level API of the reference's include/contract.h
 * (contractInfo, PRECISION, ISOSPIN, initContract, destroyContract, readPropH)
 * with the same names, argument meanings and error behaviour: invalid use
 * prints a message and terminates the process, as the reference's ABORT macro
 * (include/utils.h:12-17) does.  The work is done by libctr.so through the C
 * ABI of ctr.h.
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
 *    sigma), else the FP64 engine.
 */
#ifndef CTR_CONTRACT_H
#define CTR_CONTRACT_H

#include <string>

namespace contract {

typedef struct {
  int NeV;
  int Nt;
  std::string PropH_fileName;
  int dev;
} contractInfo;

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

}  // namespace contract

#endif
