/*
 * interface.h -- the reference's public contraction API (include/interface.h:6-10),
 * same signatures, same output files (appended, "%+e" text as the reference's
 * dumpData routines write them, lib/contract.cpp:616-1053).
 *
 * prop: host perambulator [Nt][Nt][4][4][Nev][Nev] complex (double for DOUBLE,
 * float for SINGLE).  Elemental arrays are host complex128:
 *   calculateRho     mom  [5][Nt][N][N]  (plain, smeared, 3 commutators)
 *   calculateRhoPi   P1, P2 [Nt][N][N], P1P2 [5][Nt][N][N]
 *   calculatePiPi    P1..P4 [Nt][N][N]
 *   calculateSigma   mom  [4][Nt][N][N]  (e^{+ip}, e^{-ip}, smeared e^{+ip}, smeared e^{-ip})
 *   calculateSigmaPi P1, P2 [Nt][N][N], P1P2 [2][Nt][N][N]
 */
#ifndef CTR_INTERFACE_H
#define CTR_INTERFACE_H

#include <string>

#include "contract.h"

void calculateRho(contract::contractInfo, void*, double*, contract::PRECISION, std::string outfile);
void calculateRhoPi(int idir, contract::contractInfo, void*, double*, double*, double*, contract::PRECISION,
                    std::string outfile);
void calculatePiPi(contract::contractInfo, void*, double*, double*, double*, double*, contract::PRECISION,
                   std::string outfile, contract::ISOSPIN);
void calculateSigma(contract::contractInfo, void*, double*, contract::PRECISION, std::string outfile);
void calculateSigmaPi(contract::contractInfo, void*, double*, double*, double*, contract::PRECISION,
                      std::string outfile);

#endif
