/* Generated by contractions_code_scattering_gb300/constants_headers.py from the
 * diagram tables libctr.so builds from the gamma matrices (ctr_table_*).
 * Do not edit.  Every diagram table. */
#ifndef CTR_CONSTANTS_H
#define CTR_CONSTANTS_H

#include <constants_rho.h>
#include <constants_rhopi.h>
#include <constants_pipi.h>
#include <constants_sigma.h>
#include <constants_sigmapi.h>

#endif
