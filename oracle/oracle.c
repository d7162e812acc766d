/*
 * ORACLE -- test infrastructure, not the product.
 *
 * Plain-C (OpenMP) FP64 restatement of the reference's distillation contraction
 * kernels and of the host code around them.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py call it, always as the checker or as the
 * timed CPU baseline; the product library never links it.
 *
 * Every function follows one reference routine in the reference's own chain
 * order (no sub-chain sharing): each spin row multiplies full Nev x Nev complex
 * matrices left to right, summing k = 0..Nev-1 in order, and closes with the
 * Hadamard trace sum_{ij} X_ij * conj(Y_ij) (or conj(X)*Y, as the reference does).
 * Row results are multiplied by the table coefficient, which the reference keeps
 * as float and widens to the working precision.  Host reductions over spin rows
 * and the isospin weights follow the launchers in lib/contract_kernels_*.cu.
 *
 * Complex numbers are interleaved (re, im) doubles.  Layouts:
 *   prop_row  tau(tf, t2)  [Nt(t2)][4(s1)][4(s2)][N(v1)][N(v2)]  (lib/contract.cpp:545)
 *   prop_diag tau(t, t)    [Nt][4][4][N][N]                        (lib/contract.cpp:565)
 *   mom5      [Nt][5][N][N]   Mom_matrices     (lib/interface.cpp:25)
 *   mom2      [Nt][2][N][N]   Mom_matrices_x2  (lib/interface.cpp:258)
 *   mom       [Nt][N][N]      Mom_matrix       (lib/interface.cpp:85)
 */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) {
  cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}

#define BLK(base, t, s1, s2, N) ((const cplx*)(base) + ((size_t)(t) * 16 + (s1) * 4 + (s2)) * (size_t)(N) * (N))

/* C = A * B for N x N complex row-major matrices (k summed in order 0..N-1). */
static void zgemm_nn(int N, const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < N; i++) {
    cplx* c = C + (size_t)i * N;
    for (int j = 0; j < N; j++) { c[j].re = 0.0; c[j].im = 0.0; }
    for (int k = 0; k < N; k++) {
      cplx a = A[(size_t)i * N + k];
      const cplx* b = B + (size_t)k * N;
      for (int j = 0; j < N; j++) {
        c[j].re += a.re * b[j].re - a.im * b[j].im;
        c[j].im += a.re * b[j].im + a.im * b[j].re;
      }
    }
  }
}

/* C = A * B^dagger (used by the horizontal double triangle, calculate_pipi_doubleTriangleHor_core.h:106-140) */
static void zgemm_nc(int N, const cplx* A, const cplx* B, cplx* C) {
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double re = 0.0, im = 0.0;
      for (int k = 0; k < N; k++) {
        cplx a = A[(size_t)i * N + k];
        cplx b = B[(size_t)j * N + k];
        /* a * conj(b) */
        re += a.re * b.re + a.im * b.im;
        im += -a.re * b.im + a.im * b.re;
      }
      C[(size_t)i * N + j].re = re;
      C[(size_t)i * N + j].im = im;
    }
}

/* sum_ij X_ij * conj(Y_ij) */
static cplx had_xcy(int N, const cplx* X, const cplx* Y) {
  cplx s = {0.0, 0.0};
  size_t n = (size_t)N * N;
  for (size_t e = 0; e < n; e++) {
    s.re += X[e].re * Y[e].re + X[e].im * Y[e].im;
    s.im += X[e].im * Y[e].re - X[e].re * Y[e].im;
  }
  return s;
}

static inline cplx fcoef(const float* coef, int row) {
  cplx c = {(double)coef[2 * row], (double)coef[2 * row + 1]};
  return c;
}

static cplx* scratch(int N, int nmat) { return (cplx*)malloc(sizeof(cplx) * (size_t)N * N * nmat); }

/* ------------------------------------------------------------------ rho */
/* lib/calculate_rho_core.h:1-152 launched by lib/contract_kernels_rho.cu:69-124.
 * rows[ti][768]: coef * sum conj(T2) (.) T1 with T1 = tau(tf,ti)_{s3s4} Phi_lp(ti),
 * T2 = Phi_rp(tf) tau(tf,ti)_{s1s2}.  corr[ti][16][3]: sum of the 16 spin rows of
 * each (op pair ico, direction igi) (contract_kernels_rho.cu:110-116). */
void oracle_rho_row(int N, int Nt, int tf, const double* prop_row, const double* mom5,
                    const int16_t* spin, const int16_t* lprp, const float* coef,
                    double* rows, double* corr) {
  const cplx* mom = (const cplx*)mom5;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* T1 = scratch(N, 2);
    cplx* T2 = T1 + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int bx = 0; bx < 768; bx++) {
        int s1 = spin[bx * 4 + 0], s2 = spin[bx * 4 + 1], s3 = spin[bx * 4 + 2], s4 = spin[bx * 4 + 3];
        int lp = lprp[bx * 2 + 0], rp = lprp[bx * 2 + 1];
        zgemm_nn(N, BLK(prop_row, ti, s3, s4, N), mom + ((size_t)ti * 5 + lp) * N2, T1);
        zgemm_nn(N, mom + ((size_t)tf * 5 + rp) * N2, BLK(prop_row, ti, s1, s2, N), T2);
        cplx s = had_xcy(N, T1, T2); /* T1 * conj(T2) */
        cplx r = cmul(fcoef(coef, bx), s);
        rows[((size_t)ti * 768 + bx) * 2 + 0] = r.re;
        rows[((size_t)ti * 768 + bx) * 2 + 1] = r.im;
      }
    free(T1);
  }
  for (int ti = 0; ti < Nt; ti++)
    for (int o = 0; o < 48; o++) {
      double re = 0.0, im = 0.0;
      for (int is = 0; is < 16; is++) {
        re += rows[((size_t)ti * 768 + o * 16 + is) * 2 + 0];
        im += rows[((size_t)ti * 768 + o * 16 + is) * 2 + 1];
      }
      corr[((size_t)ti * 48 + o) * 2 + 0] = re;
      corr[((size_t)ti * 48 + o) * 2 + 1] = im;
    }
}

/* ---------------------------------------------------------------- rho-pipi */
/* lib/calculate_rhopi_core.h:1-226 launched by lib/contract_kernels_rhopi.cu:64-123.
 * Table row idir*256+bx; chain Phi^{P1P2}_ip(tf) tau(tf,ti)_{s5s6} Phi_P2(ti)
 * tau(ti,ti)_{s1s2} Phi_P1(ti), closed with conj tau(tf,ti)_{s3s2}.
 * rows[ti][256], corr[ti][4] (sum of 64 spin rows per rho operator). */
void oracle_rhopi_row(int N, int Nt, int tf, int idir, const double* prop_row, const double* prop_diag,
                      const double* momP1, const double* momP2, const double* mom5P1P2,
                      const int16_t* spin6, const int16_t* ip, const float* coef,
                      double* rows, double* corr) {
  const cplx *P1 = (const cplx*)momP1, *P2 = (const cplx*)momP2, *P12 = (const cplx*)mom5P1P2;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* A = scratch(N, 2);
    cplx* B = A + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int bx = 0; bx < 256; bx++) {
        int r = idir * 256 + bx;
        int s1 = spin6[r * 6 + 0], s2 = spin6[r * 6 + 1], s3 = spin6[r * 6 + 2];
        int s5 = spin6[r * 6 + 4], s6 = spin6[r * 6 + 5];
        zgemm_nn(N, P12 + ((size_t)tf * 5 + ip[r]) * N2, BLK(prop_row, ti, s5, s6, N), A);
        zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
        zgemm_nn(N, B, BLK(prop_diag, ti, s1, s2, N), A);
        zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
        cplx s = had_xcy(N, B, BLK(prop_row, ti, s3, s2, N));
        cplx v = cmul(fcoef(coef, r), s);
        rows[((size_t)ti * 256 + bx) * 2 + 0] = v.re;
        rows[((size_t)ti * 256 + bx) * 2 + 1] = v.im;
      }
    free(A);
  }
  for (int ti = 0; ti < Nt; ti++)
    for (int ico = 0; ico < 4; ico++) {
      double re = 0.0, im = 0.0;
      for (int is = 0; is < 64; is++) {
        re += rows[((size_t)ti * 256 + ico * 64 + is) * 2 + 0];
        im += rows[((size_t)ti * 256 + ico * 64 + is) * 2 + 1];
      }
      corr[((size_t)ti * 4 + ico) * 2 + 0] = re;
      corr[((size_t)ti * 4 + ico) * 2 + 1] = im;
    }
}

/* -------------------------------------------------------------------- pipi */
/* Square: lib/calculate_pipi_square_core.h.  Phi3(tf) tau(tf,tf)_{s3s4} Phi4(tf)
 * tau(tf,ti)_{s5s6} Phi2(ti) tau(ti,ti)_{s1s2} Phi1(ti), closed with conj tau(tf,ti)_{s3s2}. */
static cplx pipi_square(int N, int tf, int ti, const int16_t* s, const double* prop_row, const double* prop_diag,
                        const cplx* P1, const cplx* P2, const cplx* P3, const cplx* P4, cplx* A, cplx* B) {
  size_t N2 = (size_t)N * N;
  zgemm_nn(N, P3 + (size_t)tf * N2, BLK(prop_diag, tf, s[2], s[3], N), A);
  zgemm_nn(N, A, P4 + (size_t)tf * N2, B);
  zgemm_nn(N, B, BLK(prop_row, ti, s[4], s[5], N), A);
  zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
  zgemm_nn(N, B, BLK(prop_diag, ti, s[0], s[1], N), A);
  zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
  return had_xcy(N, B, BLK(prop_row, ti, s[2], s[1], N));
}

/* Double triangle: lib/calculate_pipi_doubleTriangle_core.h.  Phi3(tf) tau(tf,tf)_{s5s6}
 * Phi4(tf) tau(tf,ti)_{s1s2} Phi1(ti) tau(ti,ti)_{s3s4} Phi2(ti), closed with conj tau(tf,ti)_{s5s4}. */
static cplx pipi_dtri(int N, int tf, int ti, const int16_t* s, const double* prop_row, const double* prop_diag,
                      const cplx* P1, const cplx* P2, const cplx* P3, const cplx* P4, cplx* A, cplx* B) {
  size_t N2 = (size_t)N * N;
  zgemm_nn(N, P3 + (size_t)tf * N2, BLK(prop_diag, tf, s[4], s[5], N), A);
  zgemm_nn(N, A, P4 + (size_t)tf * N2, B);
  zgemm_nn(N, B, BLK(prop_row, ti, s[0], s[1], N), A);
  zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
  zgemm_nn(N, B, BLK(prop_diag, ti, s[2], s[3], N), A);
  zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
  return had_xcy(N, B, BLK(prop_row, ti, s[4], s[3], N));
}

/* Horizontal double triangle: lib/calculate_pipi_doubleTriangleHor_core.h.  All tau = tau(tf,ti):
 * Phi3(tf) tau_{s1s2} Phi1(ti) (tau_{s3s2})^dagger Phi4(tf) tau_{s3s4} Phi2(ti), closed with conj tau_{s1s4}. */
static cplx pipi_dtri_hor(int N, int tf, int ti, const int16_t* s, const double* prop_row,
                          const cplx* P1, const cplx* P2, const cplx* P3, const cplx* P4, cplx* A, cplx* B) {
  size_t N2 = (size_t)N * N;
  zgemm_nn(N, P3 + (size_t)tf * N2, BLK(prop_row, ti, s[0], s[1], N), A);
  zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
  zgemm_nc(N, B, BLK(prop_row, ti, s[2], s[1], N), A);
  zgemm_nn(N, A, P4 + (size_t)tf * N2, B);
  zgemm_nn(N, B, BLK(prop_row, ti, s[2], s[3], N), A);
  zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
  return had_xcy(N, B, BLK(prop_row, ti, s[0], s[3], N));
}

/* Star / fish twin traces: lib/calculate_pipi_starfish_core.h, spin is = s1*4+s2.
 * tr1 = sum (Pa(tf) tau_{s1s2} P1(ti)) (.) conj tau_{s1s2};  tr2 likewise with (Pb, P2). */
static void pipi_starfish(int N, int tf, int ti, int is, const double* prop_row, const cplx* P1, const cplx* P2,
                          const cplx* Pa, const cplx* Pb, cplx* A, cplx* B, cplx* tr1, cplx* tr2) {
  size_t N2 = (size_t)N * N;
  int s1 = is / 4, s2 = is % 4;
  const cplx* T = BLK(prop_row, ti, s1, s2, N);
  zgemm_nn(N, Pa + (size_t)tf * N2, T, A);
  zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
  *tr1 = had_xcy(N, B, T);
  zgemm_nn(N, Pb + (size_t)tf * N2, T, A);
  zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
  *tr2 = had_xcy(N, B, T);
}

/* One t_sink row of run_ContractPiPi (iso=1) / run_ContractPiPi_I0 (iso=0)
 * (lib/contract_kernels_pipi.cu:170-323 and :327-502).
 * sq/dt/dth: [ti][256] coefficient-weighted rows (dth only for iso 0, may be NULL);
 * star/fish: [2][ti][16] twin traces; corr[ti][5] with the isospin weights. */
void oracle_pipi_row(int N, int Nt, int tf, int iso, const double* prop_row, const double* prop_diag,
                     const double* momP1, const double* momP2, const double* momP3, const double* momP4,
                     const int16_t* sq_spin, const float* sq_coef, const int16_t* dt_spin, const float* dt_coef,
                     const int16_t* dth_spin, const float* dth_coef,
                     double* sq, double* dt, double* dth, double* star, double* fish, double* corr) {
  const cplx *P1 = (const cplx*)momP1, *P2 = (const cplx*)momP2, *P3 = (const cplx*)momP3, *P4 = (const cplx*)momP4;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* A = scratch(N, 2);
    cplx* B = A + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int bx = 0; bx < 256; bx++) {
        cplx v = cmul(fcoef(sq_coef, bx), pipi_square(N, tf, ti, sq_spin + bx * 6, prop_row, prop_diag, P1, P2, P3, P4, A, B));
        sq[((size_t)ti * 256 + bx) * 2] = v.re; sq[((size_t)ti * 256 + bx) * 2 + 1] = v.im;
        v = cmul(fcoef(dt_coef, bx), pipi_dtri(N, tf, ti, dt_spin + bx * 6, prop_row, prop_diag, P1, P2, P3, P4, A, B));
        dt[((size_t)ti * 256 + bx) * 2] = v.re; dt[((size_t)ti * 256 + bx) * 2 + 1] = v.im;
        if (iso == 0) {
          v = cmul(fcoef(dth_coef, bx), pipi_dtri_hor(N, tf, ti, dth_spin + bx * 4, prop_row, P1, P2, P3, P4, A, B));
          dth[((size_t)ti * 256 + bx) * 2] = v.re; dth[((size_t)ti * 256 + bx) * 2 + 1] = v.im;
        }
      }
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int is = 0; is < 16; is++) {
        cplx t1, t2;
        /* star: (P3, P4) as passed; fish: P3 and P4 swapped (contract_kernels_pipi.cu:222-223) */
        pipi_starfish(N, tf, ti, is, prop_row, P1, P2, P4, P3, A, B, &t1, &t2);
        star[(0 * (size_t)Nt * 16 + ti * 16 + is) * 2] = t1.re; star[(0 * (size_t)Nt * 16 + ti * 16 + is) * 2 + 1] = t1.im;
        star[(1 * (size_t)Nt * 16 + ti * 16 + is) * 2] = t2.re; star[(1 * (size_t)Nt * 16 + ti * 16 + is) * 2 + 1] = t2.im;
        pipi_starfish(N, tf, ti, is, prop_row, P1, P2, P3, P4, A, B, &t1, &t2);
        fish[(0 * (size_t)Nt * 16 + ti * 16 + is) * 2] = t1.re; fish[(0 * (size_t)Nt * 16 + ti * 16 + is) * 2 + 1] = t1.im;
        fish[(1 * (size_t)Nt * 16 + ti * 16 + is) * 2] = t2.re; fish[(1 * (size_t)Nt * 16 + ti * 16 + is) * 2 + 1] = t2.im;
      }
    free(A);
  }
  for (int ti = 0; ti < Nt; ti++) {
    double sqr = 0, sqi = 0, dtr = 0, dti = 0, hr = 0, hi = 0;
    for (int is = 0; is < 256; is++) {
      sqr += sq[((size_t)ti * 256 + is) * 2]; sqi += sq[((size_t)ti * 256 + is) * 2 + 1];
      dtr += dt[((size_t)ti * 256 + is) * 2]; dti += dt[((size_t)ti * 256 + is) * 2 + 1];
      if (iso == 0) { hr += dth[((size_t)ti * 256 + is) * 2]; hi += dth[((size_t)ti * 256 + is) * 2 + 1]; }
    }
    double sr[2] = {0, 0}, si[2] = {0, 0}, fr[2] = {0, 0}, fi[2] = {0, 0};
    for (int is = 0; is < 16; is++)
      for (int tr = 0; tr < 2; tr++) {
        sr[tr] += star[((size_t)tr * Nt * 16 + ti * 16 + is) * 2]; si[tr] += star[((size_t)tr * Nt * 16 + ti * 16 + is) * 2 + 1];
        fr[tr] += fish[((size_t)tr * Nt * 16 + ti * 16 + is) * 2]; fi[tr] += fish[((size_t)tr * Nt * 16 + ti * 16 + is) * 2 + 1];
      }
    double str = sr[0] * sr[1] - si[0] * si[1], sti = sr[0] * si[1] + si[0] * sr[1];
    double ftr = fr[0] * fr[1] - fi[0] * fi[1], fti = fr[0] * fi[1] + fi[0] * fr[1];
    double* c = corr + (size_t)ti * 10;
    if (iso == 1) { /* contract_kernels_pipi.cu:288-303 */
      c[0] = -2. * sqr; c[1] = -2. * sqi;
      c[2] = 2. * dtr;  c[3] = 2. * dti;
      c[4] = -str;      c[5] = -sti;
      c[6] = ftr;       c[7] = fti;
      c[8] = 0.;        c[9] = 0.;
    } else {          /* contract_kernels_pipi.cu:463-478 */
      c[0] = (-1. / 3.) * sqr; c[1] = (-1. / 3.) * sqi;
      c[2] = -(1. / 3.) * dtr; c[3] = -(1. / 3.) * dti;
      c[4] = str;              c[5] = sti;
      c[6] = ftr;              c[7] = fti;
      c[8] = -(5. / 3.) * hr;  c[9] = -(5. / 3.) * hi;
    }
  }
}

/* -------------------------------------------------------------- loop-unity */
/* lib/calculate_loop_unity_core.h + lib/contract_kernels_loop_unity.cu:45-96:
 * rows[t][4] = trace(tau(t,t)_{ss} Phi(t)), loop[t] = sum over s. */
void oracle_loop_unity(int N, int Nt, const double* prop_diag, const double* mom, double* rows, double* loop) {
  const cplx* P = (const cplx*)mom;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* A = scratch(N, 1);
    #pragma omp for schedule(dynamic) collapse(2)
    for (int t = 0; t < Nt; t++)
      for (int s = 0; s < 4; s++) {
        zgemm_nn(N, BLK(prop_diag, t, s, s, N), P + (size_t)t * N2, A);
        double re = 0.0, im = 0.0;
        for (int i = 0; i < N; i++) { re += A[(size_t)i * N + i].re; im += A[(size_t)i * N + i].im; }
        rows[((size_t)t * 4 + s) * 2] = re;
        rows[((size_t)t * 4 + s) * 2 + 1] = im;
      }
    free(A);
  }
  for (int t = 0; t < Nt; t++) {
    double re = 0.0, im = 0.0;
    for (int s = 0; s < 4; s++) { re += rows[((size_t)t * 4 + s) * 2]; im += rows[((size_t)t * 4 + s) * 2 + 1]; }
    loop[(size_t)t * 2] = re;
    loop[(size_t)t * 2 + 1] = im;
  }
}

/* ------------------------------------------------------------------- sigma */
/* lib/calculate_sigma_one_fish_core.h + lib/contract_kernels_sigma.cu:69-123:
 * T1 = tau(tf,ti)_{s3s4} Phix2_rp(ti), T2 = Phix2_lp(tf) tau(tf,ti)_{s2s1},
 * row = coef * sum conj(T2) (.) T1; corr[ti][4] sums 16 spin rows per (lp, rp). */
void oracle_sigma_row(int N, int Nt, int tf, const double* prop_row, const double* mom2,
                      const int16_t* spin, const int16_t* lprp, const float* coef, double* rows, double* corr) {
  const cplx* mom = (const cplx*)mom2;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* T1 = scratch(N, 2);
    cplx* T2 = T1 + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int bx = 0; bx < 64; bx++) {
        int s1 = spin[bx * 4], s2 = spin[bx * 4 + 1], s3 = spin[bx * 4 + 2], s4 = spin[bx * 4 + 3];
        int lp = lprp[bx * 2], rp = lprp[bx * 2 + 1];
        zgemm_nn(N, BLK(prop_row, ti, s3, s4, N), mom + ((size_t)ti * 2 + rp) * N2, T1);
        zgemm_nn(N, mom + ((size_t)tf * 2 + lp) * N2, BLK(prop_row, ti, s2, s1, N), T2);
        cplx v = cmul(fcoef(coef, bx), had_xcy(N, T1, T2));
        rows[((size_t)ti * 64 + bx) * 2] = v.re;
        rows[((size_t)ti * 64 + bx) * 2 + 1] = v.im;
      }
    free(T1);
  }
  for (int ti = 0; ti < Nt; ti++)
    for (int ico = 0; ico < 4; ico++) {
      double re = 0.0, im = 0.0;
      for (int is = 0; is < 16; is++) {
        re += rows[((size_t)ti * 64 + ico * 16 + is) * 2];
        im += rows[((size_t)ti * 64 + ico * 16 + is) * 2 + 1];
      }
      corr[((size_t)ti * 4 + ico) * 2] = re;
      corr[((size_t)ti * 4 + ico) * 2 + 1] = im;
    }
}

/* ---------------------------------------------------------------- sigma-pipi */
/* Horizontal fish: lib/calculate_sigmapi_hor_fish_core.h + contract_kernels_sigmapi.cu:97-138.
 * tmp = Phi_P2(t) tau(t,t)_{s1s2} Phi_P1(t), row = coef * sum tmp (.) conj tau(t,t)_{s1s2}. */
void oracle_sigmapi_hor_fish(int N, int Nt, const double* prop_diag, const double* momP1, const double* momP2,
                             const int16_t* spin2, const float* coef, double* rows, double* corr) {
  const cplx *P1 = (const cplx*)momP1, *P2 = (const cplx*)momP2;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* A = scratch(N, 2);
    cplx* B = A + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int t = 0; t < Nt; t++)
      for (int bx = 0; bx < 16; bx++) {
        int s1 = spin2[bx * 2], s2 = spin2[bx * 2 + 1];
        zgemm_nn(N, P2 + (size_t)t * N2, BLK(prop_diag, t, s1, s2, N), A);
        zgemm_nn(N, A, P1 + (size_t)t * N2, B);
        cplx v = cmul(fcoef(coef, bx), had_xcy(N, B, BLK(prop_diag, t, s1, s2, N)));
        rows[((size_t)t * 16 + bx) * 2] = v.re;
        rows[((size_t)t * 16 + bx) * 2 + 1] = v.im;
      }
    free(A);
  }
  for (int t = 0; t < Nt; t++) {
    double re = 0.0, im = 0.0;
    for (int is = 0; is < 16; is++) { re += rows[((size_t)t * 16 + is) * 2]; im += rows[((size_t)t * 16 + is) * 2 + 1]; }
    corr[(size_t)t * 2] = re;
    corr[(size_t)t * 2 + 1] = im;
  }
}

/* Triangle: lib/calculate_sigmapi_triangle_core.h + contract_kernels_sigmapi.cu:140-185.
 * Phix2_ip(tf) tau(tf,ti)_{s2s3} Phi_P2(ti) tau(ti,ti)_{s4s5} Phi_P1(ti), closed with
 * conj tau(tf,ti)_{s1s5}.  rows[ti][128], corr[ti][2] (sum of 64 rows per ip). */
void oracle_sigmapi_triangle_row(int N, int Nt, int tf, const double* prop_row, const double* prop_diag,
                                 const double* momP1, const double* momP2, const double* mom2P1P2,
                                 const int16_t* spin5, const int16_t* ip, const float* coef,
                                 double* rows, double* corr) {
  const cplx *P1 = (const cplx*)momP1, *P2 = (const cplx*)momP2, *P12 = (const cplx*)mom2P1P2;
  size_t N2 = (size_t)N * N;
  #pragma omp parallel
  {
    cplx* A = scratch(N, 2);
    cplx* B = A + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int ti = 0; ti < Nt; ti++)
      for (int bx = 0; bx < 128; bx++) {
        const int16_t* s = spin5 + bx * 5;
        zgemm_nn(N, P12 + ((size_t)tf * 2 + ip[bx]) * N2, BLK(prop_row, ti, s[1], s[2], N), A);
        zgemm_nn(N, A, P2 + (size_t)ti * N2, B);
        zgemm_nn(N, B, BLK(prop_diag, ti, s[3], s[4], N), A);
        zgemm_nn(N, A, P1 + (size_t)ti * N2, B);
        cplx v = cmul(fcoef(coef, bx), had_xcy(N, B, BLK(prop_row, ti, s[0], s[4], N)));
        rows[((size_t)ti * 128 + bx) * 2] = v.re;
        rows[((size_t)ti * 128 + bx) * 2 + 1] = v.im;
      }
    free(A);
  }
  for (int ti = 0; ti < Nt; ti++)
    for (int iop = 0; iop < 2; iop++) {
      double re = 0.0, im = 0.0;
      for (int is = 0; is < 64; is++) {
        re += rows[((size_t)ti * 128 + iop * 64 + is) * 2];
        im += rows[((size_t)ti * 128 + iop * 64 + is) * 2 + 1];
      }
      corr[((size_t)ti * 2 + iop) * 2] = re;
      corr[((size_t)ti * 2 + iop) * 2 + 1] = im;
    }
}

/* ------------------------------------------------------------- host helpers */
/* Source-time average of the dumpData functions (lib/contract.cpp:621-631 and the
 * other dumpData bodies): avg[dt][c] = 1/Nt sum_ti corr[(ti+dt)%Nt][ti][c]. */
void oracle_source_average(int Nt, int ncorr, const double* corr, double* avg) {
  for (int dt = 0; dt < Nt; dt++)
    for (int c = 0; c < ncorr; c++) {
      double re = 0.0, im = 0.0;
      for (int ti = 0; ti < Nt; ti++) {
        int tf = (ti + dt) % Nt;
        re += corr[(((size_t)tf * Nt + ti) * ncorr + c) * 2];
        im += corr[(((size_t)tf * Nt + ti) * ncorr + c) * 2 + 1];
      }
      avg[((size_t)dt * ncorr + c) * 2] = re / Nt;
      avg[((size_t)dt * ncorr + c) * 2 + 1] = im / Nt;
    }
}

/* Perambulator file payload -> library layout (lib/contract.cpp:524-534):
 * prop[t1][t2][s1][s2][v1][v2] = file[s1][v1][t1][s2][v2][t2]. */
void oracle_reorder_prop(int N, int Nt, const double* file, double* prop) {
  for (int t1 = 0; t1 < Nt; t1++)
    for (int t2 = 0; t2 < Nt; t2++)
      for (int s1 = 0; s1 < 4; s1++)
        for (int s2 = 0; s2 < 4; s2++)
          for (int v1 = 0; v1 < N; v1++)
            for (int v2 = 0; v2 < N; v2++) {
              size_t d = ((((((size_t)t1 * Nt + t2) * 4 + s1) * 4 + s2) * N + v1) * N + v2) * 2;
              size_t s = ((((((size_t)s1 * N + v1) * Nt + t1) * 4 + s2) * N + v2) * Nt + t2) * 2;
              prop[d] = file[s];
              prop[d + 1] = file[s + 1];
            }
}

/* tau(t,t) gather of LapH_prop::copyToDeviceExtraDiag (lib/contract.cpp:559-565). */
void oracle_prop_diag(int N, int Nt, const double* prop, double* diag) {
  size_t blk = (size_t)16 * N * N * 2;
  for (int t = 0; t < Nt; t++)
    memcpy(diag + (size_t)t * blk, prop + ((size_t)t * Nt + t) * blk, blk * sizeof(double));
}

/* ------------------------------------------------------ generic two-sided */
/* The rho-rho / sigma-sigma row form with an explicit row list (same chain
 * order as lib/calculate_rho_core.h:40-152, each row recomputing both products):
 * rowvals[ti-ti0][r] = coef_r * sum conj(Phi_R(tf) tau(tf,ti)_{ab}) (.) (tau(tf,ti)_{cd} Phi_L(ti)).
 * rows[r] = (a, b, c, d, L, R); phi [Nt][nphi][N][N]. */
void oracle_twosided(int N, int Nt, int tf, int ti0, int ti1, const double* prop_row, const double* phi, int nphi,
                     int nrows, const int16_t* rows, const float* coef, double* rowvals) {
  const cplx* ph = (const cplx*)phi;
  size_t N2 = (size_t)N * N;
  int nti = ti1 - ti0;
  (void)Nt;
  #pragma omp parallel
  {
    cplx* T1 = scratch(N, 2);
    cplx* T2 = T1 + N2;
    #pragma omp for schedule(dynamic) collapse(2)
    for (int k = 0; k < nti; k++)
      for (int r = 0; r < nrows; r++) {
        int ti = ti0 + k;
        const int16_t* w = rows + 6 * r;
        zgemm_nn(N, BLK(prop_row, ti, w[2], w[3], N), ph + ((size_t)ti * nphi + w[4]) * N2, T1);
        zgemm_nn(N, ph + ((size_t)tf * nphi + w[5]) * N2, BLK(prop_row, ti, w[0], w[1], N), T2);
        cplx v = cmul(fcoef(coef, r), had_xcy(N, T1, T2));
        rowvals[((size_t)k * nrows + r) * 2] = v.re;
        rowvals[((size_t)k * nrows + r) * 2 + 1] = v.im;
      }
    free(T1);
  }
}
