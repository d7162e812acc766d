/*
 * ctr.h -- C ABI of the GB300 distillation contraction engine (libctr.so).
 *
 * Plain C: pointers, sizes and int status codes.  Every routine returns CTR_OK
 * (0) or an error code; ctr_last_error() gives the message of the last failure
 * on the calling thread.  Nothing here terminates the process (the C++ layer in
 * interface.h/contract.h turns errors into the reference's ABORT behaviour).
 *
 * Data are complex128 stored as interleaved (re, im) doubles, in the layouts of
 * the reference library:
 *   perambulator tau(t1,t2)_{s1 s2}^{v1 v2}: [t1][t2][s1][s2][v1][v2]
 *       (lib/contract.cpp:531-534).  "prop rows" = the rows t1 in [tf_begin,
 *       tf_end) of that array, i.e. a pointer to tau(tf_begin, 0).
 *   tau(t,t) ("prop diag"): [t][s1][s2][v1][v2]   (lib/contract.cpp:565)
 *   elementals Phi: [t][op][r][c]  with op count 5 (rho), 2 (sigma x2) or 1
 *       (lib/interface.cpp:25, :258, :85).
 * Device pointers must be 16-byte aligned.  "stream" is a cudaStream_t (NULL =
 * legacy default stream).  Calls are asynchronous on that stream unless noted.
 *
 * Engines:
 *   CTR_ENGINE_FP64   plain FP64 (the drop-in; <= 1e-12 relative to the oracle)
 *   CTR_ENGINE_SPLIT  split-precision tensor-core form: FP64 operands sliced
 *                     into BF16 pieces, tcgen05 MMA with FP32 accumulation in
 *                     TMEM, float-float recombination (<= 1e-9 relative).
 */
#ifndef CTR_H
#define CTR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTR_OK 0
#define CTR_ERR_ARG 1          /* invalid argument (size, pointer, index) */
#define CTR_ERR_CUDA 2         /* a CUDA runtime call failed */
#define CTR_ERR_ALLOC 3        /* device or host allocation failed */
#define CTR_ERR_UNSUPPORTED 4  /* device is not sm_103 / feature not built */
#define CTR_ERR_TIMEOUT 5      /* a bounded device-side wait gave up */
#define CTR_ERR_IO 6           /* file missing, truncated or malformed */

#define CTR_ENGINE_FP64 0
#define CTR_ENGINE_SPLIT 1

int ctr_version(void);
const char* ctr_error_string(int code);
const char* ctr_last_error(void);

/* Select the CUDA device and check it is a Blackwell sm_103 part
 * (replaces initDevice/initContract's device handling, lib/contract.cpp:25-70). */
int ctr_device_init(int device);

/* ---------------------------------------------------------------- tables
 * The diagram tables of include/constants_*.h, generated by the library from
 * the gamma matrices (devTools/comb_*.cpp).  Caller-owned host arrays. */
int ctr_table_rho(int16_t* spin /*768x4*/, int16_t* lp_rp /*768x2*/, float* coef /*768x2*/);
int ctr_table_rhopi(int16_t* spin /*768x6*/, int16_t* ip /*768*/, float* coef /*768x2*/);
int ctr_table_pipi(int16_t* sq_spin /*256x6*/, float* sq_coef /*256x2*/, int16_t* dt_spin /*256x6*/,
                   float* dt_coef /*256x2*/, int16_t* dth_spin /*256x4*/, float* dth_coef /*256x2*/);
int ctr_table_sigma(int16_t* spin /*64x4*/, int16_t* lp_rp /*64x2*/, float* coef /*64x2*/);
int ctr_table_sigmapi(int16_t* hf_spin /*16x2*/, float* hf_coef /*16x2*/, int16_t* tri_spin /*128x5*/,
                      int16_t* tri_ip /*128*/, float* tri_coef /*128x2*/);

/* ------------------------------------------------------ rho-type diagrams
 * Generic two-sided contraction, the form of the rho-rho and sigma-sigma
 * kernels (lib/calculate_rho_core.h, lib/calculate_sigma_one_fish_core.h):
 *   row(tf,ti,r) = coef_r * sum_ij conj( (Phi_{R_r}(tf) tau(tf,ti)_{a_r b_r})_ij )
 *                                    * (tau(tf,ti)_{c_r d_r} Phi_{L_r}(ti))_ij
 *   out[tf][ti][o] = sum over rows r with out_index[r] == o (ascending r).
 * rows: host array [nrows][6] = (a, b, c, d, L, R); coef host [nrows][2];
 * out_index host [nrows].  phi: device [Nt][nphi][N][N].  out: device
 * [tf_end-tf_begin][Nt][nout] complex. */
int ctr_twosided(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
                 const double* phi, int nphi, int nrows, const int16_t* rows, const float* coef,
                 const int32_t* out_index, int nout, double* out, void* stream);

/* rho-rho: run_ContractRho for t_sink rows [tf_begin, tf_end) (lib/contract_kernels_rho.cu:69-138).
 * mom5 device [Nt][5][N][N]; corr device [tf_end-tf_begin][Nt][16][3]. */
int ctr_rho(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
            const double* mom5, double* corr, void* stream);

/* sigma-sigma one-fish: run_ContractSigma (lib/contract_kernels_sigma.cu:69-147).
 * mom2 device [Nt][2][N][N]; corr device [tf_end-tf_begin][Nt][4]. */
int ctr_sigma(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
              const double* mom2, double* corr, void* stream);

/* ------------------------------------------------------------ chain diagrams
 * prop_diag: tau(t,t) [Nt][4][4][N][N] (the reference's "extra" device buffer,
 * lib/contract.cpp:549-570).  Elementals [Nt][N][N] unless noted.  With
 * CTR_ENGINE_SPLIT every block product of the chains runs on the tensor-core
 * split engine (Nev <= 128); the closing traces and the loop-unity traces are
 * FP64 on both engines (except the rho -> pi pi / sigma -> pi pi set call's, below). */

/* rho -> pi pi for gamma_idir (run_ContractRhoPi, lib/contract_kernels_rhopi.cu:64-137):
 * mom5_p1p2 [Nt][5][N][N]; corr [tf_end-tf_begin][Nt][4] (one entry per rho operator). */
int ctr_rhopi(int engine, int nev, int nt, int tf_begin, int tf_end, int idir, const double* prop_rows,
              const double* prop_diag, const double* mom_p1, const double* mom_p2, const double* mom5_p1p2,
              double* corr, void* stream);

/* pi pi -> pi pi (run_ContractPiPi, isospin 1; run_ContractPiPi_I0, isospin 0;
 * lib/contract_kernels_pipi.cu:170-502): corr [rows][Nt][5] = square, double triangle, star,
 * fish, horizontal double triangle, with the isospin weights of the reference. */
int ctr_pipi(int engine, int nev, int nt, int tf_begin, int tf_end, int isospin, const double* prop_rows,
             const double* prop_diag, const double* p1, const double* p2, const double* p3, const double* p4,
             double* corr, void* stream);

/* pi pi for many momentum sets in one call (a batched form of ctr_pipi, no counterpart in the
 * reference, which takes one set of four elementals per call): phi [Nt][nphi][N][N] holds every
 * elemental; set s contracts with P1..P4 = phi[:, sets[4s + k]] (k = 0..3, host array
 * [nset][4]).  corr [nset][tf_end-tf_begin][Nt][5], each set's entries as ctr_pipi gives them.
 * Block products and traces that several sets share (e.g. Phi(q) tau, tau Phi(q) tau^dag for the
 * sets (p, -p) and (-p, p)) are computed once; every stage of a pair batch is one launch. */
int ctr_pipi_sets(int engine, int nev, int nt, int tf_begin, int tf_end, int isospin, const double* prop_rows,
                  const double* prop_diag, const double* phi, int nphi, int nset, const int32_t* sets, double* corr,
                  void* stream);

/* rho -> pi pi (the three polarisations) and sigma -> pi pi (triangle, horizontal fish) for
 * many pion momentum pairs in one call (a batched form of ctr_rhopi and ctr_sigmapi, no
 * counterpart in the reference, which takes one pair per call): set s uses
 * P1 = phi[:, sets[2s]], P2 = phi[:, sets[2s + 1]] (phi [Nt][nphi][N][N], sets host [nset][2]);
 * the sink operators mom5_p1p2 [Nt][5][N][N] (rho) and mom2_p1p2 [Nt][2][N][N] (sigma) are
 * the same for every set.  Both families contract X = tau(tf,ti) G R(ti),
 * R = Phi_P2 taud Phi_P1: X is computed once per set and pair and multiplied by all the
 * sink operators the outputs need in one stacked launch.  Outputs (each may be NULL; then
 * its operands may be NULL too): rhopi [nset][3][tf_end-tf_begin][Nt][4] (idir 0..2, as
 * ctr_rhopi), triangle [nset][tf_end-tf_begin][Nt][2] and hor_fish [nset][Nt] (as ctr_sigmapi).
 * On the split engine the rho -> pi pi and triangle traces of a pair run as Gram products
 * on the tensor cores (the tuning knob "chains.trace_form" = 1, the default; each entry
 * within the engine's per-entry tolerance); with the knob forced to 0 they run as FP64
 * traces and every set's entries are bitwise those of its own ctr_rhopi / ctr_sigmapi. */
int ctr_rhopi_sigmapi_sets(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
                           const double* prop_diag, const double* phi, int nphi, const double* mom5_p1p2,
                           const double* mom2_p1p2, int nset, const int32_t* sets, double* rhopi, double* triangle,
                           double* hor_fish, void* stream);

/* Loop with unit spin structure (run_ContractLoopUnity, lib/contract_kernels_loop_unity.cu:45-107):
 * loop[t] = sum_s Tr[tau(t,t)_{ss} Phi(t)]. */
int ctr_loop_unity(int engine, int nev, int nt, const double* prop_diag, const double* mom, double* loop,
                   void* stream);

/* sigma -> pi pi (run_ContractSigmaPi_fish_hor and run_ContractSigmaPi_triangle,
 * lib/contract_kernels_sigmapi.cu:97-222): hor_fish [Nt] (may be NULL), triangle
 * [rows][Nt][2] (may be NULL); mom2_p1p2 [Nt][2][N][N]. */
int ctr_sigmapi(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
                const double* prop_diag, const double* mom_p1, const double* mom_p2, const double* mom2_p1p2,
                double* hor_fish, double* triangle, void* stream);

/* ------------------------------------------------ host-level API (status codes)
 * The non-terminating forms of the reference's public API; interface.h and
 * contract.h wrap them and terminate on error as the reference does.
 * single != 0: prop holds complex64 (float) data, widened on the device; the
 * rho and sigma contractions then run on the split engine. */
int ctr_contract_init(int nev, int nt, int dev);             /* initContract (lib/contract.cpp:58-70) */
int ctr_contract_destroy(void);                              /* destroyContract (lib/contract.cpp:72-88) */
/* readPropH (lib/contract.cpp:91-160): 100-byte name, uint32 Nt, uint32 Nvec, complex128 payload in
 * (s1,v1,t1,s2,v2,t2) order -> host_out [t1][t2][s1][s2][v1][v2] (complex64 if single);
 * CTR_ERR_IO on a missing/short file or a size mismatch. */
int ctr_read_prop(const char* path, int nev, int nt, int single, void* host_out);
/* Momentum list (lib/catchOpts.cpp:108-233): momcomb lines of nmom*3 integers, nmom in {1,2,4};
 * p [4][3][momcomb]; for nmom = 2 the third momentum is p1 + p2. */
int ctr_read_momenta(const char* path, int nmom, int momcomb, int* p);
/* calculate* bodies (lib/interface.cpp:6-390): host inputs, results appended to outfile. */
int ctr_calculate_rho(int nev, int nt, const void* prop, const double* mom, int single, const char* outfile);
int ctr_calculate_rhopi(int idir, int nev, int nt, const void* prop, const double* p1, const double* p2,
                        const double* p1p2, int single, const char* outfile);
int ctr_calculate_pipi(int nev, int nt, const void* prop, const double* p1, const double* p2, const double* p3,
                       const double* p4, int single, const char* outfile, int isospin);
int ctr_calculate_sigma(int nev, int nt, const void* prop, const double* mom, int single, const char* outfile);
int ctr_calculate_sigmapi(int nev, int nt, const void* prop, const double* p1, const double* p2,
                          const double* p1p2, int single, const char* outfile);

/* Batched complex block products c[b] = x[b] * y[b] (nev x nev, row-major
 * complex128, device pointers given in host arrays of length nbatch).  The unit
 * both engines build the diagram chains from (the 25x25-tiled GEMM loops of every
 * lib/calculate_*_core.h). */
int ctr_zgemm_batched(int engine, int nev, int nbatch, const double* const* x, const double* const* y,
                      double* const* c, void* stream);

/* Multi-term block products, the unit the chain diagrams are built from:
 * c = sum_{q < nterm} w_q op(a_q) op(b_q), op = conjugate transpose where bit q
 * (a_q) / bit 4+q (b_q) of flags is set; nev x nev row-major complex128 device
 * blocks.  With CTR_ENGINE_SPLIT the weights must be real powers of two (the
 * gamma_5 signs of the tables) and nterm * nev <= 512. */
typedef struct {
  const double* a[4];
  const double* b[4];
  double* c;
  float wre[4], wim[4];
  int nterm;
  int flags;
} ctr_ztask;
int ctr_zgemm_tasks(int engine, int nev, int ntask, const ctr_ztask* tasks /* host */, void* stream);

/* Failure detection check (no counterpart in the reference, whose errors end
 * the process): every device-side wait of the library is bounded; when one
 * runs out, the kernel records an error code, finishes without hanging, and
 * the next synchronising call returns CTR_ERR_TIMEOUT while the context stays
 * usable.  This runs one such wait, on an mbarrier that nothing arrives at,
 * with a limit of timeout_ms (1..1000), and returns what a caller would see:
 * CTR_ERR_TIMEOUT.  Not recordable in a CUDA graph. */
int ctr_wait_probe(int timeout_ms, void* stream);

/* Tensor-pipe probe (no counterpart in the reference): one thread per SM issues
 * the split GEMM's per-chunk MMA schedule (hp = 0: the standard configuration,
 * 15 slice pairs x 2 MMAs of M128 N128 K16; hp = 1: the high-precision one,
 * 21 x 2 of M128 N96 K16), nchunk chunks back to back from shared-memory
 * operands that stay in place, with no operand copies and no epilogue.  Returns
 * the SM clocks per MMA and the BF16 TFLOP/s of the whole device: the ceiling
 * of the schedule by itself, against which the GEMM's own rate shows what its
 * operand pipeline and accumulator hand-off cost.  Not recordable in a graph. */
int ctr_mma_schedule_probe(int hp, int nchunk, double* clocks_per_mma, double* tflops, void* stream);

/* Diagnostics of the split engine: for one product x*y (nev x nev, device),
 * write the raw FP32 tensor-core accumulators before recombination, as
 * levels[8][nev][128] (Re levels 0, 1, 2, >=3, then Im; element (i,j) at
 * [a][j][i]), in units of the per-row / per-column power-of-two scales. */
int ctr_split_levels(int nev, const double* x, const double* y, float* levels, void* stream);

/* Allocation-free rho-rho for one t_sink row: the same correlators as
 * ctr_rho(CTR_ENGINE_FP64, nev, nt, tf, tf+1, prop_row, mom5, corr, stream),
 * for callers that cannot allocate device memory when they call (their memory
 * budget is held by a fixed pool, or they must not trigger the device-wide
 * synchronisation of cudaMalloc/cudaFree).  This entry point has no
 * counterpart in the reference.  Its only scratch is a fixed 32 MiB device
 * array inside the library (enough for Nev <= 114); larger Nev are rejected
 * with CTR_ERR_ARG.  A device reserves the array when the library's module
 * holding it is loaded there; with CUDA's default lazy module loading that is
 * the first ctr_rho_noalloc call on that device, which also looks up the
 * array's device address.  Make one such warm-up call at start-up, before any
 * stream capture, so that later calls find the array in place; the device then
 * holds it until the process exits.  Each call looks the address up again
 * (cheap once loaded), so a cudaDeviceReset in between is safe.  It calls no
 * cudaMalloc/cudaFree or other allocating routine and copies nothing from the
 * host: its task lists are built on the device.  All calls share the array, and
 * each call rewrites what it reads: calls whose work overlaps on the GPU
 * (different streams, or threads) race.
 * prop_row: tau(tf, .) [Nt][4][4][N][N]; mom5 [Nt][5][N][N]; corr [Nt][16][3]. */
int ctr_rho_noalloc(int nev, int nt, int tf, const double* prop_row, const double* mom5, double* corr,
                    void* stream);
/* Size in bytes of ctr_rho_noalloc's fixed device scratch array. */
size_t ctr_rho_noalloc_scratch_bytes(void);

/* Momentum elementals from Laplacian eigenvectors, as the reference drivers build
 * them before calling calculate* (tests/compute_rho.cpp:116-223; the same loops in
 * tests/compute_{rhopi,pipi_I0,pipi_I1,sigma,sigmapi}.cpp), for every time slice t
 * and momentum p, FP64:
 *   op 0: <v_r| e^{-ip.x} |v_c>                                   (plain)
 *   op 1: sum_j <D_j v_r| e^{-ip.x} |D_j v_c>                     (smeared)
 *   op 2+j: <v_r| e^{-ip.x} |D_j v_c> - <D_j v_r| e^{-ip.x} |v_c>  (j = x, y, z)
 * with <a|b> summed over the sites and colours of the slice, the phase
 * e^{-i 2 pi (x p_x/nx + y p_y/ny + z p_z/nz)}, and the covariant derivative
 * D_j v(x) = U_j(x) v(x + j) - U_j(x - j)^dag v(x - j), periodic.  (The reference
 * takes the derivative from the gwu-qcd library, which it does not ship.)
 * evec  : device [nt][nev][nz][ny][nx][3] complex128, eigenvector c of slice t
 *         (site x + nx (y + ny z), colour fastest)
 * links : device [nt][nz][ny][nx][3][3][3] complex128, U_j(x) of slice t
 *         (direction j, row, column); may be NULL when nops == 1
 * mom   : host [nmom][3] integer momenta
 * nops  : 1 (op 0 only) or 5
 * phi   : device [nmom][nops][nt][nev][nev] complex128: per momentum the layout
 *         the drivers pass to calculateRho ([op][t][r][c])
 * Scratch: the phase table and, for nops == 5, the derivatives of every
 * eigenvector (3 x the size of evec). */
int ctr_elementals(int nev, int nt, int nx, int ny, int nz, const double* evec, const double* links, int nmom,
                   const int* mom, int nops, double* phi, void* stream);

/* ------------------------------------------------ distillation-profile adjoint
 * The elementals enter the contractions as diag(f) Phi diag(f) for a real
 * per-eigenvector profile f (no counterpart in the reference, whose
 * elementals are fixed).  A chain is Tr[F_1 ... F_n], 2 <= n <= CTR_CHAIN_MAXF;
 * a factor is a perambulator block tau(a, b)_{s1 s2} of the full perambulator
 * prop [Nt][Nt][4][4][N][N], or a profiled elemental diag(f) phi[a][b] diag(f)
 * of phi [Nt][nphi][N][N], conjugate-transposed when dag != 0.  All arrays are
 * device complex128 except the host chain description (chain_off, factors, w).
 * Gradients are vector-Jacobian products: grad[k] += Re sum_c w_c d value_c / d f_k,
 * computed by reverse mode with recomputed prefix/suffix products; every f_k must
 * be nonzero.  engine selects where the chain products run (CTR_ENGINE_SPLIT: tensor
 * cores, Nev <= 128); the diagonal reductions and traces are FP64. */
#define CTR_FACTOR_TAU 0
#define CTR_FACTOR_PHI 1
#define CTR_CHAIN_MAXF 12
typedef struct {
  int32_t kind; /* CTR_FACTOR_TAU or CTR_FACTOR_PHI */
  int32_t dag;  /* conjugate transpose */
  int32_t a, b; /* tau: (t1, t2); phi: (t, op) */
  int32_t s1, s2; /* tau: spin block */
} ctr_factor;

/* dst[m] = diag(f) src[m] diag(f) for nmat matrices (device; dst may equal src). */
int ctr_apply_profile(int nev, long long nmat, const double* f, const double* src, double* dst, void* stream);

/* Generic chains: chain c has factors[chain_off[c] .. chain_off[c+1]) (host arrays), weight
 * w[c] (host complex, may be NULL when grad is NULL).  values [nchain] complex (device, may be
 * NULL); grad [N] real (device, accumulated into, may be NULL). */
int ctr_chain_adjoint(int engine, int nev, int nt, int nphi, const double* prop, const double* phi, const double* f,
                      int nchain, const int* chain_off, const ctr_factor* factors, const double* w, double* values,
                      double* grad, void* stream);

/* rho-rho (lib/calculate_rho_core.h): w [Nt][Nt][48] complex (device) weights the
 * correlators corr[tf][ti][o] of ctr_rho; entries with zero weight are skipped.
 * corr [Nt][Nt][48] (device, may be NULL): the forward correlators of the entries
 * computed (zero elsewhere); grad [N] (device, may be NULL, accumulated into).
 * prop: full perambulator; mom5 [Nt][5][N][N]; f [N] device. */
int ctr_rho_profile_vjp(int engine, int nev, int nt, const double* prop, const double* mom5, const double* f,
                        const double* w, double* corr, double* grad, void* stream);

/* pi pi (lib/contract_kernels_pipi.cu:170-502): w [Nt][Nt][5] complex (device) weights the
 * isospin-weighted slots (square, double triangle, star, fish, horizontal double triangle)
 * of ctr_pipi; pairs whose weights are zero are skipped.  corr [Nt][Nt][5] (device, may be
 * NULL): the forward correlators of the pairs computed (zero elsewhere); grad [N] (device,
 * may be NULL, accumulated into). */
int ctr_pipi_profile_vjp(int engine, int nev, int nt, int isospin, const double* prop, const double* p1,
                         const double* p2, const double* p3, const double* p4, const double* f, const double* w,
                         double* corr, double* grad, void* stream);

/* On-device source-time average of the dumpData routines (lib/contract.cpp:616-643):
 * avg[dt][c] = scale/Nt * sum_ti corr[(ti+dt)%Nt][ti][c]; corr device [Nt][Nt][ncorr]. */
int ctr_source_average(int nt, int ncorr, const double* corr, double scale, double* avg, void* stream);

/* 1 when the split-precision tensor-core engine is compiled in. */
int ctr_split_available(void);

/* Per-entry accuracy control of the split engine (two-sided rho/sigma/ctr_twosided
 * contractions and the chain families).  Each correlator entry carries an error
 * estimate eps * sum_r |coef_r| sum_ij |A_r(i,j)|_1 |B_r(i,j)|_1 over its closing
 * traces (|z|_1 = |Re z| + |Im z|); entries whose estimate exceeds rel_tol * |entry|
 * -- those with heavy cancellation -- are recomputed (two-sided form: their spin rows
 * on the high-precision split configuration; chains: their (t_sink, t_src) pairs on
 * the FP64 engine) and patched in.  rel_tol = 0 disables the check.  Default 1e-9. */
int ctr_split_set_refine(double rel_tol);
/* Number of entries the last split call recomputed. */
long long ctr_split_refined(void);
/* Work of the split engine's high-precision and standard GEMM launches since the
 * last reset: executed_mma = BF16 tensor-core flops executed, padding included;
 * block_products = Nev x Nev complex block products of the high-precision (chain)
 * launches, 8 Nev^3 FP64-equivalent flops each.  Eager launches only (replays of
 * recorded graphs are not counted).  reset != 0 zeroes both after reading. */
int ctr_split_flops(double* executed_mma, double* block_products, int reset);
/* The same for the Gram products that take the closing traces of the split
 * engine's momentum-set calls (ctr_rhopi_sigmapi_sets): executed_mma = BF16 flops
 * of those GEMM launches, traces = closing traces they produced (8 Nev^2
 * FP64-equivalent flops each).  No counterpart in the reference. */
int ctr_gram_flops(double* executed_mma, double* traces, int reset);

/* Synchronise the stream and report the first device-side error flag. */
int ctr_sync(void* stream);

/* Free the library's cached device scratch buffers (synchronises the device). */
void ctr_release_workspace(void);

/* Launch accounting.  Every kernel launch of the library is counted per kernel
 * name; with timing enabled a CUDA event pair is recorded on the launching
 * stream around each launch.  ctr_timing_enable() clears previous records.
 * ctr_timing_report() waits for the recorded events and writes JSON
 * {"kernel": [launches, timed_launches, total_ms], ...} into buf. */
void ctr_timing_enable(int on);
long long ctr_launch_count(void);
int ctr_timing_report(char* buf, int buflen);

/* ------------------------------------------------------------ CUDA graphs
 * Record the library calls a thread issues on one stream and replay them.
 *   ctr_graph_begin(s);  ctr_rho(..., s);  ...;  ctr_graph_end(s, &g);
 *   ctr_graph_launch(g, s);  (any number of times)  ctr_graph_destroy(g);
 * While recording, nothing executes: the kernels of the calls are captured into
 * CUDA graphs, their task tables are copied once into device memory owned by
 * the graph, and their scratch comes from buffers owned by the graph (so a
 * recorded graph never shares scratch with eager calls or with other graphs).
 * A replay reads the device buffers that were passed while recording, with the
 * contents they hold at replay time.  Steps that need host decisions on device
 * results -- the split engine's recomputation of ill-conditioned entries --
 * end a graph segment; ctr_graph_launch replays the segments in order and runs
 * those steps between them, synchronising the stream there (as the eager call
 * does).  Recording needs a created stream (not the legacy default stream),
 * uses the autotuner's cached choices (it measures nothing), and rejects the
 * calls that read device data on the host to plan their work (the profile
 * adjoint entry points, the ctr_calculate_* host API and ctr_sync) as well as
 * ctr_rho_noalloc, which keeps to its own fixed array.  A call that fails while recording makes ctr_graph_end fail (the
 * capture is closed and discarded).  Launch counts of replays are added to the
 * launch accounting; per-kernel event timing is not recorded for replays. */
typedef struct ctr_graph ctr_graph;
int ctr_graph_begin(void* stream);
int ctr_graph_end(void* stream, ctr_graph** graph);
int ctr_graph_launch(ctr_graph* graph, void* stream);
/* segments, kernel nodes per replay, bytes of device memory the graph owns */
int ctr_graph_info(const ctr_graph* graph, int* nsegments, long long* nkernels, long long* device_bytes);
void ctr_graph_destroy(ctr_graph* graph);

/* --------------------------------------------------------------- autotuner
 * Tunable choices (tile schedules, kernel variants, batch sizes) are keyed by
 * knob and problem shape.  mode 0: use the cached choice, else the default;
 * mode 1: a call that meets an uncached key times the candidates on its own
 * live data and caches the fastest (kernel variants are re-launched on the same
 * inputs; batch sizes are timed on successive batches of real work, so nothing
 * is computed twice); mode 2: as 1, re-measuring cached keys.  Candidates give
 * the same results up to rounding.  ctr_tune_force(knob, value) pins a knob
 * (value -1 releases it).  The table is saved and loaded as text lines
 * "key choice". */
int ctr_tune_set_mode(int mode);
int ctr_tune_force(const char* knob, int value);
int ctr_tune_report(char* buf, int buflen); /* JSON {"key": {"choice": c, "ms": [...]}, ...} */
void ctr_tune_clear(void);
int ctr_tune_save(const char* path);
int ctr_tune_load(const char* path);

#ifdef __cplusplus
}
#endif

#endif /* CTR_H */
