// Host orchestration of the split-precision engine: two-sided (rho-type)
// contractions and batched block products.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <map>
#include <tuple>

#include "kernels.h"
#include "split.h"

namespace ctr {

namespace {

int* g_err_dev = nullptr;

int err_flag(int** out) {
  if (!g_err_dev) {
    CTR_CUDA(cudaMalloc(&g_err_dev, sizeof(int)));
    CTR_CUDA(cudaMemset(g_err_dev, 0, sizeof(int)));
  }
  *out = g_err_dev;
  return CTR_OK;
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// ff complex (column-major, ld) -> complex128 row-major nev x nev
__global__ void ff_to_f64_kernel(const float4* __restrict__ src, int ld, int nev, double2* __restrict__ dst) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nev * nev) return;
  const int i = e / nev, j = e % nev;
  const float4 v = src[(size_t)j * ld + i];
  dst[e] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}

// Error model of a split-engine correlator entry: its rounding error is
// estimated as REFINE_EPS * sum_r |coef_r| sum_ij |A_r(i,j)|_1 |B_r(i,j)|_1.
// The products' digits reach 2^-45 of the row/column scales and the errors of
// the Nev^2 terms of a trace add with random signs, which puts the typical
// error near 2^-50 of that scale.  REFINE_EPS = 2^-48 was calibrated on the
// 86 016 entries of the rho benchmark against the FP64 engine: the largest
// entry error left after refinement was 4.4e-10 at rel_tol = 1e-9.  Entries
// whose estimate exceeds rel_tol * |value| -- the few with heavy cancellation
// between their spin rows or inside their traces -- are recomputed with the
// high-precision split configuration.
constexpr double REFINE_EPS = 1.0 / 281474976710656.0;  // 2^-48

}  // namespace

int prepare_for_capture() {
  int* d;
  CTR_TRY(err_flag(&d));
  return split_kernels_prepare();
}

int wait_probe(int timeout_ms, cudaStream_t s) {
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  CTR_TRY(launch_wait_probe((unsigned long long)timeout_ms * 1000000ull, d_err, s));
  return split_error_check(s);
}

int mma_schedule_probe(int hp, int nchunk, double* clocks_per_mma, double* tflops, cudaStream_t s) {
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  void* mem;
  CTR_TRY(workspace(WS_MISC).get(sizeof(unsigned long long), &mem));
  unsigned long long* d_cyc = (unsigned long long*)mem;
  CTR_CUDA(cudaMemsetAsync(d_cyc, 0, sizeof(unsigned long long), s));
  cudaEvent_t e0, e1;
  CTR_CUDA(cudaEventCreate(&e0));
  CTR_CUDA(cudaEventCreate(&e1));
  int nsm = 0, per_chunk = 0, n = 0;
  CTR_CUDA(cudaEventRecord(e0, s));
  int rc = launch_mma_schedule_probe(hp, nchunk, d_cyc, d_err, &nsm, &per_chunk, &n, s);
  if (rc == CTR_OK) {
    const cudaError_t e = cudaEventRecord(e1, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "probe event", __FILE__, __LINE__);
  }
  unsigned long long cyc = 0;
  float ms = 0.f;
  if (rc == CTR_OK) rc = download(&cyc, d_cyc, sizeof(cyc), s);
  if (rc == CTR_OK) {
    const cudaError_t e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) rc = cuda_fail(e, "probe event", __FILE__, __LINE__);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CTR_TRY(rc);
  CTR_TRY(split_error_check(s));
  const double mmas = (double)nchunk * per_chunk;
  *clocks_per_mma = (double)cyc / nsm / mmas;
  *tflops = (double)nsm * mmas * 2.0 * SPLIT_M * n * SPLIT_K / (ms * 1e-3) / 1e12;
  return CTR_OK;
}

int split_error_check(cudaStream_t s) {
  if (!g_err_dev) return CTR_OK;
  int h = 0;
  CTR_TRY(download(&h, g_err_dev, sizeof(int), s));
  if (h != 0) {
    CTR_CUDA(cudaMemsetAsync(g_err_dev, 0, sizeof(int), s));
    // 1-5: the split GEMM's pipeline, 6-7: the grouped traces, 9: ctr_wait_probe
    return fail(CTR_ERR_TIMEOUT, "a bounded device wait timed out (code %d)", h);
  }
  return CTR_OK;
}

// Scratch budget of a two-sided batch: 16 GB, or an eighth of the device's
// memory where that is less (the tuner found the largest batch the fastest at
// Nev = 100).  The memory size is queried once, outside any stream capture; a
// call recorded before the first query uses 6 GB.  The batch size does not
// change any pair's result.
static size_t batch_budget() {
  static size_t cached = 0;
  if (cached == 0 && !capturing()) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) cached = std::min<size_t>((size_t)16 << 30, total_b / 8);
  }
  return cached ? cached : ((size_t)6 << 30);
}

// Slice Nt elementals stacked [op list] as left and right operands.
struct PhiSlices {
  int nblk = 0, mtiles = 0, ntiles = 0;
  size_t left_bytes = 0, right_bytes = 0, lexp_n = 0, rexp_n = 0;
  uint8_t* left = nullptr;   // [Nt][mtiles][nchunk][A_STAGE]
  uint8_t* right = nullptr;  // [Nt][ntiles][nchunk][B_STAGE]
  int* lexp = nullptr;       // [Nt][mtiles*128]
  int* rexp = nullptr;       // [Nt][ntiles*80]
};

static size_t phi_bytes(int N, int Nt, int nL, int nR, int nchunk) {
  const int mt = cdiv(nR * N, SPLIT_M), nt = cdiv(nL * N, SPLIT_N);
  return align256((size_t)Nt * mt * nchunk * SPLIT_A_STAGE) + align256((size_t)Nt * nt * nchunk * SPLIT_B_STAGE) +
         align256((size_t)Nt * mt * SPLIT_M * 4) + align256((size_t)Nt * nt * SPLIT_N * 4);
}

static int refine_twosided(int N, int Nt, int tf_begin, int nphi, const double* prop_rows, const double* phi,
                           const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                           const std::vector<int>& off, const std::vector<int>& ord, int nout, double* out,
                           const int* d_count, const int* d_list, cudaStream_t stream);

int twosided_split(int N, int Nt, int tf_begin, int tf_end, const double* prop_rows, const double* phi, int nphi,
                   const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                   const std::vector<int32_t>& out_index, int nout, double* out, cudaStream_t stream) {
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d (got %d)", SPLIT_MAXK, N);
  const int nrows = (int)rows.size();
  for (int r = 0; r < nrows; r++) {
    const TwoSidedRow& w = rows[r];
    if (w.a < 0 || w.a > 3 || w.b < 0 || w.b > 3 || w.c < 0 || w.c > 3 || w.d < 0 || w.d > 3 || w.L < 0 ||
        w.L >= nphi || w.R < 0 || w.R >= nphi || out_index[r] < 0 || out_index[r] >= nout)
      return fail(CTR_ERR_ARG, "two-sided row %d out of range", r);
  }
  // distinct source blocks (c,d), source elementals L, sink blocks (a,b), sink elementals R
  std::vector<int> cdl, Ll, abl, Rl;
  auto idx = [](std::vector<int>& v, int x) {
    auto it = std::find(v.begin(), v.end(), x);
    if (it != v.end()) return (int)(it - v.begin());
    v.push_back(x);
    return (int)v.size() - 1;
  };
  std::vector<int> ia(nrows), il(nrows), ib(nrows), ir(nrows);
  for (int r = 0; r < nrows; r++) {
    ia[r] = idx(cdl, rows[r].c * 4 + rows[r].d);
    il[r] = idx(Ll, rows[r].L);
    ib[r] = idx(abl, rows[r].a * 4 + rows[r].b);
    ir[r] = idx(Rl, rows[r].R);
  }
  if ((int)Ll.size() > SPLIT_MAXBLK || (int)Rl.size() > SPLIT_MAXBLK)
    return fail(CTR_ERR_ARG, "too many distinct elementals (max %d)", SPLIT_MAXBLK);
  const int nchunk = cdiv(N, SPLIT_K);
  const int ncd = (int)cdl.size(), nab = (int)abl.size(), nL = (int)Ll.size(), nR = (int)Rl.size();
  const size_t N2 = (size_t)N * N;
  const double2* tau = (const double2*)prop_rows;
  const double2* ph = (const double2*)phi;
  int* d_err;
  CTR_TRY(err_flag(&d_err));

  // ---- elementals, sliced once per call
  PhiSlices F;
  F.mtiles = cdiv(nR * N, SPLIT_M);
  F.ntiles = cdiv(nL * N, SPLIT_N);
  void* phimem;
  CTR_TRY(workspace(WS_PHI).get(phi_bytes(N, Nt, nL, nR, nchunk), &phimem));
  {
    uint8_t* p = (uint8_t*)phimem;
    F.left = p;
    p += align256((size_t)Nt * F.mtiles * nchunk * SPLIT_A_STAGE);
    F.right = p;
    p += align256((size_t)Nt * F.ntiles * nchunk * SPLIT_B_STAGE);
    F.lexp = (int*)p;
    p += align256((size_t)Nt * F.mtiles * SPLIT_M * 4);
    F.rexp = (int*)p;
  }
  {
    std::vector<SliceLeftJob> lj(Nt);
    std::vector<SliceRightJob> rj(Nt);
    for (int t = 0; t < Nt; t++) {
      SliceLeftJob& L = lj[t];
      std::memset(&L, 0, sizeof(L));
      for (int k = 0; k < nR; k++) L.blk[k] = ph + ((size_t)t * nphi + Rl[k]) * N2;
      L.rows = nR * N;
      L.out = F.left + (size_t)t * F.mtiles * nchunk * SPLIT_A_STAGE;
      L.exps = F.lexp + (size_t)t * F.mtiles * SPLIT_M;
      SliceRightJob& R = rj[t];
      std::memset(&R, 0, sizeof(R));
      for (int k = 0; k < nL; k++) R.blk[k] = ph + ((size_t)t * nphi + Ll[k]) * N2;
      R.cols = nL * N;
      R.out = F.right + (size_t)t * F.ntiles * nchunk * SPLIT_B_STAGE;
      R.exps = F.rexp + (size_t)t * F.ntiles * SPLIT_N;
    }
    void *dl, *dr;
    CTR_TRY(upload(WS_TASKS, lj.data(), lj.size() * sizeof(SliceLeftJob), &dl, stream));
    CTR_TRY(launch_slice_left((const SliceLeftJob*)dl, Nt, N, nchunk, F.mtiles, stream, 1));
    CTR_TRY(upload(WS_TASKS2, rj.data(), rj.size() * sizeof(SliceRightJob), &dr, stream));
    CTR_TRY(launch_slice_right((const SliceRightJob*)dr, Nt, N, nchunk, F.ntiles, stream, 1));
  }

  // ---- per (t_sink, t_src) pair buffers
  const int mtT = cdiv(ncd * N, SPLIT_M), ntT = cdiv(nab * N, SPLIT_N);
  const int ldA = mtT * SPLIT_M, ldB = F.mtiles * SPLIT_M;
  const size_t tl_b = align256((size_t)mtT * nchunk * SPLIT_A_STAGE), tr_b = align256((size_t)ntT * nchunk * SPLIT_B_STAGE);
  const size_t tle_b = align256((size_t)mtT * SPLIT_M * 4), tre_b = align256((size_t)ntT * SPLIT_N * 4);
  const size_t a_b = align256((size_t)F.ntiles * SPLIT_N * ldA * sizeof(float4));
  const size_t b_b = align256((size_t)ntT * SPLIT_N * ldB * sizeof(float4));
  const size_t per_pair = tl_b + tr_b + tle_b + tre_b + a_b + b_b;
  const int npairs_total = (tf_end - tf_begin) * Nt;
  const size_t budget = batch_budget();
  int batch = (int)std::max<size_t>(1, budget / per_pair);
  batch = std::min(batch, npairs_total);

  // CSR of output rows
  std::vector<int> off(nout + 1, 0), ord(nrows);
  for (int r = 0; r < nrows; r++) off[out_index[r] + 1]++;
  for (int o = 0; o < nout; o++) off[o + 1] += off[o];
  {
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int r = 0; r < nrows; r++) ord[fill[out_index[r]]++] = r;
  }
  std::vector<int> csr(off);
  csr.insert(csr.end(), ord.begin(), ord.end());
  void* d_csr;
  CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, stream));
  // refinement list: one slot per output entry of the call, plus the counter
  void* d_ref;
  const size_t nentries = (size_t)npairs_total * nout;
  CTR_TRY(workspace(WS_REFINE).get((nentries + 1) * sizeof(int), &d_ref));
  int* d_count = (int*)d_ref;
  int* d_list = d_count + 1;
  CTR_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), stream));

  // closing traces: each distinct (A block, B block) pair once (rows of different
  // outputs often share one, e.g. 48 rho rows per momentum use 32 traces); the rows
  // then combine them with their coefficients
  std::vector<TraceRow> trow;
  std::vector<int> tix(nrows);
  {
    std::map<std::pair<int, int>, int> seen;
    for (int r = 0; r < nrows; r++) {
      const int aoff = (il[r] * N) * ldA + ia[r] * N, boff = (ib[r] * N) * ldB + ir[r] * N;
      auto it = seen.find({aoff, boff});
      if (it == seen.end()) {
        it = seen.emplace(std::make_pair(aoff, boff), (int)trow.size()).first;
        trow.push_back(TraceRow{aoff, boff, {1.f, 0.f}});
      }
      tix[r] = it->second;
    }
  }
  const int ntr = (int)trow.size();
  // the same traces in groups that share their product blocks (trace_groups)
  // (trace_groups), and in quad groups of at most 2 + 2 blocks (trace_quads)
  std::vector<TraceGroup> tgroups, tquads;
  const int tg_maxcols = build_trace_groups(trow.data(), ntr, TG_MAXA, TG_MAXB, TG_MAXT, tgroups);
  build_trace_groups(trow.data(), ntr, 2, 2, 4, tquads);
  tgroups.insert(tgroups.end(), tquads.begin(), tquads.end());
  const int ngroups = (int)(tgroups.size() - tquads.size()), nquads = (int)tquads.size();
  void *d_trow, *d_tix, *d_rcoef, *d_tgroups;
  CTR_TRY(upload(WS_SPLITJOBS, trow.data(), trow.size() * sizeof(TraceRow), &d_trow, stream));
  CTR_TRY(upload(WS_TRACEGROUPS, tgroups.data(), tgroups.size() * sizeof(TraceGroup), &d_tgroups, stream));
  CTR_TRY(upload(WS_SPLITJOBS2, tix.data(), tix.size() * sizeof(int), &d_tix, stream));
  CTR_TRY(upload(WS_SPLITJOBS3, coef.data(), coef.size() * sizeof(float), &d_rcoef, stream));

  std::vector<SliceLeftJob> lj;
  std::vector<SliceRightJob> rj;
  std::vector<SplitGemmInst> ga, gb;
  std::vector<const float4*> abase, bbase;
  char shape[160];
  snprintf(shape, sizeof(shape), "nev=%d,ncd=%d,nab=%d,nL=%d,nR=%d,ntr=%d", N, ncd, nab, nL, nR, ntr);
  // one batch of pairs [p0, p0 + np): slice tau, both GEMMs, traces, per-entry sums
  auto run_batch = [&](int p0, int np) -> int {
    void *mem, *rowbuf, *absbuf;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * per_pair, &mem));
    CTR_TRY(workspace(WS_ROWS).get((size_t)np * ntr * sizeof(double2), &rowbuf));
    CTR_TRY(workspace(WS_ROWABS).get((size_t)np * ntr * sizeof(double), &absbuf));
    uint8_t* base = (uint8_t*)mem;
    double2* R = (double2*)rowbuf;
    double* Rabs = (double*)absbuf;
    lj.assign(np, SliceLeftJob{});
    rj.assign(np, SliceRightJob{});
    ga.resize(np);
    gb.resize(np);
    abase.resize(np);
    bbase.resize(np);
    for (int q = 0; q < np; q++) {
      const int pr = p0 + q;
      const int tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* tblk = tau + ((size_t)tfl * Nt + ti) * 16 * N2;
      uint8_t* pb = base + (size_t)q * per_pair;
      uint8_t* TL = pb;
      uint8_t* TR = TL + tl_b;
      int* TLe = (int*)(TR + tr_b);
      int* TRe = (int*)((uint8_t*)TLe + tle_b);
      float4* A = (float4*)((uint8_t*)TRe + tre_b);
      float4* B = (float4*)((uint8_t*)A + a_b);
      SliceLeftJob& L = lj[q];
      std::memset(&L, 0, sizeof(L));
      for (int k = 0; k < ncd; k++) L.blk[k] = tblk + (size_t)cdl[k] * N2;
      L.rows = ncd * N;
      L.out = TL;
      L.exps = TLe;
      SliceRightJob& Rj = rj[q];
      std::memset(&Rj, 0, sizeof(Rj));
      for (int k = 0; k < nab; k++) Rj.blk[k] = tblk + (size_t)abl[k] * N2;
      Rj.cols = nab * N;
      Rj.out = TR;
      Rj.exps = TRe;
      ga[q] = SplitGemmInst{TL, F.right + (size_t)ti * F.ntiles * nchunk * SPLIT_B_STAGE, TLe,
                            F.rexp + (size_t)ti * F.ntiles * SPLIT_N, A};
      gb[q] = SplitGemmInst{F.left + (size_t)tf * F.mtiles * nchunk * SPLIT_A_STAGE, TR,
                            F.lexp + (size_t)tf * F.mtiles * SPLIT_M, TRe, B};
      abase[q] = A;
      bbase[q] = B;
    }
    void* d4[4];
    CTR_TRY(upload_group(WS_TASKS,
                         {{lj.data(), lj.size() * sizeof(SliceLeftJob)},
                          {rj.data(), rj.size() * sizeof(SliceRightJob)},
                          {ga.data(), ga.size() * sizeof(SplitGemmInst)},
                          {gb.data(), gb.size() * sizeof(SplitGemmInst)}},
                         d4, stream));
    void *d_lj = d4[0], *d_rj = d4[1], *d_ga = d4[2], *d_gb = d4[3], *d_tt;
    // slicer form (autotuned; all three write the same bytes, so candidates re-run)
    auto slice_tau = [&](int form) {
      CTR_TRY(launch_slice_left((const SliceLeftJob*)d_lj, np, N, nchunk, mtT, stream, form));
      return launch_slice_right((const SliceRightJob*)d_rj, np, N, nchunk, ntT, stream, form);
    };
    int sform = 2;
    CTR_TRY(tune_resolve("slice_tau", shape, 3, 2, stream, slice_tau, &sform));
    CTR_TRY(slice_tau(sform));
    // tile walk of each GEMM (autotuned; idempotent, so candidates re-run on the same data)
    SplitGemmBatch GA{(const SplitGemmInst*)d_ga, mtT, F.ntiles, nchunk, ncd * N, nL * N, ldA};
    SplitGemmBatch GB{(const SplitGemmInst*)d_gb, F.mtiles, ntT, nchunk, nR * N, nab * N, ldB};
    for (SplitGemmBatch* G : {&GA, &GB}) {
      char gshape[96];
      snprintf(gshape, sizeof(gshape), "std,m=%d,n=%d,k=%d", G->mtiles, G->ntiles, G->nchunk);
      int order = 0;
      CTR_TRY(tune_resolve("split_gemm.order", gshape, 2, 0, stream,
                           [&](int c) {
                             SplitGemmBatch t = *G;
                             t.order = c;
                             return launch_split_gemm(t, np, d_err, stream);
                           },
                           &order));
      G->order = order;
      CTR_TRY(launch_split_gemm(*G, np, d_err, stream));
    }
    abase.insert(abase.end(), bbase.begin(), bbase.end());
    CTR_TRY(upload(WS_ROWTASKS, abase.data(), abase.size() * sizeof(const float4*), &d_tt, stream));
    // candidates: the TRACE_VARIANTS per-trace kernels, the grouped one, then
    // the two quad-group kernels
    auto traces = [&](int variant) {
      if (variant == TRACE_VARIANTS)
        return launch_trace_groups((const TraceGroup*)d_tgroups, ngroups, tg_maxcols, (const TraceRow*)d_trow, ntr,
                                   (const float4* const*)d_tt, (const float4* const*)d_tt + np, ldA, ldB, np, N, R,
                                   Rabs, d_err, stream);
      if (variant > TRACE_VARIANTS)
        return launch_trace_quads((const TraceGroup*)d_tgroups + ngroups, nquads, (const TraceRow*)d_trow, ntr,
                                  (const float4* const*)d_tt, (const float4* const*)d_tt + np, ldA, ldB, np, N, R,
                                  Rabs, variant - TRACE_VARIANTS - 1, stream);
      return launch_trace_rows((const TraceRow*)d_trow, ntr, (const float4* const*)d_tt,
                               (const float4* const*)d_tt + np, ldA, ldB, np, N, R, Rabs, variant, stream);
    };
    int variant = 0;
    CTR_TRY(tune_resolve("trace_rows", shape, TRACE_VARIANTS + 3, TRACE_VARIANTS + 1, stream, traces, &variant));
    CTR_TRY(traces(variant));
    return launch_rowsum_coef_refine(R, Rabs, ntr, (const int*)d_csr, (const int*)d_csr + (nout + 1),
                                     (const int*)d_tix, (const float*)d_rcoef, nout, np,
                                     (double2*)out + (size_t)p0 * nout,
                                     g_refine_tol > 0.0 ? REFINE_EPS / g_refine_tol : 0.0, d_count, d_list, p0,
                                     stream);
  };

  // pairs per batch: forced, cached, measured on this call's first batches, or
  // the largest that fits the scratch budget
  int p0 = 0;
  {
    const std::string bkey = tune_key("twosided.batch", shape);
    int v = tune_forced("twosided.batch");
    if (v > 0) {
      batch = std::min(v, batch);
    } else if (tune_lookup(bkey, &v) && v > 0) {
      batch = std::min(v, batch);
    } else if (tune_mode() > 0) {
      // candidates, largest first (the scratch then grows once), each run twice:
      // the first pass warms up (and resolves the kernel knobs), the second is timed
      std::vector<int> cand;
      for (int c = std::min(batch, 512); c >= 2; c /= 2) cand.push_back(c);
      int sum = 0;
      for (int c : cand) sum += c;
      while (cand.size() > 1 && 2 * sum > npairs_total) {
        sum -= cand.front();
        cand.erase(cand.begin());
      }
      if (cand.size() > 1) {
        cudaEvent_t e0, e1;
        CTR_CUDA(cudaEventCreate(&e0));
        CTR_CUDA(cudaEventCreate(&e1));
        std::vector<double> per(cand.size(), 0.0);
        int rc = CTR_OK;
        for (int rep = 0; rep < 2 && rc == CTR_OK; rep++)
          for (size_t k = 0; k < cand.size() && rc == CTR_OK; k++) {
            cudaEventRecord(e0, stream);
            rc = run_batch(p0, cand[k]);
            cudaEventRecord(e1, stream);
            p0 += cand[k];
            float ms = 0.f;
            if (rc == CTR_OK) {
              cudaError_t e = cudaEventSynchronize(e1);
              if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
              if (e != cudaSuccess) rc = cuda_fail(e, "tuning events", __FILE__, __LINE__);
            }
            if (rep == 1) per[k] = ms / cand[k];
          }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CTR_TRY(rc);
        size_t best = 0;
        for (size_t k = 1; k < cand.size(); k++)
          if (per[k] < per[best]) best = k;
        batch = cand[best];
        tune_store(bkey, batch, per);  // ms per pair of each candidate
      }
    }
  }
  for (; p0 < npairs_total; p0 += batch) CTR_TRY(run_batch(p0, std::min(batch, npairs_total - p0)));
  g_refined_last = 0;
  if (g_refine_tol <= 0.0) return CTR_OK;
  // ---- recomputation of the flagged entries: the list is read on the host, so
  // under graph recording this runs after the recorded kernels at every launch
  return host_step(stream, [=](cudaStream_t ls) {
    return refine_twosided(N, Nt, tf_begin, nphi, prop_rows, phi, rows, coef, off, ord, nout, out, d_count, d_list,
                           ls);
  });
}

// Recomputes the entries listed in d_list[0 .. *d_count) (indices pair * nout + o
// of the call's output) with the high-precision configuration and patches them.
static int refine_twosided(int N, int Nt, int tf_begin, int nphi, const double* prop_rows, const double* phi,
                           const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                           const std::vector<int>& off, const std::vector<int>& ord, int nout, double* out,
                           const int* d_count, const int* d_list, cudaStream_t stream) {
  int nflag = 0;
  CTR_TRY(download(&nflag, d_count, sizeof(int), stream));
  if (nflag == 0) return CTR_OK;
  std::vector<int> flagged(nflag);
  CTR_TRY(download(flagged.data(), d_list, nflag * sizeof(int), stream));
  std::sort(flagged.begin(), flagged.end());
  std::vector<ctr_factor> fac;
  std::vector<int> foff(1, 0), chain_row;
  auto mkf = [](int kind, int dag, int a, int b, int s1, int s2) {
    ctr_factor x;
    x.kind = kind;
    x.dag = dag;
    x.a = a;
    x.b = b;
    x.s1 = s1;
    x.s2 = s2;
    return x;
  };
  for (int e : flagged) {
    const int pr = e / nout, o = e % nout, tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
    for (int k = off[o]; k < off[o + 1]; k++) {
      const int r = ord[k];
      const TwoSidedRow& w = rows[r];
      // coef * Tr[tau_cd Phi_L(ti) (Phi_R(tf) tau_ab)^dagger]
      fac.push_back(mkf(CTR_FACTOR_TAU, 0, tfl, ti, w.c, w.d));
      fac.push_back(mkf(CTR_FACTOR_PHI, 0, ti, w.L, 0, 0));
      fac.push_back(mkf(CTR_FACTOR_TAU, 1, tfl, ti, w.a, w.b));
      fac.push_back(mkf(CTR_FACTOR_PHI, 1, tf, w.R, 0, 0));
      foff.push_back((int)fac.size());
      chain_row.push_back(r);
    }
  }
  void* dv;
  CTR_TRY(workspace(WS_REFINE).get(chain_row.size() * sizeof(double2), &dv));
  // the flagged entries' chains on the high-precision configuration (~2^-53 of the
  // row/column scales, ~2^9 below the standard one); traces in FP64
  CTR_TRY(chain_values(N, Nt, nphi, prop_rows, phi, fac, foff, (double*)dv, stream, CTR_ENGINE_SPLIT));
  std::vector<double2> vals(chain_row.size());
  CTR_TRY(download(vals.data(), dv, vals.size() * sizeof(double2), stream));
  std::vector<double2> patch(nflag);
  std::vector<int> where(nflag);
  size_t c = 0;
  for (int i = 0; i < nflag; i++) {
    const int o = flagged[i] % nout;
    double2 acc = make_double2(0.0, 0.0);
    for (int k = off[o]; k < off[o + 1]; k++, c++) {
      const int r = chain_row[c];
      const double2 v = cmul(make_double2(coef[2 * r], coef[2 * r + 1]), vals[c]);
      acc.x += v.x;
      acc.y += v.y;
    }
    patch[i] = acc;
    where[i] = flagged[i];
  }
  void *dw, *dp;
  CTR_TRY(upload(WS_TASKS, where.data(), where.size() * sizeof(int), &dw, stream));
  CTR_TRY(upload(WS_TASKS2, patch.data(), patch.size() * sizeof(double2), &dp, stream));
  CTR_TRY(launch_scatter((const int*)dw, (const double2*)dp, nflag, (double2*)out, stream));
  g_refined_last += nflag;
  return CTR_OK;
}

// Batched block products C_b = X_b Y_b through the split engine (unit-level access
// to the tensor-core GEMM; results converted back to complex128).
int zgemm_split_batched(int N, int nb, const double* const* x, const double* const* y, double* const* c,
                        cudaStream_t stream) {
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d", SPLIT_MAXK);
  const int nchunk = cdiv(N, SPLIT_K), nt = cdiv(N, SPLIT_N);
  const size_t l_b = align256((size_t)nchunk * SPLIT_A_STAGE), r_b = align256((size_t)nt * nchunk * SPLIT_B_STAGE);
  const size_t le_b = align256(SPLIT_M * 4), re_b = align256((size_t)nt * SPLIT_N * 4);
  const int ldo = SPLIT_M;
  const size_t o_b = align256((size_t)nt * SPLIT_N * ldo * sizeof(float4));
  const size_t per = l_b + r_b + le_b + re_b + o_b;
  void* mem;
  CTR_TRY(workspace(WS_SCRATCH).get((size_t)nb * per, &mem));
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  std::vector<SliceLeftJob> lj(nb);
  std::vector<SliceRightJob> rj(nb);
  std::vector<SplitGemmInst> gi(nb);
  for (int b = 0; b < nb; b++) {
    uint8_t* p = (uint8_t*)mem + (size_t)b * per;
    std::memset(&lj[b], 0, sizeof(SliceLeftJob));
    std::memset(&rj[b], 0, sizeof(SliceRightJob));
    lj[b].blk[0] = (const double2*)x[b];
    lj[b].rows = N;
    lj[b].out = p;
    lj[b].exps = (int*)(p + l_b + r_b);
    rj[b].blk[0] = (const double2*)y[b];
    rj[b].cols = N;
    rj[b].out = p + l_b;
    rj[b].exps = (int*)(p + l_b + r_b + le_b);
    gi[b] = SplitGemmInst{p, p + l_b, lj[b].exps, rj[b].exps, (float4*)(p + l_b + r_b + le_b + re_b)};
  }
  void *dl, *dr, *dg;
  CTR_TRY(upload(WS_TASKS, lj.data(), nb * sizeof(SliceLeftJob), &dl, stream));
  CTR_TRY(launch_slice_left((const SliceLeftJob*)dl, nb, N, nchunk, 1, stream, 1));
  CTR_TRY(upload(WS_TASKS2, rj.data(), nb * sizeof(SliceRightJob), &dr, stream));
  CTR_TRY(launch_slice_right((const SliceRightJob*)dr, nb, N, nchunk, nt, stream, 1));
  CTR_TRY(upload(WS_GEMM_A, gi.data(), nb * sizeof(SplitGemmInst), &dg, stream));
  SplitGemmBatch G{(const SplitGemmInst*)dg, 1, nt, nchunk, N, N, ldo};
  CTR_TRY(launch_split_gemm(G, nb, d_err, stream));
  for (int b = 0; b < nb; b++) {
    TimedLaunch tl(stream, "ff_to_f64");
    ff_to_f64_kernel<<<cdiv(N * N, 256), 256, 0, stream>>>(gi[b].out, ldo, N, (double2*)c[b]);
    CTR_CUDA(cudaGetLastError());
  }
  return CTR_OK;
}

// Diagnostics: the raw FP32 TMEM accumulators (Re/Im x levels 0, 1, >=2) of one
// product x*y, before recombination and scaling.  Used by the tests to check
// the tensor-core accumulation against an exact emulation of the slices.
int split_levels(int N, const double* x, const double* y, float* levels, cudaStream_t stream) {
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d", SPLIT_MAXK);
  const int nchunk = cdiv(N, SPLIT_K), nt = cdiv(N, SPLIT_N);
  const size_t l_b = align256((size_t)nchunk * SPLIT_A_STAGE), r_b = align256((size_t)nt * nchunk * SPLIT_B_STAGE);
  const size_t le_b = align256(SPLIT_M * 4), re_b = align256((size_t)nt * SPLIT_N * 4);
  void* mem;
  CTR_TRY(workspace(WS_SCRATCH).get(l_b + r_b + le_b + re_b + 256, &mem));
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  uint8_t* p = (uint8_t*)mem;
  SliceLeftJob lj;
  SliceRightJob rj;
  std::memset(&lj, 0, sizeof(lj));
  std::memset(&rj, 0, sizeof(rj));
  lj.blk[0] = (const double2*)x;
  lj.rows = N;
  lj.out = p;
  lj.exps = (int*)(p + l_b + r_b);
  rj.blk[0] = (const double2*)y;
  rj.cols = N;
  rj.out = p + l_b;
  rj.exps = (int*)(p + l_b + r_b + le_b);
  SplitGemmInst gi{p, p + l_b, lj.exps, rj.exps, nullptr};
  void *dl, *dr, *dg;
  CTR_TRY(upload(WS_TASKS, &lj, sizeof(lj), &dl, stream));
  CTR_TRY(launch_slice_left((const SliceLeftJob*)dl, 1, N, nchunk, 1, stream));
  CTR_TRY(upload(WS_TASKS2, &rj, sizeof(rj), &dr, stream));
  CTR_TRY(launch_slice_right((const SliceRightJob*)dr, 1, N, nchunk, nt, stream));
  CTR_TRY(upload(WS_GEMM_A, &gi, sizeof(gi), &dg, stream));
  SplitGemmBatch G{(const SplitGemmInst*)dg, 1, nt, nchunk, N, N, SPLIT_M, levels};
  return launch_split_gemm(G, 1, d_err, stream);
}

}  // namespace ctr

extern "C" int ctr_split_set_refine(double rel_tol) {
  if (!(rel_tol >= 0.0)) return ctr::fail(CTR_ERR_ARG, "ctr_split_set_refine: rel_tol must be >= 0");
  ctr::g_refine_tol = rel_tol;
  return CTR_OK;
}

extern "C" long long ctr_split_refined(void) { return ctr::g_refined_last; }

extern "C" int ctr_split_flops(double* executed_mma, double* block_products, int reset) {
  if (executed_mma) *executed_mma = ctr::g_split_mma_flops;
  if (block_products) *block_products = ctr::g_split_products;
  if (reset) ctr::g_split_mma_flops = ctr::g_split_products = 0.0;
  return CTR_OK;
}

extern "C" int ctr_gram_flops(double* executed_mma, double* traces, int reset) {
  if (executed_mma) *executed_mma = ctr::g_gram_mma_flops;
  if (traces) *traces = ctr::g_gram_traces;
  if (reset) ctr::g_gram_mma_flops = ctr::g_gram_traces = 0.0;
  return CTR_OK;
}

namespace ctr {
double g_split_mma_flops = 0.0, g_split_products = 0.0;
double g_gram_mma_flops = 0.0, g_gram_traces = 0.0;
double g_refine_tol = 1e-9;
long long g_refined_last = 0;
}  // namespace ctr

extern "C" int ctr_split_levels(int nev, const double* x, const double* y, float* levels, void* stream) {
  if (nev < 1 || !x || !y || !levels) return ctr::fail(CTR_ERR_ARG, "ctr_split_levels: bad arguments");
  return ctr::split_levels(nev, x, y, levels, (cudaStream_t)stream);
}

namespace ctr {

// Split-engine execution of a stage of FP64-engine GEMM tasks, on the
// high-precision configuration (6 slices, 5 levels, tiles of 128 x 48).  Tasks
// with the same left side (A pointers, transposes, weights) share one sliced
// left operand and stack up to SPLIT_TASK_NB right sides along N, so each GEMM
// instance is 128 x (nb N) x (nterm N); identical right sides are sliced once;
// instances of equal shape form one persistent launch, whose epilogue writes
// complex128 blocks in place.
int zgemm_split_tasks(int N, const ZTask* tasks, int ntask, cudaStream_t stream) {
  if (ntask == 0) return CTR_OK;
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d (got %d)", SPLIT_MAXK, N);
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  struct LeftKey {
    const double2* a[4];
    float w[4];
    int nterm, dag;
    bool operator<(const LeftKey& o) const { return std::memcmp(this, &o, sizeof(LeftKey)) < 0; }
  };
  std::map<LeftKey, int> gid;
  std::vector<std::vector<int>> groups;
  std::vector<LeftKey> gkey;
  for (int t = 0; t < ntask; t++) {
    const ZTask& z = tasks[t];
    if (z.nterm < 1 || z.nterm > 4 || z.nterm * N > 512)
      return fail(CTR_ERR_ARG, "split task %d: %d terms of Nev %d", t, z.nterm, N);
    LeftKey k;
    std::memset(&k, 0, sizeof(k));
    k.nterm = z.nterm;
    for (int q = 0; q < z.nterm; q++) {
      int ex;
      if (z.wim[q] != 0.f || !(z.wre[q] != 0.f) || std::fabs(std::frexp(z.wre[q], &ex)) != 0.5f)
        return fail(CTR_ERR_UNSUPPORTED, "split task %d: weight (%g, %g) is not a real power of two", t, z.wre[q],
                    z.wim[q]);
      k.a[q] = z.A[q];
      k.w[q] = z.wre[q];
      k.dag |= ((z.flags >> q) & 1) << q;
    }
    auto it = gid.find(k);
    if (it == gid.end()) {
      it = gid.emplace(k, (int)groups.size()).first;
      groups.emplace_back();
      gkey.push_back(k);
    }
    groups[it->second].push_back(t);
  }
  // instances (group, first task, count), bucketed by (nterm, nb)
  struct Inst {
    int g, t0, nb;
  };
  std::map<std::pair<int, int>, std::vector<Inst>> buckets;
  for (int g = 0; g < (int)groups.size(); g++)
    for (int t0 = 0; t0 < (int)groups[g].size(); t0 += SPLIT_TASK_NB) {
      const int nb = std::min<int>(SPLIT_TASK_NB, (int)groups[g].size() - t0);
      buckets[{gkey[g].nterm, nb}].push_back(Inst{g, t0, nb});
    }
  for (auto& bk : buckets) {
    const int nterm = bk.first.first, nb = bk.first.second;
    const int K = nterm * N, nchunk = cdiv(K, SPLIT_K), ntiles = cdiv(nb * N, CfgHP::BN);
    const int eplus = K > 128 ? 1 : 0;
    const size_t l_b = align256((size_t)nchunk * CfgHP::A_STAGE);
    const size_t r_b = align256((size_t)ntiles * nchunk * CfgHP::B_STAGE);
    const size_t le_b = align256(SPLIT_M * 4), re_b = align256((size_t)ntiles * CfgHP::BN * 4);
    const size_t per = l_b + r_b + le_b + re_b;  // one left and at most one distinct right per instance
    const std::vector<Inst>& all = bk.second;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(all.size(), ((size_t)4 << 30) / per));
    for (size_t i0 = 0; i0 < all.size(); i0 += batch) {
      const int ni = (int)std::min<size_t>(batch, all.size() - i0);
      void* mem;
      CTR_TRY(workspace(WS_SPLITTASK).get((size_t)ni * per, &mem));
      uint8_t* lbase = (uint8_t*)mem;                       // ni x (left slices + row exponents)
      uint8_t* rbase = lbase + (size_t)ni * (l_b + le_b);   // <= ni x (right slices + column exponents)
      std::vector<SliceTaskLJob> lj;
      std::vector<SliceTaskRJob> rj;
      std::map<const double2*, int> bid;          // distinct blocks -> exponent table index
      std::vector<const double2*> blks;
      auto block_index = [&](const double2* p) {
        auto b = bid.find(p);
        if (b == bid.end()) {
          b = bid.emplace(p, (int)blks.size()).first;
          blks.push_back(p);
        }
        return b->second;
      };
      std::map<int, int> lid;                     // instances of one left group share its slices
      std::map<std::vector<uintptr_t>, int> rid;  // identical right sides are sliced once
      std::vector<SplitGemmInst> gi(ni);
      std::vector<double2*> outs((size_t)ni * SPLIT_TASK_NB, nullptr);
      for (int i = 0; i < ni; i++) {
        const Inst& in = all[i0 + i];
        const LeftKey& k = gkey[in.g];
        auto lt = lid.find(in.g);
        if (lt == lid.end()) {
          uint8_t* p = lbase + lj.size() * (l_b + le_b);
          SliceTaskLJob L;
          std::memset(&L, 0, sizeof(L));
          for (int q = 0; q < nterm; q++) {
            int ex;
            std::frexp(k.w[q], &ex);  // |w| = 2^(ex-1), checked when the groups were formed
            L.a[q] = k.a[q];
            L.w[q] = k.w[q];
            L.bi[q] = block_index(k.a[q]);
            L.wexp[q] = ex - 1;
          }
          L.nterm = nterm;
          L.dag = k.dag;
          L.eplus = eplus;
          L.out = p;
          L.exps = (int*)(p + l_b);
          lt = lid.emplace(in.g, (int)lj.size()).first;
          lj.push_back(L);
        }
        const SliceTaskLJob& L = lj[lt->second];
        SliceTaskRJob R;
        std::memset(&R, 0, sizeof(R));
        R.nb = in.nb;
        R.nterm = nterm;
        R.eplus = eplus;
        std::vector<uintptr_t> key;
        for (int j = 0; j < in.nb; j++) {
          const ZTask& z = tasks[groups[in.g][in.t0 + j]];
          for (int q = 0; q < nterm; q++) {
            R.b[j][q] = z.B[q];
            R.dag |= ((z.flags >> (4 + q)) & 1) << (4 * j + q);
            key.push_back((uintptr_t)z.B[q]);
          }
          outs[(size_t)i * SPLIT_TASK_NB + j] = z.C;
        }
        key.push_back((uintptr_t)R.dag);
        auto it = rid.find(key);
        if (it == rid.end()) {
          uint8_t* q = rbase + rj.size() * (r_b + re_b);
          R.out = q;
          R.exps = (int*)(q + r_b);
          for (int j = 0; j < in.nb; j++)
            for (int t = 0; t < nterm; t++) R.bi[j][t] = block_index(R.b[j][t]);
          it = rid.emplace(key, (int)rj.size()).first;
          rj.push_back(R);
        }
        const SliceTaskRJob& Ru = rj[it->second];
        gi[i] = SplitGemmInst{L.out, Ru.out, L.exps, Ru.exps, nullptr, nullptr};
      }
      // the launch's tables in two staging copies (the instances need the
      // device address of their output pointer lists)
      void* d1[4];
      CTR_TRY(upload_group(WS_SPLITJOBS,
                           {{lj.data(), lj.size() * sizeof(SliceTaskLJob)},
                            {rj.data(), rj.size() * sizeof(SliceTaskRJob)},
                            {outs.data(), outs.size() * sizeof(double2*)},
                            {blks.data(), blks.size() * sizeof(const double2*)}},
                           d1, stream));
      void *d_lj = d1[0], *d_rj = d1[1], *d_outs = d1[2], *d_blk = d1[3], *d_gi;
      for (int i = 0; i < ni; i++) gi[i].outs = (double2* const*)d_outs + (size_t)i * SPLIT_TASK_NB;
      CTR_TRY(upload(WS_GEMM_B, gi.data(), gi.size() * sizeof(SplitGemmInst), &d_gi, stream));
      // exponent bounds of every distinct block once, then the slices
      void* d_bexp;
      CTR_TRY(workspace(WS_BLOCKEXP).get(blks.size() * 2 * N * sizeof(int), &d_bexp));
      CTR_TRY(launch_block_exp((const double2* const*)d_blk, (int)blks.size(), N, (int*)d_bexp, stream));
      CTR_TRY(launch_slice_task_left((const SliceTaskLJob*)d_lj, (int)lj.size(), N, nchunk, (const int*)d_bexp,
                                     stream));
      CTR_TRY(launch_slice_task_right((const SliceTaskRJob*)d_rj, (int)rj.size(), N, nchunk, ntiles,
                                      (const int*)d_bexp, stream));
      SplitGemmBatch G{(const SplitGemmInst*)d_gi, 1, ntiles, nchunk, N, nb * N, SPLIT_M, nullptr, 1, N, 1};
      CTR_TRY(launch_split_gemm(G, ni, d_err, stream));
      if (!capturing()) g_split_products += (double)ni * nb * nterm;
    }
  }
  return CTR_OK;
}

}  // namespace ctr

namespace ctr {

// Split-engine execution of block grids (GridTask, ctr_internal.h) on the
// high-precision configuration.  Each grid's slabs are cut into pieces of at
// most SPLIT_STACK slabs; a piece is one GEMM instance whose left operand
// stacks its slabs along M (slice_stack_left), so that M tiles carry padding
// rows only at the end of a piece; the right side (nb blocks along N) is sliced
// once per distinct right side of a launch.  Pieces of equal shape (terms,
// right blocks, slabs) form one persistent launch; the epilogue writes slab s of
// right block j at C0[j] + s Nev^2, i.e. row s Nev + r of the piece.
int zgemm_split_grids(int N, const std::vector<GridTask>& grids, cudaStream_t stream) {
  if (grids.empty()) return CTR_OK;
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d (got %d)", SPLIT_MAXK, N);
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  const size_t N2 = (size_t)N * N;
  struct Piece {
    int g, s0, ns;
  };
  std::map<std::tuple<int, int, int>, std::vector<Piece>> buckets;
  for (int g = 0; g < (int)grids.size(); g++) {
    const GridTask& G = grids[g];
    if (G.nterm < 1 || G.nterm > 4 || G.nterm * N > 512 || G.nb < 1 || G.nb > SPLIT_TASK_NB || G.nslab < 1 ||
        (int)G.A.size() != G.nslab * G.nterm)
      return fail(CTR_ERR_ARG, "split grid %d: %d terms of Nev %d, %d right blocks, %d slabs", g, G.nterm, N, G.nb,
                  G.nslab);
    for (int q = 0; q < G.nterm; q++) {
      int ex;
      if (!(G.w[q] != 0.f) || std::fabs(std::frexp(G.w[q], &ex)) != 0.5f)
        return fail(CTR_ERR_UNSUPPORTED, "split grid %d: weight %g is not a power of two", g, G.w[q]);
    }
    for (int s0 = 0; s0 < G.nslab; s0 += SPLIT_STACK) {
      const int ns = std::min(SPLIT_STACK, G.nslab - s0);
      buckets[std::make_tuple(G.nterm, G.nb, ns)].push_back(Piece{g, s0, ns});
    }
  }
  for (auto& bk : buckets) {
    const int nterm = std::get<0>(bk.first), nb = std::get<1>(bk.first), ns = std::get<2>(bk.first);
    const int K = nterm * N, nchunk = cdiv(K, SPLIT_K), ntiles = cdiv(nb * N, CfgHP::BN),
              mtiles = cdiv(ns * N, SPLIT_M);
    const int eplus = K > 128 ? 1 : 0;
    const size_t l_b = align256((size_t)mtiles * nchunk * CfgHP::A_STAGE), le_b = align256((size_t)mtiles * SPLIT_M * 4);
    const size_t r_b = align256((size_t)ntiles * nchunk * CfgHP::B_STAGE), re_b = align256((size_t)ntiles * CfgHP::BN * 4);
    const size_t per = l_b + le_b + r_b + re_b;  // one left and at most one distinct right per piece
    const std::vector<Piece>& all = bk.second;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>(all.size(), ((size_t)4 << 30) / per));
    for (size_t i0 = 0; i0 < all.size(); i0 += batch) {
      const int ni = (int)std::min<size_t>(batch, all.size() - i0);
      void* mem;
      CTR_TRY(workspace(WS_SPLITTASK).get((size_t)ni * per, &mem));
      uint8_t* lbase = (uint8_t*)mem;
      uint8_t* rbase = lbase + (size_t)ni * (l_b + le_b);
      std::vector<SliceStackLJob> lj(ni);
      std::vector<SliceTaskRJob> rj;
      std::map<const double2*, int> bid;
      std::vector<const double2*> blks;
      auto block_index = [&](const double2* p) {
        auto b = bid.find(p);
        if (b == bid.end()) {
          b = bid.emplace(p, (int)blks.size()).first;
          blks.push_back(p);
        }
        return b->second;
      };
      std::map<std::vector<uintptr_t>, int> rid;
      std::vector<SplitGemmInst> gi(ni);
      std::vector<double2*> outs((size_t)ni * SPLIT_TASK_NB, nullptr);
      for (int i = 0; i < ni; i++) {
        const Piece& pc = all[i0 + i];
        const GridTask& G = grids[pc.g];
        SliceStackLJob& L = lj[i];
        std::memset(&L, 0, sizeof(L));
        for (int q = 0; q < nterm; q++) {
          int ex;
          std::frexp(G.w[q], &ex);
          L.w[q] = G.w[q];
          L.wexp[q] = ex - 1;
        }
        for (int sl = 0; sl < pc.ns; sl++)
          for (int q = 0; q < nterm; q++) {
            const double2* a = G.A[(size_t)(pc.s0 + sl) * nterm + q];
            L.a[sl][q] = a;
            L.bi[sl][q] = block_index(a);
          }
        L.nslab = pc.ns;
        L.nterm = nterm;
        L.dag = G.adag;
        L.eplus = eplus;
        L.out = lbase + (size_t)i * (l_b + le_b);
        L.exps = (int*)(L.out + l_b);
        std::vector<uintptr_t> key;
        for (int j = 0; j < nb; j++)
          for (int q = 0; q < nterm; q++) key.push_back((uintptr_t)G.B[j][q]);
        key.push_back((uintptr_t)G.bdag);
        auto it = rid.find(key);
        if (it == rid.end()) {
          SliceTaskRJob R;
          std::memset(&R, 0, sizeof(R));
          R.nb = nb;
          R.nterm = nterm;
          R.eplus = eplus;
          R.dag = G.bdag;
          for (int j = 0; j < nb; j++)
            for (int q = 0; q < nterm; q++) {
              R.b[j][q] = G.B[j][q];
              R.bi[j][q] = block_index(G.B[j][q]);
            }
          R.out = rbase + rj.size() * (r_b + re_b);
          R.exps = (int*)(R.out + r_b);
          it = rid.emplace(key, (int)rj.size()).first;
          rj.push_back(R);
        }
        for (int j = 0; j < nb; j++) outs[(size_t)i * SPLIT_TASK_NB + j] = G.C0[j] + (size_t)pc.s0 * N2;
        gi[i] = SplitGemmInst{L.out, rj[it->second].out, L.exps, rj[it->second].exps, nullptr, nullptr};
      }
      void* d1[4];
      CTR_TRY(upload_group(WS_SPLITJOBS,
                           {{lj.data(), lj.size() * sizeof(SliceStackLJob)},
                            {rj.data(), rj.size() * sizeof(SliceTaskRJob)},
                            {outs.data(), outs.size() * sizeof(double2*)},
                            {blks.data(), blks.size() * sizeof(const double2*)}},
                           d1, stream));
      for (int i = 0; i < ni; i++) gi[i].outs = (double2* const*)d1[2] + (size_t)i * SPLIT_TASK_NB;
      void* d_gi;
      CTR_TRY(upload(WS_GEMM_B, gi.data(), gi.size() * sizeof(SplitGemmInst), &d_gi, stream));
      void* d_bexp;
      CTR_TRY(workspace(WS_BLOCKEXP).get(blks.size() * 2 * N * sizeof(int), &d_bexp));
      CTR_TRY(launch_block_exp((const double2* const*)d1[3], (int)blks.size(), N, (int*)d_bexp, stream));
      CTR_TRY(launch_slice_stack_left((const SliceStackLJob*)d1[0], ni, N, nchunk, mtiles, (const int*)d_bexp,
                                      stream));
      CTR_TRY(launch_slice_task_right((const SliceTaskRJob*)d1[1], (int)rj.size(), N, nchunk, ntiles,
                                      (const int*)d_bexp, stream));
      SplitGemmBatch B{(const SplitGemmInst*)d_gi, mtiles, ntiles, nchunk, ns * N, nb * N, mtiles * SPLIT_M,
                       nullptr, 1, N, 1};
      // persistent tile walk (N tiles or M tiles innermost), autotuned per tile shape
      // by re-launching the GEMM on the same operands (it rewrites the same outputs)
      char gshape[96];
      snprintf(gshape, sizeof(gshape), "hp,m=%d,n=%d,k=%d", mtiles, ntiles, nchunk);
      int order = 0;
      CTR_TRY(tune_resolve("split_gemm.order", gshape, 2, 0, stream,
                           [&](int c) {
                             SplitGemmBatch t = B;
                             t.order = c;
                             return launch_split_gemm(t, ni, d_err, stream);
                           },
                           &order));
      B.order = order;
      CTR_TRY(launch_split_gemm(B, ni, d_err, stream));
      if (!capturing()) g_split_products += (double)ni * ns * nb * nterm;
    }
  }
  return CTR_OK;
}

// Gram traces.  Instance ip = g * npiece + p of a launch is the product of group
// g's left and right blocks over K piece p (at most GRAM_PIECE elements of
// the flattened Nev^2): one high-precision tile pair per (M tile, N tile), its
// complex128 partial product written row-major (rows padded to M tiles,
// columns to N tiles).  Groups run in launches sized to a 4 GB arena; each
// launch slices its operands, runs the GEMM and sums its traces' pieces.
static_assert(sizeof(GramPlan::Tr) == sizeof(GramTrace) && offsetof(GramPlan::Tr, g) == offsetof(GramTrace, g) &&
                  offsetof(GramPlan::Tr, slot) == offsetof(GramTrace, slot) &&
                  offsetof(GramPlan::Tr, cre) == offsetof(GramTrace, coef),
              "a plan's traces upload as GramTrace");

int trace_gram(int N, const GramPlan& P, double2* trv, double* tra, cudaStream_t stream) {
  if (P.tr.empty()) return CTR_OK;
  if (N > SPLIT_MAXK) return fail(CTR_ERR_UNSUPPORTED, "split engine supports Nev <= %d (got %d)", SPLIT_MAXK, N);
  if (P.ngroup < 1 || P.mrows < 1 || P.ncols < 1 || P.left.size() != (size_t)P.ngroup * P.mrows ||
      P.right.size() != (size_t)P.ngroup * P.ncols)
    return fail(CTR_ERR_ARG, "Gram traces: %d groups of %d x %d blocks, tables of %zu and %zu", P.ngroup, P.mrows,
                P.ncols, P.left.size(), P.right.size());
  int* d_err;
  CTR_TRY(err_flag(&d_err));
  const int n2 = N * N;
  const int nchunk = std::min(GRAM_PIECE / SPLIT_K, cdiv(n2, SPLIT_K)), npiece = cdiv(n2, nchunk * SPLIT_K);
  const int mtiles = cdiv(P.mrows, SPLIT_M), ntiles = cdiv(P.ncols, CfgHP::BN);
  const int lrows = mtiles * SPLIT_M, rcols = ntiles * CfgHP::BN;
  // per instance: left and right slices, partial product, exponents and norms
  const size_t l_b = (size_t)mtiles * nchunk * CfgHP::A_STAGE, r_b = (size_t)ntiles * nchunk * CfgHP::B_STAGE;
  const size_t p_b = (size_t)lrows * rcols * sizeof(double2);
  const size_t per_inst = l_b + r_b + p_b + (size_t)(lrows + rcols) * (sizeof(int) + sizeof(float));
  const size_t per_group = (size_t)npiece * per_inst;
  const int run = std::max(1, P.group_run);
  int G = (int)std::max<size_t>(1, std::min<size_t>(P.ngroup, ((size_t)4 << 30) / per_group));
  if (G < P.ngroup) G = std::max(run, G / run * run);
  const int nl = cdiv(P.ngroup, G);
  // the traces of each launch: a range of the plan's list when the launches
  // follow it (start[li] .. start[li + 1]), else copies bucketed by launch
  std::vector<size_t> start(nl + 1, 0);
  bool ranges = true;
  for (size_t k = 0; k < P.tr.size(); k++) {
    const GramPlan::Tr& t = P.tr[k];
    if (t.g < 0 || t.g >= P.ngroup || t.r < 0 || t.r >= P.mrows || t.c < 0 || t.c >= P.ncols)
      return fail(CTR_ERR_ARG, "Gram traces: trace (%d, %d, %d) outside the plan", t.g, t.r, t.c);
    if (k && t.g / G < P.tr[k - 1].g / G) ranges = false;
    start[t.g / G + 1]++;
  }
  for (int li = 0; li < nl; li++) start[li + 1] += start[li];
  std::vector<std::vector<GramTrace>> by;
  if (!ranges) {
    by.resize(nl);
    for (const GramPlan::Tr& t : P.tr) by[t.g / G].push_back(GramTrace{t.g, t.r, t.c, t.slot, {t.cre, t.cim}});
  }
  for (int li = 0; li < nl; li++) {
    const int g0 = li * G, ng = std::min(G, P.ngroup - g0), ni = ng * npiece;
    void* mem;
    CTR_TRY(workspace(WS_GRAM).get((size_t)ni * per_inst + 1024, &mem));
    uint8_t* lsl = (uint8_t*)mem;
    uint8_t* rsl = lsl + (size_t)ni * l_b;
    double2* part = (double2*)(rsl + (size_t)ni * r_b);
    int* lexp = (int*)(part + (size_t)ni * lrows * rcols);
    int* rexp = lexp + (size_t)ni * lrows;
    float* lnorm = (float*)(rexp + (size_t)ni * rcols);
    float* rnorm = lnorm + (size_t)ni * lrows;
    std::vector<SplitGemmInst> gi(ni);
    std::vector<double2*> outs(ni);
    for (int ip = 0; ip < ni; ip++) {
      outs[ip] = part + (size_t)ip * lrows * rcols;
      gi[ip] = SplitGemmInst{lsl + (size_t)ip * l_b, rsl + (size_t)ip * r_b, lexp + (size_t)ip * lrows,
                             rexp + (size_t)ip * rcols, nullptr, nullptr};
    }
    const GramTrace* tl = ranges ? (const GramTrace*)P.tr.data() + start[li] : by[li].data();
    const size_t ntl = start[li + 1] - start[li];
    void* d[3];
    CTR_TRY(upload_group(WS_GRAMJOBS,
                         {{P.left.data() + (size_t)g0 * P.mrows, (size_t)ng * P.mrows * sizeof(const double2*)},
                          {P.right.data() + (size_t)g0 * P.ncols, (size_t)ng * P.ncols * sizeof(const double2*)},
                          {outs.data(), outs.size() * sizeof(double2*)}},
                         d, stream));
    void* d_tr;
    CTR_TRY(upload(WS_GRAMTRACES, tl, ntl * sizeof(GramTrace), &d_tr, stream));
    for (int ip = 0; ip < ni; ip++) gi[ip].outs = (double2* const*)d[2] + ip;
    void* d_gi;
    CTR_TRY(upload(WS_GEMM_B, gi.data(), gi.size() * sizeof(SplitGemmInst), &d_gi, stream));
    CTR_TRY(launch_slice_gram(false, (const double2* const*)d[0], ng, P.mrows, mtiles, n2, npiece, nchunk, lsl, lexp,
                              lnorm, stream));
    CTR_TRY(launch_slice_gram(true, (const double2* const*)d[1], ng, P.ncols, ntiles, n2, npiece, nchunk, rsl, rexp,
                              rnorm, stream));
    SplitGemmBatch B{(const SplitGemmInst*)d_gi, mtiles, ntiles, nchunk, P.mrows, P.ncols, lrows, nullptr, 1, rcols, 1};
    B.order = 0;
    CTR_TRY(launch_split_gemm(B, ni, d_err, stream, true));
    CTR_TRY(launch_gram_trace_sum((const GramTrace*)d_tr, (int)ntl, g0, part, npiece, lrows, rcols, lexp, rexp, lnorm,
                                  rnorm, trv, tra, stream));
  }
  if (!capturing()) g_gram_traces += (double)P.tr.size();
  return CTR_OK;
}

}  // namespace ctr
