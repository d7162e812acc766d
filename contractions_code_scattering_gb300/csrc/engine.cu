// Diagram orchestration and the C ABI entry points of the two-sided (rho-type)
// contractions.
//
// A two-sided row is coef * Tr[(Phi_R(tf) tau_ab)^dagger (tau_cd Phi_L(ti))]
// (lib/calculate_rho_core.h:40-152, lib/calculate_sigma_one_fish_core.h:38-143).
// The reference recomputes both 100^3 products for every spin row (768 rows x
// 2 products per (tf,ti) for rho).  Here the distinct factors are computed once
// per (tf,ti):  A_{cd,L} = tau_cd Phi_L(ti)  and  B_{ab,R} = Phi_R(tf) tau_ab,
// and every row is a Hadamard trace between one A and one B block.
#include <algorithm>
#include <map>
#include <tuple>

#include "kernels.h"

namespace ctr {

namespace {

struct Plan2 {
  std::vector<std::tuple<int, int, int>> keysA;  // (c, d, L)
  std::vector<std::tuple<int, int, int>> keysB;  // (a, b, R)
  std::vector<int> rowA, rowB;
  std::vector<int> off, idx;  // CSR of rows per output, ascending row index
};

int make_plan(const std::vector<TwoSidedRow>& rows, const std::vector<int32_t>& out_index, int nout, int nphi,
              Plan2& P) {
  std::map<std::tuple<int, int, int>, int> ma, mb;
  P.rowA.resize(rows.size());
  P.rowB.resize(rows.size());
  for (size_t r = 0; r < rows.size(); r++) {
    const TwoSidedRow& w = rows[r];
    if (w.a < 0 || w.a > 3 || w.b < 0 || w.b > 3 || w.c < 0 || w.c > 3 || w.d < 0 || w.d > 3)
      return fail(CTR_ERR_ARG, "two-sided row %zu: spin index out of [0,4)", r);
    if (w.L < 0 || w.L >= nphi || w.R < 0 || w.R >= nphi)
      return fail(CTR_ERR_ARG, "two-sided row %zu: elemental index out of [0,%d)", r, nphi);
    if (out_index[r] < 0 || out_index[r] >= nout)
      return fail(CTR_ERR_ARG, "two-sided row %zu: out_index %d out of [0,%d)", r, out_index[r], nout);
    auto ka = std::make_tuple((int)w.c, (int)w.d, (int)w.L);
    auto kb = std::make_tuple((int)w.a, (int)w.b, (int)w.R);
    auto ia = ma.find(ka);
    if (ia == ma.end()) ia = ma.emplace(ka, (int)P.keysA.size()).first, P.keysA.push_back(ka);
    auto ib = mb.find(kb);
    if (ib == mb.end()) ib = mb.emplace(kb, (int)P.keysB.size()).first, P.keysB.push_back(kb);
    P.rowA[r] = ia->second;
    P.rowB[r] = ib->second;
  }
  P.off.assign(nout + 1, 0);
  for (size_t r = 0; r < rows.size(); r++) P.off[out_index[r] + 1]++;
  for (int o = 0; o < nout; o++) P.off[o + 1] += P.off[o];
  P.idx.resize(rows.size());
  std::vector<int> fill(P.off.begin(), P.off.end() - 1);
  for (size_t r = 0; r < rows.size(); r++) P.idx[fill[out_index[r]]++] = (int)r;
  return CTR_OK;
}

}  // namespace

int twosided_fp64(int N, int Nt, int tf_begin, int tf_end, const double* prop_rows, const double* phi, int nphi,
                  const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                  const std::vector<int32_t>& out_index, int nout, double* out, cudaStream_t stream) {
  Plan2 P;
  CTR_TRY(make_plan(rows, out_index, nout, nphi, P));
  const int nrows = (int)rows.size();
  const size_t N2 = (size_t)N * N;
  const int nA = (int)P.keysA.size(), nB = (int)P.keysB.size();
  const size_t per_pair = (size_t)(nA + nB) * N2 * sizeof(double2);
  const size_t budget = (size_t)2 << 30;
  const int npairs_total = (tf_end - tf_begin) * Nt;
  int batch = (int)std::max<size_t>(1, budget / per_pair);
  batch = std::min(batch, npairs_total);

  // CSR of output rows (constant for all batches)
  std::vector<int> csr(P.off);
  csr.insert(csr.end(), P.idx.begin(), P.idx.end());
  void* d_csr;
  CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, stream));
  const int* d_off = (const int*)d_csr;
  const int* d_idx = d_off + (nout + 1);

  const double2* tau = (const double2*)prop_rows;
  const double2* ph = (const double2*)phi;
  std::vector<ZTask> gt;
  std::vector<TraceTask> tt;
  for (int p0 = 0; p0 < npairs_total; p0 += batch) {
    const int np = std::min(batch, npairs_total - p0);
    void *scratch, *rowbuf;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * per_pair, &scratch));
    CTR_TRY(workspace(WS_ROWS).get((size_t)np * nrows * sizeof(double2), &rowbuf));
    double2* S = (double2*)scratch;
    double2* R = (double2*)rowbuf;
    gt.clear();
    tt.clear();
    for (int q = 0; q < np; q++) {
      const int pr = p0 + q;
      const int tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* tblk = tau + ((size_t)tfl * Nt + ti) * 16 * N2;
      double2* SA = S + (size_t)q * (nA + nB) * N2;
      double2* SB = SA + (size_t)nA * N2;
      for (int k = 0; k < nA; k++) {
        int c, d, L;
        std::tie(c, d, L) = P.keysA[k];
        ZTask z{};
        z.A[0] = tblk + (size_t)(c * 4 + d) * N2;
        z.B[0] = ph + ((size_t)ti * nphi + L) * N2;
        z.C = SA + (size_t)k * N2;
        z.wre[0] = 1.f;
        z.nterm = 1;
        gt.push_back(z);
      }
      for (int k = 0; k < nB; k++) {
        int a, b, Rr;
        std::tie(a, b, Rr) = P.keysB[k];
        ZTask z{};
        z.A[0] = ph + ((size_t)tf * nphi + Rr) * N2;
        z.B[0] = tblk + (size_t)(a * 4 + b) * N2;
        z.C = SB + (size_t)k * N2;
        z.wre[0] = 1.f;
        z.nterm = 1;
        gt.push_back(z);
      }
      for (int r = 0; r < nrows; r++) {
        TraceTask t{};
        t.X = SA + (size_t)P.rowA[r] * N2;
        t.Y = SB + (size_t)P.rowB[r] * N2;
        t.out = R + (size_t)q * nrows + r;
        t.coef[0] = coef[2 * r];
        t.coef[1] = coef[2 * r + 1];
        t.mode = 0;
        tt.push_back(t);
      }
    }
    void *d_gt, *d_tt;
    CTR_TRY(upload(WS_TASKS, gt.data(), gt.size() * sizeof(ZTask), &d_gt, stream));
    CTR_TRY(launch_zgemm_f64((const ZTask*)d_gt, (int)gt.size(), N, stream, gt.data()));
    // The trace tasks live behind the GEMM tasks in a second upload slot.
    CTR_TRY(upload(WS_ROWTASKS, tt.data(), tt.size() * sizeof(TraceTask), &d_tt, stream));
    CTR_TRY(launch_trace_f64((const TraceTask*)d_tt, (int)tt.size(), N, stream));
    CTR_TRY(launch_rowsum(R, nrows, d_off, d_idx, nout, np, (double2*)out + (size_t)p0 * nout, nout, stream));
  }
  return CTR_OK;
}

// Rows of the reference's rho table in two-sided form.
static void rho_rows(std::vector<TwoSidedRow>& rows, std::vector<float>& coef, std::vector<int32_t>& oi) {
  const Tables& T = tables();
  rows.resize(768);
  coef.resize(1536);
  oi.resize(768);
  for (int r = 0; r < 768; r++) {
    const int16_t* s = T.rho_spin[r];
    rows[r] = TwoSidedRow{s[0], s[1], s[2], s[3], T.rho_lprp[r][0], T.rho_lprp[r][1]};
    coef[2 * r] = T.rho_coef[r][0];
    coef[2 * r + 1] = T.rho_coef[r][1];
    oi[r] = r / 16;  // (op pair, direction) = bx / 16 (lib/contract_kernels_rho.cu:110-116)
  }
}

// Rows of the sigma one-fish table: T1 = tau_{s3s4} Phix2_rp(ti),
// T2 = Phix2_lp(tf) tau_{s2s1} (lib/calculate_sigma_one_fish_core.h:38-103).
static void sigma_rows(std::vector<TwoSidedRow>& rows, std::vector<float>& coef, std::vector<int32_t>& oi) {
  const Tables& T = tables();
  rows.resize(64);
  coef.resize(128);
  oi.resize(64);
  for (int r = 0; r < 64; r++) {
    const int16_t* s = T.sigma_spin[r];
    rows[r] = TwoSidedRow{s[1], s[0], s[2], s[3], T.sigma_lprp[r][1], T.sigma_lprp[r][0]};
    coef[2 * r] = T.sigma_coef[r][0];
    coef[2 * r + 1] = T.sigma_coef[r][1];
    oi[r] = r / 16;
  }
}

static int check_common(int engine, int nev, int nt, int tf_begin, int tf_end, const void* prop, const void* phi,
                        const void* out) {
  if (engine != CTR_ENGINE_FP64 && engine != CTR_ENGINE_SPLIT) return fail(CTR_ERR_ARG, "unknown engine %d", engine);
  if (nev < 1 || nev > 4096) return fail(CTR_ERR_ARG, "nev %d out of range", nev);
  if (nt < 1) return fail(CTR_ERR_ARG, "nt %d out of range", nt);
  if (tf_begin < 0 || tf_end > nt || tf_begin >= tf_end)
    return fail(CTR_ERR_ARG, "t_sink range [%d,%d) invalid for Nt=%d", tf_begin, tf_end, nt);
  if (!prop || !phi || !out) return fail(CTR_ERR_ARG, "null device pointer");
  if (((uintptr_t)prop | (uintptr_t)phi | (uintptr_t)out) & 15)
    return fail(CTR_ERR_ARG, "device pointers must be 16-byte aligned");
  return CTR_OK;
}

static int dispatch_twosided(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop,
                             const double* phi, int nphi, const std::vector<TwoSidedRow>& rows,
                             const std::vector<float>& coef, const std::vector<int32_t>& oi, int nout, double* out,
                             cudaStream_t s) {
  if (engine == CTR_ENGINE_SPLIT)
    return twosided_split(nev, nt, tf_begin, tf_end, prop, phi, nphi, rows, coef, oi, nout, out, s);
  return twosided_fp64(nev, nt, tf_begin, tf_end, prop, phi, nphi, rows, coef, oi, nout, out, s);
}

}  // namespace ctr

extern "C" {

int ctr_twosided(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows, const double* phi,
                 int nphi, int nrows, const int16_t* rows, const float* coef, const int32_t* out_index, int nout,
                 double* out, void* stream) {
  CTR_TRY(ctr::check_common(engine, nev, nt, tf_begin, tf_end, prop_rows, phi, out));
  if (nrows < 1 || !rows || !coef || !out_index || nout < 1 || nphi < 1)
    return ctr::fail(CTR_ERR_ARG, "ctr_twosided: empty row table or bad sizes");
  std::vector<ctr::TwoSidedRow> rv(nrows);
  for (int r = 0; r < nrows; r++)
    rv[r] = ctr::TwoSidedRow{rows[6 * r], rows[6 * r + 1], rows[6 * r + 2], rows[6 * r + 3], rows[6 * r + 4],
                             rows[6 * r + 5]};
  std::vector<float> cv(coef, coef + 2 * (size_t)nrows);
  std::vector<int32_t> ov(out_index, out_index + nrows);
  return ctr::dispatch_twosided(engine, nev, nt, tf_begin, tf_end, prop_rows, phi, nphi, rv, cv, ov, nout, out,
                                (cudaStream_t)stream);
}

int ctr_rho(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows, const double* mom5,
            double* corr, void* stream) {
  CTR_TRY(ctr::check_common(engine, nev, nt, tf_begin, tf_end, prop_rows, mom5, corr));
  std::vector<ctr::TwoSidedRow> rows;
  std::vector<float> coef;
  std::vector<int32_t> oi;
  ctr::rho_rows(rows, coef, oi);
  return ctr::dispatch_twosided(engine, nev, nt, tf_begin, tf_end, prop_rows, mom5, 5, rows, coef, oi, 48, corr,
                                (cudaStream_t)stream);
}

int ctr_sigma(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows, const double* mom2,
              double* corr, void* stream) {
  CTR_TRY(ctr::check_common(engine, nev, nt, tf_begin, tf_end, prop_rows, mom2, corr));
  std::vector<ctr::TwoSidedRow> rows;
  std::vector<float> coef;
  std::vector<int32_t> oi;
  ctr::sigma_rows(rows, coef, oi);
  return ctr::dispatch_twosided(engine, nev, nt, tf_begin, tf_end, prop_rows, mom2, 2, rows, coef, oi, 4, corr,
                                (cudaStream_t)stream);
}

int ctr_source_average(int nt, int ncorr, const double* corr, double scale, double* avg, void* stream) {
  if (nt < 1 || ncorr < 1 || !corr || !avg) return ctr::fail(CTR_ERR_ARG, "ctr_source_average: bad arguments");
  return ctr::launch_source_average(nt, ncorr, (const double2*)corr, scale, (double2*)avg, (cudaStream_t)stream);
}

int ctr_mma_schedule_probe(int hp, int nchunk, double* clocks_per_mma, double* tflops, void* stream) {
  CTR_NO_CAPTURE("ctr_mma_schedule_probe");
  if (nchunk < 1 || nchunk > (1 << 20) || !clocks_per_mma || !tflops)
    return ctr::fail(CTR_ERR_ARG, "ctr_mma_schedule_probe: nchunk %d not in [1, 2^20] or null outputs", nchunk);
  return ctr::mma_schedule_probe(hp ? 1 : 0, nchunk, clocks_per_mma, tflops, (cudaStream_t)stream);
}

int ctr_wait_probe(int timeout_ms, void* stream) {
  CTR_NO_CAPTURE("ctr_wait_probe");
  if (timeout_ms < 1 || timeout_ms > 1000) return ctr::fail(CTR_ERR_ARG, "ctr_wait_probe: timeout %d ms not in [1, 1000]", timeout_ms);
  return ctr::wait_probe(timeout_ms, (cudaStream_t)stream);
}

int ctr_sync(void* stream) {
  CTR_NO_CAPTURE("ctr_sync");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return ctr::cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
  return ctr::split_error_check((cudaStream_t)stream);
}

int ctr_zgemm_batched(int engine, int nev, int nbatch, const double* const* x, const double* const* y,
                      double* const* c, void* stream) {
  if (engine != CTR_ENGINE_FP64 && engine != CTR_ENGINE_SPLIT) return ctr::fail(CTR_ERR_ARG, "unknown engine %d", engine);
  if (nev < 1 || nbatch < 0 || (nbatch > 0 && (!x || !y || !c)))
    return ctr::fail(CTR_ERR_ARG, "ctr_zgemm_batched: bad arguments");
  for (int b = 0; b < nbatch; b++)
    if (!x[b] || !y[b] || !c[b] || (((uintptr_t)x[b] | (uintptr_t)y[b] | (uintptr_t)c[b]) & 15))
      return ctr::fail(CTR_ERR_ARG, "ctr_zgemm_batched: null or misaligned pointer in entry %d", b);
  if (nbatch == 0) return CTR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (engine == CTR_ENGINE_SPLIT) return ctr::zgemm_split_batched(nev, nbatch, x, y, c, s);
  std::vector<ctr::ZTask> t(nbatch);
  for (int b = 0; b < nbatch; b++) {
    t[b] = ctr::ZTask{};
    t[b].A[0] = (const double2*)x[b];
    t[b].B[0] = (const double2*)y[b];
    t[b].C = (double2*)c[b];
    t[b].wre[0] = 1.f;
    t[b].nterm = 1;
  }
  void* d;
  CTR_TRY(ctr::upload(ctr::WS_TASKS, t.data(), t.size() * sizeof(ctr::ZTask), &d, s));
  return ctr::launch_zgemm_f64((const ctr::ZTask*)d, nbatch, nev, s, t.data());
}

}  // extern "C"

extern "C" int ctr_zgemm_tasks(int engine, int nev, int ntask, const ctr_ztask* tasks, void* stream) {
  static_assert(sizeof(ctr_ztask) == sizeof(ctr::ZTask), "ctr_ztask and ZTask must match");
  if (nev < 1 || ntask < 0 || (ntask > 0 && !tasks)) return ctr::fail(CTR_ERR_ARG, "ctr_zgemm_tasks: bad arguments");
  for (int t = 0; t < ntask; t++) {
    const ctr_ztask& z = tasks[t];
    if (z.nterm < 1 || z.nterm > 4 || !z.c) return ctr::fail(CTR_ERR_ARG, "ctr_zgemm_tasks: task %d malformed", t);
    for (int q = 0; q < z.nterm; q++)
      if (!z.a[q] || !z.b[q]) return ctr::fail(CTR_ERR_ARG, "ctr_zgemm_tasks: task %d operand %d is null", t, q);
  }
  const ctr::ZTask* zt = reinterpret_cast<const ctr::ZTask*>(tasks);
  cudaStream_t s = (cudaStream_t)stream;
  if (engine == CTR_ENGINE_SPLIT) return ctr::zgemm_split_tasks(nev, zt, ntask, s);
  if (engine != CTR_ENGINE_FP64) return ctr::fail(CTR_ERR_ARG, "unknown engine %d", engine);
  void* d;
  CTR_TRY(ctr::upload(ctr::WS_GEMM_A, zt, (size_t)ntask * sizeof(ctr::ZTask), &d, s));
  return ctr::launch_zgemm_f64((const ctr::ZTask*)d, ntask, nev, s, zt);
}
