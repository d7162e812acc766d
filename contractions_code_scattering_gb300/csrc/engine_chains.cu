// Chain diagrams: rho->pipi, pipi->pipi (I=1, I=0), loop-unity, sigma->pipi,
// on either engine: every GEMM stage below is a list of block-product tasks
// that runs on the FP64 tile kernel or on the split-precision tensor-core
// engine (zgemm_split_tasks); the closing traces are FP64 in both.
//
// The reference evaluates every spin row as an independent chain of 2-6 Nev^3
// products (lib/calculate_{rhopi,pipi_*,sigmapi_*,loop_unity}_core.h).  The
// tables are gamma_5-diagonal in the summed indices, so the spin sums factor
// into 4x4 spin-block matrix products, with G = diag(gamma_5) x 1:
//   R(t)  = Phi_a(t) tau(t,t)_{..} Phi_b(t)                     (per time slice)
//   L(t)  = Phi3(t) tau(t,t)_{..} Phi4(t)
//   square(tf,ti) = Tr[L G T G Rsq T^dag],  Rsq = Phi2 taud Phi1
//   dtri(tf,ti)   = Tr[L G T G Rdt T^dag],  Rdt = Phi1 taud Phi2
//   dtri_hor      = Tr[Phi3 (T Phi1 T^dag) Phi4 (T Phi2 T^dag)]
//   star / fish   = products of Tr-sums of (Phi_x(tf) tau_ab Phi_y(ti)) (.) conj tau_ab
//   rho->pipi     = sum c * Tr[Phi_ip (T G R)_{s5 s2} tau_{s3 s2}^dag]
//   sigma->pipi triangle = sum g5(s1) Tr[Phi_ik (T G R)_{s1 s5} tau_{s1 s5}^dag]
// with T = tau(tf,ti) as a 4x4 block matrix.  Each block product is one task of
// the batched FP64 GEMM (up to 4 accumulated terms with the gamma_5 signs).
#include <algorithm>
#include <cstring>

#include "kernels.h"

namespace ctr {

namespace {

constexpr int G5[4] = {1, 1, -1, -1};  // gamma_5 = diag(1,1,-1,-1) of the table basis

struct Ctx {
  int N, Nt;
  size_t N2;
  cudaStream_t s;
  int engine = CTR_ENGINE_FP64;
};

inline ZTask zt(const double2* A, const double2* B, double2* C, int flags = 0) {
  ZTask z{};
  z.A[0] = A;
  z.B[0] = B;
  z.C = C;
  z.wre[0] = 1.f;
  z.nterm = 1;
  z.flags = flags;
  return z;
}

// Stage = one launch of the batched GEMM; stages run in order on the stream.
int run_stage(const Ctx& c, const std::vector<ZTask>& tasks, int slot) {
  if (tasks.empty()) return CTR_OK;
  if (c.engine == CTR_ENGINE_SPLIT) return zgemm_split_tasks(c.N, tasks.data(), (int)tasks.size(), c.s);
  void* d;
  CTR_TRY(upload(slot, tasks.data(), tasks.size() * sizeof(ZTask), &d, c.s));
  return launch_zgemm_f64((const ZTask*)d, (int)tasks.size(), c.N, c.s, tasks.data());
}

int run_traces(const Ctx& c, const std::vector<TraceTask>& t) {
  if (t.empty()) return CTR_OK;
  void* d;
  CTR_TRY(upload(WS_ROWTASKS, t.data(), t.size() * sizeof(TraceTask), &d, c.s));
  return launch_trace_f64((const TraceTask*)d, (int)t.size(), c.N, c.s);
}

inline TraceTask tr(const double2* X, const double2* Y, double2* out, float cre, float cim, int mode) {
  TraceTask t{};
  t.X = X;
  t.Y = Y;
  t.out = out;
  t.coef[0] = cre;
  t.coef[1] = cim;
  t.mode = mode;
  return t;
}

// R(t)_{ab} = Pa(t) taud(t)_{ab} Pb(t) for all t (or the t with tmask[t] set)
// and the 16 spin blocks -> out[t][16][N][N]; tmp holds the same amount.
int per_t_chain(const Ctx& c, const double2* diag, const double2* Pa, size_t pa_t, const double2* Pb, size_t pb_t,
                double2* tmp, double2* out, const std::vector<char>* tmask = nullptr) {
  std::vector<ZTask> s1, s2;
  for (int t = 0; t < c.Nt; t++)
    for (int b = 0; b < 16 && (!tmask || (*tmask)[t]); b++) {
      const size_t o = ((size_t)t * 16 + b) * c.N2;
      s1.push_back(zt(Pa + t * pa_t, diag + o, tmp + o));
      s2.push_back(zt(tmp + o, Pb + t * pb_t, out + o));
    }
  CTR_TRY(run_stage(c, s1, WS_TASKS));
  return run_stage(c, s2, WS_TASKS2);
}

// X = M1 G M2 as 4x4 block matrices (X_{ab} = sum_c M1_{ac} g5(c) M2_{cb}).
void block_gemm_g5(const Ctx& c, const double2* M1, const double2* M2, double2* X, std::vector<ZTask>& out,
                   bool use_g5 = true) {
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      ZTask z{};
      for (int k = 0; k < 4; k++) {
        z.A[k] = M1 + (size_t)(a * 4 + k) * c.N2;
        z.B[k] = M2 + (size_t)(k * 4 + b) * c.N2;
        z.wre[k] = use_g5 ? (float)G5[k] : 1.f;
      }
      z.nterm = 4;
      z.C = X + (size_t)(a * 4 + b) * c.N2;
      out.push_back(z);
    }
}

__global__ void pipi_combine_kernel(const double2* __restrict__ tr, int ntr, int npair, int iso,
                                    double2* __restrict__ out, const double* __restrict__ trabs, double eps_over_tol,
                                    int* __restrict__ count, int* __restrict__ list, int pair_base) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const double2* t = tr + (size_t)p * ntr;
  // layout per pair: [0,16) square, [16,32) dtri, [32,48) dtri_hor,
  // [48,64) Tr[U4 W1], [64,80) Tr[U3 W2], [80,96) Tr[U3 W1], [96,112) Tr[U4 W2]
  double2 sum[7];
  double ab[7];
  for (int g = 0; g < 7; g++) {
    double re = 0, im = 0, a = 0;
    for (int k = 0; k < 16; k++) {
      re += t[g * 16 + k].x;
      im += t[g * 16 + k].y;
      if (trabs) a += trabs[(size_t)p * ntr + g * 16 + k];
    }
    sum[g] = make_double2(re, im);
    ab[g] = a;
  }
  const double2 star = cmul(sum[3], sum[4]);
  const double2 fish = cmul(sum[5], sum[6]);
  double2* o = out + (size_t)p * 5;
  if (iso == 1) {  // lib/contract_kernels_pipi.cu:288-303
    o[0] = make_double2(-2. * sum[0].x, -2. * sum[0].y);
    o[1] = make_double2(2. * sum[1].x, 2. * sum[1].y);
    o[2] = make_double2(-star.x, -star.y);
    o[3] = fish;
    o[4] = make_double2(0., 0.);
  } else {  // lib/contract_kernels_pipi.cu:463-478
    o[0] = make_double2((-1. / 3.) * sum[0].x, (-1. / 3.) * sum[0].y);
    o[1] = make_double2(-(1. / 3.) * sum[1].x, -(1. / 3.) * sum[1].y);
    o[2] = star;
    o[3] = fish;
    o[4] = make_double2(-(5. / 3.) * sum[2].x, -(5. / 3.) * sum[2].y);
  }
  if (trabs && eps_over_tol > 0.0) {
    auto mag = [](double2 v) { return sqrt(v.x * v.x + v.y * v.y); };
    const double w[3] = {iso == 1 ? 2.0 : 1.0 / 3.0, iso == 1 ? 2.0 : 1.0 / 3.0, iso == 1 ? 0.0 : 5.0 / 3.0};
    const double scale[5] = {w[0] * ab[0], w[1] * ab[1], mag(sum[3]) * ab[4] + mag(sum[4]) * ab[3],
                             mag(sum[5]) * ab[6] + mag(sum[6]) * ab[5], w[2] * ab[2]};
    // flagged: an error estimate above the tolerance (or not a number), or an
    // error scale that underflowed while the value did not
    for (int k = 0; k < 5; k++)
      if (!(scale[k] * eps_over_tol <= mag(o[k])) || (scale[k] == 0.0 && mag(o[k]) > 0.0)) {
        list[atomicAdd(count, 1)] = (pair_base + p) * 5 + k;
        break;
      }
  }
}

// ---- per-entry refinement of split-engine chains
// A chain entry's rounding error is estimated as REFINE_EPS_CHAIN times the sum
// of |coef| sum |Y|_1 |T|_1 over its closing traces (for products of traces,
// the product rule of those scales).  The chain products run on the
// high-precision split configuration (6 slices, levels 0-3 exact, exact integer
// recombination), which keeps ~2^-53 of their row/column scales.  Measured on
// the 20 480 entries of one pi pi momentum pair at Nev=100, Lt=64 against the
// FP64 engine, the largest entry error without any refinement was 1.8e-10;
// with REFINE_EPS_CHAIN = 2^-52 no entry is flagged there, and the check stays
// as the safety net for entries whose cancellation exceeds ~10^6.
constexpr double REFINE_EPS_CHAIN = 1.0 / 4503599627370496.0;  // 2^-52

struct Refine {
  bool on = false;
  double eps_over_tol = 0.0;
  int* count = nullptr;
  int* list = nullptr;
};

int refine_begin(const Ctx& c, size_t nentries, int slot, Refine& r) {
  r.on = c.engine == CTR_ENGINE_SPLIT && g_refine_tol > 0.0;
  if (!r.on) return CTR_OK;
  r.eps_over_tol = REFINE_EPS_CHAIN / g_refine_tol;
  void* p;
  CTR_TRY(workspace(slot).get((nentries + 1) * sizeof(int), &p));
  r.count = (int*)p;
  r.list = r.count + 1;
  CTR_CUDA(cudaMemsetAsync(r.count, 0, sizeof(int), c.s));
  return CTR_OK;
}

// Flagged entries e -> units e / nout (pairs or time slices); rerun(units, out,
// stream) writes their FP64 values as [units][nout] into out (device); they are
// then scattered over corr, and their number is added to g_refined_last.  The
// list is read on the host, so under graph recording this runs after the
// recorded kernels at every launch (the closure holds copies of what it needs).
template <typename Rerun>
int refine_end(const Ctx& c, const Refine& r, int nout, int slot, double2* corr, Rerun rerun) {
  if (!r.on) return CTR_OK;
  const int* count = r.count;
  const int* flagged = r.list;
  return host_step(c.s, [=](cudaStream_t s) -> int {
    int n = 0;
    CTR_TRY(download(&n, count, sizeof(int), s));
    if (n == 0) return CTR_OK;
    std::vector<int> list(n);
    CTR_TRY(download(list.data(), flagged, n * sizeof(int), s));
    std::vector<int> units;
    for (int e : list) units.push_back(e / nout);
    std::sort(units.begin(), units.end());
    units.erase(std::unique(units.begin(), units.end()), units.end());
    void* tmp;
    CTR_TRY(workspace(slot).get(units.size() * nout * sizeof(double2), &tmp));
    CTR_TRY(rerun(units, (double2*)tmp, s));
    std::vector<int> where(units.size() * nout);
    for (size_t q = 0; q < units.size(); q++)
      for (int o = 0; o < nout; o++) where[q * nout + o] = units[q] * nout + o;
    void* dw;
    CTR_TRY(upload(WS_TASKS, where.data(), where.size() * sizeof(int), &dw, s));
    CTR_TRY(launch_scatter((const int*)dw, (const double2*)tmp, (int)where.size(), corr, s));
    g_refined_last += (long long)where.size();
    return CTR_OK;
  });
}

int batch_pairs(size_t per_pair, int npairs) {
  const size_t budget = (size_t)3 << 30;
  return std::max(1, std::min(npairs, (int)(budget / std::max<size_t>(per_pair, 1))));
}

}  // namespace

// ------------------------------------------------------------------ pi pi
int pipi_chain(int N, int Nt, int tf_begin, int tf_end, int iso, const double* prop_rows, const double* prop_diag,
              const double* p1, const double* p2, const double* p3, const double* p4, double* corr, cudaStream_t s,
              int engine, const std::vector<int>* plist) {
  Ctx c{N, Nt, (size_t)N * N, s, engine};
  if (engine == CTR_ENGINE_SPLIT && !plist) g_refined_last = 0;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  const double2 *tau = (const double2*)prop_rows, *diag = (const double2*)prop_diag;
  const double2 *P1 = (const double2*)p1, *P2 = (const double2*)p2, *P3 = (const double2*)p3,
                *P4 = (const double2*)p4;
  const int npairs = plist ? (int)plist->size() : (tf_end - tf_begin) * Nt;
  auto pair_of = [&](int i) { return plist ? (*plist)[i] : i; };
  // per time slice: L = P3 taud P4 (sink times), Rsq = P2 taud P1, Rdt = P1 taud P2 (source times)
  std::vector<char> need_tf(Nt, plist ? 0 : 1), need_ti(Nt, plist ? 0 : 1);
  for (int i = 0; plist && i < npairs; i++) {
    need_tf[tf_begin + pair_of(i) / Nt] = 1;
    need_ti[pair_of(i) % Nt] = 1;
  }
  void* pt;
  CTR_TRY(workspace(WS_PHI).get(4 * (size_t)Nt * blk16 * sizeof(double2), &pt));
  double2 *L = (double2*)pt, *Rsq = L + Nt * blk16, *Rdt = Rsq + Nt * blk16, *tmp = Rdt + Nt * blk16;
  CTR_TRY(per_t_chain(c, diag, P3, N2, P4, N2, tmp, L, &need_tf));
  CTR_TRY(per_t_chain(c, diag, P2, N2, P1, N2, tmp, Rsq, &need_ti));
  CTR_TRY(per_t_chain(c, diag, P1, N2, P2, N2, tmp, Rdt, &need_ti));

  // per pair: X, Ysq, Ydt, V1, Pm, V2, Qm, F, G (16 blocks each), U3, U4, W1, W2
  const int nbuf = 13;
  const int ntr = 112;
  const size_t per_pair = (size_t)nbuf * blk16 * sizeof(double2) + ntr * sizeof(double2);
  const int batch = batch_pairs(per_pair, npairs);
  Refine rf;
  CTR_TRY(refine_begin(c, (size_t)npairs * 5, WS_REFINE, rf));
  for (int p0 = 0; p0 < npairs; p0 += batch) {
    const int np = std::min(batch, npairs - p0);
    void *mem, *trm, *tra = nullptr;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * nbuf * blk16 * sizeof(double2), &mem));
    CTR_TRY(workspace(WS_ROWS).get((size_t)np * ntr * sizeof(double2), &trm));
    if (rf.on) CTR_TRY(workspace(WS_ROWABS).get((size_t)np * ntr * sizeof(double), &tra));
    double2* B = (double2*)mem;
    double2* TR = (double2*)trm;
    double* TRA = (double*)tra;
    std::vector<ZTask> st1, st2, st3;
    std::vector<TraceTask> tt;
    for (int q = 0; q < np; q++) {
      const int pr = pair_of(p0 + q), tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* T = tau + ((size_t)tfl * Nt + ti) * blk16;
      double2* b0 = B + (size_t)q * nbuf * blk16;
      double2 *X = b0, *Ysq = b0 + blk16, *Ydt = b0 + 2 * blk16, *V1 = b0 + 3 * blk16, *Pm = b0 + 4 * blk16,
              *V2 = b0 + 5 * blk16, *Qm = b0 + 6 * blk16, *F = b0 + 7 * blk16, *Gm = b0 + 8 * blk16,
              *U3 = b0 + 9 * blk16, *U4 = b0 + 10 * blk16, *W1 = b0 + 11 * blk16, *W2 = b0 + 12 * blk16;
      const double2 *Lt = L + tf * blk16, *Rs = Rsq + ti * blk16, *Rd = Rdt + ti * blk16;
      block_gemm_g5(c, Lt, T, X, st1);  // X = L G T
      for (int b = 0; b < 16; b++) {
        const double2* tb = T + b * N2;
        if (iso == 0) {
          st1.push_back(zt(tb, P1 + ti * N2, V1 + b * N2));  // V1 = T Phi1
          st1.push_back(zt(tb, P2 + ti * N2, V2 + b * N2));  // V2 = T Phi2
        }
        st1.push_back(zt(P3 + tf * N2, tb, U3 + b * N2));       // U3 = Phi3 tau_b
        st1.push_back(zt(P4 + tf * N2, tb, U4 + b * N2));       // U4 = Phi4 tau_b
        st1.push_back(zt(P1 + ti * N2, tb, W1 + b * N2, 1 << 4));  // W1 = Phi1 tau_b^dag
        st1.push_back(zt(P2 + ti * N2, tb, W2 + b * N2, 1 << 4));  // W2 = Phi2 tau_b^dag
      }
      block_gemm_g5(c, X, Rs, Ysq, st2);  // Ysq = X G Rsq
      block_gemm_g5(c, X, Rd, Ydt, st2);  // Ydt = X G Rdt
      if (iso == 0) {
        // Pm = V1 T^dag, Qm = V2 T^dag (block (a,c) = sum_b V_{ab} tau_{cb}^dag)
        for (int a = 0; a < 4; a++)
          for (int cc = 0; cc < 4; cc++) {
            ZTask zp{}, zq{};
            for (int k = 0; k < 4; k++) {
              zp.A[k] = V1 + (a * 4 + k) * N2;
              zp.B[k] = T + (cc * 4 + k) * N2;
              zq.A[k] = V2 + (a * 4 + k) * N2;
              zq.B[k] = T + (cc * 4 + k) * N2;
              zp.wre[k] = zq.wre[k] = 1.f;
            }
            zp.nterm = zq.nterm = 4;
            zp.flags = zq.flags = 0xF0;  // B_k conj-transposed
            zp.C = Pm + (a * 4 + cc) * N2;
            zq.C = Qm + (a * 4 + cc) * N2;
            st2.push_back(zp);
            st2.push_back(zq);
          }
        for (int b = 0; b < 16; b++) {
          st3.push_back(zt(P3 + tf * N2, Pm + b * N2, F + b * N2));   // F = Phi3 P
          st3.push_back(zt(P4 + tf * N2, Qm + b * N2, Gm + b * N2));  // G = Phi4 Q
        }
      }
      double2* o = TR + (size_t)q * ntr;
      for (int b = 0; b < 16; b++) {
        const double2* tb = T + b * N2;
        tt.push_back(tr(Ysq + b * N2, tb, o + b, 1.f, 0.f, 0));
        tt.push_back(tr(Ydt + b * N2, tb, o + 16 + b, 1.f, 0.f, 0));
        if (iso == 0) {
          const int s1 = b / 4, s3 = b % 4;  // Tr[F_{s1 s3} G_{s3 s1}]
          tt.push_back(tr(F + b * N2, Gm + (s3 * 4 + s1) * N2, o + 32 + b, 1.f, 0.f, 1));
        }
        tt.push_back(tr(U4 + b * N2, W1 + b * N2, o + 48 + b, 1.f, 0.f, 1));
        tt.push_back(tr(U3 + b * N2, W2 + b * N2, o + 64 + b, 1.f, 0.f, 1));
        tt.push_back(tr(U3 + b * N2, W1 + b * N2, o + 80 + b, 1.f, 0.f, 1));
        tt.push_back(tr(U4 + b * N2, W2 + b * N2, o + 96 + b, 1.f, 0.f, 1));
      }
    }
    if (TRA)
      for (size_t k = 0; k < tt.size(); k++) tt[k].absout = TRA + (tt[k].out - TR);
    CTR_TRY(run_stage(c, st1, WS_TASKS));
    CTR_TRY(run_stage(c, st2, WS_TASKS2));
    CTR_TRY(run_stage(c, st3, WS_GEMM_A));
    CTR_TRY(run_traces(c, tt));
    {
      TimedLaunch tl(s, "pipi_combine");
      pipi_combine_kernel<<<(np + 127) / 128, 128, 0, s>>>(TR, ntr, np, iso, (double2*)corr + (size_t)p0 * 5, TRA,
                                                           rf.eps_over_tol, rf.count, rf.list, p0);
      CTR_CUDA(cudaGetLastError());
    }
  }
  return refine_end(c, rf, 5, WS_REFINE, (double2*)corr,
                    [=](const std::vector<int>& pairs, double2* out, cudaStream_t ls) {
                      return pipi_chain(N, Nt, tf_begin, tf_end, iso, prop_rows, prop_diag, p1, p2, p3, p4,
                                        (double*)out, ls, CTR_ENGINE_FP64, &pairs);
                    });
}

// ---------------------------------------------------------------- rho pipi
// Row form (lib/calculate_rhopi_core.h): coef * Tr[Phi^{P1P2}_ip(tf) tau_{s5s6}
// Phi_P2(ti) taud(ti)_{s1s2} Phi_P1(ti) tau_{s3s2}^dag] with s6 = s1, s4 = s3;
// coef = c(iop, s3, s5) * g5(s1), so the sum over s1 is (T G R)_{s5 s2}.
int rhopi_chain(int N, int Nt, int tf_begin, int tf_end, int idir, const double* prop_rows, const double* prop_diag,
                const double* mp1, const double* mp2, const double* mom5, double* corr, cudaStream_t s, int engine,
                const std::vector<int>* plist) {
  if (idir < 0 || idir > 2) return fail(CTR_ERR_ARG, "idir %d not in {0,1,2}", idir);
  Ctx c{N, Nt, (size_t)N * N, s, engine};
  if (engine == CTR_ENGINE_SPLIT && !plist) g_refined_last = 0;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  const double2 *tau = (const double2*)prop_rows, *diag = (const double2*)prop_diag;
  const double2 *P1 = (const double2*)mp1, *P2 = (const double2*)mp2, *P12 = (const double2*)mom5;
  const int npairs = plist ? (int)plist->size() : (tf_end - tf_begin) * Nt;
  auto pair_of = [&](int i) { return plist ? (*plist)[i] : i; };
  std::vector<char> need_ti(Nt, plist ? 0 : 1);
  for (int i = 0; plist && i < npairs; i++) need_ti[pair_of(i) % Nt] = 1;
  void* pt;
  CTR_TRY(workspace(WS_PHI).get(2 * (size_t)Nt * blk16 * sizeof(double2), &pt));
  double2 *R = (double2*)pt, *tmp = R + Nt * blk16;
  CTR_TRY(per_t_chain(c, diag, P2, N2, P1, N2, tmp, R, &need_ti));  // R = Phi_P2 taud Phi_P1

  // groups (iop, s2, s3): s5 from the table, c = coef * g5(s1); the 4 rows s1=0..3 share a group
  const Tables& Tb = tables();
  struct Grp { int iop, s2, s3, s5, ip; float cre, cim; };
  std::vector<Grp> grp;
  for (int bx = 0; bx < 256; bx++) {
    const int r = idir * 256 + bx;
    const int16_t* sp = Tb.rhopi_spin[r];
    const int s1 = sp[0], s2 = sp[1], s3 = sp[2], s5 = sp[4];
    if (sp[5] != s1 || sp[3] != s3) return fail(CTR_ERR_ARG, "rho-pipi table row %d not gamma_5-diagonal", r);
    if (s1 != 0) continue;  // one representative per group
    grp.push_back(Grp{bx / 64, s2, s3, s5, Tb.rhopi_ip[r], Tb.rhopi_coef[r][0] * G5[s1], Tb.rhopi_coef[r][1] * G5[s1]});
  }
  // distinct products Phi_ip(tf) X_{s5 s2}
  std::vector<int> pkeys;  // ip*16 + s5*4 + s2
  for (auto& g : grp) {
    int k = g.ip * 16 + g.s5 * 4 + g.s2;
    if (std::find(pkeys.begin(), pkeys.end(), k) == pkeys.end()) pkeys.push_back(k);
  }
  const int nprod = (int)pkeys.size(), ngrp = (int)grp.size();
  const int nbuf = 1 + (nprod + 15) / 16;
  const size_t per_pair = (size_t)(16 + nprod) * N2 * sizeof(double2) + ngrp * sizeof(double2);
  const int batch = batch_pairs(per_pair, npairs);
  (void)nbuf;
  Refine rf;
  CTR_TRY(refine_begin(c, (size_t)npairs * 4, WS_REFINE, rf));
  std::vector<int> off(5, 0), idx(ngrp);
  for (int g = 0; g < ngrp; g++) off[grp[g].iop + 1]++;
  for (int o = 0; o < 4; o++) off[o + 1] += off[o];
  {
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int g = 0; g < ngrp; g++) idx[fill[grp[g].iop]++] = g;
  }
  std::vector<int> csr(off);
  csr.insert(csr.end(), idx.begin(), idx.end());
  void* d_csr;
  CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, s));
  for (int p0 = 0; p0 < npairs; p0 += batch) {
    const int np = std::min(batch, npairs - p0);
    void *mem, *trm, *tra = nullptr;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * (16 + nprod) * N2 * sizeof(double2), &mem));
    CTR_TRY(workspace(WS_ROWS).get((size_t)np * ngrp * sizeof(double2), &trm));
    if (rf.on) CTR_TRY(workspace(WS_ROWABS).get((size_t)np * ngrp * sizeof(double), &tra));
    double2* Bm = (double2*)mem;
    double2* TR = (double2*)trm;
    double* TRA = (double*)tra;
    std::vector<ZTask> st1, st2;
    std::vector<TraceTask> tt;
    for (int q = 0; q < np; q++) {
      const int pr = pair_of(p0 + q), tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* T = tau + ((size_t)tfl * Nt + ti) * blk16;
      double2* X = Bm + (size_t)q * (16 + nprod) * N2;
      double2* Y = X + blk16;
      block_gemm_g5(c, T, R + ti * blk16, X, st1);  // X = T G R
      for (int k = 0; k < nprod; k++) {
        const int ip = pkeys[k] / 16, s5 = (pkeys[k] / 4) % 4, s2 = pkeys[k] % 4;
        st2.push_back(zt(P12 + ((size_t)tf * 5 + ip) * N2, X + (s5 * 4 + s2) * N2, Y + k * N2));
      }
      for (int g = 0; g < ngrp; g++) {
        const int k = (int)(std::find(pkeys.begin(), pkeys.end(), grp[g].ip * 16 + grp[g].s5 * 4 + grp[g].s2) -
                            pkeys.begin());
        tt.push_back(tr(Y + k * N2, T + (grp[g].s3 * 4 + grp[g].s2) * N2, TR + (size_t)q * ngrp + g, grp[g].cre,
                        grp[g].cim, 0));
      }
    }
    if (TRA)
      for (size_t k = 0; k < tt.size(); k++) tt[k].absout = TRA + (tt[k].out - TR);
    CTR_TRY(run_stage(c, st1, WS_TASKS));
    CTR_TRY(run_stage(c, st2, WS_TASKS2));
    CTR_TRY(run_traces(c, tt));
    if (rf.on)
      CTR_TRY(launch_rowsum_refine(TR, TRA, ngrp, (const int*)d_csr, (const int*)d_csr + 5, 4, np,
                                   (double2*)corr + (size_t)p0 * 4, rf.eps_over_tol, rf.count, rf.list, p0, s));
    else
      CTR_TRY(launch_rowsum(TR, ngrp, (const int*)d_csr, (const int*)d_csr + 5, 4, np,
                            (double2*)corr + (size_t)p0 * 4, 4, s));
  }
  return refine_end(c, rf, 4, WS_REFINE, (double2*)corr,
                    [=](const std::vector<int>& pairs, double2* out, cudaStream_t ls) {
                      return rhopi_chain(N, Nt, tf_begin, tf_end, idir, prop_rows, prop_diag, mp1, mp2, mom5,
                                         (double*)out, ls, CTR_ENGINE_FP64, &pairs);
                    });
}

// -------------------------------------------------------------- sigma pipi
// Horizontal fish (lib/calculate_sigmapi_hor_fish_core.h): per t,
// sum_ab coef * sum R_ab (.) conj taud_ab with R = Phi_P2 taud Phi_P1.
// Triangle (lib/calculate_sigmapi_triangle_core.h): rows with s2 = s1, s4 = s3,
// coef = g5(s1) g5(s3): sum_s3 g5(s3) tau_{s1s3} R_{s3s5} = (T G R)_{s1 s5}.
int sigmapi_chain(int N, int Nt, int tf_begin, int tf_end, const double* prop_rows, const double* prop_diag,
                  const double* mp1, const double* mp2, const double* mom2, double* hor_fish, double* tri,
                  cudaStream_t s, int engine, const std::vector<int>* plist, const std::vector<int>* tlist) {
  Ctx c{N, Nt, (size_t)N * N, s, engine};
  if (engine == CTR_ENGINE_SPLIT && !plist && !tlist) g_refined_last = 0;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  const double2 *tau = (const double2*)prop_rows, *diag = (const double2*)prop_diag;
  const double2 *P1 = (const double2*)mp1, *P2 = (const double2*)mp2, *Px2 = (const double2*)mom2;
  const Tables& Tb = tables();
  const int npairs = tri ? (plist ? (int)plist->size() : (tf_end - tf_begin) * Nt) : 0;
  const int nts = hor_fish ? (tlist ? (int)tlist->size() : Nt) : 0;
  auto pair_of = [&](int i) { return plist ? (*plist)[i] : i; };
  auto t_of = [&](int i) { return tlist ? (*tlist)[i] : i; };
  std::vector<char> need(Nt, 0);
  for (int i = 0; i < nts; i++) need[t_of(i)] = 1;
  for (int i = 0; i < npairs; i++) need[pair_of(i) % Nt] = 1;
  void* pt;
  // a recomputation (plist / tlist) keeps its own R, so that the caller's stays valid
  CTR_TRY(workspace((plist || tlist) ? WS_RPHI : WS_PHI).get(2 * (size_t)Nt * blk16 * sizeof(double2), &pt));
  double2 *R = (double2*)pt, *tmp = R + Nt * blk16;
  CTR_TRY(per_t_chain(c, diag, P2, N2, P1, N2, tmp, R, &need));
  if (hor_fish) {
    // lib/calculate_sigmapi_hor_fish_core.h: sum_ab coef * sum R_ab (.) conj taud_ab, per time slice
    Refine rf;
    CTR_TRY(refine_begin(c, (size_t)nts, WS_REFINE, rf));
    void *trm, *tra = nullptr;
    CTR_TRY(workspace(WS_ROWS).get((size_t)nts * 16 * sizeof(double2), &trm));
    if (rf.on) CTR_TRY(workspace(WS_ROWABS).get((size_t)nts * 16 * sizeof(double), &tra));
    std::vector<TraceTask> tt;
    for (int i = 0; i < nts; i++) {
      const int t = t_of(i);
      for (int b = 0; b < 16; b++) {
        const int ab = Tb.hf_spin[b][0] * 4 + Tb.hf_spin[b][1];
        tt.push_back(tr(R + t * blk16 + ab * N2, diag + t * blk16 + ab * N2, (double2*)trm + i * 16 + b,
                        Tb.hf_coef[b][0], Tb.hf_coef[b][1], 0));
        if (tra) tt.back().absout = (double*)tra + i * 16 + b;
      }
    }
    // one "pair" of nts outputs, 16 rows each
    std::vector<int> csr(nts + 1 + nts * 16);
    for (int i = 0; i <= nts; i++) csr[i] = 16 * i;
    for (int k = 0; k < nts * 16; k++) csr[nts + 1 + k] = k;
    void* d_csr;
    CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, s));
    CTR_TRY(run_traces(c, tt));
    if (rf.on)
      CTR_TRY(launch_rowsum_refine((double2*)trm, (double*)tra, nts * 16, (const int*)d_csr, (const int*)d_csr + nts + 1,
                                   nts, 1, (double2*)hor_fish, rf.eps_over_tol, rf.count, rf.list, 0, s));
    else
      CTR_TRY(launch_rowsum((double2*)trm, nts * 16, (const int*)d_csr, (const int*)d_csr + nts + 1, nts, 1,
                            (double2*)hor_fish, nts, s));
    // (the recomputation keeps its own R, so R above stays valid for the triangle)
    CTR_TRY(refine_end(c, rf, 1, WS_REFINE, (double2*)hor_fish,
                       [=](const std::vector<int>& ts, double2* out, cudaStream_t ls) {
                         return sigmapi_chain(N, Nt, tf_begin, tf_end, prop_rows, prop_diag, mp1, mp2, mom2,
                                              (double*)out, nullptr, ls, CTR_ENGINE_FP64, nullptr, &ts);
                       }));
  }
  if (!tri) return CTR_OK;
  // triangle (lib/calculate_sigmapi_triangle_core.h): X = T G R, Y_{ik, s1 s5} = Phix2_ik(tf) X_{s1 s5},
  // trace vs tau_{s1 s5}, weight g5(s1)
  const size_t per_pair = (size_t)(16 + 32) * N2 * sizeof(double2) + 32 * sizeof(double2);
  const int batch = batch_pairs(per_pair, npairs);
  std::vector<int> csr(3 + 32);
  csr[0] = 0; csr[1] = 16; csr[2] = 32;
  for (int k = 0; k < 32; k++) csr[3 + k] = k;
  void* d_csr;
  CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, s));
  Refine rf;
  CTR_TRY(refine_begin(c, (size_t)npairs * 2, WS_REFINE, rf));
  for (int p0 = 0; p0 < npairs; p0 += batch) {
    const int np = std::min(batch, npairs - p0);
    void *mem, *trm, *tra = nullptr;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * 48 * N2 * sizeof(double2), &mem));
    CTR_TRY(workspace(WS_ROWS).get((size_t)np * 32 * sizeof(double2), &trm));
    if (rf.on) CTR_TRY(workspace(WS_ROWABS).get((size_t)np * 32 * sizeof(double), &tra));
    double2* Bm = (double2*)mem;
    double2* TR = (double2*)trm;
    double* TRA = (double*)tra;
    std::vector<ZTask> st1, st2;
    std::vector<TraceTask> tt;
    for (int q = 0; q < np; q++) {
      const int pr = pair_of(p0 + q), tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* T = tau + ((size_t)tfl * Nt + ti) * blk16;
      double2* X = Bm + (size_t)q * 48 * N2;
      double2* Y = X + blk16;
      block_gemm_g5(c, T, R + ti * blk16, X, st1);
      for (int ik = 0; ik < 2; ik++)
        for (int b = 0; b < 16; b++) {
          st2.push_back(zt(Px2 + ((size_t)tf * 2 + ik) * N2, X + b * N2, Y + (ik * 16 + b) * N2));
          tt.push_back(tr(Y + (ik * 16 + b) * N2, T + b * N2, TR + (size_t)q * 32 + ik * 16 + b,
                          (float)G5[b / 4], 0.f, 0));
          if (TRA) tt.back().absout = TRA + (size_t)q * 32 + ik * 16 + b;
        }
    }
    CTR_TRY(run_stage(c, st1, WS_TASKS));
    CTR_TRY(run_stage(c, st2, WS_TASKS2));
    CTR_TRY(run_traces(c, tt));
    if (rf.on)
      CTR_TRY(launch_rowsum_refine(TR, TRA, 32, (const int*)d_csr, (const int*)d_csr + 3, 2, np,
                                   (double2*)tri + (size_t)p0 * 2, rf.eps_over_tol, rf.count, rf.list, p0, s));
    else
      CTR_TRY(launch_rowsum(TR, 32, (const int*)d_csr, (const int*)d_csr + 3, 2, np, (double2*)tri + (size_t)p0 * 2,
                            2, s));
  }
  return refine_end(c, rf, 2, WS_REFINE, (double2*)tri,
                    [=](const std::vector<int>& pairs, double2* out, cudaStream_t ls) {
                      return sigmapi_chain(N, Nt, tf_begin, tf_end, prop_rows, prop_diag, mp1, mp2, mom2, nullptr,
                                           (double*)out, ls, CTR_ENGINE_FP64, &pairs, nullptr);
                    });
}

// -------------------------------------------------------------- loop unity
// lib/calculate_loop_unity_core.h: L(t) = sum_s Tr[taud(t)_{ss} Phi(t)] (trace of a product: Nev^2 work).
int loop_unity_fp64(int N, int Nt, const double* prop_diag, const double* mom, double* loop, cudaStream_t s) {
  Ctx c{N, Nt, (size_t)N * N, s, CTR_ENGINE_FP64};
  const double2 *diag = (const double2*)prop_diag, *P = (const double2*)mom;
  void* trm;
  CTR_TRY(workspace(WS_ROWS).get((size_t)Nt * 4 * sizeof(double2), &trm));
  std::vector<TraceTask> tt;
  for (int t = 0; t < Nt; t++)
    for (int sp = 0; sp < 4; sp++)
      tt.push_back(tr(diag + ((size_t)t * 16 + sp * 5) * c.N2, P + (size_t)t * c.N2, (double2*)trm + t * 4 + sp, 1.f,
                      0.f, 1));
  std::vector<int> csr(Nt + 1 + Nt * 4);
  for (int t = 0; t <= Nt; t++) csr[t] = 4 * t;
  for (int k = 0; k < Nt * 4; k++) csr[Nt + 1 + k] = k;
  void* d_csr;
  CTR_TRY(upload(WS_MISC, csr.data(), csr.size() * sizeof(int), &d_csr, s));
  CTR_TRY(run_traces(c, tt));
  return launch_rowsum((double2*)trm, Nt * 4, (const int*)d_csr, (const int*)d_csr + Nt + 1, Nt, 1, (double2*)loop,
                       Nt, s);
}

}  // namespace ctr

// ------------------------------------------------------------------ C ABI
static int chain_args(int engine, int nev, int nt, int tf_begin, int tf_end) {
  if (engine != CTR_ENGINE_FP64 && engine != CTR_ENGINE_SPLIT) return ctr::fail(CTR_ERR_ARG, "unknown engine %d", engine);
  if (nev < 1 || nt < 1 || tf_begin < 0 || tf_end > nt || tf_begin >= tf_end)
    return ctr::fail(CTR_ERR_ARG, "bad sizes (nev=%d nt=%d t_sink [%d,%d))", nev, nt, tf_begin, tf_end);
  return CTR_OK;
}

static bool aligned(const void* p) { return p && (((uintptr_t)p & 15) == 0); }

extern "C" {

int ctr_rhopi(int engine, int nev, int nt, int tf_begin, int tf_end, int idir, const double* prop_rows,
              const double* prop_diag, const double* mom_p1, const double* mom_p2, const double* mom5_p1p2,
              double* corr, void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, tf_begin, tf_end));
  if (!aligned(prop_rows) || !aligned(prop_diag) || !aligned(mom_p1) || !aligned(mom_p2) || !aligned(mom5_p1p2) ||
      !aligned(corr))
    return ctr::fail(CTR_ERR_ARG, "ctr_rhopi: null or misaligned pointer");
  return ctr::rhopi_chain(nev, nt, tf_begin, tf_end, idir, prop_rows, prop_diag, mom_p1, mom_p2, mom5_p1p2, corr,
                          (cudaStream_t)stream, engine, nullptr);
}

int ctr_pipi(int engine, int nev, int nt, int tf_begin, int tf_end, int isospin, const double* prop_rows,
             const double* prop_diag, const double* p1, const double* p2, const double* p3, const double* p4,
             double* corr, void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, tf_begin, tf_end));
  if (isospin != 0 && isospin != 1) return ctr::fail(CTR_ERR_ARG, "isospin must be 0 (I=0) or 1 (I=1)");
  if (!aligned(prop_rows) || !aligned(prop_diag) || !aligned(p1) || !aligned(p2) || !aligned(p3) || !aligned(p4) ||
      !aligned(corr))
    return ctr::fail(CTR_ERR_ARG, "ctr_pipi: null or misaligned pointer");
  return ctr::pipi_chain(nev, nt, tf_begin, tf_end, isospin, prop_rows, prop_diag, p1, p2, p3, p4, corr,
                         (cudaStream_t)stream, engine, nullptr);
}

int ctr_loop_unity(int engine, int nev, int nt, const double* prop_diag, const double* mom, double* loop,
                   void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, 0, nt));
  if (!aligned(prop_diag) || !aligned(mom) || !aligned(loop)) return ctr::fail(CTR_ERR_ARG, "ctr_loop_unity: bad pointer");
  return ctr::loop_unity_fp64(nev, nt, prop_diag, mom, loop, (cudaStream_t)stream);
}

int ctr_sigmapi(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
                const double* prop_diag, const double* mom_p1, const double* mom_p2, const double* mom2_p1p2,
                double* hor_fish, double* triangle, void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, tf_begin, tf_end));
  if (!aligned(prop_diag) || !aligned(mom_p1) || !aligned(mom_p2) || (triangle && (!aligned(prop_rows) ||
      !aligned(mom2_p1p2) || !aligned(triangle))) || (hor_fish && !aligned(hor_fish)))
    return ctr::fail(CTR_ERR_ARG, "ctr_sigmapi: null or misaligned pointer");
  return ctr::sigmapi_chain(nev, nt, tf_begin, tf_end, prop_rows, prop_diag, mom_p1, mom_p2, mom2_p1p2, hor_fish,
                            triangle, (cudaStream_t)stream, engine, nullptr, nullptr);
}

}  // extern "C"
