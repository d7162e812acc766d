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
#include <map>
#include <tuple>
#include <utility>

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

// A stage of block grids: the split engine stacks each grid's slabs along M; the
// FP64 engine runs them as plain tasks.
int run_grids(const Ctx& c, const std::vector<GridTask>& g, int slot) {
  if (g.empty()) return CTR_OK;
  if (c.engine == CTR_ENGINE_SPLIT) return zgemm_split_grids(c.N, g, c.s);
  std::vector<ZTask> t;
  for (const GridTask& G : g)
    for (int sl = 0; sl < G.nslab; sl++)
      for (int j = 0; j < G.nb; j++) {
        ZTask z{};
        for (int q = 0; q < G.nterm; q++) {
          z.A[q] = G.A[(size_t)sl * G.nterm + q];
          z.B[q] = G.B[j][q];
          z.wre[q] = G.w[q];
        }
        z.nterm = G.nterm;
        z.flags = G.adag | (((G.bdag >> (4 * j)) & 0xF) << 4);
        z.C = G.C0[j] + (size_t)sl * c.N2;
        t.push_back(z);
      }
  return run_stage(c, t, slot);
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
// pstride: elementals of consecutive time slices are pstride blocks apart (1 for
// [Nt][N][N] arrays; nphi for one momentum of a [Nt][nphi][N][N] array).
int pipi_chain(int N, int Nt, int tf_begin, int tf_end, int iso, const double* prop_rows, const double* prop_diag,
              const double* p1, const double* p2, const double* p3, const double* p4, double* corr, cudaStream_t s,
              int engine, const std::vector<int>* plist, size_t pstride = 1) {
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
  CTR_TRY(per_t_chain(c, diag, P3, pstride * N2, P4, pstride * N2, tmp, L, &need_tf));
  CTR_TRY(per_t_chain(c, diag, P2, pstride * N2, P1, pstride * N2, tmp, Rsq, &need_ti));
  CTR_TRY(per_t_chain(c, diag, P1, pstride * N2, P2, pstride * N2, tmp, Rdt, &need_ti));

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
          st1.push_back(zt(tb, P1 + ti * pstride * N2, V1 + b * N2));  // V1 = T Phi1
          st1.push_back(zt(tb, P2 + ti * pstride * N2, V2 + b * N2));  // V2 = T Phi2
        }
        st1.push_back(zt(P3 + tf * pstride * N2, tb, U3 + b * N2));       // U3 = Phi3 tau_b
        st1.push_back(zt(P4 + tf * pstride * N2, tb, U4 + b * N2));       // U4 = Phi4 tau_b
        st1.push_back(zt(P1 + ti * pstride * N2, tb, W1 + b * N2, 1 << 4));  // W1 = Phi1 tau_b^dag
        st1.push_back(zt(P2 + ti * pstride * N2, tb, W2 + b * N2, 1 << 4));  // W2 = Phi2 tau_b^dag
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
          st3.push_back(zt(P3 + tf * pstride * N2, Pm + b * N2, F + b * N2));   // F = Phi3 P
          st3.push_back(zt(P4 + tf * pstride * N2, Qm + b * N2, Gm + b * N2));  // G = Phi4 Q
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
                                        (double*)out, ls, CTR_ENGINE_FP64, &pairs, pstride);
                    });
}

// ------------------------------------------------ pi pi over momentum sets
// One call for many momentum sets (P1..P4 chosen from one elemental array).
// The per-time-slice products Phi_a taud Phi_b are computed once per (a, b) the
// sets use.  Per batch of (t_sink, t_src) pairs, source time major, every
// product is planned once: those several sets share -- Phi(q) tau_b,
// Phi(q) tau_b^dag, tau_b Phi(q), tau Phi(q) tau^dag, Phi(q') tau Phi(q) tau^dag
// and the star / fish twin traces, which the sets (p, -p) and (-p, p) have in
// common -- are keyed by elemental index.  Each stage is a list of block grids
// (GridTask): products with the same right operand -- Phi(q) for every q
// against tau_b, every row block of X for all pairs of one t_src against R(t_src)
// -- form the slabs of one grid, which the split engine stacks along M.

namespace {

// Bump allocation of Nev x Nev product blocks inside one workspace buffer; with
// no buffer it only counts (a dry run that sizes the batches).
struct Arena {
  double2* base = nullptr;
  size_t used = 0, cap = 0, N2 = 0;
  double2* block() {
    const size_t o = used;
    used += N2;
    if (!base) return (double2*)(uintptr_t)(sizeof(double2) * (o + 1));  // stand-in address, same spacing
    return o + N2 <= cap ? base + o : nullptr;
  }
};

struct TaskKey {
  const double2* a[4];
  const double2* b[4];
  float wre[4], wim[4];
  int nterm, flags;
  bool operator<(const TaskKey& o) const { return std::memcmp(this, &o, sizeof(TaskKey)) < 0; }
};

// Stages of block products with hash-consing: an identical task (operands,
// weights, transposes) returns the block computed by its first occurrence.
struct Planner {
  Arena ar;
  std::vector<ZTask> st[4];
  std::map<TaskKey, double2*> memo;
  bool overflow = false;
  double2* task(int stage, const ZTask& z) {
    TaskKey k;
    std::memset(&k, 0, sizeof(k));
    for (int q = 0; q < z.nterm; q++) {
      k.a[q] = z.A[q];
      k.b[q] = z.B[q];
      k.wre[q] = z.wre[q];
      k.wim[q] = z.wim[q];
    }
    k.nterm = z.nterm;
    k.flags = z.flags;
    auto it = memo.find(k);
    if (it != memo.end()) return it->second;
    double2* c = ar.block();
    if (!c) {
      overflow = true;
      return nullptr;
    }
    ZTask t = z;
    t.C = c;
    st[stage].push_back(t);
    memo.emplace(k, c);
    return c;
  }
};

// Closing traces of a batch; add() returns the slot of the value.
struct TracePlan {
  std::vector<TraceTask> tt;
  int n = 0;
  bool keep = true;  // false: number the slots only (the traces run in another form)
  int add(const double2* x, const double2* y, float cre, float cim, int mode) {
    if (keep) tt.push_back(tr(x, y, nullptr, cre, cim, mode));
    return n++;
  }
};

// (set, pair) item of a pi pi batch: 112 trace slots in the layout of
// pipi_combine_kernel, combined into corr[ent * 5 ..].
__global__ void pipi_combine_sets_kernel(const double2* __restrict__ trv, const double* __restrict__ trabs,
                                         const int* __restrict__ slots, const int* __restrict__ ent, int nitem, int iso,
                                         double2* __restrict__ corr, double eps_over_tol, int* __restrict__ count,
                                         int* __restrict__ list) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitem) return;
  const int* sl = slots + (size_t)it * 112;
  double2 sum[7];
  double ab[7];
  for (int g = 0; g < 7; g++) {
    double re = 0, im = 0, a = 0;
    for (int k = 0; k < 16; k++) {
      const int j = sl[g * 16 + k];
      if (j < 0) continue;
      re += trv[j].x;
      im += trv[j].y;
      if (trabs) a += trabs[j];
    }
    sum[g] = make_double2(re, im);
    ab[g] = a;
  }
  const double2 star = cmul(sum[3], sum[4]);
  const double2 fish = cmul(sum[5], sum[6]);
  double2* o = corr + (size_t)ent[it] * 5;
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
    for (int k = 0; k < 5; k++)
      if (!(scale[k] * eps_over_tol <= mag(o[k])) || (scale[k] == 0.0 && mag(o[k]) > 0.0)) {
        list[atomicAdd(count, 1)] = ent[it] * 5 + k;
        break;
      }
  }
}

// Scratch budget of a set batch: 16 GB, or an eighth of the device's memory where less.
size_t sets_budget() {
  static size_t b = 0;
  if (!b && !capturing()) {
    size_t fr = 0, tot = 0;
    b = cudaMemGetInfo(&fr, &tot) == cudaSuccess ? std::min<size_t>((size_t)16 << 30, tot / 8) : ((size_t)6 << 30);
  }
  return b ? b : ((size_t)6 << 30);
}

}  // namespace

// Per time slice: M(a, b, t) = Phi_a(t) taud(t) Phi_b(t), 16 consecutive blocks at
// M[combo * Nt + t], for the (a, b) combos and the t flagged in need; Phi_a(t)
// taud(t)_blk is computed once for all combos with the same a.  phi [Nt][nphi][N][N].
int per_t_sets(const Ctx& c, const double2* diag, const double2* ph, int nphi,
               const std::vector<std::pair<int, int>>& combos, const std::vector<std::vector<char>>& need,
               std::vector<const double2*>& M) {
  const int Nt = c.Nt;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  auto P = [&](int q, int t) { return ph + ((size_t)t * nphi + q) * N2; };
  M.assign(combos.size() * Nt, nullptr);
  size_t nblk = 0;
  for (int pass = 0; pass < 2; pass++) {  // a dry run for the size, then the plan
    Planner pl;
    pl.ar.N2 = N2;
    if (pass == 1) {
      void* mem;
      CTR_TRY(workspace(WS_PHI).get(nblk * N2 * sizeof(double2), &mem));
      pl.ar.base = (double2*)mem;
      pl.ar.cap = nblk * N2;
    }
    std::vector<const double2*> tmp(combos.size() * Nt * 16, nullptr);
    for (size_t ci = 0; ci < combos.size(); ci++)
      for (int t = 0; t < Nt; t++)
        if (need[ci][t])
          for (int b = 0; b < 16; b++)
            tmp[(ci * Nt + t) * 16 + b] =
                pl.task(0, zt(P(combos[ci].first, t), diag + (size_t)t * blk16 + b * N2, nullptr));
    for (size_t ci = 0; ci < combos.size(); ci++)
      for (int t = 0; t < Nt; t++) {
        if (!need[ci][t]) continue;
        double2* first = nullptr;
        for (int b = 0; b < 16; b++) {
          double2* out = pl.task(1, zt(tmp[(ci * Nt + t) * 16 + b], P(combos[ci].second, t), nullptr));
          if (b == 0) first = out;
          if (!pl.overflow && out != first + b * N2)
            return fail(CTR_ERR_ARG, "per-time-slice products not consecutive");
        }
        M[ci * Nt + t] = first;
      }
    if (pl.overflow) return fail(CTR_ERR_ALLOC, "per-time-slice arena overflow");
    if (pass == 0) {
      nblk = pl.ar.used / N2;
      continue;
    }
    CTR_TRY(run_stage(c, pl.st[0], WS_TASKS));
    CTR_TRY(run_stage(c, pl.st[1], WS_TASKS2));
  }
  return CTR_OK;
}

int pipi_sets(int N, int Nt, int tf_begin, int tf_end, int iso, const double* prop_rows, const double* prop_diag,
              const double* phi_all, int nphi, int nset, const int32_t* sets, double* corr, cudaStream_t s,
              int engine) {
  Ctx c{N, Nt, (size_t)N * N, s, engine};
  if (engine == CTR_ENGINE_SPLIT) g_refined_last = 0;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  const double2 *tau = (const double2*)prop_rows, *diag = (const double2*)prop_diag,
                *ph = (const double2*)phi_all;
  const int rows = tf_end - tf_begin, npairs = rows * Nt;
  auto P = [&](int q, int t) { return ph + ((size_t)t * nphi + q) * N2; };
  for (int k = 0; k < 4 * nset; k++)
    if (sets[k] < 0 || sets[k] >= nphi) return fail(CTR_ERR_ARG, "ctr_pipi_sets: elemental index %d not in [0,%d)",
                                                    sets[k], nphi);
  // ---- per time slice: M(a, b, t) = Phi_a(t) taud(t) Phi_b(t) for the (a, b) the sets use:
  // L = (P3, P4) at the sink times, Rsq = (P2, P1) and Rdt = (P1, P2) at every source time
  std::map<std::pair<int, int>, int> combo;
  std::vector<std::pair<int, int>> combos;
  std::vector<std::vector<char>> need;
  auto use = [&](int a, int b, int t0, int t1) {
    auto it = combo.find({a, b});
    if (it == combo.end()) {
      it = combo.emplace(std::make_pair(a, b), (int)combos.size()).first;
      combos.push_back({a, b});
      need.emplace_back(Nt, 0);
    }
    for (int t = t0; t < t1; t++) need[it->second][t] = 1;
    return it->second;
  };
  std::vector<int> cL(nset), cSq(nset), cDt(nset);
  for (int k = 0; k < nset; k++) {
    const int* q = sets + 4 * k;
    cL[k] = use(q[2], q[3], tf_begin, tf_end);
    cSq[k] = use(q[1], q[0], 0, Nt);
    cDt[k] = use(q[0], q[1], 0, Nt);
  }
  std::vector<const double2*> M;
  CTR_TRY(per_t_sets(c, diag, ph, nphi, combos, need, M));
  // ---- pair batches, source time major: the pairs of one t_src share right
  // operands (Rsq, Rdt, Phi(t_src)), so their products stack along M.  Each stage
  // is a list of block grids whose outputs the plan places so that the slabs of
  // one right block are consecutive blocks.
  std::vector<int> order(npairs);
  for (int ti = 0, k = 0; ti < Nt; ti++)
    for (int tfl = 0; tfl < rows; tfl++) order[k++] = tfl * Nt + ti;
  auto index_of = [&](std::vector<int>& v, int n) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    std::vector<int> ix(n, -1);
    for (size_t a = 0; a < v.size(); a++) ix[v[a]] = (int)a;
    return ix;
  };
  // elementals on the sink side of U (P3, P4) and on the source side (P1, P2: W, V, Pm)
  std::vector<int> Qu, Qw;
  for (int k = 0; k < nset; k++) {
    Qu.push_back(sets[4 * k + 2]);
    Qu.push_back(sets[4 * k + 3]);
    Qw.push_back(sets[4 * k]);
    Qw.push_back(sets[4 * k + 1]);
  }
  const std::vector<int> iu = index_of(Qu, nphi), iw = index_of(Qw, nphi);
  const int nU = (int)Qu.size(), nW = (int)Qw.size();
  std::vector<int> CL(cL.begin(), cL.end());
  const std::vector<int> icl = index_of(CL, (int)combos.size());
  const int nCL = (int)CL.size();
  // Y families (left L combo, right combo): Ysq and Ydt of every set
  std::map<std::pair<int, int>, int> yfam;
  std::vector<std::pair<int, int>> YF;
  std::vector<int> ysq(nset), ydt(nset);
  auto fam = [&](int cl, int cr) {
    auto it = yfam.find({cl, cr});
    if (it == yfam.end()) {
      it = yfam.emplace(std::make_pair(cl, cr), (int)YF.size()).first;
      YF.push_back({cl, cr});
    }
    return it->second;
  };
  for (int k = 0; k < nset; k++) {
    ysq[k] = fam(cL[k], cSq[k]);
    ydt[k] = fam(cL[k], cDt[k]);
  }
  const int nYF = (int)YF.size();
  std::vector<std::vector<int>> yby;  // Y families grouped by their left combo
  {
    std::map<int, int> at;
    for (int f = 0; f < nYF; f++) {
      auto it = at.find(YF[f].first);
      if (it == at.end()) {
        it = at.emplace(YF[f].first, (int)yby.size()).first;
        yby.emplace_back();
      }
      yby[it->second].push_back(f);
    }
  }
  // F = Phi_qf(tf) Pm(qp): per Pm index, the elementals it is multiplied by
  std::vector<std::vector<int>> FK(nW);
  std::vector<int> fpos(nset * 2);
  if (iso == 0)
    for (int k = 0; k < nset; k++)
      for (int h = 0; h < 2; h++) {
        const int qf = sets[4 * k + 2 + h], qp = iw[sets[4 * k + h]];
        auto& v = FK[qp];
        auto it = std::find(v.begin(), v.end(), qf);
        if (it == v.end()) it = v.insert(v.end(), qf);
        fpos[2 * k + h] = (int)(it - v.begin());
      }
  int nF = 0;
  for (auto& v : FK) nF += (int)v.size();
  // star / fish twin traces Tr[U(qu) W(qw)]: (U4, W1), (U3, W2), (U3, W1), (U4, W2) of every set
  std::map<std::pair<int, int>, int> twk;
  std::vector<std::pair<int, int>> TW;
  std::vector<int> twin(4 * nset);
  for (int k = 0; k < nset; k++) {
    const int* q = sets + 4 * k;
    const std::pair<int, int> key[4] = {{q[3], q[0]}, {q[2], q[1]}, {q[2], q[0]}, {q[3], q[1]}};
    for (int h = 0; h < 4; h++) {
      auto it = twk.find(key[h]);
      if (it == twk.end()) {
        it = twk.emplace(key[h], (int)TW.size()).first;
        TW.push_back(key[h]);
      }
      twin[4 * k + h] = it->second;
    }
  }
  const int nTW = (int)TW.size();
  const size_t blk_pair = 16 * (size_t)(nU + nW + nCL + nYF + (iso == 0 ? 2 * nW + nF : 0));
  const size_t tr_pair = (size_t)nset * (iso == 0 ? 48 : 32) + 16 * (size_t)nTW;
  const size_t per_pair = blk_pair * N2 * sizeof(double2) + tr_pair * (sizeof(double2) + sizeof(double));
  const int batch = std::max(1, std::min(npairs, (int)(sets_budget() / std::max<size_t>(per_pair, 1))));
  Refine rf;
  CTR_TRY(refine_begin(c, (size_t)nset * npairs * 5, WS_REFINE, rf));
  const float g5w[4] = {(float)G5[0], (float)G5[1], (float)G5[2], (float)G5[3]};
  for (int p0 = 0; p0 < npairs; p0 += batch) {
    const int np = std::min(batch, npairs - p0);
    void* mem;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * per_pair, &mem));
    double2* base = (double2*)mem;
    size_t used = 0;
    auto alloc = [&](size_t nblk) {
      double2* p = base + used;
      used += nblk * N2;
      return p;
    };
    std::vector<int> tfv(np), tiv(np), gof(np), pos(np);
    std::vector<const double2*> Tv(np);
    std::vector<std::pair<int, int>> grp;  // (first pair, count) of each t_src run
    for (int i = 0; i < np; i++) {
      const int pair = order[p0 + i], tfl = pair / Nt;
      tfv[i] = tf_begin + tfl;
      tiv[i] = pair % Nt;
      Tv[i] = tau + ((size_t)tfl * Nt + tiv[i]) * blk16;
      if (i == 0 || tiv[i] != tiv[i - 1]) grp.push_back({i, 0});
      gof[i] = (int)grp.size() - 1;
      pos[i] = grp.back().second++;
    }
    const int ng = (int)grp.size();
    std::vector<double2*> bU(np), bW(np), bX(np), bP(np, nullptr), bV(ng, nullptr), bY((size_t)ng * nYF);
    std::vector<std::vector<double2*>> bF(np, std::vector<double2*>(nW, nullptr));
    for (int i = 0; i < np; i++) {
      bU[i] = alloc(16 * (size_t)nU);
      bW[i] = alloc(16 * (size_t)nW);
      bX[i] = alloc(16 * (size_t)nCL);
      if (iso == 0) {
        bP[i] = alloc(16 * (size_t)nW);
        for (int qp = 0; qp < nW; qp++)
          if (!FK[qp].empty()) bF[i][qp] = alloc(16 * FK[qp].size());
      }
    }
    for (int g = 0; g < ng; g++) {
      const size_t m = grp[g].second;
      if (iso == 0) bV[g] = alloc(16 * (size_t)nW * m);
      for (int f = 0; f < nYF; f++) bY[(size_t)g * nYF + f] = alloc(16 * m);
    }
    auto grid = [](int nslab, int nb, int nterm, const float* w, int adag, int bdag) {
      GridTask G;
      std::memset(G.B, 0, sizeof(G.B));
      std::memset(G.C0, 0, sizeof(G.C0));
      for (int q = 0; q < 4; q++) G.w[q] = q < nterm ? w[q] : 0.f;
      G.nslab = nslab;
      G.nb = nb;
      G.nterm = nterm;
      G.adag = adag;
      G.bdag = bdag;
      G.A.resize((size_t)nslab * nterm);
      return G;
    };
    const float one[4] = {1.f, 1.f, 1.f, 1.f};
    std::vector<GridTask> g0, g1, g2;
    for (int i = 0; i < np; i++) {
      const double2* T = Tv[i];
      for (int jb = 0; jb < 2; jb++) {
        // U(q)_b = Phi_q(tf) tau_b, W(q)_b = Phi_q(ti) tau_b^dag; slab q, right block b
        GridTask gu = grid(nU, 8, 1, one, 0, 0), gw = grid(nW, 8, 1, one, 0, 0x11111111);
        for (int sl = 0; sl < nU; sl++) gu.A[sl] = P(Qu[sl], tfv[i]);
        for (int sl = 0; sl < nW; sl++) gw.A[sl] = P(Qw[sl], tiv[i]);
        for (int j = 0; j < 8; j++) {
          const int b = 8 * jb + j;
          gu.B[j][0] = gw.B[j][0] = T + b * N2;
          gu.C0[j] = bU[i] + (size_t)b * nU * N2;
          gw.C0[j] = bW[i] + (size_t)b * nW * N2;
        }
        g0.push_back(std::move(gu));
        g0.push_back(std::move(gw));
      }
      // X = L G T: slab (L combo, row block a), right block b
      GridTask gx = grid(4 * nCL, 4, 4, g5w, 0, 0);
      for (int ci = 0; ci < nCL; ci++)
        for (int a = 0; a < 4; a++)
          for (int kk = 0; kk < 4; kk++)
            gx.A[(size_t)(ci * 4 + a) * 4 + kk] = M[(size_t)CL[ci] * Nt + tfv[i]] + (size_t)(a * 4 + kk) * N2;
      for (int j = 0; j < 4; j++) {
        for (int kk = 0; kk < 4; kk++) gx.B[j][kk] = T + (kk * 4 + j) * N2;
        gx.C0[j] = bX[i] + (size_t)j * 4 * nCL * N2;
      }
      g0.push_back(std::move(gx));
    }
    auto Xblk = [&](int cl, int i, int a, int b) { return bX[i] + ((size_t)b * 4 * nCL + icl[cl] * 4 + a) * N2; };
    auto Vblk = [&](int qi, int i, int a, int b) {
      return bV[gof[i]] + ((size_t)qi * 16 * grp[gof[i]].second + pos[i] * 16 + a * 4 + b) * N2;
    };
    auto Yblk = [&](int f, int i, int a, int c2) {
      return bY[(size_t)gof[i] * nYF + f] + ((size_t)c2 * 4 * grp[gof[i]].second + pos[i] * 4 + a) * N2;
    };
    auto Pblk = [&](int qi, int i, int a, int c2) { return bP[i] + ((size_t)c2 * 4 * nW + qi * 4 + a) * N2; };
    for (int g = 0; g < ng; g++) {
      const int i0 = grp[g].first, m = grp[g].second, ti = tiv[i0];
      if (iso == 0)  // V(q) = tau_b Phi_q(ti): slab (pair, block b), right block q
        for (int q0 = 0; q0 < nW; q0 += 8) {
          GridTask gv = grid(16 * m, std::min(8, nW - q0), 1, one, 0, 0);
          for (int pp = 0; pp < m; pp++)
            for (int b = 0; b < 16; b++) gv.A[pp * 16 + b] = Tv[i0 + pp] + b * N2;
          for (int j = 0; j < gv.nb; j++) {
            gv.B[j][0] = P(Qw[q0 + j], ti);
            gv.C0[j] = bV[g] + (size_t)(q0 + j) * 16 * m * N2;
          }
          g0.push_back(std::move(gv));
        }
      // Ysq / Ydt = X G R: slab (pair, row block a), right block b of R(t_src).  The
      // families with the same left X (a set's Ysq and Ydt) share one grid of up to
      // 8 right blocks, so that X's rows are sliced once for both.
      for (size_t h = 0; h < yby.size(); h++) {
        const std::vector<int>& fl = yby[h];
        for (size_t f0 = 0; f0 < fl.size(); f0 += 2) {
          const int nf = (int)std::min<size_t>(2, fl.size() - f0);
          GridTask gy = grid(4 * m, 4 * nf, 4, g5w, 0, 0);
          const int cl = YF[fl[f0]].first;
          for (int pp = 0; pp < m; pp++)
            for (int a = 0; a < 4; a++)
              for (int kk = 0; kk < 4; kk++) gy.A[(size_t)(pp * 4 + a) * 4 + kk] = Xblk(cl, i0 + pp, a, kk);
          for (int u = 0; u < nf; u++) {
            const int f = fl[f0 + u];
            for (int j = 0; j < 4; j++) {
              for (int kk = 0; kk < 4; kk++)
                gy.B[u * 4 + j][kk] = M[(size_t)YF[f].second * Nt + ti] + (size_t)(kk * 4 + j) * N2;
              gy.C0[u * 4 + j] = bY[(size_t)g * nYF + f] + (size_t)j * 4 * m * N2;
            }
          }
          g1.push_back(std::move(gy));
        }
      }
    }
    if (iso == 0)
      for (int i = 0; i < np; i++) {
        // Pm(q) = V(q) T^dag: block (a, c) = sum_k V_ak tau_ck^dag; slab (q, a), right block c
        GridTask gp = grid(4 * nW, 4, 4, one, 0, 0xFFFF);
        for (int qi = 0; qi < nW; qi++)
          for (int a = 0; a < 4; a++)
            for (int kk = 0; kk < 4; kk++) gp.A[(size_t)(qi * 4 + a) * 4 + kk] = Vblk(qi, i, a, kk);
        for (int j = 0; j < 4; j++) {
          for (int kk = 0; kk < 4; kk++) gp.B[j][kk] = Tv[i] + (j * 4 + kk) * N2;
          gp.C0[j] = bP[i] + (size_t)j * 4 * nW * N2;
        }
        g1.push_back(std::move(gp));
        // F(qf, qp)_b = Phi_qf(tf) Pm(qp)_b: slab qf, right block b
        for (int qp = 0; qp < nW; qp++) {
          const int nf = (int)FK[qp].size();
          if (!nf) continue;
          for (int jb = 0; jb < 2; jb++) {
            GridTask gf = grid(nf, 8, 1, one, 0, 0);
            for (int sl = 0; sl < nf; sl++) gf.A[sl] = P(FK[qp][sl], tfv[i]);
            for (int j = 0; j < 8; j++) {
              const int b = 8 * jb + j;
              gf.B[j][0] = Pblk(qp, i, b / 4, b % 4);
              gf.C0[j] = bF[i][qp] + (size_t)b * nf * N2;
            }
            g2.push_back(std::move(gf));
          }
        }
      }
    // traces: values (and error scales) after the products in the same buffer
    const size_t ntr = (size_t)np * tr_pair;
    double2* trv = base + used;
    double* tra = rf.on ? (double*)(trv + ntr) : nullptr;
    if ((used * sizeof(double2) + ntr * (sizeof(double2) + sizeof(double))) > (size_t)np * per_pair)
      return fail(CTR_ERR_ALLOC, "ctr_pipi_sets: batch arena overflow");
    TracePlan tp;
    std::vector<int> slots, ent, tws(16 * (size_t)nTW);
    for (int i = 0; i < np; i++) {
      const double2* T = Tv[i];
      for (int t = 0; t < nTW; t++)
        for (int b = 0; b < 16; b++)
          tws[t * 16 + b] = tp.add(bU[i] + ((size_t)b * nU + iu[TW[t].first]) * N2,
                                   bW[i] + ((size_t)b * nW + iw[TW[t].second]) * N2, 1.f, 0.f, 1);
      for (int k = 0; k < nset; k++) {
        const int* q = sets + 4 * k;
        for (int b = 0; b < 16; b++) slots.push_back(tp.add(Yblk(ysq[k], i, b / 4, b % 4), T + b * N2, 1.f, 0.f, 0));
        for (int b = 0; b < 16; b++) slots.push_back(tp.add(Yblk(ydt[k], i, b / 4, b % 4), T + b * N2, 1.f, 0.f, 0));
        for (int b = 0; b < 16; b++) {
          if (iso != 0) {
            slots.push_back(-1);
            continue;
          }
          // Tr[F_{s1 s3} G_{s3 s1}], F = Phi3 Pm(P1), G = Phi4 Pm(P2)
          const int s1 = b / 4, s3 = b % 4, qf1 = iw[q[0]], qf2 = iw[q[1]];
          const double2* Fb = bF[i][qf1] + ((size_t)b * FK[qf1].size() + fpos[2 * k]) * N2;
          const double2* Gb = bF[i][qf2] + ((size_t)(s3 * 4 + s1) * FK[qf2].size() + fpos[2 * k + 1]) * N2;
          slots.push_back(tp.add(Fb, Gb, 1.f, 0.f, 1));
        }
        for (int h = 0; h < 4; h++)
          for (int b = 0; b < 16; b++) slots.push_back(tws[twin[4 * k + h] * 16 + b]);
        ent.push_back(k * npairs + order[p0 + i]);
      }
    }
    for (size_t k = 0; k < tp.tt.size(); k++) {
      tp.tt[k].out = trv + k;
      if (tra) tp.tt[k].absout = tra + k;
    }
    CTR_TRY(run_grids(c, g0, WS_TASKS));
    CTR_TRY(run_grids(c, g1, WS_TASKS2));
    CTR_TRY(run_grids(c, g2, WS_GEMM_A));
    CTR_TRY(run_traces(c, tp.tt));
    void* d[2];
    CTR_TRY(upload_group(WS_MISC, {{slots.data(), slots.size() * sizeof(int)}, {ent.data(), ent.size() * sizeof(int)}},
                         d, s));
    {
      TimedLaunch tl(s, "pipi_combine");
      const int nitem = (int)ent.size();
      pipi_combine_sets_kernel<<<(nitem + 127) / 128, 128, 0, s>>>(trv, tra, (const int*)d[0], (const int*)d[1], nitem,
                                                                   iso, (double2*)corr, rf.eps_over_tol, rf.count,
                                                                   rf.list);
      CTR_CUDA(cudaGetLastError());
    }
  }
  std::vector<int32_t> set_copy(sets, sets + 4 * nset);
  return refine_end(c, rf, 5, WS_REFINE, (double2*)corr,
                    [=](const std::vector<int>& units, double2* out, cudaStream_t ls) -> int {
                      // units = set * npairs + pair, ascending: one FP64 rerun per set
                      size_t u0 = 0;
                      while (u0 < units.size()) {
                        const int k = units[u0] / npairs;
                        size_t u1 = u0;
                        std::vector<int> pl;
                        while (u1 < units.size() && units[u1] / npairs == k) pl.push_back(units[u1++] % npairs);
                        const int* q = set_copy.data() + 4 * k;
                        auto Pq = [&](int qq) { return (const double*)(ph + (size_t)qq * N2); };
                        CTR_TRY(pipi_chain(N, Nt, tf_begin, tf_end, iso, prop_rows, prop_diag, Pq(q[0]), Pq(q[1]),
                                           Pq(q[2]), Pq(q[3]), (double*)(out + u0 * 5), ls, CTR_ENGINE_FP64, &pl,
                                           (size_t)nphi));
                        u0 = u1;
                      }
                      return CTR_OK;
                    });
}

// ---------------------------------------------------------------- rho pipi
// Row form (lib/calculate_rhopi_core.h): coef * Tr[Phi^{P1P2}_ip(tf) tau_{s5s6}
// Phi_P2(ti) taud(ti)_{s1s2} Phi_P1(ti) tau_{s3s2}^dag] with s6 = s1, s4 = s3;
// coef = c(iop, s3, s5) * g5(s1), so the sum over s1 is (T G R)_{s5 s2}.
int rhopi_chain(int N, int Nt, int tf_begin, int tf_end, int idir, const double* prop_rows, const double* prop_diag,
                const double* mp1, const double* mp2, const double* mom5, double* corr, cudaStream_t s, int engine,
                const std::vector<int>* plist, size_t pstride = 1) {
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
  CTR_TRY(per_t_chain(c, diag, P2, pstride * N2, P1, pstride * N2, tmp, R, &need_ti));  // R = Phi_P2 taud Phi_P1

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
  // The trace of a row, Tr-Had(Phi_ip(tf) X_{s5 s2}, tau_{s3 s2}), is taken as
  // Tr-Had(X_{s5 s2}, Z) with Z = Phi_ip(tf)^dag tau_{s3 s2}: the same sum, but Z does not
  // depend on the pion pair (P1, P2), so a batch of pairs shares it, and it does not
  // wait for X.  Distinct Z products (ip, s3, s2):
  std::vector<int> zkeys;  // ip*16 + s3*4 + s2
  for (auto& g : grp) {
    int k = g.ip * 16 + g.s3 * 4 + g.s2;
    if (std::find(zkeys.begin(), zkeys.end(), k) == zkeys.end()) zkeys.push_back(k);
  }
  const int nprod = (int)zkeys.size(), ngrp = (int)grp.size();
  const size_t per_pair = (size_t)(16 + nprod) * N2 * sizeof(double2) + ngrp * sizeof(double2);
  const int batch = batch_pairs(per_pair, npairs);
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
    std::vector<ZTask> st1;
    std::vector<TraceTask> tt;
    for (int q = 0; q < np; q++) {
      const int pr = pair_of(p0 + q), tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* T = tau + ((size_t)tfl * Nt + ti) * blk16;
      double2* X = Bm + (size_t)q * (16 + nprod) * N2;
      double2* Z = X + blk16;
      block_gemm_g5(c, T, R + ti * blk16, X, st1);  // X = T G R
      for (int k = 0; k < nprod; k++) {
        const int ip = zkeys[k] / 16, s3 = (zkeys[k] / 4) % 4, s2 = zkeys[k] % 4;
        st1.push_back(zt(P12 + ((size_t)tf * 5 + ip) * N2, T + (s3 * 4 + s2) * N2, Z + k * N2, 1));  // Phi^dag tau
      }
      for (int g = 0; g < ngrp; g++) {
        const int k = (int)(std::find(zkeys.begin(), zkeys.end(), grp[g].ip * 16 + grp[g].s3 * 4 + grp[g].s2) -
                            zkeys.begin());
        tt.push_back(tr(X + (grp[g].s5 * 4 + grp[g].s2) * N2, Z + k * N2, TR + (size_t)q * ngrp + g, grp[g].cre,
                        grp[g].cim, 0));
      }
    }
    if (TRA)
      for (size_t k = 0; k < tt.size(); k++) tt[k].absout = TRA + (tt[k].out - TR);
    CTR_TRY(run_stage(c, st1, WS_TASKS));
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
                                         (double*)out, ls, CTR_ENGINE_FP64, &pairs, pstride);
                    });
}

// -------------------------------------------------------------- sigma pipi
// Horizontal fish (lib/calculate_sigmapi_hor_fish_core.h): per t,
// sum_ab coef * sum R_ab (.) conj taud_ab with R = Phi_P2 taud Phi_P1.
// Triangle (lib/calculate_sigmapi_triangle_core.h): rows with s2 = s1, s4 = s3,
// coef = g5(s1) g5(s3): sum_s3 g5(s3) tau_{s1s3} R_{s3s5} = (T G R)_{s1 s5}.
int sigmapi_chain(int N, int Nt, int tf_begin, int tf_end, const double* prop_rows, const double* prop_diag,
                  const double* mp1, const double* mp2, const double* mom2, double* hor_fish, double* tri,
                  cudaStream_t s, int engine, const std::vector<int>* plist, const std::vector<int>* tlist,
                  size_t pstride = 1) {
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
  CTR_TRY(per_t_chain(c, diag, P2, pstride * N2, P1, pstride * N2, tmp, R, &need));
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
                                              (double*)out, nullptr, ls, CTR_ENGINE_FP64, nullptr, &ts, pstride);
                       }));
  }
  if (!tri) return CTR_OK;
  // triangle (lib/calculate_sigmapi_triangle_core.h): X = T G R and the trace
  // Tr-Had(Phix2_ik(tf) X_{s1 s5}, tau_{s1 s5}) with weight g5(s1), taken as
  // Tr-Had(X_{s1 s5}, Z_{ik, s1 s5}) with Z = Phix2_ik(tf)^dag tau_{s1 s5}, which does not
  // depend on the pion pair and does not wait for X.
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
    std::vector<ZTask> st1;
    std::vector<TraceTask> tt;
    for (int q = 0; q < np; q++) {
      const int pr = pair_of(p0 + q), tfl = pr / Nt, ti = pr % Nt, tf = tf_begin + tfl;
      const double2* T = tau + ((size_t)tfl * Nt + ti) * blk16;
      double2* X = Bm + (size_t)q * 48 * N2;
      double2* Z = X + blk16;
      block_gemm_g5(c, T, R + ti * blk16, X, st1);
      for (int ik = 0; ik < 2; ik++)
        for (int b = 0; b < 16; b++) {
          st1.push_back(zt(Px2 + ((size_t)tf * 2 + ik) * N2, T + b * N2, Z + (ik * 16 + b) * N2, 1));
          tt.push_back(tr(X + b * N2, Z + (ik * 16 + b) * N2, TR + (size_t)q * 32 + ik * 16 + b,
                          (float)G5[b / 4], 0.f, 0));
          if (TRA) tt.back().absout = TRA + (size_t)q * 32 + ik * 16 + b;
        }
    }
    CTR_TRY(run_stage(c, st1, WS_TASKS));
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
                                           (double*)out, ls, CTR_ENGINE_FP64, &pairs, nullptr, pstride);
                    });
}

// --------------------------------------- rho -> pi pi and sigma -> pi pi over sets
// Both families contract X = T G R, R(t) = Phi_P2(t) taud(t) Phi_P1(t), with the
// sink operators: rho -> pi pi (lib/calculate_rhopi_core.h) takes Phi^{P1P2}_ip(tf)
// X_{s5 s2} for ip in {0, 1, 2 + idir}, the sigma -> pi pi triangle
// (lib/calculate_sigmapi_triangle_core.h) Phi^{x2}_ik(tf) X_b for ik in {0, 1}.
// Per set and pair, X is computed once and multiplied by all the sink operators
// the requested outputs need in one grid (slab = operator, right block = X
// block); the horizontal fish (lib/calculate_sigmapi_hor_fish_core.h) traces R
// against taud per time slice.

namespace {

// Row sums of batch items whose rows' trace values sit anywhere: row r of item it
// is trace slot rowslot[it * nrows + r], times rcoef[r] where given; output o sums
// rows idx[off[o] .. off[o+1]) in that order into out[ent[it] * nout + o]; with
// trabs, entries whose error estimate exceeds the tolerance append ent * nout + o
// to the refinement list.
__global__ void rowsum_items_kernel(const double2* __restrict__ trv, const double* __restrict__ trabs,
                                    const int* __restrict__ rowslot, int nrows, const int* __restrict__ off,
                                    const int* __restrict__ idx, const float2* __restrict__ rcoef, int nout,
                                    const int* __restrict__ ent, int nitem, double2* __restrict__ out,
                                    double eps_over_tol, int* __restrict__ count, int* __restrict__ list) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nitem * nout) return;
  const int it = g / nout, o = g % nout;
  double re = 0.0, im = 0.0, sc = 0.0;
  for (int k = off[o]; k < off[o + 1]; k++) {
    const int r = idx[k], j = rowslot[(size_t)it * nrows + r];
    double2 v = trv[j];
    double a = trabs ? trabs[j] : 0.0;
    if (rcoef) {  // the row's coefficient, applied as the trace kernel applies it
      const double2 c = make_double2((double)rcoef[r].x, (double)rcoef[r].y);
      v = cmul(c, v);
      a = sqrt(c.x * c.x + c.y * c.y) * a;
    }
    re += v.x;
    im += v.y;
    sc += a;
  }
  const size_t e = (size_t)ent[it] * nout + o;
  out[e] = make_double2(re, im);
  const double mag = sqrt(re * re + im * im);
  if (trabs && eps_over_tol > 0.0 && (!(sc * eps_over_tol <= mag) || (sc == 0.0 && mag > 0.0)))
    list[atomicAdd(count, 1)] = (int)e;
}

// Item tables of one row-sum launch (host), and their device copies.
struct RowItems {
  std::vector<int> slot, csr, ent;
  std::vector<float2> coef;  // per row, or empty
  int nrows = 0, nout = 0;
  const int *d_slot = nullptr, *d_csr = nullptr, *d_ent = nullptr;
  const float2* d_coef = nullptr;
};

// Uploads the tables of several row-sum launches in one staging copy.
int upload_items(const Ctx& c, std::vector<RowItems*> items) {
  std::vector<std::pair<const void*, size_t>> parts;
  for (RowItems* r : items) {
    parts.push_back({r->slot.data(), r->slot.size() * sizeof(int)});
    parts.push_back({r->csr.data(), r->csr.size() * sizeof(int)});
    parts.push_back({r->ent.data(), r->ent.size() * sizeof(int)});
    parts.push_back({r->coef.data(), r->coef.size() * sizeof(float2)});
  }
  std::vector<void*> d(parts.size());
  CTR_TRY(upload_group(WS_MISC, parts, d.data(), c.s));
  for (size_t i = 0; i < items.size(); i++) {
    items[i]->d_slot = (const int*)d[4 * i];
    items[i]->d_csr = (const int*)d[4 * i + 1];
    items[i]->d_ent = (const int*)d[4 * i + 2];
    items[i]->d_coef = items[i]->coef.empty() ? nullptr : (const float2*)d[4 * i + 3];
  }
  return CTR_OK;
}

int rowsum_items(const Ctx& c, const double2* trv, const double* tra, const RowItems& r, double2* out,
                 const Refine& rf) {
  if (r.ent.empty()) return CTR_OK;
  TimedLaunch tl(c.s, "rowsum_items");
  const int n = (int)r.ent.size() * r.nout;
  rowsum_items_kernel<<<(n + 127) / 128, 128, 0, c.s>>>(trv, rf.on ? tra : nullptr, r.d_slot, r.nrows, r.d_csr,
                                                        r.d_csr + r.nout + 1, r.d_coef, r.nout, r.d_ent,
                                                        (int)r.ent.size(), out, rf.eps_over_tol, rf.count, rf.list);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

}  // namespace

int rhopi_sigmapi_sets(int N, int Nt, int tf_begin, int tf_end, const double* prop_rows, const double* prop_diag,
                       const double* phi_all, int nphi, const double* mom5, const double* mom2, int nset,
                       const int32_t* sets, double* rhopi, double* tri, double* hor_fish, cudaStream_t s,
                       int engine) {
  Ctx c{N, Nt, (size_t)N * N, s, engine};
  if (engine == CTR_ENGINE_SPLIT) g_refined_last = 0;
  const size_t N2 = c.N2, blk16 = 16 * N2;
  const double2 *tau = (const double2*)prop_rows, *diag = (const double2*)prop_diag,
                *ph = (const double2*)phi_all, *P5 = (const double2*)mom5, *P2x = (const double2*)mom2;
  const int rows = tf_end - tf_begin, npairs = rows * Nt;
  const Tables& Tb = tables();
  for (int k = 0; k < 2 * nset; k++)
    if (sets[k] < 0 || sets[k] >= nphi)
      return fail(CTR_ERR_ARG, "ctr_rhopi_sigmapi_sets: elemental index %d not in [0,%d)", sets[k], nphi);
  // R(t) = Phi_P2 taud Phi_P1 for every set's (P2, P1), at every time slice
  std::map<std::pair<int, int>, int> combo;
  std::vector<std::pair<int, int>> combos;
  std::vector<int> cR(nset);
  for (int k = 0; k < nset; k++) {
    auto key = std::make_pair(sets[2 * k + 1], sets[2 * k]);
    auto it = combo.find(key);
    if (it == combo.end()) {
      it = combo.emplace(key, (int)combos.size()).first;
      combos.push_back(key);
    }
    cR[k] = it->second;
  }
  const int nC = (int)combos.size();
  std::vector<std::vector<char>> need(nC, std::vector<char>(Nt, 1));
  std::vector<const double2*> M;
  CTR_TRY(per_t_sets(c, diag, ph, nphi, combos, need, M));

  // ---- horizontal fish: per set and time slice, sum_ab coef * Tr-Had(R_ab, taud_ab)
  if (hor_fish) {
    Refine rf;
    CTR_TRY(refine_begin(c, (size_t)nset * Nt, WS_REFINE, rf));
    const size_t ntr = (size_t)nset * Nt * 16;
    void *trm, *tra = nullptr;
    CTR_TRY(workspace(WS_ROWS).get(ntr * sizeof(double2), &trm));
    if (rf.on) CTR_TRY(workspace(WS_ROWABS).get(ntr * sizeof(double), &tra));
    std::vector<TraceTask> tt;
    RowItems ri;
    ri.nrows = 16;
    ri.nout = 1;
    for (int k = 0; k < nset; k++)
      for (int t = 0; t < Nt; t++) {
        for (int b = 0; b < 16; b++) {
          const int ab = Tb.hf_spin[b][0] * 4 + Tb.hf_spin[b][1];
          tt.push_back(tr(M[(size_t)cR[k] * Nt + t] + ab * N2, diag + t * blk16 + ab * N2,
                          (double2*)trm + tt.size(), Tb.hf_coef[b][0], Tb.hf_coef[b][1], 0));
          if (tra) tt.back().absout = (double*)tra + (tt.size() - 1);
          ri.slot.push_back((int)tt.size() - 1);
        }
        ri.ent.push_back(k * Nt + t);
      }
    ri.csr = {0, 16};
    for (int b = 0; b < 16; b++) ri.csr.push_back(b);
    CTR_TRY(run_traces(c, tt));
    CTR_TRY(upload_items(c, {&ri}));
    CTR_TRY(rowsum_items(c, (double2*)trm, (double*)tra, ri, (double2*)hor_fish, rf));
    std::vector<int32_t> sc(sets, sets + 2 * nset);
    CTR_TRY(refine_end(c, rf, 1, WS_REFINE, (double2*)hor_fish,
                       [=](const std::vector<int>& units, double2* out, cudaStream_t ls) -> int {
                         size_t u0 = 0;
                         while (u0 < units.size()) {  // units = set * Nt + t: one FP64 rerun per set
                           const int k = units[u0] / Nt;
                           std::vector<int> tl;
                           size_t u1 = u0;
                           while (u1 < units.size() && units[u1] / Nt == k) tl.push_back(units[u1++] % Nt);
                           CTR_TRY(sigmapi_chain(N, Nt, tf_begin, tf_end, prop_rows, prop_diag,
                                                 (const double*)(ph + (size_t)sc[2 * k] * N2),
                                                 (const double*)(ph + (size_t)sc[2 * k + 1] * N2), mom2,
                                                 (double*)(out + u0), nullptr, ls, CTR_ENGINE_FP64, nullptr, &tl,
                                                 (size_t)nphi));
                           u0 = u1;
                         }
                         return CTR_OK;
                       }));
  }
  if (!rhopi && !tri) return CTR_OK;

  // ---- sink operators of the grid: the rho operators the three polarisations use, then sigma's two
  struct Grp {
    int iop, s2, s3, s5, slab;
    float cre, cim;
  };
  std::vector<int> ops;  // slab -> operator: 0..4 rho (mom5), 5..6 sigma (mom2)
  std::vector<int> slab_of(7, -1);
  std::vector<Grp> grp[3];
  std::vector<int> csr_rp[3];
  if (rhopi)
    for (int idir = 0; idir < 3; idir++) {
      for (int bx = 0; bx < 256; bx++) {
        const int r = idir * 256 + bx;
        const int16_t* sp = Tb.rhopi_spin[r];
        const int s1 = sp[0];
        if (sp[5] != s1 || sp[3] != sp[2])
          return fail(CTR_ERR_ARG, "rho-pipi table row %d not gamma_5-diagonal", r);
        if (s1 != 0) continue;  // one representative per group (coef x g5(s1) sums over s1)
        const int ip = Tb.rhopi_ip[r];
        if (slab_of[ip] < 0) {
          slab_of[ip] = (int)ops.size();
          ops.push_back(ip);
        }
        grp[idir].push_back(Grp{bx / 64, sp[1], sp[2], sp[4], slab_of[ip], Tb.rhopi_coef[r][0] * G5[s1],
                                Tb.rhopi_coef[r][1] * G5[s1]});
      }
      // CSR of the 4 operators over the groups, in group order (as rhopi_chain)
      std::vector<int> off(5, 0), idx(grp[idir].size());
      for (auto& g : grp[idir]) off[g.iop + 1]++;
      for (int o = 0; o < 4; o++) off[o + 1] += off[o];
      std::vector<int> fill(off.begin(), off.end() - 1);
      for (size_t g = 0; g < grp[idir].size(); g++) idx[fill[grp[idir][g].iop]++] = (int)g;
      csr_rp[idir] = off;
      csr_rp[idir].insert(csr_rp[idir].end(), idx.begin(), idx.end());
    }
  if (tri)
    for (int ik = 0; ik < 2; ik++) {
      slab_of[5 + ik] = (int)ops.size();
      ops.push_back(5 + ik);
    }
  const int nops = (int)ops.size();
  // the distinct traces (slab, X block, Z block) of the three polarisations' groups
  std::vector<std::tuple<int, int, int>> uniq;
  std::vector<int> uidx[3];
  if (rhopi) {
    std::map<std::tuple<int, int, int>, int> at;
    for (int idir = 0; idir < 3; idir++)
      for (const Grp& g : grp[idir]) {
        const auto key = std::make_tuple(g.slab, g.s5 * 4 + g.s2, g.s3 * 4 + g.s2);
        auto it = at.find(key);
        if (it == at.end()) {
          it = at.emplace(key, (int)uniq.size()).first;
          uniq.push_back(key);
        }
        uidx[idir].push_back(it->second);
      }
  }
  std::vector<int> csr_tr = {0, 16, 32};
  for (int k = 0; k < 32; k++) csr_tr.push_back(k);

  std::vector<int> order(npairs);
  for (int ti = 0, k = 0; ti < Nt; ti++)
    for (int tfl = 0; tfl < rows; tfl++) order[k++] = tfl * Nt + ti;
  const int ngr = rhopi ? (int)grp[0].size() : 0;
  const size_t blk_pair = 16 * ((size_t)nC + nops);
  const size_t tr_pair = (size_t)nset * (uniq.size() + (tri ? 32 : 0));
  const size_t per_pair = blk_pair * N2 * sizeof(double2) + tr_pair * (sizeof(double2) + sizeof(double));
  const int batch = std::max(1, std::min(npairs, (int)(sets_budget() / std::max<size_t>(per_pair, 1))));
  // closing-trace form on the split engine (chains.trace_form): when it is known
  // to be the Gram products, the FP64 trace tasks are not built
  const std::string trace_shape =
      "nev=" + std::to_string(N) + ",m=" + std::to_string(4 * nC) + ",n=" + std::to_string(4 * nops);
  int known_form = 0;
  const bool fp64_traces_needed = c.engine != CTR_ENGINE_SPLIT ||
                                  !tune_peek("chains.trace_form", trace_shape, 2, 1, &known_form) || known_form == 0;
  Refine rf_rp, rf_tr;
  if (rhopi) CTR_TRY(refine_begin(c, (size_t)nset * 3 * npairs * 4, WS_REFINE, rf_rp));
  if (tri) CTR_TRY(refine_begin(c, (size_t)nset * npairs * 2, WS_SPLITJOBS3, rf_tr));
  const float g5w[4] = {(float)G5[0], (float)G5[1], (float)G5[2], (float)G5[3]};
  const float one[4] = {1.f, 1.f, 1.f, 1.f};
  for (int p0 = 0; p0 < npairs; p0 += batch) {
    const int np = std::min(batch, npairs - p0);
    void* mem;
    CTR_TRY(workspace(WS_SCRATCH).get((size_t)np * per_pair, &mem));
    double2* base = (double2*)mem;
    size_t used = 0;
    auto alloc = [&](size_t nblk) {
      double2* p = base + used;
      used += nblk * N2;
      return p;
    };
    std::vector<int> tfv(np), tiv(np), gof(np), pos(np);
    std::vector<const double2*> Tv(np);
    std::vector<std::pair<int, int>> gr;
    for (int i = 0; i < np; i++) {
      const int pair = order[p0 + i], tfl = pair / Nt;
      tfv[i] = tf_begin + tfl;
      tiv[i] = pair % Nt;
      Tv[i] = tau + ((size_t)tfl * Nt + tiv[i]) * blk16;
      if (i == 0 || tiv[i] != tiv[i - 1]) gr.push_back({i, 0});
      gof[i] = (int)gr.size() - 1;
      pos[i] = gr.back().second++;
    }
    const int ng = (int)gr.size();
    std::vector<double2*> bX((size_t)ng * nC), bZ(np);
    for (int g = 0; g < ng; g++)
      for (int ci = 0; ci < nC; ci++) bX[(size_t)g * nC + ci] = alloc(16 * (size_t)gr[g].second);
    for (int i = 0; i < np; i++) bZ[i] = alloc(16 * (size_t)nops);
    // X(ci, i)_{a b} and Z(op slab, i)_b = Op(tf)^dag tau_b (shared by all sets)
    auto Xblk = [&](int ci, int i, int a, int b) {
      return bX[(size_t)gof[i] * nC + ci] + ((size_t)b * 4 * gr[gof[i]].second + pos[i] * 4 + a) * N2;
    };
    auto Zblk = [&](int sl, int i, int b) { return bZ[i] + ((size_t)b * nops + sl) * N2; };
    std::vector<GridTask> g0;
    for (int g = 0; g < ng; g++) {
      const int i0 = gr[g].first, m = gr[g].second, ti = tiv[i0];
      for (int ci = 0; ci < nC; ci++) {
        // X = T G R: slab (pair, row block a), right block b of R(t_src)
        GridTask gx;
        std::memset(gx.B, 0, sizeof(gx.B));
        std::memset(gx.C0, 0, sizeof(gx.C0));
        std::copy(g5w, g5w + 4, gx.w);
        gx.nslab = 4 * m;
        gx.nb = 4;
        gx.nterm = 4;
        gx.adag = gx.bdag = 0;
        gx.A.resize((size_t)16 * m);
        for (int pp = 0; pp < m; pp++)
          for (int a = 0; a < 4; a++)
            for (int kk = 0; kk < 4; kk++) gx.A[(size_t)(pp * 4 + a) * 4 + kk] = Tv[i0 + pp] + (a * 4 + kk) * N2;
        for (int j = 0; j < 4; j++) {
          for (int kk = 0; kk < 4; kk++) gx.B[j][kk] = M[(size_t)ci * Nt + ti] + (size_t)(kk * 4 + j) * N2;
          gx.C0[j] = bX[(size_t)g * nC + ci] + (size_t)j * 4 * m * N2;
        }
        g0.push_back(std::move(gx));
      }
    }
    for (int i = 0; i < np; i++)
      for (int jb = 0; jb < 2; jb++) {
        // Z = Op(tf)^dag tau_b: slab = sink operator, right block b of tau
        GridTask gz;
        std::memset(gz.B, 0, sizeof(gz.B));
        std::memset(gz.C0, 0, sizeof(gz.C0));
        std::copy(one, one + 4, gz.w);
        gz.nslab = nops;
        gz.nb = 8;
        gz.nterm = 1;
        gz.adag = 1;
        gz.bdag = 0;
        gz.A.resize(nops);
        for (int sl = 0; sl < nops; sl++)
          gz.A[sl] = ops[sl] < 5 ? P5 + ((size_t)tfv[i] * 5 + ops[sl]) * N2 : P2x + ((size_t)tfv[i] * 2 + ops[sl] - 5) * N2;
        for (int j = 0; j < 8; j++) {
          const int b = 8 * jb + j;
          gz.B[j][0] = Tv[i] + (size_t)b * N2;
          gz.C0[j] = bZ[i] + (size_t)b * nops * N2;
        }
        g0.push_back(std::move(gz));
      }
    // traces
    const size_t ntr = (size_t)np * tr_pair;
    double2* trv = base + used;
    double* tra = (rf_rp.on || rf_tr.on) ? (double*)(trv + ntr) : nullptr;
    if (used * sizeof(double2) + ntr * (sizeof(double2) + sizeof(double)) > (size_t)np * per_pair)
      return fail(CTR_ERR_ALLOC, "ctr_rhopi_sigmapi_sets: batch arena overflow");
    TracePlan tp;
    tp.keep = fp64_traces_needed;
    if (tp.keep) tp.tt.reserve((size_t)np * tr_pair);
    // on the split engine the same traces as Gram products: group i * 4 + s2 of
    // pair i pairs the X blocks (set combination ci, row block s5, column block
    // s2) with the Z blocks (sink operator slab, tau block (s3, s2)); every trace
    // takes an X and a Z block with the same s2
    GramPlan gp;
    const bool gram = c.engine == CTR_ENGINE_SPLIT;
    if (gram) {
      gp.tr.reserve((size_t)np * tr_pair);
      gp.ngroup = 4 * np;
      gp.group_run = 4;  // a pair's traces interleave its four s2 groups
      gp.mrows = 4 * nC;
      gp.ncols = 4 * nops;
      gp.left.resize((size_t)gp.ngroup * gp.mrows);
      gp.right.resize((size_t)gp.ngroup * gp.ncols);
      for (int i = 0; i < np; i++)
        for (int s2 = 0; s2 < 4; s2++) {
          const size_t g = (size_t)i * 4 + s2;
          for (int ci = 0; ci < nC; ci++)
            for (int s5 = 0; s5 < 4; s5++) gp.left[g * gp.mrows + ci * 4 + s5] = Xblk(ci, i, s5, s2);
          for (int sl = 0; sl < nops; sl++)
            for (int s3 = 0; s3 < 4; s3++) gp.right[g * gp.ncols + sl * 4 + s3] = Zblk(sl, i, s3 * 4 + s2);
        }
    }
    RowItems it_rp[3], it_tr;
    for (int idir = 0; idir < 3; idir++) {
      it_rp[idir].nrows = ngr;
      it_rp[idir].nout = 4;
      it_rp[idir].csr = csr_rp[idir];
      for (const Grp& g : grp[idir]) it_rp[idir].coef.push_back(make_float2(g.cre, g.cim));
    }
    it_tr.nrows = 32;
    it_tr.nout = 2;
    it_tr.csr = csr_tr;
    for (int i = 0; i < np; i++) {
      const int pair = order[p0 + i];
      for (int k = 0; k < nset; k++) {
        const int ci = cR[k];
        if (rhopi) {
          // Tr-Had(X_{s5 s2}, Phi_ip^dag tau_{s3 s2}) without its coefficient, once for the three
          // polarisations (those of ip = 0, 1 are shared); the row sums apply the coefficients
          const int base = tp.n;
          for (const auto& u : uniq) {
            const int xb = std::get<1>(u), zb = std::get<2>(u);
            const int slot = tp.add(Xblk(ci, i, xb / 4, xb % 4), Zblk(std::get<0>(u), i, zb), 1.f, 0.f, 0);
            if (gram) gp.tr.push_back({i * 4 + xb % 4, ci * 4 + xb / 4, std::get<0>(u) * 4 + zb / 4, slot, 1.f, 0.f});
          }
          for (int idir = 0; idir < 3; idir++) {
            for (int g = 0; g < ngr; g++) it_rp[idir].slot.push_back(base + uidx[idir][g]);
            it_rp[idir].ent.push_back((k * 3 + idir) * npairs + pair);
          }
        }
        if (tri) {
          for (int ik = 0; ik < 2; ik++)
            for (int b = 0; b < 16; b++) {
              const int slot = tp.add(Xblk(ci, i, b / 4, b % 4), Zblk(slab_of[5 + ik], i, b), (float)G5[b / 4], 0.f, 0);
              it_tr.slot.push_back(slot);
              if (gram) gp.tr.push_back({i * 4 + b % 4, ci * 4 + b / 4, slab_of[5 + ik] * 4 + b / 4, slot, (float)G5[b / 4], 0.f});
            }
          it_tr.ent.push_back(k * npairs + pair);
        }
      }
    }
    for (size_t k = 0; k < tp.tt.size(); k++) {
      tp.tt[k].out = trv + k;
      if (tra) tp.tt[k].absout = tra + k;
    }
    CTR_TRY(run_grids(c, g0, WS_TASKS));
    if (gram) {
      // 0: the FP64 trace kernel, 1: Gram products on the tensor cores
      int form = 1;
      auto run = [&](int f) { return f ? trace_gram(N, gp, trv, tra, c.s) : run_traces(c, tp.tt); };
      CTR_TRY(tune_resolve("chains.trace_form", trace_shape, 2, 1, c.s, run, &form));
      if (form == 0 && !tp.keep) return fail(CTR_ERR_ARG, "chains.trace_form: FP64 traces chosen but not planned");
      CTR_TRY(run(form));
    } else {
      CTR_TRY(run_traces(c, tp.tt));
    }
    CTR_TRY(upload_items(c, {&it_rp[0], &it_rp[1], &it_rp[2], &it_tr}));
    for (int idir = 0; idir < 3 && rhopi; idir++)
      CTR_TRY(rowsum_items(c, trv, tra, it_rp[idir], (double2*)rhopi, rf_rp));
    if (tri) CTR_TRY(rowsum_items(c, trv, tra, it_tr, (double2*)tri, rf_tr));
  }
  std::vector<int32_t> sc(sets, sets + 2 * nset);
  auto Pq = [=](int q) { return (const double*)(ph + (size_t)q * N2); };
  if (rhopi)
    CTR_TRY(refine_end(c, rf_rp, 4, WS_REFINE, (double2*)rhopi,
                       [=](const std::vector<int>& units, double2* out, cudaStream_t ls) -> int {
                         size_t u0 = 0;  // units = (set * 3 + idir) * npairs + pair
                         while (u0 < units.size()) {
                           const int kd = units[u0] / npairs, k = kd / 3, idir = kd % 3;
                           std::vector<int> pl;
                           size_t u1 = u0;
                           while (u1 < units.size() && units[u1] / npairs == kd) pl.push_back(units[u1++] % npairs);
                           CTR_TRY(rhopi_chain(N, Nt, tf_begin, tf_end, idir, prop_rows, prop_diag, Pq(sc[2 * k]),
                                               Pq(sc[2 * k + 1]), mom5, (double*)(out + u0 * 4), ls, CTR_ENGINE_FP64,
                                               &pl, (size_t)nphi));
                           u0 = u1;
                         }
                         return CTR_OK;
                       }));
  if (tri)
    CTR_TRY(refine_end(c, rf_tr, 2, WS_SPLITJOBS3, (double2*)tri,
                       [=](const std::vector<int>& units, double2* out, cudaStream_t ls) -> int {
                         size_t u0 = 0;  // units = set * npairs + pair
                         while (u0 < units.size()) {
                           const int k = units[u0] / npairs;
                           std::vector<int> pl;
                           size_t u1 = u0;
                           while (u1 < units.size() && units[u1] / npairs == k) pl.push_back(units[u1++] % npairs);
                           CTR_TRY(sigmapi_chain(N, Nt, tf_begin, tf_end, prop_rows, prop_diag, Pq(sc[2 * k]),
                                                 Pq(sc[2 * k + 1]), mom2, nullptr, (double*)(out + u0 * 2), ls,
                                                 CTR_ENGINE_FP64, &pl, nullptr, (size_t)nphi));
                           u0 = u1;
                         }
                         return CTR_OK;
                       }));
  return CTR_OK;
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

int ctr_pipi_sets(int engine, int nev, int nt, int tf_begin, int tf_end, int isospin, const double* prop_rows,
                  const double* prop_diag, const double* phi, int nphi, int nset, const int32_t* sets, double* corr,
                  void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, tf_begin, tf_end));
  if (isospin != 0 && isospin != 1) return ctr::fail(CTR_ERR_ARG, "isospin must be 0 (I=0) or 1 (I=1)");
  if (nphi < 1 || nset < 1 || !sets) return ctr::fail(CTR_ERR_ARG, "ctr_pipi_sets: nphi=%d, nset=%d", nphi, nset);
  if (!aligned(prop_rows) || !aligned(prop_diag) || !aligned(phi) || !aligned(corr))
    return ctr::fail(CTR_ERR_ARG, "ctr_pipi_sets: null or misaligned pointer");
  return ctr::pipi_sets(nev, nt, tf_begin, tf_end, isospin, prop_rows, prop_diag, phi, nphi, nset, sets, corr,
                        (cudaStream_t)stream, engine);
}

int ctr_rhopi_sigmapi_sets(int engine, int nev, int nt, int tf_begin, int tf_end, const double* prop_rows,
                           const double* prop_diag, const double* phi, int nphi, const double* mom5_p1p2,
                           const double* mom2_p1p2, int nset, const int32_t* sets, double* rhopi, double* triangle,
                           double* hor_fish, void* stream) {
  CTR_TRY(chain_args(engine, nev, nt, tf_begin, tf_end));
  if (nphi < 1 || nset < 1 || !sets)
    return ctr::fail(CTR_ERR_ARG, "ctr_rhopi_sigmapi_sets: nphi=%d, nset=%d", nphi, nset);
  if (!aligned(prop_diag) || !aligned(phi) || ((rhopi || triangle) && !aligned(prop_rows)) ||
      (rhopi && (!aligned(mom5_p1p2) || !aligned(rhopi))) || ((triangle || hor_fish) && !aligned(mom2_p1p2)) ||
      (triangle && !aligned(triangle)) || (hor_fish && !aligned(hor_fish)))
    return ctr::fail(CTR_ERR_ARG, "ctr_rhopi_sigmapi_sets: null or misaligned pointer");
  return ctr::rhopi_sigmapi_sets(nev, nt, tf_begin, tf_end, prop_rows, prop_diag, phi, nphi, mom5_p1p2, mom2_p1p2,
                                 nset, sets, rhopi, triangle, hor_fish, (cudaStream_t)stream, engine);
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
