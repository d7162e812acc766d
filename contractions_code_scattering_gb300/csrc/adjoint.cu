// Distillation-profile adjoint: gradients of diagram traces with respect to a
// per-eigenvector profile f, where every elemental Phi(t, op) enters the
// contractions as diag(f) Phi diag(f).
//
// A chain is Tr[F_1 F_2 ... F_n] (2 <= n <= CTR_CHAIN_MAXF); each factor is a
// perambulator block tau(t1,t2)_{s1 s2} or a profiled elemental
// Phi'(t, op) = D Phi(t, op) D (D = diag f), either optionally
// conjugate-transposed.  For complex chain weights w_c the kernels compute
//   value_c = Tr[chain_c]   and   grad_k += Re sum_c w_c d value_c / d f_k.
//
// Reverse mode with recomputed prefix/suffix products.  With
// P_j = F_1 ... F_j and S_j = F_j ... F_n, the derivative of a trace at one
// occurrence of D is the diagonal of the cyclic product that starts right
// after it, d Tr[..D..]/d f_k = (rest)_kk, i.e. the transposed cyclic
// co-factor (F_{j+1}...F_n F_1...F_{j-1})^T of the adjoint of a product.  A
// profiled elemental F_j holds two D's, which gives
//   f_k d/df_k Tr = sum over elementals j of [diag(S_j P_{j-1}) + diag(S_{j+1} P_j)]_k
// with P_0 = S_{n+1} = identity.  Every diag(X Y) is an O(N^2) reduction
// (diag_reduce_kernel); the only GEMMs are the n-2 prefix and n-2 suffix
// products.  They are recomputed for every call (nothing from the forward
// pass is stored) and shared between chains by hash-consing: a prefix node is
// keyed by (parent, factor), a suffix node by (factor, child), so chains with
// a common head or tail (the spin rows of one diagram, the source times of
// one sink time) compute it once.  Nodes of equal depth form one batched GEMM
// launch.  The profile must have f_k != 0 (the diagonal identity above
// yields f_k d/df_k).
//
// The diagram builders (rho: lib/calculate_rho_core.h; pi pi:
// lib/calculate_pipi_{square,doubleTriangle,doubleTriangleHor,starfish}_core.h)
// emit one chain per spin row in the reference's chain order, so the chain
// values reproduce the reference's rows.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "kernels.h"

namespace ctr {

namespace {

// ------------------------------------------------------------------ kernels
// dst[m] = diag(f) src[m] diag(f), optionally for a strided subset.
__global__ void apply_profile_kernel(const double2* __restrict__ src, double2* __restrict__ dst,
                                     const double* __restrict__ f, int N, long long nmat) {
  const long long n = nmat * N * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int ij = (int)(e % ((long long)N * N));
    const double s = f[ij / N] * f[ij % N];
    const double2 v = src[e];
    dst[e] = make_double2(v.x * s, v.y * s);
  }
}

// One diagonal reduction d_k = sum_m op(X)[k][m] op(Y)[m][k].
// mode 0: buf[out * N + k] = Re(w d_k);  mode 1: vals[out] = sum_k d_k.
struct DiagTask {
  const double2* x;
  const double2* y;
  double wre, wim;
  int xdag, ydag;
  int mode, out;
};

// One CTA per task; 32x32 tiles of op(X) (rows k) and op(Y) (columns k) are
// staged through shared memory with coalesced reads whatever the transposes,
// so both operands are read once.
__global__ void __launch_bounds__(256) diag_reduce_kernel(const DiagTask* __restrict__ tasks, int N,
                                                          double* __restrict__ buf, double2* __restrict__ vals) {
  __shared__ double2 xs[32][33];
  __shared__ double2 ys[32][33];
  __shared__ double2 part[8][32];
  __shared__ double2 tot[32];
  const DiagTask T = tasks[blockIdx.x];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double2 vsum = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < N; k0 += 32) {
    double2 acc = make_double2(0.0, 0.0);  // thread (tx = k, ty): m = ty, ty+8, ... of each tile
    for (int m0 = 0; m0 < N; m0 += 32) {
      for (int r = ty; r < 32; r += 8) {
        // xs[kk][mm] = op(X)[k0+kk][m0+mm]
        if (!T.xdag) {
          const int k = k0 + r, m = m0 + tx;
          xs[r][tx] = (k < N && m < N) ? T.x[(size_t)k * N + m] : make_double2(0.0, 0.0);
        } else {  // op(X)[k][m] = conj(X[m][k]): read row m0+r, columns k0+tx
          const int m = m0 + r, k = k0 + tx;
          double2 v = (k < N && m < N) ? T.x[(size_t)m * N + k] : make_double2(0.0, 0.0);
          xs[tx][r] = make_double2(v.x, -v.y);
        }
        // ys[mm][kk] = op(Y)[m0+mm][k0+kk]
        if (!T.ydag) {
          const int m = m0 + r, k = k0 + tx;
          ys[r][tx] = (k < N && m < N) ? T.y[(size_t)m * N + k] : make_double2(0.0, 0.0);
        } else {  // op(Y)[m][k] = conj(Y[k][m]): read row k0+r, columns m0+tx
          const int k = k0 + r, m = m0 + tx;
          double2 v = (k < N && m < N) ? T.y[(size_t)k * N + m] : make_double2(0.0, 0.0);
          ys[tx][r] = make_double2(v.x, -v.y);
        }
      }
      __syncthreads();
      // only the tile's valid m (the padding beyond N would still cost the FP64 pipe)
      const int mlim = min(32, N - m0);
      for (int mm = ty; mm < mlim; mm += 8) cmac(acc, xs[tx][mm], ys[mm][tx]);
      __syncthreads();
    }
    part[ty][tx] = acc;
    __syncthreads();
    if (ty == 0) {
      double2 d = make_double2(0.0, 0.0);
      for (int q = 0; q < 8; q++) {
        d.x += part[q][tx].x;
        d.y += part[q][tx].y;
      }
      const int k = k0 + tx;
      if (T.mode == 0) {
        if (k < N) buf[(size_t)T.out * N + k] = T.wre * d.x - T.wim * d.y;
      } else {
        tot[tx] = k < N ? d : make_double2(0.0, 0.0);
      }
    }
    __syncthreads();
    if (T.mode == 1 && threadIdx.x == 0) {
      for (int q = 0; q < 32; q++) {
        vsum.x += tot[q].x;
        vsum.y += tot[q].y;
      }
    }
    __syncthreads();
  }
  if (T.mode == 1 && threadIdx.x == 0) vals[T.out] = vsum;
}

// grad[k] += (sum_t buf[t][k]) / f[k], summed in a fixed order.
__global__ void __launch_bounds__(256) grad_reduce_kernel(const double* __restrict__ buf, int ntask, int N,
                                                          const double* __restrict__ f, double* __restrict__ grad) {
  const int k = blockIdx.x;
  double s = 0.0;
  for (int t = threadIdx.x; t < ntask; t += 256) s += buf[(size_t)t * N + k];
  s = block_sum_256(s);
  if (threadIdx.x == 0) grad[k] += s / f[k];
}

// ------------------------------------------------------------- chain program
inline int64_t factor_key(const ctr_factor& F) {
  return ((((((int64_t)F.kind * 2 + (F.dag ? 1 : 0)) * 8192 + F.a) * 8192 + F.b) * 4 + F.s1) * 4 + F.s2);
}

struct Opnd {
  const double2* p;
  int dag;
};

class ChainProgram {
 public:
  ChainProgram(int N, int Nt, int nphi, const double2* prop, const double2* phis, int engine)
      : N_(N), Nt_(Nt), nphi_(nphi), engine_(engine), prop_(prop), phis_(phis) {}

  int check_factor(const ctr_factor& F) const {
    if (F.kind == CTR_FACTOR_TAU) {
      if (F.a < 0 || F.a >= Nt_ || F.b < 0 || F.b >= Nt_ || F.s1 < 0 || F.s1 > 3 || F.s2 < 0 || F.s2 > 3)
        return fail(CTR_ERR_ARG, "chain factor: perambulator block out of range");
    } else if (F.kind == CTR_FACTOR_PHI) {
      if (F.a < 0 || F.a >= Nt_ || F.b < 0 || F.b >= nphi_)
        return fail(CTR_ERR_ARG, "chain factor: elemental out of range");
    } else {
      return fail(CTR_ERR_ARG, "chain factor: unknown kind %d", F.kind);
    }
    return CTR_OK;
  }

  Opnd leaf(const ctr_factor& F) const {
    const size_t N2 = (size_t)N_ * N_;
    if (F.kind == CTR_FACTOR_TAU)
      return Opnd{prop_ + (((size_t)F.a * Nt_ + F.b) * 16 + F.s1 * 4 + F.s2) * N2, F.dag ? 1 : 0};
    return Opnd{phis_ + ((size_t)F.a * nphi_ + F.b) * N2, F.dag ? 1 : 0};
  }

  // Adds one chain; returns the number of new GEMM nodes it needed.
  int add(const ctr_factor* F, int n, double2 w, int value_slot, bool grad) {
    Chain c;
    c.f.assign(F, F + n);
    c.w = w;
    c.value_slot = value_slot;
    c.grad = grad;
    const int before = (int)nodes_.size();
    // prefixes P_1 .. P_{n-1} (P_1 is the leaf F_1); operand ids: >= 0 node, < 0 leaf index in chain
    c.pre.assign(n, -1);
    int64_t cur = -(1 + factor_key(F[0]));
    c.pre[0] = -1;
    for (int j = 1; j < n - 1; j++) {
      cur = node(cur, -(1 + factor_key(F[j])), j + 1, F, j, true, c.pre[j - 1]);
      c.pre[j] = (int)cur;
    }
    // suffixes S_n .. S_2 (S_n is the leaf F_n); a chain without gradient needs none
    c.suf.assign(n + 1, -1);
    cur = -(1 + factor_key(F[n - 1]));
    for (int j = n - 2; j >= 1 && grad; j--) {
      cur = node(-(1 + factor_key(F[j])), cur, n - j, F, j, false, c.suf[j + 1]);
      c.suf[j] = (int)cur;
    }
    chains_.push_back(std::move(c));
    return (int)nodes_.size() - before;
  }

  size_t nodes() const { return nodes_.size(); }

  void clear() {
    nodes_.clear();
    chains_.clear();
    pre_map_.clear();
    suf_map_.clear();
  }

  // Executes the program: GEMM levels, diagonal reductions, gradient sum.
  int run(const double* f, double2* values, double* grad, cudaStream_t s);

 private:
  struct Node {
    int depth;
    int a_node, b_node;  // >= 0: operand is node; -1: leaf
    Opnd a_leaf, b_leaf;
  };
  struct Chain {
    std::vector<ctr_factor> f;
    std::vector<int> pre, suf;  // node ids (-1 = leaf)
    double2 w;
    int value_slot;
    bool grad;
  };

  // prefix node: parent (node id >= 0 or leaf key < 0) x factor F[j]
  // suffix node: factor F[j] x child
  int64_t node(int64_t left, int64_t right, int depth, const ctr_factor* F, int j, bool prefix, int other_node) {
    auto& map = prefix ? pre_map_ : suf_map_;
    const auto key = std::make_pair(left, right);
    auto it = map.find(key);
    if (it != map.end()) return it->second;
    Node nd;
    nd.depth = depth;
    if (prefix) {
      nd.a_node = other_node;  // parent node (or -1 if P_1 is a leaf)
      nd.a_leaf = leaf(F[0]);
      nd.b_node = -1;
      nd.b_leaf = leaf(F[j]);
    } else {
      nd.a_node = -1;
      nd.a_leaf = leaf(F[j]);
      nd.b_node = other_node;  // child node (or -1 if S_{j+1} is the leaf F_n)
      nd.b_leaf = leaf(F[j + 1]);
    }
    const int id = (int)nodes_.size();
    nodes_.push_back(nd);
    map.emplace(key, id);
    return id;
  }

  int N_, Nt_, nphi_, engine_;
  const double2* prop_;
  const double2* phis_;
  std::vector<Node> nodes_;
  std::vector<Chain> chains_;
  std::map<std::pair<int64_t, int64_t>, int> pre_map_, suf_map_;
};

int ChainProgram::run(const double* f, double2* values, double* grad, cudaStream_t s) {
  if (chains_.empty()) return CTR_OK;
  const size_t N2 = (size_t)N_ * N_;
  void* nodemem = nullptr;
  CTR_TRY(workspace(WS_SCRATCH).get(std::max<size_t>(1, nodes_.size()) * N2 * sizeof(double2), &nodemem));
  double2* nb = (double2*)nodemem;
  auto opnd = [&](int node_id, const Opnd& lf) { return node_id >= 0 ? Opnd{nb + (size_t)node_id * N2, 0} : lf; };

  // GEMM levels: nodes of equal depth are independent; one upload, one launch per depth
  int maxd = 0;
  for (const Node& nd : nodes_) maxd = std::max(maxd, nd.depth);
  std::vector<ZTask> tasks;
  std::vector<size_t> level_off(maxd + 2, 0);
  for (int d = 2; d <= maxd; d++) {
    level_off[d] = tasks.size();
    for (size_t i = 0; i < nodes_.size(); i++) {
      const Node& nd = nodes_[i];
      if (nd.depth != d) continue;
      const Opnd a = opnd(nd.a_node, nd.a_leaf), b = opnd(nd.b_node, nd.b_leaf);
      ZTask t;
      std::memset(&t, 0, sizeof(t));
      t.A[0] = a.p;
      t.B[0] = b.p;
      t.C = nb + i * N2;
      t.wre[0] = 1.f;
      t.nterm = 1;
      t.flags = (a.dag ? 1 : 0) | (b.dag ? 16 : 0);
      tasks.push_back(t);
    }
  }
  level_off[maxd + 1] = tasks.size();
  if (!tasks.empty() && engine_ == CTR_ENGINE_SPLIT) {
    for (int d = 2; d <= maxd; d++) {
      const size_t n0 = level_off[d], n1 = level_off[d + 1];
      if (n1 > n0) CTR_TRY(zgemm_split_tasks(N_, tasks.data() + n0, (int)(n1 - n0), s));
    }
  } else if (!tasks.empty()) {
    void* dt;
    CTR_TRY(upload(WS_GEMM_A, tasks.data(), tasks.size() * sizeof(ZTask), &dt, s));
    for (int d = 2; d <= maxd; d++) {
      const size_t n0 = level_off[d], n1 = level_off[d + 1];
      if (n1 > n0) CTR_TRY(launch_zgemm_f64((const ZTask*)dt + n0, (int)(n1 - n0), N_, s, tasks.data() + n0));
    }
  }

  // diagonal reductions (gradient) and traces (values)
  std::vector<DiagTask> dtasks;
  int ngrad = 0;
  for (const Chain& c : chains_) {
    const int n = (int)c.f.size();
    auto P = [&](int j) { return opnd(c.pre[j - 1], leaf(c.f[0])); };  // P_j, j = 1..n-1
    auto S = [&](int j) { return opnd(c.suf[j - 1], leaf(c.f[n - 1])); };  // S_j, j = 2..n
    auto F = [&](int j) { return leaf(c.f[j - 1]); };
    auto push = [&](Opnd x, Opnd y, int mode, int out) {
      DiagTask t;
      t.x = x.p;
      t.y = y.p;
      t.xdag = x.dag;
      t.ydag = y.dag;
      t.wre = c.w.x;
      t.wim = c.w.y;
      t.mode = mode;
      t.out = out;
      dtasks.push_back(t);
    };
    if (c.value_slot >= 0) push(P(n - 1), F(n), 1, c.value_slot);  // Tr = sum diag(P_{n-1} F_n)
    if (!c.grad) continue;
    for (int j = 1; j <= n; j++) {
      if (c.f[j - 1].kind != CTR_FACTOR_PHI) continue;
      // left D of F_j: diag(S_j P_{j-1}); j = 1: diag(F_1 S_2)
      if (j == 1) push(F(1), S(2), 0, ngrad++);
      else push(S(j), P(j - 1), 0, ngrad++);
      // right D of F_j: diag(S_{j+1} P_j); j = n: diag(P_{n-1} F_n)
      if (j == n) push(P(n - 1), F(n), 0, ngrad++);
      else push(S(j + 1), P(j), 0, ngrad++);
    }
  }
  if (dtasks.empty()) return CTR_OK;
  void *ddt, *dbuf = nullptr;
  CTR_TRY(upload(WS_ROWTASKS, dtasks.data(), dtasks.size() * sizeof(DiagTask), &ddt, s));
  if (ngrad > 0) CTR_TRY(workspace(WS_ROWS).get((size_t)ngrad * N_ * sizeof(double), &dbuf));
  {
    TimedLaunch tl(s, "diag_reduce");
    diag_reduce_kernel<<<(unsigned)dtasks.size(), 256, 0, s>>>((const DiagTask*)ddt, N_, (double*)dbuf, values);
    CTR_CUDA(cudaGetLastError());
  }
  if (ngrad > 0) {
    TimedLaunch tl(s, "grad_reduce");
    grad_reduce_kernel<<<N_, 256, 0, s>>>((const double*)dbuf, ngrad, N_, f, grad);
    CTR_CUDA(cudaGetLastError());
  }
  return CTR_OK;
}

// Runs chains through programs of bounded size (node storage <= budget).
class ChainRunner {
 public:
  ChainRunner(int N, int Nt, int nphi, const double2* prop, const double2* phis, const double* f, double2* values,
              double* grad, cudaStream_t s, int engine = CTR_ENGINE_FP64)
      : prog_(N, Nt, nphi, prop, phis, engine), f_(f), values_(values), grad_(grad), s_(s) {
    const size_t budget = (size_t)3 << 30;
    max_nodes_ = std::max<size_t>(64, budget / ((size_t)N * N * sizeof(double2)));
  }
  int check(const ctr_factor& F) const { return prog_.check_factor(F); }
  // Chains of one group (e.g. one (t_sink, t_src) pair) are added together.
  int add(const ctr_factor* F, int n, double2 w, int value_slot, bool grad) {
    prog_.add(F, n, w, value_slot, grad);
    return CTR_OK;
  }
  int end_group() {
    if (prog_.nodes() >= max_nodes_ / 2) return flush();
    return CTR_OK;
  }
  int flush() {
    CTR_TRY(prog_.run(f_, values_, grad_, s_));
    prog_.clear();
    return CTR_OK;
  }

 private:
  ChainProgram prog_;
  const double* f_;
  double2* values_;
  double* grad_;
  cudaStream_t s_;
  size_t max_nodes_;
};

// Scaled elemental copies diag(f) Phi diag(f) in a workspace slot.
int profiled(int N, long long nmat, const double* phi, const double* f, int slot, double2** out, cudaStream_t s) {
  void* p;
  CTR_TRY(workspace(slot).get((size_t)nmat * N * N * sizeof(double2), &p));
  TimedLaunch tl(s, "apply_profile");
  apply_profile_kernel<<<1024, 256, 0, s>>>((const double2*)phi, (double2*)p, f, N, nmat);
  CTR_CUDA(cudaGetLastError());
  *out = (double2*)p;
  return CTR_OK;
}

int check_f(int N, const double* f, cudaStream_t s) {
  std::vector<double> h(N);
  CTR_CUDA(cudaMemcpyAsync(h.data(), f, N * sizeof(double), cudaMemcpyDeviceToHost, s));
  CTR_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < N; k++)
    if (!(h[k] != 0.0) || !std::isfinite(h[k])) return fail(CTR_ERR_ARG, "profile f[%d] = %g must be finite and nonzero", k, h[k]);
  return CTR_OK;
}

inline ctr_factor tau(int t1, int t2, int s1, int s2, int dag = 0) {
  ctr_factor F;
  F.kind = CTR_FACTOR_TAU;
  F.dag = dag;
  F.a = t1;
  F.b = t2;
  F.s1 = s1;
  F.s2 = s2;
  return F;
}

inline ctr_factor phi(int t, int op, int dag = 0) {
  ctr_factor F;
  F.kind = CTR_FACTOR_PHI;
  F.dag = dag;
  F.a = t;
  F.b = op;
  F.s1 = 0;
  F.s2 = 0;
  return F;
}

inline double2 cw(double2 w, double re, double im) { return make_double2(w.x * re - w.y * im, w.x * im + w.y * re); }

int check_engine(int engine, int nev) {
  if (engine != CTR_ENGINE_FP64 && engine != CTR_ENGINE_SPLIT) return fail(CTR_ERR_ARG, "unknown engine %d", engine);
  return CTR_OK;
}

}  // namespace

int chain_values(int N, int Nt, int nphi, const double* prop, const double* phi, const std::vector<ctr_factor>& factors,
                 const std::vector<int>& off, double* values, cudaStream_t s, int engine) {
  ChainRunner R(N, Nt, nphi, (const double2*)prop, (const double2*)phi, nullptr, (double2*)values, nullptr, s, engine);
  const int nchain = (int)off.size() - 1;
  for (int c = 0; c < nchain; c++) {
    const int n = off[c + 1] - off[c];
    if (n < 2 || n > CTR_CHAIN_MAXF) return fail(CTR_ERR_ARG, "chain %d has %d factors", c, n);
    for (int j = 0; j < n; j++) CTR_TRY(R.check(factors[off[c] + j]));
    CTR_TRY(R.add(&factors[off[c]], n, make_double2(0.0, 0.0), c, false));
    CTR_TRY(R.end_group());
  }
  return R.flush();
}

}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_apply_profile(int nev, long long nmat, const double* f, const double* src, double* dst, void* stream) {
  if (nev < 1 || nmat < 0 || !f || !src || !dst) return fail(CTR_ERR_ARG, "ctr_apply_profile: bad arguments");
  if (nmat == 0) return CTR_OK;
  TimedLaunch tl((cudaStream_t)stream, "apply_profile");
  apply_profile_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>((const double2*)src, (double2*)dst, f, nev, nmat);
  CTR_CUDA(cudaGetLastError());
  return CTR_OK;
}

int ctr_chain_adjoint(int engine, int nev, int nt, int nphi, const double* prop, const double* phi, const double* f,
                      int nchain, const int* chain_off, const ctr_factor* factors, const double* w, double* values,
                      double* grad, void* stream) {
  CTR_NO_CAPTURE("ctr_chain_adjoint");
  cudaStream_t s = (cudaStream_t)stream;
  CTR_TRY(check_engine(engine, nev));
  if (nev < 1 || nt < 1 || nphi < 0 || nchain < 0 || !prop || !f || !chain_off || !factors || (!values && !grad))
    return fail(CTR_ERR_ARG, "ctr_chain_adjoint: bad arguments");
  if (grad && !w) return fail(CTR_ERR_ARG, "ctr_chain_adjoint: weights are needed for the gradient");
  if (nphi > 0 && !phi) return fail(CTR_ERR_ARG, "ctr_chain_adjoint: elementals missing");
  CTR_TRY(check_f(nev, f, s));
  double2* phis = nullptr;
  if (nphi > 0) CTR_TRY(profiled(nev, (long long)nt * nphi, phi, f, WS_PHI, &phis, s));
  ChainRunner R(nev, nt, nphi, (const double2*)prop, phis, f, (double2*)values, grad, s, engine);
  for (int c = 0; c < nchain; c++) {
    const int n = chain_off[c + 1] - chain_off[c];
    if (n < 2 || n > CTR_CHAIN_MAXF) return fail(CTR_ERR_ARG, "chain %d has %d factors (2..%d)", c, n, CTR_CHAIN_MAXF);
    for (int j = 0; j < n; j++) CTR_TRY(R.check(factors[chain_off[c] + j]));
    const double2 wc = w ? make_double2(w[2 * c], w[2 * c + 1]) : make_double2(0.0, 0.0);
    CTR_TRY(R.add(factors + chain_off[c], n, wc, values ? c : -1, grad != nullptr));
    CTR_TRY(R.end_group());
  }
  return R.flush();
}

int ctr_rho_profile_vjp(int engine, int nev, int nt, const double* prop, const double* mom5, const double* f,
                        const double* w, double* corr, double* grad, void* stream) {
  CTR_NO_CAPTURE("ctr_rho_profile_vjp");
  cudaStream_t s = (cudaStream_t)stream;
  CTR_TRY(check_engine(engine, nev));
  if (nev < 1 || nt < 1 || !prop || !mom5 || !f || !w || (!corr && !grad))
    return fail(CTR_ERR_ARG, "ctr_rho_profile_vjp: bad arguments");
  CTR_TRY(check_f(nev, f, s));
  std::vector<double> hw((size_t)nt * nt * 48 * 2);
  CTR_CUDA(cudaMemcpyAsync(hw.data(), w, hw.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  CTR_CUDA(cudaStreamSynchronize(s));
  std::vector<int> pairs;
  for (int p = 0; p < nt * nt; p++) {
    bool any = false;
    for (int k = 0; k < 96; k++) any = any || hw[(size_t)p * 96 + k] != 0.0;
    if (any) pairs.push_back(p);
  }
  double2* phis;
  CTR_TRY(profiled(nev, (long long)nt * 5, mom5, f, WS_PHI, &phis, s));
  const Tables& T = tables();
  void* dvals = nullptr;
  const size_t nval = std::max<size_t>(1, pairs.size() * 768);
  if (corr) {
    CTR_TRY(workspace(WS_TASKS2).get(nval * sizeof(double2), &dvals));
    CTR_CUDA(cudaMemsetAsync(dvals, 0, nval * sizeof(double2), s));
  }
  ChainRunner R(nev, nt, 5, (const double2*)prop, phis, f, (double2*)dvals, grad, s, engine);
  // lib/calculate_rho_core.h: coef * Tr[tau_{s3s4} Phi_lp(ti) (Phi_rp(tf) tau_{s1s2})^dagger]
  for (size_t q = 0; q < pairs.size(); q++) {
    const int tf = pairs[q] / nt, ti = pairs[q] % nt;
    for (int o = 0; o < 48; o++) {
      const size_t wi = ((size_t)pairs[q] * 48 + o) * 2;
      const double2 wo = make_double2(hw[wi], hw[wi + 1]);
      if (wo.x == 0.0 && wo.y == 0.0) continue;
      for (int is = 0; is < 16; is++) {
        const int r = o * 16 + is;
        const int s1 = T.rho_spin[r][0], s2 = T.rho_spin[r][1], s3 = T.rho_spin[r][2], s4 = T.rho_spin[r][3];
        const int lp = T.rho_lprp[r][0], rp = T.rho_lprp[r][1];
        const ctr_factor ch[4] = {tau(tf, ti, s3, s4), phi(ti, lp), tau(tf, ti, s1, s2, 1), phi(tf, rp, 1)};
        CTR_TRY(R.add(ch, 4, cw(wo, T.rho_coef[r][0], T.rho_coef[r][1]), corr ? (int)(q * 768 + r) : -1,
                      grad != nullptr));
      }
    }
    CTR_TRY(R.end_group());
  }
  CTR_TRY(R.flush());
  if (corr) {
    // corr[tf][ti][o] = sum of the 16 coefficient-weighted spin rows (lib/contract_kernels_rho.cu:108-116)
    std::vector<double2> rv(pairs.size() * 768);
    if (!rv.empty()) {
      CTR_CUDA(cudaMemcpyAsync(rv.data(), dvals, rv.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
      CTR_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<double2> hc((size_t)nt * nt * 48, make_double2(0.0, 0.0));
    for (size_t q = 0; q < pairs.size(); q++)
      for (int r = 0; r < 768; r++) {
        const double2 v = cmul(make_double2(T.rho_coef[r][0], T.rho_coef[r][1]), rv[q * 768 + r]);
        double2& c = hc[(size_t)pairs[q] * 48 + r / 16];
        c.x += v.x;
        c.y += v.y;
      }
    CTR_CUDA(cudaMemcpyAsync(corr, hc.data(), hc.size() * sizeof(double2), cudaMemcpyHostToDevice, s));
    CTR_CUDA(cudaStreamSynchronize(s));
  }
  return CTR_OK;
}

int ctr_pipi_profile_vjp(int engine, int nev, int nt, int isospin, const double* prop, const double* p1,
                         const double* p2, const double* p3, const double* p4, const double* f, const double* w,
                         double* corr, double* grad, void* stream) {
  CTR_NO_CAPTURE("ctr_pipi_profile_vjp");
  cudaStream_t s = (cudaStream_t)stream;
  CTR_TRY(check_engine(engine, nev));
  if (nev < 1 || nt < 1 || !prop || !p1 || !p2 || !p3 || !p4 || !f || !w || (!corr && !grad))
    return fail(CTR_ERR_ARG, "ctr_pipi_profile_vjp: bad arguments");
  if (isospin != 0 && isospin != 1) return fail(CTR_ERR_ARG, "isospin must be 0 (I=0) or 1 (I=1)");
  CTR_TRY(check_f(nev, f, s));
  const size_t N2 = (size_t)nev * nev;
  std::vector<double> hw((size_t)nt * nt * 5 * 2);
  CTR_CUDA(cudaMemcpyAsync(hw.data(), w, hw.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  // elementals [t][4] = P1..P4 (profiled)
  void* raw;
  CTR_TRY(workspace(WS_MISC).get((size_t)nt * 4 * N2 * sizeof(double2), &raw));
  const double* ps[4] = {p1, p2, p3, p4};
  for (int t = 0; t < nt; t++)
    for (int k = 0; k < 4; k++)
      CTR_CUDA(cudaMemcpyAsync((double2*)raw + ((size_t)t * 4 + k) * N2, (const double2*)ps[k] + (size_t)t * N2,
                               N2 * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  double2* phis;
  CTR_TRY(profiled(nev, (long long)nt * 4, (const double*)raw, f, WS_PHI, &phis, s));
  const Tables& T = tables();
  enum { P1 = 0, P2 = 1, P3 = 2, P4 = 3 };
  // isospin weights of the correlator slots (lib/contract_kernels_pipi.cu:288-303, :463-478)
  const double wsq = isospin == 1 ? -2.0 : -1.0 / 3.0, wdt = isospin == 1 ? 2.0 : -1.0 / 3.0;
  const double wstar = isospin == 1 ? -1.0 : 1.0, wfish = 1.0, wdth = isospin == 1 ? 0.0 : -5.0 / 3.0;

  std::vector<int> pairs;
  for (int p = 0; p < nt * nt; p++) {
    bool any = false;
    for (int k = 0; k < 10; k++) any = any || hw[(size_t)p * 10 + k] != 0.0;
    if (any) pairs.push_back(p);
  }
  // star / fish are products of two spin-summed traces: their values come first
  // (lib/calculate_pipi_starfish_core.h: tr = Tr[Pa(tf) tau_{s1s2} Pb(ti) tau_{s1s2}^dagger])
  auto sf_chain = [&](int tf, int ti, int is, int a, int b, ctr_factor* ch) {
    const int s1 = is / 4, s2 = is % 4;
    ch[0] = phi(tf, a);
    ch[1] = tau(tf, ti, s1, s2);
    ch[2] = phi(ti, b);
    ch[3] = tau(tf, ti, s1, s2, 1);
  };
  // [pair][4 traces: star tr1 (P4,P1), star tr2 (P3,P2), fish tr1 (P3,P1), fish tr2 (P4,P2)][16]
  const int sfa[4] = {P4, P3, P3, P4}, sfb[4] = {P1, P2, P1, P2};
  std::vector<double2> sfv(pairs.size() * 64, make_double2(0.0, 0.0));
  {
    void* dv;
    CTR_TRY(workspace(WS_TASKS2).get(std::max<size_t>(1, sfv.size()) * sizeof(double2), &dv));
    ChainRunner R(nev, nt, 4, (const double2*)prop, phis, f, (double2*)dv, nullptr, s, engine);
    for (size_t q = 0; q < pairs.size(); q++) {
      const int tf = pairs[q] / nt, ti = pairs[q] % nt;
      for (int k = 0; k < 4; k++)
        for (int is = 0; is < 16; is++) {
          ctr_factor ch[4];
          sf_chain(tf, ti, is, sfa[k], sfb[k], ch);
          CTR_TRY(R.add(ch, 4, make_double2(0.0, 0.0), (int)(q * 64 + k * 16 + is), false));
        }
      CTR_TRY(R.end_group());
    }
    CTR_TRY(R.flush());
    if (!sfv.empty()) {
      CTR_CUDA(cudaMemcpyAsync(sfv.data(), dv, sfv.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
      CTR_CUDA(cudaStreamSynchronize(s));
    }
  }
  void* dvals = nullptr;
  if (corr) {
    // per-chain values: 256 square + 256 dT + 256 dTH rows per pair
    CTR_TRY(workspace(WS_TASKS2).get(std::max<size_t>(1, pairs.size() * 768) * sizeof(double2), &dvals));
    CTR_CUDA(cudaMemsetAsync(dvals, 0, std::max<size_t>(1, pairs.size() * 768) * sizeof(double2), s));
  }
  const bool g = grad != nullptr;
  ChainRunner R(nev, nt, 4, (const double2*)prop, phis, f, (double2*)dvals, grad, s, engine);
  for (size_t q = 0; q < pairs.size(); q++) {
    const int tf = pairs[q] / nt, ti = pairs[q] % nt;
    const double* wp = &hw[(size_t)pairs[q] * 10];
    const double2 w_sq = make_double2(wp[0] * wsq, wp[1] * wsq), w_dt = make_double2(wp[2] * wdt, wp[3] * wdt);
    const double2 w_st = make_double2(wp[4] * wstar, wp[5] * wstar), w_fi = make_double2(wp[6] * wfish, wp[7] * wfish);
    const double2 w_dh = make_double2(wp[8] * wdth, wp[9] * wdth);
    for (int bx = 0; bx < 256; bx++) {
      const int16_t* sq = T.sq_spin[bx];
      // lib/calculate_pipi_square_core.h
      const ctr_factor c_sq[8] = {phi(tf, P3),          tau(tf, tf, sq[2], sq[3]), phi(tf, P4),
                                  tau(tf, ti, sq[4], sq[5]), phi(ti, P2),           tau(ti, ti, sq[0], sq[1]),
                                  phi(ti, P1),          tau(tf, ti, sq[2], sq[1], 1)};
      CTR_TRY(R.add(c_sq, 8, cw(w_sq, T.sq_coef[bx][0], T.sq_coef[bx][1]), corr ? (int)(q * 768 + bx) : -1, g));
      const int16_t* dt = T.dt_spin[bx];
      // lib/calculate_pipi_doubleTriangle_core.h
      const ctr_factor c_dt[8] = {phi(tf, P3),          tau(tf, tf, dt[4], dt[5]), phi(tf, P4),
                                  tau(tf, ti, dt[0], dt[1]), phi(ti, P1),           tau(ti, ti, dt[2], dt[3]),
                                  phi(ti, P2),          tau(tf, ti, dt[4], dt[3], 1)};
      CTR_TRY(R.add(c_dt, 8, cw(w_dt, T.dt_coef[bx][0], T.dt_coef[bx][1]), corr ? (int)(q * 768 + 256 + bx) : -1,
                    g));
      if (isospin == 0) {
        const int16_t* dh = T.dth_spin[bx];
        // lib/calculate_pipi_doubleTriangleHor_core.h (all blocks tau(tf, ti))
        const ctr_factor c_dh[8] = {phi(tf, P3),          tau(tf, ti, dh[0], dh[1]),    phi(ti, P1),
                                    tau(tf, ti, dh[2], dh[1], 1), phi(tf, P4),         tau(tf, ti, dh[2], dh[3]),
                                    phi(ti, P2),          tau(tf, ti, dh[0], dh[3], 1)};
        CTR_TRY(R.add(c_dh, 8, cw(w_dh, T.dth_coef[bx][0], T.dth_coef[bx][1]),
                      corr ? (int)(q * 768 + 512 + bx) : -1, g));
      }
    }
    // star = tr1 * tr2 (sums over 16 spins): d(star) = tr2 d(tr1) + tr1 d(tr2); fish likewise
    double2 sum[4];
    for (int k = 0; k < 4; k++) {
      sum[k] = make_double2(0.0, 0.0);
      for (int is = 0; is < 16; is++) {
        sum[k].x += sfv[q * 64 + k * 16 + is].x;
        sum[k].y += sfv[q * 64 + k * 16 + is].y;
      }
    }
    const double2 wk[4] = {cmul(w_st, sum[1]), cmul(w_st, sum[0]), cmul(w_fi, sum[3]), cmul(w_fi, sum[2])};
    for (int k = 0; k < 4 && g; k++) {
      if (wk[k].x == 0.0 && wk[k].y == 0.0) continue;
      for (int is = 0; is < 16; is++) {
        ctr_factor ch[4];
        sf_chain(tf, ti, is, sfa[k], sfb[k], ch);
        CTR_TRY(R.add(ch, 4, wk[k], -1, true));
      }
    }
    CTR_TRY(R.end_group());
  }
  CTR_TRY(R.flush());
  if (corr) {
    // corr[tf][ti][5] for the pairs with nonzero weight (zero elsewhere), isospin-weighted
    std::vector<double2> rv(pairs.size() * 768);
    if (!rv.empty()) {
      CTR_CUDA(cudaMemcpyAsync(rv.data(), dvals, rv.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
      CTR_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<double2> hc((size_t)nt * nt * 5, make_double2(0.0, 0.0));
    for (size_t q = 0; q < pairs.size(); q++) {
      double2 a[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
      for (int d = 0; d < 3; d++)
        for (int bx = 0; bx < 256; bx++) {
          const float* cf = d == 0 ? T.sq_coef[bx] : d == 1 ? T.dt_coef[bx] : T.dth_coef[bx];
          const double2 v = cmul(make_double2(cf[0], cf[1]), rv[q * 768 + d * 256 + bx]);
          a[d].x += v.x;
          a[d].y += v.y;
        }
      double2 sum[4];
      for (int k = 0; k < 4; k++) {
        sum[k] = make_double2(0.0, 0.0);
        for (int is = 0; is < 16; is++) {
          sum[k].x += sfv[q * 64 + k * 16 + is].x;
          sum[k].y += sfv[q * 64 + k * 16 + is].y;
        }
      }
      const double2 st = cmul(sum[0], sum[1]), fi = cmul(sum[2], sum[3]);
      double2* c = &hc[(size_t)pairs[q] * 5];
      c[0] = make_double2(wsq * a[0].x, wsq * a[0].y);
      c[1] = make_double2(wdt * a[1].x, wdt * a[1].y);
      c[2] = make_double2(wstar * st.x, wstar * st.y);
      c[3] = make_double2(wfish * fi.x, wfish * fi.y);
      c[4] = make_double2(wdth * a[2].x, wdth * a[2].y);
    }
    CTR_CUDA(cudaMemcpyAsync(corr, hc.data(), hc.size() * sizeof(double2), cudaMemcpyHostToDevice, s));
    CTR_CUDA(cudaStreamSynchronize(s));
  }
  return CTR_OK;
}

}  // extern "C"
