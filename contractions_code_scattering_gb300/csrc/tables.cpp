// Diagram tables (spin indices, operator / momentum selectors, coefficients).
//
// The reference ships them as generated headers include/constants_{rho,rhopi,
// pipi,sigma,sigmapi}.h, written by devTools/comb_*.cpp from the gwu-qcd gamma
// matrices.  The library builds the same tables at load time from the gamma
// matrices themselves: every entry is a product of gamma-matrix elements, and a
// spin row exists where that product is non-zero.  The basis that reproduces
// the shipped tables exactly (signed zeros included) is the chiral
// DeGrand-Rossi basis with all four gamma_mu negated, gamma_5 = diag(1,1,-1,-1).
// Products are evaluated left to right, as the generators do, so that the sign
// of a zero imaginary part matches the shipped "%+3.2f" output.
#include <cstring>

#include "ctr_internal.h"

namespace ctr {
namespace {

struct Z {
  double re, im;
};
inline Z operator*(Z a, Z b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Z neg(Z a) { return {-a.re, -a.im}; }
inline Z scale(double s, Z a) { return {s * a.re, s * a.im}; }
inline bool nonzero(Z a) { return a.re * a.re + a.im * a.im != 0.0; }

struct Spin4 {
  Z m[4][4];
};

Spin4 zero4() {
  Spin4 s;
  for (auto& r : s.m)
    for (auto& e : r) e = {0.0, 0.0};
  return s;
}

Spin4 mul4(const Spin4& a, const Spin4& b) {
  Spin4 r = zero4();
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      Z acc = {0.0, 0.0};
      for (int k = 0; k < 4; k++) {
        Z p = a.m[i][k] * b.m[k][j];
        acc = {acc.re + p.re, acc.im + p.im};
      }
      r.m[i][j] = acc;
    }
  return r;
}

// A gamma matrix of this basis is a signed permutation: row r has its single
// entry in column col[r] with value val[r].
Spin4 perm4(const int col[4], const Z val[4]) {
  Spin4 s = zero4();
  for (int r = 0; r < 4; r++) s.m[r][col[r]] = val[r];
  return s;
}

struct Gammas {
  Spin4 g[5];  // g1..g4, g5 = g1 g2 g3 g4
  Gammas() {
    const Z i1 = {0.0, 1.0}, mi = {0.0, -1.0}, p1 = {1.0, 0.0}, m1 = {-1.0, 0.0};
    const int c1[4] = {3, 2, 1, 0}, c3[4] = {2, 3, 0, 1};
    const Z v1[4] = {mi, mi, i1, i1};
    const Z v2[4] = {p1, m1, m1, p1};
    const Z v3[4] = {mi, i1, i1, mi};
    const Z v4[4] = {m1, m1, m1, m1};
    g[0] = perm4(c1, v1);
    g[1] = perm4(c1, v2);
    g[2] = perm4(c3, v3);
    g[3] = perm4(c3, v4);
    g[4] = mul4(mul4(mul4(g[0], g[1]), g[2]), g[3]);
  }
};

const Gammas& gam() {
  static Gammas G;
  return G;
}

// rho interpolator j (1..4) in direction i (devTools/comb_rho.cpp:19-49):
// gamma_i, gamma_4 gamma_i, gamma_i, gamma_4 gamma_4 / 2 (the last two with the
// smeared / commutator elementals); "dag" flips the sign where the generator does.
Z rho_op(int j, int i, int r, int c, bool dag) {
  const Gammas& G = gam();
  switch (j) {
    case 1:
    case 3:
      return dag ? neg(G.g[i].m[r][c]) : G.g[i].m[r][c];
    case 2:
      return mul4(G.g[3], G.g[i]).m[r][c];
    default: {
      Z e = mul4(G.g[3], G.g[3]).m[r][c];
      return dag ? scale(-0.5, e) : scale(0.5, e);
    }
  }
}

// Elemental used by rho operator k (0..3) in direction i: plain, plain,
// smeared, commutator_i (devTools/comb_rho.cpp:52-74, comb_rhopi.cpp compute_ip).
int rho_elemental(int k, int i) { return k < 2 ? 0 : (k == 2 ? 1 : 2 + i); }

void store(float* dst, Z z) {
  dst[0] = (float)z.re;
  dst[1] = (float)z.im;
}

void build(Tables& T) {
  const Gammas& G = gam();
  const Spin4& g5 = G.g[4];
  int n = 0;
  // rho (devTools/comb_rho.cpp): op pair (l,k), direction i, 16 spin rows each
  for (int l = 0; l < 4; l++)
    for (int k = 0; k < 4; k++)
      for (int i = 0; i < 3; i++)
        for (int s = 0; s < 256; s++) {
          int s1 = s >> 6, s2 = (s >> 4) & 3, s3 = (s >> 2) & 3, s4 = s & 3;
          Z a = rho_op(k + 1, i, s4, s2, true);
          if (l * 4 + k < 12) a = neg(a);
          Z c = a * g5.m[s2][s2] * g5.m[s1][s1] * rho_op(l + 1, i, s1, s3, false);
          if (!nonzero(c)) continue;
          int16_t* sp = T.rho_spin[n];
          sp[0] = s1; sp[1] = s2; sp[2] = s3; sp[3] = s4;
          T.rho_lprp[n][0] = rho_elemental(k, i);
          T.rho_lprp[n][1] = rho_elemental(l, i);
          store(T.rho_coef[n], c);
          n++;
        }
  // rho -> pi pi (devTools/comb_rhopi.cpp)
  n = 0;
  for (int idir = 0; idir < 3; idir++)
    for (int iop = 0; iop < 4; iop++)
      for (int s = 0; s < 4096; s++) {
        int sv[6];
        for (int q = 0; q < 6; q++) sv[q] = (s >> (2 * (5 - q))) & 3;
        Z c = rho_op(iop + 1, idir, sv[3], sv[4], false) * g5.m[sv[2]][sv[3]] * g5.m[sv[5]][sv[0]];
        if (!nonzero(c)) continue;
        for (int q = 0; q < 6; q++) T.rhopi_spin[n][q] = sv[q];
        T.rhopi_ip[n] = rho_elemental(iop, idir);
        store(T.rhopi_coef[n], c);
        n++;
      }
  // pi pi square and double triangle (devTools/comb_pipi.cpp)
  int nsq = 0, ndt = 0;
  for (int s = 0; s < 4096; s++) {
    int sv[6];
    for (int q = 0; q < 6; q++) sv[q] = (s >> (2 * (5 - q))) & 3;
    Z c = g5.m[sv[3]][sv[4]] * g5.m[sv[5]][sv[0]];
    if (nonzero(c)) {
      for (int q = 0; q < 6; q++) T.sq_spin[nsq][q] = sv[q];
      store(T.sq_coef[nsq], c);
      nsq++;
    }
    c = g5.m[sv[1]][sv[2]] * g5.m[sv[5]][sv[0]];
    if (nonzero(c)) {
      for (int q = 0; q < 6; q++) T.dt_spin[ndt][q] = sv[q];
      store(T.dt_coef[ndt], c);
      ndt++;
    }
  }
  for (int s = 0; s < 256; s++) {
    for (int q = 0; q < 4; q++) T.dth_spin[s][q] = (s >> (2 * (3 - q))) & 3;
    store(T.dth_coef[s], Z{1.0, 0.0});
  }
  // sigma one-fish (devTools/comb_sigma.cpp)
  n = 0;
  for (int l = 0; l < 2; l++)
    for (int k = 0; k < 2; k++)
      for (int s = 0; s < 256; s++) {
        int s1 = s >> 6, s2 = (s >> 4) & 3, s3 = (s >> 2) & 3, s4 = s & 3;
        Z c = g5.m[s2][s3] * g5.m[s4][s1];
        if (!nonzero(c)) continue;
        T.sigma_spin[n][0] = s1; T.sigma_spin[n][1] = s2; T.sigma_spin[n][2] = s3; T.sigma_spin[n][3] = s4;
        T.sigma_lprp[n][0] = l;
        T.sigma_lprp[n][1] = k;
        store(T.sigma_coef[n], c);
        n++;
      }
  // sigma -> pi pi (devTools/comb_sigmapi.cpp)
  for (int s = 0; s < 16; s++) {
    T.hf_spin[s][0] = s >> 2;
    T.hf_spin[s][1] = s & 3;
    store(T.hf_coef[s], Z{1.0, 0.0});
  }
  n = 0;
  for (int ik = 0; ik < 2; ik++)
    for (int s = 0; s < 1024; s++) {
      int sv[5];
      for (int q = 0; q < 5; q++) sv[q] = (s >> (2 * (4 - q))) & 3;
      Z c = g5.m[sv[0]][sv[1]] * g5.m[sv[2]][sv[3]];
      if (!nonzero(c)) continue;
      for (int q = 0; q < 5; q++) T.tri_spin[n][q] = sv[q];
      T.tri_ip[n] = ik;
      store(T.tri_coef[n], c);
      n++;
    }
}

}  // namespace

const Tables& tables() {
  static Tables* T = [] {
    Tables* t = new Tables;
    std::memset(t, 0, sizeof(Tables));
    build(*t);
    return t;
  }();
  return *T;
}

}  // namespace ctr

extern "C" {

int ctr_table_rho(int16_t* spin, int16_t* lp_rp, float* coef) {
  if (!spin || !lp_rp || !coef) return ctr::fail(CTR_ERR_ARG, "ctr_table_rho: null pointer");
  const ctr::Tables& T = ctr::tables();
  std::memcpy(spin, T.rho_spin, sizeof(T.rho_spin));
  std::memcpy(lp_rp, T.rho_lprp, sizeof(T.rho_lprp));
  std::memcpy(coef, T.rho_coef, sizeof(T.rho_coef));
  return CTR_OK;
}

int ctr_table_rhopi(int16_t* spin, int16_t* ip, float* coef) {
  if (!spin || !ip || !coef) return ctr::fail(CTR_ERR_ARG, "ctr_table_rhopi: null pointer");
  const ctr::Tables& T = ctr::tables();
  std::memcpy(spin, T.rhopi_spin, sizeof(T.rhopi_spin));
  std::memcpy(ip, T.rhopi_ip, sizeof(T.rhopi_ip));
  std::memcpy(coef, T.rhopi_coef, sizeof(T.rhopi_coef));
  return CTR_OK;
}

int ctr_table_pipi(int16_t* sq_spin, float* sq_coef, int16_t* dt_spin, float* dt_coef, int16_t* dth_spin,
                   float* dth_coef) {
  if (!sq_spin || !sq_coef || !dt_spin || !dt_coef || !dth_spin || !dth_coef)
    return ctr::fail(CTR_ERR_ARG, "ctr_table_pipi: null pointer");
  const ctr::Tables& T = ctr::tables();
  std::memcpy(sq_spin, T.sq_spin, sizeof(T.sq_spin));
  std::memcpy(sq_coef, T.sq_coef, sizeof(T.sq_coef));
  std::memcpy(dt_spin, T.dt_spin, sizeof(T.dt_spin));
  std::memcpy(dt_coef, T.dt_coef, sizeof(T.dt_coef));
  std::memcpy(dth_spin, T.dth_spin, sizeof(T.dth_spin));
  std::memcpy(dth_coef, T.dth_coef, sizeof(T.dth_coef));
  return CTR_OK;
}

int ctr_table_sigma(int16_t* spin, int16_t* lp_rp, float* coef) {
  if (!spin || !lp_rp || !coef) return ctr::fail(CTR_ERR_ARG, "ctr_table_sigma: null pointer");
  const ctr::Tables& T = ctr::tables();
  std::memcpy(spin, T.sigma_spin, sizeof(T.sigma_spin));
  std::memcpy(lp_rp, T.sigma_lprp, sizeof(T.sigma_lprp));
  std::memcpy(coef, T.sigma_coef, sizeof(T.sigma_coef));
  return CTR_OK;
}

int ctr_table_sigmapi(int16_t* hf_spin, float* hf_coef, int16_t* tri_spin, int16_t* tri_ip, float* tri_coef) {
  if (!hf_spin || !hf_coef || !tri_spin || !tri_ip || !tri_coef)
    return ctr::fail(CTR_ERR_ARG, "ctr_table_sigmapi: null pointer");
  const ctr::Tables& T = ctr::tables();
  std::memcpy(hf_spin, T.hf_spin, sizeof(T.hf_spin));
  std::memcpy(hf_coef, T.hf_coef, sizeof(T.hf_coef));
  std::memcpy(tri_spin, T.tri_spin, sizeof(T.tri_spin));
  std::memcpy(tri_ip, T.tri_ip, sizeof(T.tri_ip));
  std::memcpy(tri_coef, T.tri_coef, sizeof(T.tri_coef));
  return CTR_OK;
}

}  // extern "C"
