// Momentum elementals from Laplacian eigenvectors: the loops of the reference
// drivers (tests/compute_rho.cpp:116-201; the same construction in
// tests/compute_{rhopi,pipi_I0,pipi_I1,sigma,sigmapi}.cpp), which build, per time
// slice t and momentum p,
//   plain     Phi_0(t)_{rc} = <v_r| e^{-ip.x} |v_c>                     (:116-130)
//   smeared   Phi_1(t)_{rc} = sum_j <D_j v_r| e^{-ip.x} |D_j v_c>        (:132-163)
//   commutator Phi_{2+j}(t)_{rc} = <v_r| e^{-ip.x} |D_j v_c> - <D_j v_r| e^{-ip.x} |v_c>   (:165-201)
// with <a|b> = sum over the sites of the slice and the three colours of
// conj(a) b, and the phase e^{-i 2 pi (x p_x / n_x + y p_y / n_y + z p_z / n_z)}.
//
// On the GPU every elemental is one task of a batched FP64 kernel
//   out = sum_q w_q X_q^dag diag(phase_p) Y_q,   w_q = +-1,  q < 3,
// over K = 3 * sites (rows of X_q, Y_q are eigenvectors, or their covariant
// derivatives), so the five operators of a (t, p) need 10 products and no
// intermediate output.  The covariant derivative D_j v(x) = U_j(x) v(x + j) -
// U_j(x - j)^dag v(x - j) (periodic) is a stencil kernel; the reference takes it
// from the gwu-qcd library (lapmult::covderiv), which is not part of its
// sources, so the derivative operators follow this stated definition.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"

namespace ctr {

namespace {

struct ElTask {
  const double2* x[3];
  const double2* y[3];
  double w[3];
  int nterm;
  int p;  // momentum index into the phase table
  double2* out;
};

// phase[p][s] = exp(-i 2 pi n / V) with n = (x p_x n_y n_z + y p_y n_x n_z + z p_z n_x n_y) mod V,
// V = n_x n_y n_z (integer reduction, then one sincospi per site)
__global__ void el_phase_kernel(const int* __restrict__ mom, int nmom, int nx, int ny, int nz,
                                double2* __restrict__ phase) {
  const long long V = (long long)nx * ny * nz;
  const long long n = (long long)nmom * V;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    const int p = (int)(g / V);
    const long long s = g - p * V;
    const int x = (int)(s % nx), y = (int)((s / nx) % ny), z = (int)(s / ((long long)nx * ny));
    long long m = ((long long)x * mom[3 * p] * ny * nz + (long long)y * mom[3 * p + 1] * nx * nz +
                   (long long)z * mom[3 * p + 2] * nx * ny) % V;
    if (m < 0) m += V;
    double sn, cs;
    sincospi(-2.0 * (double)m / (double)V, &sn, &cs);
    phase[g] = make_double2(cs, sn);
  }
}

// dv[j][t][c][s][a] = sum_b U_j(s)_{ab} v[t][c][s + j][b] - sum_b conj(U_j(s - j)_{ba}) v[t][c][s - j][b]
__global__ void el_covderiv_kernel(const double2* __restrict__ v, const double2* __restrict__ links, int nev, int nt,
                                   int nx, int ny, int nz, double2* __restrict__ dv) {
  const long long V = (long long)nx * ny * nz;
  const long long n = 3LL * nt * nev * V;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    long long r = g;
    const long long s = r % V;
    r /= V;
    const int c = (int)(r % nev);
    r /= nev;
    const int t = (int)(r % nt), j = (int)(r / nt);
    const int x = (int)(s % nx), y = (int)((s / nx) % ny), z = (int)(s / ((long long)nx * ny));
    int xp = x, yp = y, zp = z, xm = x, ym = y, zm = z;
    if (j == 0) {
      xp = x + 1 == nx ? 0 : x + 1;
      xm = x == 0 ? nx - 1 : x - 1;
    } else if (j == 1) {
      yp = y + 1 == ny ? 0 : y + 1;
      ym = y == 0 ? ny - 1 : y - 1;
    } else {
      zp = z + 1 == nz ? 0 : z + 1;
      zm = z == 0 ? nz - 1 : z - 1;
    }
    const long long sp = xp + (long long)nx * (yp + (long long)ny * zp);
    const long long sm = xm + (long long)nx * (ym + (long long)ny * zm);
    const double2* vt = v + ((size_t)t * nev + c) * V * 3;
    const double2* Lt = links + (size_t)t * V * 27;
    const double2* uf = Lt + ((size_t)s * 3 + j) * 9;   // U_j(s)
    const double2* ub = Lt + ((size_t)sm * 3 + j) * 9;  // U_j(s - j)
    double2 vp[3], vm[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
      vp[b] = vt[sp * 3 + b];
      vm[b] = vt[sm * 3 + b];
    }
    double2* o = dv + (((size_t)j * nt + t) * nev + c) * V * 3 + s * 3;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      double re = 0.0, im = 0.0;
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const double2 f = uf[a * 3 + b], u = ub[b * 3 + a];  // U_j(s)_{ab}, U_j(s-j)_{ba}
        re = fma(f.x, vp[b].x, re);
        re = fma(-f.y, vp[b].y, re);
        im = fma(f.x, vp[b].y, im);
        im = fma(f.y, vp[b].x, im);
        // - conj(u) vm[b]
        re = fma(-u.x, vm[b].x, re);
        re = fma(-u.y, vm[b].y, re);
        im = fma(-u.x, vm[b].y, im);
        im = fma(u.y, vm[b].x, im);
      }
      o[a] = make_double2(re, im);
    }
  }
}

// One CTA per (TE x TE output tile, task): out[r][c] = sum_q w_q sum_k conj(X_q[r][k]) ph[k / 3] Y_q[c][k].
// Thread (tx, ty) owns rows tx + TX a (a < RX) and columns ty + TY b (b < RY); K
// is staged KC at a time in shared memory, the phase and weight applied to Y as
// it is staged.  FP64 FMAs only in the product (the FP64 pipe is the bound).
template <int TE, int RX, int RY>
__global__ void __launch_bounds__((TE / RX) * (TE / RY)) el_gemm_kernel(const ElTask* __restrict__ tasks, int nev,
                                                                          long long K,
                                                                          const double2* __restrict__ phase,
                                                                          long long V) {
  constexpr int TX = TE / RX, TY = TE / RY, NTH = TX * TY, KC = 8;
  __shared__ double2 xs[KC][TE + 1];
  __shared__ double2 ys[KC][TE + 1];
  const ElTask& T = tasks[blockIdx.y];
  const int nti = (nev + TE - 1) / TE;
  const int r0 = (blockIdx.x / nti) * TE, c0 = (blockIdx.x % nti) * TE;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const double2* ph = phase + (size_t)T.p * V;
  double2 acc[RX][RY];
#pragma unroll
  for (int a = 0; a < RX; a++)
#pragma unroll
    for (int b = 0; b < RY; b++) acc[a][b] = make_double2(0.0, 0.0);
  for (int q = 0; q < T.nterm; q++) {
    const double2* X = T.x[q];
    const double2* Y = T.y[q];
    const double w = T.w[q];
    for (long long k0 = 0; k0 < K; k0 += KC) {
      for (int e = threadIdx.x; e < TE * KC; e += NTH) {
        const int i = e / KC, kk = e - i * KC;  // consecutive threads along k
        const long long k = k0 + kk;
        const int r = r0 + i, c = c0 + i;
        xs[kk][i] = (r < nev && k < K) ? X[(size_t)r * K + k] : make_double2(0.0, 0.0);
        double2 y = make_double2(0.0, 0.0);
        if (c < nev && k < K) {
          const double2 yv = Y[(size_t)c * K + k], f = ph[k / 3];
          y = make_double2(w * (f.x * yv.x - f.y * yv.y), w * (f.x * yv.y + f.y * yv.x));
        }
        ys[kk][i] = y;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < KC; kk++) {
        double2 xv[RX], yv[RY];
#pragma unroll
        for (int a = 0; a < RX; a++) xv[a] = xs[kk][tx + TX * a];
#pragma unroll
        for (int b = 0; b < RY; b++) yv[b] = ys[kk][ty + TY * b];
#pragma unroll
        for (int a = 0; a < RX; a++)
#pragma unroll
          for (int b = 0; b < RY; b++) {
            // acc += conj(x) y
            acc[a][b].x = fma(xv[a].x, yv[b].x, acc[a][b].x);
            acc[a][b].x = fma(xv[a].y, yv[b].y, acc[a][b].x);
            acc[a][b].y = fma(xv[a].x, yv[b].y, acc[a][b].y);
            acc[a][b].y = fma(-xv[a].y, yv[b].x, acc[a][b].y);
          }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int a = 0; a < RX; a++)
#pragma unroll
    for (int b = 0; b < RY; b++) {
      const int r = r0 + tx + TX * a, c = c0 + ty + TY * b;
      if (r < nev && c < nev) T.out[(size_t)r * nev + c] = acc[a][b];
    }
}

template <int TE, int RX, int RY>
int launch_el_gemm(const ElTask* d_tasks, int ntask, int nev, long long K, const double2* phase, long long V,
                   cudaStream_t s) {
  const int nti = (nev + TE - 1) / TE;
  for (int t0 = 0; t0 < ntask; t0 += 65535) {  // grid.y limit
    const int nb = std::min(65535, ntask - t0);
    TimedLaunch tl(s, "el_gemm");
    el_gemm_kernel<TE, RX, RY><<<dim3(nti * nti, nb), (TE / RX) * (TE / RY), 0, s>>>(d_tasks + t0, nev, K, phase, V);
    CTR_CUDA(cudaGetLastError());
  }
  return CTR_OK;
}

}  // namespace

}  // namespace ctr

using namespace ctr;

int ctr_elementals(int nev, int nt, int nx, int ny, int nz, const double* evec, const double* links, int nmom,
                   const int* mom, int nops, double* phi, void* stream) {
  if (nev < 1 || nt < 1 || nx < 1 || ny < 1 || nz < 1 || nmom < 1 || !mom || !evec || !phi)
    return fail(CTR_ERR_ARG, "ctr_elementals: bad arguments");
  if (nops != 1 && nops != 5) return fail(CTR_ERR_ARG, "ctr_elementals: nops must be 1 or 5 (got %d)", nops);
  if (nops == 5 && !links) return fail(CTR_ERR_ARG, "ctr_elementals: the derivative operators need the gauge links");
  if ((((uintptr_t)evec | (uintptr_t)links | (uintptr_t)phi) & 15))
    return fail(CTR_ERR_ARG, "ctr_elementals: device pointers must be 16-byte aligned");
  const long long V = (long long)nx * ny * nz, K = 3 * V;
  if (V > (1LL << 31) / 3) return fail(CTR_ERR_ARG, "ctr_elementals: %lld sites is too many", V);
  cudaStream_t s = (cudaStream_t)stream;
  const double2* v = (const double2*)evec;
  const size_t vbytes = (size_t)nt * nev * K * sizeof(double2);
  // scratch: phase table, then (nops == 5) the three covariant derivatives of every eigenvector
  void* mem;
  const size_t ph_bytes = ((size_t)nmom * V * sizeof(double2) + 255) & ~(size_t)255;
  CTR_TRY(workspace(WS_SCRATCH).get(ph_bytes + (nops == 5 ? 3 * vbytes : 0), &mem));
  double2* phase = (double2*)mem;
  double2* dv = (double2*)((uint8_t*)mem + ph_bytes);
  void* d_mom;
  CTR_TRY(upload(WS_MISC, mom, (size_t)nmom * 3 * sizeof(int), &d_mom, s));
  {
    TimedLaunch tl(s, "el_phase");
    const long long n = nmom * V;
    el_phase_kernel<<<(int)std::min<long long>((n + 255) / 256, 65535), 256, 0, s>>>((const int*)d_mom, nmom, nx, ny,
                                                                                       nz, phase);
    CTR_CUDA(cudaGetLastError());
  }
  if (nops == 5) {
    TimedLaunch tl(s, "el_covderiv");
    const long long n = 3LL * nt * nev * V;
    el_covderiv_kernel<<<(int)std::min<long long>((n + 255) / 256, 1 << 20), 256, 0, s>>>(
        v, (const double2*)links, nev, nt, nx, ny, nz, dv);
    CTR_CUDA(cudaGetLastError());
  }
  // tasks: per (p, op, t) the output block phi[p][op][t] (the drivers' layout)
  auto vec = [&](int t) { return v + (size_t)t * nev * K; };
  auto dvec = [&](int j, int t) { return dv + ((size_t)j * nt + t) * nev * K; };
  std::vector<ElTask> tasks;
  tasks.reserve((size_t)nmom * nops * nt);
  for (int p = 0; p < nmom; p++)
    for (int op = 0; op < nops; op++)
      for (int t = 0; t < nt; t++) {
        ElTask T;
        std::memset(&T, 0, sizeof(T));
        T.p = p;
        T.out = (double2*)phi + (((size_t)p * nops + op) * nt + t) * nev * nev;
        if (op == 0) {  // <v_r| e^{-ip.x} |v_c>
          T.nterm = 1;
          T.x[0] = vec(t);
          T.y[0] = vec(t);
          T.w[0] = 1.0;
        } else if (op == 1) {  // sum_j <D_j v_r| e^{-ip.x} |D_j v_c>
          T.nterm = 3;
          for (int j = 0; j < 3; j++) {
            T.x[j] = dvec(j, t);
            T.y[j] = dvec(j, t);
            T.w[j] = 1.0;
          }
        } else {  // <v_r| e^{-ip.x} |D_j v_c> - <D_j v_r| e^{-ip.x} |v_c>
          const int j = op - 2;
          T.nterm = 2;
          T.x[0] = vec(t);
          T.y[0] = dvec(j, t);
          T.w[0] = 1.0;
          T.x[1] = dvec(j, t);
          T.y[1] = vec(t);
          T.w[1] = -1.0;
        }
        tasks.push_back(T);
      }
  void* d_tasks;
  CTR_TRY(upload(WS_TASKS, tasks.data(), tasks.size() * sizeof(ElTask), &d_tasks, s));
  const int ntask = (int)tasks.size();
  // output tile edge: 50 (250 threads, 5 x 2 outputs each) where it pads Nev least, else 32 (256 threads, 2 x 2)
  const int pad50 = ((nev + 49) / 50) * 50 - nev, pad32 = ((nev + 31) / 32) * 32 - nev;
  if (nev >= 50 && pad50 <= pad32)
    return launch_el_gemm<50, 5, 2>((const ElTask*)d_tasks, ntask, nev, K, phase, V, s);
  return launch_el_gemm<32, 2, 2>((const ElTask*)d_tasks, ntask, nev, K, phase, V, s);
}
