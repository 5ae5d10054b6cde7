// PDLSM bond coefficients, one warp per family, FP64.
//
// For family k with members m (bond vector xi = X_m - X_k):
//   A   = sum_m w_m P(xi) Q(xi)^T,  w_m = omega(xi) dv_m,
//         omega = exp(-|xi|^2 / (NLF^2 delta_k^2))           (inflFunc, pdsolve.cpp:1929-1935)
//   2D: P = [x, y, x^2, y^2, xy],  Q = [x, y, x^2/2, y^2/2, xy]                 (shapTens2D :1938-2013)
//   3D: P = [x,y,z,x^2,y^2,z^2,xy,yz,zx], Q = [x,y,z,x^2/2,y^2/2,z^2/2,xy,yz,zx] (shapTens3D :2015-2064)
//   [g; d] = A^{-1} P(xi) by LU with partial pivoting              (vec_gd2D/3D :2174-2232)
//   G = omega * Lame(d)  (symmetric d x d)                          (matG2D/3D :2277-2347)
// The reference refactorises A for every bond and every call; A does not
// depend on bond state, so it is factorised once per family here and every
// bond reuses the factors.  Outputs per bond (bond state 1):
//   coef = G dv_m dv_k            (the family-k row block of K_PD, matH + assembleInterWorkPD)
//   c    = omega g dv_m           (strain-operator column, matC2D/3D :3212-3398)
//   corr = -W_k D B(c)            (PD boundary element traction term, assemblePDBEwork*)
// A's entries are summed over the members in family order, as the reference does.
#include <cstdio>

#include "device.h"

namespace pdx {

namespace {

constexpr int kWarps = 4;

template <int D>
struct Poly;

template <>
struct Poly<2> {
  static constexpr int NA = 5;
  __device__ static double P(int r, const double* x) {
    switch (r) {
      case 0: return x[0];
      case 1: return x[1];
      case 2: return x[0] * x[0];
      case 3: return x[1] * x[1];
      default: return x[0] * x[1];
    }
  }
  __device__ static double Q(int c, const double* x) {
    switch (c) {
      case 0: return x[0];
      case 1: return x[1];
      case 2: return x[0] * x[0] * 0.5;
      case 3: return x[1] * x[1] * 0.5;
      default: return x[0] * x[1];
    }
  }
};

template <>
struct Poly<3> {
  static constexpr int NA = 9;
  __device__ static double P(int r, const double* x) {
    switch (r) {
      case 0: return x[0];
      case 1: return x[1];
      case 2: return x[2];
      case 3: return x[0] * x[0];
      case 4: return x[1] * x[1];
      case 5: return x[2] * x[2];
      case 6: return x[0] * x[1];
      case 7: return x[1] * x[2];
      default: return x[2] * x[0];
    }
  }
  __device__ static double Q(int c, const double* x) {
    switch (c) {
      case 0: return x[0];
      case 1: return x[1];
      case 2: return x[2];
      case 3: return x[0] * x[0] * 0.5;
      case 4: return x[1] * x[1] * 0.5;
      case 5: return x[2] * x[2] * 0.5;
      case 6: return x[0] * x[1];
      case 7: return x[1] * x[2];
      default: return x[0] * x[2];
    }
  }
};

__device__ __forceinline__ double influence(const double* xi, double aa, double delta) {
  return exp(-(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) / aa / delta / delta);
}

template <int D>
__global__ void __launch_bounds__(kWarps * 32) k_coeff(CoeffArgs a) {
  constexpr int NA = Poly<D>::NA;
  constexpr int NDV = D == 2 ? 3 : 6;
  constexpr int NV = D == 2 ? 3 : 6;
  constexpr int NC = D == 2 ? 3 : 6;   // symmetric coefficients
  __shared__ double sA[kWarps][NA][NA + 1];
  __shared__ int spiv[kWarps][NA];
  __shared__ int ssing[kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int f = blockIdx.x * kWarps + warp;
  if (f >= a.n_fam) return;
  const int k = a.fam_node[f];
  const int b0 = a.fam_ptr[f], b1 = a.fam_ptr[f + 1];
  const double xk[3] = {a.X[3 * k], a.X[3 * k + 1], a.X[3 * k + 2]};
  const double delta = a.fam_delta[f];
  const double aa = a.nlf * a.nlf;
  // moment matrix, entry-parallel, summed over members in order
  for (int e = lane; e < NA * NA; e += 32) {
    const int r = e / NA, c = e % NA;
    double s = 0.0;
    for (int b = b0; b < b1; b++) {
      const int m = a.nbr[b];
      const double xi[3] = {a.X[3 * m] - xk[0], a.X[3 * m + 1] - xk[1], a.X[3 * m + 2] - xk[2]};
      const double w = influence(xi, aa, delta) * a.vol[m];
      s += w * (Poly<D>::P(r, xi) * Poly<D>::Q(c, xi));
    }
    sA[warp][r][c] = s;
    if (a.A_out) a.A_out[(int64_t)f * NA * NA + e] = s;
  }
  __syncwarp();
  // LU with partial pivoting (LAPACK dgetf2 order: first largest pivot, scale by reciprocal)
  if (lane == 0) {
    int sing = 0;
    for (int j = 0; j < NA; j++) {
      int p = j;
      double best = fabs(sA[warp][j][j]);
      for (int r = j + 1; r < NA; r++) {
        const double v = fabs(sA[warp][r][j]);
        if (v > best) { best = v; p = r; }
      }
      spiv[warp][j] = p;
      if (best == 0.0) { sing = 1; break; }
      if (p != j)
        for (int c = 0; c < NA; c++) {
          const double t = sA[warp][j][c];
          sA[warp][j][c] = sA[warp][p][c];
          sA[warp][p][c] = t;
        }
      const double rp = 1.0 / sA[warp][j][j];
      for (int r = j + 1; r < NA; r++) {
        const double l = sA[warp][r][j] * rp;
        sA[warp][r][j] = l;
        for (int c = j + 1; c < NA; c++) sA[warp][r][c] -= l * sA[warp][j][c];
      }
    }
    ssing[warp] = sing;
    if (sing) atomicCAS(a.err, 0, 1 + f);
  }
  __syncwarp();
  if (ssing[warp]) return;
  const double lam = a.lambda, mu = a.mu;
  const double dvk = a.fam_cdv[f];
  const int corr0 = a.fam_corr ? a.fam_corr[f] : -1;
  const int wdi = a.fam_wd ? a.fam_wd[f] : -1;
  const double* WD = wdi >= 0 ? a.wd + (int64_t)wdi * D * NV : nullptr;
  for (int b = b0 + lane; b < b1; b += 32) {
    const int m = a.nbr[b];
    const double xi[3] = {a.X[3 * m] - xk[0], a.X[3 * m + 1] - xk[1], a.X[3 * m + 2] - xk[2]};
    double x[NA];
#pragma unroll
    for (int r = 0; r < NA; r++) x[r] = Poly<D>::P(r, xi);
#pragma unroll
    for (int j = 0; j < NA; j++) {
      const int p = spiv[warp][j];
      if (p != j) { const double t = x[j]; x[j] = x[p]; x[p] = t; }
    }
#pragma unroll
    for (int r = 1; r < NA; r++)
      for (int c = 0; c < r; c++) x[r] -= sA[warp][r][c] * x[c];
#pragma unroll
    for (int r = NA - 1; r >= 0; r--) {
      double s = x[r];
      for (int c = r + 1; c < NA; c++) s -= sA[warp][r][c] * x[c];
      x[r] = s / sA[warp][r][r];
    }
    const double omega = influence(xi, a.nlf * a.nlf, delta);
    const double dvm = a.vol[m];
    const double* dd = x + D;
    double G[D][D];
    if (D == 2) {
      G[0][0] = omega * ((2 * mu + lam) * dd[0] + mu * dd[1]);
      G[0][1] = omega * (lam + mu) * dd[2];
      G[1][0] = G[0][1];
      G[1][1] = omega * ((2 * mu + lam) * dd[1] + mu * dd[0]);
    } else {
      const double tr = dd[0] + dd[1] + dd[2];
      G[0][0] = omega * ((mu + lam) * dd[0] + mu * tr);
      G[0][1] = omega * (lam + mu) * dd[3];
      G[0][2] = omega * (lam + mu) * dd[5];
      G[1][1] = omega * ((mu + lam) * dd[1] + mu * tr);
      G[1][2] = omega * (lam + mu) * dd[4];
      G[2][2] = omega * ((mu + lam) * dd[2] + mu * tr);
      G[1][0] = G[0][1];
      G[2][0] = G[0][2];
      G[2][1] = G[1][2];
    }
    double cs[NC];
    if (D == 2) {
      cs[0] = G[0][0]; cs[1] = G[0][1]; cs[2] = G[1][1];
    } else {
      cs[0] = G[0][0]; cs[1] = G[0][1]; cs[2] = G[0][2]; cs[3] = G[1][1]; cs[4] = G[1][2]; cs[5] = G[2][2];
    }
#pragma unroll
    for (int i = 0; i < NC; i++) {
      const double v = (cs[i] * dvm) * dvk;
      a.coef64[(int64_t)i * a.n_bond + b] = v;
      if (a.coef32) a.coef32[(int64_t)i * a.n_bond + b] = (float)v;
    }
    double cv[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
      cv[i] = (omega * x[i]) * dvm;
      a.cvec[(int64_t)i * a.n_bond + b] = cv[i];
    }
    if (corr0 >= 0 && WD) {
      double P[D][D];
      if (D == 2) {
        for (int i = 0; i < 2; i++) {
          P[i][0] = -(WD[i * 3 + 0] * cv[0] + WD[i * 3 + 2] * cv[1]);
          P[i][1] = -(WD[i * 3 + 1] * cv[1] + WD[i * 3 + 2] * cv[0]);
        }
      } else {
        for (int i = 0; i < 3; i++) {
          const double* w = WD + i * 6;
          P[i][0] = -(w[0] * cv[0] + w[3] * cv[1] + w[5] * cv[2]);
          P[i][1] = -(w[1] * cv[1] + w[3] * cv[0] + w[4] * cv[2]);
          P[i][2] = -(w[2] * cv[2] + w[4] * cv[1] + w[5] * cv[0]);
        }
      }
      const int64_t slot = corr0 + (b - b0);
#pragma unroll
      for (int i = 0; i < D; i++)
#pragma unroll
        for (int j = 0; j < D; j++) {
          a.corr64[(int64_t)(i * D + j) * a.n_corr + slot] = P[i][j];
          // FP32 copy, one record per bond: 2D 4 floats; 3D 8 floats + the last in corr32_last
          const int idx = i * D + j;
          if (a.corr32) {
            if (D == 2) a.corr32[slot * 4 + idx] = (float)P[i][j];
            else if (idx < 8) a.corr32[slot * 8 + idx] = (float)P[i][j];
            else a.corr32_last[slot] = (float)P[i][j];
          }
        }
    }
    if (a.g_out)
      for (int i = 0; i < D; i++) a.g_out[(int64_t)b * D + i] = x[i];
    if (a.d_out)
      for (int i = 0; i < NDV; i++) a.d_out[(int64_t)b * NDV + i] = dd[i];
    if (a.G_out)
      for (int i = 0; i < D; i++)
        for (int j = 0; j < D; j++) a.G_out[(int64_t)b * D * D + i * D + j] = G[i][j];
  }
}

}  // namespace

cudaError_t launch_coeff(const CoeffArgs& a, cudaStream_t s) {
  if (a.n_fam == 0) return cudaSuccess;
  const int blocks = (a.n_fam + kWarps - 1) / kWarps;
  if (a.dim == 2) k_coeff<2><<<blocks, kWarps * 32, 0, s>>>(a);
  else k_coeff<3><<<blocks, kWarps * 32, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pdx
