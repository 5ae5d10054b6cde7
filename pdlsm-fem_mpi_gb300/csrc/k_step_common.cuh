// Device helpers shared by the FP64 and mixed-precision step kernels
// (k_step.cu, k_step_mixed.cu).
//
// Work split of a step launch: blocks [0, pd_blocks) take the PD families
// (LP lanes per family), the remaining blocks take the FE-only nodes (LF lanes
// per node).  Each work item computes the full internal force of its node's
// rows, so every row has exactly one writer and no atomics or force arrays
// are needed:
//   f_k = sum_bonds (C_km + P_km) (u_m - u_k)       PD + PD-boundary terms of family k
//       - sum_{FE e around k} Ke[rows of k] u_e      FE terms
//       + f_ext                                      traction BCs
// followed by the central-difference update of the node's active DOFs
// (timeIntegration_LM, pdsolve.cpp:5113-5132; first step :6010-6012) and the
// new value of its prescribed DOFs (setVaryEssentialBC :5263-5312).  The
// update runs in FP64 with one DOF per lane of the warp (the items of a warp
// are gathered by shuffles), so the narrow FP64 pipe sees full warps.
#pragma once

#include "device.h"

namespace pdx {
namespace step {

constexpr unsigned kFull = 0xffffffffu;

// Per-bond draw of the perturbed critical stretch: murmur3's 32-bit finaliser
// of (k, m, seed); U = top 24 bits / 2^24 is exact in FP32 and FP64.
__device__ __forceinline__ uint32_t bond_hash(uint32_t seed, int k, int m) {
  uint32_t x = ((uint32_t)k * 0x9e3779b1u) ^ ((uint32_t)m + 0x7f4a7c15u) ^ seed;
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ double bond_s0(const DevView& v, uint32_t h) {
  if (v.s0_pert == 0.0) return v.s0;
  return v.s0 * (1.0 + v.s0_pert * (2.0 * ((double)(h >> 8) * 0x1.0p-24) - 1.0));
}

__device__ __forceinline__ float bond_s0_f32(float s0, float pert, uint32_t h) {
  if (pert == 0.f) return s0;
  return s0 * (1.f + pert * (2.f * ((float)(h >> 8) * 0x1.0p-24f) - 1.f));
}

// The reference's stretch expression, s = |xi + eta| / |xi| - 1 > s0 (failureCriterion_stretch).
template <int D>
__device__ __forceinline__ bool stretch_over_fp64(const DevView& v, const double* u, int k, int m, uint32_t h) {
  double xi[3] = {0, 0, 0}, eta[3] = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 3; i++) xi[i] = v.X[3 * m + i] - v.X[3 * k + i];
#pragma unroll
  for (int i = 0; i < D; i++) eta[i] = u[(int64_t)m * D + i] - u[(int64_t)k * D + i];
  const double mag_ref = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
  const double mag = sqrt((xi[0] + eta[0]) * (xi[0] + eta[0]) + (xi[1] + eta[1]) * (xi[1] + eta[1]) +
                          (xi[2] + eta[2]) * (xi[2] + eta[2]));
  const double s = mag / mag_ref - 1.0;
  return s > bond_s0(v, h);
}

template <int D, int L, typename T>
__device__ __forceinline__ void warp_sum(T* acc) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < D; i++) acc[i] += __shfl_xor_sync(kFull, acc[i], o);
}

// Displacement of node n as the force sees it: stored value, plus this step's
// increment for varying prescribed DOFs.
template <int D>
struct LoadFp64 {
  const double* u;
  const uint8_t* bcflag;
  const double* dtv;
  __device__ __forceinline__ void operator()(int n, double* out) const {
    const unsigned fl = bcflag[n];
#pragma unroll
    for (int i = 0; i < D; i++) {
      const double c = u[(int64_t)n * D + i];
      out[i] = (fl >> i) & 1u ? c + dtv[3 * n + i] : c;
    }
  }
};

// Same from the FP32 node records ([2n+1] = displacement + varying-BC bits).
template <int D>
struct LoadMixed {
  const float4* nr;
  const double* dtv;
  __device__ __forceinline__ void operator()(int n, float* out) const {
    const float4 q = nr[2 * n + 1];
    const unsigned fl = __float_as_uint(q.w);
    out[0] = q.x;
    out[1] = q.y;
    if (D == 3) out[D - 1] = q.z;
    if (fl) {
#pragma unroll
      for (int i = 0; i < D; i++)
        if ((fl >> i) & 1u) out[i] += (float)dtv[3 * n + i];
    }
  }
};

// FE contribution -Ke[rows of local node al] u_e.
template <int D, typename T, typename ULoad>
__device__ __forceinline__ void fe_rows(const DevView& v, const T* ke, int e, int al, const ULoad& uload, T* acc) {
  constexpr int NEN = D == 2 ? 4 : 8;
  constexpr int ND = NEN * D;
  const T* K = ke + (int64_t)v.fe_cls[e] * ND * ND + (al * D) * ND;
#pragma unroll
  for (int jn = 0; jn < NEN; jn++) {
    const int n = v.fe_conn[e * 8 + jn];
    T un[D];
    uload(n, un);
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int jj = 0; jj < D; jj++) acc[i] -= K[i * ND + jn * D + jj] * un[jj];
  }
}

template <int D, typename T>
__device__ __forceinline__ void corr_block(const T* corr, int64_t ncorr, int64_t slot, const T* du, T* acc) {
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int j = 0; j < D; j++) acc[i] += corr[(int64_t)(i * D + j) * ncorr + slot] * du[j];
}

// Lane 0 of every item holds F (internal + external force) and its node; the
// warp's lanes then take one (item, DOF) pair each for the FP64 update, in
// rounds of 32 / D items.
template <int D, int L, bool MIXED>
__device__ __forceinline__ void warp_update(const StepArgs& a, const double* F, int node_or_neg) {
  constexpr int IPW = 32 / L;                 // items per warp
  constexpr int IPR = 32 / D;                 // items per round
  constexpr int ROUNDS = (IPW + IPR - 1) / IPR;
  const DevView& v = a.v;
  const int t = threadIdx.x & 31;
  const int jr = t / D, i = t % D;
#pragma unroll
  for (int r = 0; r < ROUNDS; r++) {
    const int j = r * IPR + jr;
    const bool act = jr < IPR && j < IPW;
    const int src = (act ? j : 0) * L;
    double Fi = 0.0;
#pragma unroll
    for (int c = 0; c < D; c++) {
      const double x = __shfl_sync(kFull, F[c], src);
      if (c == i) Fi = x;
    }
    const int n = __shfl_sync(kFull, node_or_neg, src);
    float uf = 0.f;
    if (act && n >= 0) {
      const int64_t idx = (int64_t)n * D + i;
      const double un = a.u_n[idx];
      double unew;
      if (v.eq[idx] >= 0) {
        const double tempA = Fi * v.dt2m[n];
        unew = a.mode == 0 ? un + 0.5 * tempA : fma(2.0, un, tempA) - a.u_next[idx];
      } else {
        unew = (v.bcflag[n] >> i) & 1u ? un + v.dtv[3 * n + i] : un;
      }
      a.u_next[idx] = unew;
      uf = (float)unew;
    }
    if (MIXED) {
      const float c1 = __shfl_down_sync(kFull, uf, 1);
      const float c2 = __shfl_down_sync(kFull, uf, 2);
      if (act && n >= 0 && i == 0)
        a.uf_next[2 * n + 1] = make_float4(uf, c1, D == 3 ? c2 : 0.f, __uint_as_float((unsigned)v.bcflag[n]));
    }
  }
}

template <int D>
__device__ __forceinline__ void external_force(const StepArgs& a, int node, double* fext) {
  const DevView& v = a.v;
  if (v.ext_ptr && a.nbc_val) {
    for (int j = v.ext_ptr[node]; j < v.ext_ptr[node + 1]; j++) {
      const double t = a.nbc_val[v.ext_nbc[j]];
#pragma unroll
      for (int i = 0; i < D; i++) fext[i] += t * v.ext_f[3 * j + i];
    }
  }
}

// FE-only node item: element rows, then the update.  t = thread index within
// the FE part of the grid.
template <int D, int L, typename T, bool MIXED, typename ULoad>
__device__ __forceinline__ void feonly_item(const StepArgs& a, const T* ke, int64_t t, const ULoad& uload) {
  const DevView& v = a.v;
  const int item = (int)(t / L);
  const int lane = (int)(t % L);
  const bool valid = item < v.n_feonly;
  const int node = valid ? v.feonly_node[item] : 0;
  T acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = T(0);
  if (valid) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, T>(v, ke, ent >> 3, ent & 7, uload, acc);
    }
  }
  warp_sum<D, L>(acc);
  double F[D];
#pragma unroll
  for (int i = 0; i < D; i++) F[i] = (double)acc[i];
  if (lane == 0 && valid) external_force<D>(a, node, F);
  warp_update<D, L, MIXED>(a, F, valid ? node : -1);
}

}  // namespace step
}  // namespace pdx
