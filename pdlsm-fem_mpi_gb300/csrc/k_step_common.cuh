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

#include <type_traits>

#include "device.h"
#include "fp_bits.cuh"

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

__device__ __forceinline__ double bond_s0(double s0, double pert, uint32_t h) {
  if (pert == 0.0) return s0;
  return s0 * (1.0 + pert * (2.0 * ((double)(h >> 8) * 0x1.0p-24) - 1.0));
}

__device__ __forceinline__ float bond_s0_f32(float s0, float pert, uint32_t h) {
  if (pert == 0.f) return s0;
  return s0 * (1.f + pert * (2.f * ((float)(h >> 8) * 0x1.0p-24f) - 1.f));
}

// The reference's stretch expression, s = |xi + eta| / |xi| - 1 > s_c (failureCriterion_stretch).
template <int D>
__device__ __forceinline__ bool stretch_over_fp64(const DevView& v, const double* u, int k, int m, double sc) {
  double xi[3] = {0, 0, 0}, eta[3] = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 3; i++) xi[i] = v.X[3 * m + i] - v.X[3 * k + i];
#pragma unroll
  for (int i = 0; i < D; i++) eta[i] = u[(int64_t)m * D + i] - u[(int64_t)k * D + i];
  const double mag_ref = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
  const double mag = sqrt((xi[0] + eta[0]) * (xi[0] + eta[0]) + (xi[1] + eta[1]) * (xi[1] + eta[1]) +
                          (xi[2] + eta[2]) * (xi[2] + eta[2]));
  const double s = mag / mag_ref - 1.0;
  return s > sc;
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
template <int D, int L>
struct UpdateOperands {
  static constexpr int IPW = 32 / L;          // items per warp
  static constexpr int IPR = 32 / D;          // items per round
  static constexpr int ROUNDS = (IPW + IPR - 1) / IPR;
  int n[ROUNDS];                              // node of this lane's (item, DOF) pair, -1 none
  unsigned flag[ROUNDS];                      // bcflag: bit i varying prescribed, bit 4 + i prescribed
  double un[ROUNDS], prev[ROUNDS], dt2m[ROUNDS];
  float dt2mf[ROUNDS];                        // mixed kernels: dt^2 / m in FP32
};

// Loads what the update of this lane's (item, DOF) pairs needs; it depends
// only on the items' nodes, so it can be issued before the force is known.
template <int D, int L, bool MIXED = false>
__device__ __forceinline__ void update_prefetch(const StepArgs& a, int node_or_neg, UpdateOperands<D, L>& o) {
  using O = UpdateOperands<D, L>;
  const DevView& v = a.v;
  const int t = threadIdx.x & 31;
  const int jr = t / D, i = t % D;
#pragma unroll
  for (int r = 0; r < O::ROUNDS; r++) {
    const int j = r * O::IPR + jr;
    const bool act = jr < O::IPR && j < O::IPW;
    const int n = __shfl_sync(kFull, node_or_neg, (act ? j : 0) * L);
    o.n[r] = act ? n : -1;
    o.flag[r] = 0;
    o.un[r] = o.prev[r] = o.dt2m[r] = 0.0;
    o.dt2mf[r] = 0.f;
    if (o.n[r] >= 0) {
      const int64_t idx = (int64_t)n * D + i;
      o.un[r] = a.u_n[idx];
      o.prev[r] = a.u_next[idx];
      if (MIXED) o.dt2mf[r] = v.dt2m_f[n];
      else o.dt2m[r] = v.dt2m[n];
      o.flag[r] = v.bcflag[n];
    }
  }
}

// Central-difference update of the active DOFs and the next value of the
// varying prescribed ones; the mixed kernel also writes the node record.
// F: FP64 forces (FP64 kernels) or FP32 forces (mixed kernels).  The mixed
// update forms dt^2 F / m in FP32 (the force is FP32 already) and accumulates
// it into the FP64 state as (2 u_n - u_{n-1}) + dt^2 F / m.
template <int D, int L, bool MIXED, typename FT>
__device__ __forceinline__ void update_apply(const StepArgs& a, const UpdateOperands<D, L>& o, const FT* F) {
  using O = UpdateOperands<D, L>;
  const int t = threadIdx.x & 31;
  const int jr = t / D, i = t % D;
#pragma unroll
  for (int r = 0; r < O::ROUNDS; r++) {
    const int j = r * O::IPR + jr;
    const int src = (jr < O::IPR && j < O::IPW ? j : 0) * L;
    FT Fi = FT(0);
#pragma unroll
    for (int c = 0; c < D; c++) {
      const FT x = __shfl_sync(kFull, F[c], src);
      if (c == i) Fi = x;
    }
    const int n = o.n[r];
    float uf = 0.f;
    if (n >= 0) {
      double unew;
      if (!((o.flag[r] >> (4 + i)) & 1u)) {
        if constexpr (MIXED) {
          const float tA = (float)Fi * o.dt2mf[r];
          unew = a.mode == 0 ? o.un[r] + f2d_bits(0.5f * tA) : fma(2.0, o.un[r], -o.prev[r]) + f2d_bits(tA);
        } else {
          const double tempA = (double)Fi * o.dt2m[r];
          unew = a.mode == 0 ? o.un[r] + 0.5 * tempA : fma(2.0, o.un[r], tempA) - o.prev[r];
        }
      } else {
        unew = (o.flag[r] >> i) & 1u ? o.un[r] + a.v.dtv[3 * n + i] : o.un[r];
      }
      a.u_next[(int64_t)n * D + i] = unew;
      uf = MIXED ? d2f_bits(unew) : (float)unew;
    }
    if (MIXED) {
      const float c1 = __shfl_down_sync(kFull, uf, 1);
      const float c2 = __shfl_down_sync(kFull, uf, 2);
      if (n >= 0 && i == 0)
        a.uf_next[2 * n + 1] = make_float4(uf, c1, D == 3 ? c2 : 0.f, __uint_as_float(o.flag[r]));
    }
  }
}

template <int D, int L, bool MIXED, typename FT>
__device__ __forceinline__ void warp_update(const StepArgs& a, const FT* F, int node_or_neg) {
  UpdateOperands<D, L> o;
  update_prefetch<D, L, MIXED>(a, node_or_neg, o);
  update_apply<D, L, MIXED>(a, o, F);
}

template <int D, typename FT>
__device__ __forceinline__ void external_force(const StepArgs& a, int node, FT* fext) {
  const DevView& v = a.v;
  if (v.ext_ptr && a.nbc_val) {
    for (int j = v.ext_ptr[node]; j < v.ext_ptr[node + 1]; j++) {
      const double t = a.nbc_val[v.ext_nbc[j]];
#pragma unroll
      for (int i = 0; i < D; i++) fext[i] += (FT)(t * v.ext_f[3 * j + i]);
    }
  }
}

// Stencil rows of an FE-only node: -sum_s K_s u_{nbr_s} over the node's
// neighbour slots; K_s are the assembled D x D blocks of the node's stencil
// class (st_blk32: 12 floats per 3D block, 4 per 2D block; st_blk64: D*D
// doubles).  All of a lane's slots are issued before any is used.
template <int D, int L, typename T, typename ULoad>
__device__ __forceinline__ void stencil_rows(const DevView& v, int item, int node, int cls, int dcls, int lane,
                                             const ULoad& uload, T* acc) {
  constexpr int S = D == 2 ? kStencil2 : kStencil3;
  constexpr int NS = (S + L - 1) / L;
  int j[NS];
  if (v.st_delta) {
    const int* dl = v.st_delta + (int64_t)dcls * S;
#pragma unroll
    for (int q = 0; q < NS; q++) {
      const int s = q * L + lane;
      const int d = s < S ? __ldg(dl + s) : INT32_MIN;
      j[q] = d == INT32_MIN ? -1 : node + d;
    }
  } else {
    const int* nb = v.st_nbr + (int64_t)item * S;
#pragma unroll
    for (int q = 0; q < NS; q++) {
      const int s = q * L + lane;
      j[q] = s < S ? nb[s] : -1;
    }
  }
#pragma unroll
  for (int q = 0; q < NS; q++) {
    if (j[q] < 0) continue;
    const int s = q * L + lane;
    T un[D];
    uload(j[q], un);
    if constexpr (std::is_same<T, float>::value) {
      if (D == 3) {
        const float4* B = reinterpret_cast<const float4*>(v.st_blk32) + ((int64_t)cls * S + s) * 3;
        const float4 b0 = __ldg(B), b1 = __ldg(B + 1), b2 = __ldg(B + 2);
        acc[0] -= b0.x * un[0] + b0.y * un[1] + b0.z * un[D - 1];
        acc[1] -= b0.w * un[0] + b1.x * un[1] + b1.y * un[D - 1];
        acc[D - 1] -= b1.z * un[0] + b1.w * un[1] + b2.x * un[D - 1];
      } else {
        const float4 b0 = __ldg(reinterpret_cast<const float4*>(v.st_blk32) + ((int64_t)cls * S + s));
        acc[0] -= b0.x * un[0] + b0.y * un[1];
        acc[1] -= b0.z * un[0] + b0.w * un[1];
      }
    } else {
      const double* B = v.st_blk64 + ((int64_t)cls * S + s) * D * D;
#pragma unroll
      for (int i = 0; i < D; i++)
#pragma unroll
        for (int c = 0; c < D; c++) acc[i] -= __ldg(B + i * D + c) * un[c];
    }
  }
}

// FE-only node item: stencil (or element) rows, then the update, whose
// operands are requested before the force.  t = thread index within the FE
// part of the grid.
// rest: optional list of the FE-only items to take (n_items entries), else
// items 0 .. n_feonly - 1.
template <int D, int L, typename T, bool MIXED, typename ULoad>
__device__ __forceinline__ void feonly_item(const StepArgs& a, const T* ke, int64_t t, const ULoad& uload,
                                            const int* rest = nullptr, int n_items = -1) {
  const DevView& v = a.v;
  const int pick = (int)(t / L);
  const int lane = (int)(t % L);
  const bool valid = pick < (rest ? n_items : v.n_feonly);
  const int item = rest ? (valid ? rest[pick] : 0) : pick;
  const int node = valid ? v.feonly_node[item] : 0;
  const int cls = valid && v.st_cls ? v.st_cls[item] : -1;
  const int dcls = valid && v.st_delta ? v.st_dcls[item] : 0;
  UpdateOperands<D, L> o;
  update_prefetch<D, L, MIXED>(a, valid ? node : -1, o);
  T acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = T(0);
  if (valid) {
    if (cls >= 0) {
      stencil_rows<D, L, T>(v, item, node, cls, dcls, lane, uload, acc);
    } else {
      const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
      for (int j = j0 + lane; j < j1; j += L) {
        const int ent = v.fe_adj[j];
        fe_rows<D, T>(v, ke, ent >> 3, ent & 7, uload, acc);
      }
    }
  }
  warp_sum<D, L>(acc);
  using FT = typename std::conditional<MIXED, float, double>::type;
  FT F[D];
#pragma unroll
  for (int i = 0; i < D; i++) F[i] = (FT)acc[i];
  if (lane == 0 && valid) external_force<D>(a, node, F);
  update_apply<D, L, MIXED>(a, o, F);
}

}  // namespace step
}  // namespace pdx
