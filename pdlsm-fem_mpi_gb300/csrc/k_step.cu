// Fused explicit step and internal-force kernels.
//
// One work item per node, L lanes per item (L in {4, 8, 16, 32}):
//   items [0, n_fam)            PD nodes (a family each): bonds of the family
//   items [n_fam, n_fam+n_feo)  FE-only nodes
// Each item computes the full internal force of its node's rows, so every
// row has exactly one writer and no atomics or force arrays are needed:
//   f_k = sum_bonds (C_km + P_km) (u_m - u_k)       PD + PD-boundary terms of family k
//       - sum_{FE e around k} Ke[rows of k] u_e      FE terms
//       + f_ext                                      traction BCs
// followed by the central-difference update of the node's active DOFs
// (timeIntegration_LM, pdsolve.cpp:5113-5132; first step :6010-6012) and the
// new value of its prescribed DOFs (setVaryEssentialBC :5263-5312).
//
// Critical-stretch failure (FC 3, the criterion of failureCriterion_stretch
// pdsolve.cpp:6643-6780 with s_c = s0) runs at the start of a step on the
// displacements stored by the previous step, before that step's force, which
// is the order of the reference loop (failure after the update, force at the
// next step).  A family whose damage exceeds 0.42 keeps its bonds.  Each bond
// is read, tested and cleared only by the lanes of its own family.
//
// Mixed precision: bond/element coefficients and the gathered displacements
// are FP32, forces accumulate in FP32; the state, the update and the mass are
// FP64.  The FP32 stretch test is re-evaluated in FP64 within a relative band
// of 2e-4 around the bond's threshold.
#include <type_traits>

#include "device.h"

namespace pdx {

namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Uniform draw in [0, 1) for the bond (k, m) of a seeded run.
__device__ __forceinline__ double bond_uniform(uint64_t seed, int k, int m) {
  const uint64_t key = seed * 0x9e3779b97f4a7c15ull + (uint64_t)(uint32_t)k * 0xd1b54a32d192ed03ull + (uint32_t)m;
  return (double)(splitmix64(key) >> 11) * 0x1.0p-53;
}

__device__ __forceinline__ double bond_s0(const DevView& v, int k, int m) {
  if (v.s0_pert == 0.0) return v.s0;
  return v.s0 * (1.0 + v.s0_pert * (2.0 * bond_uniform(v.s0_seed, k, m) - 1.0));
}

template <int D>
__device__ __forceinline__ bool stretch_over_fp64(const DevView& v, const double* u, int k, int m) {
  double xi[3] = {0, 0, 0}, eta[3] = {0, 0, 0};
#pragma unroll
  for (int i = 0; i < 3; i++) xi[i] = v.X[3 * m + i] - v.X[3 * k + i];
#pragma unroll
  for (int i = 0; i < D; i++) eta[i] = u[(int64_t)m * D + i] - u[(int64_t)k * D + i];
  const double mag_ref = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
  const double mag = sqrt((xi[0] + eta[0]) * (xi[0] + eta[0]) + (xi[1] + eta[1]) * (xi[1] + eta[1]) +
                          (xi[2] + eta[2]) * (xi[2] + eta[2]));
  const double s = mag / mag_ref - 1.0;
  return s > bond_s0(v, k, m);
}

template <int D, int L>
__device__ __forceinline__ void warp_sum(float* acc) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < D; i++) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
}
template <int D, int L>
__device__ __forceinline__ void warp_sum(double* acc) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < D; i++) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
}

// FE contribution -Ke[rows of local node al] u_e, u read through uget(n, i).
template <int D, typename T, typename ULoad>
__device__ __forceinline__ void fe_rows(const DevView& v, const T* ke, int e, int al, ULoad uload, T* acc) {
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
__device__ __forceinline__ void bond_block(const T* coef, const T* corr, int64_t nb, int64_t ncorr, int64_t b,
                                           int64_t slot, const T* du, T* acc) {
  if (D == 2) {
    const T c0 = coef[b], c1 = coef[nb + b], c2 = coef[2 * nb + b];
    acc[0] += c0 * du[0] + c1 * du[1];
    acc[1] += c1 * du[0] + c2 * du[1];
  } else {
    const T c0 = coef[b], c1 = coef[nb + b], c2 = coef[2 * nb + b];
    const T c3 = coef[3 * nb + b], c4 = coef[4 * nb + b], c5 = coef[5 * nb + b];
    acc[0] += c0 * du[0] + c1 * du[1] + c2 * du[2];
    acc[1] += c1 * du[0] + c3 * du[1] + c4 * du[2];
    acc[2] += c2 * du[0] + c4 * du[1] + c5 * du[2];
  }
  if (slot >= 0) {
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) acc[i] += corr[(int64_t)(i * D + j) * ncorr + slot] * du[j];
  }
}

template <int D, bool MIXED, int L>
__global__ void __launch_bounds__(256) k_step(StepArgs a) {
  using T = typename std::conditional<MIXED, float, double>::type;
  const DevView& v = a.v;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[item] : v.feonly_node[item - v.n_fam];
  const T* coef = MIXED ? (const T*)v.coef32 : (const T*)v.coef64;
  const T* corr = MIXED ? (const T*)v.corr32 : (const T*)v.corr64;
  const T* ke = MIXED ? (const T*)v.ke32 : (const T*)v.ke64;

  // displacement used by the force: stored value plus this step's prescribed increment
  auto load_u = [&](int n, T* out) {
    if (MIXED) {
      const float4 q = a.uf_n[n];
      const unsigned fl = __float_as_uint(q.w);
      out[0] = (T)q.x;
      out[1] = (T)q.y;
      if (D == 3) out[D - 1] = (T)q.z;
      if (fl) {
#pragma unroll
        for (int i = 0; i < D; i++)
          if ((fl >> i) & 1u) out[i] += (T)v.dtv[3 * n + i];
      }
    } else {
      const unsigned fl = v.bcflag[n];
#pragma unroll
      for (int i = 0; i < D; i++) {
        const double c = a.u_n[(int64_t)n * D + i];
        out[i] = (T)((fl >> i) & 1u ? c + v.dtv[3 * n + i] : c);
      }
    }
  };

  T acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0;
  int nbroken = 0;
  if (is_fam) {
    const int f = item;
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    bool brk = false;
    if (a.mode >= 1 && v.fail3) {
      const double phi = 1.0 - (double)v.fam_intact[f] / (double)(b1 - b0);
      brk = !(phi > 0.42);
    }
    const int corr0 = v.fam_corr[f];
    T uk[D];
    load_u(node, uk);
    float4 xkf = make_float4(0, 0, 0, 0);
    float4 ukf = make_float4(0, 0, 0, 0);
    if (MIXED && brk) { xkf = v.Xf[node]; ukf = a.uf_n[node]; }
    for (int b = b0 + lane; b < b1; b += L) {
      const uint32_t w = v.state[b >> 5];
      if (!((w >> (b & 31)) & 1u)) continue;
      const int m = v.nbr[b];
      if (brk) {
        bool cut;
        if (MIXED) {
          const float4 xm = v.Xf[m], um = a.uf_n[m];
          const float x0 = xm.x - xkf.x, x1 = xm.y - xkf.y, x2 = xm.z - xkf.z;
          const float e0 = um.x - ukf.x, e1 = um.y - ukf.y, e2 = D == 3 ? um.z - ukf.z : 0.f;
          const float xx = x0 * x0 + x1 * x1 + x2 * x2;
          const float xe = x0 * e0 + x1 * e1 + x2 * e2;
          const float ee = e0 * e0 + e1 * e1 + e2 * e2;
          const float lr = sqrtf(xx);
          const float lc = sqrtf(xx + 2.f * xe + ee);
          const float s = (2.f * xe + ee) / (lr * (lc + lr));
          const float sc = (float)bond_s0(v, node, m);
          if (fabsf(s - sc) <= 2e-4f * sc) cut = stretch_over_fp64<D>(v, a.u_n, node, m);
          else cut = s > sc;
        } else {
          cut = stretch_over_fp64<D>(v, a.u_n, node, m);
        }
        if (cut) {
          atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
          nbroken++;
          continue;
        }
      }
      if (a.mode == 2) continue;
      T du[D];
      load_u(m, du);
#pragma unroll
      for (int i = 0; i < D; i++) du[i] -= uk[i];
      bond_block<D, T>(coef, corr, v.n_bond, v.n_corr_bond, b, corr0 >= 0 ? (int64_t)corr0 + (b - b0) : -1, du,
                       acc);
    }
  }
  if (valid && a.mode != 2) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, T>(v, ke, ent >> 3, ent & 7, load_u, acc);
    }
  }
  warp_sum<D, L>(acc);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) nbroken += __shfl_xor_sync(0xffffffffu, nbroken, o);
  if (!valid || lane != 0) return;
  if (is_fam && nbroken) v.fam_intact[item] -= nbroken;
  if (a.mode == 2) return;
  double fext[D];
#pragma unroll
  for (int i = 0; i < D; i++) fext[i] = 0.0;
  if (v.ext_ptr && a.nbc_val) {
    for (int j = v.ext_ptr[node]; j < v.ext_ptr[node + 1]; j++) {
      const double t = a.nbc_val[v.ext_nbc[j]];
#pragma unroll
      for (int i = 0; i < D; i++) fext[i] += t * v.ext_f[3 * j + i];
    }
  }
  const double M = v.mass[node];
  const unsigned fl = v.bcflag[node];
  double unew[D];
#pragma unroll
  for (int i = 0; i < D; i++) {
    const int64_t idx = (int64_t)node * D + i;
    const double un = a.u_n[idx];
    if (v.eq[idx] >= 0) {
      const double F = __dadd_rn((double)acc[i], fext[i]);
      if (a.mode == 0) {
        unew[i] = __dadd_rn(__dmul_rn(__ddiv_rn(F, M), __dmul_rn(__dmul_rn(0.5, a.dt), a.dt)), un);
      } else {
        const double tempA = __ddiv_rn(__dmul_rn(__dmul_rn(a.dt, a.dt), F), M);
        unew[i] = __dsub_rn(__dadd_rn(__dmul_rn(un, 2.0), tempA), a.u_next[idx]);
      }
    } else {
      unew[i] = (fl >> i) & 1u ? __dadd_rn(un, v.dtv[3 * node + i]) : un;
    }
    a.u_next[idx] = unew[i];
  }
  if (MIXED) {
    a.uf_next[node] = make_float4((float)unew[0], (float)unew[1], D == 3 ? (float)unew[D - 1] : 0.f,
                                  __uint_as_float(fl));
  }
}

// Internal force F[eq] = -(K u)[eq] of a given DOF field (FP64), optionally
// plus the external force; no failure, no update.
template <int D, int L>
__global__ void __launch_bounds__(256) k_force(ForceArgs a) {
  const DevView& v = a.v;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[item] : v.feonly_node[item - v.n_fam];
  auto uget = [&](int n, int i) -> double { return a.u[(int64_t)n * D + i]; };
  auto uload = [&](int n, double* out) {
#pragma unroll
    for (int i = 0; i < D; i++) out[i] = a.u[(int64_t)n * D + i];
  };
  double acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0;
  if (is_fam) {
    const int f = item;
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    const int corr0 = v.fam_corr[f];
    double uk[D];
#pragma unroll
    for (int i = 0; i < D; i++) uk[i] = uget(node, i);
    for (int b = b0 + lane; b < b1; b += L) {
      if (!((v.state[b >> 5] >> (b & 31)) & 1u)) continue;
      const int m = v.nbr[b];
      double du[D];
#pragma unroll
      for (int i = 0; i < D; i++) du[i] = uget(m, i) - uk[i];
      bond_block<D, double>(v.coef64, v.corr64, v.n_bond, v.n_corr_bond, b,
                            corr0 >= 0 ? (int64_t)corr0 + (b - b0) : -1, du, acc);
    }
  }
  if (valid) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, double>(v, v.ke64, ent >> 3, ent & 7, uload, acc);
    }
  }
  warp_sum<D, L>(acc);
  if (!valid || lane != 0) return;
  double fext[D];
#pragma unroll
  for (int i = 0; i < D; i++) fext[i] = 0.0;
  if (v.ext_ptr && a.nbc_val) {
    for (int j = v.ext_ptr[node]; j < v.ext_ptr[node + 1]; j++) {
      const double t = a.nbc_val[v.ext_nbc[j]];
#pragma unroll
      for (int i = 0; i < D; i++) fext[i] += t * v.ext_f[3 * j + i];
    }
  }
#pragma unroll
  for (int i = 0; i < D; i++) {
    const int e = v.eq[(int64_t)node * D + i];
    if (e >= 0) a.f_eq[e] = acc[i] + fext[i] * a.ext_scale;
  }
}

template <int D, bool MIXED>
cudaError_t step_dispatch(const StepArgs& a, int lanes, cudaStream_t s) {
  const int64_t items = (int64_t)a.v.n_fam + a.v.n_feonly;
  const int64_t threads = items * lanes;
  const int blocks = (int)((threads + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  switch (lanes) {
    case 4: k_step<D, MIXED, 4><<<blocks, 256, 0, s>>>(a); break;
    case 8: k_step<D, MIXED, 8><<<blocks, 256, 0, s>>>(a); break;
    case 16: k_step<D, MIXED, 16><<<blocks, 256, 0, s>>>(a); break;
    case 32: k_step<D, MIXED, 32><<<blocks, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step(const StepArgs& a, int mixed, int lanes, cudaStream_t s) {
  if (a.v.dim == 2) return mixed ? step_dispatch<2, true>(a, lanes, s) : step_dispatch<2, false>(a, lanes, s);
  return mixed ? step_dispatch<3, true>(a, lanes, s) : step_dispatch<3, false>(a, lanes, s);
}

cudaError_t launch_force(const ForceArgs& a, cudaStream_t s) {
  const int64_t items = (int64_t)a.v.n_fam + a.v.n_feonly;
  const int L = 8;
  const int blocks = (int)((items * L + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  if (a.v.dim == 2) k_force<2, 8><<<blocks, 256, 0, s>>>(a);
  else k_force<3, 8><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pdx
