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
// new value of its prescribed DOFs (setVaryEssentialBC :5263-5312).  The
// update runs in FP64 with one DOF per lane of the warp (items of a warp are
// gathered by shuffles), so the narrow FP64 pipe sees full warps.
//
// Critical-stretch failure (FC 3, the criterion of failureCriterion_stretch
// pdsolve.cpp:6643-6780 with s_c = s0) runs at the start of a step on the
// displacements stored by the previous step, before that step's force, which
// is the order of the reference loop (failure after the update, force at the
// next step).  A family whose damage exceeds 0.42 keeps its bonds.  Each bond
// is read, tested and cleared only by the lanes of its own family.  The test
// |xi+eta| > (1+s0)|xi| is evaluated as 2 xi.eta + eta.eta > s0 (2+s0) |xi|^2
// (no square root, no division); within a relative band around the threshold
// (1e-9 in FP64, 2e-4 in FP32) the reference's own expression decides in FP64.
//
// FP64 kernel: structure-of-arrays coefficients, bond states as bits.
// Mixed kernel: one record per bond (3D: 32 B = 6 FP32 coefficients, the
// neighbour index whose sign carries the bond state, the bond's FP32
// threshold; 2D: 16 B = 3 coefficients + neighbour), forces in FP32, the
// state, update and mass in FP64.  Breaking a bond flips the record's sign
// and clears the bit of the FP64 state array as well.
#include <type_traits>

#include "device.h"

namespace pdx {

namespace {

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

// FE contribution -Ke[rows of local node al] u_e, u read through uload(n, out).
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
    const T c0 = __ldcs(coef + b), c1 = __ldcs(coef + nb + b), c2 = __ldcs(coef + 2 * nb + b);
    acc[0] += c0 * du[0] + c1 * du[1];
    acc[1] += c1 * du[0] + c2 * du[1];
  } else {
    const T c0 = __ldcs(coef + b), c1 = __ldcs(coef + nb + b), c2 = __ldcs(coef + 2 * nb + b);
    const T c3 = __ldcs(coef + 3 * nb + b), c4 = __ldcs(coef + 4 * nb + b), c5 = __ldcs(coef + 5 * nb + b);
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

template <int D, typename T>
__device__ __forceinline__ void corr_block(const T* corr, int64_t ncorr, int64_t slot, const T* du, T* acc) {
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int j = 0; j < D; j++) acc[i] += corr[(int64_t)(i * D + j) * ncorr + slot] * du[j];
}

// Lane 0 of every item holds F (internal + external force) and its node; the
// warp's lanes then take one (item, DOF) pair each for the FP64 update.
template <int D, int L, bool MIXED>
__device__ __forceinline__ void warp_update(const StepArgs& a, const double* F, int node_or_neg) {
  constexpr int IPW = 32 / L;
  const DevView& v = a.v;
  const int t = threadIdx.x & 31;
  const int j = t / D, i = t % D;
  const bool act = j < IPW;
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

template <int D, int L>
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

// ---------------------------------------------------------------- FP64 ----
template <int D, int L>
__global__ void __launch_bounds__(256, 2) k_step_fp64(StepArgs a) {
  const DevView& v = a.v;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  const int fo = is_fam ? v.fam_order[item] : 0;
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[fo] : v.feonly_node[item - v.n_fam];
  auto load_u = [&](int n, double* out) {
    const unsigned fl = v.bcflag[n];
#pragma unroll
    for (int i = 0; i < D; i++) {
      const double c = a.u_n[(int64_t)n * D + i];
      out[i] = (fl >> i) & 1u ? c + v.dtv[3 * n + i] : c;
    }
  };
  double acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0;
  int nbroken = 0;
  if (is_fam) {
    const int f = fo;
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    const bool brk = a.mode >= 1 && v.fail3 && v.fam_intact[f] >= v.fam_brk[f];
    const int corr0 = v.fam_corr[f];
    double uk[D], xk[3], ukst[D];
    load_u(node, uk);
#pragma unroll
    for (int i = 0; i < 3; i++) xk[i] = v.X[3 * node + i];
#pragma unroll
    for (int i = 0; i < D; i++) ukst[i] = a.u_n[(int64_t)node * D + i];
    for (int b = b0 + lane; b < b1; b += L) {
      const uint32_t w = v.state[b >> 5];
      if (!((w >> (b & 31)) & 1u)) continue;
      const int m = __ldcs(&v.nbr[b]);
      if (brk) {
        const uint32_t h = bond_hash(v.s0_seed32, node, m);
        double xi[3], eta[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < 3; i++) xi[i] = v.X[3 * m + i] - xk[i];
#pragma unroll
        for (int i = 0; i < D; i++) eta[i] = a.u_n[(int64_t)m * D + i] - ukst[i];
        const double xx = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
        const double lhs = 2.0 * (xi[0] * eta[0] + xi[1] * eta[1] + xi[2] * eta[2]) +
                           (eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
        const double sc = bond_s0(v, h);
        const double rhs = sc * (2.0 + sc) * xx;
        const bool cut = fabs(lhs - rhs) <= 1e-9 * rhs ? stretch_over_fp64<D>(v, a.u_n, node, m, h) : lhs > rhs;
        if (cut) {
          atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
          nbroken++;
          continue;
        }
      }
      if (a.mode == 2) continue;
      double du[D];
      load_u(m, du);
#pragma unroll
      for (int i = 0; i < D; i++) du[i] -= uk[i];
      bond_block<D, double>(v.coef64, v.corr64, v.n_bond, v.n_corr_bond, b,
                            corr0 >= 0 ? (int64_t)corr0 + (b - b0) : -1, du, acc);
    }
  }
  if (valid && a.mode != 2) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, double>(v, v.ke64, ent >> 3, ent & 7, load_u, acc);
    }
  }
  warp_sum<D, L>(acc);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) nbroken += __shfl_xor_sync(kFull, nbroken, o);
  if (lane == 0 && is_fam && nbroken) v.fam_intact[fo] -= nbroken;
  if (a.mode == 2) return;
  double F[D];
#pragma unroll
  for (int i = 0; i < D; i++) F[i] = acc[i];
  if (lane == 0 && valid) external_force<D, L>(a, node, F);
  warp_update<D, L, false>(a, F, valid ? node : -1);
}

// --------------------------------------------------------------- mixed ----
// Node records (2 float4 per node): [2n] = position (x, y, z, 0),
// [2n+1] = stored displacement (ux, uy, uz, varying-prescribed bits), so one
// 32-byte sector serves both the stretch test and the force.  Bond records are
// prefetched one iteration ahead in registers.
template <int D, int L>
__global__ void __launch_bounds__(256, 4) k_step_mixed(StepArgs a) {
  constexpr int RS = D == 3 ? 2 : 1;       // float4 per bond record
  extern __shared__ float s_ke[];
  const DevView& v = a.v;
  const float* ke = v.ke32;
  if (a.ke_smem) {
    for (int i = threadIdx.x; i < a.ke_smem; i += blockDim.x) s_ke[i] = v.ke32[i];
    __syncthreads();
    ke = s_ke;
  }
  const float4* nr = a.uf_n;               // node records of u_n
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  const int f = is_fam ? v.fam_order[item] : 0;
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[f] : v.feonly_node[item - v.n_fam];
  auto load_u = [&](int n, float* out) {
    const float4 q = nr[2 * n + 1];
    const unsigned fl = __float_as_uint(q.w);
    out[0] = q.x;
    out[1] = q.y;
    if (D == 3) out[D - 1] = q.z;
    if (fl) {
#pragma unroll
      for (int i = 0; i < D; i++)
        if ((fl >> i) & 1u) out[i] += (float)v.dtv[3 * n + i];
    }
  };
  float acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0.f;
  int nbroken = 0;
  if (is_fam) {
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    const bool brk = a.mode >= 1 && v.fail3 && v.fam_intact[f] >= v.fam_brk[f];
    const bool force = a.mode != 2;
    const int corr0 = v.fam_corr[f];
    const float4 xk = nr[2 * node];
    const float4 qk = nr[2 * node + 1];
    float uk[D];
    load_u(node, uk);
    float4* R = a.brec;
    bool deferred = false;
    int b = b0 + lane;
    float4 ra = make_float4(0, 0, 0, 0), rb = ra;
    if (b < b1) {
      ra = __ldcs(R + (int64_t)RS * b);
      if (D == 3) rb = __ldcs(R + (int64_t)RS * b + 1);
    }
    while (b < b1) {
      const int bn = b + L;
      float4 na = make_float4(0, 0, 0, 0), nb = na;
      if (bn < b1) {
        na = __ldcs(R + (int64_t)RS * bn);
        if (D == 3) nb = __ldcs(R + (int64_t)RS * bn + 1);
      }
      const int mb = __float_as_int(D == 3 ? rb.z : ra.w);
      if (mb >= 0) {
        const int m = mb;
        const float4 um = nr[2 * m + 1];
        bool cut = false;
        if (brk) {
          const float4 xm = nr[2 * m];
          const float x0 = xm.x - xk.x, x1 = xm.y - xk.y, x2 = xm.z - xk.z;
          const float e0 = um.x - qk.x, e1 = um.y - qk.y, e2 = D == 3 ? um.z - qk.z : 0.f;
          const float xx = x0 * x0 + x1 * x1 + x2 * x2;
          const float lhs = 2.f * (x0 * e0 + x1 * e1 + x2 * e2) + (e0 * e0 + e1 * e1 + e2 * e2);
          const uint32_t h = bond_hash(v.s0_seed32, node, m);
          const float sc = D == 3 ? rb.w : bond_s0_f32(a.s0f, a.pertf, h);
          const float rhs = sc * (2.f + sc) * xx;
          if (fabsf(lhs - rhs) <= 2e-4f * rhs) {
            // Near the threshold: decided in FP64 by the pass after the loop,
            // which also adds the bond's force if it stays intact.
            deferred = true;
            cut = true;
          } else if (lhs > rhs) {
            cut = true;
            int* mslot = (int*)(R + (int64_t)RS * b + (D == 3 ? 1 : 0)) + (D == 3 ? 2 : 3);
            *mslot = ~m;
            atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
            nbroken++;
          }
        }
        if (force && !cut) {
          float du[D];
          du[0] = um.x;
          du[1] = um.y;
          if (D == 3) du[D - 1] = um.z;
          const unsigned fl = __float_as_uint(um.w);
          if (fl) {
#pragma unroll
            for (int i = 0; i < D; i++)
              if ((fl >> i) & 1u) du[i] += (float)v.dtv[3 * m + i];
          }
#pragma unroll
          for (int i = 0; i < D; i++) du[i] -= uk[i];
          if (D == 2) {
            acc[0] += ra.x * du[0] + ra.y * du[1];
            acc[1] += ra.y * du[0] + ra.z * du[1];
          } else {
            acc[0] += ra.x * du[0] + ra.y * du[1] + ra.z * du[2];
            acc[1] += ra.y * du[0] + ra.w * du[1] + rb.x * du[2];
            acc[D - 1] += ra.z * du[0] + rb.x * du[1] + rb.y * du[2];
          }
          if (corr0 >= 0) corr_block<D, float>(v.corr32, v.n_corr_bond, (int64_t)corr0 + (b - b0), du, acc);
        }
      }
      b = bn;
      ra = na;
      rb = nb;
    }
    if (deferred) {
      // Rare: repeat the FP32 test on this lane's bonds and settle the ones
      // in the band with the reference's FP64 expression.
      for (b = b0 + lane; b < b1; b += L) {
        ra = R[(int64_t)RS * b];
        if (D == 3) rb = R[(int64_t)RS * b + 1];
        const int m = __float_as_int(D == 3 ? rb.z : ra.w);
        if (m < 0) continue;
        const float4 xm = nr[2 * m], um = nr[2 * m + 1];
        const float x0 = xm.x - xk.x, x1 = xm.y - xk.y, x2 = xm.z - xk.z;
        const float e0 = um.x - qk.x, e1 = um.y - qk.y, e2 = D == 3 ? um.z - qk.z : 0.f;
        const float xx = x0 * x0 + x1 * x1 + x2 * x2;
        const float lhs = 2.f * (x0 * e0 + x1 * e1 + x2 * e2) + (e0 * e0 + e1 * e1 + e2 * e2);
        const uint32_t h = bond_hash(v.s0_seed32, node, m);
        const float sc = D == 3 ? rb.w : bond_s0_f32(a.s0f, a.pertf, h);
        const float rhs = sc * (2.f + sc) * xx;
        if (!(fabsf(lhs - rhs) <= 2e-4f * rhs)) continue;
        if (stretch_over_fp64<D>(v, a.u_n, node, m, h)) {
          int* mslot = (int*)(R + (int64_t)RS * b + (D == 3 ? 1 : 0)) + (D == 3 ? 2 : 3);
          *mslot = ~m;
          atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
          nbroken++;
        } else if (force) {
          float du[D];
          load_u(m, du);
#pragma unroll
          for (int i = 0; i < D; i++) du[i] -= uk[i];
          if (D == 2) {
            acc[0] += ra.x * du[0] + ra.y * du[1];
            acc[1] += ra.y * du[0] + ra.z * du[1];
          } else {
            acc[0] += ra.x * du[0] + ra.y * du[1] + ra.z * du[2];
            acc[1] += ra.y * du[0] + ra.w * du[1] + rb.x * du[2];
            acc[D - 1] += ra.z * du[0] + rb.x * du[1] + rb.y * du[2];
          }
          if (corr0 >= 0) corr_block<D, float>(v.corr32, v.n_corr_bond, (int64_t)corr0 + (b - b0), du, acc);
        }
      }
    }
  }
  if (valid && a.mode != 2) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, float>(v, ke, ent >> 3, ent & 7, load_u, acc);
    }
  }
  warp_sum<D, L>(acc);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) nbroken += __shfl_xor_sync(kFull, nbroken, o);
  if (lane == 0 && is_fam && nbroken) v.fam_intact[f] -= nbroken;
  if (a.mode == 2) return;
  double F[D];
#pragma unroll
  for (int i = 0; i < D; i++) F[i] = (double)acc[i];
  if (lane == 0 && valid) external_force<D, L>(a, node, F);
  warp_update<D, L, true>(a, F, valid ? node : -1);
}

// Mixed-precision bond records from the FP32 coefficients, the bond states and
// the per-bond thresholds.
template <int D>
__global__ void k_pack_bonds(DevView v, float s0f, float pertf, float4* rec) {
  const int f = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (f >= v.n_fam) return;
  const int k = v.fam_node[f];
  const int64_t nb = v.n_bond;
  for (int b = v.fam_ptr[f] + (threadIdx.x & 31); b < v.fam_ptr[f + 1]; b += 32) {
    const int m = v.nbr[b];
    const bool intact = (v.state[b >> 5] >> (b & 31)) & 1u;
    const int mb = intact ? m : ~m;
    if (D == 2) {
      rec[b] = make_float4(v.coef32[b], v.coef32[nb + b], v.coef32[2 * nb + b], __int_as_float(mb));
    } else {
      const float s0b = bond_s0_f32(s0f, pertf, bond_hash(v.s0_seed32, k, m));
      rec[2 * (int64_t)b] = make_float4(v.coef32[b], v.coef32[nb + b], v.coef32[2 * nb + b], v.coef32[3 * nb + b]);
      rec[2 * (int64_t)b + 1] = make_float4(v.coef32[4 * nb + b], v.coef32[5 * nb + b], __int_as_float(mb), s0b);
    }
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


template <int D>
cudaError_t step_dispatch(const StepArgs& a, int mixed, int lanes, cudaStream_t s) {
  const int64_t items = (int64_t)a.v.n_fam + a.v.n_feonly;
  const int blocks = (int)((items * lanes + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)a.ke_smem * sizeof(float);
  if (mixed) {
    switch (lanes) {
      case 4: k_step_mixed<D, 4><<<blocks, 256, smem, s>>>(a); break;
      case 8: k_step_mixed<D, 8><<<blocks, 256, smem, s>>>(a); break;
      case 16: k_step_mixed<D, 16><<<blocks, 256, smem, s>>>(a); break;
      case 32: k_step_mixed<D, 32><<<blocks, 256, smem, s>>>(a); break;
      default: return cudaErrorInvalidValue;
    }
  } else {
    switch (lanes) {
      case 4: k_step_fp64<D, 4><<<blocks, 256, 0, s>>>(a); break;
      case 8: k_step_fp64<D, 8><<<blocks, 256, 0, s>>>(a); break;
      case 16: k_step_fp64<D, 16><<<blocks, 256, 0, s>>>(a); break;
      case 32: k_step_fp64<D, 32><<<blocks, 256, 0, s>>>(a); break;
      default: return cudaErrorInvalidValue;
    }
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step(const StepArgs& a, int mixed, int lanes, cudaStream_t s) {
  return a.v.dim == 2 ? step_dispatch<2>(a, mixed, lanes, s) : step_dispatch<3>(a, mixed, lanes, s);
}

cudaError_t launch_pack_bonds(const DevView& v, float s0f, float pertf, float4* rec, cudaStream_t s) {
  if (v.n_fam == 0) return cudaSuccess;
  const int blocks = (v.n_fam + 7) / 8;
  if (v.dim == 2) k_pack_bonds<2><<<blocks, 256, 0, s>>>(v, s0f, pertf, rec);
  else k_pack_bonds<3><<<blocks, 256, 0, s>>>(v, s0f, pertf, rec);
  return cudaGetLastError();
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
