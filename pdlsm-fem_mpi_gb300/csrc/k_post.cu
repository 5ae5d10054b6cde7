// Node stress and damage, CSR assembly through a scatter map, Newmark helpers.
//
// Stress (calGlobalNodeStresses pdsolve.cpp:9540-9604): a PD node gets
// D C u_family (calPDNodeStresses :9081-9166), every FE element around a node
// adds its Gauss-point stresses extrapolated to that node (calFEMNodeStresses_EXP
// :9168-9335, eleFitStresses flag 1), and the sum is divided by the number of
// contributions; plane strain adds sigma_zz = nu (sigma_xx + sigma_yy).
// Damage phi = 1 - intact/bonds per family (calLocalDamage :7338-7373).
//
// Assembly: each node's rows are written only by that node's work item, in a
// fixed order (bond blocks, then the diagonal block, then FE elements one at
// a time), through per-bond / per-element column offsets precomputed from the
// reference's CSR pattern (setCSRIndexes_gloStiffMat :959-1121).  No atomics,
// no binary search (findCSRIndexOfMat :1773-1802).
#include <climits>

#include "device.h"

namespace pdx {

namespace {

template <int D>
__device__ __forceinline__ int active_before(const int* eq, int n, int j) {
  int c = 0;
#pragma unroll
  for (int t = 0; t < D; t++)
    if (t < j && eq[n * D + t] >= 0) c++;
  return c;
}

template <int D, int L>
__global__ void __launch_bounds__(256) k_stress(StressArgs a) {
  constexpr int NV = D == 2 ? 3 : 6;
  constexpr int NEN = D == 2 ? 4 : 8;
  constexpr int ND = NEN * D;
  constexpr int NGP = NEN;
  const DevView& v = a.v;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[item] : v.feonly_node[item - v.n_fam];
  const int mat = valid && a.node_mat ? a.node_mat[node] : 0;
  const double* Dm = a.D + (int64_t)mat * NV * NV;
  double eps[NV], sfe[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) { eps[i] = 0; sfe[i] = 0; }
  if (is_fam) {
    const int b0 = v.fam_ptr[item], b1 = v.fam_ptr[item + 1];
    double uk[D];
#pragma unroll
    for (int i = 0; i < D; i++) uk[i] = a.u[(int64_t)node * D + i];
    for (int b = b0 + lane; b < b1; b += L) {
      if (!((v.state[b >> 5] >> (b & 31)) & 1u)) continue;
      const int m = v.nbr[b];
      double du[D], c[D];
#pragma unroll
      for (int i = 0; i < D; i++) {
        du[i] = a.u[(int64_t)m * D + i] - uk[i];
        c[i] = v.cvec[(int64_t)i * v.n_bond + b];
      }
      if (D == 2) {
        eps[0] += c[0] * du[0];
        eps[1] += c[1] * du[1];
        eps[2] += c[1] * du[0] + c[0] * du[1];
      } else {
        eps[0] += c[0] * du[0];
        eps[1] += c[1] * du[1];
        eps[2] += c[2] * du[2];
        eps[3] += c[1] * du[0] + c[0] * du[1];
        eps[4] += c[2] * du[1] + c[1] * du[2];
        eps[5] += c[2] * du[0] + c[0] * du[2];
      }
    }
  }
  int nadj = 0;
  if (valid) {
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    nadj = j1 - j0;
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      const int e = ent >> 3, al = ent & 7;
      const double* B = a.bgp + (int64_t)v.fe_cls[e] * NGP * NV * ND;
      double ue[ND];
#pragma unroll
      for (int jn = 0; jn < NEN; jn++) {
        const int n = v.fe_conn[e * 8 + jn];
#pragma unroll
        for (int jj = 0; jj < D; jj++) ue[jn * D + jj] = a.u[(int64_t)n * D + jj];
      }
      for (int g = 0; g < NGP; g++) {
        double eg[NV];
#pragma unroll
        for (int r = 0; r < NV; r++) {
          double s = 0;
#pragma unroll
          for (int c = 0; c < ND; c++) s += B[(g * NV + r) * ND + c] * ue[c];
          eg[r] = s;
        }
        const double w = a.L[al * NGP + g];
#pragma unroll
        for (int r = 0; r < NV; r++) {
          double s = 0;
#pragma unroll
          for (int c = 0; c < NV; c++) s += Dm[r * NV + c] * eg[c];
          sfe[r] += w * s;
        }
      }
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < NV; i++) {
      eps[i] += __shfl_xor_sync(0xffffffffu, eps[i], o);
      sfe[i] += __shfl_xor_sync(0xffffffffu, sfe[i], o);
    }
  if (!valid || lane != 0) return;
  double sig[NV];
#pragma unroll
  for (int r = 0; r < NV; r++) {
    double s = 0;
    if (is_fam)
#pragma unroll
      for (int c = 0; c < NV; c++) s += Dm[r * NV + c] * eps[c];
    sig[r] = s + sfe[r];
  }
  const double cnt = (double)((is_fam ? 1 : 0) + nadj);
  double* out = a.sigma ? a.sigma + (int64_t)node * 6 : nullptr;
  if (!out) {
  } else if (D == 2) {
    out[0] = sig[0] / cnt;
    out[1] = sig[1] / cnt;
    out[2] = 0.0;
    out[3] = sig[2] / cnt;
    out[4] = 0.0;
    out[5] = 0.0;
    if (a.protype == 2) out[2] = a.nu[mat] * (out[0] + out[1]);
  } else {
#pragma unroll
    for (int r = 0; r < 6; r++) out[r] = sig[r] / cnt;
  }
  if (a.phi) {
    if (is_fam) {
      const int nb = v.fam_ptr[item + 1] - v.fam_ptr[item];
      a.phi[node] = 1.0 - (double)v.fam_intact[item] / (double)nb;
    } else {
      a.phi[node] = 0.0;
    }
  }
}

template <int D, int L>
__global__ void __launch_bounds__(256) k_assemble(AsmArgs a) {
  constexpr int NEN = D == 2 ? 4 : 8;
  constexpr int ND = NEN * D;
  const DevView& v = a.v;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int item = (int)(gt / L);
  const int lane = (int)(gt % L);
  const int n_items = v.n_fam + v.n_feonly;
  const bool valid = item < n_items;
  const bool is_fam = valid && item < v.n_fam;
  const unsigned sub = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) / L * L));
  int node = 0;
  if (valid) node = is_fam ? v.fam_node[item] : v.feonly_node[item - v.n_fam];
  int64_t row[D];
#pragma unroll
  for (int i = 0; i < D; i++) {
    const int e = valid ? v.eq[(int64_t)node * D + i] : -1;
    row[i] = e >= 0 ? a.ia[e] : -1;
  }
  double dsum[D][D];
#pragma unroll
  for (int i = 0; i < D; i++)
#pragma unroll
    for (int j = 0; j < D; j++) dsum[i][j] = 0;
  if (is_fam && a.with_pd) {
    const int b0 = v.fam_ptr[item], b1 = v.fam_ptr[item + 1];
    const int corr0 = v.fam_corr[item];
    for (int b = b0 + lane; b < b1; b += L) {
      if (!((v.state[b >> 5] >> (b & 31)) & 1u)) continue;
      const int m = v.nbr[b];
      double M[D][D];
      if (D == 2) {
        const double c0 = v.coef64[b], c1 = v.coef64[v.n_bond + b], c2 = v.coef64[2 * v.n_bond + b];
        M[0][0] = c0; M[0][1] = c1; M[1][0] = c1; M[1][1] = c2;
      } else {
        const int64_t nb = v.n_bond;
        const double c0 = v.coef64[b], c1 = v.coef64[nb + b], c2 = v.coef64[2 * nb + b];
        const double c3 = v.coef64[3 * nb + b], c4 = v.coef64[4 * nb + b], c5 = v.coef64[5 * nb + b];
        M[0][0] = c0; M[0][1] = c1; M[0][2] = c2;
        M[1][0] = c1; M[1][1] = c3; M[1][2] = c4;
        M[2][0] = c2; M[2][1] = c4; M[2][2] = c5;
      }
      if (corr0 >= 0) {
        const int64_t slot = (int64_t)corr0 + (b - b0);
#pragma unroll
        for (int i = 0; i < D; i++)
#pragma unroll
          for (int j = 0; j < D; j++) M[i][j] += v.corr64[(int64_t)(i * D + j) * v.n_corr_bond + slot];
      }
      const int rel = a.rel_bond[b];
#pragma unroll
      for (int i = 0; i < D; i++) {
        if (row[i] < 0) continue;
        int jp = 0;
#pragma unroll
        for (int j = 0; j < D; j++) {
          if (v.eq[(int64_t)m * D + j] < 0) continue;
          a.a[row[i] + rel + jp] += -M[i][j];
          jp++;
        }
      }
#pragma unroll
      for (int i = 0; i < D; i++)
#pragma unroll
        for (int j = 0; j < D; j++) dsum[i][j] += M[i][j];
    }
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < D; i++)
#pragma unroll
      for (int j = 0; j < D; j++) dsum[i][j] += __shfl_xor_sync(0xffffffffu, dsum[i][j], o);
  if (is_fam && lane == 0) {
    const int rel = a.rel_self[item];
#pragma unroll
    for (int i = 0; i < D; i++) {
      if (row[i] < 0) continue;
      int jp = 0;
#pragma unroll
      for (int j = 0; j < D; j++) {
        if (v.eq[(int64_t)node * D + j] < 0) continue;
        double val = a.with_pd ? dsum[i][j] : 0.0;
        if (a.pd_diag_rho > 0 && i == j) val += a.fam_cdv[item] * a.pd_diag_rho;
        a.a[row[i] + rel + jp] += val;
        jp++;
      }
    }
  }
  __syncwarp(sub);
  if (!valid || !a.table) return;
  const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
  for (int j = j0; j < j1; j++) {
    const int ent = v.fe_adj[j];
    const int e = ent >> 3, al = ent & 7;
    const double* K = a.table + (int64_t)v.fe_cls[e] * ND * ND;
    for (int c = lane; c < ND; c += L) {
      const int jn = c / D, jj = c % D;
      const int n = v.fe_conn[e * 8 + jn];
      if (v.eq[(int64_t)n * D + jj] < 0) continue;
      const int jp = active_before<D>(v.eq, n, jj);
      const int rel = a.rel_fe[(int64_t)j * 8 + jn];
#pragma unroll
      for (int i = 0; i < D; i++) {
        if (row[i] < 0) continue;
        a.a[row[i] + rel + jp] += K[(al * D + i) * ND + c];
      }
    }
    __syncwarp(sub);
  }
}

template <int D>
__global__ void k_newmark_predict(DevView v, const double* u, const double* vel, const double* acc, double dt,
                                  double beta, double* up) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int n = (int)(i / D), d = (int)(i % D);
  const int e = v.eq[i];
  if (e >= 0) {
    up[i] = u[i] + dt * vel[e] + dt * dt * (0.5 - beta) * acc[e];
  } else {
    up[i] = (v.bcflag[n] >> d) & 1u ? u[i] + v.dtv[3 * n + d] : u[i];
  }
}

__global__ void k_newmark_update(int n, const double* vel0, const double* a0, const double* a1, double dt,
                                 double beta, double gamma, double* u_eq, double* vel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double t1 = u_eq[i] + dt * vel0[i] + dt * dt * ((0.5 - beta) * a0[i] + beta * a1[i]);
  const double t2 = vel0[i] + dt * ((1 - gamma) * a0[i] + gamma * a1[i]);
  u_eq[i] = t1;
  vel[i] = t2;
}

template <int D>
__global__ void k_scatter_eq(DevView v, const double* u_eq, double* u_all) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int e = v.eq[i];
  if (e >= 0) u_all[i] = u_eq[e];
}

template <int D>
__global__ void k_gather_eq(DevView v, const double* u_all, double* u_eq) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int e = v.eq[i];
  if (e >= 0) u_eq[e] = u_all[i];
}

// prescribed DOFs advance by their per-step increment (setVaryEssentialBC)
template <int D>
__global__ void k_advance_prescribed(DevView v, double* u_all) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int n = (int)(i / D), d = (int)(i % D);
  if (v.eq[i] < 0 && ((v.bcflag[n] >> d) & 1u)) u_all[i] = u_all[i] + v.dtv[3 * n + d];
}

// Quasi-static rule of setVaryEssentialBC (pdsolve.cpp:5263-5311, solver
// flag 2) with the load ratio 1 that FC 0 / FC 3 and every 3D model give: a
// varying EBC moves by dt * velocity while its value is 0 and holds after.
// Every node of an EBC carries the EBC's value, so the test is per DOF.
template <int D>
__global__ void k_advance_prescribed_quasi(DevView v, double* u_all) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int n = (int)(i / D), d = (int)(i % D);
  if (v.eq[i] < 0 && ((v.bcflag[n] >> d) & 1u) && u_all[i] == 0.0) u_all[i] = v.dtv[3 * n + d];
}

// Equation range [lo, hi] of the DOFs of a block's nodes (256 nodes per
// block), for staging host-resident equation-ordered vectors through shared
// memory: with the usual numbering (DOFs numbered in node order, prescribed
// ones skipped) the range is contiguous and holds exactly the block's DOFs,
// so the host link sees coalesced runs instead of 8-byte accesses three
// apart.  lo > hi when the block has no free DOF.
template <int D>
__device__ __forceinline__ void block_eq_range(const DevView& v, int* s_lo, int* s_hi) {
  if (threadIdx.x == 0) {
    *s_lo = INT_MAX;
    *s_hi = -1;
  }
  __syncthreads();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  int lo = INT_MAX, hi = -1;
  if (n < v.n_node) {
#pragma unroll
    for (int d = 0; d < D; d++) {
      const int e = v.eq[(int64_t)n * D + d];
      if (e >= 0) {
        lo = min(lo, e);
        hi = max(hi, e);
      }
    }
  }
  if (hi >= 0) {
    atomicMin(s_lo, lo);
    atomicMax(s_hi, hi);
  }
  __syncthreads();
}

constexpr int kStageNodes = 256;

// u_n and u_{n-1} in equation order into the node-ordered states in one pass
// (prescribed DOFs keep their device values), and with uf the FP32 shadow of
// u_n as k_shadow writes it.  The inputs may be the caller's page-locked host
// buffers: each block first copies its equation range of both vectors into
// shared memory with consecutive loads (when the range fits, as it does for
// the usual numbering), then scatters from there.
template <int D>
__global__ void __launch_bounds__(kStageNodes) k_load_pair(DevView v, const double* un_eq, const double* unm1_eq,
                                                          double* u_cur, double* u_prev, float4* uf) {
  __shared__ double s_n[kStageNodes * D], s_m[kStageNodes * D];
  __shared__ int s_lo, s_hi;
  block_eq_range<D>(v, &s_lo, &s_hi);
  const int lo = s_lo, cnt = s_hi - s_lo + 1;
  const bool staged = cnt > 0 && cnt <= kStageNodes * D;
  if (staged) {
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
      s_n[k] = un_eq[lo + k];
      s_m[k] = unm1_eq[lo + k];
    }
  }
  __syncthreads();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.n_node) return;
  float c[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = 0; d < D; d++) {
    const int64_t i = (int64_t)n * D + d;
    const int e = v.eq[i];
    double x;
    if (e >= 0) {
      x = staged ? s_n[e - lo] : un_eq[e];
      u_cur[i] = x;
      u_prev[i] = staged ? s_m[e - lo] : unm1_eq[e];
    } else {
      x = u_cur[i];
    }
    c[d] = (float)x;
  }
  if (uf) {
    uf[2 * n] = v.Xf[n];
    uf[2 * n + 1] = make_float4(c[0], c[1], D == 3 ? c[2] : 0.f, __uint_as_float((unsigned)v.bcflag[n]));
  }
}

// u_eq[e] = u_all[i] for the free DOFs, u_eq possibly the caller's
// page-locked host buffer: each block assembles its equation range in shared
// memory and writes it with consecutive stores (only the positions its own
// DOFs fill), else stores directly.
template <int D>
__global__ void __launch_bounds__(kStageNodes) k_store_eq(DevView v, const double* u_all, double* u_eq) {
  __shared__ double s_u[kStageNodes * D];
  __shared__ unsigned char s_set[kStageNodes * D];
  __shared__ int s_lo, s_hi;
  block_eq_range<D>(v, &s_lo, &s_hi);
  const int lo = s_lo, cnt = s_hi - s_lo + 1;
  const bool staged = cnt > 0 && cnt <= kStageNodes * D;
  if (staged)
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) s_set[k] = 0;
  __syncthreads();
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < v.n_node) {
#pragma unroll
    for (int d = 0; d < D; d++) {
      const int64_t i = (int64_t)n * D + d;
      const int e = v.eq[i];
      if (e < 0) continue;
      if (staged) {
        s_u[e - lo] = u_all[i];
        s_set[e - lo] = 1;
      } else {
        u_eq[e] = u_all[i];
      }
    }
  }
  if (!staged) return;
  __syncthreads();
  for (int k = threadIdx.x; k < cnt; k += blockDim.x)
    if (s_set[k]) u_eq[lo + k] = s_u[k];
}

template <int D>
__global__ void k_shadow(DevView v, const double* u, float4* uf) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.n_node) return;
  uf[2 * n] = v.Xf[n];
  uf[2 * n + 1] = make_float4((float)u[(int64_t)n * D], (float)u[(int64_t)n * D + 1],
                              D == 3 ? (float)u[(int64_t)n * D + 2] : 0.f, __uint_as_float((unsigned)v.bcflag[n]));
}

__global__ void k_newmark_matrix(int64_t n, double* k, const double* m, double beta, double dt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) k[i] = k[i] * beta * dt * dt + m[i];
}

__global__ void k_axpby(int64_t n, const double* x, double alpha, double* y, double beta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = alpha * x[i] + beta * y[i];
}

}  // namespace

cudaError_t launch_stress(const StressArgs& a, cudaStream_t s) {
  const int64_t items = (int64_t)a.v.n_fam + a.v.n_feonly;
  const int blocks = (int)((items * 8 + 255) / 256);
  if (!blocks) return cudaSuccess;
  if (a.v.dim == 2) k_stress<2, 8><<<blocks, 256, 0, s>>>(a);
  else k_stress<3, 8><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_assemble(const AsmArgs& a, cudaStream_t s) {
  const int64_t items = (int64_t)a.v.n_fam + a.v.n_feonly;
  const int blocks = (int)((items * 8 + 255) / 256);
  if (!blocks) return cudaSuccess;
  if (a.v.dim == 2) k_assemble<2, 8><<<blocks, 256, 0, s>>>(a);
  else k_assemble<3, 8><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_newmark_predict(const DevView& v, const double* u, const double* vel, const double* acc,
                                   double dt, double beta, double* up, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_newmark_predict<2><<<blocks, 256, 0, s>>>(v, u, vel, acc, dt, beta, up);
  else k_newmark_predict<3><<<blocks, 256, 0, s>>>(v, u, vel, acc, dt, beta, up);
  return cudaGetLastError();
}

cudaError_t launch_newmark_update(int n, const double* vel0, const double* a0, const double* a1, double dt,
                                  double beta, double gamma, double* u_eq, double* vel, cudaStream_t s) {
  k_newmark_update<<<(n + 255) / 256, 256, 0, s>>>(n, vel0, a0, a1, dt, beta, gamma, u_eq, vel);
  return cudaGetLastError();
}

cudaError_t launch_scatter_eq(const DevView& v, const double* u_eq, double* u_all, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_scatter_eq<2><<<blocks, 256, 0, s>>>(v, u_eq, u_all);
  else k_scatter_eq<3><<<blocks, 256, 0, s>>>(v, u_eq, u_all);
  return cudaGetLastError();
}

cudaError_t launch_gather_eq(const DevView& v, const double* u_all, double* u_eq, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_gather_eq<2><<<blocks, 256, 0, s>>>(v, u_all, u_eq);
  else k_gather_eq<3><<<blocks, 256, 0, s>>>(v, u_all, u_eq);
  return cudaGetLastError();
}

cudaError_t launch_advance_prescribed(const DevView& v, double* u_all, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_advance_prescribed<2><<<blocks, 256, 0, s>>>(v, u_all);
  else k_advance_prescribed<3><<<blocks, 256, 0, s>>>(v, u_all);
  return cudaGetLastError();
}

// Reaction force of one step, as calReacForc (pdsolve.cpp:5347-5404): for
// every element touching an RF node, Fe = Ke u_e (u_e = all DOF values of its
// nodes); the entries of its RF nodes are summed over the elements in order.
// Non-fused products and sums in the reference's order.
__global__ void k_reaction(int n_el, int nen, int dim, const int* conn, const double* ke, const int* mask,
                           const double* u_all, int64_t uc_index, double* part, double* hist_row) {
  const int nd = nen * dim;
  // part[(e * nen + a) * 3 + j] = Fe of RF node a, DOF j of element e
  for (int e = threadIdx.x; e < n_el; e += blockDim.x) {
    const double* K = ke + (int64_t)e * nd * nd;
    for (int a = 0; a < nen; a++) {
      if (!((mask[e] >> a) & 1)) continue;
      for (int j = 0; j < dim; j++) {
        const int r = a * dim + j;
        double acc = 0.0;
        for (int c = 0; c < nd; c++) {
          const int node = conn[(int64_t)e * nen + c / dim];
          acc = __dadd_rn(acc, __dmul_rn(K[(int64_t)r * nd + c], u_all[(int64_t)node * dim + c % dim]));
        }
        part[((int64_t)e * nen + a) * 3 + j] = acc;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[3] = {0, 0, 0};
    for (int e = 0; e < n_el; e++)
      for (int a = 0; a < nen; a++) {
        if (!((mask[e] >> a) & 1)) continue;
        for (int j = 0; j < dim; j++) t[j] = __dadd_rn(t[j], part[((int64_t)e * nen + a) * 3 + j]);
      }
    hist_row[0] = uc_index >= 0 ? u_all[uc_index] : 0.0;
    hist_row[1] = t[0];
    hist_row[2] = t[1];
    hist_row[3] = t[2];
  }
}

cudaError_t launch_reaction(int n_el, int nen, int dim, const int* conn, const double* ke, const int* mask,
                            const double* u_all, int64_t uc_index, double* part, double* hist_row, cudaStream_t s) {
  k_reaction<<<1, 256, 0, s>>>(n_el, nen, dim, conn, ke, mask, u_all, uc_index, part, hist_row);
  return cudaGetLastError();
}

// setVaryEssentialBC (pdsolve.cpp:5263-5311, solver flag 2) with a load
// ratio rati: a varying EBC at 0 moves by dt * velocity; otherwise by
// dt * (rati - 1) * value, or dt * velocity if that step is larger, or not
// at all if rati < 1.
template <int D>
__global__ void k_advance_prescribed_ratio(DevView v, double* u_all, const double* vel, double dt, double rati) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)v.n_node * D) return;
  const int n = (int)(i / D), d = (int)(i % D);
  if (!(v.eq[i] < 0 && ((v.bcflag[n] >> d) & 1u))) return;
  const double value = u_all[i], velocity = vel[3 * n + d];
  double dv;
  if (value == 0.0) {
    dv = velocity;
  } else {
    const double ndv = (rati - 1) * value;
    if (fabs(ndv) > fabs(velocity)) dv = velocity;
    else if (rati < 1) dv = 0;
    else dv = ndv;
  }
  u_all[i] = value + dt * dv;
}

cudaError_t launch_advance_prescribed_ratio(const DevView& v, double* u_all, const double* vel, double dt,
                                            double rati, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_advance_prescribed_ratio<2><<<blocks, 256, 0, s>>>(v, u_all, vel, dt, rati);
  else k_advance_prescribed_ratio<3><<<blocks, 256, 0, s>>>(v, u_all, vel, dt, rati);
  return cudaGetLastError();
}

cudaError_t launch_advance_prescribed_quasi(const DevView& v, double* u_all, cudaStream_t s) {
  const int64_t n = (int64_t)v.n_node * v.dim;
  const int blocks = (int)((n + 255) / 256);
  if (v.dim == 2) k_advance_prescribed_quasi<2><<<blocks, 256, 0, s>>>(v, u_all);
  else k_advance_prescribed_quasi<3><<<blocks, 256, 0, s>>>(v, u_all);
  return cudaGetLastError();
}

cudaError_t launch_load_pair(const DevView& v, const double* un_eq, const double* unm1_eq, double* u_cur,
                             double* u_prev, float4* uf, cudaStream_t s) {
  const int blocks = (v.n_node + kStageNodes - 1) / kStageNodes;
  if (v.dim == 2) k_load_pair<2><<<blocks, kStageNodes, 0, s>>>(v, un_eq, unm1_eq, u_cur, u_prev, uf);
  else k_load_pair<3><<<blocks, kStageNodes, 0, s>>>(v, un_eq, unm1_eq, u_cur, u_prev, uf);
  return cudaGetLastError();
}

cudaError_t launch_store_eq(const DevView& v, const double* u_all, double* u_eq, cudaStream_t s) {
  const int blocks = (v.n_node + kStageNodes - 1) / kStageNodes;
  if (v.dim == 2) k_store_eq<2><<<blocks, kStageNodes, 0, s>>>(v, u_all, u_eq);
  else k_store_eq<3><<<blocks, kStageNodes, 0, s>>>(v, u_all, u_eq);
  return cudaGetLastError();
}

cudaError_t launch_shadow(const DevView& v, const double* u_all, float4* uf, cudaStream_t s) {
  const int blocks = (v.n_node + 255) / 256;
  if (v.dim == 2) k_shadow<2><<<blocks, 256, 0, s>>>(v, u_all, uf);
  else k_shadow<3><<<blocks, 256, 0, s>>>(v, u_all, uf);
  return cudaGetLastError();
}

cudaError_t launch_newmark_matrix(int64_t nnz, double* k, const double* m, double beta, double dt, cudaStream_t s) {
  k_newmark_matrix<<<(int)((nnz + 255) / 256), 256, 0, s>>>(nnz, k, m, beta, dt);
  return cudaGetLastError();
}

cudaError_t launch_axpby_scale(int64_t n, const double* x, double alpha, double* y, double beta, cudaStream_t s) {
  k_axpby<<<(int)((n + 255) / 256), 256, 0, s>>>(n, x, alpha, y, beta);
  return cudaGetLastError();
}

}  // namespace pdx
