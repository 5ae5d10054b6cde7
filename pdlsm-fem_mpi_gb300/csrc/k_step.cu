// FP64 explicit step and internal-force kernels.
//
// One work item per node: a PD family (LP lanes) or an FE-only node (LF
// lanes); the layout of a launch and the update are described in
// k_step_common.cuh.
//
// Critical-stretch failure (FC 3, the criterion of failureCriterion_stretch
// pdsolve.cpp:6643-6780 with s_c = s0) runs at the start of a step on the
// displacements stored by the previous step, before that step's force, which
// is the order of the reference loop (failure after the update, force at the
// next step).  A family whose damage exceeds 0.42 keeps its bonds.  Each bond
// is read, tested and cleared only by the lanes of its own family.  The test
// |xi+eta| > (1+s0)|xi| is evaluated as 2 xi.eta + eta.eta > s0 (2+s0) |xi|^2
// (no square root, no division); within a relative band of 1e-9 around the
// threshold the reference's own expression decides.
//
// Coefficients are structure-of-arrays (coef[c * n_bond + b]) so that the
// lanes of one family read consecutive addresses; bond states are bits.
#include "k_step_common.cuh"

namespace pdx {

using namespace step;

namespace {

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
  if (slot >= 0) corr_block<D, T>(corr, ncorr, slot, du, acc);
}

template <int D, int L>
__device__ __forceinline__ void fp64_family_item(const StepArgs& a, int64_t t) {
  const DevView& v = a.v;
  const int item = (int)(t / L);
  const int lane = (int)(t % L);
  const bool valid = item < v.n_fam;
  const int f = valid ? v.fam_order[item] : 0;
  const int node = valid ? v.fam_node[f] : 0;
  const LoadFp64<D> load_u{a.u_n, v.bcflag, v.dtv};
  double acc[D];
#pragma unroll
  for (int i = 0; i < D; i++) acc[i] = 0;
  int nbroken = 0;
  if (valid) {
    const int b0 = v.fam_ptr[f], b1 = v.fam_ptr[f + 1];
    const bool brk = a.mode >= 1 && v.fail3 && v.fam_intact[f] >= v.fam_brk[f];
    const double s0fam = v.fam_s0[f];
    const int corr0 = v.fam_corr[f];
    double uk[D], xk[3], ukst[D];
    load_u(node, uk);
#pragma unroll
    for (int i = 0; i < 3; i++) xk[i] = v.X[3 * node + i];
#pragma unroll
    for (int i = 0; i < D; i++) ukst[i] = a.u_n[(int64_t)node * D + i];
    const bool k_moves = v.bcflag[node] != 0;
    const float s0f = (float)s0fam, pertf = (float)v.s0_pert;
    const float4 xkf = v.Xf[node];
    const float xkmag = fmaxf(fabsf(xkf.x), fmaxf(fabsf(xkf.y), fabsf(xkf.z)));
    for (int b = b0 + lane; b < b1; b += L) {
      const uint32_t w = v.state[b >> 5];
      if (!((w >> (b & 31)) & 1u)) continue;
      const int m = __ldcs(&v.nbr[b]);
      double eta[3] = {0, 0, 0};
      bool have_eta = false;
      if (brk) {
        const uint32_t h = bond_hash(v.s0_seed32, node, m);
#pragma unroll
        for (int i = 0; i < D; i++) eta[i] = a.u_n[(int64_t)m * D + i] - ukst[i];
        have_eta = true;
        // The test 2 xi.eta + eta.eta > s (2 + s) |xi|^2 in FP32 first: eta
        // rounded from its FP64 value (integer-pipe conversion), xi from the
        // FP32 node positions.  The FP32 arithmetic errs by less than 1e-6 of
        // the sum of the terms' magnitudes and the positions' rounding by
        // less than 2.1e-7 max|X| in the length of xi (so in lhs and rhs by
        // 2.1e-7 max|X| (2|eta| + 2 s (2+s) |xi|)); outside a band of ten
        // times the first and about five times the second the FP32 answer is the
        // FP64 one, and inside it the FP64 test (and within 1e-9 the
        // reference's own expression) decides.  This keeps xi, the square
        // norms, the threshold and the comparison off the 2-lane FP64 pipe
        // for nearly every bond.
        const float4 xmf = v.Xf[m];
        const float xf[3] = {xmf.x - xkf.x, xmf.y - xkf.y, xmf.z - xkf.z};
        const float xmag = fmaxf(xkmag, fmaxf(fabsf(xmf.x), fmaxf(fabsf(xmf.y), fabsf(xmf.z))));
        float ef[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < D; i++) ef[i] = d2f_bits(eta[i]);
        const float xx32 = xf[0] * xf[0] + xf[1] * xf[1] + xf[2] * xf[2];
        const float ee32 = ef[0] * ef[0] + ef[1] * ef[1] + ef[2] * ef[2];
        const float lhs32 = 2.f * (xf[0] * ef[0] + xf[1] * ef[1] + xf[2] * ef[2]) + ee32;
        const float sc32 = bond_s0_f32(s0f, pertf, h);
        const float q = sc32 * (2.f + sc32);
        const float rhs32 = q * xx32;
        const float band = 1e-5f * (2.f * sqrtf(xx32 * ee32) + ee32 + rhs32) +
                           1e-6f * xmag * (2.f * sqrtf(ee32) + 2.f * q * sqrtf(xx32));
        bool cut;
        if (fabsf(lhs32 - rhs32) > band) {
          cut = lhs32 > rhs32;
        } else {
          double xi[3];
#pragma unroll
          for (int i = 0; i < 3; i++) xi[i] = v.X[3 * m + i] - xk[i];
          const double xx = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
          const double lhs = 2.0 * (xi[0] * eta[0] + xi[1] * eta[1] + xi[2] * eta[2]) +
                             (eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
          const double sc = bond_s0(s0fam, v.s0_pert, h);
          const double rhs = sc * (2.0 + sc) * xx;
          cut = fabs(lhs - rhs) <= 1e-9 * rhs ? stretch_over_fp64<D>(v, a.u_n, node, m, sc) : lhs > rhs;
        }
        if (cut) {
          atomicAnd(&v.state[b >> 5], ~(1u << (b & 31)));
          nbroken++;
          continue;
        }
      }
      if (a.mode == 2) continue;
      double du[D];
      if (have_eta && !k_moves && v.bcflag[m] == 0) {
        // no varying prescribed value at either end: u_m - u_k is eta
#pragma unroll
        for (int i = 0; i < D; i++) du[i] = eta[i];
      } else {
        load_u(m, du);
#pragma unroll
        for (int i = 0; i < D; i++) du[i] -= uk[i];
      }
      bond_block<D, double>(v.coef64, v.corr64, v.n_bond, v.n_corr_bond, b,
                            corr0 >= 0 ? (int64_t)corr0 + (b - b0) : -1, du, acc);
    }
    if (a.mode != 2) {
      const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
      for (int j = j0 + lane; j < j1; j += L) {
        const int ent = v.fe_adj[j];
        fe_rows<D, double>(v, v.ke64, ent >> 3, ent & 7, load_u, acc);
      }
    }
  }
  warp_sum<D, L>(acc);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) nbroken += __shfl_xor_sync(kFull, nbroken, o);
  if (lane == 0 && valid && nbroken) v.fam_intact[f] -= nbroken;
  if (a.mode == 2) return;
  double F[D];
#pragma unroll
  for (int i = 0; i < D; i++) F[i] = acc[i];
  if (lane == 0 && valid) external_force<D>(a, node, F);
  warp_update<D, L, false>(a, F, valid ? node : -1);
}

template <int D, int LP, int LF>
__global__ void __launch_bounds__(256, 2) k_step_fp64(StepArgs a) {
  if ((int)blockIdx.x < a.pd_blocks) {
    fp64_family_item<D, LP>(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  } else {
    const int64_t t = (int64_t)(blockIdx.x - a.pd_blocks) * blockDim.x + threadIdx.x;
    feonly_item<D, LF, double, false>(a, a.v.ke64, t, LoadFp64<D>{a.u_n, a.v.bcflag, a.v.dtv});
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
    auto plain = [&](int n, double* out) {
#pragma unroll
      for (int i = 0; i < D; i++) out[i] = a.u[(int64_t)n * D + i];
    };
    const int j0 = v.fe_adj_ptr[node], j1 = v.fe_adj_ptr[node + 1];
    for (int j = j0 + lane; j < j1; j += L) {
      const int ent = v.fe_adj[j];
      fe_rows<D, double>(v, v.ke64, ent >> 3, ent & 7, plain, acc);
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

template <int D, int LP>
cudaError_t fp64_dispatch_lf(StepArgs a, int lf, int blocks, cudaStream_t s) {
  switch (lf) {
    case 1: k_step_fp64<D, LP, 1><<<blocks, 256, 0, s>>>(a); break;
    case 2: k_step_fp64<D, LP, 2><<<blocks, 256, 0, s>>>(a); break;
    case 4: k_step_fp64<D, LP, 4><<<blocks, 256, 0, s>>>(a); break;
    case 8: k_step_fp64<D, LP, 8><<<blocks, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int D>
cudaError_t fp64_dispatch(StepArgs a, int lp, int lf, cudaStream_t s) {
  const int pd_blocks = (int)(((int64_t)a.v.n_fam * lp + 255) / 256);
  const int fe_blocks = a.mode == 2 ? 0 : (int)(((int64_t)a.v.n_feonly * lf + 255) / 256);
  a.pd_blocks = pd_blocks;
  const int blocks = pd_blocks + fe_blocks;
  if (blocks == 0) return cudaSuccess;
  switch (lp) {
    case 4: return fp64_dispatch_lf<D, 4>(a, lf, blocks, s);
    case 8: return fp64_dispatch_lf<D, 8>(a, lf, blocks, s);
    case 16: return fp64_dispatch_lf<D, 16>(a, lf, blocks, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool step_lanes_valid(int lp, int lf) {
  return (lp == 4 || lp == 8 || lp == 16) && (lf == 1 || lf == 2 || lf == 4 || lf == 8);
}

cudaError_t launch_step(const StepArgs& a, int mixed, int lp, int lf, cudaStream_t s) {
  if (!step_lanes_valid(lp, lf)) return cudaErrorInvalidValue;
  if (mixed) return launch_step_mixed(a, lp, lf, s);
  return a.v.dim == 2 ? fp64_dispatch<2>(a, lp, lf, s) : fp64_dispatch<3>(a, lp, lf, s);
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
