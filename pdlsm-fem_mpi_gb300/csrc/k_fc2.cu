// FC 2: maximum-principal-stress bond breaking with an optional Top-K limit,
// as the reference runs it after every explicit step:
//   failureCriterion_maxPriSig (pdsolve.cpp:7184-7289): for every intact
//     bond (k, m), sigma1 = the largest eigenvalue of 0.5 (sigma_k + sigma_m)
//     (nodal stresses, 2D slots xx, yy, xy); bonds with sigma1 > sigma_ult
//     are candidates; Top-K keeps the K largest (K = 0: all);
//   Finally_TopK_andUpdate_bondStaus (:6981-7180, flag 2): every kept
//     candidate cuts a segment of half-length 0.5 min(delta) through the
//     bond's midpoint, normal to the principal direction of the largest
//     eigenvalue;
//   updateBondstate (:8910-9004) + intersection (:9081-9104): every intact
//     bond of the families of the nodes in the blocks around the segment
//     (its bounding box widened by one block) that crosses or touches the
//     segment breaks.
// The reference applies it in 2D only (failureProcess returns at once for a
// 3D model, :6594-6597).  Candidates are all found before any cut and cuts
// only clear bits, so the result does not depend on the candidates' order.
// The segment arithmetic uses non-fused multiplies and adds, as the
// reference's host code does; the 2x2 eigen-solve is closed form.
#include "device.h"

namespace pdx {

namespace {

// largest eigenvalue of the symmetric [[a, b], [b, c]] and its unit eigenvector
__device__ __forceinline__ double eig_max2(double a, double b, double c, double* e0, double* e1) {
  const double sm = 0.5 * (a + c), df = 0.5 * (a - c);
  const double l1 = sm + hypot(df, b);
  const double u0 = l1 - c, u1 = l1 - a;
  double v0, v1;
  if (b == 0.0 && u0 == 0.0 && u1 == 0.0) {
    v0 = 1.0;   // equal eigenvalues: the first eigenvector of a diagonal matrix
    v1 = 0.0;
  } else if (fabs(u0) >= fabs(u1)) {
    v0 = u0;
    v1 = b;
  } else {
    v0 = b;
    v1 = u1;
  }
  const double nv = sqrt(v0 * v0 + v1 * v1);
  *e0 = v0 / nv;
  *e1 = v1 / nv;
  return l1;
}

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// do the segments p1-p2 and q1-q2 cross or touch (the reference's test, same operation order)
__device__ bool segments_meet(const double* p1, const double* p2, const double* q1, const double* q2) {
  if (fmax(p1[0], p2[0]) < fmin(q1[0], q2[0]) || fmax(p1[1], p2[1]) < fmin(q1[1], q2[1]) ||
      fmax(q1[0], q2[0]) < fmin(p1[0], p2[0]) || fmax(q1[1], q2[1]) < fmin(p1[1], p2[1]))
    return false;
  const double d1 = sub(mul(sub(p1[0], q1[0]), sub(q2[1], q1[1])), mul(sub(p1[1], q1[1]), sub(q2[0], q1[0])));
  const double d2 = sub(mul(sub(p2[0], q1[0]), sub(q2[1], q1[1])), mul(sub(p2[1], q1[1]), sub(q2[0], q1[0])));
  if (mul(d1, d2) > 0) return false;
  const double d3 = sub(mul(sub(q1[0], p1[0]), sub(p2[1], p1[1])), mul(sub(q1[1], p1[1]), sub(p2[0], p1[0])));
  const double d4 = sub(mul(sub(q2[0], p1[0]), sub(p2[1], p1[1])), mul(sub(q2[1], p1[1]), sub(p2[0], p1[0])));
  if (mul(d3, d4) > 0) return false;
  return true;
}

__device__ __forceinline__ bool intact(const uint32_t* state, int b) { return (state[b >> 5] >> (b & 31)) & 1u; }

// one warp per family, lanes over its bonds
__global__ void k_fc2_candidates(Fc2Args a) {
  const DevView& v = a.v;
  const int f = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32);
  const int lane = threadIdx.x & 31;
  if (f >= v.n_fam) return;
  const int k = v.fam_node[f];
  const double* sk = a.sigma + (int64_t)k * 6;
  const double s0 = sk[0], s1 = sk[1], s3 = sk[3];
  for (int b = v.fam_ptr[f] + lane; b < v.fam_ptr[f + 1]; b += 32) {
    if (!intact(v.state, b)) continue;
    const double* sm = a.sigma + (int64_t)v.nbr[b] * 6;
    double e0, e1;
    const double l1 = eig_max2(0.5 * (s0 + sm[0]), 0.5 * (s3 + sm[3]), 0.5 * (s1 + sm[1]), &e0, &e1);
    // the largest sigma1 over intact bonds, from 0 (the quasi-static load ratio;
    // non-negative doubles order as their bit patterns)
    if (a.max_sigma1 && l1 > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(a.max_sigma1), (unsigned long long)__double_as_longlong(l1));
    if (l1 > a.sigult) {
      const int i = atomicAdd(a.count, 1);
      if (i < a.cap) {
        a.cand_val[i] = l1;
        a.cand_bond[i] = b;
        a.cand_fam[i] = f;
      }
    }
  }
}

// one warp per candidate (grid-stride over the count on the device)
__global__ void k_fc2_cut(Fc2Args a) {
  const DevView& v = a.v;
  const int lane = threadIdx.x & 31;
  const int nw = (int)((int64_t)gridDim.x * blockDim.x / 32);
  const int n = min(*a.count, a.cap);
  for (int c = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32); c < n; c += nw) {
    const int f = a.cand_fam[c], b = a.cand_bond[c];
    const int k = v.fam_node[f], m = v.nbr[b];
    const double* xk = v.X + (int64_t)k * 3;
    const double* xm = v.X + (int64_t)m * 3;
    const double xc0 = 0.5 * (xk[0] + xm[0]), xc1 = 0.5 * (xk[1] + xm[1]);
    const double* sk = a.sigma + (int64_t)k * 6;
    const double* sm = a.sigma + (int64_t)m * 6;
    double e0, e1;
    eig_max2(0.5 * (sk[0] + sm[0]), 0.5 * (sk[3] + sm[3]), 0.5 * (sk[1] + sm[1]), &e0, &e1);
    const double h = a.half_min_delta;
    const double q1[2] = {sub(xc0, mul(h, e1)), __dadd_rn(xc1, mul(h, e0))};
    const double q2[2] = {__dadd_rn(xc0, mul(h, e1)), sub(xc1, mul(h, e0))};
    const int ix0 = (int)((fmin(q1[0], q2[0]) - a.lbc0) / a.block_size);
    const int ix1 = (int)((fmax(q1[0], q2[0]) - a.lbc0) / a.block_size);
    const int iy0 = (int)((fmin(q1[1], q2[1]) - a.lbc1) / a.block_size);
    const int iy1 = (int)((fmax(q1[1], q2[1]) - a.lbc1) / a.block_size);
    for (int iy = iy0 - 1; iy < iy1 + 2; iy++) {
      if (iy < 0 || iy >= a.nby) continue;
      for (int ix = ix0 - 1; ix < ix1 + 2; ix++) {
        if (ix < 0 || ix >= a.nbx) continue;
        const int blk = ix + iy * a.nbx;
        for (int j = a.blk_ptr[blk]; j < a.blk_ptr[blk + 1]; j++) {
          const int f2 = a.blk_fam[j];
          const double* p1 = v.X + (int64_t)v.fam_node[f2] * 3;
          for (int b2 = v.fam_ptr[f2] + lane; b2 < v.fam_ptr[f2 + 1]; b2 += 32) {
            if (!intact(v.state, b2)) continue;
            const int m2 = v.nbr[b2];
            if (!segments_meet(p1, v.X + (int64_t)m2 * 3, q1, q2)) continue;
            const uint32_t bit = 1u << (b2 & 31);
            const uint32_t old = atomicAnd(&v.state[b2 >> 5], ~bit);
            if (old & bit) {
              atomicSub(&v.fam_intact[f2], 1);
              if (a.brec) reinterpret_cast<int*>(a.brec + b2)[3] = ~m2;
            }
          }
        }
      }
    }
  }
}

}  // namespace

cudaError_t launch_fc2_candidates(const Fc2Args& a, cudaStream_t s) {
  if (a.v.n_fam == 0) return cudaSuccess;
  const int blocks = (int)(((int64_t)a.v.n_fam * 32 + 255) / 256);
  k_fc2_candidates<<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fc2_cut(const Fc2Args& a, cudaStream_t s) {
  if (a.cap == 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>(((int64_t)a.cap * 32 + 255) / 256, 1024);
  k_fc2_cut<<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pdx
