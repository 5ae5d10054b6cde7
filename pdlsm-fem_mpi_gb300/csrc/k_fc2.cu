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
// reference's host code does, and the 2x2 eigen-solves follow LAPACK's
// steps for that size (see sigma1_sterf and vec_steqr).
#include "device.h"

namespace pdx {

namespace {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// The reference takes sigma1 and its direction from LAPACK's dsyev on the
// 2x2 matrix [[d1, e], [e, d2]]: eigenvalues only ('N': dsytrd, dsterf) for
// the candidates, eigenvectors ('V': dsytrd, dorgtr, dsteqr) for the cut.
// For n = 2 dsytrd leaves d and e as they are and dorgtr gives the identity;
// below are the published LAPACK steps for that case (dsterf and dsteqr:
// split tests, the 2x2 block by dlae2 / dlaev2, ascending sort), in
// non-fused arithmetic, so that candidates and cut directions come out as
// the reference's do.  eps = 2^-53 and safmin = 2^-1022 (dlamch 'E', 'S').
constexpr double kEps = 0x1p-53, kEps2 = kEps * kEps, kSafmin = 0x1p-1022;

// dlae2: eigenvalues of [[a, b], [b, c]], rt1 the one of larger absolute
// value; with vec also dlaev2's unit eigenvector (cs1, sn1) for rt1
__device__ void lae2(double a, double b, double c, double* rt1, double* rt2, bool vec, double* cs1, double* sn1) {
  const double sm = add(a, c), df = sub(a, c), adf = fabs(df), tb = add(b, b), ab = fabs(tb);
  double acmx, acmn;
  if (fabs(a) > fabs(c)) {
    acmx = a;
    acmn = c;
  } else {
    acmx = c;
    acmn = a;
  }
  double rt;
  if (adf > ab) {
    const double q = ab / adf;
    rt = mul(adf, sqrt(add(1.0, mul(q, q))));
  } else if (adf < ab) {
    const double q = adf / ab;
    rt = mul(ab, sqrt(add(1.0, mul(q, q))));
  } else {
    rt = mul(ab, sqrt(2.0));
  }
  int sgn1;
  if (sm < 0.0) {
    *rt1 = mul(0.5, sub(sm, rt));
    sgn1 = -1;
    *rt2 = sub(mul(acmx / *rt1, acmn), mul(b / *rt1, b));
  } else if (sm > 0.0) {
    *rt1 = mul(0.5, add(sm, rt));
    sgn1 = 1;
    *rt2 = sub(mul(acmx / *rt1, acmn), mul(b / *rt1, b));
  } else {
    *rt1 = mul(0.5, rt);
    *rt2 = mul(-0.5, rt);
    sgn1 = 1;
  }
  if (!vec) return;
  double cs;
  int sgn2;
  if (df >= 0.0) {
    cs = add(df, rt);
    sgn2 = 1;
  } else {
    cs = sub(df, rt);
    sgn2 = -1;
  }
  if (fabs(cs) > ab) {
    const double ct = -tb / cs;
    *sn1 = 1.0 / sqrt(add(1.0, mul(ct, ct)));
    *cs1 = mul(ct, *sn1);
  } else if (ab == 0.0) {
    *cs1 = 1.0;
    *sn1 = 0.0;
  } else {
    const double tn = -cs / tb;
    *cs1 = 1.0 / sqrt(add(1.0, mul(tn, tn)));
    *sn1 = mul(tn, *cs1);
  }
  if (sgn1 == sgn2) {
    const double tn = *cs1;
    *cs1 = -*sn1;
    *sn1 = tn;
  }
}

// the split test both dsterf and dsteqr make first
__device__ __forceinline__ bool split_first(double d1, double e, double d2) {
  return e == 0.0 || fabs(e) <= mul(mul(sqrt(fabs(d1)), sqrt(fabs(d2))), kEps);
}

// largest eigenvalue as dsyev('N') gives it (dsterf)
__device__ double sigma1_sterf(double d1, double e, double d2) {
  if (d1 == 0.0 && d2 == 0.0 && e == 0.0) return 0.0;
  if (split_first(d1, e, d2)) return fmax(d1, d2);
  const double e2 = mul(e, e);
  if (e2 <= mul(kEps2, fabs(mul(d1, d2)))) return fmax(d1, d2);
  double rt1, rt2, c, s;
  lae2(d1, sqrt(e2), d2, &rt1, &rt2, false, &c, &s);
  return fmax(rt1, rt2);
}

// eigenvector of the largest eigenvalue as dsyev('V') gives it (dsteqr, then
// the first maximum of the ascending eigenvalues), before the reference's
// normalisation
__device__ void vec_steqr(double d1, double e, double d2, double* v0, double* v1) {
  bool split = split_first(d1, e, d2);
  if (!split) {
    // second test, in the order of the QL or the QR sweep
    const double tst = mul(fabs(e), fabs(e));
    const double lim = fabs(d2) < fabs(d1) ? add(mul(mul(kEps2, fabs(d2)), fabs(d1)), kSafmin)
                                           : add(mul(mul(kEps2, fabs(d1)), fabs(d2)), kSafmin);
    split = tst <= lim;
  }
  if (split) {
    // identity eigenvectors; ascending sort swaps them when d2 < d1
    if (d2 > d1) {
      *v0 = 0.0;
      *v1 = 1.0;
    } else {
      *v0 = 1.0;
      *v1 = 0.0;
    }
    return;
  }
  double rt1, rt2, c, s;
  lae2(d1, e, d2, &rt1, &rt2, true, &c, &s);
  // columns (c, s) for rt1 and (-s, c) for rt2
  if (rt2 > rt1) {
    *v0 = -s;
    *v1 = c;
  } else {
    *v0 = c;
    *v1 = s;
  }
}

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
    const double l1 = sigma1_sterf(0.5 * (s0 + sm[0]), 0.5 * (s3 + sm[3]), 0.5 * (s1 + sm[1]));
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
    vec_steqr(0.5 * (sk[0] + sm[0]), 0.5 * (sk[3] + sm[3]), 0.5 * (sk[1] + sm[1]), &e0, &e1);
    // the reference normalises: eigV / sqrt(e0^2 + e1^2 + 0^2)
    const double nrm = sqrt(add(add(mul(e0, e0), mul(e1, e1)), 0.0));
    e0 = e0 / nrm;
    e1 = e1 / nrm;
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
