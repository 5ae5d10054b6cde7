// FC 1 field samples on the interaction-integral path around a crack tip
// (2D).  The path points are chosen on the host (SIFsAndPropaDire_GaussPointPDnode,
// pdsolve.cpp:8514-8679); this kernel evaluates, from the displacements on
// the device, what the integrand needs at each point:
//   an FE element's centre (DispGradAndStressAndPqPx_FEM :8303-8408 at
//   p = q = 0): the bilinear map's Jacobian, its inverse, the shape-function
//   gradients, the displacement gradient and D times the strain;
//   a PD node (DispGrad :3254-3315 and the node stress of
//   calGlobalNodeStresses): the PDLSM gradient sum over the family's intact
//   bonds with the strain-operator columns omega*g*dv_m, and the node's
//   stress as computed for the output.
#include "device.h"

namespace pdx {

namespace {

__global__ void k_fc1_points(Fc1PointArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n_pts) return;
  const int* p = a.pts + (size_t)i * 5;
  const DevView& v = a.v;
  double* o = a.out + (size_t)i * 7;
  if (p[0] == 0) {
    // shape-function derivatives of the bilinear quad at its centre
    const double dNdp[4] = {-0.25, 0.25, 0.25, -0.25};
    const double dNdq[4] = {-0.25, -0.25, 0.25, 0.25};
    double x[4][2], ue[4][2];
    for (int n = 0; n < 4; n++) {
      const int node = p[1 + n];
      x[n][0] = v.X[(size_t)node * 3];
      x[n][1] = v.X[(size_t)node * 3 + 1];
      ue[n][0] = a.u[(size_t)node * 2];
      ue[n][1] = a.u[(size_t)node * 2 + 1];
    }
    double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
    for (int n = 0; n < 4; n++) {
      J00 += dNdp[n] * x[n][0];
      J01 += dNdp[n] * x[n][1];
      J10 += dNdq[n] * x[n][0];
      J11 += dNdq[n] * x[n][1];
    }
    const double det = J00 * J11 - J01 * J10;
    const double i00 = J11 / det, i01 = -J01 / det, i10 = -J10 / det, i11 = J00 / det;
    double g[4] = {0, 0, 0, 0};   // dux/dx, duy/dy, dux/dy, duy/dx
    for (int n = 0; n < 4; n++) {
      const double b1 = i00 * dNdp[n] + i01 * dNdq[n];
      const double b2 = i10 * dNdp[n] + i11 * dNdq[n];
      g[0] += b1 * ue[n][0];
      g[1] += b2 * ue[n][1];
      g[2] += b2 * ue[n][0];
      g[3] += b1 * ue[n][1];
    }
    const double eps[3] = {g[0], g[1], g[2] + g[3]};
    for (int r = 0; r < 4; r++) o[r] = g[r];
    for (int r = 0; r < 3; r++) o[4 + r] = a.D[r * 3] * eps[0] + a.D[r * 3 + 1] * eps[1] + a.D[r * 3 + 2] * eps[2];
    return;
  }
  const int k = p[1], f = p[2];
  const double ukx = a.u[(size_t)k * 2], uky = a.u[(size_t)k * 2 + 1];
  double g[4] = {0, 0, 0, 0};
  for (int b = v.fam_ptr[f]; b < v.fam_ptr[f + 1]; b++) {
    if (!((v.state[b >> 5] >> (b & 31)) & 1u)) continue;
    const int m = v.nbr[b];
    const double dux = a.u[(size_t)m * 2] - ukx, duy = a.u[(size_t)m * 2 + 1] - uky;
    const double c0 = v.cvec[b], c1 = v.cvec[v.n_bond + b];
    g[0] += c0 * dux;
    g[1] += c1 * duy;
    g[2] += c1 * dux;
    g[3] += c0 * duy;
  }
  for (int r = 0; r < 4; r++) o[r] = g[r];
  o[4] = a.sigma[(size_t)k * 6];
  o[5] = a.sigma[(size_t)k * 6 + 1];
  o[6] = a.sigma[(size_t)k * 6 + 3];
}

}  // namespace

cudaError_t launch_fc1_points(const Fc1PointArgs& a, cudaStream_t s) {
  if (a.n_pts <= 0) return cudaSuccess;
  k_fc1_points<<<(a.n_pts + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pdx
