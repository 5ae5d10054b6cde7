// Host finite-element utilities for Q4 (2D, unit thickness) and Hex8 (3D)
// elements, in FP64: element volume and centre, constitutive matrix D,
// stiffness Ke = sum_gp B^T D B w detJ with 2-point Gauss rules, consistent
// mass, strain-displacement matrices at the stress Gauss points, the
// Gauss-to-node stress extrapolation matrix, and equivalent nodal forces of a
// unit traction.  Formulation and Gauss-point orderings follow
// pdfemEleQuad4N.cpp (detJacobi :51-70, eleFitStresses :73-131, eleVolume
// :222-250, BmatFEM :276-318, eleStiffMatFEM :320-359), pdfemEleBrick8N.cpp
// (shapeFunction, JacobiMat, BmatFEM, eleStiffMatFEM, eleVolume, eleFitStresses),
// pdfemEleLine2N.cpp:45-75, pdsolve.cpp:36-94 (D) and :9218-9247 (2D L).
#include <cmath>
#include <cstring>
#include <vector>

#include "model.h"

namespace pdx {

namespace {

const double kG = 1.0 / std::sqrt(3.0);   // 2-point Gauss abscissa, weight 1
const double kPI[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
const double kQI[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
const double kRI[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

// 3x3 determinant as the sum of the three wrapped diagonal products minus
// the three anti-diagonal ones, accumulated in that order (pdfemEles::detMat33,
// pdfemEles.cpp:155-172, and pdfemEleBrick8N::detJacobi use this scheme).
double det33(const double m[3][3]) {
  double det = 0.0;
  for (int i = 0; i < 3; i++) {
    double a1 = 1., a2 = 1.;
    for (int j = 0; j < 3; j++) {
      a1 *= m[j][(i + j) % 3];
      a2 *= m[j][(i - j + 3) % 3];
    }
    det = det + a1 - a2;
  }
  return det;
}

// dN/dx, dN/dy of Q4 at (p, q); returns detJ.
double quad4_dN(const double xN[4][3], double p, double q, double dx[4], double dy[4]) {
  const double dNdp[4] = {0.25 * (-1 + q), 0.25 * (1 - q), 0.25 * (1 + q), 0.25 * (-1 - q)};
  const double dNdq[4] = {0.25 * (-1 + p), 0.25 * (-1 - p), 0.25 * (1 + p), 0.25 * (1 - p)};
  double J[2][2] = {{0, 0}, {0, 0}};
  for (int i = 0; i < 4; i++) {
    J[0][0] += dNdp[i] * xN[i][0];
    J[0][1] += dNdp[i] * xN[i][1];
    J[1][0] += dNdq[i] * xN[i][0];
    J[1][1] += dNdq[i] * xN[i][1];
  }
  const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const double i00 = J[1][1] / det, i01 = -J[0][1] / det, i10 = -J[1][0] / det, i11 = J[0][0] / det;
  for (int i = 0; i < 4; i++) {
    dx[i] = i00 * dNdp[i] + i01 * dNdq[i];
    dy[i] = i10 * dNdp[i] + i11 * dNdq[i];
  }
  return det;
}

// dN/dX (8 x 3) of Hex8 at (p, q, r) by solving J dNdX = dNdpqr; returns detJ.
double hex8_dN(const double xN[8][3], double p, double q, double r, double dX[8][3]) {
  double dN[8][3];
  for (int i = 0; i < 8; i++) {
    dN[i][0] = 0.125 * kPI[i] * (1 + q * kQI[i]) * (1 + r * kRI[i]);
    dN[i][1] = 0.125 * kQI[i] * (1 + p * kPI[i]) * (1 + r * kRI[i]);
    dN[i][2] = 0.125 * kRI[i] * (1 + p * kPI[i]) * (1 + q * kQI[i]);
  }
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int c = 0; c < 3; c++)
    for (int i = 0; i < 8; i++) {
      J[0][c] += dN[i][0] * xN[i][c];
      J[1][c] += dN[i][1] * xN[i][c];
      J[2][c] += dN[i][2] * xN[i][c];
    }
  const double det = det33(J);
  double inv[3][3];
  inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  for (int i = 0; i < 8; i++)
    for (int a = 0; a < 3; a++) dX[i][a] = inv[a][0] * dN[i][0] + inv[a][1] * dN[i][1] + inv[a][2] * dN[i][2];
  return det;
}

void b_quad4_at(const double xN[4][3], double p, double q, double B[3][8], double* detJ) {
  double dx[4], dy[4];
  double det = quad4_dN(xN, p, q, dx, dy);
  std::memset(B, 0, sizeof(double) * 24);
  for (int i = 0; i < 4; i++) {
    B[0][2 * i] = dx[i];
    B[1][2 * i + 1] = dy[i];
    B[2][2 * i] = dy[i];
    B[2][2 * i + 1] = dx[i];
  }
  if (detJ) *detJ = det;
}

void b_hex8_at(const double xN[8][3], double p, double q, double r, double B[6][24], double* detJ) {
  double dX[8][3];
  double det = hex8_dN(xN, p, q, r, dX);
  std::memset(B, 0, sizeof(double) * 144);
  for (int i = 0; i < 8; i++) {
    B[0][3 * i] = dX[i][0];
    B[1][3 * i + 1] = dX[i][1];
    B[2][3 * i + 2] = dX[i][2];
    B[3][3 * i] = dX[i][1];
    B[3][3 * i + 1] = dX[i][0];
    B[4][3 * i + 1] = dX[i][2];
    B[4][3 * i + 2] = dX[i][1];
    B[5][3 * i] = dX[i][2];
    B[5][3 * i + 2] = dX[i][0];
  }
  if (detJ) *detJ = det;
}

template <int NV, int ND>
void add_btdb(const double B[NV][ND], const double* D, double w, double* K) {
  double DB[NV][ND];
  for (int r = 0; r < NV; r++)
    for (int c = 0; c < ND; c++) {
      double s = 0;
      for (int k = 0; k < NV; k++) s += D[r * NV + k] * B[k][c];
      DB[r][c] = s;
    }
  for (int i = 0; i < ND; i++)
    for (int j = 0; j < ND; j++) {
      double s = 0;
      for (int k = 0; k < NV; k++) s += B[k][i] * DB[k][j];
      K[i * ND + j] += s * w;
    }
}

}  // namespace

double elem_volume(const Mesh& m, int e) {
  const int* c = &m.conn[(size_t)e * 8];
  auto X = [&](int j, int a) { return m.X[(size_t)c[j] * 3 + a]; };
  if (m.dim == 2) {
    double a1[3][3] = {{1, X(0, 0), X(0, 1)}, {1, X(1, 0), X(1, 1)}, {1, X(2, 0), X(2, 1)}};
    if (m.elem_nn[e] == 3) return 0.5 * std::fabs(det33(a1));   // pdfemEleTri3N::eleVolume
    double a2[3][3] = {{1, X(2, 0), X(2, 1)}, {1, X(3, 0), X(3, 1)}, {1, X(0, 0), X(0, 1)}};
    return 0.5 * std::fabs(det33(a1)) + 0.5 * std::fabs(det33(a2));
  }
  double xN[8][3];
  for (int j = 0; j < 8; j++)
    for (int a = 0; a < 3; a++) xN[j][a] = X(j, a);
  const double g[2] = {-kG, kG};
  double V = 0;
  for (int ip = 0; ip < 2; ip++)
    for (int iq = 0; iq < 2; iq++)
      for (int ir = 0; ir < 2; ir++) {
        double dX[8][3];
        V += hex8_dN(xN, g[ip], g[iq], g[ir], dX);
      }
  return V;
}

void elem_center(const Mesh& m, int e, double xc[3]) {
  const int nn = m.elem_nn[e];
  if (nn == 3) {   // pdfemEleTri3N::eleCenter
    const int* c = &m.conn[(size_t)e * 8];
    for (int a = 0; a < 3; a++)
      xc[a] = (m.X[(size_t)c[0] * 3 + a] + m.X[(size_t)c[1] * 3 + a] + m.X[(size_t)c[2] * 3 + a]) / 3.0;
    return;
  }
  const double w = nn == 4 ? 0.25 : 0.125;
  xc[0] = xc[1] = xc[2] = 0;
  for (int j = 0; j < nn; j++)
    for (int a = 0; a < 3; a++) xc[a] += m.X[(size_t)m.conn[(size_t)e * 8 + j] * 3 + a] * w;
}

void material_D(const Mesh& m, std::vector<double>& D, double& lambda, double& mu) {
  const double E = m.E, nu = m.nu;
  mu = 0.5 * E / (1 + nu);
  if (m.dim == 2) {
    D.assign(9, 0.0);
    if (m.protype == 2) {
      lambda = E * nu / ((1 - 2 * nu) * (1 + nu));
      const double f = E / ((1 - 2 * nu) * (1 + nu));
      D[0] = f * (1 - nu); D[1] = f * nu; D[3] = f * nu; D[4] = f * (1 - nu); D[8] = f * 0.5 * (1 - 2 * nu);
    } else {
      lambda = E * nu / (1 - nu * nu);
      D[0] = E / (1 - nu * nu); D[1] = E * nu / (1 - nu * nu); D[3] = D[1]; D[4] = D[0]; D[8] = 0.5 * E / (1 + nu);
    }
  } else {
    lambda = E * nu / ((1 - 2 * nu) * (1 + nu));
    D.assign(36, 0.0);
    const double f = E / ((1.0 - 2.0 * nu) * (1.0 + nu));
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) D[i * 6 + j] = f * (i == j ? (1 - nu) : nu);
    for (int i = 3; i < 6; i++) D[i * 6 + i] = f * 0.5 * (1 - 2 * nu);
  }
}

void ke_quad4(const double xN[4][3], const double* D, double* Ke) {
  std::memset(Ke, 0, sizeof(double) * 64);
  const double g[2] = {-kG, kG};
  for (int m = 0; m < 2; m++)
    for (int n = 0; n < 2; n++) {
      double B[3][8], det;
      b_quad4_at(xN, g[m], g[n], B, &det);
      add_btdb<3, 8>(B, D, det, Ke);
    }
}

void ke_hex8(const double xN[8][3], const double* D, double* Ke) {
  std::memset(Ke, 0, sizeof(double) * 576);
  const double g[2] = {-kG, kG};
  for (int ir = 0; ir < 2; ir++)
    for (int iq = 0; iq < 2; iq++)
      for (int ip = 0; ip < 2; ip++) {
        double B[6][24], det;
        b_hex8_at(xN, g[ip], g[iq], g[ir], B, &det);
        add_btdb<6, 24>(B, D, det, Ke);
      }
}

void me_quad4(const double xN[4][3], double rho, double* Me) {
  std::memset(Me, 0, sizeof(double) * 64);
  const double g[2] = {-kG, kG};
  for (int ip = 0; ip < 2; ip++)
    for (int iq = 0; iq < 2; iq++) {
      const double p = g[ip], q = g[iq];
      double dx[4], dy[4];
      const double det = quad4_dN(xN, p, q, dx, dy);
      const double N[4] = {0.25 * (1 - p) * (1 - q), 0.25 * (1 + p) * (1 - q), 0.25 * (1 + p) * (1 + q),
                           0.25 * (1 - p) * (1 + q)};
      for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++)
          for (int d = 0; d < 2; d++) Me[(2 * a + d) * 8 + 2 * b + d] += rho * N[a] * N[b] * det;
    }
}

void me_hex8(const double xN[8][3], double rho, double* Me) {
  std::memset(Me, 0, sizeof(double) * 576);
  const double g[2] = {-kG, kG};
  for (int ip = 0; ip < 2; ip++)
    for (int iq = 0; iq < 2; iq++)
      for (int ir = 0; ir < 2; ir++) {
        const double p = g[ip], q = g[iq], r = g[ir];
        double dX[8][3];
        const double det = hex8_dN(xN, p, q, r, dX);
        double N[8];
        for (int i = 0; i < 8; i++) N[i] = 0.125 * (1 + p * kPI[i]) * (1 + q * kQI[i]) * (1 + r * kRI[i]);
        for (int a = 0; a < 8; a++)
          for (int b = 0; b < 8; b++)
            for (int d = 0; d < 3; d++) Me[(3 * a + d) * 24 + 3 * b + d] += N[a] * N[b] * rho * det;
      }
}

void b_gauss_quad4(const double xN[4][3], double* B) {
  const double g[2] = {-kG, kG};
  int cnt = 0;
  for (int nq = 0; nq < 2; nq++)
    for (int np = 0; np < 2; np++) {
      double b[3][8];
      b_quad4_at(xN, g[np], g[nq], b, nullptr);
      std::memcpy(B + (size_t)cnt * 24, b, sizeof(b));
      cnt++;
    }
}

// 3-node triangle (constant strain, pdfemEleTri3N.cpp): B = [b; c] / 2A with
// b_i = y_j - y_k, c_i = x_k - x_j over the cyclic (i, j, k).  The element is
// stored in the 4-node tables with its third node repeated in the fourth slot,
// whose rows and columns stay zero.
namespace {
void b_tri3(const double xN[4][3], double B[3][8]) {
  double a[3][3] = {{1, xN[0][0], xN[0][1]}, {1, xN[1][0], xN[1][1]}, {1, xN[2][0], xN[2][1]}};
  const double V2 = 2.0 * (0.5 * std::fabs(det33(a)));
  const double b[3] = {xN[1][1] - xN[2][1], xN[2][1] - xN[0][1], xN[0][1] - xN[1][1]};
  const double c[3] = {-xN[1][0] + xN[2][0], -xN[2][0] + xN[0][0], -xN[0][0] + xN[1][0]};
  std::memset(B, 0, sizeof(double) * 24);
  for (int i = 0; i < 3; i++) {
    B[0][2 * i] = b[i] / V2;
    B[1][2 * i + 1] = c[i] / V2;
    B[2][2 * i] = c[i] / V2;
    B[2][2 * i + 1] = b[i] / V2;
  }
}
}  // namespace

void ke_tri3(const double xN[4][3], const double* D, double* Ke) {
  std::memset(Ke, 0, sizeof(double) * 64);
  double B[3][8];
  b_tri3(xN, B);
  double a[3][3] = {{1, xN[0][0], xN[0][1]}, {1, xN[1][0], xN[1][1]}, {1, xN[2][0], xN[2][1]}};
  add_btdb<3, 8>(B, D, 0.5 * std::fabs(det33(a)), Ke);
}

void me_tri3(const double xN[4][3], double rho, double* Me) {
  std::memset(Me, 0, sizeof(double) * 64);
  double a[3][3] = {{1, xN[0][0], xN[0][1]}, {1, xN[1][0], xN[1][1]}, {1, xN[2][0], xN[2][1]}};
  const double fac = rho * (0.5 * std::fabs(det33(a))) / 12.0;
  for (int r = 0; r < 6; r++)
    for (int c = 0; c < 6; c++)
      if ((r - c) % 2 == 0) Me[r * 8 + c] = r == c ? 2 * fac : fac;
}

void b_gauss_tri3(const double xN[4][3], double* B) {
  double b[3][8];
  b_tri3(xN, b);
  for (int g = 0; g < 4; g++) std::memcpy(B + (size_t)g * 24, b, sizeof(b));
}

void b_gauss_hex8(const double xN[8][3], double* B) {
  for (int i = 0; i < 8; i++) {
    double b[6][24];
    b_hex8_at(xN, kG * kPI[i], kG * kQI[i], kG * kRI[i], b, nullptr);
    std::memcpy(B + (size_t)i * 144, b, sizeof(b));
  }
}

void extrap_L(int dim, double* L) {
  if (dim == 2) {
    const double a = 1 + 0.5 * std::sqrt(3.0), b = -0.5, c = 1 - 0.5 * std::sqrt(3.0);
    const double r[4][4] = {{a, b, c, b}, {b, a, b, c}, {c, b, a, b}, {b, c, b, a}};
    std::memcpy(L, r, sizeof(r));
    return;
  }
  for (int i = 0; i < 8; i++) {
    const double p = std::sqrt(3.0) * kPI[i], q = std::sqrt(3.0) * kQI[i], r = std::sqrt(3.0) * kRI[i];
    for (int j = 0; j < 8; j++) L[i * 8 + j] = 0.125 * (1 + kPI[j] * p) * (1 + kQI[j] * q) * (1 + kRI[j] * r);
  }
}

void nbc_unit_force(int dim, const double xN[4][3], double* Fe) {
  const double g[2] = {-kG, kG};
  if (dim == 2) {
    for (int i = 0; i < 4; i++) Fe[i] = 0;
    for (int m = 0; m < 2; m++) {
      const double p = g[m];
      const double N[2] = {0.5 * (1 - p), 0.5 * (1 + p)};
      const double dy = -0.5 * xN[0][1] + 0.5 * xN[1][1];
      const double dx = -0.5 * xN[0][0] + 0.5 * xN[1][0];
      for (int ii = 0; ii < 2; ii++) {
        Fe[ii * 2] += N[ii] * dy;
        Fe[ii * 2 + 1] += N[ii] * (-dx);
      }
    }
    return;
  }
  for (int i = 0; i < 12; i++) Fe[i] = 0;
  for (int mp = 0; mp < 2; mp++)
    for (int mq = 0; mq < 2; mq++) {
      const double p = g[mp], q = g[mq];
      const double N[4] = {0.25 * (1 - p) * (1 - q), 0.25 * (1 + p) * (1 - q), 0.25 * (1 + p) * (1 + q),
                           0.25 * (1 - p) * (1 + q)};
      const double dNdp[4] = {0.25 * (-1 + q), 0.25 * (1 - q), 0.25 * (1 + q), 0.25 * (-1 - q)};
      const double dNdq[4] = {0.25 * (-1 + p), 0.25 * (-1 - p), 0.25 * (1 + p), 0.25 * (1 - p)};
      double xp[3] = {0, 0, 0}, xq[3] = {0, 0, 0};
      for (int a = 0; a < 3; a++)
        for (int j = 0; j < 4; j++) { xp[a] += dNdp[j] * xN[j][a]; xq[a] += dNdq[j] * xN[j][a]; }
      const double n[3] = {xp[1] * xq[2] - xp[2] * xq[1], xq[0] * xp[2] - xp[0] * xq[2], xp[0] * xq[1] - xq[0] * xp[1]};
      for (int k = 0; k < 4; k++)
        for (int a = 0; a < 3; a++) Fe[3 * k + a] += N[k] * n[a];
    }
}

}  // namespace pdx
