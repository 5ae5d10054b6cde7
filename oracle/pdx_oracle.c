/*
 * CPU oracle of the PDLSM-FEM hot path (see pdx_oracle.h).  Test
 * infrastructure only: the checker of the CUDA path and the CPU baseline of
 * bench.py.  Plain C99 + OpenMP over families.
 *
 * Restated reference functions (SourceFiles/Solver/...):
 *   inflFunc                     pdsolve.cpp:1929-1935
 *   shapTens2D / shapTens3D      pdsolve.cpp:1938-2064
 *   vec_gd2D / vec_gd3D, PLUSolve pdsolve.cpp:2174-2232, calMatrixOperations.cpp:587-638
 *   matG2D / matG3D              pdsolve.cpp:2277-2347
 *   matH2D / matH3D + assembleInterWorkPD_CSRformat   pdsolve.cpp:2349-2416, 2524-2730
 *   matC2D / matC3D              pdsolve.cpp:3212-3398
 *   assemblePDBEwork_CSRformat (2D) :4049-4252, assemblePDBEwork3D_CSRformat :2732-2915,
 *   normMatArea                  :2917-2967
 *   Q4 / Hex8 eleStiffMatFEM, eleMassMat, eleFitStresses   pdfemEleQuad4N.cpp, pdfemEleBrick8N.cpp
 *   assembleSEDbyFEM_CSRformat   pdsolve.cpp:4882-5007
 *   assembleLumpedMass           :4618-4669
 *   pdfemDynamicSolver_CSRformat :5842-6090, timeIntegration_LM :5113-5132
 *   failureCriterion_stretch     :6643-6780 (s_c = s0, every bond over s_c breaks)
 *   calLocalDamage               :7338-7373
 *   calGlobalNodeStresses        :9540-9604 (calPDNodeStresses :9081, calFEMNodeStresses_EXP :9168)
 */
#include "pdx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_ctx {
  orc_model m;
  int nthreads, na, nv, nen, nd;
  int64_t nmem;
  double lam, mu, D[36];
  double* A;      /* n_fam*na*na */
  double* Gw;     /* nmem*dim*dim  omega*Lame(d) */
  double* gv;     /* nmem*dim */
  double* dv;     /* nmem*(3|6) */
  double* Kb;     /* nmem*dim*dim  dv_k dv_m G + P (PD-boundary) : row block of family k */
  double* cvec;   /* nmem*dim      omega g dv_m */
  double* Ke;     /* n_fe*nd*nd */
  double* Me;     /* n_fe*nd*nd */
  double* Bgp;    /* n_fe*ngp*nv*nd */
  double L[64];
  double* mass;   /* n_node */
  int* fam_of;    /* n_node */
  int* conn4;     /* n_elem*8: the model's connectivity, a 2D triangle's third node repeated in slot 4 */
};

/* ------------------------------------------------------------------ */

static double det3(const double m[3][3]) {
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

/* LU with partial pivoting, in place; returns 0 if singular */
static int lu_factor(double* a, int n, int* piv) {
  for (int j = 0; j < n; j++) {
    int p = j;
    double best = fabs(a[j * n + j]);
    for (int r = j + 1; r < n; r++)
      if (fabs(a[r * n + j]) > best) { best = fabs(a[r * n + j]); p = r; }
    piv[j] = p;
    if (best == 0.0) return 0;
    if (p != j)
      for (int c = 0; c < n; c++) { double t = a[j * n + c]; a[j * n + c] = a[p * n + c]; a[p * n + c] = t; }
    for (int r = j + 1; r < n; r++) {
      double l = a[r * n + j] / a[j * n + j];
      a[r * n + j] = l;
      for (int c = j + 1; c < n; c++) a[r * n + c] -= l * a[j * n + c];
    }
  }
  return 1;
}

static void lu_solve(const double* a, int n, const int* piv, double* x) {
  for (int j = 0; j < n; j++)
    if (piv[j] != j) { double t = x[j]; x[j] = x[piv[j]]; x[piv[j]] = t; }
  for (int r = 1; r < n; r++)
    for (int c = 0; c < r; c++) x[r] -= a[r * n + c] * x[c];
  for (int r = n - 1; r >= 0; r--) {
    double s = x[r];
    for (int c = r + 1; c < n; c++) s -= a[r * n + c] * x[c];
    x[r] = s / a[r * n + r];
  }
}

static void polyP(int dim, const double* x, double* P) {
  if (dim == 2) {
    P[0] = x[0]; P[1] = x[1]; P[2] = x[0] * x[0]; P[3] = x[1] * x[1]; P[4] = x[0] * x[1];
  } else {
    P[0] = x[0]; P[1] = x[1]; P[2] = x[2]; P[3] = x[0] * x[0]; P[4] = x[1] * x[1]; P[5] = x[2] * x[2];
    P[6] = x[0] * x[1]; P[7] = x[1] * x[2]; P[8] = x[2] * x[0];
  }
}

static void polyQ(int dim, const double* x, double* Q) {
  polyP(dim, x, Q);
  if (dim == 2) { Q[2] *= 0.5; Q[3] *= 0.5; }
  else { Q[3] *= 0.5; Q[4] *= 0.5; Q[5] *= 0.5; }
}

/* ---------------- FE (Q4 unit thickness, Hex8) --------------------- */

static const double PI8[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const double QI8[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const double RI8[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

static double bmat(int dim, const double (*xN)[3], double p, double q, double r, double* B /* nv x nd */) {
  if (dim == 2) {
    double dNdp[4] = {0.25 * (-1 + q), 0.25 * (1 - q), 0.25 * (1 + q), 0.25 * (-1 - q)};
    double dNdq[4] = {0.25 * (-1 + p), 0.25 * (-1 - p), 0.25 * (1 + p), 0.25 * (1 - p)};
    double J00 = 0, J01 = 0, J10 = 0, J11 = 0;
    for (int i = 0; i < 4; i++) {
      J00 += dNdp[i] * xN[i][0]; J01 += dNdp[i] * xN[i][1];
      J10 += dNdq[i] * xN[i][0]; J11 += dNdq[i] * xN[i][1];
    }
    double det = J00 * J11 - J01 * J10;
    memset(B, 0, sizeof(double) * 24);
    for (int i = 0; i < 4; i++) {
      double bx = (J11 * dNdp[i] - J01 * dNdq[i]) / det;
      double by = (-J10 * dNdp[i] + J00 * dNdq[i]) / det;
      B[0 * 8 + 2 * i] = bx;
      B[1 * 8 + 2 * i + 1] = by;
      B[2 * 8 + 2 * i] = by;
      B[2 * 8 + 2 * i + 1] = bx;
    }
    return det;
  }
  double dN[8][3], J[3][3] = {{0}};
  for (int i = 0; i < 8; i++) {
    dN[i][0] = 0.125 * PI8[i] * (1 + q * QI8[i]) * (1 + r * RI8[i]);
    dN[i][1] = 0.125 * QI8[i] * (1 + p * PI8[i]) * (1 + r * RI8[i]);
    dN[i][2] = 0.125 * RI8[i] * (1 + p * PI8[i]) * (1 + q * QI8[i]);
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) J[a][c] += dN[i][a] * xN[i][c];
  }
  double det = det3(J);
  double Jc[9];
  int piv[3];
  for (int a = 0; a < 3; a++)
    for (int c = 0; c < 3; c++) Jc[a * 3 + c] = J[a][c];
  lu_factor(Jc, 3, piv);
  memset(B, 0, sizeof(double) * 144);
  for (int i = 0; i < 8; i++) {
    double g[3] = {dN[i][0], dN[i][1], dN[i][2]};
    lu_solve(Jc, 3, piv, g);
    B[0 * 24 + 3 * i] = g[0];
    B[1 * 24 + 3 * i + 1] = g[1];
    B[2 * 24 + 3 * i + 2] = g[2];
    B[3 * 24 + 3 * i] = g[1];
    B[3 * 24 + 3 * i + 1] = g[0];
    B[4 * 24 + 3 * i + 1] = g[2];
    B[4 * 24 + 3 * i + 2] = g[1];
    B[5 * 24 + 3 * i] = g[2];
    B[5 * 24 + 3 * i + 2] = g[0];
  }
  return det;
}

/* 3-node triangle (pdfemEleTri3N.cpp) in the 4-node layout, fourth slot zero:
   K = ((B^T D) B) V with the constant-strain B, consistent mass rho V / 12
   (2 on the diagonal, 1 between like components), B at every stress point. */
static void triangle_matrices(const orc_ctx* c, const double (*xN)[3], double* Ke, double* Me, double* Bg) {
  const double mat[3][3] = {{1, xN[0][0], xN[0][1]}, {1, xN[1][0], xN[1][1]}, {1, xN[2][0], xN[2][1]}};
  const double V = 0.5 * fabs(det3(mat));
  const double b[3] = {xN[1][1] - xN[2][1], xN[2][1] - xN[0][1], xN[0][1] - xN[1][1]};
  const double cc[3] = {-xN[1][0] + xN[2][0], -xN[2][0] + xN[0][0], -xN[0][0] + xN[1][0]};
  double B[3][8];
  memset(B, 0, sizeof(B));
  for (int i = 0; i < 3; i++) {
    B[0][2 * i] = b[i] / (2.0 * V);
    B[1][2 * i + 1] = cc[i] / (2.0 * V);
    B[2][2 * i] = cc[i] / (2.0 * V);
    B[2][2 * i + 1] = b[i] / (2.0 * V);
  }
  double BtD[8][3];
  for (int i = 0; i < 8; i++)
    for (int k = 0; k < 3; k++) {
      double s = 0;
      for (int a = 0; a < 3; a++) s += B[a][i] * c->D[a * 3 + k];
      BtD[i][k] = s;
    }
  memset(Ke, 0, sizeof(double) * 64);
  memset(Me, 0, sizeof(double) * 64);
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += BtD[i][k] * B[k][j];
      Ke[i * 8 + j] = s * V;
    }
  const double fac = c->m.rho * V / 12.0;
  for (int r = 0; r < 6; r++)
    for (int q = 0; q < 6; q++)
      if ((r - q) % 2 == 0) Me[r * 8 + q] = r == q ? 2 * fac : fac;
  for (int g = 0; g < 4; g++) memcpy(Bg + (size_t)g * 24, B, sizeof(B));
}

static void element_matrices(const orc_ctx* c, const double (*xN)[3], double* Ke, double* Me, double* Bg) {
  const int dim = c->m.dim, nv = c->nv, nd = c->nd, nen = c->nen;
  const double g = 1.0 / sqrt(3.0), gp[2] = {-g, g};
  double B[144];
  memset(Ke, 0, sizeof(double) * nd * nd);
  memset(Me, 0, sizeof(double) * nd * nd);
  int ngp = dim == 2 ? 4 : 8;
  for (int t = 0; t < ngp; t++) {
    double p, q, r = 0;
    if (dim == 2) { p = gp[t >> 1]; q = gp[t & 1]; }
    else { p = gp[(t >> 2) & 1]; q = gp[(t >> 1) & 1]; r = gp[t & 1]; }
    double det = bmat(dim, xN, p, q, r, B);
    for (int i = 0; i < nd; i++)
      for (int j = 0; j < nd; j++) {
        double s = 0;
        for (int a = 0; a < nv; a++)
          for (int b = 0; b < nv; b++) s += B[a * nd + i] * c->D[a * nv + b] * B[b * nd + j];
        Ke[i * nd + j] += s * det;
      }
    double N[8];
    for (int k = 0; k < nen; k++)
      N[k] = dim == 2 ? 0.25 * (1 + p * PI8[k]) * (1 + q * QI8[k])
                      : 0.125 * (1 + p * PI8[k]) * (1 + q * QI8[k]) * (1 + r * RI8[k]);
    for (int a = 0; a < nen; a++)
      for (int b = 0; b < nen; b++)
        for (int d = 0; d < dim; d++) Me[(a * dim + d) * nd + b * dim + d] += c->m.rho * N[a] * N[b] * det;
  }
  /* B at the stress Gauss points, GP i closest to the reference's ordering */
  for (int t = 0; t < ngp; t++) {
    double p, q, r = 0;
    if (dim == 2) {
      /* eleFitStresses flag 1: q outer, p inner */
      p = gp[t & 1]; q = gp[t >> 1];
    } else {
      p = g * PI8[t]; q = g * QI8[t]; r = g * RI8[t];
    }
    bmat(dim, xN, p, q, r, Bg + (size_t)t * nv * nd);
  }
}

/* ------------------------------------------------------------------ */

orc_ctx* orc_create(const orc_model* m, int nthreads) {
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  c->m = *m;
#ifdef _OPENMP
  c->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  c->nthreads = 1;
#endif
  const int dim = m->dim;
  c->na = dim == 2 ? 5 : 9;
  c->nv = dim == 2 ? 3 : 6;
  c->nen = dim == 2 ? 4 : 8;
  c->nd = c->nen * dim;
  c->nmem = m->fam_off[m->n_fam];
  c->conn4 = (int*)malloc(sizeof(int) * (size_t)m->n_elem * 8);
  memcpy(c->conn4, m->conn, sizeof(int) * (size_t)m->n_elem * 8);
  for (int e = 0; e < m->n_elem; e++)
    if (dim == 2 && m->elem_nn[e] == 3) c->conn4[8 * e + 3] = c->conn4[8 * e + 2];
  c->m.conn = c->conn4;
  const double E = m->E, nu = m->nu;
  c->mu = 0.5 * E / (1 + nu);
  memset(c->D, 0, sizeof(c->D));
  if (dim == 2) {
    if (m->protype == 2) {
      c->lam = E * nu / ((1 - 2 * nu) * (1 + nu));
      double f = E / ((1 - 2 * nu) * (1 + nu));
      c->D[0] = f * (1 - nu); c->D[1] = f * nu; c->D[3] = f * nu; c->D[4] = f * (1 - nu); c->D[8] = f * 0.5 * (1 - 2 * nu);
    } else {
      c->lam = E * nu / (1 - nu * nu);
      c->D[0] = E / (1 - nu * nu); c->D[1] = E * nu / (1 - nu * nu); c->D[3] = c->D[1]; c->D[4] = c->D[0];
      c->D[8] = 0.5 * E / (1 + nu);
    }
  } else {
    c->lam = E * nu / ((1 - 2 * nu) * (1 + nu));
    double f = E / ((1.0 - 2.0 * nu) * (1.0 + nu));
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) c->D[i * 6 + j] = f * (i == j ? (1 - nu) : nu);
    for (int i = 3; i < 6; i++) c->D[i * 6 + i] = f * 0.5 * (1 - 2 * nu);
  }
  const int na = c->na, nv = c->nv, ndv = dim == 2 ? 3 : 6;
  c->A = (double*)calloc((size_t)m->n_fam * na * na, sizeof(double));
  c->Gw = (double*)calloc((size_t)c->nmem * dim * dim, sizeof(double));
  c->gv = (double*)calloc((size_t)c->nmem * dim, sizeof(double));
  c->dv = (double*)calloc((size_t)c->nmem * ndv, sizeof(double));
  c->Kb = (double*)calloc((size_t)c->nmem * dim * dim, sizeof(double));
  c->cvec = (double*)calloc((size_t)c->nmem * dim, sizeof(double));
  c->fam_of = (int*)malloc(sizeof(int) * m->n_node);
  for (int k = 0; k < m->n_node; k++) c->fam_of[k] = -1;
  for (int f = 0; f < m->n_fam; f++) c->fam_of[m->fam_members[m->fam_off[f]]] = f;
  /* PD-boundary weights W (dim x nv) per node */
  double* W = (double*)calloc((size_t)m->n_node * dim * nv, sizeof(double));
  for (int b = 0; b < m->n_pdbe; b++) {
    const int* id = m->pdbe + 4 * b;
    if (dim == 2) {
      const double* x1 = m->X + 3 * id[0];
      const double* x2 = m->X + 3 * id[1];
      double nx = x2[1] - x1[1], ny = x1[0] - x2[0];
      double w[6] = {0.5 * nx, 0, 0.5 * ny, 0, 0.5 * ny, 0.5 * nx};
      for (int t = 0; t < 2; t++)
        for (int i = 0; i < 6; i++) W[(size_t)id[t] * 6 + i] += w[i];
    } else {
      const double *x0 = m->X + 3 * id[0], *x1 = m->X + 3 * id[1], *x2 = m->X + 3 * id[2], *x3 = m->X + 3 * id[3];
      double v1[3], v2[3], n[3], n2[3];
      for (int i = 0; i < 3; i++) { v1[i] = x1[i] - x0[i]; v2[i] = x2[i] - x0[i]; }
      n[0] = v1[1] * v2[2] - v1[2] * v2[1]; n[1] = v2[0] * v1[2] - v1[0] * v2[2]; n[2] = v1[0] * v2[1] - v2[0] * v1[1];
      double A1 = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]), A2 = 0, w = 1.0 / 3;
      int quad = id[3] != id[2];
      if (quad) {
        for (int i = 0; i < 3; i++) { v1[i] = x3[i] - x0[i]; v2[i] = x2[i] - x0[i]; }
        n2[0] = v1[1] * v2[2] - v1[2] * v2[1]; n2[1] = v2[0] * v1[2] - v1[0] * v2[2]; n2[2] = v1[0] * v2[1] - v2[0] * v1[1];
        A2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
        w = 0.25;
      }
      double area = (A1 + A2) * 0.5;
      double N1 = n[0] / A1 * area * w, N2 = n[1] / A1 * area * w, N3 = n[2] / A1 * area * w;
      double Nm[18] = {N1, 0, 0, N2, 0, N3, 0, N2, 0, N1, N3, 0, 0, 0, N3, 0, N2, N1};
      for (int t = 0; t < (quad ? 4 : 3); t++)
        for (int i = 0; i < 18; i++) W[(size_t)id[t] * 18 + i] += Nm[i];
    }
  }
  int singular = 0;
  const double aa = m->nlf * m->nlf;
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 16) reduction(| : singular)
  for (int f = 0; f < m->n_fam; f++) {
    const int64_t q0 = m->fam_off[f], q1 = m->fam_off[f + 1];
    const int k = m->fam_members[q0];
    const double* xk = m->X + 3 * k;
    const double delta = m->fam_delta[f];
    double A[81], P[9], Q[9], LU[81];
    int piv[9];
    memset(A, 0, sizeof(A));
    for (int64_t q = q0 + 1; q < q1; q++) {
      const int mm = m->fam_members[q];
      double xi[3] = {m->X[3 * mm] - xk[0], m->X[3 * mm + 1] - xk[1], m->X[3 * mm + 2] - xk[2]};
      double om = exp(-(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) / aa / delta / delta);
      double w = om * m->vol_node[mm];
      polyP(dim, xi, P);
      polyQ(dim, xi, Q);
      for (int r = 0; r < na; r++)
        for (int cc = 0; cc < na; cc++) A[r * na + cc] += w * P[r] * Q[cc];
    }
    memcpy(c->A + (size_t)f * na * na, A, sizeof(double) * na * na);
    memcpy(LU, A, sizeof(double) * na * na);
    if (!lu_factor(LU, na, piv)) { singular = 1; continue; }
    const double* Wk = W + (size_t)k * dim * nv;
    int has_w = 0;
    for (int i = 0; i < dim * nv; i++) has_w |= Wk[i] != 0.0;
    double WD[18];
    for (int i = 0; i < dim; i++)
      for (int j = 0; j < nv; j++) {
        double s = 0;
        for (int t = 0; t < nv; t++) s += Wk[i * nv + t] * c->D[t * nv + j];
        WD[i * nv + j] = s;
      }
    for (int64_t q = q0 + 1; q < q1; q++) {
      const int mm = m->fam_members[q];
      double xi[3] = {m->X[3 * mm] - xk[0], m->X[3 * mm + 1] - xk[1], m->X[3 * mm + 2] - xk[2]};
      double om = exp(-(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]) / aa / delta / delta);
      double x[9];
      polyP(dim, xi, x);
      lu_solve(LU, na, piv, x);
      const double* d = x + dim;
      double G[9];
      const double lam = c->lam, mu = c->mu;
      if (dim == 2) {
        G[0] = om * ((2 * mu + lam) * d[0] + mu * d[1]);
        G[1] = om * (lam + mu) * d[2];
        G[2] = G[1];
        G[3] = om * ((2 * mu + lam) * d[1] + mu * d[0]);
      } else {
        double tr = d[0] + d[1] + d[2];
        G[0] = om * ((mu + lam) * d[0] + mu * tr);
        G[1] = om * (lam + mu) * d[3];
        G[2] = om * (lam + mu) * d[5];
        G[4] = om * ((mu + lam) * d[1] + mu * tr);
        G[5] = om * (lam + mu) * d[4];
        G[8] = om * ((mu + lam) * d[2] + mu * tr);
        G[3] = G[1]; G[6] = G[2]; G[7] = G[5];
      }
      const double dvm = m->vol_node[mm], dvk = m->fam_cdv[f];
      for (int i = 0; i < dim * dim; i++) {
        c->Gw[(size_t)q * dim * dim + i] = G[i];
        c->Kb[(size_t)q * dim * dim + i] = G[i] * dvm * dvk;
      }
      for (int i = 0; i < dim; i++) {
        c->gv[(size_t)q * dim + i] = x[i];
        c->cvec[(size_t)q * dim + i] = om * x[i] * dvm;
      }
      for (int i = 0; i < ndv; i++) c->dv[(size_t)q * ndv + i] = d[i];
      if (has_w) {
        /* P = -W D B(c): PD-boundary traction through the strain operator */
        const double* cv = c->cvec + (size_t)q * dim;
        double Bc[18];
        memset(Bc, 0, sizeof(Bc));
        if (dim == 2) {
          Bc[0 * 2 + 0] = cv[0]; Bc[1 * 2 + 1] = cv[1]; Bc[2 * 2 + 0] = cv[1]; Bc[2 * 2 + 1] = cv[0];
        } else {
          Bc[0 * 3 + 0] = cv[0]; Bc[1 * 3 + 1] = cv[1]; Bc[2 * 3 + 2] = cv[2];
          Bc[3 * 3 + 0] = cv[1]; Bc[3 * 3 + 1] = cv[0];
          Bc[4 * 3 + 1] = cv[2]; Bc[4 * 3 + 2] = cv[1];
          Bc[5 * 3 + 0] = cv[2]; Bc[5 * 3 + 2] = cv[0];
        }
        for (int i = 0; i < dim; i++)
          for (int j = 0; j < dim; j++) {
            double s = 0;
            for (int t = 0; t < nv; t++) s += WD[i * nv + t] * Bc[t * dim + j];
            c->Kb[(size_t)q * dim * dim + i * dim + j] -= s;
          }
      }
    }
  }
  free(W);
  if (singular) { orc_destroy(c); return NULL; }
  /* FE element matrices */
  const int nd = c->nd, ngp = c->nen;
  c->Ke = (double*)malloc(sizeof(double) * (size_t)m->n_fe * nd * nd);
  c->Me = (double*)malloc(sizeof(double) * (size_t)m->n_fe * nd * nd);
  c->Bgp = (double*)malloc(sizeof(double) * (size_t)m->n_fe * ngp * nv * nd);
#pragma omp parallel for num_threads(c->nthreads) schedule(static)
  for (int i = 0; i < m->n_fe; i++) {
    const int e = m->fe_idx[i];
    double xN[8][3];
    for (int j = 0; j < c->nen; j++)
      for (int a = 0; a < 3; a++) xN[j][a] = m->X[3 * c->conn4[8 * e + j] + a];
    if (dim == 2 && m->elem_nn[e] == 3)
      triangle_matrices(c, (const double(*)[3])xN, c->Ke + (size_t)i * nd * nd, c->Me + (size_t)i * nd * nd,
                        c->Bgp + (size_t)i * ngp * nv * nd);
    else
      element_matrices(c, (const double(*)[3])xN, c->Ke + (size_t)i * nd * nd, c->Me + (size_t)i * nd * nd,
                       c->Bgp + (size_t)i * ngp * nv * nd);
  }
  if (dim == 2) {
    double a = 1 + 0.5 * sqrt(3.0), b = -0.5, cc = 1 - 0.5 * sqrt(3.0);
    double r[16] = {a, b, cc, b, b, a, b, cc, cc, b, a, b, b, cc, b, a};
    memcpy(c->L, r, sizeof(r));
  } else {
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++)
        c->L[i * 8 + j] = 0.125 * (1 + PI8[j] * sqrt(3.0) * PI8[i]) * (1 + QI8[j] * sqrt(3.0) * QI8[i]) *
                          (1 + RI8[j] * sqrt(3.0) * RI8[i]);
  }
  /* lumped mass over all elements */
  c->mass = (double*)calloc(m->n_node, sizeof(double));
  for (int e = 0; e < m->n_elem; e++) {
    const int nn = m->elem_nn[e];
    for (int j = 0; j < nn; j++) c->mass[m->conn[8 * e + j]] += m->vol_elem[e] / nn * m->rho;
  }
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  free(c->A); free(c->Gw); free(c->gv); free(c->dv); free(c->Kb); free(c->cvec);
  free(c->Ke); free(c->Me); free(c->Bgp); free(c->mass); free(c->fam_of); free(c->conn4);
  free(c);
}

void orc_coeffs(const orc_ctx* c, double* A, double* g, double* d, double* G) {
  const orc_model* m = &c->m;
  const int dim = m->dim, ndv = dim == 2 ? 3 : 6;
  if (A) memcpy(A, c->A, sizeof(double) * (size_t)m->n_fam * c->na * c->na);
  int64_t b = 0;
  for (int f = 0; f < m->n_fam; f++)
    for (int64_t q = m->fam_off[f] + 1; q < m->fam_off[f + 1]; q++, b++) {
      if (g) memcpy(g + b * dim, c->gv + q * dim, sizeof(double) * dim);
      if (d) memcpy(d + b * ndv, c->dv + q * ndv, sizeof(double) * ndv);
      if (G) memcpy(G + b * dim * dim, c->Gw + q * dim * dim, sizeof(double) * dim * dim);
    }
}

/* f_node (n_node*dim) = internal force of every node */
static void node_force(const orc_ctx* c, const uint8_t* bs, const double* u, double* fn) {
  const orc_model* m = &c->m;
  const int dim = m->dim, nd = c->nd, nen = c->nen;
  memset(fn, 0, sizeof(double) * (size_t)m->n_node * dim);
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 64)
  for (int f = 0; f < m->n_fam; f++) {
    const int64_t q0 = m->fam_off[f], q1 = m->fam_off[f + 1];
    const int k = m->fam_members[q0];
    double acc[3] = {0, 0, 0};
    for (int64_t q = q0 + 1; q < q1; q++) {
      if (!bs[q]) continue;
      const int mm = m->fam_members[q];
      const double* K = c->Kb + q * dim * dim;
      for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) acc[i] += K[i * dim + j] * (u[(size_t)mm * dim + j] - u[(size_t)k * dim + j]);
    }
    for (int i = 0; i < dim; i++) fn[(size_t)k * dim + i] += acc[i];
  }
  for (int i = 0; i < m->n_fe; i++) {
    const int e = m->fe_idx[i];
    const double* K = c->Ke + (size_t)i * nd * nd;
    double ue[24];
    for (int j = 0; j < nen; j++)
      for (int a = 0; a < dim; a++) ue[j * dim + a] = u[(size_t)m->conn[8 * e + j] * dim + a];
    for (int r = 0; r < nd; r++) {
      double s = 0;
      for (int cc = 0; cc < nd; cc++) s += K[r * nd + cc] * ue[cc];
      fn[(size_t)m->conn[8 * e + r / dim] * dim + r % dim] -= s;
    }
  }
}

void orc_internal_force(const orc_ctx* c, const uint8_t* bs, const double* u_all, double* f_eq) {
  const orc_model* m = &c->m;
  const size_t nd = (size_t)m->n_node * m->dim;
  double* fn = (double*)malloc(sizeof(double) * nd);
  node_force(c, bs, u_all, fn);
  for (size_t i = 0; i < nd; i++)
    if (m->eq[i] >= 0) f_eq[m->eq[i]] = fn[i];
  free(fn);
}

void orc_lumped_mass(const orc_ctx* c, double* m_eq) {
  const orc_model* m = &c->m;
  for (int k = 0; k < m->n_node; k++)
    for (int i = 0; i < m->dim; i++)
      if (m->eq[k * m->dim + i] >= 0) m_eq[m->eq[k * m->dim + i]] = c->mass[k];
}

/* Per-bond uniform draw for FC 3 with a perturbed s0: murmur3's 32-bit
 * finaliser of (k, m, seed folded to 32 bits), top 24 bits / 2^24. */
double orc_bond_uniform(uint64_t seed, int k, int m) {
  uint32_t x = ((uint32_t)k * 0x9e3779b1u) ^ ((uint32_t)m + 0x7f4a7c15u) ^ (uint32_t)(seed ^ (seed >> 32));
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return (double)(x >> 8) * 0x1.0p-24;
}

static int64_t stretch_pass(const orc_ctx* c, const double* u, double s0, uint64_t seed, double pert, uint8_t* bs) {
  const orc_model* m = &c->m;
  const int dim = m->dim;
  int64_t nbroken = 0;
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 64) reduction(+ : nbroken)
  for (int f = 0; f < m->n_fam; f++) {
    const int64_t q0 = m->fam_off[f], q1 = m->fam_off[f + 1];
    const int k = m->fam_members[q0];
    double intact = 0;
    for (int64_t q = q0 + 1; q < q1; q++) intact += bs[q];
    double phi = 1.0 - intact / ((double)(q1 - q0) - 1.0);
    if (phi > 0.42) continue;
    /* decide on the states before the pass, then apply */
    int64_t cut[512];
    int ncut = 0;
    for (int64_t q = q0 + 1; q < q1; q++) {
      if (!bs[q]) continue;
      const int mm = m->fam_members[q];
      double xi[3] = {0, 0, 0}, eta[3] = {0, 0, 0};
      for (int i = 0; i < 3; i++) xi[i] = m->X[3 * mm + i] - m->X[3 * k + i];
      for (int i = 0; i < dim; i++) eta[i] = u[(size_t)mm * dim + i] - u[(size_t)k * dim + i];
      double mr = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
      double mg = sqrt((xi[0] + eta[0]) * (xi[0] + eta[0]) + (xi[1] + eta[1]) * (xi[1] + eta[1]) +
                       (xi[2] + eta[2]) * (xi[2] + eta[2]));
      double s = mg / mr - 1.0;
      double sc = pert == 0.0 ? s0 : s0 * (1.0 + pert * (2.0 * orc_bond_uniform(seed, k, mm) - 1.0));
      if (s > sc && ncut < 512) cut[ncut++] = q;
    }
    for (int i = 0; i < ncut; i++) bs[cut[i]] = 0;
    nbroken += ncut;
  }
  return nbroken;
}

int64_t orc_explicit(const orc_ctx* c, double dt, int nsteps, const uint8_t* pmask, const double* dtv, double s0,
                     uint64_t seed, double pert, double* u, uint8_t* bs, double* traj) {
  const orc_model* m = &c->m;
  const int dim = m->dim;
  const size_t nd = (size_t)m->n_node * dim;
  double* un = (double*)malloc(sizeof(double) * nd);
  double* unm1 = (double*)malloc(sizeof(double) * nd);
  double* uf = (double*)malloc(sizeof(double) * nd);
  double* fn = (double*)malloc(sizeof(double) * nd);
  int64_t broken = 0;
  memcpy(un, u, sizeof(double) * nd);
  memcpy(unm1, u, sizeof(double) * nd);
  for (int n = 0; n <= nsteps; n++) {
    /* prescribed values advance (setVaryEssentialBC), then the force */
    for (size_t i = 0; i < nd; i++) {
      const int k = (int)(i / dim), d = (int)(i % dim);
      uf[i] = (pmask[k] >> d) & 1 ? un[i] + dtv[3 * k + d] : un[i];
    }
    node_force(c, bs, uf, fn);
    for (size_t i = 0; i < nd; i++) {
      const int k = (int)(i / dim);
      double unew;
      if (m->eq[i] >= 0) {
        if (n == 0) {
          double a = fn[i] / c->mass[k];
          unew = a * (0.5 * dt * dt) + un[i];
        } else {
          double tempA = dt * dt * fn[i] / c->mass[k];
          unew = un[i] * 2.0 + tempA - unm1[i];
        }
      } else {
        unew = uf[i];
      }
      unm1[i] = un[i];
      u[i] = unew;
    }
    memcpy(un, u, sizeof(double) * nd);
    if (traj) memcpy(traj + (size_t)n * nd, un, sizeof(double) * nd);
    if (s0 > 0) broken += stretch_pass(c, un, s0, seed, pert, bs);
  }
  free(un); free(unm1); free(uf); free(fn);
  return broken;
}

void orc_stress(const orc_ctx* c, const uint8_t* bs, const double* u, double* sigma, double* phi) {
  const orc_model* m = &c->m;
  const int dim = m->dim, nv = c->nv, nd = c->nd, nen = c->nen, ngp = nen;
  int* cnt = (int*)calloc(m->n_node, sizeof(int));
  double* s = (double*)calloc((size_t)m->n_node * nv, sizeof(double));
  for (int f = 0; f < m->n_fam; f++) {
    const int64_t q0 = m->fam_off[f], q1 = m->fam_off[f + 1];
    const int k = m->fam_members[q0];
    double eps[6] = {0};
    double intact = 0;
    for (int64_t q = q0 + 1; q < q1; q++) {
      intact += bs[q];
      if (!bs[q]) continue;
      const int mm = m->fam_members[q];
      const double* cv = c->cvec + q * dim;
      double du[3] = {0, 0, 0};
      for (int i = 0; i < dim; i++) du[i] = u[(size_t)mm * dim + i] - u[(size_t)k * dim + i];
      if (dim == 2) {
        eps[0] += cv[0] * du[0]; eps[1] += cv[1] * du[1]; eps[2] += cv[1] * du[0] + cv[0] * du[1];
      } else {
        eps[0] += cv[0] * du[0]; eps[1] += cv[1] * du[1]; eps[2] += cv[2] * du[2];
        eps[3] += cv[1] * du[0] + cv[0] * du[1];
        eps[4] += cv[2] * du[1] + cv[1] * du[2];
        eps[5] += cv[2] * du[0] + cv[0] * du[2];
      }
    }
    for (int r = 0; r < nv; r++) {
      double a = 0;
      for (int t = 0; t < nv; t++) a += c->D[r * nv + t] * eps[t];
      s[(size_t)k * nv + r] = a;
    }
    cnt[k] = 1;
    if (phi) phi[k] = 1.0 - intact / ((double)(q1 - q0) - 1.0);
  }
  for (int i = 0; i < m->n_fe; i++) {
    const int e = m->fe_idx[i];
    double ue[24], sg[8][6];
    for (int j = 0; j < nen; j++)
      for (int a = 0; a < dim; a++) ue[j * dim + a] = u[(size_t)m->conn[8 * e + j] * dim + a];
    for (int g = 0; g < ngp; g++) {
      const double* B = c->Bgp + ((size_t)i * ngp + g) * nv * nd;
      double ep[6];
      for (int r = 0; r < nv; r++) {
        double a = 0;
        for (int t = 0; t < nd; t++) a += B[r * nd + t] * ue[t];
        ep[r] = a;
      }
      for (int r = 0; r < nv; r++) {
        double a = 0;
        for (int t = 0; t < nv; t++) a += c->D[r * nv + t] * ep[t];
        sg[g][r] = a;
      }
    }
    for (int j = 0; j < m->elem_nn[e]; j++) {   /* a triangle's repeated slot is not a node of it */
      const int node = m->conn[8 * e + j];
      for (int r = 0; r < nv; r++) {
        double a = 0;
        for (int g = 0; g < ngp; g++) a += c->L[j * ngp + g] * sg[g][r];
        s[(size_t)node * nv + r] += a;
      }
      cnt[node]++;
    }
  }
  for (int k = 0; k < m->n_node; k++) {
    double* o = sigma + (size_t)k * 6;
    const double* q = s + (size_t)k * nv;
    const double cc = (double)cnt[k];
    if (dim == 2) {
      o[0] = q[0] / cc; o[1] = q[1] / cc; o[2] = 0; o[3] = q[2] / cc; o[4] = 0; o[5] = 0;
      if (m->protype == 2) o[2] = m->nu * (o[0] + o[1]);
    } else {
      for (int r = 0; r < 6; r++) o[r] = q[r] / cc;
    }
    if (phi && c->fam_of[k] < 0) phi[k] = 0.0;
  }
  free(cnt);
  free(s);
}

static int64_t find_col(const int64_t* ia, const int64_t* ja, int64_t row, int64_t col) {
  int64_t lo = ia[row], hi = ia[row + 1];
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (ja[mid] == col) return mid;
    if (ja[mid] < col) lo = mid + 1; else hi = mid;
  }
  return -1;
}

void orc_assemble(const orc_ctx* c, const uint8_t* bs, const int64_t* ia, const int64_t* ja, const double* v_all,
                  double* a, double* f) {
  const orc_model* m = &c->m;
  const int dim = m->dim, nd = c->nd, nen = c->nen;
  memset(a, 0, sizeof(double) * (size_t)ia[m->n_eq]);
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 64)
  for (int f = 0; f < m->n_fam; f++) {
    const int64_t q0 = m->fam_off[f], q1 = m->fam_off[f + 1];
    const int k = m->fam_members[q0];
    double dsum[9] = {0};
    for (int64_t q = q0 + 1; q < q1; q++) {
      if (!bs[q]) continue;
      const int mm = m->fam_members[q];
      const double* K = c->Kb + q * dim * dim;
      for (int i = 0; i < dim; i++) {
        const int r = m->eq[k * dim + i];
        for (int j = 0; j < dim; j++) {
          dsum[i * dim + j] += K[i * dim + j];
          const int cl = m->eq[mm * dim + j];
          if (r >= 0 && cl >= 0) a[find_col(ia, ja, r, cl)] += -K[i * dim + j];
        }
      }
    }
    for (int i = 0; i < dim; i++) {
      const int r = m->eq[k * dim + i];
      for (int j = 0; j < dim; j++) {
        const int cl = m->eq[k * dim + j];
        if (r >= 0 && cl >= 0) a[find_col(ia, ja, r, cl)] += dsum[i * dim + j];
      }
    }
  }
  for (int i = 0; i < m->n_fe; i++) {
    const int e = m->fe_idx[i];
    const double* K = c->Ke + (size_t)i * nd * nd;
    for (int r = 0; r < nd; r++) {
      const int row = m->eq[m->conn[8 * e + r / dim] * dim + r % dim];
      if (row < 0) continue;
      for (int cc = 0; cc < nd; cc++) {
        const int col = m->eq[m->conn[8 * e + cc / dim] * dim + cc % dim];
        if (col >= 0) a[find_col(ia, ja, row, col)] += K[r * nd + cc];
      }
    }
  }
  (void)nen;
  if (f) orc_internal_force(c, bs, v_all, f);
}

void orc_consistent_mass(const orc_ctx* c, const int64_t* ia, const int64_t* ja, double* a) {
  const orc_model* m = &c->m;
  const int dim = m->dim, nd = c->nd;
  memset(a, 0, sizeof(double) * (size_t)ia[m->n_eq]);
  for (int i = 0; i < m->n_fe; i++) {
    const int e = m->fe_idx[i];
    const double* M = c->Me + (size_t)i * nd * nd;
    for (int r = 0; r < nd; r++) {
      const int row = m->eq[m->conn[8 * e + r / dim] * dim + r % dim];
      if (row < 0) continue;
      for (int cc = 0; cc < nd; cc++) {
        const int col = m->eq[m->conn[8 * e + cc / dim] * dim + cc % dim];
        if (col >= 0) a[find_col(ia, ja, row, col)] += M[r * nd + cc];
      }
    }
  }
  for (int f = 0; f < m->n_fam; f++) {
    const int k = m->fam_members[m->fam_off[f]];
    for (int i = 0; i < dim; i++) {
      const int r = m->eq[k * dim + i];
      if (r >= 0) a[find_col(ia, ja, r, r)] += m->fam_cdv[f] * m->rho;
    }
  }
}
