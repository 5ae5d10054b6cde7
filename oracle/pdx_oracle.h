/*
 * CPU oracle of the PDLSM-FEM hot path: a plain-C restatement of the
 * reference's algorithm, used only as the checker in tests/, in smoke() and
 * as the CPU baseline leg of bench.py.  It is test infrastructure and is never
 * called by the product library.  Its results are pinned against FP64 dumps
 * of the reference itself (tests/golden/, made by oracle/ref).
 *
 * Inputs are the model arrays of the host setup (families in the reference's
 * member layout, element connectivity, equation numbers).  Every function
 * names the reference function it restates.
 */
#ifndef PDX_ORACLE_H
#define PDX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model {
  int dim, protype, n_node, n_elem, n_eq, n_fam, n_pdbe, n_fe;
  const double* X;          /* n_node*3 */
  const int* conn;          /* n_elem*8, 0-based */
  const int* elem_nn;       /* n_elem */
  const int* fe_idx;        /* n_fe element indices */
  const int* eq;            /* n_node*dim, -1 prescribed */
  const double* vol_node;   /* n_node */
  const double* vol_elem;   /* n_elem */
  const int64_t* fam_off;   /* n_fam+1, member layout (member 0 = node) */
  const int* fam_members;   /* 0-based */
  const double* fam_delta;
  const double* fam_cdv;
  const int* pdbe;          /* n_pdbe*4, 0-based (2D uses 2) */
  double E, nu, rho, nlf;
} orc_model;

typedef struct orc_ctx orc_ctx;

/* Builds moment matrices, bond coefficients (bond state 1), PD-boundary
 * weights, FE stiffness matrices and the lumped mass.  NULL on a singular
 * moment matrix. nthreads <= 0 uses all host threads. */
orc_ctx* orc_create(const orc_model* m, int nthreads);
void orc_destroy(orc_ctx* c);

/* A (n_fam*na*na), g (members-1 per family * dim), d, G (dim*dim) in member
 * order with member 0 skipped. */
void orc_coeffs(const orc_ctx* c, double* A, double* g, double* d, double* G);

/* F[eq] = -(K u)[eq], calinternalForce_CSRformat, explicit form. */
void orc_internal_force(const orc_ctx* c, const uint8_t* bond_state, const double* u_all, double* f_eq);

/* Lumped mass per equation (assembleLumpedMass). */
void orc_lumped_mass(const orc_ctx* c, double* m_eq);

/* Explicit central-difference run with critical-stretch failure
 * (pdfemDynamicSolver_CSRformat + failureCriterion_stretch with s_c = s0).
 * u_all: in u0 (prescribed values at their EBC value), out u after the run;
 * dtv: n_node*3 prescribed increments (dt * velocity), 0 for fixed DOFs;
 * bond_state: in/out member layout; s0 <= 0 disables failure;
 * traj (optional): (nsteps+1) * n_node*dim displacement after every update.
 * Returns the number of bonds broken. */
int64_t orc_explicit(const orc_ctx* c, double dt, int nsteps, const uint8_t* prescribed_mask,
                     const double* dtv, double s0, uint64_t seed, double pert, double* u_all,
                     uint8_t* bond_state, double* traj);

/* Node stress (calGlobalNodeStresses) and damage (calLocalDamage). */
void orc_stress(const orc_ctx* c, const uint8_t* bond_state, const double* u_all, double* sigma, double* phi);

/* Values of K in the given CSR pattern (rows = equations, active columns)
 * and F = -K_full v (the internal force of the full DOF vector v). */
void orc_assemble(const orc_ctx* c, const uint8_t* bond_state, const int64_t* ia, const int64_t* ja,
                  const double* v_all, double* a, double* f);

/* Consistent mass in the CSR pattern (FE element mass + rho*cd_v on PD rows). */
void orc_consistent_mass(const orc_ctx* c, const int64_t* ia, const int64_t* ja, double* a);

/* Per-bond uniform draw used by FC 3 with a perturbed s0 (splitmix64). */
double orc_bond_uniform(uint64_t seed, int k, int m);

#ifdef __cplusplus
}
#endif

#endif
