// The reference-side binding of the C ABI: the bodies a maintainer of the
// reference (QibangLiu/PDLSM-FEM_mpi) puts in place of its four inner seams
// (and of its FC 1 crack-growth step) so that its solver loops call this
// library.  Each body replaces the member
// function of the same name in SourceFiles/Solver/pdsolve.cpp or
// calMatrixOperations.cpp; everything else in the reference stays as it is.
//
// tests/test_seams.py compiles this file (g++ -fsyntax-only) against the
// reference's own headers (HeaderFiles/Solver), the single-rank MPI / MKL shim
// headers of oracle/ref/shim and include/pdx.h, so the argument types of the
// prototypes in pdx.h are checked against the reference's as written.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pdsolve.h"
#include "pdx.h"

// One model per process, built from the same command file the reference read
// (pdx_model_create_from_cmd(cmdfile, &opts, &g_pdx) next to setDatModel).
pdx_model* g_pdx = nullptr;

static void pdx_or_exit(pdx_status st, int code) {
  if (st != PDX_OK) {
    std::printf("%s\n", pdx_last_error());
    std::exit(code);
  }
}

// Seam 1: pdsolve::calinternalForce_CSRformat (pdsolve.cpp:5819-5840).  The
// explicit form reads every DOF value from the pdDof objects, prescribed ones
// included; the library returns the whole internal force, so ranks other than
// 0 contribute zeros to the caller's MPI_Allreduce of cdp_F.
void pdsolve::calinternalForce_CSRformat(datModel& o_dat, int numEq, double* U_N) {
  (void)U_N;
  if (!cdp_F) cdp_F = new double[numEq];
  if (!cdp_FGlo) cdp_FGlo = new double[numEq];
  std::fill(cdp_FGlo, cdp_FGlo + numEq, 0.0);
  const int N = o_dat.getTotnumNode(), D = o_dat.ci_Numdimen;
  std::vector<double> u_all((size_t)N * D);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) u_all[(size_t)k * D + i] = o_dat.op_getNode(k)->op_getDof(i)->d_getValue();
  pdx_or_exit(pdx_internal_force(g_pdx, u_all.data(), cdp_F), 1);
  if (ci_rank != 0) std::fill(cdp_F, cdp_F + numEq, 0.0);
}

// Seam 2: pdsolve::timeIntegration_LM (pdsolve.cpp:5113-5132).  One call does
// the internal force, the central-difference update, the varying essential
// BCs and the failure pass of the step on the GPU, so the caller's loop
// (pdfemDynamicSolver_CSRformat, pdsolve.cpp:5986-6077) drops its own
// calinternalForce_CSRformat / Allreduce before this call.
void pdsolve::timeIntegration_LM(datModel& o_dat, Vector* Vu_n, Vector* Vu_nm1, Vector* Vu_np1, int numEq) {
  (void)o_dat;
  (void)numEq;
  pdx_or_exit(pdx_explicit_step_host(g_pdx, Vu_n->cdp_vecCoeff, Vu_nm1->cdp_vecCoeff, Vu_np1->cdp_vecCoeff), 1);
}

// Seam 3: calMatrixOperations::cluster_PARDISO_64Solver
// (calMatrixOperations.h:47-48).  Same arguments, zero-based CSR with the
// reference's long long indices, one right-hand side; a Krylov solve on the
// GPU judged by its true FP64 residual instead of the PARDISO factorisation.
void calMatrixOperations::cluster_PARDISO_64Solver(long long int& mkli_n, long long int* mkli_ia,
                                                   long long int* mkli_ja, double* doub_A, double* RHS,
                                                   double* v_Results, const int* comm) {
  (void)comm;
  pdx_solve_opts o = {2 /* BiCGStab: K is unsymmetric */, 1e-10, 20000, 0};
  pdx_solve_info info;
  pdx_or_exit(pdx_solve_csr(mkli_n, mkli_ia, mkli_ja, doub_A, RHS, v_Results, &o, &info), 3);
}

// Seam 4: pdsolve::pdfemAssembleEquasSys_CSRformat (pdsolve.cpp:5480-5504).
// The library returns the reference's CSR pattern (setCSRIndexes_gloStiffMat
// order) into cip_ia / cip_ja and the assembled K and F.
void pdsolve::pdfemAssembleEquasSys_CSRformat(datModel& o_dat, int numEq) {
  (void)o_dat;
  pdx_model_info info;
  pdx_or_exit(pdx_model_get_info(g_pdx, &info), 1);
  if (!cip_ia) cip_ia = new long long int[numEq + 1];
  if (!cip_ja) cip_ja = new long long int[info.nnz];
  if (!cdp_KuGlo) cdp_KuGlo = new double[info.nnz];
  if (!cdp_FGlo) cdp_FGlo = new double[numEq];
  pdx_or_exit(pdx_assemble_csr(g_pdx, 1, nullptr, cip_ia, cip_ja, cdp_KuGlo, cdp_FGlo), 1);
}

// Seam 5: pdsolve::b_cracPropag_qusiaStatic_BYKeq (pdsolve.cpp:7375-7495), for
// a quasi-static loop whose increments run through pdx_quasi_step (which ends
// with the FC 1 pass on the GPU model: SIFs, tip growth, PD-region growth and
// bond cuts).  The body copies the library's crack segments into the
// reference's crack records, writes the crack-path row the reference writes
// and returns whether a tip moved, with KEQ the last crack's Keq (the value
// failureProcess scales the next load step by).
bool pdsolve::b_cracPropag_qusiaStatic_BYKeq(datModel& o_dat, ofstream& cracPath, double& KEQ) {
  int nc = 0;
  pdx_or_exit(pdx_crack_state(g_pdx, nullptr, 0, &nc), 1);
  std::vector<double> rows((size_t)nc * 8);
  pdx_or_exit(pdx_crack_state(g_pdx, rows.data(), nc, nullptr), 1);
  bool moved = false;
  for (int ck = 0; ck < nc && ck < o_dat.ci_numCrack; ck++) {
    const double* r = &rows[(size_t)ck * 8];
    o_dat.cdp_crack[ck][0][0] = r[0];
    o_dat.cdp_crack[ck][0][1] = r[1];
    o_dat.cdp_crack[ck][1][0] = r[2];
    o_dat.cdp_crack[ck][1][1] = r[3];
    KEQ = r[6];
    moved = moved || r[7] != 0.0;
  }
  if (ci_rank == 0 && nc > 0) {
    const double* last = &rows[(size_t)(nc - 1) * 8];
    for (int ck = 0; ck < nc; ck++)
      cracPath << ck << "\t" << rows[(size_t)ck * 8 + 2] << "\t" << rows[(size_t)ck * 8 + 3] << "\t" << last[4]
               << "\t" << last[5] << "\t" << last[6] << " \"***\"\t";
    cracPath << endl;
  }
  return moved;
}
