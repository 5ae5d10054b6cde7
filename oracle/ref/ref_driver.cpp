// Driver that runs the reference's own (unmodified) C++ code and dumps its
// full-precision state, so that the project's CPU restatement and CUDA path can
// be pinned against it.  Test infrastructure only: it is built from the
// reference sources by oracle/ref/Makefile into oracle/_ref/ and is never part
// of the product.
//
// Usage (run with the case directory as cwd, because MSHFILE is relative):
//   ref_driver setup    <cmd.in> <outdir>
//   ref_driver coeffs   <cmd.in> <outdir>
//   ref_driver force    <cmd.in> <outdir> <u_all.bin>
//   ref_driver explicit <cmd.in> <outdir> <s0 or 0> <dump_every>
//   ref_driver static   <cmd.in> <outdir>
//   ref_driver assemble <cmd.in> <outdir>          (the static K and F only)
//   ref_driver newmark  <cmd.in> <outdir>
//   ref_driver quasi    <cmd.in> <outdir>
//   ref_driver explicit_fc2 <cmd.in> <outdir> <every>  (FC 2 after every step)
//   ref_driver newmark_fc2  <cmd.in> <outdir>          (Newmark with FC 2 after every step)
//   ref_driver quasi_fc2    <cmd.in> <outdir>          (quasi-static with FC 2 and its load ratio)
//   ref_driver quasi_fc1    <cmd.in> <outdir>          (quasi-static with FC 1: SIFs, crack growth,
//                                                       PD-region growth and its load ratio)
//   ref_driver solve    <cmd.in>             (the reference's own pdfemSolver)
//
// Every loop below calls the reference's member functions in the order its own
// solver uses (SourceFiles/Solver/pdsolve.cpp:5842-6090 explicit, 6092-6290
// Newmark, 6464-6590 quasi-static, 5557-5654 static); only the dumps and the
// failure step differ.  The critical-stretch failure step calls the
// reference's failureCriterion_stretch (pdsolve.cpp:6643-6780, dead code in
// the reference) with K_Ic chosen so that its s_c equals s0, TopK large (all
// bonds over s_c) and the local damage refreshed before each pass.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <limits>
#include <memory>
#include <queue>
#include <sstream>
#include <string>
#include <unordered_set>
#include <vector>

#define private public
#include "pdsolve.h"
#include "fioFile.h"
#include "datModel.h"
#undef private

calMatrixOperations matoperat;
pdGaussPt o_globGP(2);
pdGaussPt o_sigGP(2);
pdGaussPt o_sifGP(4);

namespace {

struct Dumper {
  std::string dir;
  FILE* man = nullptr;
  explicit Dumper(const std::string& d) : dir(d) {
    std::string cmd = "mkdir -p '" + d + "'";
    if (std::system(cmd.c_str()) != 0) { std::fprintf(stderr, "mkdir failed\n"); std::exit(2); }
    man = std::fopen((d + "/manifest.txt").c_str(), "w");
  }
  ~Dumper() { if (man) std::fclose(man); }
  template <class T>
  void put(const std::string& name, const char* dtype, const std::vector<long long>& shape,
           const T* data, size_t count) {
    FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
    if (count) std::fwrite(data, sizeof(T), count, f);
    std::fclose(f);
    std::fprintf(man, "%s %s", name.c_str(), dtype);
    for (long long s : shape) std::fprintf(man, " %lld", s);
    std::fprintf(man, "\n");
    std::fflush(man);
  }
  void f64(const std::string& n, const std::vector<double>& v, std::vector<long long> shape = {}) {
    if (shape.empty()) shape = {(long long)v.size()};
    put(n, "f64", shape, v.data(), v.size());
  }
  void i64(const std::string& n, const std::vector<long long>& v, std::vector<long long> shape = {}) {
    if (shape.empty()) shape = {(long long)v.size()};
    put(n, "i64", shape, v.data(), v.size());
  }
};

int num_eq(datModel& d) {
  int pre = 0;
  for (int i = 0; i < d.getTotnumEssentialBCs(); i++) pre += d.op_getEssenBC(i)->getNumNODE();
  return d.getTotnumNode() * d.ci_Numdimen - pre;
}

std::vector<double> all_dof_values(datModel& d) {
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  std::vector<double> u((size_t)N * D);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) u[(size_t)k * D + i] = d.op_getNode(k)->op_getDof(i)->d_getValue();
  return u;
}

std::vector<double> node_sigma(datModel& d) {
  int N = d.getTotnumNode();
  std::vector<double> s((size_t)N * 6);
  for (int k = 0; k < N; k++) d.op_getNode(k)->getStress(&s[(size_t)k * 6]);
  return s;
}

std::vector<double> node_damage(datModel& d) {
  int N = d.getTotnumNode();
  std::vector<double> p((size_t)N);
  for (int k = 0; k < N; k++) p[k] = d.op_getNode(k)->getLocalDamage();
  return p;
}

std::vector<long long> bond_states(datModel& d) {
  std::vector<long long> s;
  for (int f = 0; f < d.getTotnumFami(); f++) {
    pdFamily* p = d.op_getFami(f);
    for (int m = 0; m < p->getNumNode(); m++) s.push_back(p->getbondstate(m));
  }
  return s;
}

void dump_setup(datModel& d, pdsolve& sol, Dumper& out) {
  int N = d.getTotnumNode(), D = d.ci_Numdimen, E = d.getTotnumEle();
  std::vector<long long> eq((size_t)N * D), type(N), famid(N);
  std::vector<double> vn(N), ve(E);
  for (int k = 0; k < N; k++) {
    for (int i = 0; i < D; i++) eq[(size_t)k * D + i] = d.op_getNode(k)->op_getDof(i)->i_getEqInde();
    type[k] = d.op_getNode(k)->getNodeType();
    famid[k] = d.op_getNode(k)->getFamID();
    vn[k] = d.op_getNode(k)->getvolume();
  }
  for (int e = 0; e < E; e++) ve[e] = d.op_getEles(e)->cd_V;
  out.i64("eq", eq, {N, D});
  out.i64("node_type", type);
  out.i64("fam_id", famid);
  out.f64("vol_node", vn);
  out.f64("vol_elem", ve);
  std::vector<long long> off{0}, mem;
  std::vector<double> hor, cdv;
  for (int f = 0; f < d.getTotnumFami(); f++) {
    pdFamily* p = d.op_getFami(f);
    for (int m = 0; m < p->getNumNode(); m++) mem.push_back(p->getNodeID(m));
    off.push_back((long long)mem.size());
    hor.push_back(p->gethorizon());
    cdv.push_back(p->cd_v);
  }
  out.i64("fam_off", off);
  out.i64("fam_members", mem);
  out.f64("fam_horizon", hor);
  out.f64("fam_cdv", cdv);
  out.i64("bond_state0", bond_states(d));
  std::vector<long long> pdbe;
  for (int b = 0; b < d.getTotnumPDBEs(); b++) {
    int ids[4] = {0, 0, 0, 0};
    d.op_getPDBE(b)->getNodeID(ids);
    int nn = d.op_getPDBE(b)->i_getNumnode();
    for (int i = 0; i < 4; i++) pdbe.push_back(i < nn ? ids[i] : 0);
  }
  out.i64("pdbe", pdbe, {d.getTotnumPDBEs(), 4});
  std::vector<long long> pde(d.civ_pdeIDX.begin(), d.civ_pdeIDX.end());
  std::vector<long long> fe(d.civ_feIDX.begin(), d.civ_feIDX.end());
  out.i64("pde_idx", pde);
  out.i64("fe_idx", fe);
  double lbc[3], rtc[3];
  d.op_getGeomP()->getlbc(lbc);
  d.op_getGeomP()->getrtc(rtc);
  int nb[3];
  d.getNumOfBLock(nb);
  std::vector<double> geo{d.op_getGeomP()->getminDelta(), d.op_getGeomP()->getmaxDelta(),
                          d.op_getGeomP()->getBlockSize(), lbc[0], lbc[1], lbc[2], rtc[0], rtc[1], rtc[2]};
  out.f64("geom", geo);
  out.i64("nblocks", {nb[0], nb[1], nb[2]});
  sol.setCSRIndexes_gloStiffMat(d);
  int neq = num_eq(d);
  std::vector<long long> ia(sol.cip_ia, sol.cip_ia + neq + 1), ja(sol.cip_ja, sol.cip_ja + sol.cip_ia[neq]);
  out.i64("csr_ia", ia);
  out.i64("csr_ja", ja);
}

void dump_coeffs(datModel& d, pdsolve& sol, Dumper& out) {
  int D = d.ci_Numdimen;
  int na = D == 2 ? 5 : 9, nd = D == 2 ? 3 : 6;
  std::vector<double> A, g, dv, G, C;
  for (int f = 0; f < d.getTotnumFami(); f++) {
    pdFamily* p = d.op_getFami(f);
    Matrix Am(na, na);
    if (D == 2) sol.shapTens2D(&Am, p, d); else sol.shapTens3D(&Am, p, d);
    for (int r = 0; r < na; r++)
      for (int c = 0; c < na; c++) A.push_back(Am.d_getCoeff(r, c));
    double xk[3], xm[3], xi[3];
    d.op_getNode(p->getNodeID(0) - 1)->getcoor(xk);
    for (int m = 1; m < p->getNumNode(); m++) {
      d.op_getNode(p->getNodeID(m) - 1)->getcoor(xm);
      for (int i = 0; i < 3; i++) xi[i] = xm[i] - xk[i];
      double gg[3] = {0, 0, 0}, dd[6] = {0, 0, 0, 0, 0, 0};
      if (D == 2) sol.vec_gd2D(gg, dd, &Am, p, xi, d); else sol.vec_gd3D(gg, dd, &Am, p, xi, d);
      for (int i = 0; i < D; i++) g.push_back(gg[i]);
      for (int i = 0; i < nd; i++) dv.push_back(dd[i]);
      Matrix Gm(D, D);
      if (D == 2) sol.matG2D(&Gm, &Am, p, m, d); else sol.matG3D(&Gm, &Am, p, m, d);
      for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) G.push_back(Gm.d_getCoeff(r, c));
    }
    int nn = p->getNumNode();
    int nv = D == 2 ? 3 : 6;
    Matrix Cm(nv, D * nn);
    if (D == 2) sol.matC2D(&Cm, p, d); else sol.matC3D(&Cm, p, d);
    for (int r = 0; r < nv; r++)
      for (int c = 0; c < D * nn; c++) C.push_back(Cm.d_getCoeff(r, c));
  }
  out.f64("A", A);
  out.f64("g", g);
  out.f64("d", dv);
  out.f64("G", G);
  out.f64("C", C);
}

void set_all_dofs(datModel& d, const std::vector<double>& u) {
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) d.op_getNode(k)->op_getDof(i)->setValue(u[(size_t)k * D + i]);
}

std::vector<double> read_f64(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f) / 8;
  std::fseek(f, 0, SEEK_SET);
  std::vector<double> v((size_t)n);
  if (std::fread(v.data(), 8, (size_t)n, f) != (size_t)n) std::exit(2);
  std::fclose(f);
  return v;
}

// KIc such that the reference's s_c = sqrt(5 G0 / (9 kappa minDelta)), G0 = KIc^2/E, equals s0.
void set_stretch_threshold(datModel& d, double s0) {
  double E = d.op_getmaterial()->getE(), nu = d.op_getmaterial()->getnu();
  double kappa = E / (3.0 * (1 - 2 * nu));
  double delta = d.op_getGeomP()->getminDelta();
  d.op_getmaterial()->cd_KIc = std::sqrt(s0 * s0 * 9.0 * kappa * delta * E / 5.0);
}

void stretch_failure(datModel& d, pdsolve& sol) {
  bool addLoad = true;
  int saved = d.ci_solvFlag;
  d.ci_solvFlag = 0;
  sol.calLocalDamage(d);
  sol.failureCriterion_stretch(d, INT_MAX, addLoad);
  d.ci_solvFlag = saved;
}

// FC 2 after a step, as pdfemDynamicSolver_CSRformat does (pdsolve.cpp:6014-6016,
// 6060-6064): nodal stresses, then the reference's maximum-principal-stress
// criterion with the command file's Top-K
void maxprisig_failure(datModel& d, pdsolve& sol) {
  bool addLoad = true;
  sol.calGlobalNodeStresses(d);
  sol.failureCriterion_maxPriSig(d, d.ci_topk, addLoad);
}

void run_explicit(datModel& d, pdsolve& sol, Dumper& out, double s0, int every, bool fc2 = false) {
  if (s0 > 0) set_stretch_threshold(d, s0);
  int neq = num_eq(d);
  int nsteps = d.getnumTstep();
  Vector* Vu_nm1 = new Vector(neq);
  Vector* Vu_n = new Vector(neq);
  Vector* Vu_np1 = new Vector(neq);
  Vector* Va_n = new Vector(neq);
  if (!d.cb_lumpedMass) { std::fprintf(stderr, "explicit driver needs LUMPMASS ON\n"); std::exit(2); }
  sol.assembleLumpedMass(d, neq);
  std::vector<double> mass(sol.cdp_MGlo, sol.cdp_MGlo + neq);
  out.f64("mass", mass);
  double dt = d.getTstep();
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) {
      int eq = d.op_getNode(k)->op_getDof(i)->i_getEqInde();
      if (eq != -1) Vu_n->setCoeff(eq, d.op_getNode(k)->op_getDof(i)->d_getValue());
    }
  sol.setVaryEssentialBC(d, 1);
  sol.setVaryNaturalBC(d);
  std::unique_ptr<double[]> U_N = std::make_unique<double[]>(1);
  sol.calinternalForce_CSRformat(d, neq, U_N.get());
  sol.calExternalForce_CSRformat(d);
  MPI_Allreduce(sol.cdp_F, sol.cdp_FGlo, neq, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
  out.f64("force_step0", std::vector<double>(sol.cdp_FGlo, sol.cdp_FGlo + neq));
  for (int i = 0; i < neq; i++) Va_n->cdp_vecCoeff[i] = sol.cdp_FGlo[i] / sol.cdp_MGlo[i];
  matoperat.matMultiply(Va_n, 0.5 * dt * dt, Vu_np1);
  matoperat.matAdd(Vu_np1, Vu_n, Vu_np1);
  sol.storeDisplacementResult(d, Vu_np1);
  if (s0 > 0) stretch_failure(d, sol);
  if (fc2) maxprisig_failure(d, sol);
  // reaction forces (RF keyword) through the reference's own calReacForc,
  // written at full precision and read back at the end
  const bool rf = !d.civ_reacForceOfessBCId.empty();
  const std::string rf_path = out.dir + "/rf.txt";
  std::ofstream rf_out;
  if (rf) {
    rf_out.open(rf_path);
    rf_out << std::setprecision(17);
    sol.calReacForc(d, rf_out, 0);
  }
  std::vector<double> traj;
  std::vector<long long> traj_steps;
  auto snap = [&](int n) {
    std::vector<double> u = all_dof_values(d);
    traj.insert(traj.end(), u.begin(), u.end());
    traj_steps.push_back(n);
  };
  snap(0);
  for (int n = 1; n < nsteps + 1; n++) {
    for (int i = 0; i < neq; i++) {
      Vu_nm1->setCoeff(i, Vu_n->d_getCoeff(i));
      Vu_n->setCoeff(i, Vu_np1->d_getCoeff(i));
    }
    sol.setVaryEssentialBC(d, 1);
    sol.setVaryNaturalBC(d);
    sol.calinternalForce_CSRformat(d, neq, U_N.get());
    sol.calExternalForce_CSRformat(d);
    MPI_Allreduce(sol.cdp_F, sol.cdp_FGlo, neq, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
    sol.timeIntegration_LM(d, Vu_n, Vu_nm1, Vu_np1, neq);
    sol.storeDisplacementResult(d, Vu_np1);
    if (n == nsteps && !fc2) sol.calGlobalNodeStresses(d);
    if (s0 > 0) stretch_failure(d, sol);
    if (fc2) maxprisig_failure(d, sol);
    if (rf) sol.calReacForc(d, rf_out, n);
    if (n % every == 0 || n == nsteps) snap(n);
  }
  if (rf) {
    rf_out.close();
    std::ifstream in(rf_path);
    std::vector<double> rows;
    double v;
    while (in >> v) rows.push_back(v);
    out.f64("rf_rows", rows, {(long long)(rows.size() / 5), 5});
  }
  sol.calLocalDamage(d);
  long long ns = (long long)traj_steps.size();
  out.f64("u_traj", traj, {ns, (long long)N, (long long)D});
  out.i64("u_traj_steps", traj_steps);
  out.f64("sigma_final", node_sigma(d), {(long long)N, 6});
  out.f64("phi_final", node_damage(d));
  out.i64("bond_state_final", bond_states(d));
}

void run_static(datModel& d, pdsolve& sol, Dumper& out, bool solve = true) {
  d.ci_solvFlag = 1;
  int neq = num_eq(d);
  sol.pdfemAssembleEquasSys_CSRformat(d, neq);
  long long nnz = sol.cip_ia[neq];
  out.i64("K_ia", std::vector<long long>(sol.cip_ia, sol.cip_ia + neq + 1));
  out.i64("K_ja", std::vector<long long>(sol.cip_ja, sol.cip_ja + nnz));
  out.f64("K_a", std::vector<double>(sol.cdp_KuGlo, sol.cdp_KuGlo + nnz));
  out.f64("F", std::vector<double>(sol.cdp_FGlo, sol.cdp_FGlo + neq));
  if (!solve) return;
  long long n = neq;
  int comm = 0;
  Vector* Ug = new Vector(neq);
  matoperat.cluster_PARDISO_64Solver(n, sol.cip_ia, sol.cip_ja, sol.cdp_KuGlo, sol.cdp_FGlo,
                                     Ug->cdp_vecCoeff, &comm);
  sol.storeDisplacementResult(d, Ug);
  sol.calGlobalNodeStresses(d);
  sol.calLocalDamage(d);
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  out.f64("u", all_dof_values(d), {(long long)N, (long long)D});
  out.f64("sigma", node_sigma(d), {(long long)N, 6});
  out.f64("phi", node_damage(d));
}

void run_newmark(datModel& d, pdsolve& sol, Dumper& out, bool fc2 = false) {
  d.ci_solvFlag = 0;
  int neq = num_eq(d);
  int nsteps = d.getnumTstep();
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  std::unique_ptr<double[]> U_N = std::make_unique<double[]>((size_t)N * D);
  Vector* Vu_n = new Vector(neq);
  Vector* Va_n = new Vector(neq);
  Vector* Va_np1 = new Vector(neq);
  Vector* Vv_n = new Vector(neq);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) {
      int eq = d.op_getNode(k)->op_getDof(i)->i_getEqInde();
      if (eq != -1) Vu_n->setCoeff(eq, d.op_getNode(k)->op_getDof(i)->d_getValue());
    }
  Vv_n->zero();
  Va_n->zero();
  int comm = 0;
  long long n64 = neq;
  std::vector<double> traj;
  for (int n = 1; n <= nsteps; n++) {
    sol.pdfemAssembleKNFR_CSRformat(d, neq, Va_n, Vv_n, U_N.get(), n - 1);
    if (n == 1) {
      long long nnz = sol.cip_ia[neq];
      out.i64("KN_ia", std::vector<long long>(sol.cip_ia, sol.cip_ia + neq + 1));
      out.i64("KN_ja", std::vector<long long>(sol.cip_ja, sol.cip_ja + nnz));
      out.f64("KN_a", std::vector<double>(sol.cdp_KuGlo, sol.cdp_KuGlo + nnz));
      out.f64("M_a", std::vector<double>(sol.cdp_M, sol.cdp_M + nnz));
      out.f64("FN", std::vector<double>(sol.cdp_FGlo, sol.cdp_FGlo + neq));
    }
    matoperat.cluster_PARDISO_64Solver(n64, sol.cip_ia, sol.cip_ja, sol.cdp_KuGlo, sol.cdp_FGlo,
                                       Va_np1->cdp_vecCoeff, &comm);
    sol.updateDispVelo(Vu_n, Vv_n, Va_n, Va_np1, neq, d);
    sol.storeDisplacementResult(d, Vu_n);
    sol.setVaryEssentialBC(d, 1);
    sol.setVaryNaturalBC(d);
    double* t = Va_n->cdp_vecCoeff;
    Va_n->cdp_vecCoeff = Va_np1->cdp_vecCoeff;
    Va_np1->cdp_vecCoeff = t;
    if (fc2) maxprisig_failure(d, sol);   // pdsolve.cpp:6258-6261
    std::vector<double> u = all_dof_values(d);
    traj.insert(traj.end(), u.begin(), u.end());
  }
  if (fc2) {
    sol.calLocalDamage(d);
    out.i64("bond_state_final", bond_states(d));
  } else {
    sol.calGlobalNodeStresses(d);
  }
  out.f64("u_traj", traj, {(long long)nsteps, (long long)N, (long long)D});
  out.f64("v_final", std::vector<double>(Vv_n->cdp_vecCoeff, Vv_n->cdp_vecCoeff + neq));
  out.f64("a_final", std::vector<double>(Va_n->cdp_vecCoeff, Va_n->cdp_vecCoeff + neq));
  out.f64("sigma_final", node_sigma(d), {(long long)N, 6});
}

// fc: 0 no failure step, 2 FC 2, 1 FC 1 (the deck's failure flag decides
// which criterion failureProcess applies; fc only selects the dumps)
void run_quasi(datModel& d, pdsolve& sol, Dumper& out, int fc = 0) {
  const bool fc2 = fc != 0;
  d.ci_solvFlag = 2;
  int neq = num_eq(d);
  int nsteps = d.getnumTstep();
  int N = d.getTotnumNode(), D = d.ci_Numdimen;
  Vector* Vu_n = new Vector(neq);
  Vector* Vdu = new Vector(neq);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) {
      int eq = d.op_getNode(k)->op_getDof(i)->i_getEqInde();
      if (eq != -1) Vu_n->setCoeff(eq, d.op_getNode(k)->op_getDof(i)->d_getValue());
    }
  sol.setCSRIndexes_gloStiffMat(d);
  int comm = 0;
  long long n64 = neq;
  std::vector<double> traj, traj_after;
  // with FC 2: the reference's loop body (pdsolve.cpp:6527-6578): stresses,
  // failureProcess (cuts and the load ratio), reaction forces, then the load
  // step only if nothing was cut
  bool addLoad = true;
  double rati = 1.0;
  const bool rf = fc2 && !d.civ_reacForceOfessBCId.empty();
  const std::string rf_path = out.dir + "/rf.txt";
  std::ofstream rf_out, crack_out;
  if (rf) { rf_out.open(rf_path); rf_out << std::setprecision(17); }
  // FC 1: the crack-path rows the reference writes (crack, tip x, tip y, KI,
  // KII, Keq) at full precision, and the PD-region size after each increment
  const std::string cp_path = out.dir + "/cp.txt";
  std::vector<double> fc1_rows;   // n_pde, n_fam, addLoad, rati per increment
  if (fc == 1) { crack_out.open(cp_path); crack_out << std::setprecision(17) << std::scientific; }
  for (int n = 1; n < nsteps + 1; n++) {
    sol.pdfemQuasiStaticAssembleEquasSys_CSRformat(d, neq, addLoad);
    if (n == 1 || n == 2) {
      long long nnz = sol.cip_ia[neq];
      std::string s = std::to_string(n);
      out.i64("K_ia_" + s, std::vector<long long>(sol.cip_ia, sol.cip_ia + neq + 1));
      out.i64("K_ja_" + s, std::vector<long long>(sol.cip_ja, sol.cip_ja + nnz));
      out.f64("K_a_" + s, std::vector<double>(sol.cdp_KuGlo, sol.cdp_KuGlo + nnz));
      out.f64("F_" + s, std::vector<double>(sol.cdp_FGlo, sol.cdp_FGlo + neq));
    }
    matoperat.cluster_PARDISO_64Solver(n64, sol.cip_ia, sol.cip_ja, sol.cdp_KuGlo, sol.cdp_FGlo,
                                       Vdu->cdp_vecCoeff, &comm);
    matoperat.matAdd(Vu_n, Vdu, Vu_n);
    sol.storeDisplacementResult(d, Vu_n);
    if (fc2) {
      sol.calGlobalNodeStresses(d);
      rati = sol.failureProcess(d, d.ci_topk, addLoad, crack_out);
      if (rf) sol.calReacForc(d, rf_out, n);
      if (fc == 1) {
        fc1_rows.push_back((double)d.civ_pdeIDX.size());
        fc1_rows.push_back((double)d.getTotnumFami());
        fc1_rows.push_back(addLoad ? 1.0 : 0.0);
        fc1_rows.push_back(rati);
      }
    }
    std::vector<double> u = all_dof_values(d);
    traj.insert(traj.end(), u.begin(), u.end());
    if (!fc2 || addLoad) {
      sol.setVaryNaturalBC(d);
      sol.setVaryEssentialBC(d, fc2 ? rati : 1.0);
    }
    if (fc2) {
      std::vector<double> ua = all_dof_values(d);
      traj_after.insert(traj_after.end(), ua.begin(), ua.end());
    }
  }
  if (!fc2) sol.calGlobalNodeStresses(d);
  out.f64("u_traj", traj, {(long long)nsteps, (long long)N, (long long)D});
  out.f64("sigma_final", node_sigma(d), {(long long)N, 6});
  if (fc2) {
    out.f64("u_after", traj_after, {(long long)nsteps, (long long)N, (long long)D});
    out.i64("bond_state_final", bond_states(d));
    if (fc == 1) {
      crack_out.close();
      std::ifstream in(cp_path);
      std::vector<double> cp;
      std::string tok;
      while (in >> tok)
        if (tok != "\"***\"") cp.push_back(std::strtod(tok.c_str(), nullptr));
      const long long nc = d.ci_numCrack;
      out.f64("crack_rows", cp, {(long long)nsteps, nc, 6});
      out.f64("region_rows", fc1_rows, {(long long)nsteps, 4});
      std::vector<long long> pde(d.civ_pdeIDX.begin(), d.civ_pdeIDX.end());
      out.i64("pde_final", pde);
      std::vector<long long> fnode, foff(1, 0), fmem;
      for (int f = 0; f < d.getTotnumFami(); f++) {
        pdFamily* p = d.op_getFami(f);
        fnode.push_back(p->getNodeID(0) - 1);
        for (int m = 0; m < p->getNumNode(); m++) fmem.push_back(p->getNodeID(m) - 1);
        foff.push_back((long long)fmem.size());
      }
      out.i64("fam_node_final", fnode);
      out.i64("fam_off_final", foff);
      out.i64("fam_members_final", fmem);
    }
    if (rf) {
      rf_out.close();
      std::ifstream in(rf_path);
      std::vector<double> rows;
      double v;
      while (in >> v) rows.push_back(v);
      out.f64("rf_rows", rows, {(long long)(rows.size() / 5), 5});
    }
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver <mode> <cmd.in> [outdir] [...]\n");
    return 2;
  }
  std::string mode = argv[1];
  fioFiles files(0);
  datModel dat;
  std::ifstream fin(argv[2]);
  if (!fin.is_open()) { std::fprintf(stderr, "cannot open %s\n", argv[2]); return 2; }
  files.CMDfile(dat, fin);
  fin.close();
  pdsolve sol(dat, 0, 1);
  if (mode == "solve") { sol.pdfemSolver(dat, files, argv); return 0; }
  if (argc < 4) { std::fprintf(stderr, "missing outdir\n"); return 2; }
  Dumper out(argv[3]);
  if (mode == "setup") dump_setup(dat, sol, out);
  else if (mode == "coeffs") dump_coeffs(dat, sol, out);
  else if (mode == "force") {
    std::vector<double> u = read_f64(argv[4]);
    set_all_dofs(dat, u);
    int saved = dat.ci_solvFlag;
    dat.ci_solvFlag = 0;
    dat.cb_Newmark = false;
    int neq = num_eq(dat);
    std::unique_ptr<double[]> U_N = std::make_unique<double[]>(1);
    sol.calinternalForce_CSRformat(dat, neq, U_N.get());
    dat.ci_solvFlag = saved;
    out.f64("F", std::vector<double>(sol.cdp_F, sol.cdp_F + neq));
  } else if (mode == "explicit") {
    run_explicit(dat, sol, out, std::atof(argv[4]), std::atoi(argv[5]));
  } else if (mode == "explicit_fc2") {
    run_explicit(dat, sol, out, 0.0, std::atoi(argv[4]), true);
  } else if (mode == "static") run_static(dat, sol, out);
  else if (mode == "assemble") run_static(dat, sol, out, false);
  else if (mode == "newmark") run_newmark(dat, sol, out);
  else if (mode == "newmark_fc2") run_newmark(dat, sol, out, true);
  else if (mode == "quasi") run_quasi(dat, sol, out);
  else if (mode == "quasi_fc2") run_quasi(dat, sol, out, 2);
  else if (mode == "quasi_fc1") run_quasi(dat, sol, out, 1);
  else { std::fprintf(stderr, "unknown mode %s\n", mode.c_str()); return 2; }
  return 0;
}
