// Readers for the reference's command file and mesh file.
//
// read_mesh follows datModel::readdata (SourceFiles/Solver/datModel.cpp:58-326)
// token by token, including its two getline() calls before every section
// header, so any file the reference reads is read the same way here.
// read_command follows fioFiles::CMDfile / excuteCMD (fioFile.cpp:54-462):
// whitespace tokens per line, '#' comments, the same keywords and the same
// defaults (datModel.cpp:17-52).  Additive keywords: PRECISION FP64|MIXED,
// SOLVE <method> [tol] [maxit], and FC 3 s0 [seed] [pert].
// Errors are returned, never exit()ed.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "model.h"

namespace pdx {

namespace {

bool fail(Error& err, int code, const std::string& m) {
  err.code = code;
  err.msg = m;
  return false;
}

int dof_index(const std::string& s) {
  if (s == "UX") return 0;
  if (s == "UY") return 1;
  if (s == "UZ") return 2;
  return -1;
}

}  // namespace

bool read_mesh(const std::string& path, Mesh& m, Error& err) {
  std::ifstream fin(path);
  if (!fin.is_open()) return fail(err, 1, "mesh file \"" + path + "\" does not exist");
  std::string label, sdim;
  fin >> m.title;
  std::getline(fin, label);
  std::getline(fin, label);
  fin >> sdim >> m.protype;
  fin >> m.E >> m.nu >> m.rho >> m.KIc >> m.sigult;
  if (sdim == "3D") m.dim = 3;
  else if (sdim == "2D") m.dim = 2;
  else return fail(err, 2, "the problem dimension is not 3D or 2D");
  fin >> m.n_node >> m.n_elem;
  if (!fin || m.n_node <= 0 || m.n_elem <= 0) return fail(err, 2, "bad node/element counts");
  m.X.assign((size_t)m.n_node * 3, 0.0);
  for (int i = 0; i < m.n_node; i++) {
    int id;
    double x[3];
    fin >> id >> x[0] >> x[1] >> x[2];
    if (!fin || id < 1 || id > m.n_node) return fail(err, 2, "bad node record " + std::to_string(i + 1));
    // the reference stores coordinates by node id (pdNode.cpp:17-20)
    for (int c = 0; c < 3; c++) m.X[(size_t)(id - 1) * 3 + c] = x[c];
  }
  m.elem_nn.assign(m.n_elem, 0);
  m.elem_algo.assign(m.n_elem, 0);
  m.conn.assign((size_t)m.n_elem * 8, -1);
  for (int e = 0; e < m.n_elem; e++) {
    int eid, algo, nid[8];
    fin >> eid >> algo;
    int nn = m.dim == 3 ? 8 : 4;
    for (int j = 0; j < nn; j++) fin >> nid[j];
    if (!fin) return fail(err, 2, "bad element record " + std::to_string(e + 1));
    if (m.dim == 3 && !(nid[2] != nid[3] && nid[4] != nid[5]))
      return fail(err, 3, "tetrahedral elements are not supported");
    // a 2D record whose fourth node repeats the third is a 3-node triangle
    // (datModel.cpp reads it into pdfemEleTri3N)
    if (m.dim == 2 && nid[3] == nid[2]) nn = 3;
    if (algo != 1 && algo != 2) return fail(err, 2, "element algorithm type must be 1 (PD) or 2 (FE)");
    m.elem_nn[e] = nn;
    m.elem_algo[e] = algo;
    for (int j = 0; j < nn; j++) {
      if (nid[j] < 1 || nid[j] > m.n_node) return fail(err, 2, "element node id out of range");
      m.conn[(size_t)e * 8 + j] = nid[j] - 1;
    }
  }
  std::string blank;
  const int tn = m.dim == 3 ? 4 : 2;
  std::getline(fin, blank);
  std::getline(fin, blank);
  int nebc = 0;
  fin >> nebc;
  if (!fin || nebc < 0) return fail(err, 2, "bad essential BC count");
  m.ebcs.assign(nebc, EssentialBC());
  std::vector<int> nn_ebc(nebc);
  for (int i = 0; i < nebc; i++) {
    std::string sd;
    fin >> nn_ebc[i] >> sd >> m.ebcs[i].value;
    m.ebcs[i].dof = dof_index(sd);
    if (m.ebcs[i].dof < 0 || m.ebcs[i].dof >= m.dim) return fail(err, 2, "DOFs must be UX, UY, or UZ");
  }
  std::vector<uint8_t> used((size_t)m.n_node * 3, 0);
  for (int i = 0; i < nebc; i++) {
    m.ebcs[i].nodes.resize(nn_ebc[i]);
    for (int j = 0; j < nn_ebc[i]; j++) {
      int nid;
      fin >> nid;
      if (!fin || nid < 1 || nid > m.n_node) return fail(err, 2, "bad essential BC node id");
      size_t key = (size_t)(nid - 1) * 3 + m.ebcs[i].dof;
      if (used[key]) return fail(err, 2, "The DOF of node " + std::to_string(nid) + " is repeatly defined!");
      used[key] = 1;
      m.ebcs[i].nodes[j] = nid - 1;
    }
  }
  // point BCs: the reference reads none (datModel.cpp:218)
  std::getline(fin, blank);
  std::getline(fin, blank);
  int nnbc = 0;
  fin >> nnbc;
  if (!fin || nnbc < 0) return fail(err, 2, "bad natural BC count");
  m.nbcs.assign(nnbc, NaturalBC());
  std::vector<int> ne_nbc(nnbc);
  for (int i = 0; i < nnbc; i++) fin >> ne_nbc[i] >> m.nbcs[i].value;
  for (int i = 0; i < nnbc; i++) {
    m.nbcs[i].elems.resize(ne_nbc[i]);
    for (int j = 0; j < ne_nbc[i]; j++) {
      std::array<int, 4> ids{-1, -1, -1, -1};
      for (int k = 0; k < tn; k++) {
        int nid;
        fin >> nid;
        if (!fin || nid < 1 || nid > m.n_node) return fail(err, 2, "bad natural BC node id");
        ids[k] = nid - 1;
      }
      m.nbcs[i].elems[j] = ids;
    }
  }
  std::getline(fin, blank);
  std::getline(fin, blank);
  int nnf = 0;
  fin >> nnf;
  if (!fin || nnf < 0) return fail(err, 2, "bad no-fail count");
  m.nofail.resize(nnf);
  for (int i = 0; i < nnf; i++) fin >> m.nofail[i];
  std::getline(fin, blank);
  std::getline(fin, blank);
  int ncr = 0;
  fin >> ncr;
  if (!fin || ncr < 0) return fail(err, 2, "bad crack count");
  m.cracks.assign(ncr, std::array<double, 9>{0, 0, 0, 0, 0, 0, 0, 0, 0});
  int npt = m.dim == 3 ? 3 : 2;
  for (int i = 0; i < ncr; i++)
    for (int j = 0; j < npt; j++)
      for (int k = 0; k < 3; k++) fin >> m.cracks[i][j * 3 + k];
  if (!fin) return fail(err, 2, "bad crack record");
  return true;
}

bool read_command(const std::string& path, Command& c, Mesh& m, std::string& base_dir, Error& err) {
  std::ifstream fin(path);
  if (!fin.is_open()) return fail(err, 1, "Command file \"" + path + "\" is not exist.");
  size_t slash = path.find_last_of('/');
  base_dir = slash == std::string::npos ? std::string(".") : path.substr(0, slash);
  bool have_mesh = false;
  std::string line;
  while (std::getline(fin, line)) {
    std::istringstream iss(line);
    std::vector<std::string> t;
    std::string w;
    while (iss >> w) t.push_back(w);
    if (t.empty() || t[0][0] == '#') continue;
    const std::string& k = t[0];
    auto need_mesh = [&]() {
      if (!have_mesh) { c.warnings.push_back(k + " before MSHFILE is ignored"); return false; }
      return true;
    };
    if (k == "MSHFILE") {
      if (t.size() < 2) return fail(err, 2, "MSHFILE needs a file name");
      c.mesh_file = t[1];
      std::string p = t[1];
      std::ifstream probe(p);
      if (!probe.is_open() && p[0] != '/') p = base_dir + "/" + t[1];
      if (!read_mesh(p, m, err)) return false;
      have_mesh = true;
    } else if (k == "SOLVER") {
      if (t.size() < 2) return fail(err, 2, "Miss solver.");
      if (t[1] == "DYNAMIC") c.solver = 0;
      else if (t[1] == "STATIC") c.solver = 1;
      else if (t[1] == "QUASI-STATIC") c.solver = 2;
      else return fail(err, 2, "Don't exist command of \"" + t[1] + "\".");
    } else if (k == "SETSOLVING") {
      if (t.size() < 6) { c.warnings.push_back("Miss SETSOLVING CMD."); continue; }
      c.dt = std::atof(t[1].c_str());
      if (c.solver == 2) c.dt = 1;
      c.nsteps = std::atoi(t[2].c_str());
      c.save_freq = std::atoi(t[3].c_str());
      c.factor = std::atof(t[4].c_str());
      c.nlf = std::atof(t[5].c_str());
      if (t.size() > 6) c.me = std::atof(t[6].c_str());
    } else if (k == "NEWMARK") {
      if (t.size() < 2) { c.warnings.push_back("Miss NEWMARK CMD."); continue; }
      if (t[1] == "ON") c.newmark = true;
      else if (t[1] == "OFF") c.newmark = false;
      else c.warnings.push_back("ignore unknown command: NEWMARK " + t[1]);
      if (t.size() > 3) { c.gamma = std::atof(t[2].c_str()); c.beta = std::atof(t[3].c_str()); }
    } else if (k == "FENSF") {
      if (t.size() >= 2 && t[1] == "ON") c.fensf = true;
      else if (t.size() >= 2 && t[1] == "OFF") c.fensf = false;
    } else if (k == "LUMPMASS") {
      if (t.size() < 2) continue;
      if (t[1] == "ON") c.lumped = true;
      else if (t[1] == "OFF") c.lumped = false;
    } else if (k == "VEBC" || k == "EBC") {
      if (t.size() < 3 || !need_mesh()) continue;
      int id = std::atoi(t[1].c_str());
      if (id < 0 || id >= (int)m.ebcs.size()) { c.warnings.push_back("the setting of essential BC is ignored"); continue; }
      double v = std::atof(t[2].c_str());
      if (k == "VEBC") { m.ebcs[id].varying = true; m.ebcs[id].velocity = v; }
      else m.ebcs[id].value = v;   // datModel::setEssentialBC
    } else if (k == "VNBC" || k == "NBC") {
      if (t.size() < 3 || !need_mesh()) continue;
      int id = std::atoi(t[1].c_str());
      if (id < 0 || id >= (int)m.nbcs.size()) { c.warnings.push_back("the setting of natural BC is ignored"); continue; }
      double v = std::atof(t[2].c_str());
      if (k == "VNBC") { m.nbcs[id].varying = true; m.nbcs[id].velocity = v; }
      else m.nbcs[id].value = v;
    } else if (k == "FC") {
      if (t.size() < 2) continue;
      int f = std::atoi(t[1].c_str());
      c.fail_flag = f;
      if (f < 0 || f > 3) c.warnings.push_back("the failure criterion is ignored");
      else if (f == 1 && t.size() > 3) { c.mr = std::atof(t[2].c_str()); c.dcf = std::atof(t[3].c_str()); }
      else if (f == 2 && t.size() > 2) c.topk = std::atoi(t[2].c_str());
      else if (f == 3 && t.size() < 3) {
        // the reference reads a bare FC 3 and breaks no bond with it
        c.fail_flag = 0;
        c.warnings.push_back("FC 3 without a critical stretch: no bond breaking (as the reference)");
      } else if (f == 3) {
        c.s0 = std::atof(t[2].c_str());
        if (t.size() > 3) c.s0_seed = std::strtoull(t[3].c_str(), nullptr, 10);
        if (t.size() > 4) c.s0_pert = std::atof(t[4].c_str());
        if (!(c.s0 > 0) || c.s0_pert < 0 || c.s0_pert >= 1) return fail(err, 2, "FC 3: s0 > 0 and 0 <= pert < 1");
      }
    } else if (k == "TOPK") {
      if (t.size() >= 2) c.topk = std::atoi(t[1].c_str());
    } else if (k == "RF") {
      for (size_t i = 1; i < t.size(); i++) c.rf_ids.push_back(std::atoi(t[i].c_str()));
    } else if (k == "VTKFORMAT") {
      if (t.size() >= 2 && t[1] == "ASCII") c.vtk_binary = false;
      else if (t.size() >= 2 && t[1] == "BINARY") c.vtk_binary = true;
    } else if (k == "PRECISION") {
      if (t.size() >= 2 && t[1] == "FP64") c.precision = 0;
      else if (t.size() >= 2 && t[1] == "MIXED") c.precision = 1;
      else return fail(err, 2, "PRECISION must be FP64 or MIXED");
    } else if (k == "SOLVE") {
      if (t.size() < 2) continue;
      if (t[1] == "PCG") c.solve_method = 0;
      else if (t[1] == "BJPCG") c.solve_method = 1;
      else if (t[1] == "BICGSTAB") c.solve_method = 2;
      else if (t[1] == "MIXEDPCG") c.solve_method = 3;
      else if (t[1] == "GMRES") c.solve_method = 6;
      else if (t[1] == "MIXEDBICGSTAB") c.solve_method = 7;
      else if (t[1] == "TWOLEVEL") c.solve_method = 8;
      else return fail(err, 2, "SOLVE must be PCG, BJPCG, BICGSTAB, MIXEDPCG, GMRES, MIXEDBICGSTAB or TWOLEVEL");
      if (t.size() > 2) c.solve_tol = std::atof(t[2].c_str());
      if (t.size() > 3) c.solve_maxit = std::atoi(t[3].c_str());
    } else {
      c.warnings.push_back("ignore unknown command \"" + k + "\"");
    }
  }
  if (!have_mesh) return fail(err, 2, "the command file names no mesh (MSHFILE)");
  if (c.solver < 0) return fail(err, 2, "solver flag is wrong");
  return true;
}

}  // namespace pdx
