// Host-side model of a PDLSM-FEM problem: the reference's mesh (.lis) and
// command (.in) data, and the setup that pdsolve::setDatModel builds from
// them (SourceFiles/Solver/pdsolve.cpp:114-151).  Everything here is plain
// host data; the GPU copies live in device.h.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace pdx {

struct Error {
  int code;
  std::string msg;
};

// One essential (displacement) boundary condition (pdfemEssentialBCs.h).
struct EssentialBC {
  int dof = 0;                 // 0 UX, 1 UY, 2 UZ
  double value = 0.0;          // cd_value, advanced by dt*velocity when varying
  std::vector<int> nodes;      // 0-based
  bool varying = false;        // VEBC
  double velocity = 0.0;
};

// One natural (traction) boundary condition (pdfemNaturalBCs.h).
struct NaturalBC {
  double value = 0.0;
  std::vector<std::array<int, 4>> elems;   // 0-based node ids, 2 used in 2D
  bool varying = false;        // VNBC
  double velocity = 0.0;
};

// Mesh file contents (datModel::readdata, SourceFiles/Solver/datModel.cpp:58-326).
struct Mesh {
  std::string title;
  int dim = 2;
  int protype = 1;             // 1 plane stress, 2 plane strain
  double E = 0, nu = 0, rho = 0, KIc = 0, sigult = 0;
  int n_node = 0, n_elem = 0;
  std::vector<double> X;       // 3 * n_node
  std::vector<int> elem_nn;    // nodes per element (4 or 8)
  std::vector<int> elem_algo;  // 1 PD, 2 FE (may be turned to 1 by a crack)
  std::vector<int> conn;       // 8 * n_elem, 0-based, unused slots -1
  std::vector<EssentialBC> ebcs;
  std::vector<NaturalBC> nbcs;
  std::vector<int> nofail;     // read but never applied by the reference
  std::vector<std::array<double, 9>> cracks;   // 2 (2D) or 3 (3D) points
};

// Command file contents (fioFiles::excuteCMD, SourceFiles/Solver/fioFile.cpp:69-462)
// plus the additive extension keywords PRECISION and SOLVE and FC 3.
struct Command {
  std::string mesh_file;
  int solver = -1;             // 0 dynamic, 1 static, 2 quasi-static
  double dt = 1.0;
  int nsteps = 1;
  int save_freq = 1;
  double factor = 3.0;         // horizon factor (pdGeomP default 3, datModel.cpp:67)
  double nlf = 0.33;           // non-local factor of the influence function
  double me = 0.0;             // crack-element neighbourhood factor (cd_me)
  bool newmark = false;
  double gamma = 0.5, beta = 0.25;
  bool fensf = true;
  bool lumped = false;
  int fail_flag = 0;
  double mr = 6.0, dcf = 1.0;
  int topk = 0;
  std::vector<int> rf_ids;
  bool vtk_binary = true;
  // extensions
  double s0 = 0.0;             // FC 3 critical stretch
  uint64_t s0_seed = 0;        // FC 3 per-bond draw seed
  double s0_pert = 0.0;        // FC 3 half-width of the per-bond uniform draw (relative)
  int precision = 0;           // 0 FP64, 1 mixed (FP32 forces)
  int solve_method = 0;        // 0 PCG (Jacobi), 1 block-Jacobi PCG, 2 BiCGStab, 3 mixed PCG + refinement
  double solve_tol = 1e-8;
  int solve_maxit = 20000;
  std::vector<std::string> warnings;
};

// Result of pdsolve::setDatModel.
struct Setup {
  int dim = 2;
  int n_eq = 0;
  std::vector<int> eq;             // n_node * dim, -1 for prescribed DOFs
  std::vector<double> vol_elem;    // element volume (area in 2D)
  std::vector<double> vol_node;    // sum of V_e / n_e
  double min_delta = 0, max_delta = 0;
  double lbc[3] = {0, 0, 0}, rtc[3] = {0, 0, 0};
  double block_size = 0;
  int nblocks[3] = {1, 1, 1};
  std::vector<std::vector<int>> block_nodes;   // 0-based node ids in insertion order
  std::vector<std::vector<int>> block_elems;
  std::vector<int> pde;            // PD element indices in civ_pdeIDX order
  std::vector<int> fe;             // FE element indices
  std::vector<std::array<int, 4>> pdbe;        // 0-based; 2D uses 2, 3D 4 (tri repeats the 3rd)
  std::vector<int> node_type;      // 0 FE, 1 interface (PDBE), 2 PD
  std::vector<int> fam_of_node;    // -1 or family index
  // families, in PD-node index order; member 0 is the node itself
  std::vector<int> fam_node;
  std::vector<int64_t> fam_off;    // offsets into fam_members (n_fam + 1)
  std::vector<int> fam_members;    // 0-based node ids
  std::vector<double> fam_delta;   // horizon
  std::vector<double> fam_cdv;     // PD-element-only volume (cd_v)
  std::vector<uint8_t> bond_state; // per member (member 0 unused, kept 1)
  // CSR pattern of the stiffness matrix (zero-based, rows = equations)
  std::vector<int64_t> csr_ia, csr_ja;
  // element algorithm types after the crack updates (1 PD, 2 FE) and the
  // crack-cut elements found so far (civ_CracEleIDX), kept for FC 1 growth
  std::vector<int> algo;
  std::vector<int> crack_elems;
  std::vector<int> node_elem_ptr, node_elem;   // elements around each node (n_node + 1 offsets)
};

struct Model;

// input
bool read_command(const std::string& path, Command& cmd, Mesh& mesh, std::string& base_dir, Error& err);
bool read_mesh(const std::string& path, Mesh& mesh, Error& err);

// setup (pdsolve::setDatModel restated)
// device >= 0: the family member search and the CSR pattern run on that GPU
// (identical results)
// pattern = false skips the CSR pattern (and prepare_model its scatter map)
bool build_setup(const Mesh& mesh, const Command& cmd, Setup& s, Error& err, int device = -1, bool pattern = true);
// FC 1 growth of the PD region after crack tips moved (updateEnrichRegion,
// pdsolve.cpp:8871-8908): `segs` holds the new segment (old tip, new tip) of
// every crack that propagated, in crack order.  Elements cut by a segment,
// and FE elements within me * min_delta of them, become PD; PDBEs, node types
// and the CSR pattern are rebuilt; the new PD nodes get families appended
// after the existing ones (intact bonds), and the families touching the new
// PD elements gain their volume.  *grew tells whether any element became PD.
void grow_pd_region(const Mesh& mesh, const Command& cmd, Setup& s,
                    const std::vector<std::array<double, 9>>& segs, bool* grew);
// updateBondstate (pdsolve.cpp:8910-9004): every intact bond of a family in
// the blocks around `seg` that crosses it is broken; returns the count
int cut_bonds_by_segment(const Mesh& mesh, Setup& s, const std::array<double, 9>& seg);
// family members and offsets of s.fam_node on the GPU, in the host loop's
// order; err.code 7 on a CUDA failure (k_setup.cu)
bool gpu_family_search(const Mesh& m, Setup& s, const std::vector<double>& delta_node, double md, int device,
                       Error& err);
// csr_ia / csr_ja of build_csr_pattern on the GPU, identical (k_setup.cu)
bool gpu_csr_pattern(const Mesh& m, Setup& s, int device, Error& err);
void build_csr_pattern(const Mesh& mesh, Setup& s);

// element utilities (fe_host.cpp)
double elem_volume(const Mesh& mesh, int e);
void elem_center(const Mesh& mesh, int e, double xc[3]);
// D matrix (3x3 in 2D, 6x6 in 3D) and Lame constants as in pdsolve::pdsolve (pdsolve.cpp:36-94).
void material_D(const Mesh& mesh, std::vector<double>& D, double& lambda, double& mu);
void ke_quad4(const double xN[4][3], const double* D, double* Ke /*8x8*/);
void ke_hex8(const double xN[8][3], const double* D, double* Ke /*24x24*/);
void me_quad4(const double xN[4][3], double rho, double* Me);
void me_hex8(const double xN[8][3], double rho, double* Me);
// strain-displacement matrices at the stress-extrapolation Gauss points, in
// the order used by eleFitStresses (pdfemEleQuad4N.cpp:73-131, pdfemEleBrick8N.cpp).
void b_gauss_quad4(const double xN[4][3], double* B /*4 x 3 x 8*/);
// 3-node triangle in the 4-node layout (fourth slot = third node, zero rows
// and columns): constant-strain stiffness, consistent mass, B at every point
void ke_tri3(const double xN[4][3], const double* D, double* Ke /*8x8*/);
void me_tri3(const double xN[4][3], double rho, double* Me /*8x8*/);
void b_gauss_tri3(const double xN[4][3], double* B /*4 x 3 x 8*/);
void b_gauss_hex8(const double xN[8][3], double* B /*8 x 6 x 24*/);
void extrap_L(int dim, double* L /*4x4 or 8x8*/);
void nbc_unit_force(int dim, const double xN[4][3], double* Fe /*2x2 or 4x3*/);

}  // namespace pdx
