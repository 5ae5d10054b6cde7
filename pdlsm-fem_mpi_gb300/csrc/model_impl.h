// Internal definition of pdx_model: host setup, host-prepared device inputs,
// device buffers and run state.  Shared by capi.cpp and drivers.cpp.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/pdx.h"
#include "device.h"
#include "model.h"

namespace pdx {

// Host arrays derived from Setup that the kernels need.
struct Prepared {
  std::vector<double> mass_node;     // lumped mass per node (active DOFs)
  std::vector<double> mass_eq;       // per equation, as the reference's cdp_MGlo
  std::vector<uint8_t> bcflag;       // varying prescribed DOF bits
  std::vector<double> dtv;           // n_node*3
  std::vector<double> u0;            // n_node*dim initial DOF values
  std::vector<int> fam_ptr;          // bond offsets (self excluded)
  std::vector<int> nbr;              // bond neighbours
  std::vector<uint32_t> state_bits;  // initial bond states
  std::vector<int> fam_intact;
  std::vector<int> fam_brk;          // least intact count with damage <= 0.42
  std::vector<double> fam_s0;        // critical stretch per family
  std::vector<double> dt2m;          // dt^2 / mass per node
  std::vector<int> fam_corr;         // slot offset or -1
  std::vector<int> fam_wd;           // W*D index or -1
  std::vector<double> wd;            // dim x nv per corrected family
  int64_t n_corr = 0;
  std::vector<int> feonly;           // FE-only nodes (spatially tiled order)
  std::vector<int> fam_order;        // families in spatially tiled order
  // FE elements (order of Setup::fe)
  std::vector<int> fe_conn;          // 8 per element
  std::vector<int> fe_cls;
  std::vector<double> ke, me, bgp;   // per class tables
  std::vector<double> L;             // extrapolation matrix
  std::vector<int> fe_adj_ptr, fe_adj;
  int n_cls = 0;
  // node stencils of FE-only nodes (per FE-only node in feonly order)
  std::vector<int> st_cls;           // class, -1: element path
  std::vector<int> st_nbr;           // kStencil2|3 neighbour slots per node, -1 padded
  std::vector<double> st_blk;        // per class: slots x D x D blocks
  int n_st_cls = 0;
  std::vector<int> st_dcls;          // delta class per FE-only node, -1 none
  std::vector<int> st_delta;         // per delta class: slots of (neighbour - node), INT32_MIN empty
  int n_st_dcls = 0;
  bool st_use_delta = false;         // kernels read delta classes instead of st_nbr
  // 2D FE-only nodes by lattice tile (mixed step kernel; structured meshes
  // whose lattice rows are numbered consecutively): per tile, the staged
  // box's rows as (first node id, presence bits) and the stencil class of
  // each tile site (-1 none; bit 14: the PD part of the step reads the node's
  // FP32 record); per class the 2 x 2 blocks by lattice offset
  std::vector<int> tile_rows;
  std::vector<int16_t> tile_cls;
  std::vector<float> lat_blk;
  int n_tiles = 0;
  std::vector<int> fe_rest;          // with tiles: FE-only items (feonly order) outside every tile
  // traction BCs
  std::vector<int> ext_ptr, ext_nbc;
  std::vector<double> ext_f;
  // scatter map into the CSR pattern
  std::vector<int> rel_bond, rel_self, rel_fe;
  std::vector<double> D;             // constitutive matrix
  double lambda = 0, mu = 0;
};

// A specimen of a batched model: where its nodes, family members, equations,
// families and bonds start in the merged arrays.
struct BatchPart {
  int64_t node_off = 0, member_off = 0, eq_off = 0, fam_off = 0, bond_off = 0;
  int64_t n_node = 0, n_member = 0, n_eq = 0;
  int n_fam = 0;
  double dt = 0;
  std::string title;
};

// Families [fam0, fam0 + n_fam) get their PDLSM coefficients with these constants.
struct CoeffSeg {
  int fam0 = 0, n_fam = 0;
  double nlf = 0, lambda = 0, mu = 0;
};

struct DevBuf {
  std::vector<void*> ptrs;
  template <typename T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (T*)p;
  }
  void free_all() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

struct Learned;

// The coarse grid of the two-level BiCGStab (method 8) of a 2D model.
struct TwoLevelHost {
  DevBuf buf;
  TwoLevelDev dev;
  double cell_len[2] = {0.0, 0.0};   // coarse cell size per axis (no coupling may be longer)
};

}  // namespace pdx

struct pdx_model {
  pdx::Mesh mesh;
  pdx::Command cmd;
  pdx::Setup setup;
  pdx::Prepared prep;
  std::string base_dir;
  int device = -1;
  int mixed = 0;
  int verbose = 0;
  int lanes = 0;                     // lanes per PD family in the step kernel
  int fe_lanes = 0;                  // lanes per FE-only node
  bool tune = false, tune_lanes = false, tune_fe_lanes = false;
  bool has_device = false;
  cudaStream_t stream = nullptr;
  pdx::DevBuf buf;
  pdx::DevView view{};
  // device arrays kept by name for updates
  double* d_u[2] = {nullptr, nullptr};
  float4* d_uf[2] = {nullptr, nullptr};
  float4* d_brec = nullptr;          // mixed-precision bond records
  // reaction forces (RF keyword): the elements touching the RF nodes, their
  // stiffness and RF-node masks, and one history row (uc, RFx, RFy, RFz) per step
  bool rf = false;
  int rf_n_el = 0;
  int64_t rf_uc_index = -1;          // u_all index of the first RF EBC's DOF, or -1
  int* d_rf_conn = nullptr;
  double* d_rf_ke = nullptr;
  int* d_rf_mask = nullptr;
  double* d_rf_part = nullptr;
  double* d_rf_hist = nullptr;
  int64_t rf_cap = 0;
  int64_t rf_rows = 0;               // rows written so far (highest row + 1)
  // FC 2 bond breaking (2D explicit runs): block lists and candidate buffers
  bool fc2 = false;
  int* d_fc2_blk_ptr = nullptr;
  int* d_fc2_blk_fam = nullptr;
  double* d_fc2_val = nullptr;
  int* d_fc2_bond = nullptr;
  int* d_fc2_fam = nullptr;
  int* d_fc2_count = nullptr;
  int fc2_cap = 0;
  double* d_fc2_max = nullptr;       // largest sigma1 of the last pass (quasi-static load ratio)
  double* d_ebc_vel = nullptr;       // n_node*3 velocities of the varying EBC DOFs (quasi-static FC 2)
  int fc2_kept = 0;                  // candidates cut by the last pass
  double fc2_max = 0.0;
  int quasi_load = 0;                // quasi-static load steps applied (natural-BC row)
  int ke_smem = 0;                   // floats of FE classes staged in shared memory
  uint32_t* d_state = nullptr;
  int* d_intact = nullptr;
  double* d_nbcval = nullptr;        // (nsteps + 2) * n_nbc
  double* d_D = nullptr;
  double* d_bgp = nullptr;
  double* d_L = nullptr;
  double* d_me = nullptr;
  int64_t* d_ia = nullptr;
  int* d_ja = nullptr;
  int* d_rel_bond = nullptr;
  int* d_rel_self = nullptr;
  int* d_rel_fe = nullptr;
  double* d_fam_cdv = nullptr;
  double* d_Kval = nullptr;
  double* d_Mval = nullptr;
  double* d_sigma = nullptr;
  double* d_phi = nullptr;
  double* d_tmp_all = nullptr;       // n_node*dim scratch
  double* d_tmp_eq[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // explicit run state
  // batched models (empty for a single specimen)
  std::vector<pdx::BatchPart> batch;
  std::vector<pdx::CoeffSeg> coeff_segs;
  std::vector<double> mat_D, mat_nu; // per specimen: constitutive matrix, Poisson ratio
  std::vector<int> node_mat;         // specimen of each node
  int* d_node_mat = nullptr;
  double* d_mat_nu = nullptr;
  // implicit Newmark state (pdx_newmark_*) and the learned preconditioner
  double* d_vel = nullptr;
  double* d_acc = nullptr;
  bool newmark_ready = false;
  pdx::Learned* learned = nullptr;
  pdx::TwoLevelHost* twolevel = nullptr;   // built at the first method-8 solve
  // FC 1 (2D): the current crack segments (previous tip, tip), per crack the
  // last evaluation (KI, KII, Keq, moved), the last crack's Keq (the load
  // ratio's reference value) and whether any tip moved in the last pass
  std::vector<std::array<double, 9>> cracks;
  std::vector<std::array<double, 4>> crack_sif;
  double fc1_keq = 0.0;
  bool fc1_moved = false;
  bool fc1_changed = false;          // the set-up differs from the mesh's (growth or cut bonds)
  int cur = 0;                       // index of the buffer holding u_n
  int64_t steps_done = 0;
  // explicit runs apply a step's FC 3 failure pass at the start of the next
  // step; pdx_get_state applies it when the state is read.  Quasi-static
  // increments and Newmark steps finish their own passes.
  bool explicit_run = true;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int graph_parity = 0;
};

namespace pdx {
pdx_status set_error(pdx_status code, const std::string& msg);
// host arrays the kernels need, from m->setup (prepare.cpp); step_tables =
// false leaves out the explicit step's FE-only node stencils and tiles (the
// step then takes the element path for those nodes)
bool prepare_model(pdx_model* m, Error& err, bool step_tables = true);
pdx_status cuda_check(cudaError_t e, const char* what);
void write_vtk(const pdx_model* m, const std::string& path, const std::vector<double>& u_all,
               const std::vector<double>& sigma, const std::vector<double>& phi, bool binary);
// <base>.sig and <base>.disp, the text files beside an ASCII VTK result
void write_sig_disp(const pdx_model* m, const std::string& base, const std::vector<double>& u_all,
                    const std::vector<double>& sigma);
pdx_status model_stress(pdx_model* m, const double* d_u_all, bool sigma, bool phi);
pdx_status rf_record(pdx_model* m, int64_t row);
// FC 2 pass on the current state; with `report` it also reads back how many
// candidates were cut (fc2_kept) and the largest sigma1 (fc2_max)
pdx_status fc2_pass(pdx_model* m, bool report = false);
// FC 1 pass on the current state (node stresses already computed): SIFs of
// every crack from the interaction integral, tip growth where Keq > K_Ic and,
// with `grow` (quasi-static runs), the PD region and bond states updated
// (fc1.cpp)
pdx_status fc1_pass(pdx_model* m, bool grow);
// PD-region growth and bond cuts of the moved cracks' new segments, then the
// device model brought up to date (fc1.cpp)
pdx_status apply_growth(pdx_model* m, const std::vector<std::array<double, 9>>& moved);
// cracks back to the mesh's pre-cracks and, if a run changed it, the set-up
// and device model back to the mesh's (fc1.cpp)
pdx_status fc1_reset(pdx_model* m);
// the device model re-derived from m->setup after FC 1 changed it, keeping
// displacements, node stresses and the reaction-force history; with
// keep_twolevel, method 8's coarse grid and inverse stay for the next solves
// (capi.cpp)
pdx_status rebuild_device(pdx_model* m, bool keep_twolevel = false);
// bond states of m->setup uploaded into the device's state bits (capi.cpp)
pdx_status upload_bond_states(pdx_model* m);
pdx_status assemble_device(pdx_model* m, int mode, const double* d_v_all, int nbc_row);
extern const int kEqTemps;
pdx_status explicit_step_launch(pdx_model* m, int mode, int64_t step_index);
bool merge_batch(const std::vector<pdx_model*>& parts, pdx_model* out, Error& err);
void learned_destroy(pdx_model* m);
// method 8's coarse grid for the model (2D only), built once
pdx_status twolevel_prepare(pdx_model* m);
void twolevel_destroy(pdx_model* m);
inline void fill_solve_info(pdx_solve_info* info, const KrylovResult& kr, double seconds) {
  if (!info) return;
  info->iterations = kr.iterations;
  info->rel_residual = kr.rel_residual;
  info->seconds = seconds;
  info->converged = kr.converged;
  info->method_used = kr.method;
  info->refinements = kr.refinements;
  info->setup_seconds = kr.setup_ms * 1e-3;
}
}  // namespace pdx
