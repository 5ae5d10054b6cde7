// Device-resident model: structure-of-arrays layouts in HBM for nodes, PD
// families and bonds, FE elements and the CSR stiffness pattern, plus the
// launch wrappers of the kernels in k_*.cu.  Bond arrays are component-major
// (coef[c * n_bond + b]) so that the lanes working on one family read
// consecutive addresses.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace pdx {

constexpr int kMaxFeAdj = 8;      // FE elements around a node (Q4: 4, Hex8: 8)
constexpr int kStencil2 = 9;      // neighbour slots of an FE-only node's stencil (Q4)
constexpr int kStencil3 = 27;     // (Hex8)

// Lattice tiles of 2D FE-only nodes (mixed step kernel): one block of 256
// threads per tile of 16 x 16 lattice sites, one node per thread; the tile's
// nodes and a one-site halo (18 x 18 sites) are staged in shared memory.
struct Tile2 {
  static constexpr int X = 16, Y = 16;
  static constexpr int WX = X + 2, WY = Y + 2;
  static constexpr int ROWS = WY;               // staged rows (x runs)
  static constexpr int SITES = WX * WY;         // staged sites
  static constexpr int NODES = X * Y;           // tile sites (= threads)
  static constexpr int SLOTS = 9;               // lattice offsets {-1,0,1}^2
  static constexpr int BW = 4;                  // floats per 2 x 2 block
};
constexpr int kTileShadowBit = 1 << 14;
constexpr int kTileClsMask = kTileShadowBit - 1;

// Everything a kernel needs, as raw device pointers (passed by value).
struct DevView {
  int dim, n_node, n_fam, n_feonly, n_eq;
  int64_t n_bond;
  int n_corr_bond;
  // nodes
  const double* X;          // n_node*3
  const float4* Xf;         // n_node (x, y, z, 0) FP32 copy
  const int* eq;            // n_node*dim
  const double* mass;       // n_node lumped mass of the node's active DOFs
  const uint8_t* bcflag;    // bit i: DOF i prescribed and varying (VEBC)
  const double* dtv;        // n_node*3 per-step increment of varying prescribed DOFs
  // families
  const int* fam_node;
  const int* fam_ptr;       // n_fam+1 bond offsets
  const int* fam_order;     // family of each step-kernel work item (spatially tiled order)
  const int* fam_corr;      // offset of the family's bonds in the PDBE-correction arrays, -1 if none
  int* fam_intact;          // intact bond count
  const int* feonly_node;   // nodes without family
  // bonds
  const int* nbr;
  uint32_t* state;          // 1 bit per bond, 1 = intact
  const double* coef64;     // (3|6) * n_bond symmetric block G*dv_k*dv_m
  const float* coef32;
  const double* corr64;     // (4|9) * n_corr_bond general PD-boundary block
  const float* corr32;      // FP32 per bond record: 2D 4 floats, 3D 8 floats (+ corr32_last)
  const float* corr32_last; // 3D: the ninth entry of each block
  const double* cvec;       // dim * n_bond strain-operator columns omega*g*dv_m
  // FE
  const int* fe_conn;       // n_fe*8
  const int* fe_cls;        // n_fe
  const double* ke64;       // n_cls * nd*nd
  const float* ke32;
  const int* fe_adj_ptr;    // n_node+1
  const int* fe_adj;        // (fe_local << 3) | local node
  // node stencils of FE-only nodes (indexed like feonly_node)
  const int* st_cls;        // stencil class, -1 = element path; null = none
  const int* st_nbr;        // kStencil2|3 neighbour nodes per FE-only node, -1 padded (when st_delta is null)
  const int* st_dcls;       // delta class per FE-only node
  const int* st_delta;      // per delta class: kStencil2|3 offsets neighbour - node, INT32_MIN empty; or null
  const float* st_blk32;    // per class and slot: 3D 12 floats (3x3 row-major + pad), 2D 4 floats
  const double* st_blk64;   // per class and slot: D*D doubles
  // lattice tiles of 2D FE-only nodes (n_tiles = 0: none)
  int n_tiles;
  const int2* tile_rows;    // per tile Tile2::ROWS (first node id, presence bits of the row's WX sites)
  const int16_t* tile_cls;  // per tile Tile2::NODES: class | kTileShadowBit, -1 no FE-only node
  const float* lat_blk;     // per class Tile2::SLOTS 2 x 2 blocks by lattice offset (dx + 1) + 3 (dy + 1)
  const int* fe_rest;       // with tiles: FE-only items outside every tile (per-node path)
  int n_rest;
  // external force (traction BCs): per node list of (nbc id, unit force)
  const int* ext_ptr;       // n_node+1 or null
  const int* ext_nbc;
  const double* ext_f;      // 3 per entry
  int n_nbc;
  // material / failure
  double s0, s0_pert;
  uint64_t s0_seed;
  uint32_t s0_seed32;       // folded seed of the per-bond draw
  int fail3;
  const int* fam_brk;       // least intact-bond count at which a family may still break (damage <= 0.42)
  const double* fam_s0;     // critical stretch of each family (before the per-bond draw)
  const float* fam_s0f;
  const double* dt2m;       // dt^2 / lumped mass per node (0 without active DOFs)
  const float* dt2m_f;      // the same in FP32 (mixed-precision update)
};

struct StepArgs {
  DevView v;
  const double* u_n;        // n_node*dim, stored DOF values after the previous step
  double* u_next;           // u_{n-1} in, u_{n+1} out (same buffer)
  const float4* uf_n;       // mixed: node records of u_n, [2n] position, [2n+1] displacement + flags
  float4* uf_next;
  const double* nbc_val;    // n_nbc values for this step (null without NBCs)
  double dt;
  int mode;                 // 0 first step, 1 regular step, 2 failure pass only
  float4* brec;             // mixed: per-bond records (3D: 2 float4, 2D: 1)
  int ke_smem;              // mixed: floats of FE stiffness classes staged in shared memory (0: global)
  float s0f, pertf;         // FP32 copies of s0 and its relative perturbation
  int pd_blocks;            // set by the launcher: blocks [0, pd_blocks) take the PD families
};

struct ForceArgs {
  DevView v;
  const double* u;          // n_node*dim DOF values
  double* f_eq;             // n_eq output
  const double* nbc_val;    // add external forces when non-null
  double ext_scale;
};

struct CoeffArgs {
  int dim, n_fam;
  int64_t n_bond;
  int64_t n_corr;           // bonds of families with a PD-boundary correction
  const double* X;
  const double* vol;
  const int* fam_node;
  const int* fam_ptr;
  const int* nbr;
  const double* fam_delta;
  const double* fam_cdv;
  const int* fam_corr;
  const double* wd;         // per corrected family: dim x nv matrix W*D
  const int* fam_wd;        // index into wd per family, -1 none
  double nlf, lambda, mu;
  double* coef64;
  float* coef32;
  double* corr64;
  float* corr32;            // per bond record (see DevView)
  float* corr32_last;
  double* cvec;
  double* A_out;            // optional dumps
  double* g_out;
  double* d_out;
  double* G_out;
  int* err;                 // set to 1 + family on a singular moment matrix
};

struct StressArgs {
  DevView v;
  const double* u;
  const double* D;          // nv x nv per material
  const int* node_mat;      // material of each node (null: material 0)
  const double* bgp;        // per class: ngp * nv * nd strain-displacement at stress Gauss points
  const double* L;          // ngp x ngp extrapolation
  int protype;
  const double* nu;         // Poisson ratio per material
  double* sigma;            // n_node*6
  double* phi;              // n_node
};

struct AsmArgs {
  DevView v;
  const int64_t* ia;
  const int* rel_bond;      // per bond: column offset of node m in row of node k
  const int* rel_self;      // per family: column offset of node k in its own row
  const int* rel_fe;        // per FE adjacency entry: 8 column offsets
  const double* table;      // element matrix table (Ke or Me classes), nd*nd per class
  double* a;                // nnz values (accumulated)
  int with_pd;              // add PD bond blocks
  double pd_diag_rho;       // >0: add rho*cd_v on the diagonal of family rows (consistent mass)
  const double* fam_cdv;
};

// kernel launchers (return cudaError_t of the launch)
cudaError_t launch_coeff(const CoeffArgs& a, cudaStream_t s);
// lp: lanes per PD family (4, 8, 16); lf: lanes per FE-only node (2, 4, 8)
bool step_lanes_valid(int lp, int lf);
cudaError_t launch_step(const StepArgs& a, int mixed, int lp, int lf, cudaStream_t s);
cudaError_t launch_step_mixed(const StepArgs& a, int lp, int lf, cudaStream_t s);
cudaError_t launch_force(const ForceArgs& a, cudaStream_t s);
// lanes: lanes per PD family of the step kernel that will read the records
// (3D records name the neighbour of the bond 2 * lanes further on)
cudaError_t launch_pack_bonds(const DevView& v, float pertf, int lanes, float4* rec, cudaStream_t s);
cudaError_t launch_stress(const StressArgs& a, cudaStream_t s);
// FC 1 sample points of the interaction-integral path (2D): per point
// {kind, n0, n1, n2, n3}; kind 0 is an FE element evaluated at its centre
// (nodes n0..n3, a triangle repeats its third node), kind 1 a PD node n0 of
// family n1.  Writes per point the displacement gradient (dux/dx, duy/dy,
// dux/dy, duy/dx) and the stress (xx, yy, xy): 7 doubles.
struct Fc1PointArgs {
  DevView v;
  const double* u;          // n_node * 2
  const double* sigma;      // n_node * 6 node stresses
  const double* D;          // 3 x 3 constitutive matrix
  const int* pts;           // 5 per point
  int n_pts;
  double* out;              // 7 per point
};
cudaError_t launch_fc1_points(const Fc1PointArgs& a, cudaStream_t s);
cudaError_t launch_assemble(const AsmArgs& a, cudaStream_t s);
cudaError_t launch_newmark_predict(const DevView& v, const double* u, const double* vel, const double* acc,
                                   double dt, double beta, double* upred, cudaStream_t s);
cudaError_t launch_newmark_update(int n, const double* vel0, const double* a0, const double* a1, double dt,
                                  double beta, double gamma, double* u_eq, double* vel, cudaStream_t s);
cudaError_t launch_axpby_scale(int64_t n, const double* x, double alpha, double* y, double beta, cudaStream_t s);
cudaError_t launch_scatter_eq(const DevView& v, const double* u_eq, double* u_all, cudaStream_t s);
cudaError_t launch_gather_eq(const DevView& v, const double* u_all, double* u_eq, cudaStream_t s);
cudaError_t launch_advance_prescribed(const DevView& v, double* u_all, cudaStream_t s);
cudaError_t launch_advance_prescribed_quasi(const DevView& v, double* u_all, cudaStream_t s);
// the quasi-static rule with a load ratio (setVaryEssentialBC, FC 2): vel =
// n_node*3 velocities of the varying EBC DOFs
cudaError_t launch_advance_prescribed_ratio(const DevView& v, double* u_all, const double* vel, double dt,
                                            double rati, cudaStream_t s);

// FC 2 (maximum principal stress, Top-K) bond breaking after an explicit step, 2D (k_fc2.cu)
struct Fc2Args {
  DevView v;
  const double* sigma;      // n_node * 6 nodal stresses of the new state
  double sigult;            // ultimate stress of the material
  double half_min_delta;    // half-length of a cut segment: 0.5 * min(delta)
  double lbc0, lbc1, block_size;   // the set-up's block grid
  int nbx, nby;
  const int* blk_ptr;       // nbx * nby + 1
  const int* blk_fam;       // families of each block's nodes, in the block's node order
  float4* brec;             // mixed-precision bond records (sign = state), or null
  double* cand_val;         // candidates: sigma1, bond, family
  int* cand_bond;
  int* cand_fam;
  int* count;               // number of candidates found (may exceed cap)
  int cap;
  double* max_sigma1;       // largest sigma1 over intact bonds (from 0), or null
};
// reaction forces of one step (k_post.cu): Fe = Ke u_e over the elements
// touching the RF nodes, summed over those nodes in element order;
// hist_row = (uc, RFx, RFy, RFz), uc = u_all[uc_index] (0 if uc_index < 0)
cudaError_t launch_reaction(int n_el, int nen, int dim, const int* conn, const double* ke, const int* mask,
                            const double* u_all, int64_t uc_index, double* part, double* hist_row, cudaStream_t s);
cudaError_t launch_fc2_candidates(const Fc2Args& a, cudaStream_t s);
cudaError_t launch_fc2_cut(const Fc2Args& a, cudaStream_t s);
cudaError_t launch_newmark_matrix(int64_t nnz, double* k, const double* m, double beta, double dt, cudaStream_t s);
cudaError_t launch_shadow(const DevView& v, const double* u_all, float4* uf, cudaStream_t s);
cudaError_t launch_load_pair(const DevView& v, const double* un_eq, const double* unm1_eq, double* u_cur,
                             double* u_prev, float4* uf, cudaStream_t s);
cudaError_t launch_store_eq(const DevView& v, const double* u_all, double* u_eq, cudaStream_t s);

// Krylov solvers on a device CSR matrix (k_krylov.cu)
struct DevCsr {
  int64_t n = 0, nnz = 0;
  const int64_t* ia = nullptr;
  const int* ja = nullptr;
  const double* a = nullptr;
};
struct KrylovResult {
  int iterations = 0;
  double rel_residual = 0;
  int converged = 0;
  int method = -1;        // the method that produced the iterate
  int refinements = 0;    // method 3: FP64 refinement steps
  double setup_ms = 0;    // method 8: forming the coarse matrix and its inverse
};
// Two-level right preconditioner of BiCGStab method 8 (2D): Jacobi plus the
// Galerkin coarse correction P (P^T A P)^-1 P^T on a lattice coarse grid over
// the nodes' bounding box, P bilinear per DOF component.  Built by the model
// (drivers.cpp: twolevel_prepare); the coarse matrix and its inverse are
// formed on the device for every solve (twolevel_setup).
struct TwoLevelDev {
  int nc = 0;                 // coarse DOFs
  int nxn = 0, nyn = 0;       // coarse nodes per axis
  int64_t n = 0;              // fine equations
  const int* pidx = nullptr;  // n * 4: coarse DOF of each bilinear corner
  const float* pw = nullptr;  // n * 4: weights
  const int* ecell = nullptr; // n: the equation's cell x | y << 12 | component << 24
  const int* rptr = nullptr;  // nc + 1: rows of P^T
  const int* ridx = nullptr;  // fine equation
  const float* rw = nullptr;  // weight
  double* B = nullptr;        // n * 32: A P on each row's 4x4-node, 2-component window
  double* M = nullptr;        // nc x 2 nc: [P^T A P | I], after setup [diagonal | (P^T A P)^-1]
  double* colk = nullptr;     // nc: reciprocals of the final diagonal
  double* colbuf = nullptr;   // 2 nc: the pivot column of a step and of the next, contiguous
  double* diag0 = nullptr;    // nc: the diagonal before elimination
  double* rpiv = nullptr;     // 2: reciprocal of a step's pivot and of the next
  double* rc = nullptr;       // nc: restricted vector
  double* yc = nullptr;       // nc: coarse solution
  int* ok = nullptr;          // set to 0 when a pivot vanishes
  unsigned long long* hash = nullptr;   // fingerprint of the matrix values (device word)
  // host side: the Gauss-Jordan sequence (2 nc launches on fixed buffers),
  // captured once as a CUDA graph and replayed for every solve
  cudaGraphExec_t gj = nullptr;
  // host side: the fingerprint of the values whose coarse inverse M holds
  bool have_inverse = false;
  unsigned long long inverse_of = 0;
  // host side: keep_stale lets the inverse serve a changed matrix (set after
  // a local change such as an FC 1 growth step) while a solve needs at most
  // 1.5 times the iterations of the first solve with it (its_ref)
  bool keep_stale = false;
  bool formed = false;        // the last set-up formed the inverse
  int its_ref = 0;
};
cudaError_t twolevel_setup(const DevCsr& A, TwoLevelDev& t, cudaStream_t s, bool* usable);
cudaError_t krylov_solve(const DevCsr& A, const double* b, double* x, int method, double rtol, int max_iter,
                         int block_dim, cudaStream_t s, KrylovResult* res, TwoLevelDev* tl = nullptr);
cudaError_t spmv(const DevCsr& A, const double* x, double* y, cudaStream_t s);

// Additive second level of a preconditioner: z += C(r) (learned.cpp, k_learned.cu).
struct CoarseCorrection {
  virtual ~CoarseCorrection() = default;
  virtual cudaError_t add(const double* r, double* z, cudaStream_t s) = 0;
};
// Called with the current iterate, residual and preconditioned residual every
// `every` iterations of a flexible CG solve (training-data collection).
struct IterHook {
  virtual ~IterHook() = default;
  int every = 1;
  virtual cudaError_t on_iter(int it, const double* x, const double* r, const double* z, cudaStream_t s) = 0;
};
// Flexible CG with block-Jacobi (d x d blocks of consecutive rows) plus an
// optional additive coarse correction; each direction is A-orthogonalised
// against the last `trunc` directions (trunc = 1 with a fixed preconditioner
// is PCG); stops on the true FP64 residual.  A solve whose residual has not
// dropped 10x over `stall_window` iterations (0: never) stops early with
// res->converged = 0, so that the caller can fall back.
cudaError_t krylov_fcg(const DevCsr& A, const double* b, double* x, double rtol, int max_iter, int block_dim,
                       CoarseCorrection* coarse, IterHook* hook, int stall_window, int trunc, cudaStream_t s,
                       KrylovResult* res);
// Jacobi PCG with its work space in a fixed device array (no allocation);
// n <= noalloc_max_n(), one solve at a time per device.
cudaError_t krylov_pcg_noalloc(const DevCsr& A, const double* b, double* x, double rtol, int max_iter, int use_x0,
                               cudaStream_t s, KrylovResult* res);
int64_t noalloc_max_n();

}  // namespace pdx
