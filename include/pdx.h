/*
 * pdx.h - C ABI of the GB300 PDLSM-FEM hot path.
 *
 * The reference (QibangLiu/PDLSM-FEM_mpi) is one MPI executable with no
 * library API.  This header is the seam a host program binds instead of the
 * reference's internals; every entry point names the reference function it
 * replaces.  Plain C types only: the caller owns every host pointer, the
 * library owns the device buffers of a model.  Errors are returned as
 * pdx_status codes (the reference prints and exit()s); pdx_last_error() gives
 * the message of the last failing call on the calling thread.  All compute
 * runs on one GPU; a model is used from one host thread at a time and its work
 * is ordered on the model's own CUDA stream.
 */
#ifndef PDX_H
#define PDX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pdx_status {
  PDX_OK = 0,
  PDX_ERR_IO = 1,           /* a file cannot be opened or written */
  PDX_ERR_PARSE = 2,        /* malformed command or mesh file, bad keyword value */
  PDX_ERR_UNSUPPORTED = 3,  /* input outside this library's scope (Tet4, FC 1 in dynamic runs, ...) */
  PDX_ERR_INVALID = 4,      /* bad argument (null pointer, wrong size, wrong state) */
  PDX_ERR_CUDA = 5,         /* a CUDA runtime call failed */
  PDX_ERR_SINGULAR = 6,     /* a PDLSM moment matrix is singular (reference: dgesv info > 0) */
  PDX_ERR_NOCONV = 7,       /* Krylov solve did not reach the tolerance */
  PDX_ERR_NODEVICE = 8,     /* compute requested on a model created without a device */
  PDX_ERR_NUMERIC = 9       /* NaN or Inf detected in the state */
} pdx_status;

typedef struct pdx_model pdx_model;

typedef struct pdx_options {
  int device;      /* CUDA device ordinal; -1 builds the host setup only (no compute) */
  int precision;   /* -1: PRECISION keyword of the command file; 0 FP64; 1 mixed (FP32 forces) */
  int lanes;       /* lanes per PD family in the step kernel (4, 8, 16); 0 = default (3D 8, 2D 4);
                      < 0 = timed on the model at pdx_explicit_init.  The lane counts
                      fix the order of the force sums: a tuned choice may change
                      results in the last bits from run to run. */
  int verbose;
  int fe_lanes;    /* lanes per FE-only node in the step kernel (1, 2, 4, 8); 0 = default (3D 4, 2D 1);
                      < 0 = timed on the model */
} pdx_options;

typedef struct pdx_model_info {
  int dim, n_node, n_elem, n_eq, n_fam, n_pdbe, n_fe, n_fe_classes;
  int64_t n_bond, nnz;
  int solver;      /* 0 dynamic, 1 static, 2 quasi-static (SOLVER keyword) */
  int newmark, lumped, fail_flag, precision, nsteps, save_freq, lanes, fe_lanes;
  double dt, min_delta, max_delta, s0, s0_pert;
} pdx_model_info;

typedef struct pdx_solve_opts {
  int method;      /* 0 Jacobi PCG, 1 block-Jacobi PCG, 2 BiCGStab (Jacobi), 3 mixed PCG + FP64 refinement,
                      6 GMRES(30) (Jacobi), 7 mixed BiCGStab + FP64 refinement (FP32 inner solves with
                      an FP32 copy of the matrix; FP64 residuals and updates) */
  double rtol;     /* relative true residual ||b - A x|| / ||b|| */
  int max_iter;
  int use_x0;      /* 1: x holds the initial guess */
} pdx_solve_opts;

typedef struct pdx_solve_info {
  int iterations;        /* summed over the requested method and its fallbacks */
  double rel_residual;   /* true FP64 residual ||b - A x|| / ||b|| */
  double seconds;        /* device time of the solve */
  int converged;
  int method_used;       /* the method whose iterate was returned: the requested
                            one, or 2 (BiCGStab) / 6 (GMRES) after a fallback */
  int refinements;       /* methods 3 and 7: FP64 refinement steps (FP32 inner solves) */
  double setup_seconds;  /* method 8: device time of forming the coarse matrix and its inverse (in seconds) */
} pdx_solve_info;

const char* pdx_last_error(void);
const char* pdx_version(void);

/* Reads the command file and the mesh it names, then builds the model exactly
 * as pdsolve::pdsolve + setDatModel do (SourceFiles/Solver/pdsolve.cpp:20-151,
 * fioFile.cpp:54-462, datModel.cpp:58-326): DOF numbering, volumes, block hash,
 * PD/FE split with crack-cut elements, PD boundary elements, families by the
 * union rule, pre-crack bond states and the CSR pattern.  With a device it
 * uploads the model and builds every bond's PDLSM coefficients on the GPU. */
pdx_status pdx_model_create_from_cmd(const char* cmd_path, const pdx_options* opts, pdx_model** out);
void pdx_model_destroy(pdx_model* m);
pdx_status pdx_model_get_info(const pdx_model* m, pdx_model_info* info);

/* Host setup arrays, by name (count in elements): "eq" (int32, N*d), "vol_node",
 * "vol_elem" (f64), "node_type", "fam_off" (int64, reference member layout,
 * member 0 = the node itself), "fam_members" (int32, 0-based), "fam_horizon",
 * "fam_cdv" (f64), "bond_state0" (uint8, member layout), "pdbe" (int32, n*4),
 * "pde_idx", "fe_idx" (int32), "csr_ia", "csr_ja" (int64), "mass" (f64, lumped
 * per equation), "u0" (f64, N*d initial DOF values), "geom" (f64: min delta,
 * max delta, block size, lbc[3], rtc[3]); the mixed step kernel's lattice
 * tiles of 2D FE-only nodes: "tile_rows" (int32, per tile and staged row:
 * first node id, presence bits), "tile_cls" (int16, per tile site: stencil
 * class | 1 << 14 when the PD part reads the node's FP32 record, -1 none),
 * "lat_blk" (f32, per class 9 blocks of 2 x 2 by lattice offset
 * (dx + 1) + 3 (dy + 1)), "fe_rest" (int32: the FE-only items, in "feonly"
 * order, that no tile covers); the assembly's scatter map (int32): "rel_bond"
 * (per bond, the offset of the neighbour's first column in its node's rows),
 * "rel_self" (per family, the node's own), "rel_fe" (8 per node-element
 * adjacency entry), with "fe_adj_ptr", "fe_adj" (element << 3 | local node)
 * and "fe_conn" (8 node ids per FE element, in "fe_idx" order). */
pdx_status pdx_model_array_len(const pdx_model* m, const char* name, int64_t* count);
pdx_status pdx_model_array(const pdx_model* m, const char* name, void* dst, int64_t count);

/* PDLSM moment matrices and bond coefficients computed on the GPU
 * (shapTens2D/3D pdsolve.cpp:1938-2064, vec_gd2D/3D :2174-2232, matG2D/3D
 * :2277-2347).  A: n_fam*na*na (na = 5 or 9), g: n_bond*d, dvec: n_bond*(3|6),
 * G: n_bond*d*d, all with bond state 1.  Any pointer may be NULL. */
pdx_status pdx_bond_coefficients(pdx_model* m, double* A, double* g, double* dvec, double* G);

/* Internal force of a displacement field, replacing
 * pdsolve::calinternalForce_CSRformat (pdsolve.cpp:5819-5840) in its explicit
 * form: F[eq] = -(K u)[eq] over PD bonds, PD boundary elements and FE elements,
 * u_all = every DOF's value (N*d, prescribed ones included), f_eq = n_eq values.
 * Uses the model's current bond states. */
pdx_status pdx_internal_force(pdx_model* m, const double* u_all, double* f_eq);

/* Explicit central-difference solve (pdfemDynamicSolver_CSRformat,
 * pdsolve.cpp:5842-6090, lumped mass) with critical-stretch bond breaking
 * (FC 3) or maximum-principal-stress breaking with Top-K after every step
 * (FC 2, 2D).  pdx_explicit_init resets the state to the mesh's initial values
 * and the pre-crack bond states; pdx_explicit_advance runs n steps on the
 * device (the first call runs step 0, u1 = u0 + dt^2/2 a0).  Steps are
 * launched as CUDA graphs when no natural BC, FC 2 or RF output needs
 * per-step work; FC 2 with Top-K > 0 reads the candidate count on the host. */
pdx_status pdx_explicit_init(pdx_model* m);
pdx_status pdx_explicit_advance(pdx_model* m, int nsteps);
/* Same as advance, timed with CUDA events on the model's stream (ms). */
pdx_status pdx_explicit_advance_timed(pdx_model* m, int nsteps, double* ms);
/* One explicit step through host buffers, the contract of timeIntegration_LM
 * (pdsolve.cpp:5113-5132): u_n and u_nm1 (n_eq, active DOFs) in, u_np1 out;
 * prescribed values and bond states are the model's.  With page-locked
 * buffers (cudaHostAlloc / cudaHostRegister, all three) the GPU reads and
 * writes them in place over the coherent host link; pageable buffers are
 * copied through device staging.  Returns after u_np1 is written. */
pdx_status pdx_explicit_step_host(pdx_model* m, const double* u_n, const double* u_nm1, double* u_np1);
int64_t pdx_explicit_step_count(const pdx_model* m);
/* Reaction forces of the RF keyword's essential BCs, one row per recorded
 * step as calReacForc writes them (pdsolve.cpp:5347-5404): (U, RFx, RFy,
 * RFz) with U the first RF EBC's current value and RF the sum of Ke u_e over
 * the elements touching the RF nodes, taken at those nodes.  Rows are
 * indexed by step: explicit runs record steps 0..n, quasi-static increments
 * and Newmark steps 1..n (row 0 stays zero).  *count = rows recorded; rows
 * (max_rows x 4) may be NULL. */
pdx_status pdx_reaction_forces(const pdx_model* m, double* rows, int64_t max_rows, int64_t* count);
/* FC 1 crack state (2D models with FC 1; replaces the crack-path rows the
 * reference writes to <title>_cp.out, pdsolve.cpp:7481-7489, and its
 * cdp_crack array).  One row of 8 doubles per pre-existing crack: the current
 * segment (x0, y0, x1, y1; x1, y1 the tip, x0, y0 the tip before the last
 * growth) and the last evaluation's KI, KII, Keq and 1 if the tip then moved
 * (0 otherwise).  pdx_quasi_step evaluates the cracks after every increment
 * (and in quasi-static runs grows the PD region behind a moved tip); a
 * static run evaluates them once.  *n_cracks = number of cracks; rows
 * (max_cracks x 8) may be NULL. */
pdx_status pdx_crack_state(const pdx_model* m, double* rows, int max_cracks, int* n_cracks);
/* One FC 1 growth step with tips given by the caller (2D; a model without a
 * device too): every crack k with moved[k] != 0 gets the segment from its
 * current tip to (tips[2k], tips[2k+1]); then, as after a moved tip in a
 * quasi-static increment (updateEnrichRegion and updateBondstate,
 * pdsolve.cpp:8871-9004), the elements those segments cut (and the FE
 * elements within me * min_delta of them) become PD, new PD nodes get
 * families after the existing ones, and every bond crossing a new segment
 * breaks.  The set-up arrays (pdx_model_array) and the device model follow. */
pdx_status pdx_crack_advance(pdx_model* m, const double* tips, const uint8_t* moved);

/* Current state: u_all (N*d), node stress sigma (N*6, slots xx yy zz xy yz zx as
 * calGlobalNodeStresses pdsolve.cpp:9540-9604), damage phi (N, calLocalDamage
 * :7338-7373) and bond states in the reference's member layout.  Stress and
 * damage are recomputed on the GPU from the current state.  NULL skips. */
pdx_status pdx_get_state(pdx_model* m, double* u_all, double* sigma, double* phi, uint8_t* bond_state);

/* Stiffness assembly in the reference's CSR layout and order through a
 * precomputed scatter map (pdfemAssembleEquasSys_CSRformat :5480-5504,
 * pdfemQuasiStaticAssembleEquasSys_CSRformat :6434-6462,
 * pdfemAssembleKNFR_CSRformat :6327-6397).  mode 1 static: F = f_ext - K_pp u_p;
 * mode 2 quasi-static: F = f_ext - K u_all; mode 3 Newmark: a = beta dt^2 K + M,
 * F = f_ext - K v.  v_all: N*d DOF values (NULL = model state).  Outputs: ia
 * (n_eq+1), ja (nnz), a (nnz), f (n_eq); any may be NULL.  ia and ja are
 * `long long`, the type of pdsolve::cip_ia / cip_ja (HeaderFiles/Solver/
 * pdsolve.h:254-255), so the reference's own arrays are passed without casts. */
pdx_status pdx_assemble_csr(pdx_model* m, int mode, const double* v_all, long long* ia, long long* ja,
                            double* a, double* f);

/* Sparse solve replacing calMatrixOperations::cluster_PARDISO_64Solver
 * (calMatrixOperations.h:47-48, calMatrixOperations.cpp:378-498): zero-based
 * CSR, real unsymmetric, one right-hand side, caller-owned host arrays.  The
 * first six arguments take the reference's own (long long& n, long long* ia,
 * long long* ja, double* a, double* rhs, double* x) without casts.  The
 * reference factorises with MKL PARDISO; this is a Krylov solve on the GPU
 * judged by the true FP64 residual. */
pdx_status pdx_solve_csr(long long n, const long long* ia, const long long* ja, const double* a,
                         const double* rhs, double* x, const pdx_solve_opts* opts, pdx_solve_info* info);

/* Allocation-free Jacobi PCG (no counterpart in the reference).  The same
 * solve as pdx_solve_csr with opts->method 0, on device-resident arrays of the
 * current CUDA device (d_ja: int32 column indices), ordered on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  All work space lives in
 * one fixed device array of the library (12.6 MB), so the call allocates no
 * device memory: for callers that reserve the GPU's memory up front or must
 * not let an allocator run inside their time-step loop.
 *   - n <= 262144 equations; larger n returns PDX_ERR_INVALID;
 *   - opts->method must be 0 (else PDX_ERR_UNSUPPORTED); use_x0 = 0 zeroes d_x;
 *   - nothing has to be zeroed beforehand;
 *   - calls that overlap in time on the same device share the work space and
 *     race: serialise them;
 *   - the first call on a device looks up the work space's address; make it
 *     before any stream capture starts.
 * info->seconds is not measured (0). */
pdx_status pdx_pcg_solve_noalloc(int64_t n, int64_t nnz, const int64_t* d_ia, const int32_t* d_ja,
                                 const double* d_a, const double* d_rhs, double* d_x, const pdx_solve_opts* opts,
                                 void* stream, pdx_solve_info* info);

/* Implicit Newmark dynamics one step at a time (pdfemDynamicNewmarkSolver_CSRformat,
 * pdsolve.cpp:6092-6290, beta and gamma from the NEWMARK keyword): predictor,
 * K_N = beta dt^2 K + M assembled on the GPU (pdfemAssembleKNFR_CSRformat
 * :6327-6397), K_N a = F solved by `method`, update (updateDispVelo
 * :6399-6422).  The reference factorises K_N with PARDISO at every step.
 * method: 0-3, 6 and 7 as pdx_solve_opts.method; 8 (2D models) BiCGStab right
 * preconditioned by Jacobi plus the Galerkin coarse correction P (P^T K P)^-1 P^T
 * on a lattice coarse grid over the nodes (bilinear P, up to 20 x 20 cells); 4 block-Jacobi flexible CG (the plain
 * method); 5 flexible CG with block-Jacobi plus the learned coarse correction,
 * falling back to 4 and then BiCGStab when it stalls.  collect = 1 (method 4)
 * stores one training pair per iteration of the solve.  info: iterations,
 * true FP64 residual, device time of the solve. */
pdx_status pdx_newmark_init(pdx_model* m);
pdx_status pdx_newmark_step(pdx_model* m, int method, int collect, pdx_solve_info* info);

/* Learned two-level preconditioner (no counterpart in the reference, which
 * solves directly).  A regular coarse grid of cx x cy (x cz) cells over the
 * model's bounding box, trilinear prolongation P and restriction P^T, and a
 * 3-layer MLP (hidden width `hidden`, Xavier-uniform weights from `seed`)
 * that maps the normalised restricted residual to the coarse error; trained
 * with BF16 operands and FP32 accumulation on the pairs that
 * pdx_newmark_step(m, 4, 1, ...) collects (at most max_samples). */
pdx_status pdx_learned_setup(pdx_model* m, int cx, int cy, int cz, int hidden, uint64_t seed, int max_samples);
int64_t pdx_learned_samples(const pdx_model* m);
/* More training pairs from the solver: nprobe block-Jacobi flexible CG solves
 * of the last Newmark matrix K_N with right-hand sides uniform in [-1, 1)
 * drawn from `seed`; every iterate of a converged solve gives a pair.  The
 * Newmark right-hand sides of successive steps are alike, and probes widen
 * the set of residuals the network sees.  Needs one pdx_newmark_step first. */
pdx_status pdx_learned_probe(pdx_model* m, int nprobe, uint64_t seed);
/* Learned-solve settings (after pdx_learned_setup): trunc = directions kept
 * for A-orthogonalisation (1..32, default 1; the learned correction is not
 * linear, and more directions keep the search directions A-orthogonal when
 * it varies more from one residual to the next), stall_window =
 * iterations after which the learned correction is given up if the residual
 * has not fallen 10x (default 60; 0 = never). */
pdx_status pdx_learned_options(pdx_model* m, int trunc, int stall_window);
/* 1 while method 5 uses the learned correction: the network is trained and
 * has not been switched off.  Plain block-Jacobi flexible CG (method 4) is
 * the arbiter: a learned solve is cut at the mean iteration count of the plain
 * Newmark solves (plain FCG finishes it), and after two learned solves in a
 * row slower than the mean plain solve (by time where plain solves that
 * collected nothing were timed, else by iterations) method 5 runs the plain
 * method until pdx_learned_train is called again. */
int pdx_learned_active(const pdx_model* m);
/* Copy the collected pairs out: r (count x nc) = P^T r_j, e (count x nc) =
 * coarse averages of the errors x* - x_j.  With r = e = NULL only *count
 * and *nc are written. */
pdx_status pdx_learned_pairs(const pdx_model* m, float* r, float* e, int64_t* count, int* nc);
/* Adam over all collected pairs for `epochs` epochs (batches of 64, order
 * shuffled from `seed`); final_loss = mean relative squared error of the
 * last epoch. */
pdx_status pdx_learned_train(pdx_model* m, int epochs, float lr, uint64_t seed, float* final_loss);
/* Network parameters (FP32: W1 b1 W2 b2 W3 b3, row-major): count, read (get)
 * and/or replace (set); NULL skips. */
pdx_status pdx_mlp_params(pdx_model* m, float* get, const float* set, int64_t* count);
/* Loss sum_b w_b |N(x_b) - t_b|^2 and its gradient with respect to the
 * parameters for a batch (<= 64) of inputs x (batch x n_coarse, rounded to
 * BF16 as in training) and targets t; for gradient checks. */
pdx_status pdx_mlp_loss_grad(pdx_model* m, int batch, const float* x, const float* t, const float* w, float* loss,
                             float* grad);

/* Batched explicit runs (no counterpart in the reference, which runs one
 * model per process): n independent specimens, one command file each, merged
 * into one model whose explicit step is a single launch over every
 * specimen's families and nodes.  The result is a pdx_model: pdx_explicit_*,
 * pdx_get_state (concatenated nodes and family members) and
 * pdx_model_get_info work on it; pdx_run does not.  Specimens must share the
 * dimension, precision, failure criterion and per-bond draw (seed,
 * perturbation), and be explicit dynamic runs without traction BCs;
 * materials, time steps, critical stretch, sizes and BCs may differ.  Each
 * specimen's set-up is built exactly as for a single model, so its fields
 * and broken bonds equal a single-model run's. */
pdx_status pdx_batch_create(const char* const* cmd_paths, int n, const pdx_options* opts, pdx_model** out);
/* Number of specimens of a batched model (0 for a single model). */
int pdx_batch_size(const pdx_model* m);
/* Where specimen i starts in the batch's arrays (n+1 entries each, NULL
 * skips): nodes (u_all rows, sigma, phi), family members (bond_state of
 * pdx_get_state), equations. */
pdx_status pdx_batch_offsets(const pdx_model* m, int64_t* node_off, int64_t* member_off, int64_t* eq_off);

/* Runs the solver the command file selects (pdsolve::pdfemSolver,
 * pdsolve.cpp:5073-5103) and writes the reference's outputs under
 * results_dir: <title>_<step>.vtk, <title>RF.out (static: _static/_PD/_FEM),
 * and for quasi-static runs <title>_cp.out (the FC 1 crack path). */
pdx_status pdx_run(pdx_model* m, const char* results_dir);

/* Quasi-static increments one at a time, the loop body of
 * pdfemQuasiStaticSolver_CSRformat (pdsolve.cpp:6464-6590) with the direct
 * PARDISO solve replaced by a Krylov method: pdx_quasi_init resets the state
 * (initial DOF values, pre-crack bond states, and with FC 1 the pre-cracks
 * and the PD region as read); each pdx_quasi_step assembles
 * K and f_ext - K u through the scatter map, solves K du = f_ext - K u to the
 * command file's tolerance with `method` (as pdx_solve_opts, or 8 in 2D: the
 * two-level BiCGStab of pdx_newmark_step; BiCGStab and then GMRES(30) take
 * over if it does not converge), updates u, applies FC 3 or FC 2 bond
 * failure or the FC 1 crack pass (SIFs, tip growth, PD-region growth and
 * bond cuts behind a moved tip, pdx_crack_state), recomputes the stresses,
 * records the reaction forces and advances
 * the prescribed DOFs by the reference's quasi-static rule
 * (setVaryEssentialBC, pdsolve.cpp:5263-5311): a varying EBC whose value is
 * 0 takes dt * velocity; after that, with FC 0 / FC 3 (load ratio 1) it
 * holds, so increment 1 solves the unloaded state and increment 2 the loaded
 * one; with FC 2 the load steps by the ratio 1.001 sigma_ult / max sigma1
 * (capped by the velocity) after an increment that cut no bond and holds
 * after one that did; with FC 1 it steps by 1.001 K_Ic / Keq (last crack)
 * when no tip moved and holds when one did.  info->seconds is the device time
 * of the solve. */
pdx_status pdx_quasi_init(pdx_model* m);
pdx_status pdx_quasi_step(pdx_model* m, int method, pdx_solve_info* info);

#ifdef __cplusplus
}
#endif

#endif /* PDX_H */
