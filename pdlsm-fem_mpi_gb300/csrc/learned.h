// Learned two-level preconditioner: device structures (k_learned.cu) and the
// host side (learned.cpp).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "model_impl.h"

namespace pdx {

// Regular coarse grid over the model's bounding box and the transfer
// operators between fine equations and coarse DOFs (device arrays).
struct CoarseSpace {
  int dim = 3;
  int cells[3] = {1, 1, 1};
  int nc = 0;                 // coarse DOFs = coarse nodes * dim
  int64_t n = 0;              // fine equations
  int np = 8;                 // prolongation entries per fine equation (8 in 3D, 4 in 2D)
  int* pidx = nullptr;        // n * np coarse DOF or -1
  float* pw = nullptr;        // n * np trilinear weights
  int* rptr = nullptr;        // nc + 1: rows of P^T (restriction)
  int* ridx = nullptr;        // fine equation
  float* rw = nullptr;        // P^T weights
  float* aw = nullptr;        // P^T weights divided by the row sums (coarse average)
};

constexpr int kInferMaxIn = 8192;
constexpr int kInferMaxH = 1024;

// 3-layer MLP nin -> H -> H -> nout with tanh hidden layers.  Parameters in
// one FP32 block (W1, b1, W2, b2, W3, b3, row-major) with a BF16 copy for the
// GEMMs, Adam moments, and the activations of one batch (<= Bmax rows).
struct Mlp {
  int nin = 0, nout = 0, H = 0, Bmax = 0;
  int step = 0;
  float* w = nullptr;
  __nv_bfloat16* w16 = nullptr;
  float* g = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *Y = nullptr, *dY = nullptr, *dH = nullptr, *dZ = nullptr;
  __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *dY16 = nullptr, *dZ16 = nullptr;
  float* loss_row = nullptr;
  float* loss = nullptr;
  float* work = nullptr;             // split-K partial products of the GEMMs (gemm_work_floats)
  int64_t n_params() const { return (int64_t)H * nin + H + (int64_t)H * H + H + (int64_t)nout * H + nout; }
  void param_views(float* base, float** W1, float** b1, float** W2, float** b2, float** W3, float** b3) const;
  // forward on X (B x nin, BF16); with T (B x nout) also the loss
  // sum_m wrow[m] |Y_m - T_m|^2 into *loss; with grads the gradient into g
  cudaError_t forward_backward(int B, const __nv_bfloat16* X, const float* T, const float* wrow, bool grads,
                               cudaStream_t s);
  cudaError_t adam_step(float lr, cudaStream_t s);
  cudaError_t sync_bf16(cudaStream_t s);
  // one input x16 (nin, BF16) -> y (nout, FP32); uses rows 0 of H1 and H2
  cudaError_t infer(const __nv_bfloat16* x16, float* y, cudaStream_t s);
  // Inference copy of the BF16 weights, rows padded to 16 bytes, for the
  // one-block inference kernel (inputs up to kInferMaxIn, width up to kInferMaxH)
  __nv_bfloat16* wi = nullptr;
  int64_t n_infer() const;
  bool block_infer_ok() const;
  cudaError_t pack_infer(cudaStream_t s);
  // x (nin, FP32, not normalised) -> y; *scale = |x| sigma; one block
  cudaError_t infer_block(const float* x, float sigma, float* y, float* scale, cudaStream_t s);
};

// Floats of split-K work space the GEMMs of Mlp::forward_backward need for
// batches of up to B rows.
int64_t gemm_work_floats(int B, int nin, int H, int nout);

cudaError_t coarse_restrict(const CoarseSpace& cs, bool average, const double* r, float* out, cudaStream_t s);
cudaError_t coarse_prolong_add(const CoarseSpace& cs, const float* c, const float* scale, double* z,
                               cudaStream_t s);
cudaError_t coarse_normalize(int n, const float* x, __nv_bfloat16* x16, float sigma, float* scale, cudaStream_t s);
cudaError_t learned_err(int first, int last, int nc, const float* ax, float* S, cudaStream_t s);
cudaError_t learned_norms(int count, int nc, const float* S, float* norms, cudaStream_t s);
cudaError_t learned_stage(int B, int nc, const int* idx, const float* S_r, const float* S_e, const float* norms,
                          float sigma, __nv_bfloat16* X, float* T, float* W, cudaStream_t s);
cudaError_t learned_stage_raw(int B, int nc, const float* Xf, __nv_bfloat16* X, cudaStream_t s);
// *acc += *x on the device (one thread; stream ordered)
cudaError_t learned_add_scalar(const float* x, float* acc, cudaStream_t s);
cudaError_t learned_random_rhs(int64_t n, uint64_t seed, double* b, cudaStream_t s);

// Everything the learned preconditioner of one model owns.
struct Learned : CoarseCorrection {
  CoarseSpace cs;
  Mlp net;
  DevBuf buf;
  float sigma = 1.f;          // target scale: the network predicts errors / (|R r| sigma)
  int trunc = 1;              // directions kept for A-orthogonalisation in the learned solve
  int stall_window = 60;      // the learned correction is dropped if the residual has not
                              // fallen 10x within this many iterations
  // plain block-Jacobi FCG as the arbiter: mean iterations and seconds of the
  // method-4 Newmark solves, learned solves in a row that lost to them, and
  // whether the learned correction is switched off (until it is retrained)
  double plain_its = 0.0, plain_sec = 0.0;   // plain_sec: only solves that collected nothing
  int plain_n = 0, plain_sec_n = 0;
  int losses = 0;
  bool disabled = false;
  bool trained = false;
  // inference scratch
  float* rc = nullptr;        // nc
  __nv_bfloat16* x16 = nullptr;
  float* y = nullptr;
  float* scale = nullptr;
  // training samples
  int cap = 0, count = 0, solve_first = 0;
  float* S_r = nullptr;       // cap * nc: restricted residuals P^T r_j
  float* S_x = nullptr;       // cap * nc: coarse averages of the iterates, then of the errors x* - x_j
  float* S_scale = nullptr;   // cap: |P^T r_j|
  float* ax = nullptr;        // nc: coarse average of a converged solution
  // batch staging
  int* bidx = nullptr;
  __nv_bfloat16* Xb = nullptr;
  float* Tb = nullptr;
  float* Wb = nullptr;
  cudaError_t add(const double* r, double* z, cudaStream_t s) override;
};

}  // namespace pdx
