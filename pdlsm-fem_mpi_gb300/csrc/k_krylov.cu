// Krylov solves of K x = b on the GPU, standing beside the reference's
// direct solve (cluster_PARDISO_64Solver, calMatrixOperations.cpp:378-498,
// real unsymmetric, one right-hand side).
//
//   method 0  PCG, Jacobi preconditioner
//   method 1  PCG, block-Jacobi (the d x d diagonal block of every node)
//   method 2  BiCGStab, Jacobi (K is unsymmetric: family k's row uses A_k and
//             delta_k while row m uses A_m and delta_m)
//   method 3  block-Jacobi PCG in FP32 (FP32 matrix copy and vectors) inside
//             FP64 iterative refinement: r = b - A x in FP64, A d ~= r in FP32,
//             x += d
//   method 6  GMRES(30), right Jacobi (the fallback once BiCGStab diverges)
//   method 7  BiCGStab in FP32 inside the same FP64 iterative refinement (the
//             mixed-precision solve for the unsymmetric stiffness, on which
//             CG stalls)
//   method 8  BiCGStab, right preconditioned by Jacobi plus the Galerkin
//             coarse correction on a lattice coarse grid (2D; TwoLevelDev)
//
// Convergence is always judged on the true FP64 residual ||b - A x|| / ||b||.
// Scalars stay on the device; iterations are launched in chunks and the host
// reads the residual once per chunk.  Reductions are two-pass (per-block
// partials then one block) so results are bitwise reproducible.
//
// GB300 runs FP64 arithmetic (and float<->double conversion) at 2 lanes per
// clock per SM against about 128 for FP32: the FP64 mat-vec at 30 nonzeros
// per row is bound by that rate (FP64 pipe 77 % busy, DRAM 48 %), and a
// division in every thread costs microseconds per kernel.  Every scalar ratio
// (alpha, beta, omega) is therefore formed once, by the last block of the
// reduction that produces it; the FP32 inner solves of methods 3 and 7 do
// their element arithmetic in FP32 and widen only their block partials to
// FP64.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

#include "device.h"

namespace pdx {

namespace {

constexpr int kRedBlocks = 1024;
constexpr int kCgStallIts = 400;
constexpr double kInnerTol = 1e-4;   // relative residual of the FP32 inner solves (methods 3, 7)
constexpr int kThreads = 256;

template <typename T, int L>
__global__ void __launch_bounds__(256) k_spmv(int64_t n, const int64_t* __restrict__ ia, const int* __restrict__ ja,
                                              const T* __restrict__ a, const T* __restrict__ x, T* __restrict__ y) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = gt / L;
  const int lane = (int)(gt % L);
  T s = 0;
  if (row < n) {
    const int64_t p0 = ia[row], p1 = ia[row + 1];
    for (int64_t p = p0 + lane; p < p1; p += L) s += a[p] * x[ja[p]];
  }
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (row < n && lane == 0) y[row] = s;
}

// Sum over the block, returned to every thread: warp shuffles (xor tree),
// then thread 0 adds the warp sums in warp order.  Two barriers instead of
// the eight of a shared-memory tree; the extra FP64 adds of the shuffle
// levels cost less than the barriers (a dot product with its final step:
// 5.0 against 5.7 us on the GB300).  sh: at least 33 words.
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

template <typename T>
__global__ void k_dot_partial(int64_t n, const T* x, const T* y, double* part) {
  __shared__ double sh[kThreads];
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)x[i] * (double)y[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_dot_final(const double* part, int np, double* out) {
  __shared__ double sh[kThreads];
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

// inverse of the diagonal blocks; blocks given by bptr (rows [bptr[i], bptr[i+1]))
__global__ void k_block_inverse(int64_t nb, const int64_t* bptr, const int64_t* ia, const int* ja, const double* a,
                                double* binv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int64_t r0 = bptr[i];
  const int s = (int)(bptr[i + 1] - r0);
  double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int r = 0; r < s; r++)
    for (int64_t p = ia[r0 + r]; p < ia[r0 + r + 1]; p++) {
      const int64_t c = ja[p] - r0;
      if (c >= 0 && c < s) M[r][c] = a[p];
    }
  double I[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int k = 0; k < s; k++) {
    int p = k;
    for (int r = k + 1; r < s; r++)
      if (fabs(M[r][k]) > fabs(M[p][k])) p = r;
    if (p != k)
      for (int c = 0; c < 3; c++) {
        double t = M[k][c]; M[k][c] = M[p][c]; M[p][c] = t;
        t = I[k][c]; I[k][c] = I[p][c]; I[p][c] = t;
      }
    const double d = M[k][k] != 0.0 ? M[k][k] : 1.0;
    for (int c = 0; c < 3; c++) { M[k][c] /= d; I[k][c] /= d; }
    for (int r = 0; r < s; r++) {
      if (r == k) continue;
      const double f = M[r][k];
      for (int c = 0; c < 3; c++) { M[r][c] -= f * M[k][c]; I[r][c] -= f * I[k][c]; }
    }
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) binv[i * 9 + r * 3 + c] = (r < s && c < s) ? I[r][c] : 0.0;
}

template <typename T>
__global__ void k_apply_block(int64_t nb, const int64_t* bptr, const double* binv, const T* r, T* z) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int64_t r0 = bptr[i];
  const int s = (int)(bptr[i + 1] - r0);
  double v[3] = {0, 0, 0};
  for (int c = 0; c < s; c++) v[c] = (double)r[r0 + c];
  for (int rr = 0; rr < s; rr++) {
    double acc = 0;
    for (int c = 0; c < s; c++) acc += binv[i * 9 + rr * 3 + c] * v[c];
    z[r0 + rr] = (T)acc;
  }
}

// p = z + beta p, beta = rz_new / rz_old set by the last block of the
// reduction that summed rz_new
template <typename T>
__global__ void k_cg_dir(int64_t n, const T* beta, const T* z, T* p) {
  const T b = *beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

template <typename T>
__global__ void k_jacobi(int64_t n, const T* dinv, const T* r, T* z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];
}

__global__ void k_diag_inv(int64_t n, const int64_t* ia, const int* ja, const double* a, double* dinv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = 0;
  for (int64_t p = ia[i]; p < ia[i + 1]; p++)
    if (ja[p] == i) d = a[p];
  dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
}

__global__ void k_residual(int64_t n, const double* b, const double* ax, double* r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - ax[i];
}

template <typename S, typename T>
__global__ void k_convert(int64_t n, const S* a, T* b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (T)a[i];
}

template <typename T>
__global__ void k_sub(int64_t n, const T* b, const T* q, T* r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - q[i];
}

// x += sign d
__global__ void k_add_to(int64_t n, const float* d, double sign, double* x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] += sign * (double)d[i];
}

// Fused BiCGStab steps.  The dot products keep the fixed order of
// k_dot_partial / k_dot_final (grid-stride partial sums over red_grid
// blocks, block_sum, one final block), so the fused solve gives the same
// bits as separate kernels; scalars stay on the device.


// The reductions with their final step folded in: every block writes its
// partial, and the block that finishes last (thread 0 fences its partial,
// then takes an atomic ticket) adds the partials in block order exactly as
// k_dot_final does, so the bits do not change and a single-block launch per
// reduction disappears.  The ticket is reset by that last block for the next
// use.
__device__ __forceinline__ bool last_block(unsigned* ticket) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return last;
}

__device__ __forceinline__ double sum_partials(const double* part, int np, double* sh) {
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += __ldcg(part + i);
  return block_sum(s, sh);
}

// Reductions in the precision T of the vectors.  FP64: the block tree of
// block_sum.  FP32: the products are summed in FP32 within a thread and a
// block (warp shuffles), and only the block partials are widened to FP64 for
// the final sum, so no FP64 arithmetic runs per element.
__device__ __forceinline__ double block_total(double v, double* sh) { return block_sum(v, sh); }
__device__ __forceinline__ float block_total(float v, double* shd) {
  float* sh = reinterpret_cast<float*>(shd);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
  __syncthreads();
  return t;   // valid in thread 0
}

// the block's partial, stored in T (part viewed as T*)
template <typename T>
__device__ __forceinline__ void put_partial(double* part, T v) {
  if (threadIdx.x == 0) reinterpret_cast<T*>(part)[blockIdx.x] = v;
}

template <typename T>
__device__ __forceinline__ double sum_partials_t(const double* part, int np, double* sh) {
  const T* pt = reinterpret_cast<const T*>(part);
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += (double)__ldcg(pt + i);
  return block_sum(s, sh);
}

// BiCGStab scalars: FP64 masters (rho, alpha, omega, beta) formed by the
// last blocks, and their copies in T that the element loops read (the same
// words when T is double).
template <typename T>
struct BicgScalars {
  double* alpha;
  double* omega;
  double* beta;
  T* alpha_t;
  T* omega_t;
  T* beta_t;
};

// starting scalars: alpha = omega = rho_prev = 1
__global__ void k_bicg_start(double* alpha, double* omega, double* rho_prev) {
  *alpha = 1.0;
  *omega = 1.0;
  *rho_prev = 1.0;
}

// beta of the first iteration, (rho / rho_prev)(alpha / omega) with the
// starting values; later ones are set by k_bicg_x_rho
template <typename T>
__global__ void k_bicg_beta0(const double* rho, const double* rho_prev, BicgScalars<T> c) {
  const double b = (*rho / *rho_prev) * (*c.alpha / *c.omega);
  *c.beta = b;
  *c.beta_t = (T)b;
  *c.alpha_t = (T)*c.alpha;
  *c.omega_t = (T)*c.omega;
}

// p = r + beta (p - omega v); ph = D^-1 p
template <typename T>
__global__ void k_bicg_p2(int64_t n, const T* beta_p, const T* omega_p, const T* r, const T* v, const T* dinv, T* p,
                          T* ph) {
  const T beta = *beta_p, omega = *omega_p;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T pi = r[i] + beta * (p[i] - omega * v[i]);
    p[i] = pi;
    ph[i] = dinv[i] * pi;
  }
}

// s = r - alpha v; sh = D^-1 s
template <typename T>
__global__ void k_bicg_s2(int64_t n, const T* alpha_p, const T* r, const T* v, const T* dinv, T* s, T* sh) {
  const T alpha = *alpha_p;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T si = r[i] - alpha * v[i];
    s[i] = si;
    sh[i] = dinv[i] * si;
  }
}

// partials of r0 . v; the last block sets alpha = rho / (r0 . v) (0 if the dot is 0)
template <typename T>
__global__ void k_bicg_alpha(int64_t n, const T* r0, const T* v, double* part, unsigned* ticket, const double* rho,
                             BicgScalars<T> c) {
  __shared__ double sh[kThreads];
  T acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += r0[i] * v[i];
  put_partial<T>(part, block_total(acc, sh));
  if (!last_block(ticket)) return;
  const double d = sum_partials_t<T>(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    const double a = d != 0.0 ? *rho / d : 0.0;
    *c.alpha = a;
    *c.alpha_t = (T)a;
    *ticket = 0;
  }
}

// partials of t.s and t.t; the last block sets omega = (t.s) / (t.t) (0 if t.t is 0)
template <typename T>
__global__ void k_bicg_omega(int64_t n, const T* t, const T* s, double* part_ts, double* part_tt, unsigned* ticket,
                             BicgScalars<T> c) {
  __shared__ double sh[kThreads];
  T a = 0, b = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    a += t[i] * s[i];
    b += t[i] * t[i];
  }
  put_partial<T>(part_ts, block_total(a, sh));
  put_partial<T>(part_tt, block_total(b, sh));
  if (!last_block(ticket)) return;
  const double sa = sum_partials_t<T>(part_ts, gridDim.x, sh);
  const double sb = sum_partials_t<T>(part_tt, gridDim.x, sh);
  if (threadIdx.x == 0) {
    const double o = sb != 0.0 ? sa / sb : 0.0;
    *c.omega = o;
    *c.omega_t = (T)o;
    *ticket = 0;
  }
}

// x += alpha ph + omega sh; r = s - omega t; the last block sets rho_next =
// r0 . r and the next iteration's beta = (rho_next / rho)(alpha / omega)
template <typename T>
__global__ void k_bicg_x_rho(int64_t n, const T* ph, const T* shat, const T* s, const T* t, const T* r0, T* x, T* r,
                             double* part, unsigned* ticket, const double* rho, double* rho_next, BicgScalars<T> c) {
  __shared__ double sh[kThreads];
  const T alpha = *c.alpha_t, omega = *c.omega_t;
  T acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * ph[i] + omega * shat[i];
    const T ri = s[i] - omega * t[i];
    r[i] = ri;
    acc += r0[i] * ri;
  }
  put_partial<T>(part, block_total(acc, sh));
  if (!last_block(ticket)) return;
  const double d = sum_partials_t<T>(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *rho_next = d;
    const double b = (d / *rho) * (*c.alpha / *c.omega);
    *c.beta = b;
    *c.beta_t = (T)b;
    *ticket = 0;
  }
}

// Two-level preconditioner of method 8 (2D): z = D^-1 v + P (P^T A P)^-1 P^T v
// with P bilinear per DOF component on a lattice coarse grid (TwoLevelDev).
// The coarse matrix is formed in two fixed-order passes, so its bits do not
// depend on scheduling: B = A P on each fine row's window of 4x4 coarse nodes
// and 2 components (every coupling of a row reaches at most one cell over,
// which the model checks when it picks the grid), then P^T B on each coarse
// row's window of 5x5 nodes.

// B[i][s]: one warp per fine row, lane = window slot (x offset -1..2, y
// offset -1..2, component), the row's entries in CSR order
__global__ void k_tl_ap(int64_t n, const int64_t* ia, const int* ja, const double* a, TwoLevelDev t) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int s = threadIdx.x & 31;
  if (row >= n) return;
  const int q0 = t.ecell[row];   // the row's cell (x, y) and component
  const int sx = (q0 & 0xfff) + (s & 3) - 1, sy = ((q0 >> 12) & 0xfff) + ((s >> 2) & 3) - 1, sc = s >> 4;
  double acc = 0;
#pragma unroll 4
  for (int64_t p = ia[row]; p < ia[row + 1]; p++) {
    const int j = ja[p];
    const int q = t.ecell[j];
    const int ex = sx - (q & 0xfff), ey = sy - ((q >> 12) & 0xfff);
    if ((q >> 24) == sc && (unsigned)ex <= 1u && (unsigned)ey <= 1u)
      acc += a[p] * (double)t.pw[(int64_t)j * 4 + ex + 2 * ey];
  }
  t.B[row * 32 + s] = acc;
}

// [0 | I]: the augmented matrix before the coarse rows are written
__global__ void k_tl_init(TwoLevelDev t) {
  const int64_t w = 2 * (int64_t)t.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < (int64_t)t.nc * w;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = k / w, c = k % w;
    t.M[k] = c == t.nc + r ? 1.0 : 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *t.ok = 1;
}

// row I of P^T A P: one block of 64 threads per coarse DOF, thread = slot of
// the 5x5-node, 2-component window, P^T's row in order.  A coarse DOF with no
// free fine equation in its support (a hole, prescribed DOFs only) gets a
// unit diagonal: its restricted residual is always zero, so it stays zero.
__global__ void k_tl_coarse(TwoLevelDev t) {
  const int I = blockIdx.x;
  const int s = threadIdx.x;
  if (s >= 50) return;
  const int nI = I >> 1;
  const int JX = nI % t.nxn + s % 5 - 2, JY = nI / t.nxn + (s / 5) % 5 - 2, jc = s / 25;
  if (JX < 0 || JX >= t.nxn || JY < 0 || JY >= t.nyn) return;
  if (t.rptr[I] == t.rptr[I + 1]) {
    if (s == 12 + 25 * (I & 1)) t.M[(int64_t)I * 2 * t.nc + I] = 1.0;   // the diagonal slot
    return;
  }
  double acc = 0;
  for (int k = t.rptr[I]; k < t.rptr[I + 1]; k++) {
    const int i = t.ridx[k];
    const int q = t.ecell[i];
    const int dx = JX - (q & 0xfff) + 1, dy = JY - ((q >> 12) & 0xfff) + 1;
    if ((unsigned)dx <= 3u && (unsigned)dy <= 3u)
      acc += (double)t.rw[k] * t.B[(int64_t)i * 32 + jc * 16 + dy * 4 + dx];
  }
  t.M[(int64_t)I * 2 * t.nc + (JX + t.nxn * JY) * 2 + jc] = acc;
}

// Gauss-Jordan elimination of [A_c | I] without pivoting, one launch per
// column: A_c = P^T A P is symmetric positive definite up to the small
// unsymmetric part of the PD stiffness, for which elimination in the natural
// order is stable; a pivot below 1e-10 of its original diagonal clears *ok
// and the solve runs with Jacobi alone.  Rows are scaled once at the end
// (the left half ends diagonal), so within a step no thread writes what
// another reads: step k reads column k (colbuf[k & 1], contiguous) and the
// reciprocal of its pivot (rpiv[k & 1], one division by one thread of the
// previous step), and writes column k + 1 and its pivot's reciprocal into
// the other slots.

// column 0, the original diagonal and the first pivot's reciprocal
__global__ void k_gj_first(const double* M, int nc, double* colbuf, double* diag0, double* rpiv, int* ok) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nc) return;
  const int64_t w = 2 * (int64_t)nc;
  colbuf[r] = M[r * w];
  diag0[r] = M[r * w + r];
  if (r == 0) {
    const double pv = M[0];
    if (fabs(pv) > 0.0) rpiv[0] = 1.0 / pv;
    else *ok = 0;
  }
}

// M[r][c] -= (M[r][k] / M[k][k]) M[k][c] for r != k and k < c <= k + nc:
// row k is zero right of column nc + k (the part of I no step has reached
// yet), so nothing else changes; column k itself is left as it is and never
// read again
__global__ void k_gj_step(double* M, int nc, int k, const double* colbuf, double* colbuf_next, const double* rpiv,
                          double* rpiv_next, const double* diag0, int* ok) {
  if (*ok == 0) return;
  const int64_t w = 2 * (int64_t)nc;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nc * nc) return;
  const int64_t r = t / nc, c = k + 1 + t % nc;
  double v = M[r * w + c];
  if (r != k) {
    const double pk = M[(int64_t)k * w + c];
    if (pk != 0.0) {
      const double f = colbuf[r] * rpiv[0];
      if (f != 0.0) {
        v -= f * pk;
        M[r * w + c] = v;
      }
    }
  }
  if (c == k + 1) {
    colbuf_next[r] = v;
    if (r == k + 1) {
      if (fabs(v) > 1e-10 * fabs(diag0[r])) rpiv_next[0] = 1.0 / v;
      else *ok = 0;
    }
  }
}

// reciprocals of the final diagonal
__global__ void k_gj_rdiag(const double* M, int nc, double* rd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nc) rd[r] = 1.0 / M[(int64_t)r * 2 * nc + r];
}

// the right half scaled by the rows' reciprocals: the inverse
__global__ void k_gj_finish(double* M, int nc, const double* rd, const int* ok) {
  if (*ok == 0) return;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nc * nc) return;
  const int64_t r = t / nc, c = t % nc;
  M[r * 2 * nc + nc + c] *= rd[r];
}

// rc = P^T v: one block per coarse DOF, P^T's row in order
__global__ void k_tl_restrict(TwoLevelDev t, const double* v) {
  __shared__ double sh[kThreads];
  const int I = blockIdx.x;
  double acc = 0;
  for (int k = t.rptr[I] + threadIdx.x; k < t.rptr[I + 1]; k += blockDim.x) acc += (double)t.rw[k] * v[t.ridx[k]];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) t.rc[I] = acc;
}

// yc = (P^T A P)^-1 rc: one block of 128 threads per coarse row of the
// inverse (four warps keep enough loads in flight for a 7 KB row)
__global__ void __launch_bounds__(128) k_tl_coarse_mv(TwoLevelDev t) {
  __shared__ double sh[4];
  const int row = blockIdx.x;
  const double* Mi = t.M + (int64_t)row * 2 * t.nc + t.nc;
  double acc = 0;
  for (int c = threadIdx.x; c < t.nc; c += blockDim.x) acc += Mi[c] * t.rc[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) t.yc[row] = (sh[0] + sh[1]) + (sh[2] + sh[3]);
}

// z += P yc
__global__ void k_tl_prolong_add(TwoLevelDev t, double* z) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n) return;
  double acc = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float w = t.pw[i * 4 + k];
    if (w != 0.f) acc += (double)w * t.yc[t.pidx[i * 4 + k]];
  }
  z[i] += acc;
}

// A 64-bit fingerprint of the matrix values: the sum (mod 2^64) of a mixed
// (splitmix64) function of each value's bits and position, so the order of
// the atomic additions does not matter.
__global__ void k_values_hash(int64_t nnz, const double* a, unsigned long long* h) {
  unsigned long long acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long x = (unsigned long long)__double_as_longlong(a[i]) ^ ((unsigned long long)i * 0x9e3779b97f4a7c15ull);
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    acc += x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(h, acc);
}

void twolevel_apply(const TwoLevelDev& t, const double* v, double* z, cudaStream_t s) {
  k_tl_restrict<<<t.nc, kThreads, 0, s>>>(t, v);
  k_tl_coarse_mv<<<t.nc, 128, 0, s>>>(t);
  k_tl_prolong_add<<<(int)((t.n + 255) / 256), 256, 0, s>>>(t, z);
}

// Fused PCG steps in the precision T of the vectors (reductions as above).
// partials of p.q; the last block sets alpha = rz / (p.q) (0 if p.q is 0)
template <typename T>
__global__ void k_cg_pq(int64_t n, const T* p, const T* q, double* part, unsigned* ticket, const double* rz,
                        T* alpha) {
  __shared__ double sh[kThreads];
  T acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += p[i] * q[i];
  put_partial<T>(part, block_total(acc, sh));
  if (!last_block(ticket)) return;
  const double d = sum_partials_t<T>(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *alpha = (T)(d != 0.0 ? *rz / d : 0.0);
    *ticket = 0;
  }
}

// x += alpha p; r -= alpha q; with dinv also z = D^-1 r and the partials of
// r.z, the last block storing rz_new and beta = rz_new / rz (0 if rz is 0)
template <typename T>
__global__ void k_cg_update_jacobi(int64_t n, const T* alpha_p, const T* p, const T* q, T* x, T* r, const T* dinv,
                                   T* z, double* part, unsigned* ticket, const double* rz, double* rz_new, T* beta) {
  __shared__ double sh[kThreads];
  const T alpha = *alpha_p;
  T acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = x[i] + alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    r[i] = ri;
    if (dinv) {
      const T zi = dinv[i] * ri;
      z[i] = zi;
      acc += ri * zi;
    }
  }
  if (!dinv) return;
  put_partial<T>(part, block_total(acc, sh));
  if (!last_block(ticket)) return;
  const double d = sum_partials_t<T>(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *rz_new = d;
    *beta = (T)(*rz != 0.0 ? d / *rz : 0.0);
    *ticket = 0;
  }
}

// block-Jacobi z = B^-1 r over the node blocks and the partials of r.z; the
// last block stores rz_new and beta = rz_new / rz (0 if rz is 0)
template <typename T>
__global__ void k_cg_block_rz(int64_t nb, const int64_t* bptr, const double* binv, const T* r, T* z, double* part,
                              unsigned* ticket, const double* rz, double* rz_new, T* beta) {
  __shared__ double sh[kThreads];
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = bptr[i];
    const int s = (int)(bptr[i + 1] - r0);
    double v[3] = {0, 0, 0};
    for (int c = 0; c < s; c++) v[c] = (double)r[r0 + c];
    for (int rr = 0; rr < s; rr++) {
      double zi = 0;
      for (int c = 0; c < s; c++) zi += binv[i * 9 + rr * 3 + c] * v[c];
      z[r0 + rr] = (T)zi;
      acc += v[rr] * (double)(T)zi;
    }
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
  if (!last_block(ticket)) return;
  const double d = sum_partials(part, gridDim.x, sh);
  if (threadIdx.x == 0) {
    *rz_new = d;
    *beta = (T)(*rz != 0.0 ? d / *rz : 0.0);
    *ticket = 0;
  }
}

// Restarted GMRES: Arnoldi basis V (rows of length ld), classical
// Gram-Schmidt applied twice, Givens rotations of the small Hessenberg column
// on the host.  Partial sums keep a fixed order (grid-stride, block tree,
// one final block per basis vector) as the other reductions here.
constexpr int kGmresRestart = 30;
constexpr int kMdotChunk = 8;

// per-block partials of v_k . w for k in [k0, k0 + nk), nk <= kMdotChunk;
// part[k * np + block]
__global__ void k_mdot_partial(int64_t n, const double* V, int64_t ld, int k0, int nk, const double* w, double* part,
                               int np) {
  __shared__ double sh[kThreads];
  double acc[kMdotChunk];
#pragma unroll
  for (int k = 0; k < kMdotChunk; k++) acc[k] = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double wi = w[i];
#pragma unroll
    for (int k = 0; k < kMdotChunk; k++)
      if (k < nk) acc[k] += V[(int64_t)(k0 + k) * ld + i] * wi;
  }
#pragma unroll
  for (int k = 0; k < kMdotChunk; k++) {
    if (k < nk) {
      const double t = block_sum(acc[k], sh);
      if (threadIdx.x == 0) part[(int64_t)(k0 + k) * np + blockIdx.x] = t;
    }
  }
}

// out[k] = sum of part[k * np ...] (one block per k); acc[k] += out[k] if acc
__global__ void k_mdot_final(const double* part, int np, double* out, double* acc) {
  __shared__ double sh[kThreads];
  const int k = blockIdx.x;
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[(int64_t)k * np + i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    out[k] = s;
    if (acc) acc[k] += s;
  }
}

// w -= sum_{k < nk} h[k] v_k
__global__ void k_msub(int64_t n, const double* V, int64_t ld, int nk, const double* h, double* w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int k = 0; k < nk; k++) s -= h[k] * V[(int64_t)k * ld + i];
    w[i] = s;
  }
}

// *hsub = ||w|| from its square; w /= ||w|| (left as is when the norm is 0)
__global__ void k_gmres_normalise(int64_t n, const double* nn, double* hsub, double* w) {
  const double nv = sqrt(*nn);
  if (blockIdx.x == 0 && threadIdx.x == 0) *hsub = nv;
  if (!(nv > 0.0)) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = w[i] / nv;
}

// x += D^-1 sum_{k < nk} y[k] v_k
__global__ void k_gmres_x(int64_t n, const double* V, int64_t ld, int nk, const double* y, const double* dinv,
                          double* x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int k = 0; k < nk; k++) s += y[k] * V[(int64_t)k * ld + i];
    x[i] += dinv[i] * s;
  }
}

template <typename T>
struct Work {
  T* buf = nullptr;
  size_t n = 0;
};

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + kThreads - 1) / kThreads, kRedBlocks); }
// Blocks of the reductions (dot products, and the vector steps that end in
// one): two per SM, so the last block adds few partials.  On the 320k-row
// plate system a dot product with its final step folded in took 5.0 us with
// 304 blocks and 7.6 us with 1024; plain vector steps keep grid_for.
constexpr int kRedGrid = 304;
int red_grid(int64_t n) { return (int)std::min<int64_t>((n + kThreads - 1) / kThreads, kRedGrid); }

struct Ctx {
  cudaStream_t s;
  double* part;   // kRedBlocks
  template <typename T>
  void dot(int64_t n, const T* x, const T* y, double* out) {
    const int g = red_grid(n);
    k_dot_partial<T><<<g, kThreads, 0, s>>>(n, x, y, part);
    k_dot_final<<<1, kThreads, 0, s>>>(part, g, out);
  }
};

template <typename T>
void spmv_t(int64_t n, double avg, const int64_t* ia, const int* ja, const T* a, const T* x, T* y, cudaStream_t s) {
  // Lanes per row: on the 2.49M-equation Newmark matrix of the penny-crack
  // box (94 entries per row on average, 369 at most) 4 lanes ran at 5.4 TB/s,
  // 8 lanes 5.3, 32 lanes 2.3 (a warp per row leaves most lanes idle in the
  // last pass and makes eight times the blocks).
  if (avg > 256) {
    k_spmv<T, 8><<<(int)((n * 8 + 255) / 256), 256, 0, s>>>(n, ia, ja, a, x, y);
  } else if (avg > 12) {
    k_spmv<T, 4><<<(int)((n * 4 + 255) / 256), 256, 0, s>>>(n, ia, ja, a, x, y);
  } else {
    k_spmv<T, 2><<<(int)((n * 2 + 255) / 256), 256, 0, s>>>(n, ia, ja, a, x, y);
  }
}

// Preconditioned CG in precision T on (ia, ja, aT); solves for x given b, both in T.
// Returns iterations; stops when the recursive residual is below rtol*||b|| or max_iter.
template <typename T>
// ticket: a zeroed device word for the reductions' last-block step (the
// caller's; the allocation-free solve keeps it in its fixed work space);
// graphs: replay chunks of iterations as a CUDA graph (off where nothing
// may be allocated).
int pcg_core(Ctx& c, int64_t n, double avg, const int64_t* ia, const int* ja, const T* aT, const T* b, T* x,
             const T* dinv, int64_t nb, const int64_t* bptr, const double* binv, double rtol, int max_iter,
             double* dscal, T* r, T* z, T* p, T* q, unsigned* ticket, bool graphs) {
  cudaStream_t s = c.s;
  double* rz = dscal + 0;
  double* rz_new = dscal + 1;
  double* bb = dscal + 3;
  double* rr = dscal + 4;
  T* alpha = reinterpret_cast<T*>(dscal + 5);   // set by k_cg_pq
  T* beta = reinterpret_cast<T*>(dscal + 6);    // set with rz_new
  const int g = grid_for(n);
  spmv_t<T>(n, avg, ia, ja, aT, x, q, s);
  k_sub<T><<<g, kThreads, 0, s>>>(n, b, q, r);
  c.dot<T>(n, b, b, bb);
  auto precond = [&](const T* rin, T* zout) {
    if (binv) k_apply_block<T><<<(int)((nb + 255) / 256), 256, 0, s>>>(nb, bptr, binv, rin, zout);
    else k_jacobi<T><<<g, kThreads, 0, s>>>(n, dinv, rin, zout);
  };
  precond(r, z);
  c.dot<T>(n, r, z, rz);
  cudaMemcpyAsync(p, z, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  double hb = 0;
  cudaMemcpyAsync(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double bnorm = std::sqrt(hb);
  if (bnorm == 0.0) {
    cudaMemsetAsync(x, 0, n * sizeof(T), s);
    return 0;
  }
  int it = 0;
  const int chunk = 10;
  // CG is not made for the unsymmetric PD stiffness and can stall on it: the
  // solve stops once the residual has not halved for kCgStallIts iterations
  // (the caller then sees a true residual above rtol and may switch method)
  double best = INFINITY;
  int best_it = 0;
  // r.z of the iteration and of the one before in two slots (rz, rz_new by
  // parity, no copy); the reductions' final step, with the ratio alpha or
  // beta, runs in their last block; the preconditioner and r.z are fused
  // into the update (Jacobi) or into one block-Jacobi kernel: four launches
  // per iteration, five with block-Jacobi; chunks of ten iterations replay a
  // CUDA graph
  const int gb = binv ? red_grid(nb) : 0;
  const int gr = red_grid(n);
  auto iteration = [&](int k) {
    double* rz_cur = (k & 1) ? rz_new : rz;
    double* rz_next = (k & 1) ? rz : rz_new;
    spmv_t<T>(n, avg, ia, ja, aT, p, q, s);
    k_cg_pq<T><<<gr, kThreads, 0, s>>>(n, p, q, c.part, ticket, rz_cur, alpha);
    if (binv) {
      k_cg_update_jacobi<T><<<g, kThreads, 0, s>>>(n, alpha, p, q, x, r, nullptr, z, c.part, ticket, rz_cur,
                                                   rz_next, beta);
      k_cg_block_rz<T><<<gb, kThreads, 0, s>>>(nb, bptr, binv, r, z, c.part, ticket, rz_cur, rz_next, beta);
    } else {
      k_cg_update_jacobi<T><<<gr, kThreads, 0, s>>>(n, alpha, p, q, x, r, dinv, z, c.part, ticket, rz_cur,
                                                    rz_next, beta);
    }
    k_cg_dir<T><<<g, kThreads, 0, s>>>(n, beta, z, p);
  };
  cudaGraphExec_t gexec = nullptr;
  if (graphs) {
    cudaGraph_t graph;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (int k = 0; k < chunk; k++) iteration(k);   // chunks start at an even iteration
      if (cudaStreamEndCapture(s, &graph) == cudaSuccess) {
        if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaGetLastError();
  }
  while (it < max_iter) {
    if (gexec && max_iter - it >= chunk) {
      cudaGraphLaunch(gexec, s);
      it += chunk;
    } else {
      for (int k = 0; k < chunk && it < max_iter; k++, it++) iteration(it);
    }
    c.dot<T>(n, r, r, rr);
    double hr = 0;
    cudaMemcpyAsync(&hr, rr, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const double rn = std::sqrt(hr);
    if (!(rn > rtol * bnorm)) break;
    if (!(rn == rn)) break;
    if (rn < 0.5 * best) {
      best = rn;
      best_it = it;
    } else if (it - best_it >= kCgStallIts) {
      break;
    }
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  return it;
}

// BiCGStab with right Jacobi preconditioning in precision T on (ia, ja, aT),
// from the iterate x (in T).  Stops when the recursive residual is at most
// rtol ||b|| (read after each chunk of ten iterations), on a non-finite
// residual, at max_iter, or (stall > 0) once the residual has not halved for
// `stall` iterations.  Seven launches per iteration: two SpMVs and three
// fused vector steps, two of them with their reductions' final step folded
// in; a chunk of ten iterations is captured once as a CUDA graph and
// replayed.  w: eight work vectors of n (w[0] the residual r, w[3] the
// direction p); part2: 2 kRedBlocks words.  Returns iterations.
template <typename T>
int bicg_core(Ctx& c, int64_t n, double avg, const int64_t* ia, const int* ja, const T* aT, const T* b, T* x,
              const T* dinv, double rtol, int max_iter, int stall, double* dscal, T* const w[8], double* part2,
              unsigned* ticket, const TwoLevelDev* tl = nullptr) {
  cudaStream_t s = c.s;
  T *r = w[0], *r0 = w[1], *v = w[2], *p = w[3], *ss = w[4], *t = w[5], *ph = w[6], *sh = w[7];
  const int g = grid_for(n);
  const int gr = red_grid(n);
  BicgScalars<T> sc;
  sc.alpha = dscal + 2;
  sc.omega = dscal + 3;
  sc.beta = dscal + 14;
  if constexpr (std::is_same<T, double>::value) {
    sc.alpha_t = sc.alpha;
    sc.omega_t = sc.omega;
    sc.beta_t = sc.beta;
  } else {
    sc.alpha_t = reinterpret_cast<T*>(dscal + 4);
    sc.omega_t = sc.alpha_t + 1;
    sc.beta_t = reinterpret_cast<T*>(dscal + 5);
  }
  double* bb = dscal + 6;
  double* rr = dscal + 7;
  double* rhos = dscal + 12;   // rho of the iteration and of the one before, by parity
  spmv_t<T>(n, avg, ia, ja, aT, x, v, s);   // v holds A x for the moment
  k_sub<T><<<g, kThreads, 0, s>>>(n, b, v, r);
  cudaMemcpyAsync(r0, r, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(v, 0, n * sizeof(T), s);
  cudaMemsetAsync(p, 0, n * sizeof(T), s);
  k_bicg_start<<<1, 1, 0, s>>>(sc.alpha, sc.omega, rhos + 1);
  c.dot<T>(n, b, b, bb);
  c.dot<T>(n, r0, r, rhos);
  k_bicg_beta0<T><<<1, 1, 0, s>>>(rhos, rhos + 1, sc);
  double hb = 0;
  cudaMemcpyAsync(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double bnorm = std::sqrt(hb);
  auto iteration = [&](int it) {
    double* rho_cur = rhos + (it & 1);
    double* rho_next = rhos + ((it + 1) & 1);
    k_bicg_p2<T><<<g, kThreads, 0, s>>>(n, sc.beta_t, sc.omega_t, r, v, dinv, p, ph);
    if constexpr (std::is_same<T, double>::value) {
      if (tl) twolevel_apply(*tl, p, ph, s);   // ph += P (P^T A P)^-1 P^T p
    }
    spmv_t<T>(n, avg, ia, ja, aT, ph, v, s);
    k_bicg_alpha<T><<<gr, kThreads, 0, s>>>(n, r0, v, c.part, ticket, rho_cur, sc);
    k_bicg_s2<T><<<g, kThreads, 0, s>>>(n, sc.alpha_t, r, v, dinv, ss, sh);
    if constexpr (std::is_same<T, double>::value) {
      if (tl) twolevel_apply(*tl, ss, sh, s);
    }
    spmv_t<T>(n, avg, ia, ja, aT, sh, t, s);
    k_bicg_omega<T><<<gr, kThreads, 0, s>>>(n, t, ss, part2, part2 + kRedBlocks, ticket, sc);
    k_bicg_x_rho<T><<<gr, kThreads, 0, s>>>(n, ph, sh, ss, t, r0, x, r, c.part, ticket, rho_cur, rho_next, sc);
  };
  const int chunk = 10;
  cudaGraphExec_t gexec = nullptr;
  {
    cudaGraph_t graph;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      for (int k = 0; k < chunk; k++) iteration(k);   // chunks start at an even iteration
      if (cudaStreamEndCapture(s, &graph) == cudaSuccess) {
        if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaGetLastError();
  }
  int iters = 0;
  double best = INFINITY;
  int best_it = 0;
  while (bnorm > 0 && iters < max_iter) {
    if (gexec && max_iter - iters >= chunk) {
      cudaGraphLaunch(gexec, s);
      iters += chunk;
    } else {
      for (int k = 0; k < chunk && iters < max_iter; k++, iters++) iteration(iters);
    }
    c.dot<T>(n, r, r, rr);
    double hr = 0;
    cudaMemcpyAsync(&hr, rr, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const double rn = std::sqrt(hr);
    if (!(rn > rtol * bnorm) || !std::isfinite(hr)) break;
    if (rn < 0.5 * best) {
      best = rn;
      best_it = iters;
    } else if (stall > 0 && iters - best_it >= stall) {
      break;
    }
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  return iters;
}

// GMRES(kGmresRestart) with right Jacobi preconditioning, A (D^-1 y) = b,
// x = D^-1 y.  Unlike BiCGStab its residual never grows, so it also solves
// the unsymmetric, indefinite stiffness of a cracked body on which BiCGStab
// diverges; an empty row (a node with every bond broken) with a zero right
// side keeps a zero solution.  Each cycle starts from the true residual; the
// solve stops when the rotated residual |g_{j+1}| of a cycle and then the
// true residual are at most rtol ||b||.  Returns iterations (mat-vecs).
int gmres_core(Ctx& c, const DevCsr& A, const double* b, double* x, const double* dinv, double rtol, int max_iter,
               double* dscal, double* z) {
  cudaStream_t s = c.s;
  const int64_t n = A.n;
  const double avg = n ? (double)A.nnz / (double)n : 0.0;
  const int M = kGmresRestart;
  const int g = grid_for(n);
  const int64_t ld = n;
  double *V = nullptr, *part = nullptr, *hd = nullptr, *tmp = nullptr, *yd = nullptr;
  cudaMallocAsync(&V, (size_t)(M + 1) * n * sizeof(double), s);
  cudaMallocAsync(&part, (size_t)(M + 1) * g * sizeof(double), s);
  cudaMallocAsync(&hd, (size_t)(M + 1) * M * sizeof(double), s);
  cudaMallocAsync(&tmp, (size_t)(M + 1) * sizeof(double), s);
  cudaMallocAsync(&yd, (size_t)M * sizeof(double), s);
  double* bb = dscal + 8;
  double* nn = dscal + 9;
  c.dot<double>(n, b, b, bb);
  double hb = 0;
  cudaMemcpyAsync(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double bnorm = std::sqrt(hb);
  std::vector<double> H((size_t)(M + 1) * M), cs(M), sn(M), gv(M + 1), y(M);
  // v_k . w for k < nk into out (acc += out if given), in chunks of kMdotChunk
  auto project = [&](int nk, const double* w, double* out, double* acc) {
    for (int k0 = 0; k0 < nk; k0 += kMdotChunk)
      k_mdot_partial<<<g, kThreads, 0, s>>>(n, V, ld, k0, std::min(kMdotChunk, nk - k0), w, part, g);
    k_mdot_final<<<nk, kThreads, 0, s>>>(part, g, out, acc);
  };
  int its = 0;
  while (bnorm > 0 && its < max_iter) {
    double* v0 = V;
    spmv_t<double>(n, avg, A.ia, A.ja, A.a, x, z, s);
    k_residual<<<g, kThreads, 0, s>>>(n, b, z, v0);
    c.dot<double>(n, v0, v0, nn);
    double hr = 0;
    cudaMemcpyAsync(&hr, nn, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const double beta = std::sqrt(hr);
    if (!(beta > rtol * bnorm)) break;   // converged, or a NaN residual
    k_gmres_normalise<<<g, kThreads, 0, s>>>(n, nn, tmp, v0);
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int k = 0;   // basis vectors of this cycle that enter the update
    bool stop = false;
    for (int j = 0; j < M && its < max_iter; j++) {
      double* w = V + (int64_t)(j + 1) * ld;
      double* hc = hd + (size_t)j * (M + 1);
      k_jacobi<double><<<g, kThreads, 0, s>>>(n, dinv, V + (int64_t)j * ld, z);
      spmv_t<double>(n, avg, A.ia, A.ja, A.a, z, w, s);
      project(j + 1, w, hc, nullptr);
      k_msub<<<g, kThreads, 0, s>>>(n, V, ld, j + 1, hc, w);
      project(j + 1, w, tmp, hc);   // second Gram-Schmidt pass, added into the column
      k_msub<<<g, kThreads, 0, s>>>(n, V, ld, j + 1, tmp, w);
      c.dot<double>(n, w, w, nn);
      k_gmres_normalise<<<g, kThreads, 0, s>>>(n, nn, hc + j + 1, w);
      double* h = H.data() + (size_t)j * (M + 1);
      cudaMemcpyAsync(h, hc, (size_t)(j + 2) * sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      its++;
      for (int i = 0; i < j; i++) {
        const double t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
        h[i] = t;
      }
      const double hsub = h[j + 1];
      const double r = std::hypot(h[j], hsub);
      if (!std::isfinite(r)) {
        stop = true;   // a non-finite column: keep the iterate of the last cycle
        break;
      }
      cs[j] = r > 0 ? h[j] / r : 1.0;
      sn[j] = r > 0 ? hsub / r : 0.0;
      h[j] = r;
      h[j + 1] = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      k = j + 1;
      if (std::fabs(gv[j + 1]) <= rtol * bnorm || !(hsub > 0.0)) break;
    }
    // y = R^-1 g (a zero pivot drops its direction)
    for (int i = k - 1; i >= 0; i--) {
      double t = gv[i];
      for (int l = i + 1; l < k; l++) t -= H[(size_t)l * (M + 1) + i] * y[l];
      const double d = H[(size_t)i * (M + 1) + i];
      y[i] = d != 0.0 ? t / d : 0.0;
    }
    if (k > 0) {
      cudaMemcpyAsync(yd, y.data(), (size_t)k * sizeof(double), cudaMemcpyHostToDevice, s);
      k_gmres_x<<<g, kThreads, 0, s>>>(n, V, ld, k, yd, dinv, x);
      cudaStreamSynchronize(s);   // y leaves scope in the next cycle
    }
    if (stop || k == 0) break;
  }
  cudaFreeAsync(V, s);
  cudaFreeAsync(part, s);
  cudaFreeAsync(hd, s);
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(yd, s);
  return its;
}

}  // namespace

cudaError_t spmv(const DevCsr& A, const double* x, double* y, cudaStream_t s) {
  const double avg = A.n ? (double)A.nnz / (double)A.n : 0.0;
  spmv_t<double>(A.n, avg, A.ia, A.ja, A.a, x, y, s);
  return cudaGetLastError();
}

cudaError_t twolevel_setup(const DevCsr& A, TwoLevelDev& t, cudaStream_t s, bool* usable) {
  const int nc = t.nc;
  // the inverse of the last solve stays valid while the values are the same
  // (a quasi-static increment in which no bond broke reassembles the same K)
  unsigned long long h = 0;
  cudaMemsetAsync(t.hash, 0, sizeof(unsigned long long), s);
  k_values_hash<<<grid_for(A.nnz), kThreads, 0, s>>>(A.nnz, A.a, t.hash);
  cudaMemcpyAsync(&h, t.hash, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaError_t e0 = cudaStreamSynchronize(s);
  if (e0 != cudaSuccess) return e0;
  t.formed = false;
  if (t.have_inverse && (h == t.inverse_of || t.keep_stale)) {
    *usable = true;
    return cudaSuccess;
  }
  t.have_inverse = false;
  t.formed = true;
  k_tl_ap<<<(int)((A.n * 32 + 255) / 256), 256, 0, s>>>(A.n, A.ia, A.ja, A.a, t);
  k_tl_init<<<1024, 256, 0, s>>>(t);
  k_tl_coarse<<<nc, 64, 0, s>>>(t);
  auto gauss_jordan = [&]() {
    k_gj_first<<<(nc + 255) / 256, 256, 0, s>>>(t.M, nc, t.colbuf, t.diag0, t.rpiv, t.ok);
    for (int k = 0; k < nc; k++) {
      const int64_t work = (int64_t)nc * nc;
      k_gj_step<<<(int)((work + 255) / 256), 256, 0, s>>>(t.M, nc, k, t.colbuf + (k & 1) * nc,
                                                          t.colbuf + ((k + 1) & 1) * nc, t.rpiv + (k & 1),
                                                          t.rpiv + ((k + 1) & 1), t.diag0, t.ok);
    }
    k_gj_rdiag<<<(nc + 255) / 256, 256, 0, s>>>(t.M, nc, t.colk);
    k_gj_finish<<<(int)(((int64_t)nc * nc + 255) / 256), 256, 0, s>>>(t.M, nc, t.colk, t.ok);
  };
  if (!t.gj) {
    cudaGraph_t graph;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      gauss_jordan();
      if (cudaStreamEndCapture(s, &graph) == cudaSuccess) {
        if (cudaGraphInstantiate(&t.gj, graph, 0) != cudaSuccess) t.gj = nullptr;
        cudaGraphDestroy(graph);
      }
    }
    cudaGetLastError();
  }
  if (t.gj) cudaGraphLaunch(t.gj, s);
  else gauss_jordan();
  int ok = 0;
  cudaMemcpyAsync(&ok, t.ok, sizeof(int), cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  *usable = e == cudaSuccess && ok != 0;
  t.have_inverse = *usable;
  t.inverse_of = h;
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t krylov_solve(const DevCsr& A, const double* b, double* x, int method, double rtol, int max_iter,
                         int block_dim, cudaStream_t s, KrylovResult* res, TwoLevelDev* tl) {
  const int64_t n = A.n;
  const double avg = n ? (double)A.nnz / (double)n : 0.0;
  Ctx c{s, nullptr};
  double* dscal = nullptr;
  cudaMallocAsync(&c.part, kRedBlocks * sizeof(double), s);
  cudaMallocAsync(&dscal, 16 * sizeof(double), s);
  double* dinv = nullptr;
  cudaMallocAsync(&dinv, n * sizeof(double), s);
  k_diag_inv<<<(int)((n + 255) / 256), 256, 0, s>>>(n, A.ia, A.ja, A.a, dinv);
  unsigned* ticket = nullptr;   // the reductions' last-block ticket
  cudaMallocAsync(&ticket, sizeof(unsigned), s);
  cudaMemsetAsync(ticket, 0, sizeof(unsigned), s);
  // diagonal blocks for block-Jacobi: consecutive rows in groups of block_dim
  int64_t nb = 0;
  int64_t* bptr = nullptr;
  double* binv = nullptr;
  if (method == 1 || method == 3) {
    const int bd = block_dim > 0 ? block_dim : 3;
    nb = (n + bd - 1) / bd;
    std::vector<int64_t> hp(nb + 1);
    for (int64_t i = 0; i <= nb; i++) hp[i] = std::min<int64_t>(i * bd, n);
    cudaMallocAsync(&bptr, (nb + 1) * sizeof(int64_t), s);
    cudaMemcpyAsync(bptr, hp.data(), (nb + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s);
    cudaMallocAsync(&binv, nb * 9 * sizeof(double), s);
    k_block_inverse<<<(int)((nb + 255) / 256), 256, 0, s>>>(nb, bptr, A.ia, A.ja, A.a, binv);
    cudaStreamSynchronize(s);  // hp leaves scope
  }
  double *r, *z, *p, *q, *ax;
  cudaMallocAsync(&r, n * sizeof(double), s);
  cudaMallocAsync(&z, n * sizeof(double), s);
  cudaMallocAsync(&p, n * sizeof(double), s);
  cudaMallocAsync(&q, n * sizeof(double), s);
  cudaMallocAsync(&ax, n * sizeof(double), s);
  const int g = grid_for(n);
  int iters = 0;
  int outer_steps = 0;
  if (method == 0 || method == 1) {
    iters = pcg_core<double>(c, n, avg, A.ia, A.ja, A.a, b, x, dinv, nb, bptr, binv, rtol, max_iter, dscal, r, z,
                             p, q, ticket, true);
  } else if (method == 2 || method == 8) {
    // BiCGStab, right Jacobi preconditioning, from the caller's x; method 8
    // adds the Galerkin coarse correction (the coarse matrix and its inverse
    // are formed here, for this matrix; Jacobi alone if a pivot vanished)
    bool two_level = false;
    if (method == 8 && tl) {
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, s);
      const cudaError_t e = twolevel_setup(A, *tl, s, &two_level);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      res->setup_ms = ms;
      if (e != cudaSuccess) return e;
    }
    double* w[8] = {r, nullptr, nullptr, p, nullptr, nullptr, nullptr, nullptr};
    for (int k : {1, 2, 4, 5, 6, 7}) cudaMallocAsync(&w[k], n * sizeof(double), s);
    double* part2 = nullptr;
    cudaMallocAsync(&part2, 2 * kRedBlocks * sizeof(double), s);
    iters = bicg_core<double>(c, n, avg, A.ia, A.ja, A.a, b, x, dinv, rtol, max_iter, 0, dscal, w, part2, ticket,
                              two_level ? tl : nullptr);
    if (method == 8 && !two_level) method = 2;
    if (method == 8 && tl) {
      // an inverse kept for a changed matrix is formed anew once it costs
      // half as many iterations again as when it was formed
      if (tl->formed) tl->its_ref = iters;
      else if (tl->keep_stale && iters > tl->its_ref + tl->its_ref / 2) tl->have_inverse = false;
    }
    cudaFreeAsync(part2, s);
    for (int k : {1, 2, 4, 5, 6, 7}) cudaFreeAsync(w[k], s);
  } else if (method == 3 || method == 7) {
    // FP32 inner solves (PCG, or BiCGStab for the unsymmetric stiffness)
    // inside FP64 iterative refinement: r = b - A x in FP64, A d ~= r with
    // the FP32 matrix copy to kInnerTol, x += d
    float *af, *rf, *df, *dinvf;
    float* wf[8];
    for (int k = 0; k < 8; k++) cudaMallocAsync(&wf[k], n * sizeof(float), s);
    cudaMallocAsync(&dinvf, n * sizeof(float), s);
    cudaMallocAsync(&af, A.nnz * sizeof(float), s);
    cudaMallocAsync(&rf, n * sizeof(float), s);
    cudaMallocAsync(&df, n * sizeof(float), s);
    double* part2 = nullptr;
    if (method == 7) cudaMallocAsync(&part2, 2 * kRedBlocks * sizeof(double), s);
    k_convert<double, float><<<grid_for(A.nnz), kThreads, 0, s>>>(A.nnz, A.a, af);
    k_convert<double, float><<<g, kThreads, 0, s>>>(n, dinv, dinvf);
    double* bb = dscal + 8;
    double* rr = dscal + 9;
    c.dot<double>(n, b, b, bb);
    double hb = 0;
    cudaMemcpyAsync(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const double bnorm = std::sqrt(hb);
    double last = INFINITY;
    for (int outer = 0; outer < 60 && bnorm > 0 && iters < max_iter; outer++) {
      spmv(A, x, ax, s);
      k_residual<<<g, kThreads, 0, s>>>(n, b, ax, r);
      c.dot<double>(n, r, r, rr);
      double hr = 0;
      cudaMemcpyAsync(&hr, rr, sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      const double rn = std::sqrt(hr);
      if (!(rn > rtol * bnorm)) break;   // converged
      if (!(rn < 0.5 * last)) {
        // the last correction did not halve the FP64 residual: the FP32
        // matrix's rounding (about 6e-8 relative) times the condition number
        // bounds what a refinement step can gain.  A step that made things
        // worse is taken back; the caller falls back to an FP64 method.
        if (!(rn < last)) {
          k_add_to<<<g, kThreads, 0, s>>>(n, df, -1.0, x);
          outer_steps--;
        }
        break;
      }
      last = rn;
      k_convert<double, float><<<g, kThreads, 0, s>>>(n, r, rf);
      cudaMemsetAsync(df, 0, n * sizeof(float), s);
      if (method == 3)
        iters += pcg_core<float>(c, n, avg, A.ia, A.ja, af, rf, df, dinvf, nb, bptr, binv, kInnerTol,
                                 max_iter - iters, dscal, wf[0], wf[1], wf[2], wf[3], ticket, true);
      else
        iters += bicg_core<float>(c, n, avg, A.ia, A.ja, af, rf, df, dinvf, kInnerTol, max_iter - iters, kCgStallIts,
                                  dscal, wf, part2, ticket);
      k_add_to<<<g, kThreads, 0, s>>>(n, df, 1.0, x);
      outer_steps++;
    }
    if (part2) cudaFreeAsync(part2, s);
    for (int k = 0; k < 8; k++) cudaFreeAsync(wf[k], s);
    cudaFreeAsync(dinvf, s);
    cudaFreeAsync(af, s); cudaFreeAsync(rf, s); cudaFreeAsync(df, s);
  } else if (method == 6) {
    iters = gmres_core(c, A, b, x, dinv, rtol, max_iter, dscal, z);
  }
  // true residual
  spmv(A, x, ax, s);
  k_residual<<<g, kThreads, 0, s>>>(n, b, ax, r);
  c.dot<double>(n, r, r, dscal + 10);
  c.dot<double>(n, b, b, dscal + 11);
  double h[2] = {0, 0};
  cudaMemcpyAsync(h, dscal + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t err = cudaStreamSynchronize(s);
  res->iterations = iters;
  res->rel_residual = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
  res->converged = res->rel_residual <= rtol;
  res->method = method;
  res->refinements = outer_steps;
  cudaFreeAsync(r, s); cudaFreeAsync(z, s); cudaFreeAsync(p, s); cudaFreeAsync(q, s); cudaFreeAsync(ax, s);
  cudaFreeAsync(dinv, s); cudaFreeAsync(c.part, s); cudaFreeAsync(dscal, s); cudaFreeAsync(ticket, s);
  if (bptr) cudaFreeAsync(bptr, s);
  if (binv) cudaFreeAsync(binv, s);
  if (err == cudaSuccess) err = cudaGetLastError();
  return err;
}

// ---------------------------------------------------------------------------
// Flexible CG with block-Jacobi and an optional additive coarse correction.
// Each new direction p = z - sum_j (z . q_j / p_j . q_j) p_j is A-orthogonal
// to the last `trunc` directions (q_j = A p_j): with a fixed SPD
// preconditioner and trunc = 1 this is PCG; with the learned (nonlinear)
// coarse correction the longer memory keeps the iteration from stalling.

namespace {

// Flexible CG in five kernels per iteration (plus the coarse correction):
// k_fcg_zq (z . q_j for every kept direction), k_fcg_dir (new direction p and
// the r . p partials), the SpMV, the p . q partials, k_fcg_update (x, r and
// the block-Jacobi z).  Each block repeats the final reduction of the
// partials in the order k_dot_final uses, so the fused iteration gives the
// same bits as one kernel per operation.
constexpr int kFcgMaxDirs = 32;

struct FcgDirs {
  const double* P[kFcgMaxDirs];
  const double* Q[kFcgMaxDirs];
  const double* pq[kFcgMaxDirs];   // p_j . q_j of each kept direction
  int m;                           // kept directions, most recent first
};

// sum of np partials in the order of k_dot_final (thread-strided, then block_sum)
__device__ __forceinline__ double reduce_partials(const double* part, int np, double* sh) {
  double s = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  return block_sum(s, sh);
}

// part[j * gridDim.x + block] = partial of z . q_j
__global__ void k_fcg_zq(int64_t n, const double* z, FcgDirs d, double* part) {
  __shared__ double sh[kThreads];
  for (int j = 0; j < d.m; j++) {
    const double* q = d.Q[j];
    double acc = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      acc += z[i] * q[i];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[j * gridDim.x + blockIdx.x] = acc;
  }
}

// p = z - sum_j (z.q_j / p_j.q_j) p_j (most recent first); part_rp = partials of r . p
__global__ void k_fcg_dir(int64_t n, const double* z, FcgDirs d, const double* part_zq, const double* r, double* p,
                          double* part_rp) {
  __shared__ double sh[kThreads];
  __shared__ double coef[kFcgMaxDirs];
  for (int j = 0; j < d.m; j++) {
    const double zq = reduce_partials(part_zq + j * gridDim.x, gridDim.x, sh);
    if (threadIdx.x == 0) coef[j] = *d.pq[j] != 0.0 ? zq / *d.pq[j] : 0.0;
  }
  __syncthreads();
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double pi = z[i];
    for (int j = 0; j < d.m; j++) pi -= coef[j] * d.P[j][i];
    p[i] = pi;
    acc += r[i] * pi;
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) part_rp[blockIdx.x] = acc;
}

// alpha = r.p / p.q from the partials; x += alpha p, r -= alpha q and
// z = B^-1 r over the d x d diagonal blocks (a thread owns whole blocks)
__global__ void k_fcg_update(int64_t nb, const int64_t* bptr, const double* binv, const double* part_rp,
                             const double* part_pq, int np, double* pq_out, const double* p, const double* q, double* x,
                             double* r, double* z) {
  __shared__ double sh[kThreads];
  const double rp = reduce_partials(part_rp, np, sh);
  const double pq = reduce_partials(part_pq, np, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) *pq_out = pq;
  const double alpha = pq != 0.0 ? rp / pq : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = bptr[i];
    const int sz = (int)(bptr[i + 1] - r0);
    double v[3] = {0, 0, 0};
    for (int c = 0; c < sz; c++) {
      const int64_t k = r0 + c;
      x[k] = x[k] + alpha * p[k];
      const double rk = r[k] - alpha * q[k];
      r[k] = rk;
      v[c] = rk;
    }
    for (int rr = 0; rr < sz; rr++) {
      double a = 0;
      for (int c = 0; c < sz; c++) a += binv[i * 9 + rr * 3 + c] * v[c];
      z[r0 + rr] = a;
    }
  }
}

}  // namespace

cudaError_t krylov_fcg(const DevCsr& A, const double* b, double* x, double rtol, int max_iter, int block_dim,
                       CoarseCorrection* coarse, IterHook* hook, int stall_window, int trunc, cudaStream_t s,
                       KrylovResult* res) {
  const int64_t n = A.n;
  const double avg = n ? (double)A.nnz / (double)n : 0.0;
  const int g = grid_for(n);
  Ctx c{s, nullptr};
  double* dscal = nullptr;
  cudaMallocAsync(&c.part, kRedBlocks * sizeof(double), s);
  cudaMallocAsync(&dscal, 16 * sizeof(double), s);
  double* rr = dscal + 2;
  double* bb = dscal + 3;
  // block-Jacobi: inverses of the d x d diagonal blocks of consecutive rows
  const int bd = block_dim > 0 ? block_dim : 3;
  const int64_t nb = (n + bd - 1) / bd;
  std::vector<int64_t> hp(nb + 1);
  for (int64_t i = 0; i <= nb; i++) hp[i] = std::min<int64_t>(i * bd, n);
  int64_t* bptr = nullptr;
  double* binv = nullptr;
  cudaMallocAsync(&bptr, (nb + 1) * sizeof(int64_t), s);
  cudaMallocAsync(&binv, nb * 9 * sizeof(double), s);
  cudaMemcpyAsync(bptr, hp.data(), (nb + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s);
  k_block_inverse<<<(int)((nb + 255) / 256), 256, 0, s>>>(nb, bptr, A.ia, A.ja, A.a, binv);
  // ring of the last `trunc` directions p_j, q_j = A p_j (and the new one)
  const int mt = std::min(std::max(1, trunc), kFcgMaxDirs) + 1;
  const int gb = (int)std::min<int64_t>((nb + kThreads - 1) / kThreads, kRedBlocks);
  double *part_zq = nullptr, *part_rp = nullptr, *part_pq = nullptr;
  cudaMallocAsync(&part_zq, (size_t)(mt - 1) * g * sizeof(double), s);
  cudaMallocAsync(&part_rp, g * sizeof(double), s);
  cudaMallocAsync(&part_pq, g * sizeof(double), s);
  std::vector<double*> P(mt, nullptr), Q(mt, nullptr);
  double *r, *z, *pqs;
  cudaMallocAsync(&r, n * sizeof(double), s);
  cudaMallocAsync(&z, n * sizeof(double), s);
  cudaMallocAsync(&pqs, mt * sizeof(double), s);
  for (int j = 0; j < mt; j++) {
    cudaMallocAsync(&P[j], n * sizeof(double), s);
    cudaMallocAsync(&Q[j], n * sizeof(double), s);
  }
  cudaError_t err = cudaSuccess;
  auto precond = [&](const double* rin, double* zout) {
    k_apply_block<double><<<(int)((nb + 255) / 256), 256, 0, s>>>(nb, bptr, binv, rin, zout);
    if (coarse && err == cudaSuccess) err = coarse->add(rin, zout, s);
  };
  spmv_t<double>(n, avg, A.ia, A.ja, A.a, x, Q[0], s);
  k_sub<double><<<g, kThreads, 0, s>>>(n, b, Q[0], r);
  c.dot<double>(n, b, b, bb);
  precond(r, z);
  double hb = 0;
  cudaMemcpyAsync(&hb, bb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double bnorm = std::sqrt(hb);
  int it = 0;
  bool stalled = false;
  if (bnorm == 0.0) {
    cudaMemsetAsync(x, 0, n * sizeof(double), s);
  } else {
    const int chunk = 10;
    double win_start = -1.0;
    int win_it = 0;
    while (it < max_iter && err == cudaSuccess) {
      for (int k = 0; k < chunk && it < max_iter; k++, it++) {
        const int slot = it % mt;
        double* p = P[slot];
        double* q = Q[slot];
        FcgDirs d;
        d.m = std::min(it, mt - 1);
        for (int j = 1; j <= d.m; j++) {
          const int js = (it - j) % mt;
          d.P[j - 1] = P[js];
          d.Q[j - 1] = Q[js];
          d.pq[j - 1] = pqs + js;
        }
        if (d.m > 0) k_fcg_zq<<<g, kThreads, 0, s>>>(n, z, d, part_zq);
        k_fcg_dir<<<g, kThreads, 0, s>>>(n, z, d, part_zq, r, p, part_rp);
        spmv_t<double>(n, avg, A.ia, A.ja, A.a, p, q, s);
        k_dot_partial<double><<<g, kThreads, 0, s>>>(n, p, q, part_pq);
        k_fcg_update<<<gb, kThreads, 0, s>>>(nb, bptr, binv, part_rp, part_pq, g, pqs + slot, p, q, x, r, z);
        if (coarse && err == cudaSuccess) err = coarse->add(r, z, s);
        if (hook && (it + 1) % hook->every == 0 && err == cudaSuccess) err = hook->on_iter(it + 1, x, r, z, s);
      }
      c.dot<double>(n, r, r, rr);
      double hr = 0;
      cudaMemcpyAsync(&hr, rr, sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      const double rn = std::sqrt(hr);
      if (!(rn > rtol * bnorm)) break;
      if (!(rn == rn)) { stalled = true; break; }
      if (stall_window > 0) {
        if (win_start < 0) {
          win_start = rn;
          win_it = it;
        } else if (it - win_it >= stall_window) {
          if (rn > 0.1 * win_start) { stalled = true; break; }
          win_start = rn;
          win_it = it;
        }
      }
    }
  }
  // true residual
  spmv_t<double>(n, avg, A.ia, A.ja, A.a, x, Q[0], s);
  k_residual<<<g, kThreads, 0, s>>>(n, b, Q[0], r);
  c.dot<double>(n, r, r, dscal + 10);
  c.dot<double>(n, b, b, dscal + 11);
  double h[2] = {0, 0};
  cudaMemcpyAsync(h, dscal + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (err == cudaSuccess) err = e2;
  res->iterations = it;
  res->rel_residual = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
  res->converged = !stalled && res->rel_residual <= rtol;
  res->method = coarse ? 5 : 4;
  res->refinements = 0;
  cudaFreeAsync(r, s);
  cudaFreeAsync(z, s);
  cudaFreeAsync(pqs, s);
  for (int j = 0; j < mt; j++) {
    cudaFreeAsync(P[j], s);
    cudaFreeAsync(Q[j], s);
  }
  cudaFreeAsync(bptr, s);
  cudaFreeAsync(binv, s);
  cudaFreeAsync(part_zq, s);
  cudaFreeAsync(part_rp, s);
  cudaFreeAsync(part_pq, s);
  cudaFreeAsync(c.part, s);
  cudaFreeAsync(dscal, s);
  if (err == cudaSuccess) err = cudaGetLastError();
  return err;
}

// ---------------------------------------------------------------------------
// Allocation-free Jacobi PCG.
//
// Some callers cannot let a library allocate device memory during a solve: a
// host code that reserves the whole memory budget of the GPU up front for its
// own pools, or a time-stepping loop that must not be stalled by the
// allocator between two steps.  For them the Jacobi PCG above also runs with
// all of its work space (dot-product partials, scalars, 1/diag, r, z, p, q
// and the residual vector) carved out of one fixed device array,
// g_noalloc_scratch, so the solve itself issues no cudaMalloc, cudaMallocAsync
// or cudaFree and calls no allocating library routine.
//
// Limits and rules of use:
//  - n <= kNoAllocMaxN equations (the array holds 6 * kNoAllocMaxN + 1040
//    doubles, 12.6 MB per device); larger systems are rejected with
//    cudaErrorInvalidValue before anything is launched;
//  - the array is global to the device: two solves that overlap in time on
//    the same device (different streams or host threads) race on it and must
//    be serialised by the caller;
//  - no part of the scratch has to start at zero: every word is written
//    before it is read in each call;
//  - the first call on a device looks the array's address up with
//    cudaGetSymbolAddress (once per device, cached); make that first call
//    before any stream capture begins.
constexpr int64_t kNoAllocMaxN = 262144;
constexpr size_t kNoAllocWords = 6 * (size_t)kNoAllocMaxN + kRedBlocks + 16;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocWords];

namespace {
constexpr int kNoAllocMaxDevices = 64;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mu;
}  // namespace

cudaError_t noalloc_scratch_setup(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

int64_t noalloc_max_n() { return kNoAllocMaxN; }

cudaError_t krylov_pcg_noalloc(const DevCsr& A, const double* b, double* x, double rtol, int max_iter, int use_x0,
                               cudaStream_t s, KrylovResult* res) {
  const int64_t n = A.n;
  if (n <= 0 || n > kNoAllocMaxN) return cudaErrorInvalidValue;
  double* w = nullptr;
  cudaError_t err = noalloc_scratch_setup(&w);
  if (err != cudaSuccess) return err;
  const double avg = (double)A.nnz / (double)n;
  Ctx c{s, w};
  double* dscal = w + kRedBlocks;
  double* dinv = dscal + 16;
  double* r = dinv + n;
  double* z = r + n;
  double* p = z + n;
  double* q = p + n;
  double* ax = q + n;
  if (!use_x0) cudaMemsetAsync(x, 0, n * sizeof(double), s);
  k_diag_inv<<<(int)((n + 255) / 256), 256, 0, s>>>(n, A.ia, A.ja, A.a, dinv);
  // the reductions' ticket: a word of the fixed work space, zeroed here
  unsigned* ticket = reinterpret_cast<unsigned*>(dscal + 15);
  cudaMemsetAsync(ticket, 0, sizeof(unsigned), s);
  const int iters = pcg_core<double>(c, n, avg, A.ia, A.ja, A.a, b, x, dinv, 0, nullptr, nullptr, rtol, max_iter,
                                     dscal, r, z, p, q, ticket, false);
  // true residual
  const int g = grid_for(n);
  spmv_t<double>(n, avg, A.ia, A.ja, A.a, x, ax, s);
  k_residual<<<g, kThreads, 0, s>>>(n, b, ax, r);
  c.dot<double>(n, r, r, dscal + 10);
  c.dot<double>(n, b, b, dscal + 11);
  double h[2] = {0, 0};
  cudaMemcpyAsync(h, dscal + 10, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  err = cudaStreamSynchronize(s);
  res->iterations = iters;
  res->rel_residual = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
  res->converged = res->rel_residual <= rtol;
  res->method = 0;
  res->refinements = 0;
  if (err == cudaSuccess) err = cudaGetLastError();
  return err;
}

}  // namespace pdx
