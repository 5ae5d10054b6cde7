// Learned two-level preconditioner: kernels.
//
// Coarse space: a regular grid over the model's bounding box; fine equation
// e (node k, DOF i) interpolates DOF i of the 8 (3D) / 4 (2D) corners of the
// coarse cell around node k with trilinear weights (prolongation P).
// Residuals are restricted by R = P^T; a fine field is averaged onto the
// grid by R~ = diag(1 / row sums of P^T) P^T (the training target of an
// error).
//
// Network: y = W3 tanh(W2 tanh(W1 x + b1) + b2) + b3 with x = R r / |R r|;
// the coarse correction added to the preconditioned residual is
// P (|R r| sigma y), sigma a fixed target scale.  The map it learns is close
// to the linear, odd coarse solve; tanh keeps the network near-odd and
// near-linear on inputs unlike its training set (ReLU did not), so the
// correction stays useful once it has removed the smooth error the training
// residuals were made of.  Training (forward, backward,
// Adam) runs its GEMMs on the tensor cores (mma.sync, BF16 operands, FP32
// accumulation, split K for the long products); inference of one residual
// is one block-wide kernel (k_infer_block) per Krylov iteration.
// Reductions have a fixed order and there are no atomics, so results are
// reproducible.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "learned.h"

namespace pdx {

namespace {

constexpr int kT = 256;
using bf16 = __nv_bfloat16;

// C[M x N] = alpha op(A)[M x K] op(B)[K x N] + beta C, A and B in BF16, C in FP32:
// op(A)(m, k) = TA ? A[k lda + m] : A[m lda + k]; op(B)(k, n) = TB ? B[n ldb + k] : B[k ldb + n].
// Tensor cores: mma.sync m16n8k16 with BF16 operands and FP32 accumulators.
// A block of 4 warps computes a 64 x 64 tile of C over the K range of its
// split (blockIdx.z); each warp a 32 x 32 quarter as 2 x 4 MMA tiles.  K
// slices of 32 are staged in shared memory as As[m][k] and Bs[n][k] (k
// contiguous, rows padded to 40 BF16 against bank conflicts).  With several
// splits the partial tiles go to `part` and k_gemm_reduce adds them in split
// order, so the result does not depend on scheduling.
constexpr int kGT = 64, kGK = 32, kGPad = 40;

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_tc(int M, int N, int K, int kchunk, const bf16* __restrict__ A,
                                                 int lda, const bf16* __restrict__ B, int ldb, float* __restrict__ C,
                                                 int ldc, float alpha, float beta, float* __restrict__ part) {
  __shared__ __align__(16) bf16 As[kGT][kGPad];
  __shared__ __align__(16) bf16 Bs[kGT][kGPad];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int g = lane >> 2, tg = lane & 3;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  const bf16 zero = __float2bfloat16(0.f);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
  for (int k0 = kb; k0 < ke; k0 += kGK) {
    for (int e = threadIdx.x; e < kGT * kGK; e += blockDim.x) {
      // threads run along the contiguous index of the source
      const int mm = TA ? e % kGT : e / kGK, kk = TA ? e / kGT : e % kGK;
      const int m = m0 + mm, k = k0 + kk;
      As[mm][kk] = (m < M && k < ke) ? (TA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k]) : zero;
    }
    for (int e = threadIdx.x; e < kGT * kGK; e += blockDim.x) {
      const int nn = TB ? e / kGK : e % kGT, kk = TB ? e % kGK : e / kGT;
      const int n = n0 + nn, k = k0 + kk;
      Bs[nn][kk] = (n < N && k < ke) ? (TB ? B[(int64_t)n * ldb + k] : B[(int64_t)k * ldb + n]) : zero;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kGK; ks += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int r = wm + i * 16 + g;
        af[i][0] = ld_pair(&As[r][ks + 2 * tg]);
        af[i][1] = ld_pair(&As[r + 8][ks + 2 * tg]);
        af[i][2] = ld_pair(&As[r][ks + 2 * tg + 8]);
        af[i][3] = ld_pair(&As[r + 8][ks + 2 * tg + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int c = wn + j * 8 + g;
        bfr[j][0] = ld_pair(&Bs[c][ks + 2 * tg]);
        bfr[j][1] = ld_pair(&Bs[c][ks + 2 * tg + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  float* P = part ? part + (int64_t)blockIdx.z * M * N : nullptr;
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int m = m0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
        const int n = n0 + wn + j * 8 + 2 * tg + (q & 1);
        if (m >= M || n >= N) continue;
        if (P) {
          P[(int64_t)m * N + n] = acc[i][j][q];
        } else {
          float* cp = C + (int64_t)m * ldc + n;
          *cp = beta == 0.f ? alpha * acc[i][j][q] : alpha * acc[i][j][q] + beta * *cp;
        }
      }
}

// C = alpha sum_z part[z] + beta C, the splits added in order
__global__ void k_gemm_reduce(int M, int N, int splits, const float* __restrict__ part, float* __restrict__ C,
                              int ldc, float alpha, float beta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  float s = 0.f;
  for (int z = 0; z < splits; z++) s += part[(int64_t)z * M * N + i];
  float* cp = C + (i / N) * ldc + (i % N);
  *cp = beta == 0.f ? alpha * s : alpha * s + beta * *cp;
}

// Splits of K for an M x N x K product: enough blocks to cover the SMs about
// twice, each split at least 64 deep.
int gemm_splits(int M, int N, int K) {
  const int tiles = ((M + kGT - 1) / kGT) * ((N + kGT - 1) / kGT);
  const int want = (304 + tiles - 1) / tiles;
  return std::max(1, std::min(want, K / 64));
}

template <bool TA, bool TB>
void gemm(int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc, float alpha,
          float beta, float* work, cudaStream_t s) {
  const int splits = work ? gemm_splits(M, N, K) : 1;
  const int kchunk = ((K + splits - 1) / splits + kGK - 1) / kGK * kGK;
  const int nz = (K + kchunk - 1) / kchunk;
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, nz);
  k_gemm_tc<TA, TB><<<grid, 128, 0, s>>>(M, N, K, kchunk, A, lda, B, ldb, C, ldc, alpha, beta,
                                          nz > 1 ? work : nullptr);
  if (nz > 1) k_gemm_reduce<<<(int)(((int64_t)M * N + 255) / 256), 256, 0, s>>>(M, N, nz, work, C, ldc, alpha, beta);
}

// Z[m][n] += bias[n]; H = BF16(tanh(Z)) (or Z without activation)
__global__ void k_bias_act(int M, int N, float* Z, const float* bias, bf16* H, int act) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  const float z = Z[i] + bias[i % N];
  Z[i] = z;
  if (H) H[i] = __float2bfloat16(act ? tanhf(z) : z);
}

// dY = 2 w_m (Y - T); loss_row[m] = w_m |Y_m - T_m|^2 (one block per row)
__global__ void k_loss_grad(int M, int N, const float* Y, const float* T, const float* w, float* dY, bf16* dY16,
                            float* loss_row) {
  const int m = blockIdx.x;
  __shared__ float sh[kT];
  float acc = 0.f;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    const int64_t i = (int64_t)m * N + n;
    const float d = Y[i] - T[i];
    acc += d * d;
    const float g = 2.f * w[m] * d;
    dY[i] = g;
    dY16[i] = __float2bfloat16(g);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_row[m] = w[m] * sh[0];
}

// dZ = dH (1 - tanh(Z)^2)
__global__ void k_act_back(int64_t n, const float* dH, const float* Z, float* dZ, bf16* dZ16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float th = tanhf(Z[i]);
  const float g = dH[i] * (1.f - th * th);
  dZ[i] = g;
  dZ16[i] = __float2bfloat16(g);
}

// db[n] = sum_m dZ[m][n] in row order
__global__ void k_colsum(int M, int N, const float* dZ, float* db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; m++) s += dZ[(int64_t)m * N + n];
  db[n] = s;
}

__global__ void k_sum(int n, const float* x, float* out) {
  __shared__ float sh[kT];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void k_adam(int64_t n, float* w, const float* g, float* m1, float* m2, float lr, float b1, float b2,
                       float eps, float c1, float c2, bf16* w16) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  const float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[i] = wi;
  if (w16) w16[i] = __float2bfloat16(wi);
}

__global__ void k_to_bf16(int64_t n, const float* x, bf16* y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// coarse[c] = sum_j w_j r[e_j] over restriction row c (FP64 accumulation)
// out[c] = sum_j rw[j] r[ridx[j]] over row c of P^T; one block per row,
// thread-strided FP64 sums combined in a fixed order (same bits on every run)
__global__ void __launch_bounds__(kT) k_restrict(int nc, const int* rptr, const int* ridx, const float* rw,
                                                 const double* r, float* out) {
  __shared__ double red[kT / 32];
  const int c = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double s = 0.0;
  const int j1 = rptr[c + 1];
  for (int j = rptr[c] + threadIdx.x; j < j1; j += kT) s += (double)rw[j] * r[ridx[j]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kT / 32; w++) t += red[w];
    out[c] = (float)t;
  }
}

// z[e] += scale sum_j P_ej c[j]
template <int NP>
__global__ void k_prolong_add(int64_t n, const int* pidx, const float* pw, const float* c, const float* scale,
                              double* z) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < NP; j++) {
    const int ci = pidx[e * NP + j];
    if (ci >= 0) s += pw[e * NP + j] * c[ci];
  }
  z[e] += (double)(*scale) * (double)s;
}

// one block: x16 = BF16(x / |x|), *scale_out = |x| sigma
__global__ void k_normalize(int n, const float* x, bf16* x16, float sigma, float* scale_out) {
  __shared__ float sh[kT];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i] * x[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const float nrm = sqrtf(sh[0]);
  const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x16[i] = __float2bfloat16(x[i] * inv);
  if (threadIdx.x == 0) *scale_out = nrm * sigma;
}

// inference layer (batch 1): h[row] = act(W[row] . x + b[row]), one warp per row
__global__ void k_gemv_rows(int rows, int cols, const bf16* W, const bf16* x, const float* b, int act, bf16* h16,
                            float* hf) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  float s = 0.f;
  const bf16* w = W + (int64_t)row * cols;
  for (int k = lane; k < cols; k += 32) s = fmaf(__bfloat162float(w[k]), __bfloat162float(x[k]), s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const float z = s + b[row];
    const float a = act ? tanhf(z) : z;
    if (h16) h16[row] = __float2bfloat16(a);
    if (hf) hf[row] = a;
  }
}

// Inference copy of the BF16 weights with rows padded to a multiple of 8
// (16-byte rows): W1 (H x ldi), W2 (H x ldh), W3 (nout x ldh); pads are 0.
__global__ void k_pack_infer(int nin, int H, int nout, int ldi, int ldh, const bf16* w16, bf16* wi) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n1 = (int64_t)H * ldi, n2 = (int64_t)H * ldh, n3 = (int64_t)nout * ldh;
  if (i >= n1 + n2 + n3) return;
  const bf16* W2 = w16 + (int64_t)H * nin + H;
  const bf16* W3 = W2 + (int64_t)H * H + H;
  bf16 v = __float2bfloat16(0.f);
  if (i < n1) {
    const int row = (int)(i / ldi), col = (int)(i % ldi);
    if (col < nin) v = w16[(int64_t)row * nin + col];
  } else if (i < n1 + n2) {
    const int64_t k = i - n1;
    const int row = (int)(k / ldh), col = (int)(k % ldh);
    if (col < H) v = W2[(int64_t)row * H + col];
  } else {
    const int64_t k = i - n1 - n2;
    const int row = (int)(k / ldh), col = (int)(k % ldh);
    if (col < H) v = W3[(int64_t)row * H + col];
  }
  wi[i] = v;
}

// One layer of the one-block inference: out[row] = W[row] . in (+ b, tanh),
// G consecutive threads per row (G a power of 2 <= 32), each summing every
// G-th 16-byte slice (8 BF16) of the row; the G partials are combined by a
// butterfly within the group.  W rows have ld elements, ld % 8 == 0; `in` is
// in shared memory.  Rows are taken in passes of blockDim / G.
template <int G>
__device__ __forceinline__ void layer_rows(int rows, int ld, const bf16* __restrict__ W, const bf16* in,
                                           const float* b, bool act, bf16* out16, float* outf) {
  const int ld8 = ld / 8;
  const int sub = threadIdx.x & (G - 1);
  for (int row0 = 0; row0 < rows; row0 += blockDim.x / G) {
    const int row = row0 + threadIdx.x / G;
    float s = 0.f;
    if (row < rows) {
      const uint4* w = reinterpret_cast<const uint4*>(W + (int64_t)row * ld);
      const uint4* x = reinterpret_cast<const uint4*>(in);
      for (int k = sub; k < ld8; k += G) {
        const uint4 a = __ldg(w + k);
        const uint4 v = x[k];
        const __nv_bfloat162* a2 = reinterpret_cast<const __nv_bfloat162*>(&a);
        const __nv_bfloat162* v2 = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float2 fa = __bfloat1622float2(a2[q]);
          const float2 fv = __bfloat1622float2(v2[q]);
          s = fmaf(fa.x, fv.x, s);
          s = fmaf(fa.y, fv.y, s);
        }
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (row < rows && sub == 0) {
      const float z = s + b[row];
      if (out16) out16[row] = __float2bfloat16(act ? tanhf(z) : z);
      if (outf) outf[row] = act ? tanhf(z) : z;
    }
  }
}

// The whole inference of one residual in one block: |x|, x16 = BF16(x / |x|),
// two tanh layers and the linear output layer; *scale_out = |x| sigma.
__global__ void __launch_bounds__(1024) k_infer_block(int nin, int H, int nout, int ldi, int ldh, const float* x,
                                                      float sigma, const bf16* __restrict__ wi, const float* b1,
                                                      const float* b2, const float* b3, float* y, float* scale_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16* xs = reinterpret_cast<bf16*>(smem_raw);
  bf16* h1 = xs + ldi;
  bf16* h2 = h1 + ldh;
  __shared__ float red[32];
  __shared__ float nrm_sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float s = 0.f;
  for (int i = threadIdx.x; i < nin; i += blockDim.x) s += x[i] * x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  if (warp == 0) {
    float t = lane < nw ? red[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) nrm_sh = sqrtf(t);
  }
  __syncthreads();
  const float nrm = nrm_sh;
  const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
  for (int i = threadIdx.x; i < ldi; i += blockDim.x) xs[i] = __float2bfloat16(i < nin ? x[i] * inv : 0.f);
  for (int i = H + threadIdx.x; i < ldh; i += blockDim.x) {
    h1[i] = __float2bfloat16(0.f);
    h2[i] = __float2bfloat16(0.f);
  }
  __syncthreads();
  const bf16* W1 = wi;
  const bf16* W2 = W1 + (int64_t)H * ldi;
  const bf16* W3 = W2 + (int64_t)H * ldh;
  layer_rows<8>(H, ldi, W1, xs, b1, true, h1, nullptr);
  __syncthreads();
  layer_rows<8>(H, ldh, W2, h1, b2, true, h2, nullptr);
  __syncthreads();
  layer_rows<2>(nout, ldh, W3, h2, b3, false, nullptr, y);
  if (threadIdx.x == 0) *scale_out = nrm * sigma;
}

// S[j] = ax - S[j] for samples j in [first, last): iterate averages -> error averages
__global__ void k_err(int first, int last, int nc, const float* ax, float* S) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)(last - first) * nc;
  if (i >= n) return;
  const int64_t j = (int64_t)first * nc + i;
  S[j] = ax[i % nc] - S[j];
}

// norms[j] = |S_j| (one block per sample)
__global__ void k_rownorm(int nc, const float* S, float* norms) {
  __shared__ float sh[kT];
  const float* x = S + (int64_t)blockIdx.x * nc;
  float s = 0.f;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) s += x[i] * x[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) norms[blockIdx.x] = sqrtf(sh[0]);
}

// batch row m from sample idx[m]: X = S_r / |S_r| (BF16), T = S_e / (|S_r| sigma), W = 1 / (|T|^2 B)
__global__ void k_stage(int B, int nc, const int* idx, const float* S_r, const float* S_e, const float* norms,
                        float sigma, bf16* X, float* T, float* W) {
  __shared__ float sh[kT];
  const int m = blockIdx.x;
  const int j = idx[m];
  const float nr = norms[j];
  const float inv = nr > 0.f ? 1.f / nr : 0.f;
  const float tinv = inv / sigma;
  float s = 0.f;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    X[(int64_t)m * nc + i] = __float2bfloat16(S_r[(int64_t)j * nc + i] * inv);
    const float t = S_e[(int64_t)j * nc + i] * tinv;
    T[(int64_t)m * nc + i] = t;
    s += t * t;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) W[m] = sh[0] > 0.f ? 1.f / (sh[0] * (float)B) : 0.f;
}

__global__ void k_stage_raw(int64_t n, const float* Xf, bf16* X) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) X[i] = __float2bfloat16(Xf[i]);
}

// b[i] uniform in [-1, 1) from a 64-bit mix of (seed, i) (splitmix64 finaliser)
__global__ void k_rand_rhs(int64_t n, uint64_t seed, double* b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  b[i] = (double)(z >> 11) * 0x1.0p-52 - 1.0;
}

int grid_of(int64_t n) { return (int)((n + kT - 1) / kT); }

}  // namespace

// ----------------------------------------------------------------- MLP ----

int64_t gemm_work_floats(int Bmax, int nin, int H, int nout) {
  int64_t mx = 0;
  for (int B = 1; B <= Bmax; B++) {   // any batch size up to Bmax
    const int shapes[8][3] = {{B, H, nin}, {B, H, H},   {B, nout, H}, {nout, H, B},
                              {B, H, nout}, {H, H, B}, {B, H, H},    {H, nin, B}};
    for (const auto& sh : shapes) {
      const int splits = gemm_splits(sh[0], sh[1], sh[2]);
      if (splits > 1) mx = std::max(mx, (int64_t)splits * sh[0] * sh[1]);
    }
  }
  return mx;
}

void Mlp::param_views(float* base, float** W1, float** b1, float** W2, float** b2, float** W3, float** b3) const {
  float* p = base;
  *W1 = p; p += (size_t)H * nin;
  *b1 = p; p += H;
  *W2 = p; p += (size_t)H * H;
  *b2 = p; p += H;
  *W3 = p; p += (size_t)nout * H;
  *b3 = p;
}

cudaError_t Mlp::forward_backward(int B, const bf16* X, const float* T, const float* wrow, bool grads,
                                  cudaStream_t s) {
  // split K only with the work space sized for Bmax rows (B <= Bmax)
  float *W1, *b1, *W2, *b2, *W3, *b3;
  param_views(w, &W1, &b1, &W2, &b2, &W3, &b3);
  const bf16* W1h = w16;
  const bf16* W2h = W1h + (size_t)H * nin + H;
  const bf16* W3h = W2h + (size_t)H * H + H;
  const int g1 = grid_of((int64_t)B * H), g3 = grid_of((int64_t)B * nout);
  gemm<false, true>(B, H, nin, X, nin, W1h, nin, Z1, H, 1.f, 0.f, work, s);
  k_bias_act<<<g1, kT, 0, s>>>(B, H, Z1, b1, H1, 1);
  gemm<false, true>(B, H, H, H1, H, W2h, H, Z2, H, 1.f, 0.f, work, s);
  k_bias_act<<<g1, kT, 0, s>>>(B, H, Z2, b2, H2, 1);
  gemm<false, true>(B, nout, H, H2, H, W3h, H, Y, nout, 1.f, 0.f, work, s);
  k_bias_act<<<g3, kT, 0, s>>>(B, nout, Y, b3, nullptr, 0);
  if (!T) return cudaGetLastError();
  k_loss_grad<<<B, kT, 0, s>>>(B, nout, Y, T, wrow, dY, dY16, loss_row);
  k_sum<<<1, kT, 0, s>>>(B, loss_row, loss);
  if (!grads) return cudaGetLastError();
  float *gW1, *gb1, *gW2, *gb2, *gW3, *gb3;
  param_views(g, &gW1, &gb1, &gW2, &gb2, &gW3, &gb3);
  // layer 3: gW3 = dY^T H2, gb3 = sum dY, dH2 = dY W3
  gemm<true, false>(nout, H, B, dY16, nout, H2, H, gW3, H, 1.f, 0.f, work, s);
  k_colsum<<<grid_of(nout), kT, 0, s>>>(B, nout, dY, gb3);
  gemm<false, false>(B, H, nout, dY16, nout, W3h, H, dH, H, 1.f, 0.f, work, s);
  k_act_back<<<g1, kT, 0, s>>>((int64_t)B * H, dH, Z2, dZ, dZ16);
  // layer 2
  gemm<true, false>(H, H, B, dZ16, H, H1, H, gW2, H, 1.f, 0.f, work, s);
  k_colsum<<<grid_of(H), kT, 0, s>>>(B, H, dZ, gb2);
  gemm<false, false>(B, H, H, dZ16, H, W2h, H, dH, H, 1.f, 0.f, work, s);
  k_act_back<<<g1, kT, 0, s>>>((int64_t)B * H, dH, Z1, dZ, dZ16);
  // layer 1
  gemm<true, false>(H, nin, B, dZ16, H, X, nin, gW1, nin, 1.f, 0.f, work, s);
  k_colsum<<<grid_of(H), kT, 0, s>>>(B, H, dZ, gb1);
  return cudaGetLastError();
}

cudaError_t Mlp::adam_step(float lr, cudaStream_t s) {
  step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  const int64_t n = n_params();
  k_adam<<<grid_of(n), kT, 0, s>>>(n, w, g, m1, m2, lr, b1, b2, 1e-8f, c1, c2, w16);
  return cudaGetLastError();
}

cudaError_t Mlp::sync_bf16(cudaStream_t s) {
  const int64_t n = n_params();
  k_to_bf16<<<grid_of(n), kT, 0, s>>>(n, w, w16);
  return cudaGetLastError();
}

int64_t Mlp::n_infer() const {
  const int ldi = (nin + 7) / 8 * 8, ldh = (H + 7) / 8 * 8;
  return (int64_t)H * ldi + (int64_t)H * ldh + (int64_t)nout * ldh;
}

bool Mlp::block_infer_ok() const { return nin <= kInferMaxIn && nout <= kInferMaxIn && H <= kInferMaxH; }

cudaError_t Mlp::pack_infer(cudaStream_t s) {
  if (!wi) return cudaSuccess;
  const int ldi = (nin + 7) / 8 * 8, ldh = (H + 7) / 8 * 8;
  k_pack_infer<<<grid_of(n_infer()), kT, 0, s>>>(nin, H, nout, ldi, ldh, w16, wi);
  return cudaGetLastError();
}

cudaError_t Mlp::infer_block(const float* x, float sigma, float* y, float* scale, cudaStream_t s) {
  float *W1, *b1, *W2, *b2, *W3, *b3;
  param_views(w, &W1, &b1, &W2, &b2, &W3, &b3);
  const int ldi = (nin + 7) / 8 * 8, ldh = (H + 7) / 8 * 8;
  const size_t smem = (size_t)(ldi + 2 * ldh) * sizeof(bf16);
  k_infer_block<<<1, 1024, smem, s>>>(nin, H, nout, ldi, ldh, x, sigma, wi, b1, b2, b3, y, scale);
  return cudaGetLastError();
}

cudaError_t Mlp::infer(const bf16* x16, float* y, cudaStream_t s) {
  float *W1, *b1, *W2, *b2, *W3, *b3;
  param_views(w, &W1, &b1, &W2, &b2, &W3, &b3);
  const bf16* W1h = w16;
  const bf16* W2h = W1h + (size_t)H * nin + H;
  const bf16* W3h = W2h + (size_t)H * H + H;
  k_gemv_rows<<<(H + 7) / 8, 256, 0, s>>>(H, nin, W1h, x16, b1, 1, H1, nullptr);
  k_gemv_rows<<<(H + 7) / 8, 256, 0, s>>>(H, H, W2h, H1, b2, 1, H2, nullptr);
  k_gemv_rows<<<(nout + 7) / 8, 256, 0, s>>>(nout, H, W3h, H2, b3, 0, nullptr, y);
  return cudaGetLastError();
}

// ------------------------------------------------------ transfer, data ----

cudaError_t coarse_restrict(const CoarseSpace& cs, bool average, const double* r, float* out, cudaStream_t s) {
  if (cs.nc <= 0) return cudaSuccess;
  k_restrict<<<cs.nc, kT, 0, s>>>(cs.nc, cs.rptr, cs.ridx, average ? cs.aw : cs.rw, r, out);
  return cudaGetLastError();
}

cudaError_t coarse_prolong_add(const CoarseSpace& cs, const float* c, const float* scale, double* z,
                               cudaStream_t s) {
  if (cs.np == 8) k_prolong_add<8><<<grid_of(cs.n), kT, 0, s>>>(cs.n, cs.pidx, cs.pw, c, scale, z);
  else k_prolong_add<4><<<grid_of(cs.n), kT, 0, s>>>(cs.n, cs.pidx, cs.pw, c, scale, z);
  return cudaGetLastError();
}

cudaError_t coarse_normalize(int n, const float* x, bf16* x16, float sigma, float* scale, cudaStream_t s) {
  k_normalize<<<1, kT, 0, s>>>(n, x, x16, sigma, scale);
  return cudaGetLastError();
}

cudaError_t learned_err(int first, int last, int nc, const float* ax, float* S, cudaStream_t s) {
  const int64_t n = (int64_t)(last - first) * nc;
  if (n <= 0) return cudaSuccess;
  k_err<<<grid_of(n), kT, 0, s>>>(first, last, nc, ax, S);
  return cudaGetLastError();
}

cudaError_t learned_norms(int count, int nc, const float* S, float* norms, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  k_rownorm<<<count, kT, 0, s>>>(nc, S, norms);
  return cudaGetLastError();
}

cudaError_t learned_stage(int B, int nc, const int* idx, const float* S_r, const float* S_e, const float* norms,
                          float sigma, bf16* X, float* T, float* W, cudaStream_t s) {
  k_stage<<<B, kT, 0, s>>>(B, nc, idx, S_r, S_e, norms, sigma, X, T, W);
  return cudaGetLastError();
}

cudaError_t learned_stage_raw(int B, int nc, const float* Xf, bf16* X, cudaStream_t s) {
  const int64_t n = (int64_t)B * nc;
  k_stage_raw<<<grid_of(n), kT, 0, s>>>(n, Xf, X);
  return cudaGetLastError();
}

namespace {
__global__ void k_add_scalar(const float* x, float* acc) { *acc += *x; }
}  // namespace

cudaError_t learned_add_scalar(const float* x, float* acc, cudaStream_t s) {
  k_add_scalar<<<1, 1, 0, s>>>(x, acc);
  return cudaGetLastError();
}

cudaError_t learned_random_rhs(int64_t n, uint64_t seed, double* b, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_rand_rhs<<<grid_of(n), kT, 0, s>>>(n, seed, b);
  return cudaGetLastError();
}

}  // namespace pdx
