// Learned two-level preconditioner (host side) and step-by-step implicit
// Newmark dynamics.
//
// The Newmark step restates pdfemDynamicNewmarkSolver_CSRformat
// (pdsolve.cpp:6092-6290): predictor, K_N = beta dt^2 K + M assembled through
// the scatter map (pdfemAssembleKNFR_CSRformat :6327-6397), K_N a_{n+1} = F,
// update of displacement and velocity (updateDispVelo :6399-6422).  The
// reference factorises K_N with PARDISO at every step; here the solve is a
// Krylov method chosen per call:
//   0-3  the methods of krylov_solve (Jacobi PCG, block-Jacobi PCG, BiCGStab,
//        mixed PCG + FP64 refinement); 6 its restarted GMRES
//   4    block-Jacobi flexible CG: the plain method the learned one is judged by
//   5    flexible CG with block-Jacobi plus the learned coarse correction; if
//        it stalls or needs more iterations than the plain solves did,
//        block-Jacobi flexible CG and then BiCGStab take over from the current
//        iterate.  Plain block-Jacobi FCG is also the arbiter: after two learned
//        solves in a row slower than the plain ones, method 5 runs the plain
//        method until the network is retrained (pdx_learned_active tells).
// With `collect`, a method-4 solve stores one training pair per iteration:
// the restricted residual P^T r_j and the coarse average of the error
// x* - x_j, known once the solve has converged (the solver generates its own
// training data); pdx_learned_probe adds solves with random right-hand sides.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>

#include "learned.h"

namespace pdx {

namespace {

// training pairs are kept while |P^T r_j| >= kTailCut * tol * |P^T r_0|
constexpr double kTailCut = 1e3;

struct Collector : IterHook {
  Learned* L = nullptr;
  cudaError_t on_iter(int, const double* x, const double* r, const double*, cudaStream_t s) override {
    if (L->count >= L->cap) return cudaSuccess;
    const int64_t o = (int64_t)L->count * L->cs.nc;
    cudaError_t e = coarse_restrict(L->cs, false, r, L->S_r + o, s);
    if (e == cudaSuccess) e = coarse_restrict(L->cs, true, x, L->S_x + o, s);
    L->count++;
    return e;
  }
};

// Coarse grid over the bounding box of the nodes; every fine equation gets
// the trilinear (bilinear in 2D) weights of the corners of its node's cell.
void build_coarse(const pdx_model* m, const int cells_in[3], std::vector<int>& pidx, std::vector<float>& pw,
                  std::vector<int>& rptr, std::vector<int>& ridx, std::vector<float>& rw, std::vector<float>& aw,
                  int& nc, int& np, int cells[3]) {
  const int D = m->mesh.dim, N = m->mesh.n_node;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < N; k++)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], m->mesh.X[(size_t)k * 3 + a]);
      hi[a] = std::max(hi[a], m->mesh.X[(size_t)k * 3 + a]);
    }
  for (int a = 0; a < 3; a++) cells[a] = a < D ? std::max(1, cells_in[a]) : 0;
  const int nxn = cells[0] + 1, nyn = cells[1] + 1, nzn = D == 3 ? cells[2] + 1 : 1;
  nc = nxn * nyn * nzn * D;
  np = D == 3 ? 8 : 4;
  const int64_t n = m->setup.n_eq;
  pidx.assign((size_t)n * np, -1);
  pw.assign((size_t)n * np, 0.f);
  for (int k = 0; k < N; k++) {
    int ci[3] = {0, 0, 0};
    double t[3] = {0, 0, 0};
    for (int a = 0; a < D; a++) {
      const double len = hi[a] - lo[a];
      const double u = len > 0 ? (m->mesh.X[(size_t)k * 3 + a] - lo[a]) / len * cells[a] : 0.0;
      const int c = std::min(std::max((int)std::floor(u), 0), cells[a] - 1);
      ci[a] = c;
      t[a] = std::min(std::max(u - c, 0.0), 1.0);
    }
    for (int i = 0; i < D; i++) {
      const int e = m->setup.eq[(size_t)k * D + i];
      if (e < 0) continue;
      for (int corner = 0; corner < np; corner++) {
        const int dx = corner & 1, dy = (corner >> 1) & 1, dz = (corner >> 2) & 1;
        double w = (dx ? t[0] : 1 - t[0]) * (dy ? t[1] : 1 - t[1]);
        if (D == 3) w *= dz ? t[2] : 1 - t[2];
        const int node = (ci[0] + dx) + nxn * ((ci[1] + dy) + nyn * (D == 3 ? ci[2] + dz : 0));
        pidx[(size_t)e * np + corner] = node * D + i;
        pw[(size_t)e * np + corner] = (float)w;
      }
    }
  }
  // transpose: restriction rows per coarse DOF, fine equations in order
  rptr.assign(nc + 1, 0);
  for (size_t j = 0; j < pidx.size(); j++)
    if (pidx[j] >= 0 && pw[j] != 0.f) rptr[pidx[j] + 1]++;
  for (int c = 0; c < nc; c++) rptr[c + 1] += rptr[c];
  ridx.assign(rptr[nc], 0);
  rw.assign(rptr[nc], 0.f);
  std::vector<int> fill(rptr.begin(), rptr.end() - 1);
  for (int64_t e = 0; e < n; e++)
    for (int j = 0; j < np; j++) {
      const int c = pidx[(size_t)e * np + j];
      if (c < 0 || pw[(size_t)e * np + j] == 0.f) continue;
      ridx[fill[c]] = (int)e;
      rw[fill[c]++] = pw[(size_t)e * np + j];
    }
  aw.assign(rw.size(), 0.f);
  for (int c = 0; c < nc; c++) {
    double s = 0;
    for (int j = rptr[c]; j < rptr[c + 1]; j++) s += rw[j];
    for (int j = rptr[c]; j < rptr[c + 1]; j++) aw[j] = s > 0 ? (float)(rw[j] / s) : 0.f;
  }
}

template <typename T>
T* dev_upload(DevBuf& b, const std::vector<T>& h, cudaStream_t s) {
  T* d = b.alloc<T>(h.size());
  if (d && !h.empty()) cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  return d;
}

DevCsr model_csr(const pdx_model* m) {
  DevCsr A;
  A.n = m->setup.n_eq;
  A.nnz = (int64_t)m->setup.csr_ja.size();
  A.ia = m->d_ia;
  A.ja = m->d_ja;
  A.a = m->d_Kval;
  return A;
}

// Block-Jacobi flexible CG on the model's current matrix.  With L, every
// iterate gives a training pair; the pairs are kept only if the solve
// converges, and only up to the point where |P^T r_j| comes within kTailCut
// of the tolerance: the converged x stands in for x*, and past that point
// x* - x_j is mostly the error of the stand-in.
pdx_status plain_solve(pdx_model* m, const double* b, double* x, Learned* L, KrylovResult* kr) {
  Collector col;
  if (L) {
    col.L = L;
    col.every = 1;
    L->solve_first = L->count;
  }
  pdx_status st = cuda_check(krylov_fcg(model_csr(m), b, x, m->cmd.solve_tol, m->cmd.solve_maxit, m->mesh.dim,
                                        nullptr, L ? &col : nullptr, 0, 1, m->stream, kr), "flexible CG");
  if (st || !L) return st;
  if (!kr->converged) {
    L->count = L->solve_first;
    return PDX_OK;
  }
  st = cuda_check(coarse_restrict(L->cs, true, x, L->ax, m->stream), "restriction");
  if (!st) st = cuda_check(learned_err(L->solve_first, L->count, L->cs.nc, L->ax, L->S_x, m->stream), "errors");
  if (st) return st;
  const int first = L->solve_first, cnt = L->count - first;
  if (cnt < 1) return PDX_OK;
  const int64_t nc = L->cs.nc;
  std::vector<float> nr((size_t)cnt);
  st = cuda_check(learned_norms(cnt, (int)nc, L->S_r + first * nc, L->S_scale + first, m->stream), "norms");
  if (!st) cudaMemcpyAsync(nr.data(), L->S_scale + first, (size_t)cnt * 4, cudaMemcpyDeviceToHost, m->stream);
  if (!st) st = cuda_check(cudaStreamSynchronize(m->stream), "norms");
  if (st) return st;
  const double cut = kTailCut * m->cmd.solve_tol * nr[0];
  int keep = 0;
  while (keep < cnt && nr[keep] >= cut) keep++;
  L->count = first + keep;
  return PDX_OK;
}

pdx_status solve_newmark_system(pdx_model* m, int method, bool collect, double* x, KrylovResult* kr) {
  const DevCsr A = model_csr(m);
  const double* b = m->d_tmp_eq[0];
  const double tol = m->cmd.solve_tol;
  const int maxit = m->cmd.solve_maxit;
  const int bd = m->mesh.dim;
  Learned* L = m->learned;
  if (method == 8) {
    const pdx_status st8 = twolevel_prepare(m);
    if (st8) return st8;
    return cuda_check(krylov_solve(A, b, x, 8, tol, maxit, bd, m->stream, kr, &m->twolevel->dev), "Krylov solve");
  }
  if (method <= 3 || method >= 6) return cuda_check(krylov_solve(A, b, x, method, tol, maxit, bd, m->stream, kr), "Krylov solve");
  if (method == 4) return plain_solve(m, b, x, collect ? L : nullptr, kr);
  if (!L || !L->trained) return set_error(PDX_ERR_INVALID, "learned preconditioner not set up and trained");
  if (L->disabled) return plain_solve(m, b, x, nullptr, kr);
  pdx_status st = cuda_check(L->net.pack_infer(m->stream), "inference weights");
  if (st) return st;
  // A learned solve that needs more iterations than the plain ones has lost:
  // it is cut there and plain flexible CG finishes from the current iterate.
  const int cap = L->plain_n > 0 ? std::min(maxit, (int)std::ceil(L->plain_its)) : maxit;
  st = cuda_check(krylov_fcg(A, b, x, tol, cap, bd, L, nullptr, L->stall_window, L->trunc, m->stream, kr),
                  "learned flexible CG");
  if (st || kr->converged) return st;
  const int its = kr->iterations;
  st = cuda_check(krylov_fcg(A, b, x, tol, maxit, bd, nullptr, nullptr, 400, 1, m->stream, kr), "flexible CG");
  kr->iterations += its;
  if (st || kr->converged) return st;
  const int its2 = kr->iterations;
  st = cuda_check(krylov_solve(A, b, x, 2, tol, maxit, bd, m->stream, kr), "BiCGStab");
  kr->iterations += its2;
  return st;
}

}  // namespace

// Coarse grid of the two-level BiCGStab (method 8): kTwoLevelCells cells per
// axis over the nodes' bounding box, fewer where a coupling of the matrix (a
// bond or an element) is longer than a cell, so that every row's couplings
// stay within one cell of its own (the windows of k_tl_ap and k_tl_coarse).
// On C3's loaded increment (320k equations) the exact Galerkin correction
// gives 168 BiCGStab iterations with 10x10 cells, 132 with 14x14, 95 with
// 20x20, 83 with 28x28 and 60 with 40x40, against 1,835 with Jacobi
// (oracle/twolevel_study.py); 20x20 keeps the coarse inverse (882 DOFs) a
// few milliseconds to form.
constexpr int kTwoLevelCells = 20;

pdx_status twolevel_prepare(pdx_model* m) {
  if (m->twolevel) return PDX_OK;
  if (m->mesh.dim != 2) return set_error(PDX_ERR_UNSUPPORTED, "method 8 (two-level BiCGStab) is built for 2D models");
  const int N = m->mesh.n_node;
  const int64_t n = m->setup.n_eq;
  const std::vector<double>& X = m->mesh.X;
  std::vector<int> eq_node((size_t)n, 0);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < 2; i++) {
      const int e = m->setup.eq[(size_t)k * 2 + i];
      if (e >= 0) eq_node[e] = k;
    }
  double lo[2] = {1e300, 1e300}, hi[2] = {-1e300, -1e300}, reach[2] = {0.0, 0.0};
  for (int k = 0; k < N; k++)
    for (int a = 0; a < 2; a++) {
      lo[a] = std::min(lo[a], X[(size_t)k * 3 + a]);
      hi[a] = std::max(hi[a], X[(size_t)k * 3 + a]);
    }
  const std::vector<int64_t>& ia = m->setup.csr_ia;
  const std::vector<int64_t>& ja = m->setup.csr_ja;
  for (int64_t r = 0; r < n && (size_t)r + 1 < ia.size(); r++) {
    const int kr = eq_node[r];
    for (int64_t p = ia[r]; p < ia[r + 1]; p++) {
      const int kc = eq_node[ja[p]];
      for (int a = 0; a < 2; a++) reach[a] = std::max(reach[a], std::fabs(X[(size_t)kr * 3 + a] - X[(size_t)kc * 3 + a]));
    }
  }
  int cells[3] = {1, 1, 0};
  for (int a = 0; a < 2; a++) {
    const double len = hi[a] - lo[a];
    if (len > 0 && reach[a] > 0)
      cells[a] = std::max(1, std::min(kTwoLevelCells, (int)std::floor(len / (1.001 * reach[a]))));
  }
  std::vector<int> pidx, rptr, ridx;
  std::vector<float> pw, rw, aw;
  int nc = 0, np = 0, cells_out[3] = {0, 0, 0};
  build_coarse(m, cells, pidx, pw, rptr, ridx, rw, aw, nc, np, cells_out);
  std::vector<int> ecell((size_t)n, 0);
  for (int64_t e = 0; e < n; e++) {
    const int q = pidx[(size_t)e * 4];   // corner 0: the cell's lower-left coarse node and the component
    const int node = q >> 1;
    ecell[e] = (node % (cells_out[0] + 1)) | ((node / (cells_out[0] + 1)) << 12) | ((q & 1) << 24);
  }
  TwoLevelHost* T = new TwoLevelHost();
  m->twolevel = T;
  for (int a = 0; a < 2; a++) T->cell_len[a] = (hi[a] - lo[a]) / std::max(1, cells_out[a]);
  TwoLevelDev& t = T->dev;
  cudaStream_t s = m->stream;
  t.nc = nc;
  t.nxn = cells_out[0] + 1;
  t.nyn = cells_out[1] + 1;
  t.n = n;
  t.pidx = dev_upload(T->buf, pidx, s);
  t.pw = dev_upload(T->buf, pw, s);
  t.ecell = dev_upload(T->buf, ecell, s);
  t.rptr = dev_upload(T->buf, rptr, s);
  t.ridx = dev_upload(T->buf, ridx, s);
  t.rw = dev_upload(T->buf, rw, s);
  t.B = T->buf.alloc<double>((size_t)n * 32);
  t.M = T->buf.alloc<double>((size_t)nc * 2 * nc);
  t.colk = T->buf.alloc<double>(nc);
  t.colbuf = T->buf.alloc<double>(2 * (size_t)nc);
  t.diag0 = T->buf.alloc<double>(nc);
  t.rpiv = T->buf.alloc<double>(2);
  t.rc = T->buf.alloc<double>(nc);
  t.yc = T->buf.alloc<double>(nc);
  t.ok = T->buf.alloc<int>(1);
  t.hash = T->buf.alloc<unsigned long long>(1);
  const pdx_status st = cuda_check(cudaStreamSynchronize(s), "two-level set-up");   // host arrays leave scope
  if (st || !t.pidx || !t.pw || !t.ecell || !t.rptr || !t.ridx || !t.rw || !t.B || !t.M || !t.colk || !t.colbuf || !t.diag0 || !t.rpiv || !t.rc || !t.yc || !t.ok || !t.hash) {
    twolevel_destroy(m);
    return st ? st : set_error(PDX_ERR_CUDA, "two-level set-up: device allocation failed");
  }
  return PDX_OK;
}

void twolevel_destroy(pdx_model* m) {
  if (!m->twolevel) return;
  if (m->twolevel->dev.gj) cudaGraphExecDestroy(m->twolevel->dev.gj);
  m->twolevel->buf.free_all();
  delete m->twolevel;
  m->twolevel = nullptr;
}

void learned_destroy(pdx_model* m) {
  if (!m->learned) return;
  m->learned->buf.free_all();
  delete m->learned;
  m->learned = nullptr;
}

cudaError_t Learned::add(const double* r, double* z, cudaStream_t s) {
  cudaError_t e = coarse_restrict(cs, false, r, rc, s);
  if (e == cudaSuccess) {
    if (net.wi) {
      e = net.infer_block(rc, sigma, y, scale, s);
    } else {
      e = coarse_normalize(cs.nc, rc, x16, sigma, scale, s);
      if (e == cudaSuccess) e = net.infer(x16, y, s);
    }
  }
  if (e == cudaSuccess) e = coarse_prolong_add(cs, y, scale, z, s);
  return e;
}

}  // namespace pdx

using namespace pdx;

#define NEED_DEV(m)                                                                      \
  do {                                                                                   \
    if (!(m)) return set_error(PDX_ERR_INVALID, "null model");                           \
    if (!(m)->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device"); \
    cudaSetDevice((m)->device);                                                          \
  } while (0)

extern "C" {

pdx_status pdx_learned_setup(pdx_model* m, int cx, int cy, int cz, int hidden, uint64_t seed, int max_samples) {
  NEED_DEV(m);
  if (hidden <= 0 || max_samples <= 0) return set_error(PDX_ERR_INVALID, "hidden width and sample count must be > 0");
  learned_destroy(m);
  Learned* L = new Learned();
  m->learned = L;
  cudaStream_t s = m->stream;
  std::vector<int> pidx, rptr, ridx;
  std::vector<float> pw, rw, aw;
  const int cin[3] = {cx, cy, cz};
  int nc = 0, np = 0;
  build_coarse(m, cin, pidx, pw, rptr, ridx, rw, aw, nc, np, L->cs.cells);
  CoarseSpace& cs = L->cs;
  cs.dim = m->mesh.dim;
  cs.nc = nc;
  cs.n = m->setup.n_eq;
  cs.np = np;
  cs.pidx = dev_upload(L->buf, pidx, s);
  cs.pw = dev_upload(L->buf, pw, s);
  cs.rptr = dev_upload(L->buf, rptr, s);
  cs.ridx = dev_upload(L->buf, ridx, s);
  cs.rw = dev_upload(L->buf, rw, s);
  cs.aw = dev_upload(L->buf, aw, s);
  // network: Xavier-uniform weights from the seed, zero biases
  Mlp& net = L->net;
  net.nin = nc;
  net.nout = nc;
  net.H = hidden;
  net.Bmax = 64;
  const int64_t npar = net.n_params();
  std::vector<float> w0((size_t)npar, 0.f);
  {
    std::mt19937_64 rng(seed);
    float *W1, *b1, *W2, *b2, *W3, *b3;
    net.param_views(w0.data(), &W1, &b1, &W2, &b2, &W3, &b3);
    auto fill = [&](float* p, int rows, int cols) {
      const float a = std::sqrt(6.f / (float)(rows + cols));
      std::uniform_real_distribution<float> u(-a, a);
      for (int64_t i = 0; i < (int64_t)rows * cols; i++) p[i] = u(rng);
    };
    fill(W1, hidden, nc);
    fill(W2, hidden, hidden);
    fill(W3, nc, hidden);
  }
  net.w = dev_upload(L->buf, w0, s);
  net.w16 = L->buf.alloc<__nv_bfloat16>(npar);
  if (net.block_infer_ok()) net.wi = L->buf.alloc<__nv_bfloat16>(net.n_infer());
  net.g = L->buf.alloc<float>(npar);
  net.m1 = L->buf.alloc<float>(npar);
  net.m2 = L->buf.alloc<float>(npar);
  const int B = net.Bmax;
  net.Z1 = L->buf.alloc<float>((size_t)B * hidden);
  net.Z2 = L->buf.alloc<float>((size_t)B * hidden);
  net.Y = L->buf.alloc<float>((size_t)B * nc);
  net.dY = L->buf.alloc<float>((size_t)B * nc);
  net.dH = L->buf.alloc<float>((size_t)B * hidden);
  net.dZ = L->buf.alloc<float>((size_t)B * hidden);
  net.H1 = L->buf.alloc<__nv_bfloat16>((size_t)B * hidden);
  net.H2 = L->buf.alloc<__nv_bfloat16>((size_t)B * hidden);
  net.dY16 = L->buf.alloc<__nv_bfloat16>((size_t)B * nc);
  net.dZ16 = L->buf.alloc<__nv_bfloat16>((size_t)B * hidden);
  net.loss_row = L->buf.alloc<float>(B);
  net.loss = L->buf.alloc<float>(1);
  {
    const int64_t wf = gemm_work_floats(B, nc, hidden, nc);
    if (wf > 0) net.work = L->buf.alloc<float>(wf);
  }
  L->rc = L->buf.alloc<float>(nc);
  L->x16 = L->buf.alloc<__nv_bfloat16>(nc);
  L->y = L->buf.alloc<float>(nc);
  L->scale = L->buf.alloc<float>(1);
  L->ax = L->buf.alloc<float>(nc);
  L->cap = max_samples;
  L->S_r = L->buf.alloc<float>((size_t)max_samples * nc);
  L->S_x = L->buf.alloc<float>((size_t)max_samples * nc);
  L->S_scale = L->buf.alloc<float>(max_samples);
  L->bidx = L->buf.alloc<int>(B);
  L->Xb = L->buf.alloc<__nv_bfloat16>((size_t)B * nc);
  L->Tb = L->buf.alloc<float>((size_t)B * nc);
  L->Wb = L->buf.alloc<float>(B);
  for (void* p : L->buf.ptrs)
    if (!p) return set_error(PDX_ERR_CUDA, "device allocation failed (learned preconditioner)");
  cudaMemsetAsync(net.m1, 0, npar * 4, s);
  cudaMemsetAsync(net.m2, 0, npar * 4, s);
  pdx_status st = cuda_check(net.sync_bf16(s), "network set-up");
  if (st) return st;
  return cuda_check(cudaStreamSynchronize(s), "learned set-up");
}

int64_t pdx_learned_samples(const pdx_model* m) { return m && m->learned ? m->learned->count : 0; }

int pdx_learned_active(const pdx_model* m) {
  return m && m->learned && m->learned->trained && !m->learned->disabled ? 1 : 0;
}

pdx_status pdx_learned_options(pdx_model* m, int trunc, int stall_window) {
  if (!m || !m->learned) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  if (trunc < 1 || trunc > 32 || stall_window < 0) return set_error(PDX_ERR_INVALID, "trunc in 1..32, stall window >= 0");
  m->learned->trunc = trunc;
  m->learned->stall_window = stall_window;
  return PDX_OK;
}

pdx_status pdx_learned_probe(pdx_model* m, int nprobe, uint64_t seed) {
  NEED_DEV(m);
  Learned* L = m->learned;
  if (!L) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  if (!m->newmark_ready || m->steps_done < 1) return set_error(PDX_ERR_INVALID, "run a Newmark step first");
  const int64_t ne = m->setup.n_eq;
  double* b = m->d_tmp_eq[5];
  double* x = m->d_tmp_eq[6];
  for (int p = 0; p < nprobe; p++) {
    pdx_status st = cuda_check(learned_random_rhs(ne, seed + (uint64_t)p * 0x51ed27ull, b, m->stream), "probe rhs");
    if (st) return st;
    cudaMemsetAsync(x, 0, (size_t)ne * 8, m->stream);
    KrylovResult kr;
    st = plain_solve(m, b, x, L, &kr);
    if (st) return st;
  }
  return cuda_check(cudaStreamSynchronize(m->stream), "probe solves");
}

pdx_status pdx_learned_pairs(const pdx_model* m, float* r, float* e, int64_t* count, int* nc) {
  if (!m || !m->learned) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  const Learned* L = m->learned;
  if (count) *count = L->count;
  if (nc) *nc = L->cs.nc;
  const size_t bytes = (size_t)L->count * L->cs.nc * 4;
  if (r) cudaMemcpyAsync(r, L->S_r, bytes, cudaMemcpyDeviceToHost, m->stream);
  if (e) cudaMemcpyAsync(e, L->S_x, bytes, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "training pairs");
}

pdx_status pdx_learned_train(pdx_model* m, int epochs, float lr, uint64_t seed, float* final_loss) {
  NEED_DEV(m);
  Learned* L = m->learned;
  if (!L) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  if (L->count < 2) return set_error(PDX_ERR_INVALID, "not enough training pairs collected");
  cudaStream_t s = m->stream;
  const int nc = L->cs.nc, n = L->count, B = L->net.Bmax;
  // per-sample |P^T r| and the target scale sigma = median |e_c| / |P^T r|
  pdx_status st = cuda_check(learned_norms(n, nc, L->S_r, L->S_scale, s), "norms");
  if (st) return st;
  std::vector<float> nr(n), ne(n);
  float* tmp = nullptr;
  cudaMallocAsync(&tmp, n * sizeof(float), s);
  learned_norms(n, nc, L->S_x, tmp, s);
  cudaMemcpyAsync(nr.data(), L->S_scale, n * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(ne.data(), tmp, n * 4, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(tmp, s);
  st = cuda_check(cudaStreamSynchronize(s), "norms");
  if (st) return st;
  std::vector<float> ratio;
  for (int j = 0; j < n; j++)
    if (nr[j] > 0 && ne[j] > 0) ratio.push_back(ne[j] / nr[j]);
  if (ratio.empty()) return set_error(PDX_ERR_NUMERIC, "training pairs are all zero");
  std::nth_element(ratio.begin(), ratio.begin() + ratio.size() / 2, ratio.end());
  L->sigma = ratio[ratio.size() / 2];
  // every epoch's shuffled order goes to the device at once, and the batch
  // losses are summed there: the loop issues kernels only and synchronises
  // once at the end
  std::mt19937_64 rng(seed);
  std::vector<int> order(n), orders((size_t)epochs * n);
  std::iota(order.begin(), order.end(), 0);
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(order.begin(), order.end(), rng);
    std::copy(order.begin(), order.end(), orders.begin() + (size_t)ep * n);
  }
  int* d_orders = nullptr;
  float* d_loss_sum = nullptr;
  st = cuda_check(cudaMallocAsync(&d_orders, orders.size() * sizeof(int), s), "training orders");
  if (!st) st = cuda_check(cudaMallocAsync(&d_loss_sum, sizeof(float), s), "training loss");
  if (st) return st;
  cudaMemcpyAsync(d_orders, orders.data(), orders.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(d_loss_sum, 0, sizeof(float), s);
  int nbatch = 0;
  for (int ep = 0; ep < epochs && !st; ep++) {
    if (ep == epochs - 1) cudaMemsetAsync(d_loss_sum, 0, sizeof(float), s);
    nbatch = 0;
    for (int i0 = 0; i0 + 1 < n && !st; i0 += B) {
      const int b = std::min(B, n - i0);
      st = cuda_check(learned_stage(b, nc, d_orders + (size_t)ep * n + i0, L->S_r, L->S_x, L->S_scale, L->sigma,
                                    L->Xb, L->Tb, L->Wb, s), "stage");
      if (!st) st = cuda_check(L->net.forward_backward(b, L->Xb, L->Tb, L->Wb, true, s), "forward/backward");
      if (!st) st = cuda_check(L->net.adam_step(lr, s), "Adam");
      if (!st && ep == epochs - 1) st = cuda_check(learned_add_scalar(L->net.loss, d_loss_sum, s), "loss");
      nbatch++;
    }
  }
  float last_sum = 0.f;
  if (!st) cudaMemcpyAsync(&last_sum, d_loss_sum, sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d_orders, s);
  cudaFreeAsync(d_loss_sum, s);
  pdx_status st2 = cuda_check(cudaStreamSynchronize(s), "training");
  if (st) return st;
  if (st2) return st2;
  const float last = nbatch ? last_sum / nbatch : 0.f;
  L->trained = true;
  L->losses = 0;
  L->disabled = false;
  if (final_loss) *final_loss = last;
  return PDX_OK;
}

pdx_status pdx_mlp_params(pdx_model* m, float* get, const float* set, int64_t* count) {
  NEED_DEV(m);
  Learned* L = m->learned;
  if (!L) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  const int64_t npar = L->net.n_params();
  if (count) *count = npar;
  if (set) {
    cudaMemcpyAsync(L->net.w, set, npar * 4, cudaMemcpyHostToDevice, m->stream);
    L->net.sync_bf16(m->stream);
  }
  if (get) cudaMemcpyAsync(get, L->net.w, npar * 4, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "parameters");
}

pdx_status pdx_mlp_loss_grad(pdx_model* m, int batch, const float* x, const float* t, const float* w, float* loss,
                             float* grad) {
  NEED_DEV(m);
  Learned* L = m->learned;
  if (!L) return set_error(PDX_ERR_INVALID, "pdx_learned_setup first");
  if (batch <= 0 || batch > L->net.Bmax || !x || !t || !w) return set_error(PDX_ERR_INVALID, "bad batch");
  cudaStream_t s = m->stream;
  const int nc = L->cs.nc;
  float* xf = nullptr;
  cudaMallocAsync(&xf, (size_t)batch * nc * 4, s);
  cudaMemcpyAsync(xf, x, (size_t)batch * nc * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(L->Tb, t, (size_t)batch * nc * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(L->Wb, w, (size_t)batch * 4, cudaMemcpyHostToDevice, s);
  learned_stage_raw(batch, nc, xf, L->Xb, s);
  cudaFreeAsync(xf, s);
  pdx_status st = cuda_check(L->net.forward_backward(batch, L->Xb, L->Tb, L->Wb, true, s), "forward/backward");
  if (st) return st;
  if (loss) cudaMemcpyAsync(loss, L->net.loss, 4, cudaMemcpyDeviceToHost, s);
  if (grad) cudaMemcpyAsync(grad, L->net.g, L->net.n_params() * 4, cudaMemcpyDeviceToHost, s);
  return cuda_check(cudaStreamSynchronize(s), "loss/gradient");
}

pdx_status pdx_newmark_init(pdx_model* m) {
  NEED_DEV(m);
  if (!m->batch.empty()) return set_error(PDX_ERR_UNSUPPORTED, "batched models run explicit dynamics only");
  pdx_status st = pdx_explicit_init(m);
  if (st) return st;
  const size_t ne = (size_t)std::max(m->setup.n_eq, 1);
  if (!m->d_vel) m->d_vel = m->buf.alloc<double>(ne);
  if (!m->d_acc) m->d_acc = m->buf.alloc<double>(ne);
  if (!m->d_vel || !m->d_acc) return set_error(PDX_ERR_CUDA, "device allocation failed");
  cudaMemsetAsync(m->d_vel, 0, ne * 8, m->stream);
  cudaMemsetAsync(m->d_acc, 0, ne * 8, m->stream);
  m->cur = 0;
  m->steps_done = 0;
  m->rf_rows = 0;
  m->explicit_run = false;
  m->newmark_ready = true;
  return cuda_check(cudaStreamSynchronize(m->stream), "Newmark init");
}

pdx_status pdx_newmark_step(pdx_model* m, int method, int collect, pdx_solve_info* info) {
  NEED_DEV(m);
  if (!m->newmark_ready) return set_error(PDX_ERR_INVALID, "pdx_newmark_init first");
  if (method < 0 || method > 8) return set_error(PDX_ERR_INVALID, "method must be 0..8");
  const int ne = m->setup.n_eq;
  double* u_all = m->d_u[0];
  double* upred = m->d_u[1];
  double* acc1 = m->d_tmp_eq[3];
  double* ueq = m->d_tmp_eq[4];
  const int n = (int)m->steps_done + 1;
  pdx_status st = cuda_check(launch_newmark_predict(m->view, u_all, m->d_vel, m->d_acc, m->cmd.dt, m->cmd.beta,
                                                    upred, m->stream), "Newmark predictor");
  if (st) return st;
  st = assemble_device(m, 3, upred, n - 1);
  if (st) return st;
  cudaMemcpyAsync(acc1, m->d_acc, (size_t)ne * 8, cudaMemcpyDeviceToDevice, m->stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, m->stream);
  KrylovResult kr;
  st = solve_newmark_system(m, method, collect != 0, acc1, &kr);
  cudaEventRecord(e1, m->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (info) {
    fill_solve_info(info, kr, ms * 1e-3);
  }
  if (!kr.converged)
    return set_error(PDX_ERR_NOCONV, "Newmark solve stopped at relative residual " + std::to_string(kr.rel_residual));
  if (Learned* L = m->learned) {
    if (method == 4) {
      L->plain_its = (L->plain_its * L->plain_n + kr.iterations) / (L->plain_n + 1);
      L->plain_n++;
      if (!collect) {
        L->plain_sec = (L->plain_sec * L->plain_sec_n + ms * 1e-3) / (L->plain_sec_n + 1);
        L->plain_sec_n++;
      }
    } else if (method == 5 && L->trained && !L->disabled) {
      // judged by time where plain solve times are known, else by iterations
      const bool lost = L->plain_sec_n > 0 ? ms * 1e-3 >= L->plain_sec
                                           : (L->plain_n > 0 && kr.iterations >= L->plain_its);
      L->losses = lost ? L->losses + 1 : 0;
      if (L->losses >= 2) L->disabled = true;
    }
  }
  launch_gather_eq(m->view, u_all, ueq, m->stream);
  launch_newmark_update(ne, m->d_vel, m->d_acc, acc1, m->cmd.dt, m->cmd.beta, m->cmd.gamma, ueq, m->d_vel,
                        m->stream);
  launch_scatter_eq(m->view, ueq, u_all, m->stream);
  launch_advance_prescribed(m->view, u_all, m->stream);
  cudaMemcpyAsync(m->d_acc, acc1, (size_t)ne * 8, cudaMemcpyDeviceToDevice, m->stream);
  m->steps_done = n;
  // FC 2 after the step, on the state with the advanced prescribed values
  // (pdsolve.cpp:6249-6261), then the reaction forces
  pdx_status rs = fc2_pass(m);
  if (!rs) rs = rf_record(m, n);
  if (rs) return rs;
  return cuda_check(cudaStreamSynchronize(m->stream), "Newmark step");
}

}  // extern "C"
