// pdx_run: the solver selected by the command file (pdsolve::pdfemSolver,
// pdsolve.cpp:5073-5103), on the GPU, writing the reference's result files.
//   explicit dynamic, lumped mass   pdfemDynamicSolver_CSRformat   :5842-6090
//   Newmark implicit dynamic        pdfemDynamicNewmarkSolver_CSRformat :6092-6290
//   static                          pdfemStaticSolver_CSRformat    :5557-5654
//   quasi-static                    pdfemQuasiStaticSolver_CSRformat :6464-6590
// The direct sparse solves of the reference become Krylov solves judged by
// the true FP64 residual (SOLVE keyword; default BiCGStab, tolerance 1e-8;
// a solve that does not converge falls back to BiCGStab, then GMRES(30)).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "model_impl.h"

namespace pdx {

namespace {

struct HostState {
  std::vector<double> u, sigma, phi;
};

pdx_status fetch(pdx_model* m, const double* d_u, HostState& h) {
  const int N = m->mesh.n_node, D = m->mesh.dim;
  h.u.resize((size_t)N * D);
  h.sigma.resize((size_t)N * 6);
  h.phi.resize(N);
  cudaMemcpyAsync(h.u.data(), d_u, h.u.size() * 8, cudaMemcpyDeviceToHost, m->stream);
  cudaMemcpyAsync(h.sigma.data(), m->d_sigma, h.sigma.size() * 8, cudaMemcpyDeviceToHost, m->stream);
  cudaMemcpyAsync(h.phi.data(), m->d_phi, h.phi.size() * 8, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "state download");
}

std::string out_name(const pdx_model* m, const std::string& dir, const std::string& tag) {
  return dir + "/" + m->mesh.title + "_" + tag + ".vtk";
}

// Result files written on a host thread while the GPU steps on.  The state of
// a save step (u, the nodal stresses and damage already computed on the
// device) is copied into pinned host buffers on the model's stream, so the
// copy is ordered after that step and before the next one overwrites it; the
// thread waits for the copy's event, then formats and writes the files.  Two
// buffer sets alternate, and a set is reused only after its last write ends.
class AsyncWriter {
 public:
  explicit AsyncWriter(pdx_model* m) : m_(m) {
    const size_t N = (size_t)m->mesh.n_node;
    nu_ = N * m->mesh.dim;
    ns_ = N * 6;
    np_ = N;
    for (Slot& s : slot_) {
      if (cudaMallocHost(&s.buf, (nu_ + ns_ + np_) * sizeof(double)) != cudaSuccess) s.buf = nullptr;
      if (cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess) s.ev = nullptr;
    }
  }
  ~AsyncWriter() {
    finish();
    for (Slot& s : slot_) {
      if (s.buf) cudaFreeHost(s.buf);
      if (s.ev) cudaEventDestroy(s.ev);
    }
  }
  pdx_status submit(const double* d_u, const std::string& path) {
    Slot& s = slot_[next_];
    next_ ^= 1;
    if (s.th.joinable()) s.th.join();
    if (!s.buf || !s.ev) return set_error(PDX_ERR_CUDA, "pinned result buffers");
    cudaMemcpyAsync(s.buf, d_u, nu_ * 8, cudaMemcpyDeviceToHost, m_->stream);
    cudaMemcpyAsync(s.buf + nu_, m_->d_sigma, ns_ * 8, cudaMemcpyDeviceToHost, m_->stream);
    cudaMemcpyAsync(s.buf + nu_ + ns_, m_->d_phi, np_ * 8, cudaMemcpyDeviceToHost, m_->stream);
    pdx_status st = cuda_check(cudaEventRecord(s.ev, m_->stream), "result copy");
    if (st) return st;
    const bool binary = m_->cmd.vtk_binary;
    s.th = std::thread([this, &s, path, binary] {
      if (cudaEventSynchronize(s.ev) != cudaSuccess) return;
      const std::vector<double> u(s.buf, s.buf + nu_), sig(s.buf + nu_, s.buf + nu_ + ns_),
          phi(s.buf + nu_ + ns_, s.buf + nu_ + ns_ + np_);
      write_vtk(m_, path, u, sig, phi, binary);
    });
    return PDX_OK;
  }
  void finish() {
    for (Slot& s : slot_)
      if (s.th.joinable()) s.th.join();
  }

 private:
  struct Slot {
    double* buf = nullptr;
    cudaEvent_t ev = nullptr;
    std::thread th;
  };
  pdx_model* m_;
  size_t nu_ = 0, ns_ = 0, np_ = 0;
  Slot slot_[2];
  int next_ = 0;
};

pdx_status solve_device_method(pdx_model* m, const double* b, double* x, int method, KrylovResult* kr) {
  DevCsr A;
  A.n = m->setup.n_eq;
  A.nnz = (int64_t)m->setup.csr_ja.size();
  A.ia = m->d_ia;
  A.ja = m->d_ja;
  A.a = m->d_Kval;
  TwoLevelDev* tl = nullptr;
  if (method == 8) {
    pdx_status st8 = twolevel_prepare(m);
    if (st8) return st8;
    tl = &m->twolevel->dev;
  }
  cudaError_t e = krylov_solve(A, b, x, method, m->cmd.solve_tol, m->cmd.solve_maxit, m->mesh.dim, m->stream, kr, tl);
  pdx_status st = cuda_check(e, "Krylov solve");
  if (st) return st;
  int spent = kr->iterations;   // iterations are summed over the fallbacks
  if (!kr->converged) {
    // BiCGStab as the fallback of a stalled CG on the unsymmetric stiffness
    if (method != 2 && method != 6) {
      e = krylov_solve(A, b, x, 2, m->cmd.solve_tol, m->cmd.solve_maxit, m->mesh.dim, m->stream, kr);
      st = cuda_check(e, "Krylov solve");
      if (st) return st;
      kr->iterations += spent;
      spent = kr->iterations;
    }
    if (!kr->converged && method != 6) {
      // GMRES(30) when BiCGStab does not converge: once a crack has cut a
      // piece loose the stiffness is strongly unsymmetric and indefinite, and
      // BiCGStab's residual grows without bound (the reference's direct
      // solve has no such limit).  GMRES never lets its residual grow; it
      // starts from zero after a non-finite BiCGStab iterate.
      if (!(kr->rel_residual < 1.0)) cudaMemsetAsync(x, 0, (size_t)A.n * 8, m->stream);
      e = krylov_solve(A, b, x, 6, m->cmd.solve_tol, m->cmd.solve_maxit, m->mesh.dim, m->stream, kr);
      st = cuda_check(e, "Krylov solve");
      if (st) return st;
      kr->iterations += spent;
    }
    if (!kr->converged)
      return set_error(PDX_ERR_NOCONV, "Krylov solve stopped at relative residual " + std::to_string(kr->rel_residual));
  }
  return PDX_OK;
}

pdx_status solve_device(pdx_model* m, const double* b, double* x, KrylovResult* kr) {
  return solve_device_method(m, b, x, m->cmd.solve_method, kr);
}

// <title>RF.out: the header and one row per recorded step, formatted as the
// reference's stream is (default 6 significant digits in the dynamic
// solvers, scientific with 4 digits in the quasi-static one)
pdx_status write_rf(pdx_model* m, const std::string& dir, int first_row, bool scientific4) {
  std::ofstream f(dir + "/" + m->mesh.title + "RF.out");
  if (!f) return set_error(PDX_ERR_IO, "cannot write " + m->mesh.title + "RF.out");
  if (scientific4) f << std::left << std::scientific << std::setprecision(4);
  f << "Step\t" << "U\t" << "RFx\t" << "RFy\t" << "RFz\n";
  int64_t n = 0;
  pdx_status st = pdx_reaction_forces(m, nullptr, 0, &n);
  if (st || n == 0) return st;
  std::vector<double> rows((size_t)n * 4);
  st = pdx_reaction_forces(m, rows.data(), n, nullptr);
  if (st) return st;
  for (int64_t r = first_row; r < n; r++)
    f << r << "\t" << rows[r * 4] << "\t" << rows[r * 4 + 1] << "\t" << rows[r * 4 + 2] << "\t" << rows[r * 4 + 3]
      << std::endl;
  return PDX_OK;
}

pdx_status run_explicit(pdx_model* m, const std::string& dir) {
  if (!m->cmd.lumped) return set_error(PDX_ERR_UNSUPPORTED, "explicit dynamics needs LUMPMASS ON");
  pdx_status st = pdx_explicit_init(m);
  if (st) return st;
  st = pdx_explicit_advance(m, 1);   // step 0: u1 = u0 + dt^2/2 a0
  if (st) return st;
  const int nsteps = m->cmd.nsteps, save = std::max(1, m->cmd.save_freq);
  int n = 0;
  AsyncWriter writer(m);
  while (n < nsteps) {
    int next = std::min(nsteps, (n / save + 1) * save);
    st = pdx_explicit_advance(m, next - n);
    if (st) return st;
    n = next;
    st = pdx_get_state(m, nullptr, nullptr, nullptr, nullptr);   // stresses and damage on the device
    if (st) return st;
    st = writer.submit(m->d_u[m->cur], out_name(m, dir, std::to_string(n)));
    if (st) return st;
  }
  writer.finish();
  return write_rf(m, dir, 0, false);
}

pdx_status run_static(pdx_model* m, const std::string& dir) {
  const int N = m->mesh.n_node, D = m->mesh.dim;
  std::vector<double> v(m->prep.u0);
  for (size_t i = 0; i < v.size(); i++)
    if (m->setup.eq[i] >= 0) v[i] = 0.0;
  cudaMemcpyAsync(m->d_u[0], v.data(), v.size() * 8, cudaMemcpyHostToDevice, m->stream);
  pdx_status st = assemble_device(m, 1, m->d_u[0], 0);
  if (st) return st;
  double* x = m->d_tmp_eq[1];
  cudaMemsetAsync(x, 0, (size_t)m->setup.n_eq * 8, m->stream);
  KrylovResult kr;
  st = solve_device(m, m->d_tmp_eq[0], x, &kr);
  if (st) return st;
  launch_scatter_eq(m->view, x, m->d_u[0], m->stream);
  m->cur = 0;
  st = model_stress(m, m->d_u[0], true, true);
  if (st) return st;
  HostState h;
  st = fetch(m, m->d_u[0], h);
  if (st) return st;
  (void)N; (void)D;
  std::printf("static solve: %d iterations, relative residual %.3e\n", kr.iterations, kr.rel_residual);
  if (m->cmd.fail_flag == 1 && m->mesh.dim == 2) {
    // the static solver's failure pass (pdsolve.cpp:5637): SIFs of every
    // crack, printed as the reference prints them with solver flag 1
    st = fc1_pass(m, false);
    if (st) return st;
    for (const auto& f : m->crack_sif) std::printf("KI= %e, KII=%e, Keq=%e\n", f[0], f[1], f[2]);
  }
  write_vtk(m, out_name(m, dir, "static"), h.u, h.sigma, h.phi, m->cmd.vtk_binary);
  return PDX_OK;
}

// One quasi-static increment n, the body of the increment loop of
// pdfemQuasiStaticSolver_CSRformat (pdsolve.cpp:6464-6590): K du = f_ext - K u
// solved by `method` (BiCGStab if it does not converge), u += du, then bond
// failure (FC 3) and the stresses of the new state.  The prescribed DOFs are
// advanced by the caller, by the quasi-static rule of setVaryEssentialBC
// (a varying EBC takes dt * velocity once, from 0, and holds).  With solve_ms, the solve is timed with CUDA events.
pdx_status quasi_increment(pdx_model* m, int n, int method, KrylovResult* kr, float* solve_ms) {
  double* u_all = m->d_u[0];
  const int ne = m->setup.n_eq;
  double* du = m->d_tmp_eq[1];
  double* ueq = m->d_tmp_eq[2];
  // natural BC row: the load steps applied so far (n - 1 unless FC 2 held the load)
  pdx_status st = assemble_device(m, 2, u_all, m->quasi_load);
  if (st) return st;
  cudaMemsetAsync(du, 0, (size_t)ne * 8, m->stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (solve_ms) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, m->stream);
  }
  st = solve_device_method(m, m->d_tmp_eq[0], du, method, kr);
  if (solve_ms) {
    cudaEventRecord(e1, m->stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(solve_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (st) return st;
  launch_gather_eq(m->view, u_all, ueq, m->stream);
  launch_axpby_scale(ne, du, 1.0, ueq, 1.0, m->stream);
  launch_scatter_eq(m->view, ueq, u_all, m->stream);
  m->steps_done = n;
  if (m->cmd.fail_flag == 1 && m->mesh.dim == 2) {
    // FC 1: stresses, then SIFs, crack growth and the PD-region and bond
    // updates (which may re-derive the device model), then damage
    st = model_stress(m, u_all, true, false);
    if (!st) st = fc1_pass(m, true);
    if (st) return st;
    return model_stress(m, m->d_u[0], false, true);
  }
  if (m->fc2) {
    // FC 2 with the cut count and the largest sigma1 for the load ratio
    st = fc2_pass(m, true);
    if (st) return st;
    return model_stress(m, u_all, false, true);
  }
  if (m->view.fail3) {
    st = model_stress(m, u_all, true, false);
    if (st) return st;
    if (m->mixed) launch_shadow(m->view, u_all, m->d_uf[0], m->stream);
    st = explicit_step_launch(m, 2, n);
    if (st) return st;
    return model_stress(m, u_all, false, true);
  }
  return model_stress(m, u_all, true, true);
}

// The load step after an increment (the end of the reference's increment
// loop, pdsolve.cpp:6570-6578): with FC 2 the load advances only if the
// increment cut no bond, scaled by the ratio rati = 1.001 sigma_ult / max
// sigma1 (failureProcess :6615-6628); otherwise rati = 1 (a varying EBC
// takes dt * velocity once, from 0, and holds).
pdx_status quasi_advance(pdx_model* m) {
  double* u_all = m->d_u[0];
  if (m->cmd.fail_flag == 1 && m->d_ebc_vel) {
    // FC 1 (failureProcess :6601-6614): the load holds while a tip moved,
    // otherwise rati = 1.001 K_Ic / Keq of the last crack
    if (m->fc1_moved) return PDX_OK;
    const double kic = m->mesh.KIc, mx = m->fc1_keq;
    const double rati = std::fabs(mx) < 1e-20 * kic ? 1.0 : 1.001 * kic / mx;
    m->quasi_load++;
    return cuda_check(launch_advance_prescribed_ratio(m->view, u_all, m->d_ebc_vel, m->cmd.dt, rati, m->stream),
                      "prescribed values");
  }
  if (m->fc2) {
    if (m->fc2_kept > 0) return PDX_OK;   // bonds were cut: the load holds
    const double sig = m->mesh.sigult, mx = m->fc2_max;
    const double rati = std::fabs(mx) < 1e-20 * sig ? 1.0 : 1.001 * sig / mx;
    m->quasi_load++;
    return cuda_check(launch_advance_prescribed_ratio(m->view, u_all, m->d_ebc_vel, m->cmd.dt, rati, m->stream),
                      "prescribed values");
  }
  m->quasi_load++;
  return cuda_check(launch_advance_prescribed_quasi(m->view, u_all, m->stream), "prescribed values");
}

pdx_status run_quasi(pdx_model* m, const std::string& dir) {
  pdx_status st = fc1_reset(m);
  if (!st) st = pdx_explicit_init(m);   // u = initial DOF values, bond states reset
  m->explicit_run = false;
  if (st) return st;
  m->cur = 0;
  m->quasi_load = 0;
  // <title>_cp.out: the crack path of FC 1, one row per increment with each
  // crack's tip and the last crack's KI, KII and Keq, as the reference writes
  // it (pdsolve.cpp:6496-6504, 7481-7489)
  std::ofstream cp(dir + "/" + m->mesh.title + "_cp.out");
  cp << std::left << std::scientific << std::setprecision(4);
  const bool fc1 = m->cmd.fail_flag == 1 && m->mesh.dim == 2;
  if (fc1) cp << "crack ID\t tip_x\t tip_y \t KI \tKII \t Keq\n";
  AsyncWriter writer(m);
  for (int n = 1; n <= m->cmd.nsteps; n++) {
    KrylovResult kr;
    st = quasi_increment(m, n, m->cmd.solve_method, &kr, nullptr);
    if (!st) st = rf_record(m, n);
    if (st) return st;
    if (fc1 && !m->cracks.empty()) {
      const auto& last = m->crack_sif.back();
      for (size_t k = 0; k < m->cracks.size(); k++)
        cp << k << "\t" << m->cracks[k][3] << "\t" << m->cracks[k][4] << "\t" << last[0] << "\t" << last[1] << "\t"
           << last[2] << " \"***\"\t";
      cp << std::endl;
    }
    if (n % std::max(1, m->cmd.save_freq) == 0 || n == m->cmd.nsteps || n == 1) {
      st = writer.submit(m->d_u[0], out_name(m, dir, std::to_string(n)));
      if (st) return st;
    }
    st = quasi_advance(m);
    if (st) return st;
  }
  st = cuda_check(cudaStreamSynchronize(m->stream), "quasi-static");
  if (st) return st;
  writer.finish();
  return write_rf(m, dir, 1, true);
}

pdx_status run_newmark(pdx_model* m, const std::string& dir) {
  pdx_status st = pdx_explicit_init(m);
  if (st) return st;
  m->explicit_run = false;
  double* u_all = m->d_u[0];
  m->cur = 0;
  const int ne = m->setup.n_eq;
  double* vel = m->d_tmp_eq[1];
  double* acc = m->d_tmp_eq[2];
  double* acc1 = m->d_tmp_eq[3];
  double* ueq = m->d_tmp_eq[4];
  double* upred = m->d_u[1];
  cudaMemsetAsync(vel, 0, (size_t)ne * 8, m->stream);
  cudaMemsetAsync(acc, 0, (size_t)ne * 8, m->stream);
  AsyncWriter writer(m);
  for (int n = 1; n <= m->cmd.nsteps; n++) {
    st = cuda_check(launch_newmark_predict(m->view, u_all, vel, acc, m->cmd.dt, m->cmd.beta, upred, m->stream),
                    "Newmark predictor");
    if (st) return st;
    st = assemble_device(m, 3, upred, n - 1);
    if (st) return st;
    cudaMemcpyAsync(acc1, acc, (size_t)ne * 8, cudaMemcpyDeviceToDevice, m->stream);
    KrylovResult kr;
    st = solve_device(m, m->d_tmp_eq[0], acc1, &kr);
    if (st) return st;
    launch_gather_eq(m->view, u_all, ueq, m->stream);
    launch_newmark_update(ne, vel, acc, acc1, m->cmd.dt, m->cmd.beta, m->cmd.gamma, ueq, vel, m->stream);
    launch_scatter_eq(m->view, ueq, u_all, m->stream);
    launch_advance_prescribed(m->view, u_all, m->stream);
    std::swap(acc, acc1);
    m->steps_done = n;
    st = fc2_pass(m);
    if (!st) st = rf_record(m, n);
    if (st) return st;
    if (n % std::max(1, m->cmd.save_freq) == 0 || n == m->cmd.nsteps) {
      st = model_stress(m, u_all, true, true);
      if (st) return st;
      st = writer.submit(u_all, out_name(m, dir, std::to_string(n)));
      if (st) return st;
    }
  }
  st = cuda_check(cudaStreamSynchronize(m->stream), "Newmark");
  if (st) return st;
  writer.finish();
  return write_rf(m, dir, 1, false);
}

}  // namespace

}  // namespace pdx

using namespace pdx;

extern "C" pdx_status pdx_run(pdx_model* m, const char* results_dir) {
  if (!m || !results_dir) return set_error(PDX_ERR_INVALID, "null argument");
  if (!m->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device");
  if (!m->batch.empty())
    return set_error(PDX_ERR_UNSUPPORTED, "a batched model is stepped with pdx_explicit_advance, not pdx_run");
  cudaSetDevice(m->device);
  mkdir(results_dir, 0755);
  const std::string dir(results_dir);
  // FC 2 breaks bonds after every explicit or Newmark step and every
  // quasi-static increment (with its load-ratio control), as the reference
  // does; FC 1 grows cracks after every quasi-static increment and reports
  // the SIFs of a static solve (in dynamic runs the reference only moves its
  // tip records, without breaking a bond: not offered)
  if (m->cmd.solver == 0 && m->cmd.fail_flag == 1)
    return set_error(PDX_ERR_UNSUPPORTED, "failure criterion FC 1 runs with the static and quasi-static solvers");
  switch (m->cmd.solver) {
    case 0: return m->cmd.newmark ? run_newmark(m, dir) : run_explicit(m, dir);
    case 1: return run_static(m, dir);
    case 2: return run_quasi(m, dir);
    default: return set_error(PDX_ERR_PARSE, "solver flag is wrong");
  }
}

extern "C" pdx_status pdx_quasi_init(pdx_model* m) {
  if (!m) return set_error(PDX_ERR_INVALID, "null model");
  if (!m->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device");
  if (!m->batch.empty()) return set_error(PDX_ERR_UNSUPPORTED, "quasi-static increments take one specimen");
  cudaSetDevice(m->device);
  pdx_status st = fc1_reset(m);
  if (!st) st = pdx_explicit_init(m);
  if (st) return st;
  m->cur = 0;
  m->steps_done = 0;
  m->quasi_load = 0;
  m->explicit_run = false;
  return PDX_OK;
}

extern "C" pdx_status pdx_quasi_step(pdx_model* m, int method, pdx_solve_info* info) {
  if (!m) return set_error(PDX_ERR_INVALID, "null model");
  if (!m->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device");
  if (!m->batch.empty()) return set_error(PDX_ERR_UNSUPPORTED, "quasi-static increments take one specimen");
  if (method < 0 || (method > 3 && method < 6) || method > 8)
    return set_error(PDX_ERR_INVALID, "method must be 0..3 or 6..8");
  cudaSetDevice(m->device);
  KrylovResult kr;
  float ms = 0.f;
  pdx_status st = quasi_increment(m, (int)m->steps_done + 1, method, &kr, &ms);
  if (!st) st = rf_record(m, m->steps_done);
  fill_solve_info(info, kr, ms * 1e-3);
  if (st) return st;
  st = quasi_advance(m);
  if (st) return st;
  return cuda_check(cudaStreamSynchronize(m->stream), "quasi-static increment");
}
