// C ABI (include/pdx.h): model lifecycle, upload, PDLSM coefficient build,
// internal force, explicit stepping, state export, CSR assembly, sparse solve.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "model_impl.h"

namespace pdx {

const int kEqTemps = 8;

namespace {
thread_local std::string g_err;

template <typename T>
T* upload(pdx_model* m, const std::vector<T>& h) {
  T* d = m->buf.alloc<T>(h.size());
  if (d && !h.empty()) cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, m->stream);
  return d;
}

int nv_of(int dim) { return dim == 2 ? 3 : 6; }

std::vector<float> to_f32(const std::vector<double>& v) {
  std::vector<float> r(v.size());
  for (size_t i = 0; i < v.size(); i++) r[i] = (float)v[i];
  return r;
}

// NBC value after r increments, r = 0..nsteps+1 (rows of the table)
std::vector<double> nbc_table(const pdx_model* m, int rows) {
  const auto& nb = m->mesh.nbcs;
  std::vector<double> t((size_t)rows * nb.size(), 0.0);
  for (size_t b = 0; b < nb.size(); b++) {
    double v = nb[b].value;
    for (int r = 0; r < rows; r++) {
      t[(size_t)r * nb.size() + b] = v;
      if (nb[b].varying) v = v + m->cmd.dt * nb[b].velocity;
    }
  }
  return t;
}

}  // namespace

pdx_status set_error(pdx_status code, const std::string& msg) {
  g_err = msg;
  return code;
}

pdx_status cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PDX_OK;
  return set_error(PDX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static pdx_status upload_model(pdx_model* m) {
  const Setup& s = m->setup;
  const Prepared& p = m->prep;
  const Mesh& me = m->mesh;
  const int D = me.dim, N = me.n_node;
  DevView& v = m->view;
  v = DevView{};
  v.dim = D;
  v.n_node = N;
  v.n_fam = (int)s.fam_node.size();
  v.n_feonly = (int)p.feonly.size();
  v.n_eq = s.n_eq;
  v.n_bond = (int64_t)p.nbr.size();
  v.n_corr_bond = (int)p.n_corr;
  v.X = upload(m, me.X);
  std::vector<float4> xf(N);
  for (int k = 0; k < N; k++)
    xf[k] = make_float4((float)me.X[3 * k], (float)me.X[3 * k + 1], (float)me.X[3 * k + 2], 0.f);
  v.Xf = upload(m, xf);
  v.eq = upload(m, s.eq);
  v.mass = upload(m, p.mass_node);
  v.bcflag = upload(m, p.bcflag);
  v.dtv = upload(m, p.dtv);
  v.fam_node = upload(m, s.fam_node);
  v.fam_ptr = upload(m, p.fam_ptr);
  v.fam_order = upload(m, p.fam_order);
  v.fam_corr = upload(m, p.fam_corr);
  m->d_intact = upload(m, p.fam_intact);
  v.fam_intact = m->d_intact;
  v.feonly_node = upload(m, p.feonly);
  v.nbr = upload(m, p.nbr);
  m->d_state = upload(m, p.state_bits);
  v.state = m->d_state;
  const int NC = D == 2 ? 3 : 6;
  double* coef64 = m->buf.alloc<double>((size_t)NC * v.n_bond);
  float* coef32 = m->buf.alloc<float>((size_t)NC * v.n_bond);
  double* corr64 = m->buf.alloc<double>((size_t)D * D * std::max<int64_t>(p.n_corr, 1));
  float* corr32 = m->buf.alloc<float>((size_t)(D == 2 ? 4 : 8) * std::max<int64_t>(p.n_corr, 1));
  float* corr32_last = m->buf.alloc<float>((size_t)std::max<int64_t>(p.n_corr, 1));
  double* cvec = m->buf.alloc<double>((size_t)D * v.n_bond);
  v.coef64 = coef64; v.coef32 = coef32; v.corr64 = corr64; v.corr32 = corr32; v.cvec = cvec;
  v.corr32_last = corr32_last;
  v.fe_conn = upload(m, p.fe_conn);
  v.fe_cls = upload(m, p.fe_cls);
  v.ke64 = upload(m, p.ke);
  v.ke32 = upload(m, to_f32(p.ke));
  m->d_me = upload(m, p.me);
  v.fe_adj_ptr = upload(m, p.fe_adj_ptr);
  v.fe_adj = upload(m, p.fe_adj);
  if (p.n_st_cls > 0) {
    v.st_cls = upload(m, p.st_cls);
    if (p.st_use_delta) {
      v.st_dcls = upload(m, p.st_dcls);
      v.st_delta = upload(m, p.st_delta);
    } else {
      v.st_nbr = upload(m, p.st_nbr);
    }
    v.st_blk64 = upload(m, p.st_blk);
    const int dd = me.dim * me.dim, w = me.dim == 3 ? 12 : 4;
    std::vector<float> b32(p.st_blk.size() / dd * w, 0.f);
    for (size_t i = 0; i < p.st_blk.size() / dd; i++)
      for (int e = 0; e < dd; e++) b32[i * w + e] = (float)p.st_blk[i * dd + e];
    v.st_blk32 = upload(m, b32);
  }
  v.n_tiles = p.n_tiles;
  if (p.n_tiles > 0) {
    v.tile_rows = reinterpret_cast<const int2*>(upload(m, p.tile_rows));
    v.tile_cls = upload(m, p.tile_cls);
    v.lat_blk = upload(m, p.lat_blk);
    v.n_rest = (int)p.fe_rest.size();
    if (v.n_rest) v.fe_rest = upload(m, p.fe_rest);
  }
  v.n_nbc = (int)me.nbcs.size();
  if (v.n_nbc) {
    v.ext_ptr = upload(m, p.ext_ptr);
    v.ext_nbc = upload(m, p.ext_nbc);
    v.ext_f = upload(m, p.ext_f);
    m->d_nbcval = upload(m, nbc_table(m, m->cmd.nsteps + 2));
  }
  v.s0 = m->cmd.s0;
  v.s0_pert = m->cmd.s0_pert;
  v.s0_seed = m->cmd.s0_seed;
  v.s0_seed32 = (uint32_t)(m->cmd.s0_seed ^ (m->cmd.s0_seed >> 32));
  v.fam_brk = upload(m, p.fam_brk);
  v.fam_s0 = upload(m, p.fam_s0);
  v.fam_s0f = upload(m, to_f32(p.fam_s0));
  v.dt2m = upload(m, p.dt2m);
  v.dt2m_f = upload(m, to_f32(p.dt2m));
  v.fail3 = m->cmd.fail_flag == 3 ? 1 : 0;
  if (m->batch.empty()) {
    m->d_D = upload(m, p.D);
    m->d_mat_nu = upload(m, std::vector<double>{me.nu});
  } else {
    m->d_D = upload(m, m->mat_D);
    m->d_mat_nu = upload(m, m->mat_nu);
    m->d_node_mat = upload(m, m->node_mat);
  }
  m->d_bgp = upload(m, p.bgp);
  m->d_L = upload(m, p.L);
  m->d_fam_cdv = upload(m, s.fam_cdv);
  if (!s.csr_ia.empty()) {   // (batched models have no CSR pattern)
    m->d_ia = upload(m, s.csr_ia);
    std::vector<int> ja32(s.csr_ja.begin(), s.csr_ja.end());
    m->d_ja = upload(m, ja32);
    m->d_rel_bond = upload(m, p.rel_bond);
    m->d_rel_self = upload(m, p.rel_self);
    m->d_rel_fe = upload(m, p.rel_fe);
  }
  for (int i = 0; i < 2; i++) {
    m->d_u[i] = m->buf.alloc<double>((size_t)N * D);
    m->d_uf[i] = m->buf.alloc<float4>((size_t)2 * N);
  }
  m->d_brec = m->buf.alloc<float4>((size_t)(D == 3 ? 2 : 1) * std::max<int64_t>(v.n_bond, 1));
  {
    const int nd = (D == 2 ? 4 : 8) * D;
    const size_t floats = (size_t)p.n_cls * nd * nd;
    m->ke_smem = floats * sizeof(float) <= 48 * 1024 ? (int)floats : 0;
  }
  m->d_sigma = m->buf.alloc<double>((size_t)N * 6);
  m->d_phi = m->buf.alloc<double>((size_t)N);
  m->d_tmp_all = m->buf.alloc<double>((size_t)N * D);
  for (int i = 0; i < kEqTemps; i++) m->d_tmp_eq[i] = m->buf.alloc<double>((size_t)std::max(s.n_eq, 1));
  m->d_Kval = m->buf.alloc<double>((size_t)std::max<int64_t>((int64_t)s.csr_ja.size(), 1));
  // FC 2 (2D explicit): the families of each block's nodes, in the block's
  // node order, and room for one candidate per bond
  m->fc2 = m->cmd.fail_flag == 2 && D == 2 && m->batch.empty() && v.n_fam > 0;
  if (m->fc2) {
    const int nbx = s.nblocks[0], nby = s.nblocks[1];
    std::vector<int> bptr(1, 0), bfam;
    for (int b = 0; b < nbx * nby; b++) {
      if (b < (int)s.block_nodes.size())
        for (int node : s.block_nodes[b])
          if (s.fam_of_node[node] >= 0) bfam.push_back(s.fam_of_node[node]);
      bptr.push_back((int)bfam.size());
    }
    if (bfam.empty()) bfam.push_back(0);
    m->d_fc2_blk_ptr = upload(m, bptr);
    m->d_fc2_blk_fam = upload(m, bfam);
    m->fc2_cap = (int)std::max<int64_t>(v.n_bond, 1);
    m->d_fc2_val = m->buf.alloc<double>(m->fc2_cap);
    m->d_fc2_bond = m->buf.alloc<int>(m->fc2_cap);
    m->d_fc2_fam = m->buf.alloc<int>(m->fc2_cap);
    m->d_fc2_count = m->buf.alloc<int>(1);
    m->d_fc2_max = m->buf.alloc<double>(1);
  }
  // the varying EBCs' velocities, for the load-ratio step of FC 1 and FC 2
  // quasi-static runs
  if (m->fc2 || (m->cmd.fail_flag == 1 && D == 2 && m->batch.empty())) {
    std::vector<double> vel((size_t)N * 3, 0.0);
    for (const EssentialBC& b : me.ebcs)
      if (b.varying)
        for (int node : b.nodes) vel[(size_t)node * 3 + b.dof] = b.velocity;
    m->d_ebc_vel = upload(m, vel);
  }
  // reaction forces (setReacForcNode, datModel.cpp:664-735): the nodes of the
  // RF essential BCs, every element with one of them (in element order) with
  // its stiffness, and a mask of its RF nodes
  if (!m->cmd.rf_ids.empty() && m->batch.empty()) {
    std::vector<int> rfn;
    for (int id : m->cmd.rf_ids)
      if (id >= 0 && id < (int)me.ebcs.size()) rfn.insert(rfn.end(), me.ebcs[id].nodes.begin(), me.ebcs[id].nodes.end());
    std::sort(rfn.begin(), rfn.end());
    rfn.erase(std::unique(rfn.begin(), rfn.end()), rfn.end());
    const int nen = D == 2 ? 4 : 8, nd = nen * D;
    std::vector<int> conn, mask;
    std::vector<double> ke;
    for (int e = 0; e < me.n_elem && !rfn.empty(); e++) {
      int mk = 0;
      for (int a = 0; a < me.elem_nn[e]; a++)
        if (std::binary_search(rfn.begin(), rfn.end(), me.conn[(size_t)e * 8 + a])) mk |= 1 << a;
      if (!mk) continue;
      // a triangle takes the 4-node layout with its third node repeated
      const bool tri = me.elem_nn[e] == 3;
      double xN[8][3];
      for (int a = 0; a < nen; a++) {
        const int node = me.conn[(size_t)e * 8 + (tri && a == 3 ? 2 : a)];
        conn.push_back(node);
        for (int c = 0; c < 3; c++) xN[a][c] = me.X[(size_t)node * 3 + c];
      }
      std::vector<double> K((size_t)nd * nd);
      if (D == 2 && tri) ke_tri3(xN, p.D.data(), K.data());
      else if (D == 2) ke_quad4(xN, p.D.data(), K.data());
      else ke_hex8(xN, p.D.data(), K.data());
      ke.insert(ke.end(), K.begin(), K.end());
      mask.push_back(mk);
    }
    m->rf_n_el = (int)mask.size();
    const int id0 = m->cmd.rf_ids[0];
    if (id0 >= 0 && id0 < (int)me.ebcs.size() && !me.ebcs[id0].nodes.empty())
      m->rf_uc_index = (int64_t)me.ebcs[id0].nodes[0] * D + me.ebcs[id0].dof;
    m->rf = true;
    m->rf_cap = (int64_t)m->cmd.nsteps + 2;
    m->d_rf_hist = m->buf.alloc<double>((size_t)m->rf_cap * 4);
    cudaMemsetAsync(m->d_rf_hist, 0, (size_t)m->rf_cap * 4 * 8, m->stream);
    if (m->rf_n_el > 0) {
      m->d_rf_conn = upload(m, conn);
      m->d_rf_ke = upload(m, ke);
      m->d_rf_mask = upload(m, mask);
      m->d_rf_part = m->buf.alloc<double>((size_t)m->rf_n_el * nen * 3);
    }
  }
  // coefficients
  CoeffArgs ca{};
  ca.dim = D;
  ca.n_fam = v.n_fam;
  ca.n_bond = v.n_bond;
  ca.n_corr = std::max<int64_t>(p.n_corr, 1);
  ca.X = v.X;
  ca.vol = upload(m, s.vol_node);
  ca.fam_node = v.fam_node;
  ca.fam_ptr = v.fam_ptr;
  ca.nbr = v.nbr;
  ca.fam_delta = upload(m, s.fam_delta);
  ca.fam_cdv = m->d_fam_cdv;
  ca.fam_corr = v.fam_corr;
  ca.wd = upload(m, p.wd);
  ca.fam_wd = upload(m, p.fam_wd);
  ca.nlf = m->cmd.nlf;
  ca.lambda = p.lambda;
  ca.mu = p.mu;
  ca.coef64 = coef64; ca.coef32 = coef32; ca.corr64 = corr64; ca.corr32 = corr32; ca.cvec = cvec;
  ca.corr32_last = corr32_last;
  int* derr = m->buf.alloc<int>(1);
  cudaMemsetAsync(derr, 0, sizeof(int), m->stream);
  ca.err = derr;
  v.n_corr_bond = (int)ca.n_corr;
  for (void* pp : m->buf.ptrs)
    if (!pp) return set_error(PDX_ERR_CUDA, "device allocation failed");
  // one launch per coefficient segment (a batch: one per specimen, with its
  // own Lame constants); all indices inside are global
  std::vector<CoeffSeg> segs = m->coeff_segs;
  if (segs.empty()) segs.push_back({0, v.n_fam, m->cmd.nlf, p.lambda, p.mu});
  pdx_status st = PDX_OK;
  for (const CoeffSeg& sg : segs) {
    if (sg.n_fam == 0) continue;
    CoeffArgs c = ca;
    c.n_fam = sg.n_fam;
    c.fam_node = ca.fam_node + sg.fam0;
    c.fam_ptr = ca.fam_ptr + sg.fam0;
    c.fam_delta = ca.fam_delta + sg.fam0;
    c.fam_cdv = ca.fam_cdv + sg.fam0;
    c.fam_corr = ca.fam_corr + sg.fam0;
    c.fam_wd = ca.fam_wd + sg.fam0;
    c.nlf = sg.nlf;
    c.lambda = sg.lambda;
    c.mu = sg.mu;
    st = cuda_check(launch_coeff(c, m->stream), "coefficient kernel launch");
    if (st) return st;
  }
  int herr = 0;
  cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
  st = cuda_check(cudaStreamSynchronize(m->stream), "coefficient kernel");
  if (st) return st;
  if (herr) {
    const int f = herr - 1;
    return set_error(PDX_ERR_SINGULAR, "moment matrix of family " + std::to_string(f) + " (node " +
                                           std::to_string(m->setup.fam_node[f] + 1) + ") is singular");
  }
  return PDX_OK;
}

pdx_status rebuild_device(pdx_model* m, bool keep_twolevel) {
  const size_t nd = (size_t)m->mesh.n_node * m->mesh.dim;
  std::vector<double> u(nd), sig((size_t)m->mesh.n_node * 6), rf;
  cudaMemcpyAsync(u.data(), m->d_u[0], nd * 8, cudaMemcpyDeviceToHost, m->stream);
  cudaMemcpyAsync(sig.data(), m->d_sigma, sig.size() * 8, cudaMemcpyDeviceToHost, m->stream);
  if (m->rf && m->d_rf_hist) {
    rf.resize((size_t)m->rf_cap * 4);
    cudaMemcpyAsync(rf.data(), m->d_rf_hist, rf.size() * 8, cudaMemcpyDeviceToHost, m->stream);
  }
  pdx_status st = cuda_check(cudaStreamSynchronize(m->stream), "state before rebuild");
  if (st) return st;
  if (m->graph) {
    cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
  }
  learned_destroy(m);
  if (keep_twolevel && m->twolevel) m->twolevel->dev.keep_stale = true;
  else twolevel_destroy(m);
  m->buf.free_all();
  m->d_vel = m->d_acc = nullptr;
  m->newmark_ready = false;
  m->prep = Prepared();
  Error err{0, ""};
  // a rebuild serves the quasi-static FC 1 loop: no explicit step tables
  if (!prepare_model(m, err, false)) return set_error(err.code == 6 ? PDX_ERR_SINGULAR : PDX_ERR_PARSE, err.msg);
  st = upload_model(m);
  if (st) return st;
  for (int i = 0; i < 2; i++) cudaMemcpyAsync(m->d_u[i], u.data(), nd * 8, cudaMemcpyHostToDevice, m->stream);
  cudaMemcpyAsync(m->d_sigma, sig.data(), sig.size() * 8, cudaMemcpyHostToDevice, m->stream);
  if (!rf.empty() && m->d_rf_hist)
    cudaMemcpyAsync(m->d_rf_hist, rf.data(), rf.size() * 8, cudaMemcpyHostToDevice, m->stream);
  m->cur = 0;
  return cuda_check(cudaStreamSynchronize(m->stream), "device rebuild");
}

pdx_status upload_bond_states(pdx_model* m) {
  const Setup& s = m->setup;
  Prepared& p = m->prep;
  const int nf = (int)s.fam_node.size();
  std::fill(p.state_bits.begin(), p.state_bits.end(), 0u);
  p.fam_intact.assign(nf, 0);
  for (int f = 0; f < nf; f++)
    for (int64_t q = s.fam_off[f] + 1; q < s.fam_off[f + 1]; q++)
      if (s.bond_state[q]) {
        const int64_t b = p.fam_ptr[f] + (q - s.fam_off[f] - 1);
        p.state_bits[b >> 5] |= 1u << (b & 31);
        p.fam_intact[f]++;
      }
  cudaMemcpyAsync(m->d_state, p.state_bits.data(), p.state_bits.size() * 4, cudaMemcpyHostToDevice, m->stream);
  cudaMemcpyAsync(m->d_intact, p.fam_intact.data(), p.fam_intact.size() * 4, cudaMemcpyHostToDevice, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "bond state upload");
}

pdx_status model_stress(pdx_model* m, const double* d_u_all, bool sigma, bool phi) {
  StressArgs a{};
  a.v = m->view;
  a.u = d_u_all;
  a.D = m->d_D;
  a.node_mat = m->d_node_mat;
  a.bgp = m->d_bgp;
  a.L = m->d_L;
  a.protype = m->mesh.protype;
  a.nu = m->d_mat_nu;
  a.sigma = sigma ? m->d_sigma : nullptr;
  a.phi = phi ? m->d_phi : nullptr;
  return cuda_check(launch_stress(a, m->stream), "stress kernel");
}

// Reaction-force row `row` of the current state (calReacForc, pdsolve.cpp:5347-5404).
pdx_status rf_record(pdx_model* m, int64_t row) {
  if (!m->rf || row < 0 || row >= m->rf_cap) return PDX_OK;
  m->rf_rows = std::max(m->rf_rows, row + 1);
  double* h = m->d_rf_hist + row * 4;
  if (m->rf_n_el == 0) {
    cudaMemsetAsync(h, 0, 4 * 8, m->stream);
    if (m->rf_uc_index >= 0)
      cudaMemcpyAsync(h, m->d_u[m->cur] + m->rf_uc_index, 8, cudaMemcpyDeviceToDevice, m->stream);
    return cuda_check(cudaGetLastError(), "reaction forces");
  }
  const int nen = m->mesh.dim == 2 ? 4 : 8;
  return cuda_check(launch_reaction(m->rf_n_el, nen, m->mesh.dim, m->d_rf_conn, m->d_rf_ke, m->d_rf_mask,
                                    m->d_u[m->cur], m->rf_uc_index, m->d_rf_part, h, m->stream),
                    "reaction forces");
}

// FC 2 pass on the state just stepped to (the reference calls
// calGlobalNodeStresses and then failureProcess after every explicit step,
// pdsolve.cpp:6014-6016, 6060-6064): nodal stresses, candidates, Top-K
// selection, cuts.  Top-K (K > 0) selects on the host: the K largest sigma1,
// ties by bond index.
pdx_status fc2_pass(pdx_model* m, bool report) {
  if (!m->fc2) return PDX_OK;
  pdx_status st = model_stress(m, m->d_u[m->cur], true, false);
  if (st) return st;
  const Setup& s = m->setup;
  Fc2Args a{};
  a.v = m->view;
  a.sigma = m->d_sigma;
  a.sigult = m->mesh.sigult;
  a.half_min_delta = 0.5 * s.min_delta;
  a.lbc0 = s.lbc[0];
  a.lbc1 = s.lbc[1];
  a.block_size = s.block_size;
  a.nbx = s.nblocks[0];
  a.nby = s.nblocks[1];
  a.blk_ptr = m->d_fc2_blk_ptr;
  a.blk_fam = m->d_fc2_blk_fam;
  a.brec = m->mixed ? m->d_brec : nullptr;
  a.cand_val = m->d_fc2_val;
  a.cand_bond = m->d_fc2_bond;
  a.cand_fam = m->d_fc2_fam;
  a.count = m->d_fc2_count;
  a.cap = m->fc2_cap;
  a.max_sigma1 = report ? m->d_fc2_max : nullptr;
  cudaMemsetAsync(a.count, 0, sizeof(int), m->stream);
  if (report) cudaMemsetAsync(m->d_fc2_max, 0, sizeof(double), m->stream);
  st = cuda_check(launch_fc2_candidates(a, m->stream), "FC 2 candidates");
  if (st) return st;
  const int K = m->cmd.topk;
  if (report) {
    int nc = 0;
    cudaMemcpyAsync(&nc, a.count, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
    cudaMemcpyAsync(&m->fc2_max, m->d_fc2_max, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
    st = cuda_check(cudaStreamSynchronize(m->stream), "FC 2 report");
    if (st) return st;
    nc = std::min(nc, a.cap);
    m->fc2_kept = K > 0 ? std::min(nc, K) : nc;
  }
  if (K > 0) {
    int n = 0;
    cudaMemcpyAsync(&n, a.count, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
    st = cuda_check(cudaStreamSynchronize(m->stream), "FC 2 count");
    if (st) return st;
    n = std::min(n, a.cap);
    if (n > K) {
      std::vector<double> val(n);
      std::vector<int> bond(n), fam(n), order(n);
      cudaMemcpyAsync(val.data(), a.cand_val, (size_t)n * 8, cudaMemcpyDeviceToHost, m->stream);
      cudaMemcpyAsync(bond.data(), a.cand_bond, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream);
      cudaMemcpyAsync(fam.data(), a.cand_fam, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream);
      st = cuda_check(cudaStreamSynchronize(m->stream), "FC 2 candidates");
      if (st) return st;
      for (int i = 0; i < n; i++) order[i] = i;
      std::partial_sort(order.begin(), order.begin() + K, order.end(), [&](int x, int y) {
        return val[x] != val[y] ? val[x] > val[y] : bond[x] < bond[y];
      });
      std::vector<double> v2(K);
      std::vector<int> b2(K), f2(K);
      for (int i = 0; i < K; i++) {
        v2[i] = val[order[i]];
        b2[i] = bond[order[i]];
        f2[i] = fam[order[i]];
      }
      cudaMemcpyAsync(a.cand_val, v2.data(), (size_t)K * 8, cudaMemcpyHostToDevice, m->stream);
      cudaMemcpyAsync(a.cand_bond, b2.data(), (size_t)K * 4, cudaMemcpyHostToDevice, m->stream);
      cudaMemcpyAsync(a.cand_fam, f2.data(), (size_t)K * 4, cudaMemcpyHostToDevice, m->stream);
      cudaMemcpyAsync(a.count, &K, sizeof(int), cudaMemcpyHostToDevice, m->stream);
      st = cuda_check(cudaStreamSynchronize(m->stream), "FC 2 Top-K");
      if (st) return st;
    }
  }
  return cuda_check(launch_fc2_cut(a, m->stream), "FC 2 cuts");
}

static StepArgs step_args(pdx_model* m, int mode, int64_t step_index) {
  StepArgs a{};
  a.v = m->view;
  a.u_n = m->d_u[m->cur];
  a.u_next = m->d_u[1 - m->cur];
  a.uf_n = m->d_uf[m->cur];
  a.uf_next = m->d_uf[1 - m->cur];
  a.dt = m->cmd.dt;
  a.mode = mode;
  a.brec = m->d_brec;
  a.ke_smem = m->ke_smem;
  a.s0f = (float)m->cmd.s0;
  a.pertf = (float)m->cmd.s0_pert;
  if (m->view.n_nbc) {
    int64_t row = std::min<int64_t>(step_index + 1, m->cmd.nsteps + 1);
    a.nbc_val = m->d_nbcval + row * m->view.n_nbc;
  }
  return a;
}

pdx_status explicit_step_launch(pdx_model* m, int mode, int64_t step_index) {
  StepArgs a = step_args(m, mode, step_index);
  if (mode == 2) {
    a.u_next = m->d_u[m->cur];   // not written in mode 2
    a.uf_next = m->d_uf[m->cur];
  }
  pdx_status st = cuda_check(launch_step(a, m->mixed, m->lanes, m->fe_lanes, m->stream), "explicit step kernel");
  if (st) return st;
  if (mode != 2) m->cur ^= 1;
  return PDX_OK;
}

// K (mode 1, 2) or K_N = beta dt^2 K + M (mode 3) into d_Kval and
// F = f_ext(row) - K_full v into d_tmp_eq[0]; d_v_all is already masked for mode 1.
pdx_status assemble_device(pdx_model* m, int mode, const double* d_v_all, int nbc_row) {
  const int64_t nnz = (int64_t)m->setup.csr_ja.size();
  cudaMemsetAsync(m->d_Kval, 0, nnz * 8, m->stream);
  AsmArgs aa{};
  aa.v = m->view;
  aa.ia = m->d_ia;
  aa.rel_bond = m->d_rel_bond;
  aa.rel_self = m->d_rel_self;
  aa.rel_fe = m->d_rel_fe;
  aa.table = m->view.ke64;
  aa.a = m->d_Kval;
  aa.with_pd = 1;
  aa.fam_cdv = m->d_fam_cdv;
  pdx_status st = cuda_check(launch_assemble(aa, m->stream), "assembly kernel");
  if (st) return st;
  if (mode == 3) {
    if (!m->d_Mval) {
      m->d_Mval = m->buf.alloc<double>((size_t)std::max<int64_t>(nnz, 1));
      cudaMemsetAsync(m->d_Mval, 0, nnz * 8, m->stream);
      AsmArgs ma = aa;
      ma.table = m->d_me;
      ma.a = m->d_Mval;
      ma.with_pd = 0;
      ma.pd_diag_rho = m->mesh.rho;
      st = cuda_check(launch_assemble(ma, m->stream), "mass assembly kernel");
      if (st) return st;
    }
    // K_N = K * beta * dt * dt + M  (pdfemAssembleKNFR_CSRformat :6392-6395)
    st = cuda_check(launch_newmark_matrix(nnz, m->d_Kval, m->d_Mval, m->cmd.beta, m->cmd.dt, m->stream), "K_N");
    if (st) return st;
  }
  ForceArgs fa{};
  fa.v = m->view;
  fa.u = d_v_all;
  fa.f_eq = m->d_tmp_eq[0];
  if (m->view.n_nbc) fa.nbc_val = m->d_nbcval + (int64_t)nbc_row * m->view.n_nbc;
  fa.ext_scale = 1.0;
  return cuda_check(launch_force(fa, m->stream), "force kernel");
}

}  // namespace pdx

using namespace pdx;

static pdx_status finish_create(pdx_model* m, const pdx_options& o, pdx_model** out);

extern "C" {

const char* pdx_last_error(void) { return g_err.c_str(); }
const char* pdx_version(void) { return "pdlsm-gb300 0.1"; }

pdx_status pdx_model_create_from_cmd(const char* cmd_path, const pdx_options* opts, pdx_model** out) {
  if (!cmd_path || !out) return set_error(PDX_ERR_INVALID, "null argument");
  *out = nullptr;
  pdx_options o{0, -1, 0, 0, 0};
  if (opts) o = *opts;
  pdx_model* m = new pdx_model();
  Error err{0, ""};
  // verbose > 1 reports the host set-up phases on stderr
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  bool ok = read_command(cmd_path, m->cmd, m->mesh, m->base_dir, err);
  const auto t1 = clk::now();
  // with a device the family search runs on it; a host-only model (device
  // -1) keeps the host search
  int n_dev = 0;
  const int fam_dev = o.device >= 0 && cudaGetDeviceCount(&n_dev) == cudaSuccess && o.device < n_dev ? o.device : -1;
  ok = ok && build_setup(m->mesh, m->cmd, m->setup, err, fam_dev);
  const auto t2 = clk::now();
  ok = ok && prepare_model(m, err);
  const auto t3 = clk::now();
  if (o.verbose > 1) {
    auto sec = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    std::fprintf(stderr, "pdx: set-up %s: read %.3f s, build_setup %.3f s, prepare %.3f s\n", cmd_path, sec(t0, t1),
                 sec(t1, t2), sec(t2, t3));
  }
  if (!ok) {
    delete m;
    pdx_status code = err.code == 1 ? PDX_ERR_IO
                      : err.code == 3 ? PDX_ERR_UNSUPPORTED
                      : err.code == 6 ? PDX_ERR_SINGULAR
                      : err.code == 7 ? PDX_ERR_CUDA
                                      : PDX_ERR_PARSE;
    return set_error(code, err.msg);
  }
  return finish_create(m, o, out);
}

}  // extern "C"

// Options, device upload and initial explicit state of a model whose host
// set-up is complete; deletes the model on failure.
static pdx_status finish_create(pdx_model* m, const pdx_options& o, pdx_model** out) {
  m->mixed = o.precision >= 0 ? o.precision : m->cmd.precision;
  m->cracks = m->mesh.cracks;
  m->crack_sif.assign(m->cracks.size(), {0.0, 0.0, 0.0, 0.0});
  m->verbose = o.verbose;
  // Lanes per family / per FE-only node: given (> 0), the fixed default (0),
  // or timed on this model by pdx_explicit_init (< 0, autotune_lanes).  The
  // lane counts set the order of the force sums, so a fixed choice gives
  // bitwise reproducible runs and a tuned one may differ in the last bits.
  m->tune = o.lanes < 0 || o.fe_lanes < 0;
  m->lanes = o.lanes > 0 ? o.lanes : (m->mesh.dim == 3 ? 8 : 4);
  // FE-only nodes: one lane per node in 2D (9-node stencils: C4's batch of
  // 256 plates ran 2.1x faster than with 4 lanes), 4 lanes in 3D (27 nodes)
  m->fe_lanes = o.fe_lanes > 0 ? o.fe_lanes : (m->mesh.dim == 3 ? 4 : 1);
  m->tune_lanes = o.lanes < 0;
  m->tune_fe_lanes = o.fe_lanes < 0;
  if (!step_lanes_valid(m->lanes, m->fe_lanes)) {
    delete m;
    return set_error(PDX_ERR_INVALID, "lanes must be 4, 8 or 16 and fe_lanes 1, 2, 4 or 8");
  }
  if (o.device >= 0) {
    m->device = o.device;
    pdx_status st = cuda_check(cudaSetDevice(o.device), "cudaSetDevice");
    if (!st) st = cuda_check(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!st) {
      // The Krylov solves take their work space (up to the FP32 matrix copy
      // of the mixed methods, 0.9 GB on the 2.5M-equation Newmark system)
      // from the device's stream-ordered pool at every solve; keeping freed
      // blocks in the pool instead of returning them at each synchronisation
      // saves re-mapping them (one mixed Newmark step took 183 ms instead of
      // 68 ms when the pool had given its memory back).
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, o.device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    }
    if (!st) st = upload_model(m);
    if (st) {
      std::string keep = g_err;
      pdx_model_destroy(m);
      g_err = keep;
      return st;
    }
    m->has_device = true;
    pdx_explicit_init(m);
  }
  *out = m;
  return PDX_OK;
}

static pdx_status create_error(const Error& err) {
  const pdx_status code = err.code == 1   ? PDX_ERR_IO
                          : err.code == 3 ? PDX_ERR_UNSUPPORTED
                          : err.code == 4 ? PDX_ERR_INVALID
                          : err.code == 6 ? PDX_ERR_SINGULAR
                                          : PDX_ERR_PARSE;
  return set_error(code, err.msg);
}

extern "C" {

pdx_status pdx_batch_create(const char* const* cmd_paths, int n, const pdx_options* opts, pdx_model** out) {
  if (!cmd_paths || n <= 0 || !out) return set_error(PDX_ERR_INVALID, "bad argument");
  *out = nullptr;
  pdx_options o{0, -1, 0, 0, 0};
  if (opts) o = *opts;
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  // host set-up of every specimen, in parallel (independent models)
  std::vector<pdx_model*> parts(n, nullptr);
  std::vector<Error> errs(n, Error{0, ""});
  {
    const int nt = std::max(1, std::min<int>(n, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        for (int i = t; i < n; i += nt) {
          if (!cmd_paths[i]) { errs[i] = {4, "null command path"}; continue; }
          pdx_model* q = new pdx_model();
          if (!read_command(cmd_paths[i], q->cmd, q->mesh, q->base_dir, errs[i]) ||
              !build_setup(q->mesh, q->cmd, q->setup, errs[i], -1, false) || !prepare_model(q, errs[i])) {
            delete q;
            continue;
          }
          parts[i] = q;
        }
      });
    for (auto& x : th) x.join();
  }
  auto drop = [&]() {
    for (pdx_model* q : parts) delete q;
  };
  for (int i = 0; i < n; i++)
    if (!parts[i]) {
      Error e = errs[i];
      e.msg = "batch specimen " + std::to_string(i) + " (" + cmd_paths[i] + "): " + e.msg;
      drop();
      return create_error(e);
    }
  const auto t1 = clk::now();
  pdx_model* m = new pdx_model();
  Error err{0, ""};
  if (!merge_batch(parts, m, err)) {
    drop();
    delete m;
    return create_error(err);
  }
  m->base_dir = parts[0]->base_dir;
  drop();
  const auto t2 = clk::now();
  const pdx_status st = finish_create(m, o, out);
  if (o.verbose > 1) {
    auto sec = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    std::fprintf(stderr, "pdx: batch of %d: specimen set-ups %.3f s, merge %.3f s, device set-up %.3f s\n", n,
                 sec(t0, t1), sec(t1, t2), sec(t2, clk::now()));
  }
  return st;
}

pdx_status pdx_batch_offsets(const pdx_model* m, int64_t* node_off, int64_t* member_off, int64_t* eq_off) {
  if (!m) return set_error(PDX_ERR_INVALID, "null argument");
  const size_t n = m->batch.size();
  if (n == 0) return set_error(PDX_ERR_INVALID, "not a batched model");
  for (size_t i = 0; i <= n; i++) {
    const bool end = i == n;
    const BatchPart& b = m->batch[end ? n - 1 : i];
    if (node_off) node_off[i] = end ? b.node_off + b.n_node : b.node_off;
    if (member_off) member_off[i] = end ? b.member_off + b.n_member : b.member_off;
    if (eq_off) eq_off[i] = end ? b.eq_off + b.n_eq : b.eq_off;
  }
  return PDX_OK;
}

int pdx_batch_size(const pdx_model* m) { return m ? (int)m->batch.size() : 0; }

void pdx_model_destroy(pdx_model* m) {
  if (!m) return;
  if (m->has_device || m->stream) {
    cudaSetDevice(m->device);
    if (m->graph) cudaGraphExecDestroy(m->graph);
    if (m->stream) cudaStreamSynchronize(m->stream);
    learned_destroy(m);
    twolevel_destroy(m);
    m->buf.free_all();
    if (m->stream) cudaStreamDestroy(m->stream);
  }
  delete m;
}

pdx_status pdx_model_get_info(const pdx_model* m, pdx_model_info* info) {
  if (!m || !info) return set_error(PDX_ERR_INVALID, "null argument");
  pdx_model_info i{};
  i.dim = m->mesh.dim;
  i.n_node = m->mesh.n_node;
  i.n_elem = m->mesh.n_elem;
  i.n_eq = m->setup.n_eq;
  i.n_fam = (int)m->setup.fam_node.size();
  i.n_pdbe = (int)m->setup.pdbe.size();
  i.n_fe = (int)m->setup.fe.size();
  i.n_fe_classes = m->prep.n_cls;
  i.n_bond = (int64_t)m->prep.nbr.size();
  i.nnz = (int64_t)m->setup.csr_ja.size();
  i.solver = m->cmd.solver;
  i.newmark = m->cmd.newmark;
  i.lumped = m->cmd.lumped;
  i.fail_flag = m->cmd.fail_flag;
  i.precision = m->mixed;
  i.nsteps = m->cmd.nsteps;
  i.save_freq = m->cmd.save_freq;
  i.lanes = m->lanes;
  i.fe_lanes = m->fe_lanes;
  i.dt = m->cmd.dt;
  i.min_delta = m->setup.min_delta;
  i.max_delta = m->setup.max_delta;
  i.s0 = m->cmd.s0;
  i.s0_pert = m->cmd.s0_pert;
  *info = i;
  return PDX_OK;
}

static bool array_ref(const pdx_model* m, const std::string& n, const void** ptr, int64_t* count, size_t* esz,
                      std::vector<double>* tmp) {
  const Setup& s = m->setup;
  const Prepared& p = m->prep;
  auto set = [&](const void* q, size_t c, size_t e) { *ptr = q; *count = (int64_t)c; *esz = e; return true; };
  if (n == "eq") return set(s.eq.data(), s.eq.size(), 4);
  if (n == "vol_node") return set(s.vol_node.data(), s.vol_node.size(), 8);
  if (n == "vol_elem") return set(s.vol_elem.data(), s.vol_elem.size(), 8);
  if (n == "node_type") return set(s.node_type.data(), s.node_type.size(), 4);
  if (n == "fam_off") return set(s.fam_off.data(), s.fam_off.size(), 8);
  if (n == "fam_members") return set(s.fam_members.data(), s.fam_members.size(), 4);
  if (n == "fam_horizon") return set(s.fam_delta.data(), s.fam_delta.size(), 8);
  if (n == "fam_cdv") return set(s.fam_cdv.data(), s.fam_cdv.size(), 8);
  if (n == "bond_state0") return set(s.bond_state.data(), s.bond_state.size(), 1);
  if (n == "pdbe") return set(s.pdbe.data(), s.pdbe.size() * 4, 4);
  if (n == "pde_idx") return set(s.pde.data(), s.pde.size(), 4);
  if (n == "fe_idx") return set(s.fe.data(), s.fe.size(), 4);
  if (n == "csr_ia") return set(s.csr_ia.data(), s.csr_ia.size(), 8);
  if (n == "csr_ja") return set(s.csr_ja.data(), s.csr_ja.size(), 8);
  if (n == "mass") return set(p.mass_eq.data(), p.mass_eq.size(), 8);
  if (n == "u0") return set(p.u0.data(), p.u0.size(), 8);
  if (n == "geom") {
    tmp->assign({s.min_delta, s.max_delta, s.block_size, s.lbc[0], s.lbc[1], s.lbc[2], s.rtc[0], s.rtc[1], s.rtc[2]});
    return set(tmp->data(), tmp->size(), 8);
  }
  if (n == "X") return set(m->mesh.X.data(), m->mesh.X.size(), 8);
  if (n == "conn") return set(m->mesh.conn.data(), m->mesh.conn.size(), 4);
  if (n == "elem_nn") return set(m->mesh.elem_nn.data(), m->mesh.elem_nn.size(), 4);
  if (n == "feonly") return set(p.feonly.data(), p.feonly.size(), 4);
  if (n == "st_cls") return set(p.st_cls.data(), p.st_cls.size(), 4);
  if (n == "st_nbr") return set(p.st_nbr.data(), p.st_nbr.size(), 4);
  if (n == "st_blk") return set(p.st_blk.data(), p.st_blk.size(), 8);
  if (n == "tile_rows") return set(p.tile_rows.data(), p.tile_rows.size(), 4);
  if (n == "tile_cls") return set(p.tile_cls.data(), p.tile_cls.size(), 2);
  if (n == "lat_blk") return set(p.lat_blk.data(), p.lat_blk.size(), 4);
  if (n == "fe_rest") return set(p.fe_rest.data(), p.fe_rest.size(), 4);
  if (n == "rel_bond") return set(p.rel_bond.data(), p.rel_bond.size(), 4);
  if (n == "rel_self") return set(p.rel_self.data(), p.rel_self.size(), 4);
  if (n == "rel_fe") return set(p.rel_fe.data(), p.rel_fe.size(), 4);
  if (n == "fe_adj_ptr") return set(p.fe_adj_ptr.data(), p.fe_adj_ptr.size(), 4);
  if (n == "fe_adj") return set(p.fe_adj.data(), p.fe_adj.size(), 4);
  if (n == "fe_conn") return set(p.fe_conn.data(), p.fe_conn.size(), 4);
  if (n == "bcflag") return set(p.bcflag.data(), p.bcflag.size(), 1);
  if (n == "dtv") return set(p.dtv.data(), p.dtv.size(), 8);
  if (n == "material") {
    const Mesh& me = m->mesh;
    tmp->assign({me.E, me.nu, me.rho, me.KIc, me.sigult, m->cmd.nlf, m->cmd.factor, (double)me.protype,
                 m->cmd.dt, (double)m->cmd.nsteps, m->cmd.s0, (double)m->cmd.s0_seed, m->cmd.s0_pert});
    return set(tmp->data(), tmp->size(), 8);
  }
  return false;
}

pdx_status pdx_model_array_len(const pdx_model* m, const char* name, int64_t* count) {
  if (!m || !name || !count) return set_error(PDX_ERR_INVALID, "null argument");
  const void* ptr;
  size_t esz;
  std::vector<double> tmp;
  if (!array_ref(m, name, &ptr, count, &esz, &tmp)) return set_error(PDX_ERR_INVALID, std::string("unknown array ") + name);
  return PDX_OK;
}

pdx_status pdx_model_array(const pdx_model* m, const char* name, void* dst, int64_t count) {
  if (!m || !name || !dst) return set_error(PDX_ERR_INVALID, "null argument");
  const void* ptr;
  int64_t n;
  size_t esz;
  std::vector<double> tmp;
  if (!array_ref(m, name, &ptr, &n, &esz, &tmp)) return set_error(PDX_ERR_INVALID, std::string("unknown array ") + name);
  if (count != n) return set_error(PDX_ERR_INVALID, std::string("wrong count for ") + name);
  if (n) std::memcpy(dst, ptr, (size_t)n * esz);
  return PDX_OK;
}

#define NEED_DEVICE(m)                                                                    \
  do {                                                                                    \
    if (!(m)) return set_error(PDX_ERR_INVALID, "null model");                            \
    if (!(m)->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device");  \
    cudaSetDevice((m)->device);                                                           \
  } while (0)

pdx_status pdx_bond_coefficients(pdx_model* m, double* A, double* g, double* dvec, double* G) {
  NEED_DEVICE(m);
  const int D = m->mesh.dim, NA = D == 2 ? 5 : 9, ND = D == 2 ? 3 : 6;
  const int nf = m->view.n_fam;
  const int64_t nb = m->view.n_bond;
  DevBuf tmp;
  double* dA = tmp.alloc<double>((size_t)nf * NA * NA);
  double* dg = tmp.alloc<double>((size_t)nb * D);
  double* dd = tmp.alloc<double>((size_t)nb * ND);
  double* dG = tmp.alloc<double>((size_t)nb * D * D);
  int* derr = tmp.alloc<int>(1);
  if (!dA || !dg || !dd || !dG || !derr) { tmp.free_all(); return set_error(PDX_ERR_CUDA, "allocation failed"); }
  // scratch outputs so the model's coefficients stay untouched
  double* c64 = tmp.alloc<double>((size_t)(D == 2 ? 3 : 6) * nb);
  double* cv = tmp.alloc<double>((size_t)D * nb);
  double* cr = tmp.alloc<double>((size_t)D * D * std::max<int64_t>(m->prep.n_corr, 1));
  CoeffArgs ca{};
  ca.dim = D; ca.n_fam = nf; ca.n_bond = nb; ca.n_corr = std::max<int64_t>(m->prep.n_corr, 1);
  ca.X = m->view.X;
  DevBuf t2;
  ca.vol = t2.alloc<double>(m->setup.vol_node.size());
  cudaMemcpy((void*)ca.vol, m->setup.vol_node.data(), m->setup.vol_node.size() * 8, cudaMemcpyHostToDevice);
  double* dl = t2.alloc<double>(m->setup.fam_delta.size());
  cudaMemcpy(dl, m->setup.fam_delta.data(), m->setup.fam_delta.size() * 8, cudaMemcpyHostToDevice);
  ca.fam_delta = dl;
  ca.fam_node = m->view.fam_node; ca.fam_ptr = m->view.fam_ptr; ca.nbr = m->view.nbr;
  ca.fam_cdv = m->d_fam_cdv;
  ca.fam_corr = nullptr; ca.wd = nullptr; ca.fam_wd = nullptr;
  ca.nlf = m->cmd.nlf; ca.lambda = m->prep.lambda; ca.mu = m->prep.mu;
  ca.coef64 = c64; ca.coef32 = nullptr; ca.corr64 = cr; ca.corr32 = nullptr; ca.cvec = cv;
  ca.A_out = dA; ca.g_out = dg; ca.d_out = dd; ca.G_out = dG;
  cudaMemset(derr, 0, sizeof(int));
  ca.err = derr;
  pdx_status st = cuda_check(launch_coeff(ca, nullptr), "coefficient kernel");
  if (!st) st = cuda_check(cudaDeviceSynchronize(), "coefficient kernel");
  if (!st) {
    if (A) cudaMemcpy(A, dA, (size_t)nf * NA * NA * 8, cudaMemcpyDeviceToHost);
    if (g) cudaMemcpy(g, dg, (size_t)nb * D * 8, cudaMemcpyDeviceToHost);
    if (dvec) cudaMemcpy(dvec, dd, (size_t)nb * ND * 8, cudaMemcpyDeviceToHost);
    if (G) cudaMemcpy(G, dG, (size_t)nb * D * D * 8, cudaMemcpyDeviceToHost);
  }
  tmp.free_all();
  t2.free_all();
  return st;
}

pdx_status pdx_internal_force(pdx_model* m, const double* u_all, double* f_eq) {
  NEED_DEVICE(m);
  if (!u_all || !f_eq) return set_error(PDX_ERR_INVALID, "null argument");
  const size_t nd = (size_t)m->mesh.n_node * m->mesh.dim;
  cudaMemcpyAsync(m->d_tmp_all, u_all, nd * 8, cudaMemcpyHostToDevice, m->stream);
  ForceArgs a{};
  a.v = m->view;
  a.u = m->d_tmp_all;
  a.f_eq = m->d_tmp_eq[0];
  a.nbc_val = nullptr;
  a.ext_scale = 0.0;
  pdx_status st = cuda_check(launch_force(a, m->stream), "force kernel");
  if (st) return st;
  cudaMemcpyAsync(f_eq, m->d_tmp_eq[0], (size_t)m->setup.n_eq * 8, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "internal force");
}

}  // extern "C"

// Initial state of an explicit run: u_0 in both buffers, FP32 node records,
// initial bond states and, for mixed precision, the packed bond records.
static pdx_status explicit_reset(pdx_model* m) {
  const size_t nd = (size_t)m->mesh.n_node * m->mesh.dim;
  for (int i = 0; i < 2; i++)
    cudaMemcpyAsync(m->d_u[i], m->prep.u0.data(), nd * 8, cudaMemcpyHostToDevice, m->stream);
  launch_shadow(m->view, m->d_u[0], m->d_uf[0], m->stream);
  launch_shadow(m->view, m->d_u[1], m->d_uf[1], m->stream);
  cudaMemcpyAsync(m->d_state, m->prep.state_bits.data(), m->prep.state_bits.size() * 4, cudaMemcpyHostToDevice,
                  m->stream);
  cudaMemcpyAsync(m->d_intact, m->prep.fam_intact.data(), m->prep.fam_intact.size() * 4, cudaMemcpyHostToDevice,
                  m->stream);
  if (m->mixed) {
    pdx_status st = cuda_check(
        launch_pack_bonds(m->view, (float)m->cmd.s0_pert, m->lanes, m->d_brec, m->stream), "pack bonds");
    if (st) return st;
  }
  m->cur = 0;
  m->steps_done = 0;
  m->rf_rows = 0;
  m->explicit_run = true;
  return cuda_check(cudaStreamSynchronize(m->stream), "explicit init");
}

// Times the step kernel on this model for every (lanes per family, lanes per
// FE-only node) pair left open by the options and keeps the fastest.  The
// trial steps run on the model's own buffers; the caller resets the state
// afterwards, so tuning changes no result except the FP32 summation order of
// the mixed-precision forces.
static pdx_status autotune_lanes(pdx_model* m) {
  static const int kLp[3] = {4, 8, 16}, kLf[4] = {1, 2, 4, 8};
  const int nlp = m->tune_lanes ? 3 : 1, nlf = m->tune_fe_lanes ? 4 : 1;
  const int lp0 = m->lanes, lf0 = m->fe_lanes;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pdx_status st = cuda_check(cudaEventCreate(&e0), "event");
  if (!st) st = cuda_check(cudaEventCreate(&e1), "event");
  float best = 1e30f;
  int best_lp = lp0, best_lf = lf0;
  for (int i = 0; i < nlp && !st; i++) {
    for (int j = 0; j < nlf && !st; j++) {
      m->lanes = m->tune_lanes ? kLp[i] : lp0;
      m->fe_lanes = m->tune_fe_lanes ? kLf[j] : lf0;
      // 3D records are laid out for the lane count that reads them
      if (m->mixed)
        st = cuda_check(launch_pack_bonds(m->view, (float)m->cmd.s0_pert, m->lanes, m->d_brec, m->stream),
                        "pack bonds");
      for (int w = 0; w < 2 && !st; w++) st = explicit_step_launch(m, 1, 0);
      if (!st) st = cuda_check(cudaEventRecord(e0, m->stream), "event record");
      for (int w = 0; w < 5 && !st; w++) st = explicit_step_launch(m, 1, 0);
      if (!st) st = cuda_check(cudaEventRecord(e1, m->stream), "event record");
      if (!st) st = cuda_check(cudaEventSynchronize(e1), "event sync");
      float ms = 0.f;
      if (!st) st = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event time");
      if (!st && ms < best) {
        best = ms;
        best_lp = m->lanes;
        best_lf = m->fe_lanes;
      }
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  m->lanes = best_lp;
  m->fe_lanes = best_lf;
  if (m->graph) {
    cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
  }
  if (m->verbose) fprintf(stderr, "pdx: step lanes %d per family, %d per FE node (%.1f us/step)\n", best_lp, best_lf,
                          1000.f * best / 5);
  return st;
}

extern "C" {

pdx_status pdx_explicit_init(pdx_model* m) {
  NEED_DEVICE(m);
  pdx_status st = explicit_reset(m);
  if (st || !m->tune) return st;
  m->tune = false;
  st = autotune_lanes(m);
  if (st) return st;
  return explicit_reset(m);
}

static pdx_status build_graph(pdx_model* m, int gsteps) {
  if (m->graph) { cudaGraphExecDestroy(m->graph); m->graph = nullptr; }
  cudaGraph_t g;
  const int cur0 = m->cur;
  pdx_status st = cuda_check(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
  if (st) return st;
  for (int i = 0; i < gsteps; i++) {
    StepArgs a = step_args(m, 1, 0);
    launch_step(a, m->mixed, m->lanes, m->fe_lanes, m->stream);
    m->cur ^= 1;
  }
  st = cuda_check(cudaStreamEndCapture(m->stream, &g), "graph capture end");
  m->cur = cur0;
  if (st) return st;
  st = cuda_check(cudaGraphInstantiate(&m->graph, g, 0), "graph instantiate");
  cudaGraphDestroy(g);
  m->graph_steps = gsteps;
  m->graph_parity = cur0;
  return st;
}

static pdx_status advance(pdx_model* m, int nsteps) {
  const bool graphs = m->view.n_nbc == 0 && !m->fc2 && !m->rf;
  const int G = 64;
  int done = 0;
  pdx_status st = PDX_OK;
  while (done < nsteps) {
    const int left = nsteps - done;
    if (m->steps_done > 0 && graphs && left >= G) {
      if (!m->graph || m->graph_parity != m->cur) {
        st = build_graph(m, G);
        if (st) return st;
      }
      st = cuda_check(cudaGraphLaunch(m->graph, m->stream), "graph launch");
      if (st) return st;
      m->steps_done += G;
      done += G;
      continue;
    }
    st = explicit_step_launch(m, m->steps_done == 0 ? 0 : 1, m->steps_done);
    if (st) return st;
    st = fc2_pass(m);
    if (!st) st = rf_record(m, m->steps_done);
    if (st) return st;
    m->steps_done++;
    done++;
  }
  return PDX_OK;
}

pdx_status pdx_explicit_advance(pdx_model* m, int nsteps) {
  NEED_DEVICE(m);
  if (nsteps < 0) return set_error(PDX_ERR_INVALID, "nsteps < 0");
  pdx_status st = advance(m, nsteps);
  if (st) return st;
  return cuda_check(cudaStreamSynchronize(m->stream), "explicit advance");
}

pdx_status pdx_explicit_advance_timed(pdx_model* m, int nsteps, double* ms) {
  NEED_DEVICE(m);
  if (nsteps < 0 || !ms) return set_error(PDX_ERR_INVALID, "bad argument");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, m->stream);
  pdx_status st = advance(m, nsteps);
  cudaEventRecord(e1, m->stream);
  if (!st) st = cuda_check(cudaEventSynchronize(e1), "explicit advance");
  float f = 0;
  cudaEventElapsedTime(&f, e0, e1);
  *ms = f;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

namespace {
// The device address of a page-locked (pinned or registered) host buffer,
// or null for pageable memory.
const void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
}  // namespace

// With page-locked host buffers (all three), the step reads u_n and u_{n-1}
// and writes u_{n+1} in place over the coherent host link: one load kernel
// (scatter and FP32 shadow fused), the step, one store kernel into the
// caller's buffer, both moving each block's equation range as consecutive
// words.  Pageable buffers take staged copies.
pdx_status pdx_explicit_step_host(pdx_model* m, const double* u_n, const double* u_nm1, double* u_np1) {
  NEED_DEVICE(m);
  if (!u_n || !u_nm1 || !u_np1) return set_error(PDX_ERR_INVALID, "null argument");
  const size_t ne = (size_t)m->setup.n_eq;
  const double* dn = static_cast<const double*>(mapped_host(u_n));
  const double* dm = static_cast<const double*>(mapped_host(u_nm1));
  double* dout = static_cast<double*>(const_cast<void*>(mapped_host(u_np1)));
  if (!dn || !dm || !dout) {
    cudaMemcpyAsync(m->d_tmp_eq[0], u_n, ne * 8, cudaMemcpyHostToDevice, m->stream);
    cudaMemcpyAsync(m->d_tmp_eq[1], u_nm1, ne * 8, cudaMemcpyHostToDevice, m->stream);
    dn = m->d_tmp_eq[0];
    dm = m->d_tmp_eq[1];
    dout = nullptr;
  }
  launch_load_pair(m->view, dn, dm, m->d_u[m->cur], m->d_u[1 - m->cur], m->mixed ? m->d_uf[m->cur] : nullptr,
                   m->stream);
  pdx_status st = explicit_step_launch(m, m->steps_done == 0 ? 0 : 1, m->steps_done);
  if (st) return st;
  st = fc2_pass(m);
  if (!st) st = rf_record(m, m->steps_done);
  if (st) return st;
  m->steps_done++;
  if (dout) launch_store_eq(m->view, m->d_u[m->cur], dout, m->stream);
  else launch_gather_eq(m->view, m->d_u[m->cur], m->d_tmp_eq[2], m->stream);
  if (!dout) cudaMemcpyAsync(u_np1, m->d_tmp_eq[2], ne * 8, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "explicit step");
}

int64_t pdx_explicit_step_count(const pdx_model* m) { return m ? m->steps_done : -1; }

pdx_status pdx_reaction_forces(const pdx_model* m, double* rows, int64_t max_rows, int64_t* count) {
  if (!m) return set_error(PDX_ERR_INVALID, "null model");
  const int64_t n = m->rf ? m->rf_rows : 0;
  if (count) *count = n;
  if (!rows || n == 0 || max_rows <= 0) return PDX_OK;
  if (!m->has_device) return set_error(PDX_ERR_NODEVICE, "model has no GPU device");
  cudaSetDevice(m->device);
  cudaMemcpyAsync(rows, m->d_rf_hist, (size_t)std::min(n, max_rows) * 4 * 8, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "reaction forces");
}

pdx_status pdx_crack_state(const pdx_model* m, double* rows, int max_cracks, int* n_cracks) {
  if (!m) return set_error(PDX_ERR_INVALID, "null model");
  const int n = (int)m->cracks.size();
  if (n_cracks) *n_cracks = n;
  for (int k = 0; rows && k < n && k < max_cracks; k++) {
    const auto& c = m->cracks[k];
    const auto& f = m->crack_sif[k];
    const double r[8] = {c[0], c[1], c[3], c[4], f[0], f[1], f[2], f[3]};
    std::memcpy(rows + (size_t)k * 8, r, sizeof r);
  }
  return PDX_OK;
}

pdx_status pdx_get_state(pdx_model* m, double* u_all, double* sigma, double* phi, uint8_t* bond_state) {
  NEED_DEVICE(m);
  const int N = m->mesh.n_node, D = m->mesh.dim;
  // the reference computes node stress before the step's failure pass and
  // damage after it (pdfemDynamicSolver_CSRformat :6060-6075)
  // (with FC 2 the last pass computed the stresses before its cuts)
  pdx_status st = m->fc2 && m->steps_done > 0 ? PDX_OK : model_stress(m, m->d_u[m->cur], true, false);
  if (st) return st;
  if (m->explicit_run && m->steps_done > 0 && m->view.fail3) st = explicit_step_launch(m, 2, m->steps_done);
  if (st) return st;
  st = model_stress(m, m->d_u[m->cur], false, true);
  if (st) return st;
  if (u_all) cudaMemcpyAsync(u_all, m->d_u[m->cur], (size_t)N * D * 8, cudaMemcpyDeviceToHost, m->stream);
  if (sigma) cudaMemcpyAsync(sigma, m->d_sigma, (size_t)N * 6 * 8, cudaMemcpyDeviceToHost, m->stream);
  if (phi) cudaMemcpyAsync(phi, m->d_phi, (size_t)N * 8, cudaMemcpyDeviceToHost, m->stream);
  std::vector<uint32_t> bits;
  if (bond_state) {
    bits.resize(m->prep.state_bits.size());
    cudaMemcpyAsync(bits.data(), m->d_state, bits.size() * 4, cudaMemcpyDeviceToHost, m->stream);
  }
  st = cuda_check(cudaStreamSynchronize(m->stream), "get state");
  if (st) return st;
  if (bond_state) {
    const auto& s = m->setup;
    for (size_t f = 0; f < s.fam_node.size(); f++) {
      bond_state[s.fam_off[f]] = 1;
      for (int b = m->prep.fam_ptr[f]; b < m->prep.fam_ptr[f + 1]; b++)
        bond_state[s.fam_off[f] + 1 + (b - m->prep.fam_ptr[f])] = (bits[b >> 5] >> (b & 31)) & 1u;
    }
  }
  return PDX_OK;
}

// The CSR index arrays of the seams are the reference's `long long` (64-bit
// here, like the int64_t arrays the library keeps).
static_assert(sizeof(long long) == sizeof(int64_t), "CSR indices are 64-bit");

pdx_status pdx_assemble_csr(pdx_model* m, int mode, const double* v_all, long long* ia, long long* ja, double* a,
                            double* f) {
  NEED_DEVICE(m);
  if (mode < 1 || mode > 3) return set_error(PDX_ERR_INVALID, "mode must be 1, 2 or 3");
  if (!m->batch.empty()) return set_error(PDX_ERR_UNSUPPORTED, "batched models run explicit dynamics only");
  const int N = m->mesh.n_node, D = m->mesh.dim;
  const int64_t nnz = (int64_t)m->setup.csr_ja.size();
  const size_t nd = (size_t)N * D;
  std::vector<double> v(nd);
  if (v_all) std::memcpy(v.data(), v_all, nd * 8);
  else cudaMemcpy(v.data(), m->d_u[m->cur], nd * 8, cudaMemcpyDeviceToHost);
  if (mode == 1)
    for (size_t i = 0; i < nd; i++)
      if (m->setup.eq[i] >= 0) v[i] = 0.0;
  cudaMemcpyAsync(m->d_tmp_all, v.data(), nd * 8, cudaMemcpyHostToDevice, m->stream);
  pdx_status st = assemble_device(m, mode, m->d_tmp_all, 0);
  if (st) return st;
  if (ia) std::memcpy(ia, m->setup.csr_ia.data(), m->setup.csr_ia.size() * 8);
  if (ja) std::memcpy(ja, m->setup.csr_ja.data(), nnz * 8);
  if (a) cudaMemcpyAsync(a, m->d_Kval, nnz * 8, cudaMemcpyDeviceToHost, m->stream);
  if (f) cudaMemcpyAsync(f, m->d_tmp_eq[0], (size_t)m->setup.n_eq * 8, cudaMemcpyDeviceToHost, m->stream);
  return cuda_check(cudaStreamSynchronize(m->stream), "assembly");
}

pdx_status pdx_solve_csr(long long n, const long long* ia, const long long* ja, const double* a, const double* rhs,
                         double* x, const pdx_solve_opts* opts, pdx_solve_info* info) {
  if (n <= 0 || !ia || !ja || !a || !rhs || !x) return set_error(PDX_ERR_INVALID, "bad argument");
  pdx_solve_opts o{2, 1e-8, 20000, 0};
  if (opts) o = *opts;
  if (o.method == 8)
    return set_error(PDX_ERR_INVALID, "method 8 builds its coarse grid from the model's nodes: use pdx_quasi_step or "
                                      "pdx_newmark_step");
  if (o.method < 0 || (o.method > 3 && o.method < 6) || o.method > 7)
    return set_error(PDX_ERR_INVALID, "method must be 0..3, 6 or 7");
  const int64_t nnz = ia[n];
  std::vector<int> ja32(ja, ja + nnz);
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return set_error(PDX_ERR_CUDA, "no CUDA device");
  DevBuf b;
  int64_t* dia = b.alloc<int64_t>(n + 1);
  int* dja = b.alloc<int>(nnz);
  double* da = b.alloc<double>(nnz);
  double* db = b.alloc<double>(n);
  double* dx = b.alloc<double>(n);
  if (!dia || !dja || !da || !db || !dx) {
    b.free_all();
    cudaStreamDestroy(s);
    return set_error(PDX_ERR_CUDA, "allocation failed");
  }
  cudaMemcpyAsync(dia, ia, (n + 1) * 8, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dja, ja32.data(), nnz * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(da, a, nnz * 8, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(db, rhs, n * 8, cudaMemcpyHostToDevice, s);
  if (o.use_x0) cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, s);
  else cudaMemsetAsync(dx, 0, n * 8, s);
  DevCsr A;
  A.n = n; A.nnz = nnz; A.ia = dia; A.ja = dja; A.a = da;
  KrylovResult kr;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  cudaError_t ce = krylov_solve(A, db, dx, o.method, o.rtol, o.max_iter, 3, s, &kr);
  cudaEventRecord(e1, s);
  cudaMemcpyAsync(x, dx, n * 8, cudaMemcpyDeviceToHost, s);
  cudaError_t ce2 = cudaStreamSynchronize(s);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b.free_all();
  cudaStreamDestroy(s);
  if (ce != cudaSuccess || ce2 != cudaSuccess)
    return set_error(PDX_ERR_CUDA, std::string("Krylov solve: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ce2));
  fill_solve_info(info, kr, ms * 1e-3);
  if (!kr.converged)
    return set_error(PDX_ERR_NOCONV, "Krylov solve stopped at relative residual " + std::to_string(kr.rel_residual));
  return PDX_OK;
}

// Jacobi PCG on a device-resident CSR system with the work space in a fixed
// device array: allocates no device memory (k_krylov.cu, krylov_pcg_noalloc).
pdx_status pdx_pcg_solve_noalloc(int64_t n, int64_t nnz, const int64_t* d_ia, const int32_t* d_ja,
                                 const double* d_a, const double* d_rhs, double* d_x, const pdx_solve_opts* opts,
                                 void* stream, pdx_solve_info* info) {
  if (n <= 0 || nnz <= 0 || !d_ia || !d_ja || !d_a || !d_rhs || !d_x) return set_error(PDX_ERR_INVALID, "bad argument");
  if (n > noalloc_max_n())
    return set_error(PDX_ERR_INVALID, "pdx_pcg_solve_noalloc: n = " + std::to_string(n) + " exceeds the fixed work space (" +
                                          std::to_string(noalloc_max_n()) + " equations)");
  pdx_solve_opts o{0, 1e-8, 20000, 0};
  if (opts) o = *opts;
  if (o.method != 0) return set_error(PDX_ERR_UNSUPPORTED, "pdx_pcg_solve_noalloc runs Jacobi PCG only (method 0)");
  DevCsr A;
  A.n = n;
  A.nnz = nnz;
  A.ia = d_ia;
  A.ja = d_ja;
  A.a = d_a;
  KrylovResult kr;
  cudaError_t ce =
      krylov_pcg_noalloc(A, d_rhs, d_x, o.rtol, o.max_iter, o.use_x0, static_cast<cudaStream_t>(stream), &kr);
  if (ce != cudaSuccess) return set_error(PDX_ERR_CUDA, std::string("Krylov solve: ") + cudaGetErrorString(ce));
  fill_solve_info(info, kr, 0.0);
  if (!kr.converged)
    return set_error(PDX_ERR_NOCONV, "Krylov solve stopped at relative residual " + std::to_string(kr.rel_residual));
  return PDX_OK;
}

}  // extern "C"
