// Batched explicit runs: many independent specimens (one command file each)
// merged into one model, so that one step launch covers every family and node
// of every specimen.  The reference runs one model per process; there is no
// counterpart to copy.  Each specimen's host set-up is built on its own (the
// same code as a single model), then every array is concatenated with its
// node, element, family, bond, equation and class offsets.  Materials, time
// steps, critical stretch and boundary values stay per specimen: they live in
// per-node (mass, dt^2/m, BC increments), per-family (critical stretch) and
// per-class (element and stencil blocks) arrays; the PDLSM coefficients are
// computed per specimen with its own Lame constants (coefficient segments).
#include <algorithm>
#include <string>

#include "model_impl.h"

namespace pdx {

namespace {

template <typename T>
void append(std::vector<T>& dst, const std::vector<T>& src) {
  dst.insert(dst.end(), src.begin(), src.end());
}

// dst += src + off for entries >= 0, negative entries kept
// (capacity grows geometrically: reserving the exact size on every append
// would copy the whole array once per specimen)
template <typename T, typename O>
void append_off(std::vector<T>& dst, const std::vector<T>& src, O off) {
  const size_t need = dst.size() + src.size();
  if (dst.capacity() < need) dst.reserve(std::max(need, 2 * dst.capacity()));
  for (const T& x : src) dst.push_back(x >= 0 ? (T)(x + off) : x);
}

}  // namespace

bool merge_batch(const std::vector<pdx_model*>& parts, pdx_model* out, Error& err) {
  if (parts.empty()) { err = {4, "empty batch"}; return false; }
  const pdx_model* p0 = parts[0];
  const int D = p0->mesh.dim;
  for (size_t i = 0; i < parts.size(); i++) {
    const pdx_model* q = parts[i];
    const std::string who = "batch specimen " + std::to_string(i) + ": ";
    if (q->mesh.dim != D) { err = {3, who + "all specimens must have the same dimension"}; return false; }
    if (D == 2 && q->mesh.protype != p0->mesh.protype) { err = {3, who + "mixed plane stress / strain"}; return false; }
    if (q->cmd.solver != 0 || q->cmd.newmark) { err = {3, who + "only explicit dynamic runs can be batched"}; return false; }
    if (q->cmd.fail_flag != p0->cmd.fail_flag) { err = {3, who + "failure criteria differ"}; return false; }
    if (q->cmd.fail_flag == 2) { err = {3, who + "FC 2 runs on single models only"}; return false; }
    if (q->cmd.precision != p0->cmd.precision) { err = {3, who + "precisions differ"}; return false; }
    if (q->cmd.s0_pert != p0->cmd.s0_pert || q->cmd.s0_seed != p0->cmd.s0_seed) {
      err = {3, who + "per-bond draws (seed, perturbation) must agree"}; return false;
    }
    if (!q->mesh.nbcs.empty()) { err = {3, who + "traction BCs are not supported in a batch"}; return false; }
  }
  Mesh& M = out->mesh;
  Setup& S = out->setup;
  Prepared& P = out->prep;
  M = Mesh{};
  S = Setup{};
  P = Prepared{};
  out->cmd = p0->cmd;
  M.title = "batch";
  M.dim = D;
  M.protype = p0->mesh.protype;
  M.E = p0->mesh.E; M.nu = p0->mesh.nu; M.rho = p0->mesh.rho; M.KIc = p0->mesh.KIc; M.sigult = p0->mesh.sigult;
  S.dim = D;
  S.min_delta = 1e300;
  S.max_delta = 0;
  P.fam_ptr.push_back(0);
  P.fe_adj_ptr.push_back(0);
  S.fam_off.push_back(0);
  // no CSR pattern or scatter maps: a batch runs explicit steps only (the
  // assembly entry points refuse batched models)
  out->batch.clear();
  out->coeff_segs.clear();
  out->mat_D.clear();
  out->mat_nu.clear();
  out->node_mat.clear();
  int64_t node_off = 0, elem_off = 0, fam_off = 0, bond_off = 0, eq_off = 0, member_off = 0, fe_off = 0;
  int64_t cls_off = 0, st_off = 0, corr_off = 0, wd_off = 0, adj_off = 0, dcls_off = 0;
  bool all_delta = true;
  int64_t feonly_off = 0;
  const int NV = D == 2 ? 3 : 6;
  for (size_t i = 0; i < parts.size(); i++) {
    const pdx_model* q = parts[i];
    const Mesh& m = q->mesh;
    const Setup& s = q->setup;
    const Prepared& p = q->prep;
    const int nf = (int)s.fam_node.size();
    BatchPart bp;
    bp.node_off = node_off; bp.member_off = member_off; bp.eq_off = eq_off; bp.fam_off = fam_off;
    bp.bond_off = bond_off; bp.n_node = m.n_node; bp.n_member = (int64_t)s.fam_members.size(); bp.n_eq = s.n_eq;
    bp.n_fam = nf; bp.dt = q->cmd.dt; bp.title = m.title;
    out->batch.push_back(bp);
    out->coeff_segs.push_back({(int)fam_off, nf, q->cmd.nlf, p.lambda, p.mu});
    append(out->mat_D, p.D);
    out->mat_nu.push_back(m.nu);
    out->node_mat.insert(out->node_mat.end(), m.n_node, (int)i);
    // mesh
    M.n_node += m.n_node;
    M.n_elem += m.n_elem;
    append(M.X, m.X);
    append(M.elem_nn, m.elem_nn);
    append(M.elem_algo, m.elem_algo);
    append_off(M.conn, m.conn, node_off);
    // set-up
    S.n_eq += s.n_eq;
    append_off(S.eq, s.eq, eq_off);
    append(S.vol_elem, s.vol_elem);
    append(S.vol_node, s.vol_node);
    S.min_delta = std::min(S.min_delta, s.min_delta);
    S.max_delta = std::max(S.max_delta, s.max_delta);
    append_off(S.pde, s.pde, elem_off);
    append_off(S.fe, s.fe, elem_off);
    for (auto e : s.pdbe) {
      for (int& x : e) x = x >= 0 ? (int)(x + node_off) : x;
      S.pdbe.push_back(e);
    }
    append(S.node_type, s.node_type);
    append_off(S.fam_of_node, s.fam_of_node, fam_off);
    append_off(S.fam_node, s.fam_node, node_off);
    for (size_t f = 1; f < s.fam_off.size(); f++) S.fam_off.push_back(s.fam_off[f] + member_off);
    append_off(S.fam_members, s.fam_members, node_off);
    append(S.fam_delta, s.fam_delta);
    append(S.fam_cdv, s.fam_cdv);
    append(S.bond_state, s.bond_state);
    // prepared arrays
    append(P.mass_node, p.mass_node);
    append(P.mass_eq, p.mass_eq);
    append(P.bcflag, p.bcflag);
    append(P.dtv, p.dtv);
    append(P.u0, p.u0);
    for (int f = 1; f <= nf; f++) P.fam_ptr.push_back((int)(p.fam_ptr[f] + bond_off));
    append_off(P.nbr, p.nbr, node_off);
    const int64_t nb = (int64_t)p.nbr.size();
    P.state_bits.resize((size_t)((bond_off + nb + 31) / 32), 0u);
    for (int64_t b = 0; b < nb; b++)
      if ((p.state_bits[b >> 5] >> (b & 31)) & 1u) {
        const int64_t g = bond_off + b;
        P.state_bits[g >> 5] |= 1u << (g & 31);
      }
    append(P.fam_intact, p.fam_intact);
    append(P.fam_brk, p.fam_brk);
    P.fam_s0.insert(P.fam_s0.end(), nf, q->cmd.s0);
    append(P.dt2m, p.dt2m);
    append_off(P.fam_corr, p.fam_corr, corr_off);
    append_off(P.fam_wd, p.fam_wd, wd_off);
    append(P.wd, p.wd);
    P.n_corr += p.n_corr;
    append_off(P.feonly, p.feonly, node_off);
    append_off(P.fam_order, p.fam_order, fam_off);
    append_off(P.fe_conn, p.fe_conn, node_off);
    append_off(P.fe_cls, p.fe_cls, cls_off);
    append(P.ke, p.ke);
    append(P.me, p.me);
    append(P.bgp, p.bgp);
    if (i == 0) P.L = p.L;
    P.n_cls += p.n_cls;
    for (int k = 1; k <= m.n_node; k++) P.fe_adj_ptr.push_back((int)(p.fe_adj_ptr[k] + adj_off));
    for (int e : p.fe_adj) P.fe_adj.push_back((int)((((int64_t)(e >> 3) + fe_off) << 3) | (e & 7)));
    if (p.n_st_cls > 0) {
      append_off(P.st_cls, p.st_cls, st_off);
      append(P.st_blk, p.st_blk);
      P.n_st_cls += p.n_st_cls;
    } else {
      P.st_cls.insert(P.st_cls.end(), p.feonly.size(), -1);
    }
    {
      const int S3 = D == 2 ? kStencil2 : kStencil3;
      if (p.st_nbr.size() == p.feonly.size() * (size_t)S3) append_off(P.st_nbr, p.st_nbr, node_off);
      else P.st_nbr.insert(P.st_nbr.end(), p.feonly.size() * (size_t)S3, -1);
    }
    if (p.n_st_cls > 0 && p.st_use_delta) {
      append_off(P.st_dcls, p.st_dcls, dcls_off);
      append(P.st_delta, p.st_delta);
      dcls_off += p.n_st_dcls;
    } else {
      P.st_dcls.insert(P.st_dcls.end(), p.feonly.size(), -1);
      if (p.n_st_cls > 0) all_delta = false;
    }
    // lattice tiles: node ids and classes shifted; a specimen without tiles
    // lists its FE-only items for the per-node path
    if (p.n_tiles > 0) {
      const size_t r0 = P.tile_rows.size();
      P.tile_rows.insert(P.tile_rows.end(), p.tile_rows.begin(), p.tile_rows.end());
      for (size_t r = r0; r < P.tile_rows.size(); r += 2)
        if (P.tile_rows[r + 1] != 0) P.tile_rows[r] += (int)node_off;
      for (int16_t c : p.tile_cls)
        P.tile_cls.push_back(c < 0 ? c : (int16_t)(((c & kTileClsMask) + st_off) | (c & kTileShadowBit)));
      append(P.lat_blk, p.lat_blk);
      P.n_tiles += p.n_tiles;
    } else {
      for (size_t it = 0; it < p.feonly.size(); it++) P.fe_rest.push_back((int)(feonly_off + (int64_t)it));
      // keep the class numbering of lat_blk aligned with st_cls
      P.lat_blk.insert(P.lat_blk.end(), (size_t)p.n_st_cls * Tile2::SLOTS * Tile2::BW, 0.f);
    }
    feonly_off += (int64_t)p.feonly.size();
    if (i == 0) { P.D = p.D; P.lambda = p.lambda; P.mu = p.mu; }
    // offsets
    node_off += m.n_node;
    elem_off += m.n_elem;
    fam_off += nf;
    bond_off += nb;
    eq_off += s.n_eq;
    member_off += (int64_t)s.fam_members.size();
    fe_off += (int64_t)s.fe.size();
    cls_off += p.n_cls;
    st_off += p.n_st_cls;
    corr_off += p.n_corr;
    wd_off += (int64_t)(p.wd.size() / ((size_t)D * NV));
    adj_off += (int64_t)p.fe_adj.size();
    if (node_off > INT32_MAX || bond_off > INT32_MAX || (fe_off << 3) > INT32_MAX) {
      err = {3, "batch too large for 32-bit node, bond or element indices"};
      return false;
    }
  }
  if (P.n_tiles == 0 || st_off > kTileClsMask) {
    P.tile_rows.clear();
    P.tile_cls.clear();
    P.lat_blk.clear();
    P.n_tiles = 0;
    P.fe_rest.clear();
  }
  P.n_st_dcls = (int)dcls_off;
  P.st_use_delta = P.n_st_cls > 0 && all_delta;
  if (P.n_st_cls == 0) {
    P.st_cls.clear();
    P.st_nbr.clear();
  }
  // one material for the record; the kernels read the per-node/per-class arrays
  M.nu = parts[0]->mesh.nu;
  return true;
}

}  // namespace pdx
