// Host preparation of the arrays the kernels consume, from the model setup:
//   lumped mass (assembleLumpedMass, pdsolve.cpp:4618-4669),
//   prescribed-DOF increments (setVaryEssentialBC :5263-5312),
//   bond lists and initial bond states, per family,
//   PD-boundary traction weights W_k (2D: 1/2 N per segment, assemblePDBEwork_CSRformat
//   :4049-4252; 3D: area-weighted normal matrix of every face, normMatArea :2917-2967
//   and assemblePDBEwork3D_CSRformat :2732-2915) folded with D,
//   FE stiffness/mass classes: elements whose node positions relative to their
//   first node agree to 1e-12 of the element size share one Ke / Me (FP64),
//   node -> FE element adjacency, traction-BC unit forces (pdfemEleLine2N.cpp:45-75,
//   pdfemEleQuad4N.cpp eleEquivNodalForce), and the scatter map of every bond /
//   element block into the CSR pattern.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>

#include "model_impl.h"

namespace pdx {

namespace {

struct VecHash {
  size_t operator()(const std::vector<int64_t>& v) const {
    uint64_t h = 1469598103934665603ull;
    for (int64_t x : v) { h ^= (uint64_t)x; h *= 1099511628211ull; }
    return (size_t)h;
  }
};

void norm_mat_area(const double xN[4][3], bool quad, double Nmat[3][6], bool& ok) {
  double v1[3], v2[3];
  for (int i = 0; i < 3; i++) { v1[i] = xN[1][i] - xN[0][i]; v2[i] = xN[2][i] - xN[0][i]; }
  double N1 = v1[1] * v2[2] - v1[2] * v2[1];
  double N2 = v2[0] * v1[2] - v1[0] * v2[2];
  double N3 = v1[0] * v2[1] - v2[0] * v1[1];
  const double A1 = std::sqrt(N1 * N1 + N2 * N2 + N3 * N3);
  ok = A1 != 0;
  double A2 = 0, w = 1.0 / 3;
  if (quad) {
    for (int i = 0; i < 3; i++) { v1[i] = xN[3][i] - xN[0][i]; v2[i] = xN[2][i] - xN[0][i]; }
    const double t1 = v1[1] * v2[2] - v1[2] * v2[1];
    const double t2 = v2[0] * v1[2] - v1[0] * v2[2];
    const double t3 = v1[0] * v2[1] - v2[0] * v1[1];
    A2 = std::sqrt(t1 * t1 + t2 * t2 + t3 * t3);
    w = 0.25;
  }
  const double area = (A1 + A2) * 0.5;
  N1 = N1 / A1 * area * w;
  N2 = N2 / A1 * area * w;
  N3 = N3 / A1 * area * w;
  std::memset(Nmat, 0, sizeof(double) * 18);
  Nmat[0][0] = N1; Nmat[1][1] = N2; Nmat[2][2] = N3;
  Nmat[0][3] = N2; Nmat[0][5] = N3;
  Nmat[1][3] = N1; Nmat[1][4] = N3;
  Nmat[2][4] = N2; Nmat[2][5] = N1;
}

// Node stencils of the FE-only nodes.  The FE rows of such a node are
// -sum_j K_kj u_j with K_kj = sum over the elements around k of the element
// matrix block (k, j); nodes whose surroundings are the same up to a
// translation share one table of blocks (a stencil class).  The element
// entries of a node are taken in the order of their centroids relative to
// the node and the neighbours in the order of their relative positions, both
// quantised to 1e-6 of the surrounding element size, so equal surroundings
// give equal keys and bitwise equal blocks.  Nodes with more than
// kStencil2/kStencil3 neighbours, or meshes whose classes would not be
// shared, keep the element path (st_cls = -1).
void build_stencils(const Mesh& me, Prepared& p) {
  const int D = me.dim;
  const int nen = D == 2 ? 4 : 8;
  const int nd = nen * D;
  const int S = D == 2 ? kStencil2 : kStencil3;
  const int nfo = (int)p.feonly.size();
  p.st_cls.assign(nfo, -1);
  p.st_nbr.assign((size_t)nfo * S, -1);
  p.st_blk.clear();
  p.n_st_cls = 0;
  std::unordered_map<std::vector<int64_t>, int, VecHash> classes;
  struct Ent { std::array<int64_t, 3> c; int fe, al; };
  // per-node work space, reused (the loop runs once per FE-only node)
  std::vector<Ent> ent;
  std::vector<std::pair<std::array<int64_t, 3>, int>> nb;
  std::vector<int64_t> key;
  for (int it = 0; it < nfo; it++) {
    const int k = p.feonly[it];
    const double* xk = &me.X[(size_t)k * 3];
    ent.clear();
    double Le = 0;
    for (int j = p.fe_adj_ptr[k]; j < p.fe_adj_ptr[k + 1]; j++) {
      const int i = p.fe_adj[j] >> 3;
      for (int a = 0; a < nen; a++)
        for (int c = 0; c < 3; c++)
          Le = std::max(Le, std::fabs(me.X[(size_t)p.fe_conn[(size_t)i * 8 + a] * 3 + c] - xk[c]));
    }
    if (Le <= 0) continue;
    const double q = 1e-6 * Le;
    auto qpos = [&](const double* x) {
      return std::array<int64_t, 3>{std::llround((x[0] - xk[0]) / q), std::llround((x[1] - xk[1]) / q),
                                    std::llround((x[2] - xk[2]) / q)};
    };
    for (int j = p.fe_adj_ptr[k]; j < p.fe_adj_ptr[k + 1]; j++) {
      const int i = p.fe_adj[j] >> 3;
      double c[3] = {0, 0, 0};
      for (int a = 0; a < nen; a++)
        for (int d = 0; d < 3; d++) c[d] += me.X[(size_t)p.fe_conn[(size_t)i * 8 + a] * 3 + d] / nen;
      ent.push_back({qpos(c), i, p.fe_adj[j] & 7});
    }
    std::sort(ent.begin(), ent.end(), [](const Ent& x, const Ent& y) {
      return x.c != y.c ? x.c < y.c : x.fe < y.fe;
    });
    nb.clear();
    for (const Ent& e : ent)
      for (int a = 0; a < nen; a++) {
        const int n = p.fe_conn[(size_t)e.fe * 8 + a];
        nb.push_back({qpos(&me.X[(size_t)n * 3]), n});
      }
    std::sort(nb.begin(), nb.end());
    nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
    if ((int)nb.size() > S) continue;
    // slot of a neighbour node in nb (every node of ent's elements is there)
    auto slot_of = [&](int n) {
      int i = 0;
      while (nb[(size_t)i].second != n) i++;
      return i;
    };
    key.clear();
    key.push_back((int64_t)nb.size());
    for (const Ent& e : ent) {
      key.push_back(p.fe_cls[e.fe]);
      key.push_back(e.al);
      for (int a = 0; a < nen; a++) key.push_back(slot_of(p.fe_conn[(size_t)e.fe * 8 + a]));
    }
    auto f = classes.find(key);
    int cls;
    if (f == classes.end()) {
      cls = (int)classes.size();
      classes.emplace(key, cls);
      std::vector<double> blk((size_t)S * D * D, 0.0);
      for (const Ent& e : ent) {
        const double* K = &p.ke[(size_t)p.fe_cls[e.fe] * nd * nd];
        for (int a = 0; a < nen; a++) {
          const int sl = slot_of(p.fe_conn[(size_t)e.fe * 8 + a]);
          for (int r = 0; r < D; r++)
            for (int c = 0; c < D; c++) blk[(size_t)sl * D * D + r * D + c] += K[(e.al * D + r) * nd + a * D + c];
        }
      }
      p.st_blk.insert(p.st_blk.end(), blk.begin(), blk.end());
    } else {
      cls = f->second;
    }
    p.st_cls[it] = cls;
    for (size_t i = 0; i < nb.size(); i++) p.st_nbr[(size_t)it * S + i] = nb[i].second;
  }
  p.n_st_cls = (int)classes.size();
  // worth it only when classes are shared
  if (p.n_st_cls == 0 || (int64_t)p.n_st_cls * 8 > nfo || p.n_st_cls > 4096) {
    std::fill(p.st_cls.begin(), p.st_cls.end(), -1);
    p.st_blk.clear();
    p.n_st_cls = 0;
  }
  // Neighbour lists as offsets from the node (node numbering that repeats,
  // as on structured meshes): nodes with equal offset lists share one delta
  // class, and the kernel reads a class index instead of S node ids.
  p.st_dcls.assign(nfo, -1);
  p.st_delta.clear();
  p.n_st_dcls = 0;
  if (p.n_st_cls > 0) {
    std::unordered_map<std::vector<int64_t>, int, VecHash> dcl;
    std::vector<int64_t> key(S);
    for (int it = 0; it < nfo; it++) {
      if (p.st_cls[it] < 0) continue;
      const int k = p.feonly[it];
      for (int i = 0; i < S; i++) {
        const int j = p.st_nbr[(size_t)it * S + i];
        key[i] = j < 0 ? INT32_MIN : (int64_t)j - k;
      }
      auto f = dcl.find(key);
      if (f == dcl.end()) {
        f = dcl.emplace(key, (int)dcl.size()).first;
        for (int i = 0; i < S; i++) p.st_delta.push_back((int)key[i]);
      }
      p.st_dcls[it] = f->second;
    }
    p.n_st_dcls = (int)dcl.size();
  }
  p.st_use_delta = p.n_st_cls > 0 && (int64_t)p.n_st_dcls * 8 <= nfo && p.n_st_dcls <= 65536;
}

}  // namespace

// Lattice tiles of the FE-only nodes of a 2D model for the mixed step kernel.
// Applies when every node sits on a regular lattice (per-axis spacing, to
// 1e-6 of a spacing), every FE-only node has a stencil class whose
// neighbours lie at lattice offsets in {-1, 0, 1}^2, and the nodes present
// along any lattice row are numbered consecutively in x (meshes written row
// by row, holes removed).  A tile of Tile2::X x Tile2::Y sites is stored as
// the staged box's rows (first node id, presence bits) and one class entry
// per site; the kernel finds a site's node as the row's first id plus the
// number of present sites before it.  Anything else leaves n_tiles = 0 (the
// per-node stencil path).  3D models keep the per-node path: tiles of
// 4 x 4 x 4 nodes with four lanes per node measured slower on the GB300
// (26.8 against 23.5 us per step on a 121 x 61 x 21-node box without PD
// zone), the 27-point stencil's chain of dependent loads being the bound.
void build_fe_tiles(const Mesh& me, const Setup& s, Prepared& p) {
  using T = Tile2;
  const int D = me.dim, N = me.n_node;
  const int nfo = (int)p.feonly.size();
  p.tile_rows.clear();
  p.tile_cls.clear();
  p.lat_blk.clear();
  p.fe_rest.clear();
  p.n_tiles = 0;
  if (D != 2 || nfo == 0 || p.n_st_cls == 0 || p.n_st_cls > kTileClsMask) return;
  for (int it = 0; it < nfo; it++)
    if (p.st_cls[it] < 0) return;
  // lattice: per axis, the least spacing between distinct coordinates
  int64_t dims[2] = {1, 1};
  std::vector<int64_t> lc((size_t)N * 2, 0);
  for (int a = 0; a < 2; a++) {
    std::vector<double> v(N);
    for (int k = 0; k < N; k++) v[k] = me.X[(size_t)k * 3 + a];
    std::sort(v.begin(), v.end());
    const double range = v.back() - v.front();
    if (!(range > 0)) return;
    double h = range;
    for (int k = 1; k < N; k++) {
      const double d = v[k] - v[k - 1];
      if (d > 1e-9 * range) h = std::min(h, d);
    }
    for (int k = 0; k < N; k++) {
      const double q = (me.X[(size_t)k * 3 + a] - v.front()) / h;
      const int64_t i = std::llround(q);
      if (std::fabs(q - (double)i) > 1e-6) return;
      lc[(size_t)k * 2 + a] = i;
      dims[a] = std::max(dims[a], i + 1);
    }
  }
  if (dims[0] * dims[1] > (int64_t)64 * N + 1024) return;   // too sparse a lattice
  std::vector<int> node_at((size_t)(dims[0] * dims[1]), -1);
  for (int k = 0; k < N; k++) {
    int& slot = node_at[(size_t)(lc[(size_t)k * 2] + dims[0] * lc[(size_t)k * 2 + 1])];
    if (slot >= 0) return;   // two nodes on one site
    slot = k;
  }
  // class slots by lattice offset, the same for every node of a class
  const int S = kStencil2;
  std::vector<int> slot_off((size_t)p.n_st_cls * S, -2);   // -2 unknown, -1 empty
  for (int it = 0; it < nfo; it++) {
    const int k = p.feonly[it], c = p.st_cls[it];
    for (int q = 0; q < S; q++) {
      const int n = p.st_nbr[(size_t)it * S + q];
      int o = -1;
      if (n >= 0) {
        const int dx = (int)(lc[(size_t)n * 2] - lc[(size_t)k * 2]);
        const int dy = (int)(lc[(size_t)n * 2 + 1] - lc[(size_t)k * 2 + 1]);
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1) return;
        o = (dx + 1) + 3 * (dy + 1);
      }
      int& so = slot_off[(size_t)c * S + q];
      if (so == -2) so = o;
      else if (so != o) return;
    }
  }
  // nodes whose FP32 record the PD part of the step reads: family members
  // and the nodes of the elements around PD nodes
  std::vector<uint8_t> shadow(N, 0);
  for (int64_t q = 0; q < (int64_t)s.fam_members.size(); q++) shadow[s.fam_members[q]] = 1;
  for (int k : s.fam_node)
    for (int j = p.fe_adj_ptr[k]; j < p.fe_adj_ptr[k + 1]; j++) {
      const int e = p.fe_adj[j] >> 3;
      for (int a = 0; a < 4; a++) shadow[p.fe_conn[(size_t)e * 8 + a]] = 1;
    }
  std::vector<int> cls_of(N, -1);
  for (int it = 0; it < nfo; it++) cls_of[p.feonly[it]] = p.st_cls[it];
  std::vector<int> rows_all;
  std::vector<int16_t> cls_all;
  std::vector<int> rows(T::ROWS * 2);
  std::vector<int16_t> cls(T::NODES);
  int64_t covered = 0;
  int n_tiles = 0;
  const int64_t ntx = (dims[0] + T::X - 1) / T::X, nty = (dims[1] + T::Y - 1) / T::Y;
  for (int64_t ty = 0; ty < nty; ty++)
    for (int64_t tx = 0; tx < ntx; tx++) {
      const int64_t i0 = tx * T::X, j0 = ty * T::Y;
      int here = 0;
      for (int y = 0; y < T::Y; y++)
        for (int x = 0; x < T::X; x++) {
          const int64_t i = i0 + x, j = j0 + y;
          int16_t c = -1;
          if (i < dims[0] && j < dims[1]) {
            const int n = node_at[(size_t)(i + dims[0] * j)];
            if (n >= 0 && cls_of[n] >= 0) {
              c = (int16_t)(cls_of[n] | (shadow[n] ? kTileShadowBit : 0));
              here++;
            }
          }
          cls[(size_t)x + T::X * y] = c;
        }
      if (!here) continue;
      for (int y = 0; y < T::WY; y++) {
        const int64_t j = j0 + y - 1;
        int base = 0, nprev = -1;
        uint32_t mask = 0;
        for (int x = 0; x < T::WX; x++) {
          const int64_t i = i0 + x - 1;
          if (i < 0 || j < 0 || i >= dims[0] || j >= dims[1]) continue;
          const int n = node_at[(size_t)(i + dims[0] * j)];
          if (n < 0) continue;
          if (nprev < 0) base = n;
          else if (n != nprev + 1) return;   // a row not numbered consecutively: no tiles
          nprev = n;
          mask |= 1u << x;
        }
        rows[(size_t)y * 2] = base;
        rows[(size_t)y * 2 + 1] = (int)mask;
      }
      rows_all.insert(rows_all.end(), rows.begin(), rows.end());
      cls_all.insert(cls_all.end(), cls.begin(), cls.end());
      n_tiles++;
      covered += here;
    }
  if (covered != nfo) return;
  p.lat_blk.assign((size_t)p.n_st_cls * T::SLOTS * T::BW, 0.f);
  for (int c = 0; c < p.n_st_cls; c++)
    for (int q = 0; q < S; q++) {
      const int o = slot_off[(size_t)c * S + q];
      if (o < 0) continue;
      for (int e = 0; e < 4; e++)
        p.lat_blk[((size_t)c * T::SLOTS + o) * T::BW + e] = (float)p.st_blk[((size_t)c * S + q) * 4 + e];
    }
  p.tile_rows.swap(rows_all);
  p.tile_cls.swap(cls_all);
  p.n_tiles = n_tiles;
}

bool prepare_model(pdx_model* m, Error& err, bool step_tables) {
  const Mesh& me = m->mesh;
  const Setup& s = m->setup;
  const Command& c = m->cmd;
  Prepared& p = m->prep;
  const int D = me.dim, N = me.n_node;
  const int NV = D == 2 ? 3 : 6;
  material_D(me, p.D, p.lambda, p.mu);
  // lumped mass over all elements, in element order
  p.mass_node.assign(N, 0.0);
  for (int e = 0; e < me.n_elem; e++) {
    const int nn = me.elem_nn[e];
    const double dv = s.vol_elem[e] / nn;
    for (int i = 0; i < nn; i++) {
      const int n = me.conn[(size_t)e * 8 + i];
      p.mass_node[n] = p.mass_node[n] + dv * me.rho;
    }
  }
  p.mass_eq.assign(s.n_eq, 0.0);
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++)
      if (s.eq[(size_t)k * D + i] >= 0) p.mass_eq[s.eq[(size_t)k * D + i]] = p.mass_node[k];
  // prescribed DOFs
  p.bcflag.assign(N, 0);
  p.dtv.assign((size_t)N * 3, 0.0);
  p.u0.assign((size_t)N * D, 0.0);
  for (const auto& b : me.ebcs)
    for (int n : b.nodes) {
      p.u0[(size_t)n * D + b.dof] = b.value;
      if (b.varying) {
        p.bcflag[n] |= (uint8_t)(1u << b.dof);
        p.dtv[(size_t)n * 3 + b.dof] = c.dt * b.velocity;
      }
    }
  // bit 4 + i: DOF i has no equation (prescribed), so the update needs no eq
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++)
      if (s.eq[(size_t)k * D + i] < 0) p.bcflag[k] |= (uint8_t)(1u << (4 + i));
  // bonds
  const int nf = (int)s.fam_node.size();
  p.fam_ptr.assign(nf + 1, 0);
  p.nbr.clear();
  std::vector<uint8_t> st;
  for (int f = 0; f < nf; f++) {
    for (int64_t q = s.fam_off[f] + 1; q < s.fam_off[f + 1]; q++) {
      p.nbr.push_back(s.fam_members[q]);
      st.push_back(s.bond_state[q]);
    }
    p.fam_ptr[f + 1] = (int)p.nbr.size();
    if (s.fam_off[f + 1] - s.fam_off[f] < 2) { err.code = 6; err.msg = "a PD family has no member"; return false; }
  }
  const int64_t nb = (int64_t)p.nbr.size();
  p.state_bits.assign((size_t)(nb + 31) / 32 + 1, 0u);
  p.fam_intact.assign(nf, 0);
  for (int f = 0; f < nf; f++)
    for (int b = p.fam_ptr[f]; b < p.fam_ptr[f + 1]; b++)
      if (st[b]) { p.state_bits[b >> 5] |= 1u << (b & 31); p.fam_intact[f]++; }
  // the damage test of failureCriterion_stretch, phi = 1 - intact/(n-1) > 0.42,
  // evaluated once per possible intact count so the kernel compares integers
  p.fam_brk.assign(nf, 0);
  for (int f = 0; f < nf; f++) {
    const int nbf = p.fam_ptr[f + 1] - p.fam_ptr[f];
    int t = nbf + 1;
    for (int i = 0; i <= nbf; i++)
      if (!(1.0 - (double)i / ((double)(nbf + 1) - 1.0) > 0.42)) { t = i; break; }
    p.fam_brk[f] = t;
  }
  p.fam_s0.assign(nf, c.s0);
  p.dt2m.assign(N, 0.0);
  for (int k = 0; k < N; k++)
    if (p.mass_node[k] > 0) p.dt2m[k] = c.dt * c.dt / p.mass_node[k];
  // PD-boundary weights W per node
  std::vector<std::vector<double>> W(N);
  auto addW = [&](int n, const double* w) {
    if (W[n].empty()) W[n].assign((size_t)D * NV, 0.0);
    for (int i = 0; i < D * NV; i++) W[n][i] += w[i];
  };
  for (const auto& b : s.pdbe) {
    if (D == 2) {
      const double* x1 = &me.X[(size_t)b[0] * 3];
      const double* x2 = &me.X[(size_t)b[1] * 3];
      const double nx = x2[1] - x1[1], ny = x1[0] - x2[0];
      const double w[6] = {0.5 * nx, 0.0, 0.5 * ny, 0.0, 0.5 * ny, 0.5 * nx};
      addW(b[0], w);
      addW(b[1], w);
    } else {
      double xN[4][3];
      for (int i = 0; i < 4; i++)
        for (int a = 0; a < 3; a++) xN[i][a] = me.X[(size_t)b[i] * 3 + a];
      const bool quad = b[3] != b[2];
      double Nm[3][6];
      bool ok;
      norm_mat_area(xN, quad, Nm, ok);
      if (!ok) { err.code = 2; err.msg = "Area is zero!"; return false; }
      const int nn = quad ? 4 : 3;
      for (int i = 0; i < nn; i++) addW(b[i], &Nm[0][0]);
    }
  }
  p.fam_corr.assign(nf, -1);
  p.fam_wd.assign(nf, -1);
  p.wd.clear();
  p.n_corr = 0;
  for (int f = 0; f < nf; f++) {
    const int k = s.fam_node[f];
    if (W[k].empty()) continue;
    p.fam_wd[f] = (int)(p.wd.size() / ((size_t)D * NV));
    for (int i = 0; i < D; i++)
      for (int j = 0; j < NV; j++) {
        double acc = 0;
        for (int t = 0; t < NV; t++) acc += W[k][(size_t)i * NV + t] * p.D[(size_t)t * NV + j];
        p.wd.push_back(acc);
      }
    p.fam_corr[f] = (int)p.n_corr;
    p.n_corr += p.fam_ptr[f + 1] - p.fam_ptr[f];
  }
  // FE-only nodes; families and FE-only nodes are handed to the step kernel in
  // spatial tiles (4x4x4 in 3D, 8x8 in 2D, tile edge in units of the smallest
  // element size) so that the neighbours one thread block gathers fit in L1
  p.feonly.clear();
  for (int k = 0; k < N; k++)
    if (s.node_type[k] == 0) p.feonly.push_back(k);
  {
    const double tile = (D == 3 ? 4.0 : 8.0) * s.min_delta;
    auto key = [&](int k) {
      int64_t t[3], r[3];
      for (int a = 0; a < 3; a++) {
        const double x = (me.X[(size_t)k * 3 + a] - s.lbc[a]) / tile;
        t[a] = (int64_t)std::floor(x);
        r[a] = (int64_t)std::floor((x - (double)t[a]) * 64.0);
      }
      return std::array<int64_t, 7>{t[2], t[1], t[0], r[2], r[1], r[0], (int64_t)k};
    };
    std::vector<std::array<int64_t, 7>> kf(nf);
    for (int f = 0; f < nf; f++) kf[f] = key(s.fam_node[f]);
    p.fam_order.resize(nf);
    for (int f = 0; f < nf; f++) p.fam_order[f] = f;
    std::sort(p.fam_order.begin(), p.fam_order.end(), [&](int a, int b) { return kf[a] < kf[b]; });
    std::vector<std::array<int64_t, 7>> ke(p.feonly.size());
    for (size_t i = 0; i < p.feonly.size(); i++) ke[i] = key(p.feonly[i]);
    std::vector<int> idx(p.feonly.size());
    for (size_t i = 0; i < idx.size(); i++) idx[i] = (int)i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return ke[a] < ke[b]; });
    std::vector<int> tmp(p.feonly.size());
    for (size_t i = 0; i < idx.size(); i++) tmp[i] = p.feonly[idx[i]];
    p.feonly.swap(tmp);
  }
  // FE elements and stiffness classes
  const int nen = D == 2 ? 4 : 8;
  const int nd = nen * D;
  const int ngp = nen;
  const int nfe = (int)s.fe.size();
  p.fe_conn.assign((size_t)nfe * 8, 0);
  p.fe_cls.assign(nfe, 0);
  p.ke.clear(); p.me.clear(); p.bgp.clear();
  std::unordered_map<std::vector<int64_t>, int, VecHash> classes;
  for (int i = 0; i < nfe; i++) {
    const int e = s.fe[i];
    const bool tri = me.elem_nn[e] == 3;   // stored with its third node repeated in the fourth slot
    double xN[8][3];
    for (int j = 0; j < nen; j++) {
      const int n = me.conn[(size_t)e * 8 + (tri && j == 3 ? 2 : j)];
      p.fe_conn[(size_t)i * 8 + j] = n;
      for (int a = 0; a < 3; a++) xN[j][a] = me.X[(size_t)n * 3 + a];
    }
    double Le = 0;
    for (int j = 1; j < nen; j++)
      for (int a = 0; a < 3; a++) Le = std::max(Le, std::fabs(xN[j][a] - xN[0][a]));
    const double q = Le > 0 ? 1e-12 * Le : 1.0;
    std::vector<int64_t> key;
    key.reserve(nen * 3);
    for (int j = 1; j < nen; j++)
      for (int a = 0; a < 3; a++) key.push_back(std::llround((xN[j][a] - xN[0][a]) / q));
    key.push_back(std::llround(std::log2(q) * 1e6));
    key.push_back(me.elem_nn[e]);
    auto it = classes.find(key);
    int cls;
    if (it == classes.end()) {
      cls = (int)classes.size();
      classes.emplace(key, cls);
      std::vector<double> K((size_t)nd * nd), Me((size_t)nd * nd), B((size_t)ngp * NV * nd);
      if (D == 2) {
        double x4[4][3];
        std::memcpy(x4, xN, sizeof(x4));
        if (tri) {
          ke_tri3(x4, p.D.data(), K.data());
          me_tri3(x4, me.rho, Me.data());
          b_gauss_tri3(x4, B.data());
        } else {
          ke_quad4(x4, p.D.data(), K.data());
          me_quad4(x4, me.rho, Me.data());
          b_gauss_quad4(x4, B.data());
        }
      } else {
        ke_hex8(xN, p.D.data(), K.data());
        me_hex8(xN, me.rho, Me.data());
        b_gauss_hex8(xN, B.data());
      }
      p.ke.insert(p.ke.end(), K.begin(), K.end());
      p.me.insert(p.me.end(), Me.begin(), Me.end());
      p.bgp.insert(p.bgp.end(), B.begin(), B.end());
    } else {
      cls = it->second;
    }
    p.fe_cls[i] = cls;
  }
  p.n_cls = (int)classes.size();
  p.L.assign((size_t)ngp * ngp, 0.0);
  extrap_L(D, p.L.data());
  // node -> FE element adjacency, in FE element order (a triangle's repeated
  // fourth slot is not an adjacency: its rows are zero)
  auto slots = [&](int i) { return me.elem_nn[s.fe[i]] == 3 ? 3 : nen; };
  p.fe_adj_ptr.assign(N + 1, 0);
  for (int i = 0; i < nfe; i++)
    for (int j = 0; j < slots(i); j++) p.fe_adj_ptr[p.fe_conn[(size_t)i * 8 + j] + 1]++;
  for (int k = 0; k < N; k++) p.fe_adj_ptr[k + 1] += p.fe_adj_ptr[k];
  p.fe_adj.assign(p.fe_adj_ptr[N], 0);
  {
    std::vector<int> fill(p.fe_adj_ptr.begin(), p.fe_adj_ptr.end() - 1);
    for (int i = 0; i < nfe; i++)
      for (int j = 0; j < slots(i); j++) {
        const int n = p.fe_conn[(size_t)i * 8 + j];
        p.fe_adj[fill[n]++] = (i << 3) | j;
      }
  }
  for (int k = 0; k < N; k++)
    if (p.fe_adj_ptr[k + 1] - p.fe_adj_ptr[k] > kMaxFeAdj && D == 3) {
      err.code = 3; err.msg = "more than 8 FE elements around a node"; return false;
    }
  // node stencils and lattice tiles of FE-only nodes: tables of the explicit
  // step only (without them it takes the element path, same results)
  if (step_tables) {
    build_stencils(me, p);
    build_fe_tiles(me, s, p);
  }
  // traction BCs: unit forces per node and NBC
  {
    std::map<std::pair<int, int>, std::array<double, 3>> acc;
    for (size_t bi = 0; bi < me.nbcs.size(); bi++)
      for (const auto& el : me.nbcs[bi].elems) {
        double xN[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        const int nn = D == 2 ? 2 : 4;
        for (int j = 0; j < nn; j++)
          for (int a = 0; a < 3; a++) xN[j][a] = me.X[(size_t)el[j] * 3 + a];
        double Fe[12];
        nbc_unit_force(D, xN, Fe);
        for (int j = 0; j < nn; j++) {
          auto& v = acc[{el[j], (int)bi}];
          for (int a = 0; a < D; a++) v[a] += Fe[j * D + a];
        }
      }
    p.ext_ptr.assign(N + 1, 0);
    p.ext_nbc.clear();
    p.ext_f.clear();
    for (const auto& kv : acc) p.ext_ptr[kv.first.first + 1]++;
    for (int k = 0; k < N; k++) p.ext_ptr[k + 1] += p.ext_ptr[k];
    p.ext_nbc.assign(acc.size(), 0);
    p.ext_f.assign(acc.size() * 3, 0.0);
    std::vector<int> fill(p.ext_ptr.begin(), p.ext_ptr.end() - 1);
    for (const auto& kv : acc) {
      const int slot = fill[kv.first.first]++;
      p.ext_nbc[slot] = kv.first.second;
      for (int a = 0; a < 3; a++) p.ext_f[(size_t)slot * 3 + a] = kv.second[a];
    }
  }
  // scatter map: offset of every neighbour's first column inside a node's rows
  // (none without a CSR pattern: batch specimens).  Equations are numbered in
  // node order, so a row's columns are sorted by node, and the offset of node
  // n's first column in node k's rows is the number of the row's columns
  // below n's first equation (eq_start[n]); all rows of a node have the same
  // columns.  A node without a row (every DOF prescribed) is never written.
  if (!s.csr_ia.empty()) {
    std::vector<int64_t> eq_start((size_t)N + 1, 0);
    std::vector<int64_t> first_row(N, -1);
    for (int k = 0; k < N; k++) {
      int64_t c = 0;
      for (int d = 0; d < D; d++) {
        const int e = s.eq[(size_t)k * D + d];
        if (e < 0) continue;
        if (first_row[k] < 0) first_row[k] = e;
        c++;
      }
      eq_start[k + 1] = eq_start[k] + c;
    }
    auto lookup = [&](int k, int n) -> int {
      const int64_t r = first_row[k];
      if (r < 0) return 0;
      const int64_t* b = s.csr_ja.data() + s.csr_ia[r];
      const int64_t* e = s.csr_ja.data() + s.csr_ia[r + 1];
      return (int)(std::lower_bound(b, e, eq_start[n]) - b);
    };
    p.rel_bond.assign(nb, 0);
    p.rel_self.assign(nf, 0);
    for (int f = 0; f < nf; f++) {
      const int k = s.fam_node[f];
      p.rel_self[f] = lookup(k, k);
      for (int b = p.fam_ptr[f]; b < p.fam_ptr[f + 1]; b++) p.rel_bond[b] = lookup(k, p.nbr[b]);
    }
    p.rel_fe.assign((size_t)p.fe_adj.size() * 8, 0);
    for (int k = 0; k < N; k++)
      for (int j = p.fe_adj_ptr[k]; j < p.fe_adj_ptr[k + 1]; j++) {
        const int i = p.fe_adj[j] >> 3;
        for (int a = 0; a < nen; a++) p.rel_fe[(size_t)j * 8 + a] = lookup(k, p.fe_conn[(size_t)i * 8 + a]);
      }
  }
  return true;
}

}  // namespace pdx
