// Model setup: the order-dependent steps of pdsolve::setDatModel
// (SourceFiles/Solver/pdsolve.cpp:114-151), restated on plain arrays so that
// families, bond states, PD boundary elements (PDBEs) and the CSR pattern
// come out identical to the reference's:
//   DOF numbering          Setdof_Index          pdsolve.cpp:241-268
//   volumes, min/max delta setDeltaMaxMin_EleV_NV :367-439
//   domain box             findDomainDimen       :153-195
//   block hash             setBlock              :441-502
//   PD/FE split + cracks   initializePDE_FE, updatePDEbyCrack, b_eleIntersectCrack :504-822
//   PDBEs                  updatePDBE, assignPDBE :1221-1413, :1703-1771
//   node types             UpdateNodeType        :1415-1440
//   families (union rule)  initialPDN_Fami       :1442-1568
//   pre-crack bond states  initialBondState, updateBondstate :1823-1915, :8910-9004
//   crack geometry tests   intersection, segmentPlaneIntersection :9058-9079, :1123-1210
//   CSR pattern            setCSRIndexes_gloStiffMat :959-1121
// Floating-point expressions that decide membership (distances, horizons)
// are written in the same operation order; the file is compiled without
// FP contraction so x86 and Arm hosts agree.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>

#include "model.h"

namespace pdx {

namespace {

bool seg_intersect_2d(const double* a1, const double* a2, const double* b1, const double* b2) {
  if ((a1[0] > a2[0] ? a1[0] : a2[0]) < (b1[0] < b2[0] ? b1[0] : b2[0]) ||
      (a1[1] > a2[1] ? a1[1] : a2[1]) < (b1[1] < b2[1] ? b1[1] : b2[1]) ||
      (b1[0] > b2[0] ? b1[0] : b2[0]) < (a1[0] < a2[0] ? a1[0] : a2[0]) ||
      (b1[1] > b2[1] ? b1[1] : b2[1]) < (a1[1] < a2[1] ? a1[1] : a2[1]))
    return false;
  if ((((a1[0] - b1[0]) * (b2[1] - b1[1]) - (a1[1] - b1[1]) * (b2[0] - b1[0])) *
       ((a2[0] - b1[0]) * (b2[1] - b1[1]) - (a2[1] - b1[1]) * (b2[0] - b1[0]))) > 0 ||
      (((b1[0] - a1[0]) * (a2[1] - a1[1]) - (b1[1] - a1[1]) * (a2[0] - a1[0])) *
       ((b2[0] - a1[0]) * (a2[1] - a1[1]) - (b2[1] - a1[1]) * (a2[0] - a1[0]))) > 0)
    return false;
  return true;
}

void cross(const double* a, const double* b, double* n) {
  n[0] = a[1] * b[2] - a[2] * b[1];
  n[1] = a[2] * b[0] - a[0] * b[2];
  n[2] = a[0] * b[1] - a[1] * b[0];
}

// Segment p1-p2 against the triangle t (3 points).  A segment end point on the
// triangle's plane counts as crossing wherever it lies (the reference's rule).
bool seg_tri_3d(const double* p1, const double* p2, const double* t) {
  double v1[3], v2[3], nrm[3];
  for (int i = 0; i < 3; i++) { v1[i] = t[3 + i] - t[i]; v2[i] = t[6 + i] - t[i]; }
  cross(v1, v2, nrm);
  for (int i = 0; i < 3; i++) { v1[i] = p1[i] - t[i]; v2[i] = p2[i] - t[i]; }
  double t1 = v1[0] * nrm[0] + v1[1] * nrm[1] + v1[2] * nrm[2];
  double t2 = v2[0] * nrm[0] + v2[1] * nrm[1] + v2[2] * nrm[2];
  if (t1 * t2 > 0) return false;
  if (t1 * t2 == 0) return true;
  double w1[3], w2[3];
  for (int i = 0; i < 3; i++) { w1[i] = t[i] - p1[i]; w2[i] = p2[i] - p1[i]; }
  double d = (w1[0] * nrm[0] + w1[1] * nrm[1] + w1[2] * nrm[2]) / (w2[0] * nrm[0] + w2[1] * nrm[1] + w2[2] * nrm[2]);
  double xs[3];
  for (int i = 0; i < 3; i++) xs[i] = p1[i] + d * w2[i];
  double A = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  double n2[3];
  for (int i = 0; i < 3; i++) { v1[i] = t[3 + i] - xs[i]; v2[i] = t[6 + i] - xs[i]; }
  cross(v1, v2, n2);
  double A0 = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
  for (int i = 0; i < 3; i++) { v1[i] = xs[i] - t[i]; v2[i] = t[6 + i] - t[i]; }
  cross(v1, v2, n2);
  double A1 = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
  for (int i = 0; i < 3; i++) { v1[i] = t[3 + i] - t[i]; v2[i] = xs[i] - t[i]; }
  cross(v1, v2, n2);
  double A2 = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
  return !(std::fabs(A0 + A1 + A2 - A) > A * 1.0e-14);
}

struct Ctx {
  const Mesh& m;
  Setup& s;
  std::vector<int> algo;
  std::vector<int> crack_elems;
  const double* X(int n) const { return &m.X[(size_t)n * 3]; }
  int block_of(const double* x, int ib[3]) const {
    for (int i = 0; i < 3; i++) ib[i] = (int)((x[i] - s.lbc[i]) / s.block_size);
    return ib[0] + ib[1] * s.nblocks[0] + ib[2] * s.nblocks[0] * s.nblocks[1];
  }
  bool in_range(int x, int y, int z) const {
    return x >= 0 && x < s.nblocks[0] && y >= 0 && y < s.nblocks[1] && z >= 0 && z < s.nblocks[2];
  }
  int bindex(int x, int y, int z) const { return x + y * s.nblocks[0] + z * s.nblocks[0] * s.nblocks[1]; }
  void crack_block_range(const std::array<double, 9>& cr, int lo[3], int hi[3]) const {
    const int fn = m.dim;
    for (int k = 0; k < 3; k++) {
      double mn = cr[k], mx = cr[k];
      for (int p = 1; p < fn; p++) { mn = std::min(mn, cr[p * 3 + k]); mx = std::max(mx, cr[p * 3 + k]); }
      lo[k] = (int)((mn - s.lbc[k]) / s.block_size);
      hi[k] = (int)((mx - s.lbc[k]) / s.block_size);
    }
    if (m.dim == 2) { lo[2] = 0; hi[2] = 0; }
  }
  bool elem_cut(int e, const std::array<double, 9>& cr) const {
    const int* c = &m.conn[(size_t)e * 8];
    if (m.dim == 2) {
      const int nn = m.elem_nn[e];
      for (int i = 0; i < nn; i++)
        if (seg_intersect_2d(X(c[i]), X(c[(i + 1) % nn]), &cr[0], &cr[3])) return true;
      return false;
    }
    static const int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4},
                                    {0, 4}, {1, 5}, {2, 6}, {3, 7}};
    for (int i = 0; i < 12; i++)
      if (seg_tri_3d(X(c[edge[i][0]]), X(c[edge[i][1]]), cr.data())) return true;
    return false;
  }
};

// Crack-cut elements of segment `cr` not found before are appended to
// cx.crack_elems (updatePDEbyCrack, first half); returns how many.
size_t update_pde_by_crack(Ctx& cx, const std::array<double, 9>& cr) {
  Setup& s = cx.s;
  int lo[3], hi[3];
  cx.crack_block_range(cr, lo, hi);
  const size_t old = cx.crack_elems.size();
  for (int x = lo[0] - 1; x < hi[0] + 2; x++)
    for (int y = lo[1] - 1; y < hi[1] + 2; y++)
      for (int z = lo[2] - 1; z < hi[2] + 2; z++) {
        if (!cx.in_range(x, y, z)) continue;
        for (int e : s.block_elems[cx.bindex(x, y, z)])
          if (cx.elem_cut(e, cr) &&
              std::find(cx.crack_elems.begin(), cx.crack_elems.end(), e) == cx.crack_elems.end())
            cx.crack_elems.push_back(e);
      }
  return cx.crack_elems.size() - old;
}

// The second half of updatePDEbyCrack: FE elements whose centres lie within
// me * min_delta of a crack element found since `old` become PD, appended to
// s.pde in block order.
void pde_near_crack_elems(Ctx& cx, size_t old, double me) {
  Setup& s = cx.s;
  const Mesh& m = cx.m;
  const size_t n = cx.crack_elems.size() - old;
  if (n == 0) return;
  std::vector<std::array<double, 3>> cc(n);
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (size_t i = 0; i < n; i++) {
    elem_center(m, cx.crack_elems[old + i], cc[i].data());
    for (int a = 0; a < 3; a++) { mn[a] = std::min(mn[a], cc[i][a]); mx[a] = std::max(mx[a], cc[i][a]); }
  }
  int blo[3], bhi[3];
  for (int i = 0; i < 3; i++) {
    blo[i] = (int)((mn[i] - s.lbc[i]) / s.block_size);
    bhi[i] = (int)((mx[i] - s.lbc[i]) / s.block_size);
  }
  const double mf = me + 1e-15;
  const double Rsq = s.min_delta * s.min_delta * mf * mf;
  for (int x = blo[0] - 1; x < bhi[0] + 2; x++)
    for (int y = blo[1] - 1; y < bhi[1] + 2; y++)
      for (int z = blo[2] - 1; z < bhi[2] + 2; z++) {
        if (!cx.in_range(x, y, z)) continue;
        for (int e : s.block_elems[cx.bindex(x, y, z)]) {
          if (cx.algo[e] != 2) continue;
          double c[3];
          elem_center(m, e, c);
          for (size_t i = 0; i < n; i++) {
            const double dis = (c[0] - cc[i][0]) * (c[0] - cc[i][0]) + (c[1] - cc[i][1]) * (c[1] - cc[i][1]) +
                               (c[2] - cc[i][2]) * (c[2] - cc[i][2]);
            if (dis < Rsq) { cx.algo[e] = 1; s.pde.push_back(e); break; }
          }
        }
      }
}

// PDBEs (element edges in 2D, faces in 3D of PD elements not shared by two PD
// elements) and node types (2 PD, 1 on a PDBE, 0 FE) of the current s.pde.
// The set of PDBEs is what the reference keeps after its incremental updates
// too (an edge or face is shared by at most two elements); the kernels use it
// through per-node sums of at most two terms in 2D, so its order is free.
void pdbe_and_node_types(const Mesh& m, Setup& s) {
  const int D = m.dim;
  s.pdbe.clear();
  std::vector<std::array<int, 5>> list;
  for (int e : s.pde) {
    const int* c = &m.conn[(size_t)e * 8];
    if (D == 2) {
      const int nn = m.elem_nn[e];
      for (int j = 0; j < nn; j++) {
        const int a = c[j], b = c[(j + 1) % nn];
        if (a < b) list.push_back({a, b, 1, 0, 0});
        else list.push_back({b, a, -1, 0, 0});
      }
    } else {
      const int face[6][4] = {{c[0], c[1], c[2], c[3]}, {c[4], c[5], c[6], c[7]}, {c[0], c[3], c[7], c[4]},
                              {c[1], c[2], c[6], c[5]}, {c[0], c[4], c[5], c[1]}, {c[3], c[7], c[6], c[2]}};
      const int sgn[6] = {-1, 1, -1, 1, -1, 1};
      for (int j = 0; j < 6; j++) {
        const int pos = (int)(std::min_element(face[j], face[j] + 4) - face[j]);
        list.push_back({face[j][pos], face[j][(pos + 1) % 4], face[j][(pos + 2) % 4], face[j][(pos + 3) % 4], sgn[j]});
      }
    }
  }
  std::stable_sort(list.begin(), list.end(), [](const std::array<int, 5>& a, const std::array<int, 5>& b) {
    return a[0] < b[0];
  });
  std::vector<uint8_t> dead(list.size(), 0);
  for (size_t i = 0; i < list.size(); i++) {
    if (dead[i]) continue;
    for (size_t j = i + 1; j < list.size() && list[j][0] == list[i][0]; j++) {
      if (dead[j]) continue;
      const bool same = D == 2 ? list[j][1] == list[i][1]
                               : (list[j][1] == list[i][1] && list[j][2] == list[i][2] && list[j][3] == list[i][3]);
      if (same) { dead[i] = dead[j] = 1; break; }
    }
  }
  for (size_t i = 0; i < list.size(); i++) {
    if (dead[i]) continue;
    const auto& a = list[i];
    if (D == 2) {
      if (a[2] == 1) s.pdbe.push_back({a[0], a[1], -1, -1});
      else s.pdbe.push_back({a[1], a[0], -1, -1});
    } else {
      if (a[4] == 1) s.pdbe.push_back({a[0], a[1], a[2], a[3]});
      else s.pdbe.push_back({a[3], a[2], a[1], a[0]});
    }
  }
  s.node_type.assign(m.n_node, 0);
  for (int e : s.pde)
    for (int i = 0; i < m.elem_nn[e]; i++) s.node_type[m.conn[(size_t)e * 8 + i]] = 2;
  const int pn = D == 2 ? 2 : 4;
  for (const auto& b : s.pdbe)
    for (int i = 0; i < pn; i++) s.node_type[b[i]] = 1;
}

// Members of families f0.. (the union rule of initialPDN_Fami / updatePDN_Fami:
// j joins k's family when within either node's horizon), appended to
// s.fam_members / s.fam_off, which hold families 0..f0-1.
void host_members(const Ctx& cx, int f0, const std::vector<double>& delta_node) {
  Setup& s = cx.s;
  const Mesh& m = cx.m;
  const double md = s.min_delta;
  for (int f = f0; f < (int)s.fam_node.size(); f++) {
    const int k = s.fam_node[f];
    const double dk = s.fam_delta[f];
    const double* xk = &m.X[(size_t)k * 3];
    s.fam_members.push_back(k);
    int ib[3];
    cx.block_of(xk, ib);
    for (int x = ib[0] - 1; x < ib[0] + 2; x++)
      for (int y = ib[1] - 1; y < ib[1] + 2; y++)
        for (int z = ib[2] - 1; z < ib[2] + 2; z++) {
          if (!cx.in_range(x, y, z)) continue;
          for (int j : s.block_nodes[cx.bindex(x, y, z)]) {
            const double* xm = &m.X[(size_t)j * 3];
            const double dj = delta_node[j];
            const double dist = ((xm[0] - xk[0]) * (xm[0] - xk[0]) + (xm[1] - xk[1]) * (xm[1] - xk[1]) +
                                 (xm[2] - xk[2]) * (xm[2] - xk[2]));
            if (dist > md * md * 1.0e-16 &&
                (dist < (dk * dk + md * md * 1.0e-16) || dist < (dj * dj + md * md * 1.0e-16)))
              s.fam_members.push_back(j);
          }
        }
    s.fam_off.push_back((int64_t)s.fam_members.size());
  }
}

std::vector<double> node_horizons(const Mesh& m, const Command& cmd, const Setup& s) {
  std::vector<double> delta_node(m.n_node);
  for (int k = 0; k < m.n_node; k++) delta_node[k] = cmd.factor * std::pow(s.vol_node[k], 1.0 / m.dim);
  return delta_node;
}

// updateBondstate for one crack segment (2D) or triangle (3D)
int cut_bonds(const Ctx& cx, const std::array<double, 9>& cr) {
  Setup& s = cx.s;
  const int D = cx.m.dim;
  int lo[3], hi[3], cut = 0;
  cx.crack_block_range(cr, lo, hi);
  for (int x = lo[0] - 1; x < hi[0] + 2; x++)
    for (int y = lo[1] - 1; y < hi[1] + 2; y++)
      for (int z = lo[2] - 1; z < hi[2] + 2; z++) {
        if (!cx.in_range(x, y, z)) continue;
        for (int node : s.block_nodes[cx.bindex(x, y, z)]) {
          const int f = s.fam_of_node[node];
          if (f < 0) continue;
          const int k = s.fam_node[f];
          for (int64_t p = s.fam_off[f] + 1; p < s.fam_off[f + 1]; p++) {
            if (s.bond_state[p] != 1) continue;
            const int mm = s.fam_members[p];
            const bool c = D == 3 ? seg_tri_3d(cx.X(k), cx.X(mm), cr.data())
                                  : seg_intersect_2d(cx.X(k), cx.X(mm), &cr[0], &cr[3]);
            if (c) { s.bond_state[p] = 0; cut++; }
          }
        }
      }
  return cut;
}

// The CSR pattern after the element types of the nodes in `nodes` (sorted,
// unique) changed: only those nodes' rows change (a row holds the node's own
// family members and the nodes of the FE elements around it), so their
// column sets are recomputed and every other row is copied.
void update_csr_rows(const Ctx& cx, const std::vector<int>& nodes) {
  Setup& s = cx.s;
  const Mesh& m = cx.m;
  const int D = m.dim;
  std::vector<std::vector<int>> cols(nodes.size());
  for (size_t i = 0; i < nodes.size(); i++) {
    const int k = nodes[i];
    std::vector<int>& v = cols[i];
    const int f = s.fam_of_node[k];
    if (f >= 0) v.assign(s.fam_members.begin() + s.fam_off[f], s.fam_members.begin() + s.fam_off[f + 1]);
    for (int q = s.node_elem_ptr[k]; q < s.node_elem_ptr[k + 1]; q++) {
      const int e = s.node_elem[q];
      if (s.algo[e] != 2) continue;
      const int* c = &m.conn[(size_t)e * 8];
      v.insert(v.end(), c, c + m.elem_nn[e]);
    }
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  std::vector<int64_t> ia((size_t)s.n_eq + 1, 0), ja;
  ja.reserve(s.csr_ja.size() + 64 * nodes.size());
  size_t next = 0;
  for (int k = 0; k < m.n_node; k++) {
    const bool changed = next < nodes.size() && nodes[next] == k;
    for (int d = 0; d < D; d++) {
      const int row = s.eq[(size_t)k * D + d];
      if (row < 0) continue;
      if (changed) {
        for (int j : cols[next])
          for (int jj = 0; jj < D; jj++) {
            const int col = s.eq[(size_t)j * D + jj];
            if (col >= 0) ja.push_back(col);
          }
      } else {
        ja.insert(ja.end(), s.csr_ja.begin() + s.csr_ia[row], s.csr_ja.begin() + s.csr_ia[row + 1]);
      }
      ia[(size_t)row + 1] = (int64_t)ja.size();
    }
    if (changed) next++;
  }
  s.csr_ia.swap(ia);
  s.csr_ja.swap(ja);
}

}  // namespace

bool build_setup(const Mesh& m, const Command& cmd, Setup& s, Error& err, int device, bool pattern) {
  const int D = m.dim, N = m.n_node, E = m.n_elem;
  s = Setup();
  s.dim = D;
  // DOF numbering
  std::vector<uint8_t> active((size_t)N * D, 1);
  for (const auto& b : m.ebcs)
    for (int n : b.nodes) active[(size_t)n * D + b.dof] = 0;
  s.eq.assign((size_t)N * D, -1);
  int cnt = 0;
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++)
      if (active[(size_t)k * D + i]) s.eq[(size_t)k * D + i] = cnt++;
  s.n_eq = cnt;
  // element and node volumes
  s.vol_elem.assign(E, 0.0);
  s.vol_node.assign(N, 0.0);
  double vmax = -std::numeric_limits<double>::max(), vmin = std::numeric_limits<double>::max();
  for (int e = 0; e < E; e++) {
    const double dv = elem_volume(m, e);
    s.vol_elem[e] = dv;
    const int nn = m.elem_nn[e];
    for (int i = 0; i < nn; i++) s.vol_node[m.conn[(size_t)e * 8 + i]] += dv / nn;
    if (dv > vmax) vmax = dv;
    if (dv < vmin) vmin = dv;
  }
  s.min_delta = std::pow(vmin, 1.0 / D);
  s.max_delta = std::pow(vmax, 1.0 / D);
  // domain box
  for (int i = 0; i < 3; i++) s.lbc[i] = s.rtc[i] = m.X[i];
  for (int k = 1; k < N; k++)
    for (int j = 0; j < D; j++) {
      const double v = m.X[(size_t)k * 3 + j];
      if (v < s.lbc[j]) s.lbc[j] = v;
      if (v > s.rtc[j]) s.rtc[j] = v;
    }
  for (int i = 0; i < D; i++) {
    s.lbc[i] = s.lbc[i] - 1.0E-14 * std::fabs(s.lbc[i]);
    s.rtc[i] = s.rtc[i] + 1.0E-14 * std::fabs(s.rtc[i]);
  }
  // blocks
  s.block_size = 2.5 * cmd.factor * s.min_delta;
  for (int i = 0; i < 3; i++) s.nblocks[i] = (int)((s.rtc[i] - s.lbc[i]) / s.block_size + 1);
  if (D == 2) s.nblocks[2] = 1;
  const size_t nb = (size_t)s.nblocks[0] * s.nblocks[1] * s.nblocks[2];
  s.block_nodes.assign(nb, {});
  s.block_elems.assign(nb, {});
  Ctx cx{m, s, m.elem_algo, {}};
  for (int e = 0; e < E; e++) {
    double c[3];
    elem_center(m, e, c);
    int ib[3];
    const int bi = cx.block_of(c, ib);
    if (bi < 0 || (size_t)bi >= nb) { err.code = 2; err.msg = "element centre outside the block grid"; return false; }
    s.block_elems[bi].push_back(e);
  }
  for (int k = 0; k < N; k++) {
    int ib[3];
    const int bi = cx.block_of(&m.X[(size_t)k * 3], ib);
    if (bi < 0 || (size_t)bi >= nb) { err.code = 2; err.msg = "node outside the block grid"; return false; }
    s.block_nodes[bi].push_back(k);
  }
  // PD / FE split, crack-cut FE elements become PD
  for (int e = 0; e < E; e++)
    if (cx.algo[e] == 1) s.pde.push_back(e);
  for (const auto& cr : m.cracks) {
    const size_t old = cx.crack_elems.size();
    if (update_pde_by_crack(cx, cr) == 0) {
      err.code = 2;
      err.msg = "a pre-existing crack cuts no element";
      return false;
    }
    pde_near_crack_elems(cx, old, cmd.me);
  }
  for (int e = 0; e < E; e++)
    if (cx.algo[e] == 2) s.fe.push_back(e);
  pdbe_and_node_types(m, s);
  // families
  s.fam_of_node.assign(N, -1);
  for (int k = 0; k < N; k++)
    if (s.node_type[k]) {
      s.fam_of_node[k] = (int)s.fam_node.size();
      s.fam_node.push_back(k);
      s.fam_delta.push_back(cmd.factor * std::pow(s.vol_node[k], 1.0 / D));
    }
  const int nf = (int)s.fam_node.size();
  s.fam_cdv.assign(nf, 0.0);
  for (int e : s.pde) {
    const double dv = s.vol_elem[e];
    const int nn = m.elem_nn[e];
    for (int i = 0; i < nn; i++) {
      const int f = s.fam_of_node[m.conn[(size_t)e * 8 + i]];
      s.fam_cdv[f] = s.fam_cdv[f] + dv / nn;
    }
  }
  const std::vector<double> delta_node = node_horizons(m, cmd, s);
  if (device >= 0) {
    // the same search, one warp per family, on the model's GPU (k_setup.cu)
    if (!gpu_family_search(m, s, delta_node, s.min_delta, device, err)) return false;
  } else {
    s.fam_off.assign(1, 0);
    host_members(cx, 0, delta_node);
  }
  s.bond_state.assign(s.fam_members.size(), 1);
  // pre-crack bond states
  for (const auto& cr : m.cracks) cut_bonds(cx, cr);
  s.algo = cx.algo;
  s.crack_elems = cx.crack_elems;
  // elements around each node, for the CSR rows an FC 1 growth changes
  s.node_elem_ptr.assign((size_t)N + 1, 0);
  for (int e = 0; e < E; e++)
    for (int a = 0; a < m.elem_nn[e]; a++) s.node_elem_ptr[m.conn[(size_t)e * 8 + a] + 1]++;
  for (int k = 0; k < N; k++) s.node_elem_ptr[k + 1] += s.node_elem_ptr[k];
  s.node_elem.assign(s.node_elem_ptr[N], 0);
  {
    std::vector<int> fill(s.node_elem_ptr.begin(), s.node_elem_ptr.end() - 1);
    for (int e = 0; e < E; e++)
      for (int a = 0; a < m.elem_nn[e]; a++) s.node_elem[fill[m.conn[(size_t)e * 8 + a]]++] = e;
  }
  if (!pattern) return true;   // batch specimens: no CSR pattern (not merged)
  if (device >= 0) return gpu_csr_pattern(m, s, device, err);   // k_setup.cu
  build_csr_pattern(m, s);
  return true;
}

void grow_pd_region(const Mesh& m, const Command& cmd, Setup& s, const std::vector<std::array<double, 9>>& segs,
                    bool* grew) {
  Ctx cx{m, s, s.algo, s.crack_elems};
  const size_t old_pde = s.pde.size();
  // a segment that cuts no new element adds no PD element (the reference
  // reads the bounds of an empty centre list there)
  for (const auto& seg : segs) {
    const size_t old = cx.crack_elems.size();
    if (update_pde_by_crack(cx, seg) > 0) pde_near_crack_elems(cx, old, cmd.me);
  }
  s.crack_elems = cx.crack_elems;
  *grew = s.pde.size() > old_pde;
  if (!*grew) return;
  s.algo = cx.algo;
  s.fe.clear();
  for (int e = 0; e < m.n_elem; e++)
    if (s.algo[e] == 2) s.fe.push_back(e);
  pdbe_and_node_types(m, s);
  // new PD nodes get families after the existing ones, in the order of the
  // new PD elements and their nodes (updatePDN_Fami)
  const int D = m.dim;
  const int f0 = (int)s.fam_node.size();
  for (size_t i = old_pde; i < s.pde.size(); i++) {
    const int e = s.pde[i];
    for (int a = 0; a < m.elem_nn[e]; a++) {
      const int k = m.conn[(size_t)e * 8 + a];
      if (s.fam_of_node[k] >= 0) continue;
      s.fam_of_node[k] = (int)s.fam_node.size();
      s.fam_node.push_back(k);
      s.fam_delta.push_back(cmd.factor * std::pow(s.vol_node[k], 1.0 / D));
    }
  }
  s.fam_cdv.resize(s.fam_node.size(), 0.0);
  for (size_t i = old_pde; i < s.pde.size(); i++) {
    const int e = s.pde[i];
    const double dv = s.vol_elem[e];
    const int nn = m.elem_nn[e];
    for (int a = 0; a < nn; a++) {
      const int f = s.fam_of_node[m.conn[(size_t)e * 8 + a]];
      s.fam_cdv[f] = s.fam_cdv[f] + dv / nn;
    }
  }
  host_members(cx, f0, node_horizons(m, cmd, s));
  s.bond_state.resize(s.fam_members.size(), 1);
  std::vector<int> touched;
  for (size_t i = old_pde; i < s.pde.size(); i++)
    for (int a = 0; a < m.elem_nn[s.pde[i]]; a++) touched.push_back(m.conn[(size_t)s.pde[i] * 8 + a]);
  std::sort(touched.begin(), touched.end());
  touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
  update_csr_rows(cx, touched);
}

int cut_bonds_by_segment(const Mesh& m, Setup& s, const std::array<double, 9>& seg) {
  Ctx cx{m, s, {}, {}};
  return cut_bonds(cx, seg);
}

void build_csr_pattern(const Mesh& m, Setup& s) {
  const int N = m.n_node, D = m.dim;
  std::vector<std::vector<int>> inter(N);
  for (size_t f = 0; f < s.fam_node.size(); f++) {
    const int k = s.fam_node[f];
    inter[k].assign(s.fam_members.begin() + s.fam_off[f], s.fam_members.begin() + s.fam_off[f + 1]);
  }
  for (int e : s.fe) {
    const int nn = m.elem_nn[e];
    for (int a = 0; a < nn; a++)
      for (int b = 0; b < nn; b++) inter[m.conn[(size_t)e * 8 + a]].push_back(m.conn[(size_t)e * 8 + b]);
  }
  for (int k = 0; k < N; k++) {
    std::sort(inter[k].begin(), inter[k].end());
    inter[k].erase(std::unique(inter[k].begin(), inter[k].end()), inter[k].end());
  }
  s.csr_ia.assign((size_t)s.n_eq + 1, 0);
  s.csr_ja.clear();
  for (int k = 0; k < N; k++)
    for (int i = 0; i < D; i++) {
      const int row = s.eq[(size_t)k * D + i];
      if (row < 0) continue;
      for (int j : inter[k])
        for (int jj = 0; jj < D; jj++) {
          const int col = s.eq[(size_t)j * D + jj];
          if (col < 0) continue;
          s.csr_ja.push_back(col);
          s.csr_ia[(size_t)row + 1]++;
        }
    }
  for (int i = 0; i < s.n_eq; i++) s.csr_ia[(size_t)i + 1] += s.csr_ia[i];
}

}  // namespace pdx
