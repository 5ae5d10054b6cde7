// FC 1: crack growth by the maximum circumferential tensile stress criterion
// with stress intensity factors from the interaction integral (2D), the
// reference's b_cracPropag_qusiaStatic_BYKeq (SourceFiles/Solver/pdsolve.cpp:7375-7495).
//
// Per crack:
//   path    the node nearest the tip (in the tip's block) sets the radius
//           R = mr * horizon / factor; every element of the blocks around the
//           tip with some but not all of its nodes inside R contributes
//           sample points: an FE element its centre, a PD element its nodes
//           outside R (SIFsAndPropaDire_GaussPointPDnode :8514-8679);
//   fields  displacement gradient and stress at the points, evaluated on the
//           GPU from the resident displacements (k_fc1.cu);
//   sum     the points sorted by polar angle around the tip and closed into
//           a loop; along each chord the trapezoidal rule integrates the
//           interaction integrals of the actual field with the pure mode I
//           and mode II near-tip fields, in the crack-tip frame
//           (Jintegrand_GPPDN :8681-8869), giving KI and KII;
//   growth  theta_c from the maximum hoop stress, Keq, and where Keq > K_Ic
//           the tip moves dcf * min_delta along theta_c.
// In a quasi-static run the moved cracks then grow the PD region and break
// the bonds crossing their new segments (updateEnrichRegion :8871-8908,
// updateBondstate :8910-9004): host set-up update, device rebuild.
//
// The sample order, the sort (std::sort on the angle, as the reference) and
// the integrand's operation order follow the reference so that the path and
// the sums are the same; the tip search reproduces its "last nearest node"
// tie rule.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "model_impl.h"

namespace pdx {

namespace {

struct PathPoint {
  double x[2];
  double theta;
  double sigma[3];   // xx, yy, xy
  double dg[4];      // dux/dx, duy/dy, dux/dy, duy/dx
};

// Interaction integrals of one chord p1-p2 of the path with the mode I and
// mode II auxiliary fields (Williams' near-tip stresses and displacement
// gradients for unit K), trapezoidal in the chord, in the frame of the crack
// direction tip0 -> tip1.  The chord normal is not normalised: it carries the
// chord length.
void chord_integrals(const PathPoint& p1, const PathPoint& p2, const double* tip0, const double* tip1, double E,
                     double nu, int protype, double* I1, double* I2) {
  const double pi = std::acos(-1.0);
  const PathPoint* p[2] = {&p1, &p2};
  const double nx = p2.x[1] - p1.x[1], ny = -(p2.x[0] - p1.x[0]);
  const double kappa = protype == 1 ? (3 - nu) / (1 + nu) : (3 - 4 * nu);
  const double alpha = std::atan2(tip1[1] - tip0[1], tip1[0] - tip0[0]);
  const double ca = std::cos(alpha), sa = std::sin(alpha);
  double r[2], th[2];
  for (int i = 0; i < 2; i++) {
    const double dx = p[i]->x[0] - tip1[0], dy = p[i]->x[1] - tip1[1];
    r[i] = std::sqrt(dx * dx + dy * dy);
    const double lx = ca * dx + sa * dy, ly = -sa * dx + ca * dy;
    th[i] = std::atan2(ly, lx);
  }
  const double n0 = ca * nx + sa * ny, n1 = -sa * nx + ca * ny;
  // actual stress and displacement gradient rotated into the crack frame
  double s[2][3], gx[2], gy[2];
  for (int i = 0; i < 2; i++) {
    const double* g = p[i]->sigma;
    s[i][0] = (ca * g[0] + sa * g[2]) * ca + (ca * g[2] + sa * g[1]) * sa;
    s[i][1] = -(-sa * g[0] + ca * g[2]) * sa + (-sa * g[2] + ca * g[1]) * ca;
    s[i][2] = -(ca * g[0] + sa * g[2]) * sa + (ca * g[2] + sa * g[1]) * ca;
    const double* d = p[i]->dg;
    gx[i] = (ca * d[0] + sa * d[3]) * ca + (ca * d[2] + sa * d[1]) * sa;
    gy[i] = (-sa * d[0] + ca * d[3]) * ca + (-sa * d[2] + ca * d[1]) * sa;
  }
  // strain (tensor shear) of an auxiliary stress with out-of-plane stress sz
  // (0 in plane stress)
  auto strain = [&](const double* a, double sz, double* e) {
    e[0] = 1.0 / E * (a[0] - nu * (a[1] + sz));
    e[1] = 1.0 / E * (a[1] - nu * (a[0] + sz));
    e[2] = a[2] * (1 + nu) / E;
  };
  auto contract = [](const double* a, const double* e) { return a[0] * e[0] + a[1] * e[1] + 2 * a[2] * e[2]; };
  auto traction_grad = [&](const double* a, double ux, double uy) {
    return a[0] * ux * n0 + a[2] * (ux * n1 + uy * n0) + a[1] * uy * n1;
  };
  double w1[2], w2[2], sec1[2], sec2[2], thr1[2], thr2[2];
  for (int i = 0; i < 2; i++) {
    const double c = 1.0 / std::sqrt(2 * pi * r[i]);
    const double ch = std::cos(0.5 * th[i]), sh = std::sin(0.5 * th[i]);
    const double c3 = std::cos(1.5 * th[i]), s3 = std::sin(1.5 * th[i]);
    const double m1[3] = {c * ch * (1 - sh * s3), c * ch * (1 + sh * s3), c * sh * ch * c3};
    const double m2[3] = {-c * sh * (2 + ch * c3), c * sh * ch * c3, c * ch * (1 - sh * s3)};
    // the mode II strain takes the mode I field's out-of-plane stress, as
    // the reference does
    const double sz = protype == 2 ? nu * (m1[0] + m1[1]) : 0.0;
    double e1[3], e2[3];
    strain(m1, sz, e1);
    strain(m2, sz, e2);
    w1[i] = contract(s[i], e1) * n0;
    w2[i] = contract(s[i], e2) * n0;
    const double f = (1 + nu) / E / std::sqrt(2 * pi * r[i]);
    const double st = std::sin(th[i]);
    const double u1x = f * ch * ((kappa - 1) * 0.5 - sh * s3);
    const double u1y = f * sh * (-0.5 * (kappa + 1) + ch * ch - st * st);
    const double u2x = f * sh * (st * st - ch * ch - 0.5 * (kappa + 1));
    const double u2y = f * ch * (-sh * s3 - 0.5 * (kappa - 1));
    sec1[i] = traction_grad(s[i], u1x, u1y);
    sec2[i] = traction_grad(s[i], u2x, u2y);
    thr1[i] = traction_grad(m1, gx[i], gy[i]);
    thr2[i] = traction_grad(m2, gx[i], gy[i]);
  }
  *I1 = (w1[0] + w1[1]) * 0.5 - (sec1[0] + sec1[1]) * 0.5 - (thr1[0] + thr1[1]) * 0.5;
  *I2 = (w2[0] + w2[1]) * 0.5 - (sec2[0] + sec2[1]) * 0.5 - (thr2[0] + thr2[1]) * 0.5;
}

struct CrackPath {
  std::vector<PathPoint> pts;
  size_t first = 0;   // index of the crack's first point in the launch
};

}  // namespace

pdx_status fc1_pass(pdx_model* m, bool grow) {
  const Mesh& me = m->mesh;
  Setup& s = m->setup;
  const Command& c = m->cmd;
  if (me.dim != 2) return set_error(PDX_ERR_UNSUPPORTED, "FC 1 is two-dimensional");
  if (me.protype != 1 && me.protype != 2) return set_error(PDX_ERR_PARSE, "problem type is not 1 or 2");
  const int nc = (int)m->cracks.size();
  m->crack_sif.assign(nc, {0.0, 0.0, 0.0, 0.0});
  m->fc1_moved = false;
  if (nc == 0) return PDX_OK;
  const int nbx = s.nblocks[0], nby = s.nblocks[1];
  auto X = [&](int n) { return &me.X[(size_t)n * 3]; };
  // path points of every crack, one launch for all
  std::vector<CrackPath> paths(nc);
  std::vector<int> pts;
  for (int ck = 0; ck < nc; ck++) {
    const double* tip = &m->cracks[ck][3];
    int id[3];
    for (int i = 0; i < 3; i++) id[i] = (int)((tip[i] - s.lbc[i]) / s.block_size);
    if (id[0] < 0 || id[0] >= nbx || id[1] < 0 || id[1] >= nby)
      return set_error(PDX_ERR_INVALID, "crack tip " + std::to_string(ck) + " lies outside the model");
    int nearest = -1;
    double best = 1.0e200;
    for (int n : s.block_nodes[(size_t)id[0] + (size_t)id[1] * nbx]) {
      const double* xn = X(n);
      const double d = (xn[0] - tip[0]) * (xn[0] - tip[0]) + (xn[1] - tip[1]) * (xn[1] - tip[1]);
      if (d <= best) { best = d; nearest = n; }
    }
    const int fk = nearest >= 0 ? s.fam_of_node[nearest] : -1;
    if (fk < 0)
      return set_error(PDX_ERR_UNSUPPORTED, "the node nearest crack tip " + std::to_string(ck) +
                                                " has no PD family (the tip must lie in the PD region)");
    const double R = c.mr * (s.fam_delta[fk] / c.factor);
    const int nsb = (int)(c.mr / c.factor) + 1;
    CrackPath& cp = paths[ck];
    cp.first = pts.size() / 5;
    for (int ix = id[0] - nsb; ix < id[0] + nsb + 1; ix++)
      for (int iy = id[1] - nsb; iy < id[1] + nsb + 1; iy++) {
        if (ix < 0 || ix >= nbx || iy < 0 || iy >= nby) continue;
        for (int e : s.block_elems[(size_t)ix + (size_t)iy * nbx]) {
          const int* cn = &me.conn[(size_t)e * 8];
          const int nn = me.elem_nn[e];
          const int q[4] = {cn[0], cn[1], cn[2], nn == 3 ? cn[2] : cn[3]};
          int inside = 0;
          for (int a = 0; a < 4; a++) {
            const double* xn = X(q[a]);
            const double d = (xn[0] - tip[0]) * (xn[0] - tip[0]) + (xn[1] - tip[1]) * (xn[1] - tip[1]);
            if (d < R * R) inside++;
          }
          if (inside == 0 || inside == 4) continue;
          if (s.algo[e] == 2) {
            PathPoint p{};
            for (int a = 0; a < 4; a++)
              for (int j = 0; j < 2; j++) p.x[j] = p.x[j] + X(q[a])[j] * 0.25;
            p.theta = std::atan2(p.x[1] - tip[1], p.x[0] - tip[0]);
            cp.pts.push_back(p);
            pts.insert(pts.end(), {0, q[0], q[1], q[2], q[3]});
          } else {
            for (int a = 0; a < nn; a++) {
              const int n = cn[a];
              const double* xn = X(n);
              const double d = (xn[0] - tip[0]) * (xn[0] - tip[0]) + (xn[1] - tip[1]) * (xn[1] - tip[1]);
              if (!(d > R * R)) continue;
              if (s.fam_of_node[n] < 0) return set_error(PDX_ERR_INVALID, "a PD element node has no family");
              PathPoint p{};
              p.x[0] = xn[0];
              p.x[1] = xn[1];
              p.theta = std::atan2(xn[1] - tip[1], xn[0] - tip[0]);
              cp.pts.push_back(p);
              pts.insert(pts.end(), {1, n, s.fam_of_node[n], 0, 0});
            }
          }
        }
      }
    if (cp.pts.empty())
      return set_error(PDX_ERR_INVALID, "no element crosses the J-integral path of crack " + std::to_string(ck));
  }
  // fields at the points (GPU)
  const int np = (int)(pts.size() / 5);
  std::vector<double> vals((size_t)np * 7);
  int* d_pts = nullptr;
  double* d_out = nullptr;
  pdx_status st = cuda_check(cudaMallocAsync((void**)&d_pts, pts.size() * sizeof(int), m->stream), "FC 1 points");
  if (!st) st = cuda_check(cudaMallocAsync((void**)&d_out, vals.size() * sizeof(double), m->stream), "FC 1 points");
  if (!st) {
    cudaMemcpyAsync(d_pts, pts.data(), pts.size() * sizeof(int), cudaMemcpyHostToDevice, m->stream);
    Fc1PointArgs a{};
    a.v = m->view;
    a.u = m->d_u[0];
    a.sigma = m->d_sigma;
    a.D = m->d_D;
    a.pts = d_pts;
    a.n_pts = np;
    a.out = d_out;
    st = cuda_check(launch_fc1_points(a, m->stream), "FC 1 point kernel");
  }
  if (!st) cudaMemcpyAsync(vals.data(), d_out, vals.size() * sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  if (d_pts) cudaFreeAsync(d_pts, m->stream);
  if (d_out) cudaFreeAsync(d_out, m->stream);
  if (!st) st = cuda_check(cudaStreamSynchronize(m->stream), "FC 1 points");
  if (st) return st;
  // SIFs and growth, crack by crack
  const double E = me.E, nu = me.nu;
  const double Ep = me.protype == 1 ? E : E / (1 - nu * nu);
  std::vector<std::array<double, 9>> moved;
  for (int ck = 0; ck < nc; ck++) {
    CrackPath& cp = paths[ck];
    for (size_t i = 0; i < cp.pts.size(); i++) {
      const double* v = &vals[(cp.first + i) * 7];
      for (int r = 0; r < 4; r++) cp.pts[i].dg[r] = v[r];
      for (int r = 0; r < 3; r++) cp.pts[i].sigma[r] = v[4 + r];
    }
    std::sort(cp.pts.begin(), cp.pts.end(), [](const PathPoint& a, const PathPoint& b) { return a.theta < b.theta; });
    cp.pts.push_back(cp.pts.front());
    std::array<double, 9>& cr = m->cracks[ck];
    double I1 = 0, I2 = 0;
    for (size_t i = 0; i + 1 < cp.pts.size(); i++) {
      double a1, a2;
      chord_integrals(cp.pts[i], cp.pts[i + 1], &cr[0], &cr[3], E, nu, me.protype, &a1, &a2);
      I1 = I1 + a1;
      I2 = I2 + a2;
    }
    const double KI = 0.5 * Ep * I1, KII = 0.5 * Ep * I2;
    double tc = 0.0;
    if (KII > 0) tc = 2 * std::atan(0.25 * (KI / KII - std::sqrt(KI * KI / KII / KII + 8.0)));
    else if (KII < 0) tc = 2 * std::atan(0.25 * (KI / KII + std::sqrt(KI * KI / KII / KII + 8.0)));
    const double keq =
        std::cos(0.5 * tc) * (KI * std::cos(0.5 * tc) * std::cos(0.5 * tc) - 1.5 * KII * std::sin(tc));
    m->fc1_keq = keq;
    const bool move = keq > me.KIc;
    m->crack_sif[ck] = {KI, KII, keq, move ? 1.0 : 0.0};
    if (!move) continue;
    m->fc1_moved = true;
    const double al = std::atan2(cr[4] - cr[1], cr[3] - cr[0]);
    const double dir[2] = {std::cos(al) * std::cos(tc) - std::sin(al) * std::sin(tc),
                           std::sin(al) * std::cos(tc) + std::cos(al) * std::sin(tc)};
    const double step = c.dcf * s.min_delta;
    const double tip[2] = {cr[3], cr[4]};
    cr[0] = tip[0];
    cr[1] = tip[1];
    cr[3] = tip[0] + dir[0] * step;
    cr[4] = tip[1] + dir[1] * step;
    moved.push_back(cr);
  }
  if (!grow || moved.empty()) return PDX_OK;
  return apply_growth(m, moved);
}

pdx_status apply_growth(pdx_model* m, const std::vector<std::array<double, 9>>& moved) {
  bool grew = false;
  const int f0 = (int)m->setup.fam_node.size();
  grow_pd_region(m->mesh, m->cmd, m->setup, moved, &grew);
  int cut = 0;
  for (const auto& seg : moved) cut += cut_bonds_by_segment(m->mesh, m->setup, seg);
  if (grew || cut > 0) m->fc1_changed = true;
  if (!m->has_device) {
    // a host-only model keeps its host arrays in step with the set-up
    if (!grew && cut == 0) return PDX_OK;
    m->prep = Prepared();
    Error err{0, ""};
    if (!prepare_model(m, err, false)) return set_error(PDX_ERR_INVALID, err.msg);
    return PDX_OK;
  }
  if (grew) {
    // Method 8's coarse grid stays valid while no coupling is longer than a
    // coarse cell: only the new families add couplings.  Its inverse then
    // keeps serving the locally changed matrix (formed anew once the
    // iterations grow by half).
    bool keep = m->twolevel != nullptr;
    const Setup& s = m->setup;
    for (int f = f0; keep && f < (int)s.fam_node.size(); f++) {
      const double* xk = &m->mesh.X[(size_t)s.fam_node[f] * 3];
      for (int64_t q = s.fam_off[f] + 1; keep && q < s.fam_off[f + 1]; q++) {
        const double* xm = &m->mesh.X[(size_t)s.fam_members[q] * 3];
        for (int a = 0; a < 2; a++)
          if (std::fabs(xm[a] - xk[a]) * 1.001 > m->twolevel->cell_len[a]) keep = false;
      }
    }
    return rebuild_device(m, keep);
  }
  if (cut > 0) {
    if (m->twolevel) m->twolevel->dev.keep_stale = true;
    return upload_bond_states(m);
  }
  return PDX_OK;
}

pdx_status fc1_reset(pdx_model* m) {
  m->cracks = m->mesh.cracks;
  m->crack_sif.assign(m->cracks.size(), {0.0, 0.0, 0.0, 0.0});
  m->fc1_keq = 0.0;
  m->fc1_moved = false;
  if (!m->fc1_changed) return PDX_OK;
  // a run grew the PD region or broke bonds: back to the mesh's set-up
  Error err{0, ""};
  if (!build_setup(m->mesh, m->cmd, m->setup, err, m->device))
    return set_error(err.code == 7 ? PDX_ERR_CUDA : PDX_ERR_PARSE, err.msg);
  m->fc1_changed = false;
  return rebuild_device(m);
}

}  // namespace pdx

extern "C" pdx_status pdx_crack_advance(pdx_model* m, const double* tips, const uint8_t* moved) {
  using namespace pdx;
  if (!m || !tips || !moved) return set_error(PDX_ERR_INVALID, "null argument");
  if (m->mesh.dim != 2) return set_error(PDX_ERR_UNSUPPORTED, "crack growth is two-dimensional");
  std::vector<std::array<double, 9>> segs;
  for (size_t k = 0; k < m->cracks.size(); k++) {
    if (!moved[k]) continue;
    auto& cr = m->cracks[k];
    cr[0] = cr[3];
    cr[1] = cr[4];
    cr[3] = tips[2 * k];
    cr[4] = tips[2 * k + 1];
    segs.push_back(cr);
  }
  if (segs.empty()) return PDX_OK;
  if (m->has_device) cudaSetDevice(m->device);
  return apply_growth(m, segs);
}
