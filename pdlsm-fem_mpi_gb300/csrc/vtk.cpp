// Legacy VTK UNSTRUCTURED_GRID writers, byte-compatible with
// fioFiles::writeReslutsTOTAL_vtk_Binary / _ASCII (SourceFiles/Solver/fioFile.cpp:562-769):
// POINTS (float32), CELLS (count + 0-based ids), CELL_TYPES (9 Q4, 12 Hex8),
// POINT_DATA: VECTORS U (3 per node, 2D z = 0), TENSORS sigma (9 per node in the
// order xx xy zx / xy yy yz / zx yz zz), SCALARS phi.  BINARY is big-endian.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

#include "model_impl.h"

namespace pdx {

namespace {
// VTK cell type of an element with nn nodes (the reference's ci_eleType):
// triangle 5, quadrilateral 9, hexahedron 12
int vtk_cell_type(int nn) { return nn == 3 ? 5 : nn == 4 ? 9 : 12; }
}  // namespace

namespace {

void put_be32(std::ofstream& f, const void* p) {
  uint32_t v;
  std::memcpy(&v, p, 4);
  const unsigned char b[4] = {(unsigned char)(v >> 24), (unsigned char)(v >> 16), (unsigned char)(v >> 8),
                              (unsigned char)v};
  f.write((const char*)b, 4);
}

const int kSigIdx[9] = {0, 3, 5, 3, 1, 4, 5, 4, 2};

}  // namespace

void write_vtk(const pdx_model* m, const std::string& path, const std::vector<double>& u_all,
               const std::vector<double>& sigma, const std::vector<double>& phi, bool binary) {
  const Mesh& me = m->mesh;
  const int N = me.n_node, E = me.n_elem, D = me.dim;
  std::ofstream f(path, binary ? std::ios::binary : std::ios::out);
  f << "# vtk DataFile Version 3.0" << std::endl;
  f << me.title << std::endl;
  f << (binary ? "BINARY" : "ASCII") << std::endl;
  f << "DATASET UNSTRUCTURED_GRID" << std::endl;
  f << "POINTS " << N << " float" << std::endl;
  auto U = [&](int k, int j) { return j < D ? u_all[(size_t)k * D + j] : 0.0; };
  int size_list = 0;
  for (int e = 0; e < E; e++) size_list += me.elem_nn[e];
  size_list += E;
  if (binary) {
    for (int k = 0; k < N; k++)
      for (int j = 0; j < 3; j++) {
        const float x = (float)me.X[(size_t)k * 3 + j];
        put_be32(f, &x);
      }
    f << std::endl;
    f << "CELLS " << E << ' ' << size_list << std::endl;
    for (int e = 0; e < E; e++) {
      const int nn = me.elem_nn[e];
      put_be32(f, &nn);
      for (int j = 0; j < nn; j++) put_be32(f, &me.conn[(size_t)e * 8 + j]);
    }
    f << std::endl;
    f << "CELL_TYPES " << E << std::endl;
    for (int e = 0; e < E; e++) {
      const int t = vtk_cell_type(me.elem_nn[e]);
      put_be32(f, &t);
    }
    f << std::endl;
    f << "POINT_DATA " << N << std::endl;
    f << "VECTORS " << "U " << "float" << std::endl;
    for (int k = 0; k < N; k++)
      for (int j = 0; j < 3; j++) {
        const float v = (float)U(k, j);
        put_be32(f, &v);
      }
    f << std::endl;
    f << "TENSORS " << "sigma " << "float\n";
    for (int k = 0; k < N; k++)
      for (int j = 0; j < 9; j++) {
        const float v = (float)sigma[(size_t)k * 6 + kSigIdx[j]];
        put_be32(f, &v);
      }
    f << std::endl;
    f << "SCALARS " << "phi " << "float " << 1 << std::endl;
    f << "LOOKUP_TABLE  " << "default  " << std::endl;
    for (int k = 0; k < N; k++) {
      const float v = (float)phi[k];
      put_be32(f, &v);
    }
    f << std::endl;
    return;
  }
  f << std::setiosflags(std::ios::scientific) << std::setprecision(4);
  for (int k = 0; k < N; k++)
    f << me.X[(size_t)k * 3] << ' ' << me.X[(size_t)k * 3 + 1] << ' ' << me.X[(size_t)k * 3 + 2] << std::endl;
  f << std::endl;
  f << "CELLS " << E << ' ' << size_list << std::endl;
  for (int e = 0; e < E; e++) {
    f << me.elem_nn[e] << ' ';
    for (int j = 0; j < me.elem_nn[e]; j++) f << me.conn[(size_t)e * 8 + j] << ' ';
    f << std::endl;
  }
  f << std::endl;
  f << "CELL_TYPES " << E << std::endl;
  for (int e = 0; e < E; e++) f << vtk_cell_type(me.elem_nn[e]) << std::endl;
  f << "POINT_DATA " << N << std::endl;
  f << "VECTORS " << "U " << "float" << std::endl;
  for (int k = 0; k < N; k++) {
    for (int j = 0; j < 3; j++) f << float(U(k, j)) << ' ';
    f << std::endl;
  }
  f << "TENSORS " << "sigma " << "float\n";
  for (int k = 0; k < N; k++) {
    float s[6];
    for (int j = 0; j < 6; j++) s[j] = (float)sigma[(size_t)k * 6 + j];
    f << s[0] << ' ' << s[3] << ' ' << s[5] << std::endl;
    f << s[3] << ' ' << s[1] << ' ' << s[4] << std::endl;
    f << s[5] << ' ' << s[4] << ' ' << s[2] << std::endl;
    f << std::endl;
  }
  f << "SCALARS " << "phi " << "float " << 1 << std::endl;
  f << "LOOKUP_TABLE  " << "default  " << std::endl;
  for (int k = 0; k < N; k++) {
    f << float(phi[k]) << ' ';
    if (k % 20 == 0) f << std::endl;
  }
  f.close();
  // an ASCII result also writes <title>_<step>.sig and .disp beside it
  const std::string base = path.size() > 4 ? path.substr(0, path.size() - 4) : path;
  write_sig_disp(m, base, u_all, sigma);
}

// fioFiles::writeSigofNode and writeUofNode (fioFile.cpp:486-503, 528-547)
// with the rows of pdNode::printStress and printFinalU (pdNode.cpp:92-103,
// 120-130): one row per node, node id (1-based), coordinates, then the six
// stresses (scientific, 5 digits) or the three displacements (scientific, 4
// digits; the z entry of a 2D node is its unused third DOF, 0).
void write_sig_disp(const pdx_model* m, const std::string& base, const std::vector<double>& u_all,
                    const std::vector<double>& sigma) {
  const Mesh& me = m->mesh;
  const int N = me.n_node, D = me.dim;
  {
    std::ofstream f(base + ".sig");
    f << "*****The stress of  point*****" << std::endl;
    f << std::left;
    f << "NID" << "\t" << "x" << "\t" << "y" << "\t" << "z" << "\t" << "Sxx" << "\t" << "Syy" << "\t" << "Szz" << "\t"
      << "Sxy" << "\t" << "Syz" << "\t" << "Szx" << std::endl;
    f << std::setiosflags(std::ios::scientific) << std::setprecision(5);
    for (int k = 0; k < N; k++) {
      f << k + 1 << "\t";
      f << me.X[(size_t)k * 3] << "\t" << me.X[(size_t)k * 3 + 1] << "\t" << me.X[(size_t)k * 3 + 2];
      for (int j = 0; j < 6; j++) f << "\t" << sigma[(size_t)k * 6 + j];
      f << std::endl;
    }
  }
  std::ofstream f(base + ".disp");
  f << "*****The final displacement of  point*****" << std::endl;
  f << std::left;
  f << "ID" << "\t" << "x" << "\t" << "y" << "\t" << "z" << "\t" << "Ux" << "\t" << "Uy" << "\t" << "Uz" << std::endl;
  f << std::setiosflags(std::ios::scientific) << std::setprecision(4);
  for (int k = 0; k < N; k++) {
    f << k + 1 << "\t" << me.X[(size_t)k * 3] << "\t" << me.X[(size_t)k * 3 + 1] << "\t" << me.X[(size_t)k * 3 + 2]
      << "\t";
    f << u_all[(size_t)k * D] << "\t" << u_all[(size_t)k * D + 1] << "\t" << (D == 3 ? u_all[(size_t)k * D + 2] : 0.0)
      << std::endl;
  }
}

}  // namespace pdx
