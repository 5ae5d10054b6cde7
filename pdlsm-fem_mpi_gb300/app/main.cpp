// PDLSM-FEM command-line front end on the GB300 library: the reference's CLI
// (SourceFiles/main.cpp, SourceFiles/Solver/pdfem_mpi.cpp:19-71) -
//   PDLSM-FEM [cmdfile]        (default PDFEMcmd.in)
// reads the same command and mesh files and writes Results/<title>_<step>.vtk
// in the working directory.  Unlike the reference, errors give a non-zero exit
// status and a message instead of exit(0).
#include <chrono>
#include <cstdio>
#include <string>

#include "../../include/pdx.h"

int main(int argc, char** argv) {
  const std::string cmd = argc > 1 ? argv[1] : "PDFEMcmd.in";
  pdx_options opt{0, -1, 0, 0, 0};
  pdx_model* m = nullptr;
  pdx_status st = pdx_model_create_from_cmd(cmd.c_str(), &opt, &m);
  if (st != PDX_OK) {
    std::printf("ERROR: %s\n", pdx_last_error());
    return 1;
  }
  pdx_model_info info;
  pdx_model_get_info(m, &info);
  std::printf("PDLSM-FEM solving project (%d nodes, %d families, %lld bonds, %d equations).........\n", info.n_node,
              info.n_fam, (long long)info.n_bond, info.n_eq);
  const auto t0 = std::chrono::steady_clock::now();
  st = pdx_run(m, "Results");
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st != PDX_OK) {
    std::printf("ERROR: %s\n", pdx_last_error());
    pdx_model_destroy(m);
    return 1;
  }
  std::printf("Elapsed time of PDLSM-FEM GB300 solving is %f s\n", s);
  std::printf("PDLSM-FEM program finished.\n");
  pdx_model_destroy(m);
  return 0;
}
