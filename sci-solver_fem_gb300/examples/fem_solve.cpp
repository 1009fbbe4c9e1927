// fem_solve -- command-line solve through the FEMSolver drop-in (include/FEMSolver.h),
// the counterpart of the reference's two example programs (src/examples/example1.cu for
// tetrahedral .node/.ele meshes, src/examples/example2.cu for .ply triangle meshes).
//
//   fem_solve -i <mesh> [-A <A.mat>] [-b <b.mat>] [-o <x.mat>] [-s <solverType>] [-v]
//
// <mesh> is a TetGen base name (<mesh>.node / <mesh>.ele) or a .ply file.  The operator is
// assembled from the mesh, or replaced by the sparse matrix in -A (same pattern); b is all
// ones unless -b names a single-column array; -s sets FEMSolver::solverType_ (default as
// in the reference: 0, one V-cycle; 1: PCG).  The solution goes to -o (default
// output.mat) and, as point data, to <mesh name>.vtk in the working directory.
//
// Build: g++ -O2 -std=c++17 -I include fem_solve.cpp libfemgpu.so -Wl,-rpath,<lib dir>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "FEMSolver.h"

static bool ends_with(const std::string& s, const std::string& tail) {
  return s.size() >= tail.size() && s.compare(s.size() - tail.size(), tail.size(), tail) == 0;
}

int main(int argc, char** argv) {
  std::string mesh, a_name, b_name, out_name = "output.mat";
  bool verbose = false;
  int solver_type = -1;
  for (int i = 1; i < argc; i++) {
    const std::string arg = argv[i];
    const bool has_value = i + 1 < argc;
    if (arg == "-v") verbose = true;
    else if (arg == "-i" && has_value) mesh = argv[++i];
    else if (arg == "-A" && has_value) a_name = argv[++i];
    else if (arg == "-b" && has_value) b_name = argv[++i];
    else if (arg == "-o" && has_value) out_name = argv[++i];
    else if (arg == "-s" && has_value) solver_type = std::atoi(argv[++i]);
    else {
      std::cerr << "usage: " << argv[0]
                << " -i <mesh base | mesh.ply> [-A A.mat] [-b b.mat] [-o x.mat] [-s solverType] [-v]\n";
      return 2;
    }
  }
  if (mesh.empty()) {
    std::cerr << "no mesh given (-i)\n";
    return 2;
  }
  const bool tet = !ends_with(mesh, ".ply");
  try {
    FEMSolver cfg(mesh, tet, verbose);
    if (solver_type >= 0) cfg.solverType_ = solver_type;
    if (!a_name.empty() && cfg.readMatlabSparseMatrix(a_name) != 0) {
      std::cerr << "failed to read the A matrix: " << a_name << "\n";
      return 1;
    }
    Vector_h_CG b(cfg.getMatrixRows(), 1.0);
    if (!b_name.empty() && cfg.readMatlabArray(b_name, &b) != 0) {
      std::cerr << "failed to read the b array: " << b_name << "\n";
      return 1;
    }
    Vector_h_CG x(cfg.getMatrixRows(), 0.0);
    cfg.solveFEM(&x, &b);
    if (cfg.writeMatlabArray(out_name, x) != 0) {
      std::cerr << "failed to write " << out_name << "\n";
      return 1;
    }
    // VTK named after the mesh file: directory and (for .ply) extension dropped
    std::string name = cfg.filename_;
    const size_t slash = name.find_last_of("/\\");
    if (slash != std::string::npos) name = name.substr(slash + 1);
    if (!tet) name = name.substr(0, name.find_last_of('.'));
    std::vector<double> values(x.size());
    for (size_t i = 0; i < x.size(); i++) values[i] = x[i];
    cfg.writeVTK(values, name);
    if (verbose) std::cout << "solved " << x.size() << " unknowns; wrote " << out_name << " and " << name << ".vtk\n";
  } catch (const std::exception& e) {
    std::cerr << "fem_solve: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
