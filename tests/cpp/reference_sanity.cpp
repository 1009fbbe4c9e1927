// The reference's three end-to-end tests (src/test/sanity2D.cc, sanity3D.cc,
// tetVol.cc) written against the FEMSolver drop-in: same calls, same bounds.
// Usage: reference_sanity <data_dir>; exit code 0 when every check passes.
#include <cmath>
#include <cstdio>
#include <string>

#include "FEMSolver.h"

static int failures = 0;
#define CHECK(cond, ...)                 \
  do {                                   \
    if (!(cond)) {                       \
      printf("FAILED: " __VA_ARGS__);    \
      printf("\n");                      \
      failures++;                        \
    }                                    \
  } while (0)

static double error_norm(const Vector_h_CG& x, const Vector_h_CG& ans) {
  double e = 0.0;
  for (size_t i = 0; i < x.size(); i++) e += (x[i] - ans[i]) * (x[i] - ans[i]);
  return std::sqrt(e);
}

static void run(const std::string& dir, const std::string& mesh, bool tet, const std::string& A,
                const std::string& b, const std::string& ans, double bound, int solverType) {
  FEMSolver cfg(dir + "/" + mesh, tet, false);
  cfg.solverType_ = solverType;
  cfg.tolerance_ = 1e-8;
  cfg.maxIters_ = 400;
  cfg.flexibleCG_ = 1;
  CHECK(cfg.readMatlabSparseMatrix(dir + "/" + A) == 0, "reading %s", A.c_str());
  Vector_h_CG b_h(cfg.getMatrixRows(), 1.0), x_h(cfg.getMatrixRows(), 0.0), x_answer;
  CHECK(cfg.readMatlabArray(dir + "/" + b, &b_h) == 0, "reading %s", b.c_str());
  cfg.solveFEM(&x_h, &b_h);
  CHECK(cfg.readMatlabArray(dir + "/" + ans, &x_answer) == 0, "reading %s", ans.c_str());
  double err = error_norm(x_h, x_answer);
  printf("%s (solverType %d): error %.6e (bound %g), iterations %d, relres %.3e\n", mesh.c_str(), solverType, err,
         bound, cfg.lastStats_.iterations, cfg.lastStats_.relative_residual);
  CHECK(err < bound, "%s error %g >= %g", mesh.c_str(), err, bound);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    printf("usage: %s <data_dir>\n", argv[0]);
    return 2;
  }
  std::string dir = argv[1];
  try {
    // sanity3D.cc (EggCarton3D): error < 1
    run(dir, "simple", true, "simple.mat", "simpleb.mat", "simpleAns.mat", 1.0, 1);
    // sanity2D.cc (EggCarton2D): error < 100
    run(dir, "simple.ply", false, "simpleTri.mat", "simpleTrib.mat", "simpleTriAns.mat", 100.0, 1);
    // tetVol.cc: error < 25
    run(dir, "tetVol", true, "tetVolA.mat", "tetVolb.mat", "tetVolAns.mat", 25.0, 1);
    // the reference default solverType_ = 0 runs one V-cycle (amg.cu:187-194)
    run(dir, "simple", true, "simple.mat", "simpleb.mat", "simpleAns.mat", 1.0, 0);
    // writers round trip
    FEMSolver cfg(dir + "/simple", true, false);
    Vector_h_CG v(cfg.getMatrixRows(), 0.5), back;
    CHECK(cfg.writeMatlabArray("femsolver_out.mat", v) == 0, "writeMatlabArray");
    CHECK(cfg.readMatlabArray("femsolver_out.mat", &back) == 0 && back.size() == v.size() && back[7] == 0.5,
          "readMatlabArray round trip");
    std::vector<double> vals(cfg.getMatrixRows(), 1.0);
    cfg.writeVTK(vals, "femsolver_out");
    FILE* f = fopen("femsolver_out.vtk", "r");
    CHECK(f != nullptr, "writeVTK output");
    if (f) fclose(f);
    // empty-matrix check throws std::invalid_argument (FEMSolver.cu:131-139)
    Matrix_ell_h empty;
    bool threw = false;
    try {
      cfg.checkMatrixForValidContents(&empty);
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    CHECK(threw, "checkMatrixForValidContents on an empty matrix");
    // a missing mesh is an exception, not exit(0)
    threw = false;
    try {
      FEMSolver bad(dir + "/does_not_exist", true, false);
    } catch (const std::runtime_error&) {
      threw = true;
    }
    CHECK(threw, "missing mesh file");
  } catch (const std::exception& e) {
    printf("FAILED with exception: %s\n", e.what());
    return 1;
  }
  printf(failures ? "FAILED (%d)\n" : "ALL PASSED\n", failures);
  return failures ? 1 : 0;
}
