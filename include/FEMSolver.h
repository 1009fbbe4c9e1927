/*
 * FEMSolver.h -- C++ drop-in for SCI-Solver_FEM's FEMSolver class
 * (src/FEMSolver.h:14-67 of the reference): same constructor, methods, public
 * option members and defaults, running the GB300 CUDA path through the C ABI
 * in femgpu.h.  Code written against the reference's header compiles unchanged:
 *
 *   FEMSolver cfg(mesh_base, true, false);
 *   cfg.readMatlabSparseMatrix(A_mat);           // optional operator override
 *   Vector_h_CG b_h(cfg.getMatrixRows(), 1.0), x_h(cfg.getMatrixRows(), 0.0);
 *   cfg.readMatlabArray(b_mat, &b_h);
 *   cfg.solveFEM(&x_h, &b_h);
 *
 * Differences a caller can observe: failures throw std::runtime_error instead of
 * exit(), the AMG random seed is the member seed_ instead of time(NULL), the
 * outer PCG uses the FP64 assembled values (the reference rounds them to FP32),
 * and the permuted level-0 operator is applied consistently, so solveFEM solves
 * A x = b.
 */
#ifndef FEMGPU_FEMSOLVER_H
#define FEMGPU_FEMSOLVER_H

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "femgpu.h"

/* Host FP64 vector with the cusp::array1d<double, host_memory> surface the
 * reference's callers use (types.h:28: Vector_h_CG). */
class Vector_h_CG {
 public:
  Vector_h_CG() {}
  explicit Vector_h_CG(size_t n, double v = 0.0) : d_(n, v) {}
  size_t size() const { return d_.size(); }
  double& operator[](size_t i) { return d_[i]; }
  const double& operator[](size_t i) const { return d_[i]; }
  void push_back(double v) { d_.push_back(v); }
  void clear() { d_.clear(); }
  void resize(size_t n, double v = 0.0) { d_.resize(n, v); }
  double* data() { return d_.data(); }
  const double* data() const { return d_.data(); }
  std::vector<double>::iterator begin() { return d_.begin(); }
  std::vector<double>::iterator end() { return d_.end(); }
  std::vector<double>::const_iterator begin() const { return d_.begin(); }
  std::vector<double>::const_iterator end() const { return d_.end(); }

 private:
  std::vector<double> d_;
};

/* Host copy of the assembled operator (the reference's Matrix_ell_h A_h_), CSR
 * with sorted columns; num_rows / num_cols / num_entries as in CUSP. */
struct Matrix_ell_h {
  size_t num_rows = 0, num_cols = 0, num_entries = 0;
  std::vector<int32_t> row_offsets, column_indices;
  std::vector<double> values;
};

/* Mesh containers (tetmesh.h / TriMesh.h): vertices, elements, labels and the
 * per-vertex neighbour lists of need_neighbors() (sorted, without the vertex). */
struct TetMesh {
  std::vector<std::array<double, 3>> vertices;
  std::vector<std::array<int, 4>> tets;
  std::vector<int> matlabels;
  std::vector<std::vector<int>> neighbors;
};
struct TriMesh {
  std::vector<std::array<double, 3>> vertices;
  std::vector<std::array<int, 3>> faces;
  std::vector<std::vector<int>> neighbors;
};

class FEMSolver {
 public:
  FEMSolver(std::string fname = "../src/test/test_data/simple", bool isTetMesh = true, bool verbose = false);
  virtual ~FEMSolver();
  FEMSolver(const FEMSolver&) = delete;
  FEMSolver& operator=(const FEMSolver&) = delete;

  void solveFEM(Vector_h_CG* x_h, Vector_h_CG* b_h);
  void getMatrixFromMesh();
  int readMatlabSparseMatrix(const std::string& filename);
  int readMatlabArray(const std::string& filename, Vector_h_CG* rhs);
  int writeMatlabArray(const std::string& filename, const Vector_h_CG& array);
  void checkMatrixForValidContents(Matrix_ell_h* A_h);
  void writeVTK(std::vector<double> values, std::string fname);
  size_t getMatrixRows();

  // option members (src/FEMSolver.h:37-58), same names and defaults
  bool verbose_;
  std::string filename_;
  int maxLevels_;
  int maxIters_;
  int preInnerIters_;
  int postInnerIters_;
  int postRelaxes_;
  int cycleIters_;
  int dsType_;
  int topSize_;
  int randMisParameters_;
  int partitionMaxSize_;
  int aggregatorType_;
  int convergeType_;
  double tolerance_;
  int cycleType_;
  int solverType_;
  double smootherWeight_;
  double proOmega_;
  int device_;
  int blockSize_;
  TetMesh* tetMesh_;
  TriMesh* triMesh_;
  Matrix_ell_h A_h_;
  // additions
  unsigned seed_;      // MIS seed (the reference uses time(NULL))
  int precision_;      // 0: FP32 hierarchy (reference), 1: FP64 hierarchy
  int flexibleCG_;     // 1: Polak-Ribiere beta
  int smoother_;       // 0: partition-block Jacobi (reference), 1: l1-Jacobi
  femgpu_solve_stats lastStats_;

 private:
  femgpu_config config() const;
  femgpu_handle h_;
};

#endif
