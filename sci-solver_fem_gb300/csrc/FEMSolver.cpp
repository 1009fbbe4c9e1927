// FEMSolver.cpp -- the reference's FEMSolver API (src/FEMSolver.cu) over the C ABI.
#include "../../include/FEMSolver.h"

#include <algorithm>
#include <cstdio>
#include <stdexcept>

namespace {

void check(femgpu_status st, femgpu_handle h, const char* what) {
  if (st != FEMGPU_OK) {
    std::string msg = std::string(what) + ": " + femgpu_status_string(st);
    const char* detail = femgpu_last_error(h);
    if (detail && *detail) msg += std::string(" (") + detail + ")";
    throw std::runtime_error(msg);
  }
}

}  // namespace

// FEMSolver::FEMSolver (src/FEMSolver.cu:9-44): read the mesh and assemble.
FEMSolver::FEMSolver(std::string fname, bool isTetMesh, bool verbose)
    : verbose_(verbose),
      filename_(fname),
      maxLevels_(100),
      maxIters_(100),
      preInnerIters_(5),
      postInnerIters_(5),
      postRelaxes_(1),
      cycleIters_(1),
      dsType_(0),
      topSize_(256),
      randMisParameters_(90102),
      partitionMaxSize_(512),
      aggregatorType_(0),
      convergeType_(0),
      tolerance_(1e-6),
      cycleType_(0),
      solverType_(0),
      smootherWeight_(1.0),
      proOmega_(0.67),
      device_(0),
      blockSize_(256),
      tetMesh_(nullptr),
      triMesh_(nullptr),
      seed_(1),
      precision_(0),
      flexibleCG_(0),
      smoother_(0),
      lastStats_(),
      h_(nullptr) {
  int64_t nv = 0, ne = 0;
  if (isTetMesh) {
    std::string node = filename_ + ".node", ele = filename_ + ".ele";
    check(femgpu_read_tetgen(node.c_str(), ele.c_str(), &nv, &ne, nullptr, nullptr, nullptr), nullptr,
          "reading .node/.ele");
    std::vector<double> xyz(nv * 3);
    std::vector<int32_t> conn(ne * 4), lab(ne);
    check(femgpu_read_tetgen(node.c_str(), ele.c_str(), &nv, &ne, xyz.data(), conn.data(), lab.data()), nullptr,
          "reading .node/.ele");
    tetMesh_ = new TetMesh();
    tetMesh_->vertices.resize(nv);
    for (int64_t i = 0; i < nv; i++) tetMesh_->vertices[i] = {xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]};
    tetMesh_->tets.resize(ne);
    for (int64_t e = 0; e < ne; e++) tetMesh_->tets[e] = {conn[e * 4], conn[e * 4 + 1], conn[e * 4 + 2], conn[e * 4 + 3]};
    tetMesh_->matlabels.assign(lab.begin(), lab.end());
  } else {
    check(femgpu_read_ply(filename_.c_str(), &nv, &ne, nullptr, nullptr), nullptr, "reading PLY");
    std::vector<double> xyz(nv * 3);
    std::vector<int32_t> conn(ne * 3);
    check(femgpu_read_ply(filename_.c_str(), &nv, &ne, xyz.data(), conn.data()), nullptr, "reading PLY");
    triMesh_ = new TriMesh();
    triMesh_->vertices.resize(nv);
    for (int64_t i = 0; i < nv; i++) triMesh_->vertices[i] = {xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]};
    triMesh_->faces.resize(ne);
    for (int64_t e = 0; e < ne; e++) triMesh_->faces[e] = {conn[e * 3], conn[e * 3 + 1], conn[e * 3 + 2]};
  }
  femgpu_config c = config();
  check(femgpu_create(&h_, &c), nullptr, "creating the CUDA context");
  getMatrixFromMesh();
}

FEMSolver::~FEMSolver() {
  if (h_) femgpu_destroy(h_);
  delete tetMesh_;
  delete triMesh_;
}

femgpu_config FEMSolver::config() const {
  femgpu_config c;
  femgpu_config_default(&c);
  c.verbose = verbose_;
  c.maxLevels = maxLevels_;
  c.maxIters = maxIters_;
  c.preInnerIters = preInnerIters_;
  c.postInnerIters = postInnerIters_;
  c.postRelaxes = postRelaxes_;
  c.cycleIters = cycleIters_;
  c.dsType = dsType_;
  c.topSize = topSize_;
  c.randMisParameters = randMisParameters_;
  c.partitionMaxSize = partitionMaxSize_;
  c.aggregatorType = aggregatorType_;
  c.convergeType = convergeType_;
  c.tolerance = tolerance_;
  c.cycleType = cycleType_;
  c.solverType = solverType_;
  c.smootherWeight = smootherWeight_;
  c.proOmega = proOmega_;
  c.device = device_;
  c.blockSize = blockSize_;
  c.seed = seed_;
  c.precision = precision_;
  c.flexibleCG = flexibleCG_;
  c.smoother = smoother_;
  return c;
}

// FEMSolver::getMatrixFromMesh (src/FEMSolver.cu:141-171): pattern + K + M with the
// label coefficients; the host copy A_h_ keeps FP64 values.
void FEMSolver::getMatrixFromMesh() {
  if (!tetMesh_ && !triMesh_) throw std::runtime_error("no mesh");
  std::vector<double> xyz;
  std::vector<int32_t> conn, lab;
  int dim = tetMesh_ ? 3 : 2;
  if (tetMesh_) {
    for (auto& v : tetMesh_->vertices) xyz.insert(xyz.end(), v.begin(), v.end());
    for (auto& t : tetMesh_->tets) conn.insert(conn.end(), t.begin(), t.end());
    lab.assign(tetMesh_->matlabels.begin(), tetMesh_->matlabels.end());
  } else {
    for (auto& v : triMesh_->vertices) xyz.insert(xyz.end(), v.begin(), v.end());
    for (auto& t : triMesh_->faces) conn.insert(conn.end(), t.begin(), t.end());
  }
  int64_t nv = (int64_t)xyz.size() / 3, ne = (int64_t)conn.size() / (dim + 1);
  check(femgpu_set_mesh(h_, dim, nv, xyz.data(), ne, conn.data(), lab.empty() ? nullptr : lab.data()), h_,
        "building the mesh pattern");
  check(femgpu_assemble(h_, nullptr, 1.0), h_, "assembly");
  int64_t n = 0, nnz = 0;
  check(femgpu_get_matrix(h_, &n, &nnz, nullptr, nullptr, nullptr), h_, "reading the operator");
  A_h_.num_rows = A_h_.num_cols = (size_t)n;
  A_h_.num_entries = (size_t)nnz;
  A_h_.row_offsets.resize(n + 1);
  A_h_.column_indices.resize(nnz);
  A_h_.values.resize(nnz);
  check(femgpu_get_matrix(h_, &n, &nnz, A_h_.row_offsets.data(), A_h_.column_indices.data(), A_h_.values.data()), h_,
        "reading the operator");
  // need_neighbors (tetmesh.cu:112-170), sorted by tetmesh2ell: the pattern row without i
  std::vector<std::vector<int>>& nb = tetMesh_ ? tetMesh_->neighbors : triMesh_->neighbors;
  nb.assign(n, {});
  for (int64_t i = 0; i < n; i++)
    for (int32_t e = A_h_.row_offsets[i]; e < A_h_.row_offsets[i + 1]; e++)
      if (A_h_.column_indices[e] != i) nb[i].push_back(A_h_.column_indices[e]);
}

void FEMSolver::checkMatrixForValidContents(Matrix_ell_h* A_h) {
  if (A_h->num_rows == 0) {
    if (verbose_) printf("Error no matrix specified\n");
    throw std::invalid_argument("Error no matrix specified");
  }
}

// FEMSolver::solveFEM (src/FEMSolver.cu:58-93): upload A_h_, build the hierarchy,
// solve; x_h holds the initial guess on entry.
void FEMSolver::solveFEM(Vector_h_CG* x_h, Vector_h_CG* b_h) {
  checkMatrixForValidContents(&A_h_);
  if (!x_h || !b_h || x_h->size() != A_h_.num_rows || b_h->size() != A_h_.num_rows)
    throw std::invalid_argument("x and b must have getMatrixRows() entries");
  femgpu_config c = config();
  check(femgpu_set_config(h_, &c), h_, "options");
  check(femgpu_set_matrix_csr(h_, (int64_t)A_h_.num_rows, A_h_.row_offsets.data(), A_h_.column_indices.data(),
                              A_h_.values.data()),
        h_, "uploading the operator");
  check(femgpu_setup(h_), h_, "AMG setup");
  femgpu_status st = femgpu_solve(h_, b_h->data(), x_h->data(), &lastStats_);
  if (st == FEMGPU_ERR_NOT_CONVERGED) {
    // the reference returns silently after maxIters_ (cgcycle.cu:33-56)
    if (verbose_) printf("PCG stopped after %d iterations, relative residual %.3e\n", lastStats_.iterations,
                         lastStats_.relative_residual);
  } else {
    check(st, h_, "solve");
  }
  if (verbose_) {
    int levels = 0;
    femgpu_num_levels(h_, &levels);
    printf("AMG levels: %d, iterations: %d, relative residual: %.3e, setup %.3f ms, solve %.3f ms\n", levels,
           lastStats_.iterations, lastStats_.relative_residual, lastStats_.setup_ms, lastStats_.solve_ms);
  }
}

size_t FEMSolver::getMatrixRows() { return A_h_.num_rows; }

// FEMSolver::readMatlabSparseMatrix (src/FEMSolver.cu:177-356): the file matrix
// plus 1e-12 on every entry of the mesh pattern (union of the two patterns).
int FEMSolver::readMatlabSparseMatrix(const std::string& filename) {
  int64_t rows = 0, cols = 0, nnz = 0;
  if (femgpu_read_mat_sparse(filename.c_str(), &rows, &cols, &nnz, nullptr, nullptr, nullptr) != FEMGPU_OK) {
    fprintf(stderr, "could not read sparse matrix: %s\n", filename.c_str());
    return 1;
  }
  std::vector<int32_t> rp(rows + 1), ci(nnz);
  std::vector<double> v(nnz);
  if (femgpu_read_mat_sparse(filename.c_str(), &rows, &cols, &nnz, rp.data(), ci.data(), v.data()) != FEMGPU_OK)
    return 1;
  const size_t n = A_h_.num_rows;
  if ((size_t)rows != n || (size_t)cols != n) {
    fprintf(stderr, "%s: %lld x %lld does not match the mesh (%zu rows)\n", filename.c_str(), (long long)rows,
            (long long)cols, n);
    return 1;
  }
  Matrix_ell_h out;
  out.num_rows = out.num_cols = n;
  out.row_offsets.assign(n + 1, 0);
  for (size_t i = 0; i < n; i++) {
    int32_t a = A_h_.row_offsets[i], ae = A_h_.row_offsets[i + 1];
    int32_t b = rp[i], be = rp[i + 1];
    while (a < ae || b < be) {
      int32_t ca = a < ae ? A_h_.column_indices[a] : INT32_MAX;
      int32_t cb = b < be ? ci[b] : INT32_MAX;
      int32_t col = std::min(ca, cb);
      double val = 0.0;
      if (cb == col) val += v[b++];
      if (ca == col) {
        val += 1e-12;
        a++;
      }
      out.column_indices.push_back(col);
      out.values.push_back(val);
    }
    out.row_offsets[i + 1] = (int32_t)out.column_indices.size();
  }
  out.num_entries = out.values.size();
  A_h_ = std::move(out);
  return 0;
}

int FEMSolver::readMatlabArray(const std::string& filename, Vector_h_CG* rhs) {
  int64_t n = 0;
  if (femgpu_read_mat_array(filename.c_str(), &n, nullptr) != FEMGPU_OK) {
    fprintf(stderr, "could not read array: %s\n", filename.c_str());
    return -1;
  }
  std::vector<double> v(n);
  if (femgpu_read_mat_array(filename.c_str(), &n, v.data()) != FEMGPU_OK) return -1;
  rhs->clear();
  for (double x : v) rhs->push_back(x);
  return 0;
}

int FEMSolver::writeMatlabArray(const std::string& filename, const Vector_h_CG& array) {
  return femgpu_write_mat_array(filename.c_str(), (int64_t)array.size(), array.data()) == FEMGPU_OK ? 0 : 1;
}

// FEMSolver::writeVTK (src/FEMSolver.cu:519-582): writes fname + ".vtk".
void FEMSolver::writeVTK(std::vector<double> values, std::string fname) {
  std::vector<double> xyz;
  std::vector<int32_t> conn;
  int dim = tetMesh_ ? 3 : 2;
  if (tetMesh_) {
    for (auto& v : tetMesh_->vertices) xyz.insert(xyz.end(), v.begin(), v.end());
    for (auto& t : tetMesh_->tets) conn.insert(conn.end(), t.begin(), t.end());
  } else if (triMesh_) {
    for (auto& v : triMesh_->vertices) xyz.insert(xyz.end(), v.begin(), v.end());
    for (auto& t : triMesh_->faces) conn.insert(conn.end(), t.begin(), t.end());
  } else {
    return;
  }
  int64_t nv = (int64_t)xyz.size() / 3;
  values.resize(nv, 0.0);
  std::string path = fname + ".vtk";
  femgpu_write_vtk(path.c_str(), dim, nv, xyz.data(), (int64_t)conn.size() / (dim + 1), conn.data(), values.data());
}
