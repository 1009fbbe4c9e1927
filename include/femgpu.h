/*
 * femgpu.h -- C ABI of the GB300-native P1 FEM -> smoothed-aggregation AMG -> PCG
 * solver.  Plain pointers and sizes only; every call returns a status code and
 * never exits the process.
 *
 * The reference exposes this path as the C++ class FEMSolver (src/FEMSolver.h:14-67
 * of SCI-Solver_FEM).  The C++ drop-in (include/FEMSolver.h) is a thin layer over
 * these entry points; foreign-language bindings (ctypes, cgo, JNI) call them
 * directly.  Each declaration names the reference interface it replaces.
 *
 * Ownership: the caller owns every host buffer and the library copies on entry;
 * device memory belongs to the handle and is released by femgpu_destroy.  All
 * device work runs on the handle's stream (config.stream, NULL = a private stream).
 * Calls on one handle must not overlap; distinct handles are independent.
 */
#ifndef FEMGPU_H
#define FEMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FEMGPU_OK = 0,
  FEMGPU_ERR_INVALID = 1,        /* bad argument or call order */
  FEMGPU_ERR_CUDA = 2,           /* CUDA runtime error */
  FEMGPU_ERR_NOT_READY = 3,      /* mesh / matrix / hierarchy missing */
  FEMGPU_ERR_BREAKDOWN = 4,      /* PCG breakdown (non-positive p'Ap, NaN/Inf), singular coarse matrix */
  FEMGPU_ERR_NOT_CONVERGED = 5,  /* max iterations reached */
  FEMGPU_ERR_LIMIT = 6,          /* a bounded loop or a size limit was hit */
  FEMGPU_ERR_IO = 7,             /* file could not be read / parsed */
  FEMGPU_ERR_ALLOC = 8,          /* device allocation failed */
  FEMGPU_ERR_NO_DEVICE = 9       /* no CUDA device visible */
} femgpu_status;

typedef struct femgpu_ctx* femgpu_handle;

/* Solver options.  The first block mirrors the public members of the reference's
 * FEMSolver (src/FEMSolver.h:37-56) with the same defaults (src/FEMSolver.cu:9-35). */
typedef struct {
  int verbose;              /* verbose_            0 */
  int maxLevels;            /* maxLevels_          100 */
  int maxIters;             /* maxIters_           100 */
  int preInnerIters;        /* preInnerIters_      5 */
  int postInnerIters;       /* postInnerIters_     5 */
  int postRelaxes;          /* postRelaxes_        1 */
  int cycleIters;           /* cycleIters_         1 */
  int dsType;               /* dsType_             0 (only the symmetric split is built) */
  int topSize;              /* topSize_            256 */
  int randMisParameters;    /* randMisParameters_  90102 */
  int partitionMaxSize;     /* partitionMaxSize_   512 */
  int aggregatorType;       /* aggregatorType_     0 (OldMIS; others rejected) */
  int convergeType;         /* convergeType_       0 (the PCG test is relative, as in the reference) */
  double tolerance;         /* tolerance_          1e-6 */
  int cycleType;            /* cycleType_          0 (V); 1 (W) and 2 (F) visit the next coarser
                               level twice (W: W then W, F: W then V, the visit patterns of the
                               reference's W_Cycle / F_Cycle), the second visit correcting the
                               first with the coarse residual */
  int solverType;           /* solverType_         0 = one V-cycle, 1 = PCG */
  double smootherWeight;    /* smootherWeight_     1.0 */
  double proOmega;          /* proOmega_           0.67 */
  int device;               /* device_             0 */
  int blockSize;            /* blockSize_          256 */
  /* Additions (no counterpart in the reference). */
  uint32_t seed;            /* replaces srand(time(NULL)) in the MIS: 1 */
  int precision;            /* 0 = FP32 hierarchy in an FP64 outer PCG (reference), 1 = FP64 hierarchy */
  int flexibleCG;           /* 0 = Fletcher-Reeves beta (reference), 1 = Polak-Ribiere (flexible) */
  void* stream;             /* cudaStream_t to run on; NULL = library-owned stream */
  void* mem_pool;           /* cudaMemPool_t for device buffers; NULL = a pool owned by the handle
                               that keeps freed memory for reuse until femgpu_destroy */
  int autotune;             /* 1 (default): at setup, time each level's result-neutral launch
                               choices (cross-partition lanes per row, cluster smoother CTAs per
                               group) once per device and level shape and keep the fastest; the
                               choices are cached for the process, and in the file named by the
                               environment variable FEMGPU_TUNE_CACHE when set.  0: fixed rules */
  int smoother;             /* 0 (default): the reference's partition-block weighted Jacobi
                               (gauss_seidel.cu dsType 0); 1: l1-Jacobi on every level's whole
                               operator, x += w (b - A x) / l1 with l1_i = sum_j |a_ij|,
                               preInnerIters / postInnerIters sweeps (a performance option:
                               no partitions, no shared-memory groups, one pass over A per sweep) */
} femgpu_config;

typedef struct {
  int iterations;           /* PCG iterations (SpMVs) performed */
  double relative_residual; /* ||b - A x|| / ||b|| at exit */
  double setup_ms;          /* last femgpu_setup: hierarchy build */
  double solve_ms;          /* last solve: device time */
  int num_levels;
} femgpu_solve_stats;

/* Per-level statistics (AMG::printGridStatistics, src/core/cuda/amg.cu:202-231). */
typedef struct {
  int64_t rows, nnz, aggregates, partitions, nnz_p;
} femgpu_level_info;

/* Defaults of the FEMSolver constructor (src/FEMSolver.cu:9-35). */
void femgpu_config_default(femgpu_config* cfg);

/* Creates a solver context on cfg->device.  Replaces FEMSolver::InitCUDA
 * (src/FEMSolver.cu:99-129), which the reference never calls. */
femgpu_status femgpu_create(femgpu_handle* h, const femgpu_config* cfg);
femgpu_status femgpu_destroy(femgpu_handle h);
/* Replaces the options of an existing context (device, stream and pool stay); the next
 * femgpu_setup uses them.  The reference reads its option members when solveFEM
 * constructs the AMG object (src/FEMSolver.cu:66-73). */
femgpu_status femgpu_set_config(femgpu_handle h, const femgpu_config* cfg);
const char* femgpu_status_string(femgpu_status s);
/* Last error message recorded on this handle (empty string if none). */
const char* femgpu_last_error(femgpu_handle h);

/* Sets the mesh and builds the CSR sparsity pattern on the device.
 * dim = 3: tetrahedra (nodes_per_elem = 4); dim = 2: triangles (3).
 * xyz: nverts x 3 doubles (z ignored for dim 2); conn: nelems x nodes_per_elem
 * 0-based vertex ids; labels: per-element material labels or NULL.
 * Replaces TetMesh::read / TriMesh::read + need_neighbors + tetmesh2ell /
 * trimesh2ell (src/core/cuda/tetmesh.cu:112-170,251-376; cutil.cu:168-230,297-348). */
femgpu_status femgpu_set_mesh(femgpu_handle h, int dim, int64_t nverts, const double* xyz,
                              int64_t nelems, const int32_t* conn, const int32_t* labels);

/* Assembles A = sum_e c_e K_e + lambda_mass M_e into the pattern.  coef (per
 * element, host) gives c_e; when coef is NULL, c_e comes from the labels
 * (1,1,2,3,4,5,6 for labels 0..6) in 3D and is 1 in 2D.  Replaces
 * FEM3D::assemble / FEM2D::assemble + element_loop_3d_kernel / element_loop_kernel
 * (src/core/cuda/FEM3D.cu:501-557; perform_element_loop_3D.cuh:480-627;
 * FEM2D.cu:358-378; perform_element_loop_2D.cuh:287-372); the reference fixes
 * lambda_mass = 1 and coef = NULL. */
femgpu_status femgpu_assemble(femgpu_handle h, const double* coef, double lambda_mass);
/* Same with the per-element coefficients in device memory (d_coef may be NULL); returns once
 * the operator is assembled.  No reference counterpart (device-resident callers such as the
 * PyTorch binding). */
femgpu_status femgpu_assemble_device(femgpu_handle h, const double* d_coef, double lambda_mass);

/* Load vector b = M f (consistent P1 mass) for nodal f (host arrays, nverts).
 * No reference counterpart: its force function is 0 (perform_element_loop_3D.cuh:22-26). */
femgpu_status femgpu_load_vector(femgpu_handle h, const double* f, double* b);

/* Symmetric Dirichlet elimination u = 0 on mask[i] != 0: rows and columns zeroed,
 * unit diagonal.  No reference counterpart (the reference applies no BC). */
femgpu_status femgpu_set_dirichlet(femgpu_handle h, const uint8_t* mask);

/* Replaces the operator with a host CSR matrix (sorted columns); the level-0
 * aggregation graph stays the mesh graph when a mesh is set, else it is the
 * matrix pattern.  Replaces the MAT-override path of
 * FEMSolver::readMatlabSparseMatrix (src/FEMSolver.cu:177-356). */
femgpu_status femgpu_set_matrix_csr(femgpu_handle h, int64_t n, const int32_t* rowptr,
                                    const int32_t* cols, const double* vals);

/* Builds the AMG hierarchy for the current operator.  Replaces AMG::setup
 * (src/core/cuda/amg.cu:80-144) with createNextLevel / OldMIS / RAP. */
femgpu_status femgpu_setup(femgpu_handle h);

/* Writes the handle's AMG hierarchy (every level, the level-0 permutation and the outer
 * operator) to a file, and reads one back into a handle that holds the same operator
 * (checked by size and a fingerprint of its pattern and values; FEMGPU_ERR_INVALID
 * otherwise) and the same precision setting, in place of femgpu_setup.  The file is in
 * the writing machine's byte order.  No reference counterpart (the reference rebuilds
 * its hierarchy in every AMG::setup). */
femgpu_status femgpu_save_hierarchy(femgpu_handle h, const char* path);
femgpu_status femgpu_load_hierarchy(femgpu_handle h, const char* path);

/* Solves A x = b.  x holds the initial guess on entry (host arrays, n doubles).
 * solverType 0: one V-cycle; 1: PCG to tolerance.  Replaces FEMSolver::solveFEM
 * (src/FEMSolver.cu:58-93) -> AMG::solve (amg.cu:174-200) -> CG_Flex_Cycle
 * (cgcycle.cu:6-69).  stats may be NULL. */
femgpu_status femgpu_solve(femgpu_handle h, const double* b, double* x, femgpu_solve_stats* stats);

/* nrhs right-hand sides with one hierarchy: column j of B (and of X, which holds the
 * initial guesses) is nverts doubles at B + j * nverts (host arrays).  With solverType 1
 * the columns are solved eight at a time: each column runs its own flexible PCG, the
 * eight in lockstep, and every operator and V-cycle application works on the n x 8 block
 * at once (sparse matrix times block), so the operators are read once per eight columns;
 * a column stops when it reaches the tolerance (W and F cycles, and solverType 0, solve
 * the columns one at a time).  stats: summed iterations, largest
 * relative residual, total solve time; the first failing column's status is returned.
 * No reference counterpart (the reference solves one right-hand side per
 * FEMSolver::solveFEM). */
femgpu_status femgpu_solve_multi(femgpu_handle h, int nrhs, const double* B, double* X,
                                 femgpu_solve_stats* stats);
/* Same with device arrays and leading dimensions ldb, ldx >= nverts. */
femgpu_status femgpu_solve_multi_device(femgpu_handle h, int nrhs, const double* d_B, int64_t ldb, double* d_X,
                                       int64_t ldx, femgpu_solve_stats* stats);

/* Independent problems at once: for each i, femgpu_setup(h[i]) when setup != 0, then
 * femgpu_solve(h[i], b[i], x[i], &stats[i]) (host arrays, each the size of its own
 * operator).  The handles must be distinct, each with its own stream (the default;
 * handles sharing a stream are refused with FEMGPU_ERR_INVALID).  The setups run on up
 * to `threads` host threads (0: one per handle), so the small problems' setup round trips
 * overlap.  With solverType 1 on one device, the PCG solves then run as ONE CUDA graph
 * launch: a branch per handle with its own device-side loop, so the meshes' iterations
 * share the GPU with no host round trip; the graph is kept for the same list of handles
 * and captured again when a hierarchy changes (stats[i].solve_ms is the whole graph's
 * time).  Otherwise (solverType 0, FEMGPU_HOST_LOOP set, a failed setup) each solve runs on
 * the host threads.  Every problem is attempted; the first failing status (in index
 * order) is returned, and each failing handle's femgpu_last_error names its problem.
 * stats may be NULL.
 * No reference counterpart (the reference solves one mesh per FEMSolver). */
femgpu_status femgpu_solve_batch(int count, femgpu_handle* h, const double* const* b, double* const* x, int setup,
                                 int threads, femgpu_solve_stats* stats);

/* Same as femgpu_solve with device pointers on the handle's stream (no copies). */
femgpu_status femgpu_solve_device(femgpu_handle h, const double* d_b, double* d_x,
                                  femgpu_solve_stats* stats);

/* Gradient of a loss L(u) with respect to theta_e = log c_e, the per-element
 * log-coefficients of the operator assembled by femgpu_assemble (A(theta) u = b with
 * the Dirichlet rows of femgpu_set_dirichlet eliminated): solves the adjoint system
 * A lambda = dL/du (its Dirichlet entries set to 0) with the current hierarchy and PCG
 * options, then dL/dtheta_e = -c_e lambda_e^T K_e u_e with K_e the element stiffness
 * for c_e = 1 (the mass term does not depend on theta).  Host arrays: dLdu and u
 * (nverts, u = the forward solution), dLdtheta (nelems).  stats may be NULL.
 * No reference counterpart: the reference computes no gradients. */
femgpu_status femgpu_adjoint_grad(femgpu_handle h, const double* dLdu, const double* u, double* dLdtheta,
                                 femgpu_solve_stats* stats);
/* Same with device pointers on the handle's stream. */
femgpu_status femgpu_adjoint_grad_device(femgpu_handle h, const double* d_dLdu, const double* d_u,
                                        double* d_grad, femgpu_solve_stats* stats);

/* y = A x with the level-0 FP64 operator, device pointers, original numbering.
 * Replaces cusp::multiply(Ahyb_d_CG, ...) in cgcycle.cu:24,38. */
femgpu_status femgpu_spmv_device(femgpu_handle h, const double* d_x, double* d_y);

/* ---- allocation-free load vector ----------------------------------------------- */
/* No reference counterpart.  Same result as femgpu_load_vector, but f and b are
 * device arrays (nverts doubles, original numbering) and the call allocates no
 * device memory.  It exists for callers that rebuild the right-hand side inside a
 * time step and cannot allocate there: applications that hand almost all device
 * memory to their own pool at start-up, or run under a fixed per-process memory
 * cap, where a hidden allocation mid-step can fail.
 * The two per-element scratch arrays live in a fixed region built into the
 * library: 2 x FEMGPU_NOALLOC_MAX_ELEMENTS doubles (32 MiB) per device, reserved
 * when this part of the library is first used under CUDA's lazy module loading (the
 * default since CUDA 12.2; with CUDA_MODULE_LOADING=EAGER, when the library is
 * loaded into a device context).  Meshes with more elements are
 * rejected with FEMGPU_ERR_LIMIT.  Nothing in the region has to start at zero:
 * each call writes every slot it reads.
 * The region is shared by every handle on a device, so calls that can overlap
 * on one device (different streams or threads) race; calls on one stream are
 * ordered.  The work is enqueued on the handle's stream and the call returns
 * without waiting.  The first call on each handle looks the region up (the first
 * on a device may also load this part of the library): make it before any stream
 * capture begins. */
#define FEMGPU_NOALLOC_MAX_ELEMENTS 2097152
femgpu_status femgpu_load_vector_device_noalloc(femgpu_handle h, const double* d_f, double* d_b);

/* ---- inspection (parity tests, statistics) --------------------------------- */
/* Pattern/values of the assembled level-0 matrix (original numbering). Any
 * output pointer may be NULL; n and nnz are always written. */
femgpu_status femgpu_get_matrix(femgpu_handle h, int64_t* n, int64_t* nnz, int32_t* rowptr,
                                int32_t* cols, double* vals);
/* Number of levels of the current hierarchy (AMG::num_levels). */
femgpu_status femgpu_num_levels(femgpu_handle h, int* levels);
femgpu_status femgpu_get_level_info(femgpu_handle h, int level, femgpu_level_info* info);
/* Level arrays: A (level's own numbering, values as double), the permutation
 * (old -> new), aggregate and partition offsets (SmoothedMG_AMG_Level members
 * permutation_d / aggregateIdx_d / partitionIdx_d) and P.  NULL skips an array. */
femgpu_status femgpu_level_get(femgpu_handle h, int level, int32_t* A_rowptr, int32_t* A_cols,
                               double* A_vals, int32_t* perm, int32_t* agg_idx, int32_t* part_idx,
                               int32_t* P_rowptr, int32_t* P_cols, double* P_vals);
/* One V-cycle z = M r on host vectors (AMG_Level::cycle_level0, amg_level.cu:74-128). */
femgpu_status femgpu_vcycle(femgpu_handle h, const double* r, double* z);
/* Times one hot kernel with CUDA events on the handle's stream (3 untimed launches,
 * then `reps`) and reports its average time and its algorithmic bytes per launch:
 * 0 = outer PCG FP64 SpMV (+ dot), 1 = level-0 pre-smoother, 2 = level-0 post-smoother
 * sweeps alone, 3 = level-0 restriction, 4 = level-0 prolongation, 5 = the level-0
 * post-smoother as a PCG iteration runs it (b - A_out x, sweeps, z in FP64 and the z.r
 * partials), 6 = the assembly's element kernel, 7 = its row-gather kernel (6 and 7 need
 * an operator assembled from the mesh, 0-5 a hierarchy; the operator is not changed).
 * No reference counterpart (measurement support). */
femgpu_status femgpu_profile_kernel(femgpu_handle h, int which, int reps, double* avg_ms, double* bytes);
/* Failure-detection testing: the level-0 register smoother waits at most `polls` polls
 * for the bulk copies of each group's entries before it records FEMGPU_ERR_LIMIT for the
 * solve (0: it gives up at once; negative: the default limit again).  A smoother CTA that
 * gives up still waits, with the full limit, for the copies it started, so the context
 * stays usable.  No reference counterpart. */
femgpu_status femgpu_test_copy_wait_limit(femgpu_handle h, int polls);
/* Number of kernel launches issued by the library on this handle so far. */
femgpu_status femgpu_kernel_launches(femgpu_handle h, int64_t* count);

/* ---- file IO (host) ---------------------------------------------------------- */
/* Reads .node/.ele (TetMesh::read, tetmesh.cu:251-376) or ASCII/binary-LE PLY
 * (TriMesh::read, TriMesh_io.cu:146-257).  Two-call protocol: with NULL arrays
 * only the counts are returned.  Coordinates are parsed as float, as the reference. */
femgpu_status femgpu_read_tetgen(const char* node_file, const char* ele_file, int64_t* nverts,
                                 int64_t* nelems, double* xyz, int32_t* conn, int32_t* labels);
femgpu_status femgpu_read_ply(const char* file, int64_t* nverts, int64_t* nfaces, double* xyz,
                              int32_t* conn);
/* MAT v5 (uncompressed) sparse matrix / double array, FEMSolver::readMatlabSparseMatrix /
 * readMatlabArray (src/FEMSolver.cu:177-449).  Sparse output is CSR with sorted columns. */
femgpu_status femgpu_read_mat_sparse(const char* file, int64_t* rows, int64_t* cols, int64_t* nnz,
                                     int32_t* rowptr, int32_t* colidx, double* vals);
femgpu_status femgpu_read_mat_array(const char* file, int64_t* n, double* vals);
/* FEMSolver::writeMatlabArray / writeVTK (src/FEMSolver.cu:451-582). */
femgpu_status femgpu_write_mat_array(const char* file, int64_t n, const double* vals);
femgpu_status femgpu_write_vtk(const char* file, int dim, int64_t nverts, const double* xyz,
                               int64_t nelems, const int32_t* conn, const double* values);

#ifdef __cplusplus
}
#endif
#endif /* FEMGPU_H */
