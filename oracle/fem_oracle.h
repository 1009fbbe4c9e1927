/*
 * fem_oracle.h -- CPU restatement of SCI-Solver_FEM's P1 FEM -> SA-AMG -> PCG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * implementation in sci-solver_fem_gb300/ and the timed CPU baseline of bench.py.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product path never calls it.
 *
 * Parity pins: the quadrature tables, the glibc rand() stream, the element
 * matrices and the fixture solves are checked against the reference's own test
 * data (src/test/test_data) and against libc in tests/test_oracle_*.py.
 *
 * Every function cites the reference file:line it restates.  Deliberate
 * deviations from the reference are listed in each function's comment:
 *   - randomizedMIS takes a seed instead of srand(time(NULL));
 *   - the level-0 permutation is applied to b and x (the reference forgets it);
 *   - the coarsest solve is an FP64 dense Cholesky/LU instead of a host FP32 LU;
 *   - never-ending loops of the reference end with an error status.
 */
#ifndef FEM_ORACLE_H
#define FEM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* glibc TYPE_3 rand() restated: srand(seed) then n draws. */
void orc_glibc_rand(uint32_t seed, int n, int32_t* out);

/* FEM3D quadrature (FEM3D.cu:58-557): reference-tet mass integrand, 10 values. */
void orc_tet_mass_integrand(double out[10]);
/* FEM2D quadrature (FEM2D.cu:200-378): 6 zeros/weights in x and y. */
void orc_tri_quadrature(double zx[6], double wx[6], double zy[6], double wy[6]);

/* Mesh pattern (tetmesh.cu:112-170 + cutil.cu:168-230): CSR with sorted columns,
 * diagonal included.  rowptr has nv+1 entries; cols must hold cap ints.
 * Returns nnz or -1 if cap is too small / input invalid. */
int64_t orc_build_pattern(int nv, int ne, int nvpe, const int32_t* conn,
                          int32_t* rowptr, int32_t* cols, int64_t cap);

/* Element assembly into the CSR pattern.  dim 3: tets (perform_element_loop_3D.cuh:480-627),
 * dim 2: triangles (perform_element_loop_2D.cuh:287-372).  xyz holds 3 doubles per
 * vertex in both cases (z ignored in 2D).  coef[e] scales element e's stiffness; when
 * coef is NULL the 3D coefficient comes from labels (co table) and 2D uses 1.
 * vals receives A = sum_e coef_e K_e + lambda_mass M_e, summed in element order.
 * Tetrahedra: reference_formula = 1 evaluates the reference's 4x4 cofactor inverse term
 * for term (perform_element_loop_3D.cuh:525-583); 0 evaluates the library's fused
 * multiply-add gradients (fem_assembly.cu tet_gradients), which the GPU matches bit for
 * bit and which agree with the reference formula to 1e-13 relative. */
int orc_assemble(int dim, int nv, const double* xyz, int ne, const int32_t* conn,
                 const int32_t* labels, const double* coef, double lambda_mass,
                 const int32_t* rowptr, const int32_t* cols, double* vals, int reference_formula);

/* Consistent P1 load vector b_i = sum_e int f_h phi_i (exact P1 mass). */
int orc_load_vector(int dim, int nv, const double* xyz, int ne, const int32_t* conn,
                    const double* f, double* b);

/* Symmetric Dirichlet elimination: rows/cols of masked dofs zeroed, unit diagonal. */
void orc_apply_dirichlet(int n, const int32_t* rowptr, const int32_t* cols, double* vals,
                         const uint8_t* mask, double* b /* may be NULL */);

/* Distance-k randomized MIS (randomizedMIS_GPU.cu:3-272), seeded. mis[i] in {0,1}. */
int orc_random_mis(int n, const int32_t* xadj, const int32_t* adj, int k, uint32_t seed,
                   int32_t* mis);

/* OldMIS two-level aggregation (ComputePermutationMethods.cu:22-151).
 * Output arrays need capacity n (+1 for index arrays); adj_out capacity = nnz(adj).
 * Returns 0 on success. */
int orc_oldmis(int n, const int32_t* xadj, const int32_t* adj, int params, int part_max,
               uint32_t seed, int32_t* permutation, int32_t* ipermutation,
               int32_t* aggregate_idx, int32_t* n_agg, int32_t* partition_idx,
               int32_t* n_part, int32_t* partition_label, int32_t* xadj_out,
               int32_t* adj_out, int32_t* nnz_out);

/* ---- AMG hierarchy + solver ------------------------------------------------ */
typedef struct orc_amg orc_amg;

typedef struct {
  int max_levels;        /* maxLevels_ 100 */
  int top_size;          /* topSize_ 256 */
  int rand_mis_params;   /* randMisParameters_ 90102 */
  int partition_max;     /* partitionMaxSize_ 512 */
  int pre_inner;         /* preInnerIters_ 5 */
  int post_inner;        /* postInnerIters_ 5 */
  int post_relaxes;      /* postRelaxes_ 1 */
  double smoother_weight;/* smootherWeight_ 1.0 */
  double pro_omega;      /* proOmega_ 0.67 */
  uint32_t seed;         /* replaces srand(time(NULL)) */
  int fp64_hierarchy;    /* 0: FP32 hierarchy (reference), 1: FP64 */
  int threads;           /* OpenMP threads for the timed baseline (0 = default) */
  int cycle_type;        /* cycleType_ 0 = V, 1 = W, 2 = F (the reference's W_Cycle / F_Cycle
                            visit patterns, second visits in residual-correction form) */
  int smoother;          /* 0 = partition-block Jacobi (reference), 1 = l1-Jacobi on Ap */
} orc_config;

void orc_config_default(orc_config* c);

/* Build the hierarchy from an FP64 CSR matrix (sorted columns) and the level-0
 * aggregation graph (CSR without self loops).  Returns NULL on failure; *status gets
 * an error code. */
orc_amg* orc_amg_setup(const orc_config* cfg, int n, const int32_t* rowptr,
                       const int32_t* cols, const double* vals, const int32_t* gxadj,
                       const int32_t* gadj, int* status);
void orc_amg_free(orc_amg* h);
int orc_amg_num_levels(const orc_amg* h);
/* Level info: n, nnz(A), n_agg, n_part, nnz(P). */
int orc_amg_level_info(const orc_amg* h, int level, int64_t* info5);
/* Copy level arrays out (any pointer may be NULL). A is the level matrix in the
 * level's own (unpermuted) numbering, values converted to double. */
int orc_amg_level_get(const orc_amg* h, int level, int32_t* A_rowptr, int32_t* A_cols,
                      double* A_vals, int32_t* perm, int32_t* agg_idx, int32_t* part_idx,
                      int32_t* P_rowptr, int32_t* P_cols, double* P_vals);
/* One V-cycle z = M r on the original (unpermuted) level-0 numbering. */
int orc_amg_vcycle(orc_amg* h, const double* r, double* z);
/* PCG (cgcycle.cu:6-69): flexible = 0 standard Fletcher-Reeves, 1 Polak-Ribiere.
 * x holds the initial guess.  Returns 0 converged, 5 not converged, 4 breakdown. */
int orc_amg_pcg(orc_amg* h, const double* b, double* x, double tol, int max_iters,
                int flexible, int* iters, double* relres);
/* Plain FP64 CG without preconditioner on a CSR (used as the 1e-12 reference). */
int orc_cg(int n, const int32_t* rowptr, const int32_t* cols, const double* vals,
           const double* b, double* x, double tol, int max_iters, int* iters, double* relres);

#ifdef __cplusplus
}
#endif
#endif
