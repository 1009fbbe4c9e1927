// context.cuh -- solver context (one per femgpu_handle) and the AMG level layout.
//
// Device layout of one level (all arrays in HBM, indices int32):
//   A      CSR of the level operator in the level's own numbering (T values);
//   perm   old -> new row id (aggregate-contiguous, partition-contiguous order);
//   Ap     CSR of perm(A) with sorted columns;
//   diag   diagonal of Ap;
//   Ain    per row: in-partition off-diagonal entries (upper value mirrored);
//   Aout   per row: cross-partition entries;
//   P, R   prolongator (n x n_agg) and its transpose;
//   agg_idx / part_idx   aggregate offsets over new rows, partition offsets over aggregates.
// The coarsest level keeps the explicit inverse of its dense matrix (FP64).
#pragma once

#include <atomic>
#include <memory>
#include <string>

#include "common.cuh"

namespace femgpu {

extern std::atomic<int64_t> g_kernel_launches;

#define FG_LAUNCH(kernel, grid, block, smem, stream, ...)                     \
  do {                                                                        \
    ::femgpu::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);      \
    kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);               \
    FG_CHECK_LAUNCH();                                                        \
  } while (0)

// A kernel launch with programmatic dependent launch (the kernel calls pdl_wait() before
// it touches memory that other kernels write), counted like FG_LAUNCH.  The attribute is
// set only inside a PdlScope that allows it: the V-cycle of a level with at most
// kPdlLevelRows rows, whose small kernels are bound by launch latency.  Elsewhere (the
// large level-0 kernels, the PCG vector kernels) early-scheduled successors waiting on
// the SMs slowed the running kernel, so those launch plainly.
extern bool g_pdl_enabled;
extern thread_local bool t_pdl_scope;
constexpr int64_t kPdlLevelRows = 1 << 18;
struct PdlScope {
  bool old;
  explicit PdlScope(bool on) : old(t_pdl_scope) { t_pdl_scope = on; }
  ~PdlScope() { t_pdl_scope = old; }
};
template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl_enabled && t_pdl_scope ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

#define FG_LAUNCH_PDL(kernel, grid, block, smem, stream, ...)                                  \
  do {                                                                                         \
    ::femgpu::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);                       \
    FG_CUDA(::femgpu::launch_pdl((kernel), dim3(grid), dim3(block), (smem), (stream), __VA_ARGS__)); \
  } while (0)

struct Mesh {
  int dim = 0, k = 0;
  int64_t nv = 0, ne = 0;
  bool has_labels = false;
  DBuf<double> xyz;       // nv x 3
  DBuf<int32_t> conn;     // ne x k
  DBuf<int32_t> labels;   // ne
  DBuf<int32_t> vstart;   // nv + 1: incidence offsets
  DBuf<int32_t> inc;      // ne * k: e * k + a, sorted per vertex
  // slot[q * k + b]: position, within the row of incidence q's vertex, of the column of
  // vertex b of q's element (rows of at most kSlotRowMax entries; empty otherwise)
  DBuf<uint8_t> slot;
};
constexpr int kSlotRowMax = 32;

template <class T>
struct Level {
  int n = 0, nagg = 0, npart = 0;
  bool coarsest = false;
  DCsr<T> A;
  DBuf<int32_t> gxadj, gadj;  // aggregation graph of this level
  int64_t gnnz = 0;
  DBuf<int32_t> perm, iperm, agg_idx, part_idx, agg_of;
  DCsr<T> Ap, Ain, Aout, P, R;
  DBuf<T> diag, dinv;  // diagonal of Ap and its reciprocal
  int max_part_rows = 0;
  int max_part_entries = 0;  // in-partition off-diagonal entries of the largest partition
  int max_in_row = 0;        // longest in-partition row
  // smoother work groups: consecutive partitions packed per CTA (row offsets)
  DBuf<int32_t> grows;
  int ngroups = 0, max_group_rows = 0, max_group_ents = 0;
  // register smoother: the in-partition entries of every 32-row block of a group in
  // jagged-diagonal order (the block's rows sorted by decreasing length, stable; entry k
  // of the row at sorted position p sits at (block's first entry) + (entries of the
  // block's diagonals 0..k-1) + p), so lane p of a warp reads its entries from consecutive
  // addresses.  jv: values; jc16: the column relative to the group's first row plus
  // c * xcopy_stride<T>() for the copy of x the entry reads (chosen at setup to spread a
  // warp's gathers over the shared-memory banks); jrow: per slot of a block, the sorted
  // row's offset in the block.  jv and jc16 carry 16 entries of slack like Ain.v, so
  // 16-byte rounded bulk copies stay inside.
  DBuf<T> jv;
  DBuf<uint16_t> jc16;
  DBuf<uint8_t> jrow;
  // shared-memory smoother plan: lanes per row, CTAs per cluster (one cluster per
  // group), rows and entries of the largest CTA row slice, launch shape
  int smooth_lanes = 1, cluster = 1, slice_rows = 0, slice_ents = 0, smooth_threads = 0, smooth_grid = 0;
  int smooth_k = 0;  // entries per lane of the register-resident cluster smoother (0: not used)
  bool smooth_staged = false;
  size_t smooth_smem = 0;
  // coarsest: explicit inverse, row-major n x n
  DBuf<double> Ainv;
  // work vectors (level numbering / permuted numbering)
  DBuf<T> b, x, r, xo, t, bp;  // bp: post-smoother right-hand side
  DBuf<T> wr, wd;              // W- and F-cycles: residual and correction of a second visit
  int aout_lanes_tuned = 0;    // lanes per row of the cross-partition products (0: the rule)
  DBuf<T> l1inv;               // l1-Jacobi smoother: 1 / sum_j |a_ij| of Ap's rows
  // mixed precision: A's values in FP64 when its Galerkin product was formed in FP64 (the
  // coarse end of the hierarchy); the coarsest level's dense factorisation reads them
  DBuf<double> A64v;
};

// Level-0-style smoother in registers: rows of at most 16 in-partition entries and
// partitions of at most 512 rows (one thread per row).
// Mixed precision forms the Galerkin products whose result has at most
// kFp64GalerkinPerTop x topSize rows in FP64 (FP32 operands widened exactly, products and
// sums in double in the usual generation order, the result rounded to FP32 for the level).
// At the benchmark configurations these are the two coarsest levels' products.
constexpr int kFp64GalerkinPerTop = 32;

constexpr int kRegRow = 16;
constexpr int kRegGroupRows = 512;
// The register smoother keeps kXCopies copies of the group's x in shared memory,
// xcopy_stride<T>() elements apart: a stride 32 bytes past a multiple of 128 bytes, so
// copy c of an element sits 8c banks further on.  Slot kRegGroupRows of copy 0 is spare.
constexpr int kXCopies = 4;
template <class T>
__host__ __device__ constexpr int xcopy_stride() {
  return sizeof(T) == 4 ? 520 : 516;
}
inline bool smoother_in_registers(int max_in_row, int max_part_rows) {
  return max_in_row <= kRegRow && max_part_rows <= kRegGroupRows;
}

// Lanes per row of the shared-memory smoother's in-partition sums (the CPU oracle
// uses the same rule): doubled while every lane still adds at least 3 entries of an
// average row and rows x lanes stay within one wave of 152 SMs x 2048 threads, then
// while the longest row leaves a lane more than 16 entries (so they fit registers).
constexpr int64_t kSmoothThreadBudget = 152LL * 2048;
constexpr int kLaneEntries = 16;
inline int smooth_lanes_for(int64_t rows, int64_t in_nnz, int max_row) {
  const int64_t avg = rows > 0 ? (in_nnz + rows - 1) / rows : 0;
  int s = 1;
  while (s < 32 && 3 * (2 * s) <= avg && rows * (2 * s) <= kSmoothThreadBudget) s <<= 1;
  while (s < 32 && (max_row + s - 1) / s > kLaneEntries) s <<= 1;
  return s;
}

struct HierarchyBase {
  virtual ~HierarchyBase() {}
  int num_levels = 0;
};

template <class T>
struct Hierarchy : HierarchyBase {
  std::vector<std::unique_ptr<Level<T>>> L;
};

// Work state of the multi-right-hand-side solve (block_solve.cu), kept per handle.
struct BlockStateBase {
  virtual ~BlockStateBase() {}
};

struct Ctx {
  femgpu_config cfg{};
  int device = 0;
  cudaStream_t stream = 0;
  bool own_stream = false;
  cudaMemPool_t pool = nullptr;  // every device buffer of the handle comes from here
  bool own_pool = false;
  std::string last_error;

  Mesh mesh;
  bool has_mesh = false;
  DBuf<double> coef;             // per-element coefficients of the last femgpu_assemble (empty: labels / 1)
  double lambda_mass = 0.0;      // mass weight of the last femgpu_assemble
  DBuf<uint8_t> dmask;           // Dirichlet mask of the last femgpu_set_dirichlet (empty: none)
  bool assembled_from_mesh = false;
  DCsr<double> A;                // level-0 operator, original numbering, FP64
  DBuf<int32_t> gxadj, gadj;     // level-0 aggregation graph
  int64_t graph_nnz = 0;
  bool has_matrix = false;

  // hierarchy (built by femgpu_setup)
  std::unique_ptr<HierarchyBase> H;
  DBuf<int32_t> perm0;           // level-0 old -> new (identity if level 0 is the coarsest)
  DCsr<double> A0p;              // FP64 level-0 operator in permuted order (outer PCG)
  // The same operator as slices of 32 rows (used instead of A0p when padding is small):
  // entry k of row 32 s + j sits at s_off[s] + 32 k + j; padding has column -1.
  bool sliced = false;
  int64_t s_padded = 0;
  DBuf<int32_t> s_off, s_ci;
  DBuf<double> s_v;
  bool has_hierarchy = false;
  double setup_ms = 0.0;

  // PCG work vectors (permuted order)
  DBuf<double> vb, vx, vr, vz, vp, vy, vrold;
  DBuf<double> red;              // reduction partials + scalars
  DBuf<unsigned> rcount;         // last-block tickets of the fused reductions
  double* h_scalars = nullptr;   // pinned host mirror of the device scalars
  // one PCG iteration captured as a CUDA graph, rebuilt when the hierarchy changes
  uint64_t hier_gen = 0, graph_gen = ~0ull;
  int graph_flexible = -1;
  cudaGraphExec_t pcg_exec = nullptr;
  int64_t graph_nodes = 0;
  // z.r (and z.r_old) of the PCG iteration being enqueued, requested from the level-0
  // post-smoother that writes z; `done` tells whether it took them (and formed beta)
  struct ZDot {
    const double* r = nullptr;
    const double* rold = nullptr;
    double* part = nullptr;
    bool done = false;
  };
  ZDot* zdot = nullptr;
  // polls of the register smoother's wait for its staged entries before it gives up
  // (femgpu_test_copy_wait_limit lowers it to exercise the error path)
  int copy_wait_limit = kMbarWaitLimit;
  // block vectors and scalars of the multi-right-hand-side solve, rebuilt with the hierarchy
  std::unique_ptr<BlockStateBase> block;
  // device address of the no-alloc load vector's built-in scratch region, looked up by
  // the first such call on this handle (a handle lives in one device context)
  double* noalloc_scratch = nullptr;
  // stage timing of a V-cycle run outside capture (FEMGPU_PROFILE set): named events
  std::vector<std::pair<std::string, cudaEvent_t>>* stage_marks = nullptr;
  // b and x of this handle's branch in a batch graph (original numbering)
  DBuf<double> bat_b, bat_x;

  ~Ctx() {
    if (pcg_exec) cudaGraphExecDestroy(pcg_exec);
  }
};

// fem_assembly.cu
void build_mesh_pattern(Ctx& c);
// coef: per-element coefficients (host array, or device array when coef_on_device), or null
void assemble_operator(Ctx& c, const double* coef_host, double lambda, bool coef_on_device = false);
void load_vector(Ctx& c, const double* f_host, double* b_host);
// The two load-vector passes on device f/b with caller-provided scratch (`scale`
// and `fsum`, one double per element each); enqueued on c.stream, allocates nothing.
void load_vector_enqueue(Ctx& c, const double* d_f, double* d_b, double* scale, double* fsum);
void apply_dirichlet(Ctx& c, const uint8_t* mask_host);
// out = in with the Dirichlet rows set to zero (n = rows of the operator).
void zero_dirichlet_rows(Ctx& c, const double* d_in, double* d_out);
// dL/dtheta_e = -c_e lambda_e^T K_e u_e for theta_e = log c_e (per element, device arrays).
void element_log_coef_gradient(Ctx& c, const double* d_lam, const double* d_u, double* d_grad);
// Times the assembly's element kernel (which = 6) or row-gather kernel (which = 7) with
// CUDA events on c.stream for the current mesh and coefficients, writing into scratch
// buffers (the operator is left as it is); reports the average time and the algorithmic
// bytes per launch.
void profile_assembly(Ctx& c, int which, int reps, double* ms, double* bytes);

// amg_setup.cu
void amg_setup(Ctx& c);

// hierarchy_io.cu: the hierarchy to / from a file (the load checks that the handle holds
// the operator it was built for)
void save_hierarchy(Ctx& c, const char* path);
void load_hierarchy(Ctx& c, const char* path);

// amg_solve.cu
struct SolveResult {
  int iterations = 0;
  double relres = 0.0;
  femgpu_status status = FEMGPU_OK;
};
SolveResult amg_solve_device(Ctx& c, const double* d_b, double* d_x);
// Chooses the smoother's launch plan for a level whose groups are built.
template <class T>
void plan_smoother(Ctx& c, Level<T>& L);
// Times the level's result-neutral launch choices (cross-partition lanes, cluster size) and
// keeps the fastest (cached per device and level shape); no-op when cfg.autotune is 0.
template <class T>
void autotune_level(Ctx& c, Level<T>& L);
// The PCG solves of several handles (same device, hierarchies built) as one CUDA graph
// launched on hs[0]'s stream: per handle an independent branch with its own device-side
// loop, reading b and x from c.bat_b / c.bat_x (filled by the caller after batch_prepare)
// and writing x back there.  The graph is kept per handle list and recaptured when a
// hierarchy changes.  Returns false when the graph could not be built (nothing ran).
void batch_prepare(Ctx& c);
bool batch_solve_graph(const std::vector<Ctx*>& hs, std::vector<SolveResult>& res, float* ms);
void batch_forget(Ctx* c);  // drops the kept graphs that use c (before c is destroyed)
void amg_vcycle_device(Ctx& c, const double* d_r, double* d_z);
void spmv_original(Ctx& c, const double* d_x, double* d_y);
void profile_kernel(Ctx& c, int which, int reps, double* ms, double* bytes);

// block_solve.cu: nrhs right-hand sides (column j at d_B + j * ldb, initial guesses and
// solutions at d_X + j * ldx), eight at a time in lockstep PCGs whose operator and V-cycle
// applications are block (SpMM) kernels; per column: iterations, relative residual, status.
void block_solve_device(Ctx& c, int nrhs, const double* d_B, int64_t ldb, double* d_X, int64_t ldx, int* iters,
                        double* relres, femgpu_status* status);

}  // namespace femgpu
