// capi.cu -- extern "C" entry points of include/femgpu.h.
//
// Every entry point catches library errors and CUDA failures and turns them into
// a status code (the reference calls exit() on bad input, gauss_seidel.cu:2060-2064;
// tetmesh.cu:257-260); the message is kept on the handle (femgpu_last_error).
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "context.cuh"

using namespace femgpu;

struct femgpu_ctx : Ctx {};

namespace {

thread_local std::string g_last_global_error;

// Routes the handle's allocations to its pool for the duration of one call.
struct PoolScope {
  cudaMemPool_t saved;
  explicit PoolScope(femgpu_handle h) : saved(g_alloc_pool) { g_alloc_pool = h ? h->pool : nullptr; }
  ~PoolScope() { g_alloc_pool = saved; }
};

// Runs fn for an entry point: the handle's memory pool and device, exceptions turned into
// status codes, and (with a name) an NVTX range around the call.
femgpu_status guard(femgpu_handle h, const std::function<void()>& fn, const char* trace = nullptr) {
  PoolScope scope(h);
  TraceRange range(trace);
  try {
    if (h) FG_CUDA(cudaSetDevice(h->device));
    fn();
    return FEMGPU_OK;
  } catch (const Error& e) {
    if (h) h->last_error = e.what();
    else g_last_global_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    if (h) h->last_error = e.what();
    else g_last_global_error = e.what();
    return FEMGPU_ERR_INVALID;
  }
}

__global__ void graph_count_kernel(int n, const int32_t* rp, const int32_t* ci, int32_t* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int c = 0;
    for (int e = rp[i]; e < rp[i + 1]; e++) c += ci[e] != i;
    cnt[i] = c;
  }
}

__global__ void graph_fill_kernel(int n, const int32_t* rp, const int32_t* ci, const int32_t* xadj, int32_t* adj) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int o = xadj[i];
    for (int e = rp[i]; e < rp[i + 1]; e++)
      if (ci[e] != i) adj[o++] = ci[e];
  }
}

// Aggregation graph from the operator's own pattern (used without a mesh).
void graph_from_matrix(Ctx& c) {
  cudaStream_t s = c.stream;
  const int n = c.A.n;
  DBuf<int32_t> cnt(n + 1, s);
  FG_LAUNCH(graph_count_kernel, grid_for(n, 256), 256, 0, s, n, c.A.rp.p, c.A.ci.p, cnt.p);
  c.gxadj.alloc(n + 1, s);
  c.graph_nnz = exclusive_scan(cnt.p, c.gxadj.p, n, s);
  c.gadj.alloc(c.graph_nnz > 0 ? c.graph_nnz : 1, s);
  FG_LAUNCH(graph_fill_kernel, grid_for(n, 256), 256, 0, s, n, c.A.rp.p, c.A.ci.p, c.gxadj.p, c.gadj.p);
}

void invalidate_hierarchy(Ctx& c) {
  c.H.reset();
  c.has_hierarchy = false;
}

template <class T>
Level<T>& level_of(Ctx& c, int level) {
  auto& H = static_cast<Hierarchy<T>&>(*c.H);
  FG_REQUIRE(level >= 0 && level < (int)H.L.size(), FEMGPU_ERR_INVALID, "level out of range");
  return *H.L[level];
}

template <class T>
void fill_level_info(Ctx& c, int level, femgpu_level_info* info) {
  Level<T>& L = level_of<T>(c, level);
  info->rows = L.A.n;
  info->nnz = L.A.nnz;
  info->aggregates = L.coarsest ? 0 : L.nagg;
  info->partitions = L.coarsest ? 0 : L.npart;
  info->nnz_p = L.coarsest ? 0 : L.P.nnz;
}

template <class T>
void copy_vals(const DBuf<T>& src, int64_t n, double* dst) {
  std::vector<T> h(n);
  src.download(h.data(), n);
  FG_CUDA(cudaStreamSynchronize(src.s));
  for (int64_t i = 0; i < n; i++) dst[i] = (double)h[i];
}

template <class T>
void get_level(Ctx& c, int level, int32_t* Arp, int32_t* Aci, double* Av, int32_t* perm, int32_t* agg,
               int32_t* part, int32_t* Prp, int32_t* Pci, double* Pv) {
  Level<T>& L = level_of<T>(c, level);
  cudaStream_t s = c.stream;
  if (Arp) L.A.rp.download(Arp, L.A.n + 1);
  if (Aci) L.A.ci.download(Aci, L.A.nnz);
  if (Av) copy_vals(L.A.v, L.A.nnz, Av);
  if (!L.coarsest) {
    if (perm) L.perm.download(perm, L.n);
    if (agg) L.agg_idx.download(agg, L.nagg + 1);
    if (part) L.part_idx.download(part, L.npart + 1);
    if (Prp) L.P.rp.download(Prp, L.n + 1);
    if (Pci) L.P.ci.download(Pci, L.P.nnz);
    if (Pv) copy_vals(L.P.v, L.P.nnz, Pv);
  }
  FG_CUDA(cudaStreamSynchronize(s));
  // P's columns are kept in the next level's own order when that level is not the
  // coarsest; report them in its original (aggregate) numbering
  if (!L.coarsest && Pci && level + 1 < c.H->num_levels) {
    const Level<T>& N = level_of<T>(c, level + 1);
    if (!N.coarsest) {
      std::vector<int32_t> ip = N.iperm.to_host();
      for (int64_t e = 0; e < L.P.nnz; e++) Pci[e] = ip[Pci[e]];
    }
  }
}

}  // namespace

extern "C" {

void femgpu_config_default(femgpu_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->verbose = 0;
  c->maxLevels = 100;
  c->maxIters = 100;
  c->preInnerIters = 5;
  c->postInnerIters = 5;
  c->postRelaxes = 1;
  c->cycleIters = 1;
  c->dsType = 0;
  c->topSize = 256;
  c->randMisParameters = 90102;
  c->partitionMaxSize = 512;
  c->aggregatorType = 0;
  c->convergeType = 0;
  c->tolerance = 1e-6;
  c->cycleType = 0;
  c->solverType = 0;
  c->smootherWeight = 1.0;
  c->proOmega = 0.67;
  c->device = 0;
  c->blockSize = 256;
  c->seed = 1;
  c->precision = 0;
  c->flexibleCG = 0;
  c->stream = nullptr;
  c->mem_pool = nullptr;
  c->autotune = 1;
  c->smoother = 0;
}

const char* femgpu_status_string(femgpu_status s) {
  switch (s) {
    case FEMGPU_OK: return "ok";
    case FEMGPU_ERR_INVALID: return "invalid argument";
    case FEMGPU_ERR_CUDA: return "CUDA error";
    case FEMGPU_ERR_NOT_READY: return "not ready";
    case FEMGPU_ERR_BREAKDOWN: return "breakdown";
    case FEMGPU_ERR_NOT_CONVERGED: return "not converged";
    case FEMGPU_ERR_LIMIT: return "limit reached";
    case FEMGPU_ERR_IO: return "I/O error";
    case FEMGPU_ERR_ALLOC: return "allocation failed";
    case FEMGPU_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char* femgpu_last_error(femgpu_handle h) { return h ? h->last_error.c_str() : g_last_global_error.c_str(); }

femgpu_status femgpu_create(femgpu_handle* out, const femgpu_config* cfg) {
  if (!out) return FEMGPU_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    g_last_global_error = "no CUDA device visible";
    return FEMGPU_ERR_NO_DEVICE;
  }
  femgpu_ctx* h = new femgpu_ctx();
  if (cfg) h->cfg = *cfg;
  else femgpu_config_default(&h->cfg);
  if (h->cfg.device < 0 || h->cfg.device >= count) {
    delete h;
    g_last_global_error = "device index out of range";
    return FEMGPU_ERR_INVALID;
  }
  if (h->cfg.cycleType < 0 || h->cfg.cycleType > 2 || (h->cfg.precision != 0 && h->cfg.precision != 1) ||
      (h->cfg.smoother != 0 && h->cfg.smoother != 1)) {
    delete h;
    g_last_global_error = "cycleType must be 0 (V), 1 (W) or 2 (F), precision and smoother 0 or 1";
    return FEMGPU_ERR_INVALID;
  }
  h->device = h->cfg.device;
  femgpu_status st = guard(h, [&] {
    if (h->cfg.stream) {
      h->stream = (cudaStream_t)h->cfg.stream;
    } else {
      FG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
      h->own_stream = true;
    }
    if (h->cfg.mem_pool) {
      h->pool = (cudaMemPool_t)h->cfg.mem_pool;
    } else {
      // freed memory stays in the pool for the next setup instead of going back to
      // the driver at every synchronization
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = h->device;
      FG_CUDA(cudaMemPoolCreate(&h->pool, &props));
      h->own_pool = true;
      uint64_t keep = UINT64_MAX;
      FG_CUDA(cudaMemPoolSetAttribute(h->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
  });
  if (st != FEMGPU_OK) {
    g_last_global_error = h->last_error;
    if (h->own_stream) cudaStreamDestroy(h->stream);
    if (h->own_pool) cudaMemPoolDestroy(h->pool);
    delete h;
    return st;
  }
  *out = h;
  return FEMGPU_OK;
}

femgpu_status femgpu_destroy(femgpu_handle h) {
  if (!h) return FEMGPU_ERR_INVALID;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  cudaStream_t s = h->stream;
  bool own = h->own_stream;
  cudaMemPool_t pool = h->own_pool ? h->pool : nullptr;
  batch_forget(h);  // kept batch graphs that point into this handle's buffers
  if (h->h_scalars) cudaFreeHost(h->h_scalars);
  delete h;  // buffers free asynchronously on s
  cudaStreamSynchronize(s);
  if (own) cudaStreamDestroy(s);
  if (pool) cudaMemPoolDestroy(pool);
  return FEMGPU_OK;
}

femgpu_status femgpu_set_config(femgpu_handle h, const femgpu_config* cfg) {
  if (!h || !cfg) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(cfg->maxLevels >= 1 && cfg->topSize >= 1 && cfg->maxIters >= 0, FEMGPU_ERR_INVALID,
               "maxLevels, topSize must be >= 1 and maxIters >= 0");
    FG_REQUIRE(cfg->partitionMaxSize >= 1 && cfg->preInnerIters >= 0 && cfg->postInnerIters >= 0 &&
                   cfg->postRelaxes >= 0,
               FEMGPU_ERR_INVALID, "invalid smoother options");
    FG_REQUIRE(cfg->precision == 0 || cfg->precision == 1, FEMGPU_ERR_INVALID, "precision must be 0 or 1");
    FG_REQUIRE(cfg->cycleType >= 0 && cfg->cycleType <= 2, FEMGPU_ERR_INVALID, "cycleType must be 0 (V), 1 (W) or 2 (F)");
    FG_REQUIRE(cfg->smoother == 0 || cfg->smoother == 1, FEMGPU_ERR_INVALID, "smoother must be 0 or 1");
    femgpu_config c = *cfg;
    c.device = h->cfg.device;
    c.stream = h->cfg.stream;
    c.mem_pool = h->cfg.mem_pool;
    bool rebuild = c.precision != h->cfg.precision || c.seed != h->cfg.seed || c.maxLevels != h->cfg.maxLevels ||
                   c.topSize != h->cfg.topSize || c.randMisParameters != h->cfg.randMisParameters ||
                   c.partitionMaxSize != h->cfg.partitionMaxSize || c.proOmega != h->cfg.proOmega ||
                   c.aggregatorType != h->cfg.aggregatorType;
    h->cfg = c;
    if (rebuild) invalidate_hierarchy(*h);
    h->hier_gen++;  // captured solve loops hold the old options (cycle, sweeps, weights): capture again
  });
}

femgpu_status femgpu_set_mesh(femgpu_handle h, int dim, int64_t nverts, const double* xyz, int64_t nelems,
                              const int32_t* conn, const int32_t* labels) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(dim == 2 || dim == 3, FEMGPU_ERR_INVALID, "dim must be 2 or 3");
    FG_REQUIRE(nverts > 0 && nelems > 0 && xyz && conn, FEMGPU_ERR_INVALID, "empty mesh");
    FG_REQUIRE(nverts < INT32_MAX && nelems * (dim + 1) < INT32_MAX, FEMGPU_ERR_LIMIT, "mesh exceeds int32 indexing");
    invalidate_hierarchy(*h);
    cudaStream_t s = h->stream;
    Mesh& M = h->mesh;
    M.dim = dim;
    M.k = dim + 1;
    M.nv = nverts;
    M.ne = nelems;
    M.xyz.alloc(nverts * 3, s);
    M.xyz.upload(xyz, nverts * 3);
    M.conn.alloc(nelems * M.k, s);
    M.conn.upload(conn, nelems * M.k);
    M.has_labels = labels != nullptr;
    if (labels) {
      M.labels.alloc(nelems, s);
      M.labels.upload(labels, nelems);
    }
    build_mesh_pattern(*h);
    h->has_mesh = true;
    h->has_matrix = false;
    FG_CUDA(cudaStreamSynchronize(s));
  });
}

femgpu_status femgpu_assemble(femgpu_handle h, const double* coef, double lambda_mass) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    invalidate_hierarchy(*h);
    assemble_operator(*h, coef, lambda_mass);
    h->has_matrix = true;
    h->assembled_from_mesh = true;
    h->dmask.release();
    FG_CUDA(cudaStreamSynchronize(h->stream));
  }, "femgpu_assemble");
}

femgpu_status femgpu_assemble_device(femgpu_handle h, const double* d_coef, double lambda_mass) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    invalidate_hierarchy(*h);
    assemble_operator(*h, d_coef, lambda_mass, true);
    h->has_matrix = true;
    h->assembled_from_mesh = true;
    h->dmask.release();
    FG_CUDA(cudaStreamSynchronize(h->stream));
  }, "femgpu_assemble_device");
}

femgpu_status femgpu_load_vector(femgpu_handle h, const double* f, double* b) {
  if (!h || !f || !b) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    load_vector(*h, f, b);
  });
}

femgpu_status femgpu_set_dirichlet(femgpu_handle h, const uint8_t* mask) {
  if (!h || !mask) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_matrix, FEMGPU_ERR_NOT_READY, "no operator to constrain");
    invalidate_hierarchy(*h);
    apply_dirichlet(*h, mask);
  });
}

femgpu_status femgpu_set_matrix_csr(femgpu_handle h, int64_t n, const int32_t* rowptr, const int32_t* cols,
                                    const double* vals) {
  if (!h || !rowptr || n <= 0) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(n < INT32_MAX, FEMGPU_ERR_LIMIT, "matrix exceeds int32 indexing");
    int64_t nnz = rowptr[n];
    FG_REQUIRE(nnz >= 0 && (nnz == 0 || (cols && vals)), FEMGPU_ERR_INVALID, "bad CSR arrays");
    for (int64_t i = 0; i < n; i++) {
      FG_REQUIRE(rowptr[i] <= rowptr[i + 1], FEMGPU_ERR_INVALID, "row offsets not monotone");
      for (int64_t e = rowptr[i]; e < rowptr[i + 1]; e++) {
        FG_REQUIRE(cols[e] >= 0 && cols[e] < n, FEMGPU_ERR_INVALID, "column index out of range");
        FG_REQUIRE(e == rowptr[i] || cols[e] > cols[e - 1], FEMGPU_ERR_INVALID, "columns must be sorted and unique");
      }
    }
    invalidate_hierarchy(*h);
    h->assembled_from_mesh = false;
    cudaStream_t s = h->stream;
    DCsr<double>& A = h->A;
    A.n = A.m = (int)n;
    A.nnz = nnz;
    A.rp.alloc(n + 1, s);
    A.rp.upload(rowptr, n + 1);
    A.ci.alloc(nnz > 0 ? nnz : 1, s);
    A.ci.upload(cols, nnz);
    A.v.alloc(nnz > 0 ? nnz : 1, s);
    A.v.upload(vals, nnz);
    if (!(h->has_mesh && h->mesh.nv == n)) graph_from_matrix(*h);
    h->has_matrix = true;
    FG_CUDA(cudaStreamSynchronize(s));
  });
}

femgpu_status femgpu_setup(femgpu_handle h) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] { amg_setup(*h); }, "femgpu_setup");
}

femgpu_status femgpu_save_hierarchy(femgpu_handle h, const char* path) {
  if (!h || !path) return FEMGPU_ERR_INVALID;
  return guard(h, [&] { save_hierarchy(*h, path); }, "femgpu_save_hierarchy");
}

femgpu_status femgpu_load_hierarchy(femgpu_handle h, const char* path) {
  if (!h || !path) return FEMGPU_ERR_INVALID;
  return guard(h, [&] { load_hierarchy(*h, path); }, "femgpu_load_hierarchy");
}

femgpu_status femgpu_solve_device(femgpu_handle h, const double* d_b, double* d_x, femgpu_solve_stats* stats) {
  if (!h || !d_b || !d_x) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    if (!h->has_hierarchy) amg_setup(*h);
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    FG_CUDA(cudaEventRecord(e0, h->stream));
    SolveResult r = amg_solve_device(*h, d_b, d_x);
    FG_CUDA(cudaEventRecord(e1, h->stream));
    FG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
      stats->iterations = r.iterations;
      stats->relative_residual = r.relres;
      stats->setup_ms = h->setup_ms;
      stats->solve_ms = ms;
      stats->num_levels = h->H ? h->H->num_levels : 0;
    }
    result = r.status;
    if (r.status == FEMGPU_ERR_NOT_CONVERGED) h->last_error = "PCG reached maxIters";
    if (r.status == FEMGPU_ERR_BREAKDOWN) h->last_error = "PCG breakdown (non-positive curvature or NaN)";
  }, "femgpu_solve_device");
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_solve(femgpu_handle h, const double* b, double* x, femgpu_solve_stats* stats) {
  if (!h || !b || !x) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    FG_REQUIRE(h->has_matrix, FEMGPU_ERR_NOT_READY, "no operator");
    const int64_t n = h->A.n;
    DBuf<double> db(n, h->stream), dx(n, h->stream);
    db.upload(b, n);
    dx.upload(x, n);
    result = femgpu_solve_device(h, db.p, dx.p, stats);
    dx.download(x, n);
    FG_CUDA(cudaStreamSynchronize(h->stream));
  }, "femgpu_solve");
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_solve_multi_device(femgpu_handle h, int nrhs, const double* d_B, int64_t ldb, double* d_X,
                                       int64_t ldx, femgpu_solve_stats* stats) {
  if (!h || !d_B || !d_X || nrhs < 0) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    FG_REQUIRE(h->has_matrix, FEMGPU_ERR_NOT_READY, "no operator");
    const int64_t n = h->A.n;
    FG_REQUIRE(ldb >= n && ldx >= n, FEMGPU_ERR_INVALID, "leading dimension smaller than the rows");
    if (!h->has_hierarchy) amg_setup(*h);
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    FG_CUDA(cudaEventRecord(e0, h->stream));
    int iters = 0;
    double worst = 0.0;
    if (h->cfg.solverType == 1 && h->cfg.cycleType == 0 && h->cfg.smoother == 0) {
      // PCG with V-cycles: the columns eight at a time, each block in lockstep with SpMM kernels
      std::vector<int> it(nrhs);
      std::vector<double> rr(nrhs);
      std::vector<femgpu_status> stc(nrhs, FEMGPU_OK);
      block_solve_device(*h, nrhs, d_B, ldb, d_X, ldx, it.data(), rr.data(), stc.data());
      for (int j = 0; j < nrhs; j++) {
        iters += it[j];
        worst = std::max(worst, rr[j]);
        if (stc[j] != FEMGPU_OK && result == FEMGPU_OK) result = stc[j];
      }
    } else {
      for (int j = 0; j < nrhs; j++) {
        // one column at a time: one V-cycle per column (AMG_SOLVER), or PCG with W/F cycles
        SolveResult r = amg_solve_device(*h, d_B + j * ldb, d_X + j * ldx);
        iters += r.iterations;
        worst = std::max(worst, r.relres);
        if (r.status != FEMGPU_OK && result == FEMGPU_OK) result = r.status;
      }
    }
    FG_CUDA(cudaEventRecord(e1, h->stream));
    FG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
      stats->iterations = iters;
      stats->relative_residual = worst;
      stats->setup_ms = h->setup_ms;
      stats->solve_ms = ms;
      stats->num_levels = h->H ? h->H->num_levels : 0;
    }
    if (result == FEMGPU_ERR_NOT_CONVERGED) h->last_error = "PCG reached maxIters on a right-hand side";
    if (result == FEMGPU_ERR_BREAKDOWN) h->last_error = "PCG breakdown on a right-hand side";
  }, "femgpu_solve_multi_device");
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_solve_multi(femgpu_handle h, int nrhs, const double* B, double* X,
                                 femgpu_solve_stats* stats) {
  if (!h || !B || !X || nrhs < 0) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    FG_REQUIRE(h->has_matrix, FEMGPU_ERR_NOT_READY, "no operator");
    const int64_t n = h->A.n, total = n * (int64_t)nrhs;
    DBuf<double> db(total, h->stream), dx(total, h->stream);
    db.upload(B, total);
    dx.upload(X, total);
    result = femgpu_solve_multi_device(h, nrhs, db.p, n, dx.p, n, stats);
    dx.download(X, total);
    FG_CUDA(cudaStreamSynchronize(h->stream));
  });
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_solve_batch(int count, femgpu_handle* hs, const double* const* b, double* const* x, int setup,
                                 int threads, femgpu_solve_stats* stats) {
  if (count < 0 || threads < 0) return FEMGPU_ERR_INVALID;
  if (count == 0) return FEMGPU_OK;
  const TraceRange range("femgpu_solve_batch");
  if (!hs || !b || !x) return FEMGPU_ERR_INVALID;
  std::vector<femgpu_handle> seen(hs, hs + count);
  for (int i = 0; i < count; i++)
    if (!hs[i] || !b[i] || !x[i]) return FEMGPU_ERR_INVALID;
  std::sort(seen.begin(), seen.end());
  if (std::adjacent_find(seen.begin(), seen.end()) != seen.end()) return FEMGPU_ERR_INVALID;  // one thread per handle
  // concurrent threads must not share a stream (each captures its PCG loop on its own)
  std::vector<cudaStream_t> streams(count);
  for (int i = 0; i < count; i++) streams[i] = hs[i]->stream;
  std::sort(streams.begin(), streams.end());
  if (std::adjacent_find(streams.begin(), streams.end()) != streams.end()) return FEMGPU_ERR_INVALID;
  std::vector<femgpu_status> status(count, FEMGPU_OK);
  // jobs spread over host threads (each handle's size reads and flags overlap the others')
  auto run_threads = [&](const std::function<femgpu_status(int)>& job) {
    std::atomic<int> next{0};
    auto work = [&]() {
      for (int i = next.fetch_add(1); i < count; i = next.fetch_add(1))
        if (status[i] == FEMGPU_OK) status[i] = job(i);  // a handle whose setup failed is done
    };
    const int nt = threads == 0 ? count : std::min(threads, count);
    std::vector<std::thread> pool;
    try {
      for (int t = 1; t < nt; t++) pool.emplace_back(work);
    } catch (...) {
      // fewer threads than asked (the remaining work is shared by the ones running)
    }
    work();
    for (auto& t : pool) t.join();
    for (int i = 0; i < count; i++)
      if (status[i] != FEMGPU_OK) return status[i];
    return FEMGPU_OK;
  };
  bool graph = !getenv("FEMGPU_HOST_LOOP");
  if (setup) graph = run_threads([&](int i) { return femgpu_setup(hs[i]); }) == FEMGPU_OK && graph;
  // PCG solves of handles on one device: one graph launch with a branch per handle
  for (int i = 0; graph && i < count; i++)
    graph = hs[i]->cfg.solverType == 1 && hs[i]->cfg.maxIters > 0 && hs[i]->device == hs[0]->device &&
            hs[i]->has_hierarchy;
  if (graph) {
    for (int i = 0; i < count; i++) {
      femgpu_status st = guard(hs[i], [&] {
        Ctx& c = *hs[i];
        batch_prepare(c);
        c.bat_b.upload(b[i], c.A.n);
        c.bat_x.upload(x[i], c.A.n);
      });
      if (st != FEMGPU_OK) return st;
    }
    std::vector<Ctx*> list(hs, hs + count);
    std::vector<SolveResult> res;
    float ms = 0.0f;
    bool ran = false;
    femgpu_status st = guard(hs[0], [&] { ran = batch_solve_graph(list, res, &ms); });
    if (st != FEMGPU_OK) return st;
    if (ran) {
      femgpu_status result = FEMGPU_OK;
      for (int i = 0; i < count; i++) {
        Ctx& c = *hs[i];
        st = guard(hs[i], [&] {
          c.bat_x.download(x[i], c.A.n);
          FG_CUDA(cudaStreamSynchronize(c.stream));
        });
        if (st != FEMGPU_OK) return st;
        if (stats) {
          stats[i].iterations = res[i].iterations;
          stats[i].relative_residual = res[i].relres;
          stats[i].setup_ms = c.setup_ms;
          stats[i].solve_ms = ms;  // the whole batch graph (the branches run together)
          stats[i].num_levels = c.H ? c.H->num_levels : 0;
        }
        if (res[i].status == FEMGPU_ERR_NOT_CONVERGED) c.last_error = "PCG reached maxIters";
        if (res[i].status == FEMGPU_ERR_BREAKDOWN) c.last_error = "PCG breakdown (non-positive curvature or NaN)";
        if (res[i].status == FEMGPU_ERR_LIMIT) c.last_error = "smoother copy wait ran out";
        if (res[i].status != FEMGPU_OK && result == FEMGPU_OK) result = res[i].status;
      }
      return result;
    }
  }
  return run_threads([&](int i) { return femgpu_solve(hs[i], b[i], x[i], stats ? &stats[i] : nullptr); });
}

femgpu_status femgpu_adjoint_grad_device(femgpu_handle h, const double* d_dLdu, const double* d_u,
                                        double* d_grad, femgpu_solve_stats* stats) {
  if (!h || !d_dLdu || !d_u || !d_grad) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    FG_REQUIRE(h->has_mesh && h->has_matrix && h->assembled_from_mesh, FEMGPU_ERR_NOT_READY,
               "the adjoint gradient needs an operator assembled from the mesh (femgpu_assemble)");
    if (!h->has_hierarchy) amg_setup(*h);
    const int64_t n = h->A.n;
    cudaStream_t s = h->stream;
    DBuf<double> g(n, s), lam(n, s);
    zero_dirichlet_rows(*h, d_dLdu, g.p);  // u is fixed on Dirichlet rows
    lam.zero();
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    FG_CUDA(cudaEventRecord(e0, s));
    SolveResult r = amg_solve_device(*h, g.p, lam.p);  // A is symmetric: A^T lambda = dL/du
    element_log_coef_gradient(*h, lam.p, d_u, d_grad);
    FG_CUDA(cudaEventRecord(e1, s));
    FG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
      stats->iterations = r.iterations;
      stats->relative_residual = r.relres;
      stats->setup_ms = h->setup_ms;
      stats->solve_ms = ms;
      stats->num_levels = h->H ? h->H->num_levels : 0;
    }
    result = r.status;
    if (r.status == FEMGPU_ERR_NOT_CONVERGED) h->last_error = "adjoint PCG reached maxIters";
    if (r.status == FEMGPU_ERR_BREAKDOWN) h->last_error = "adjoint PCG breakdown (non-positive curvature or NaN)";
  }, "femgpu_adjoint_grad_device");
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_adjoint_grad(femgpu_handle h, const double* dLdu, const double* u, double* dLdtheta,
                                 femgpu_solve_stats* stats) {
  if (!h || !dLdu || !u || !dLdtheta) return FEMGPU_ERR_INVALID;
  femgpu_status result = FEMGPU_OK;
  femgpu_status st = guard(h, [&] {
    FG_REQUIRE(h->has_mesh, FEMGPU_ERR_NOT_READY, "femgpu_set_mesh first");
    const int64_t n = h->A.n, ne = h->mesh.ne;
    DBuf<double> dg(n, h->stream), du(n, h->stream), dt(ne, h->stream);
    dg.upload(dLdu, n);
    du.upload(u, n);
    result = femgpu_adjoint_grad_device(h, dg.p, du.p, dt.p, stats);
    dt.download(dLdtheta, ne);
    FG_CUDA(cudaStreamSynchronize(h->stream));
  });
  return st != FEMGPU_OK ? st : result;
}

femgpu_status femgpu_spmv_device(femgpu_handle h, const double* d_x, double* d_y) {
  if (!h || !d_x || !d_y) return FEMGPU_ERR_INVALID;
  return guard(h, [&] { spmv_original(*h, d_x, d_y); });
}

femgpu_status femgpu_get_matrix(femgpu_handle h, int64_t* n, int64_t* nnz, int32_t* rowptr, int32_t* cols,
                                double* vals) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_mesh || h->has_matrix, FEMGPU_ERR_NOT_READY, "no operator");
    if (n) *n = h->A.n;
    if (nnz) *nnz = h->A.nnz;
    if (rowptr) h->A.rp.download(rowptr, h->A.n + 1);
    if (cols) h->A.ci.download(cols, h->A.nnz);
    if (vals) h->A.v.download(vals, h->A.nnz);
    FG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

femgpu_status femgpu_num_levels(femgpu_handle h, int* levels) {
  if (!h || !levels) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
    *levels = h->H->num_levels;
  });
}

femgpu_status femgpu_get_level_info(femgpu_handle h, int level, femgpu_level_info* info) {
  if (!h || !info) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
    if (h->cfg.precision == 1) fill_level_info<double>(*h, level, info);
    else fill_level_info<float>(*h, level, info);
  });
}

femgpu_status femgpu_level_get(femgpu_handle h, int level, int32_t* A_rowptr, int32_t* A_cols, double* A_vals,
                               int32_t* perm, int32_t* agg_idx, int32_t* part_idx, int32_t* P_rowptr,
                               int32_t* P_cols, double* P_vals) {
  if (!h) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
    if (h->cfg.precision == 1)
      get_level<double>(*h, level, A_rowptr, A_cols, A_vals, perm, agg_idx, part_idx, P_rowptr, P_cols, P_vals);
    else
      get_level<float>(*h, level, A_rowptr, A_cols, A_vals, perm, agg_idx, part_idx, P_rowptr, P_cols, P_vals);
  });
}

femgpu_status femgpu_vcycle(femgpu_handle h, const double* r, double* z) {
  if (!h || !r || !z) return FEMGPU_ERR_INVALID;
  return guard(h, [&] {
    FG_REQUIRE(h->has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
    const int64_t n = h->A.n;
    DBuf<double> dr(n, h->stream), dz(n, h->stream);
    dr.upload(r, n);
    amg_vcycle_device(*h, dr.p, dz.p);
    dz.download(z, n);
    FG_CUDA(cudaStreamSynchronize(h->stream));
  }, "femgpu_vcycle");
}

femgpu_status femgpu_profile_kernel(femgpu_handle h, int which, int reps, double* avg_ms, double* bytes) {
  if (!h || !avg_ms || !bytes) return FEMGPU_ERR_INVALID;
  return guard(h, [&] { profile_kernel(*h, which, reps, avg_ms, bytes); });
}

femgpu_status femgpu_test_copy_wait_limit(femgpu_handle h, int polls) {
  if (!h) return FEMGPU_ERR_INVALID;
  h->copy_wait_limit = polls < 0 ? kMbarWaitLimit : polls;
  h->hier_gen++;  // the captured PCG loop holds the old limit: capture it again
  return FEMGPU_OK;
}

femgpu_status femgpu_kernel_launches(femgpu_handle h, int64_t* count) {
  (void)h;
  if (!count) return FEMGPU_ERR_INVALID;
  *count = g_kernel_launches.load();
  return FEMGPU_OK;
}

}  // extern "C"
