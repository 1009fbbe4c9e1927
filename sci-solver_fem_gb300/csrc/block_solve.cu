// block_solve.cu -- several right-hand sides with one hierarchy, solved together.
//
// The columns are taken in blocks of kBlock = 8.  Inside a block every column runs its
// own flexible PCG (CG_Flex_Cycle, cgcycle.cu:6-69, the method of the single-column
// solve) with its own step lengths, but the eight advance in lockstep and every operator
// application is a sparse matrix times an n x 8 block (SpMM): the FP64 outer operator,
// each level's in-partition and cross-partition entries, R and P are read once per block
// instead of once per column, and the coarsest solve X = A_c^{-1} B is a dense FP64
// product on the tensor cores (DMMA, mma.sync m8n8k4 f64).  A column that has converged
// keeps its x and r (its step length is zero) while the others go on.  Block vectors are
// row-major n x 8, so one gather of a column index fetches the row's eight values in one
// 32-byte (FP32) or 64-byte (FP64) access.
//
// The smoother is the partition-block weighted Jacobi of the single-column V-cycle
// (gauss_seidel.cu:1278-1376, 3626-3736) on the same groups of partitions, with row sums
// in entry order; the V-cycle is AMG_Level::cycle (amg_level.cu:22-71).
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "context.cuh"

namespace femgpu {

namespace {

constexpr int kBlock = 8;
constexpr int kBG = 608;   // fixed reduction grid (4 x 152 SMs) x kBT threads
constexpr int kBT = 256;
constexpr unsigned kAll = 0xffffffffu;

// per-column scalar slots: slot s of column j is sc[s * kBlock + j]
enum BSlot { B_BN = 0, B_NR, B_PY, B_ALPHA, B_RZ, B_RZNEW, B_ZROLD, B_BETA, B_ACTIVE, B_ITS, B_FLAG, B_NSLOT };
// block-wide slots after the per-column ones
enum BGlobal { G_FIRST = B_NSLOT * kBlock, G_IT, G_TOL, G_MAXIT, G_ANY, G_FLEX, G_COUNT };

template <class T>
struct V8 {
  T v[kBlock];
};

template <class T>
__device__ __forceinline__ V8<T> ld8(const T* p) {
  V8<T> r;
  if constexpr (sizeof(T) == 4) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
    r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const double2 a = reinterpret_cast<const double2*>(p)[q];
      r.v[2 * q] = a.x;
      r.v[2 * q + 1] = a.y;
    }
  }
  return r;
}

template <class T>
__device__ __forceinline__ void st8(T* p, const V8<T>& r) {
  if constexpr (sizeof(T) == 4) {
    reinterpret_cast<float4*>(p)[0] = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    reinterpret_cast<float4*>(p)[1] = make_float4(r.v[4], r.v[5], r.v[6], r.v[7]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++) reinterpret_cast<double2*>(p)[q] = make_double2(r.v[2 * q], r.v[2 * q + 1]);
  }
}

// ---- reductions: eight columns at once over the fixed grid -----------------------------
// Block sums of v[0..7] (blockDim kBT); valid in thread 0.
__device__ __forceinline__ void block_sum8(double v[kBlock], double (*sh)[kBlock]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kBlock; j++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(kAll, v[j], o);
    if (lane == 0) sh[w][j] = v[j];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < kBlock; j++) {
      double t = sh[0][j];
      for (int q = 1; q < kBT / 32; q++) t += sh[q][j];
      v[j] = t;
    }
  }
  __syncthreads();
}

// After every block wrote its partials: true in the block that finishes last.
__device__ __forceinline__ bool last_block(unsigned* counter) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Totals of partial[j * kBG + b] over b for each column j, in a fixed order (thread t adds
// b = t, t + kBT, ...; then the block sum); valid in thread 0.
__device__ __forceinline__ void column_totals(const double* partial, double tot[kBlock], double (*sh)[kBlock]) {
#pragma unroll
  for (int j = 0; j < kBlock; j++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < kBG; b += kBT) s += partial[j * kBG + b];
    tot[j] = s;
  }
  block_sum8(tot, sh);
}

// ---- FP64 outer kernels -------------------------------------------------------------
// out (n x 8, permuted order) from the caller's column-major B (column j at B + j * ldb)
__global__ void blk_in_kernel(int n, int kc, const int32_t* __restrict__ perm, const double* __restrict__ B,
                              int64_t ldb, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V8<double> r;
#pragma unroll
  for (int j = 0; j < kBlock; j++) r.v[j] = j < kc ? B[j * ldb + i] : 0.0;
  st8(out + (int64_t)perm[i] * kBlock, r);
}

__global__ void blk_out_kernel(int n, int kc, const int32_t* __restrict__ perm, const double* __restrict__ in,
                               double* __restrict__ X, int64_t ldx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V8<double> r = ld8(in + (int64_t)perm[i] * kBlock);
#pragma unroll
  for (int j = 0; j < kBlock; j++)
    if (j < kc) X[j * ldx + i] = r.v[j];
}

// sc[slot] = a.b per column (and sc[slot2] = a.c when c != nullptr).
__global__ void __launch_bounds__(kBT) blk_dot_kernel(int n, const double* __restrict__ a,
                                                       const double* __restrict__ b, const double* __restrict__ c,
                                                       double* partial, double* sc, int slot, int slot2,
                                                       unsigned* counter) {
  __shared__ double sh[kBT / 32][kBlock];
  double s1[kBlock] = {}, s2[kBlock] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V8<double> va = ld8(a + (int64_t)i * kBlock), vb = ld8(b + (int64_t)i * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) s1[j] = fma(va.v[j], vb.v[j], s1[j]);
    if (c) {
      const V8<double> vc = ld8(c + (int64_t)i * kBlock);
#pragma unroll
      for (int j = 0; j < kBlock; j++) s2[j] = fma(va.v[j], vc.v[j], s2[j]);
    }
  }
  block_sum8(s1, sh);
  if (threadIdx.x == 0)
    for (int j = 0; j < kBlock; j++) partial[j * kBG + blockIdx.x] = s1[j];
  if (c) {
    block_sum8(s2, sh);
    if (threadIdx.x == 0)
      for (int j = 0; j < kBlock; j++) partial[(kBlock + j) * kBG + blockIdx.x] = s2[j];
  }
  if (!last_block(counter)) return;
  double t[kBlock];
  column_totals(partial, t, sh);
  if (threadIdx.x == 0)
    for (int j = 0; j < kBlock; j++) sc[slot * kBlock + j] = t[j];
  if (c) {
    column_totals(partial + kBlock * kBG, t, sh);
    if (threadIdx.x == 0)
      for (int j = 0; j < kBlock; j++) sc[slot2 * kBlock + j] = t[j];
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// Row i of the outer FP64 operator times the block (sliced layout when off != nullptr:
// rows 32 s .. 32 s + 31 column-major from off[s], padding column -1; else CSR).
__device__ __forceinline__ V8<double> outer_row(int i, const int32_t* __restrict__ off, const int32_t* __restrict__ rp,
                                                const int32_t* __restrict__ ci, const double* __restrict__ v,
                                                const double* __restrict__ p) {
  V8<double> s;
#pragma unroll
  for (int j = 0; j < kBlock; j++) s.v[j] = 0.0;
  int e = off ? off[i >> 5] + (i & 31) : rp[i];
  const int end = off ? off[(i >> 5) + 1] : rp[i + 1];
  const int step = off ? 32 : 1;
  for (; e < end; e += step) {
    const int col = ci[e];
    if (col < 0) break;  // slice padding comes after a row's entries
    const double a = v[e];
    const V8<double> x = ld8(p + (int64_t)col * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) s.v[j] = fma(a, x.v[j], s.v[j]);
  }
  return s;
}

// y = A p, p.y per column; the last block forms alpha = rz / p.y for the active columns
// (a non-positive or non-finite p.y flags the column and stops it).
__global__ void __launch_bounds__(kBT) blk_spmv_dot_kernel(int n, const int32_t* __restrict__ off,
                                                            const int32_t* __restrict__ rp,
                                                            const int32_t* __restrict__ ci,
                                                            const double* __restrict__ v,
                                                            const double* __restrict__ p, double* __restrict__ y,
                                                            double* partial, double* sc, unsigned* counter) {
  __shared__ double sh[kBT / 32][kBlock];
  double acc[kBlock] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V8<double> s = outer_row(i, off, rp, ci, v, p);
    st8(y + (int64_t)i * kBlock, s);
    const V8<double> pi = ld8(p + (int64_t)i * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) acc[j] = fma(s.v[j], pi.v[j], acc[j]);
  }
  block_sum8(acc, sh);
  if (threadIdx.x == 0)
    for (int j = 0; j < kBlock; j++) partial[j * kBG + blockIdx.x] = acc[j];
  if (!last_block(counter)) return;
  double t[kBlock];
  column_totals(partial, t, sh);
  if (threadIdx.x == 0) {
    for (int j = 0; j < kBlock; j++) {
      double* s = sc;
      s[B_PY * kBlock + j] = t[j];
      double alpha = 0.0;
      if (s[B_ACTIVE * kBlock + j] != 0.0) {
        if (t[j] > 0.0 && isfinite(t[j])) {
          alpha = s[B_RZ * kBlock + j] / t[j];
        } else {
          s[B_FLAG * kBlock + j] = 1.0;
          s[B_ACTIVE * kBlock + j] = 0.0;
        }
      }
      s[B_ALPHA * kBlock + j] = alpha;
    }
    *counter = 0u;
  }
}

// y = A x (start of the solve).
__global__ void blk_spmv_kernel(int n, const int32_t* __restrict__ off, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ ci, const double* __restrict__ v,
                                const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) st8(y + (int64_t)i * kBlock, outer_row(i, off, rp, ci, v, x));
}

// r = b - y
__global__ void blk_sub_kernel(int n, const double* __restrict__ b, const double* __restrict__ y,
                               double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V8<double> vb = ld8(b + (int64_t)i * kBlock), vy = ld8(y + (int64_t)i * kBlock);
  V8<double> o;
#pragma unroll
  for (int j = 0; j < kBlock; j++) o.v[j] = vb.v[j] - vy.v[j];
  st8(r + (int64_t)i * kBlock, o);
}

// beta per column (cgcycle.cu:52-54; Polak-Ribiere when flexible), 0 on the first
// iteration and for stopped columns; rz = rz_new.
__global__ void blk_beta_kernel(double* sc) {
  const int j = threadIdx.x;
  if (j >= kBlock) return;
  const bool first = sc[G_FIRST] != 0.0, flex = sc[G_FLEX] != 0.0;
  const double rz = sc[B_RZ * kBlock + j], rzn = sc[B_RZNEW * kBlock + j];
  double beta = 0.0;
  if (!first && sc[B_ACTIVE * kBlock + j] != 0.0) beta = flex ? (rzn - sc[B_ZROLD * kBlock + j]) / rz : rzn / rz;
  sc[B_BETA * kBlock + j] = beta;
  sc[B_RZ * kBlock + j] = rzn;
  __syncwarp(0xffu);
  if (j == 0) sc[G_FIRST] = 0.0;
}

// p = z + beta p
__global__ void blk_pupdate_kernel(int n, const double* __restrict__ sc, const double* __restrict__ z,
                                   double* __restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V8<double> vz = ld8(z + (int64_t)i * kBlock), vp = ld8(p + (int64_t)i * kBlock);
  V8<double> o;
#pragma unroll
  for (int j = 0; j < kBlock; j++) o.v[j] = fma(sc[B_BETA * kBlock + j], vp.v[j], vz.v[j]);
  st8(p + (int64_t)i * kBlock, o);
}

// x += alpha p; r -= alpha y (rold = r first when flexible); r.r per column; the last
// block advances the iteration count and stops converged, broken or exhausted columns.
__global__ void __launch_bounds__(kBT) blk_update_kernel(int n, double* sc, const double* __restrict__ p,
                                                          const double* __restrict__ y, double* __restrict__ x,
                                                          double* __restrict__ r, double* __restrict__ rold,
                                                          double* partial, unsigned* counter) {
  __shared__ double sh[kBT / 32][kBlock];
  double alpha[kBlock], acc[kBlock] = {};
#pragma unroll
  for (int j = 0; j < kBlock; j++) alpha[j] = sc[B_ALPHA * kBlock + j];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int64_t o = (int64_t)i * kBlock;
    const V8<double> vr = ld8(r + o), vp = ld8(p + o), vx = ld8(x + o), vy = ld8(y + o);
    if (rold) st8(rold + o, vr);
    V8<double> nx, nr;
#pragma unroll
    for (int j = 0; j < kBlock; j++) {
      nx.v[j] = fma(alpha[j], vp.v[j], vx.v[j]);
      nr.v[j] = fma(-alpha[j], vy.v[j], vr.v[j]);
      acc[j] = fma(nr.v[j], nr.v[j], acc[j]);
    }
    st8(x + o, nx);
    st8(r + o, nr);
  }
  block_sum8(acc, sh);
  if (threadIdx.x == 0)
    for (int j = 0; j < kBlock; j++) partial[j * kBG + blockIdx.x] = acc[j];
  if (!last_block(counter)) return;
  double t[kBlock];
  column_totals(partial, t, sh);
  if (threadIdx.x == 0) {
    const double it = sc[G_IT] + 1.0;
    sc[G_IT] = it;
    double any = 0.0;
    for (int j = 0; j < kBlock; j++) {
      sc[B_NR * kBlock + j] = t[j];
      if (sc[B_ACTIVE * kBlock + j] == 0.0) continue;
      sc[B_ITS * kBlock + j] = it;
      const double bn = sqrt(sc[B_BN * kBlock + j]);
      const double nr = sqrt(t[j]);
      if (!isfinite(nr)) {
        sc[B_FLAG * kBlock + j] = 1.0;
        sc[B_ACTIVE * kBlock + j] = 0.0;
      } else if (nr / (bn > 0.0 ? bn : 1.0) <= sc[G_TOL]) {
        sc[B_ACTIVE * kBlock + j] = 0.0;
      } else {
        any = 1.0;
      }
    }
    sc[G_ANY] = (any != 0.0 && it < sc[G_MAXIT]) ? 1.0 : 0.0;
    *counter = 0u;
  }
}

// ---- V-cycle kernels (hierarchy precision T) ------------------------------------------------
template <class T>
__global__ void blk_cast_in_kernel(int64_t m, const double* __restrict__ in, T* __restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < m) out[q] = (T)in[q];
}

template <class T>
__global__ void blk_cast_out_kernel(int64_t m, const T* __restrict__ in, double* __restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < m) out[q] = (double)in[q];
}

template <class T>
__device__ __forceinline__ T relax1(T x, T b, T sax, T d, T dinv, T w) {
  T t = b - sax;
  t = t - d * x;
  return x + (w * t) * dinv;
}

// Partition-block weighted Jacobi on one group of consecutive partitions per CTA (rows
// [grows[g], grows[g + 1])), all eight columns at once: the group's x double-buffered in
// shared memory (m x 8), the right-hand side b (pre) or b - A_out x_in (post) staged
// beside it.  In-partition entries are used for all eight columns: with STAGED they are
// copied once (coalesced) into shared memory with group-local 16-bit columns, otherwise
// they are read from global memory (L2) in every sweep.  Pre (POST == false):
// x0 = w b / d, `inner` sweeps, then x and r = b - A_in x - d x.  Post: `inner` sweeps
// from x_in.
template <class T, bool POST, bool STAGED>
__global__ void __launch_bounds__(512) blk_smooth_kernel(
    const int32_t* __restrict__ grows, const int32_t* __restrict__ irp, const int32_t* __restrict__ ici,
    const T* __restrict__ iv, const int32_t* __restrict__ orp, const int32_t* __restrict__ oci,
    const T* __restrict__ ov, const T* __restrict__ diag, const T* __restrict__ dinv, const T* __restrict__ b, T w,
    int inner, const T* __restrict__ x_in, T* __restrict__ x_out, T* __restrict__ r_out, int mcap, int ecap) {
  extern __shared__ __align__(16) unsigned char sm[];
  T* xa = reinterpret_cast<T*>(sm);
  T* xb = xa + (int64_t)mcap * kBlock;
  T* sb = xb + (int64_t)mcap * kBlock;
  T* sv = sb + (int64_t)mcap * kBlock;
  uint16_t* sc16 = reinterpret_cast<uint16_t*>(sv + ecap);
  const int rs = grows[blockIdx.x], m = grows[blockIdx.x + 1] - rs;
  const int es = irp[rs];
  if (STAGED)
    for (int q = threadIdx.x; q < irp[rs + m] - es; q += blockDim.x) {
      sv[q] = iv[es + q];
      sc16[q] = (uint16_t)(ici[es + q] - rs);
    }
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int row = rs + t;
    V8<T> bb = ld8(b + (int64_t)row * kBlock), x0;
    if (POST) {
      x0 = ld8(x_in + (int64_t)row * kBlock);
      for (int e = orp[row]; e < orp[row + 1]; e++) {
        const T a = ov[e];
        const V8<T> xo = ld8(x_in + (int64_t)oci[e] * kBlock);
#pragma unroll
        for (int j = 0; j < kBlock; j++) bb.v[j] = bb.v[j] - a * xo.v[j];
      }
    } else {
      const T di = dinv[row];
#pragma unroll
      for (int j = 0; j < kBlock; j++) x0.v[j] = (w * bb.v[j]) * di;
    }
    st8(sb + (int64_t)t * kBlock, bb);
    st8(xa + (int64_t)t * kBlock, x0);
  }
  __syncthreads();
  auto row_sum = [&](const T* cur, int row) {
    V8<T> s;
#pragma unroll
    for (int j = 0; j < kBlock; j++) s.v[j] = (T)0;
    for (int e = irp[row]; e < irp[row + 1]; e++) {
      const T a = STAGED ? sv[e - es] : iv[e];
      const int col = STAGED ? (int)sc16[e - es] : ici[e] - rs;
      const V8<T> xv = ld8(cur + (int64_t)col * kBlock);
#pragma unroll
      for (int j = 0; j < kBlock; j++) s.v[j] = fma(a, xv.v[j], s.v[j]);
    }
    return s;
  };
  T* cur = xa;
  T* nxt = xb;
  for (int it = 0; it < inner; it++) {
    for (int t = threadIdx.x; t < m; t += blockDim.x) {
      const int row = rs + t;
      const V8<T> s = row_sum(cur, row), xc = ld8(cur + (int64_t)t * kBlock), bb = ld8(sb + (int64_t)t * kBlock);
      const T d = diag[row], di = dinv[row];
      V8<T> xn;
#pragma unroll
      for (int j = 0; j < kBlock; j++) xn.v[j] = relax1(xc.v[j], bb.v[j], s.v[j], d, di, w);
      st8(nxt + (int64_t)t * kBlock, xn);
    }
    __syncthreads();
    T* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int row = rs + t;
    const V8<T> xc = ld8(cur + (int64_t)t * kBlock);
    st8(x_out + (int64_t)row * kBlock, xc);
    if (!POST) {
      const V8<T> s = row_sum(cur, row), bb = ld8(sb + (int64_t)t * kBlock);
      const T d = diag[row];
      V8<T> r;
#pragma unroll
      for (int j = 0; j < kBlock; j++) r.v[j] = (bb.v[j] - s.v[j]) - d * xc.v[j];
      st8(r_out + (int64_t)row * kBlock, r);
    }
  }
}

// r -= A_out x (preAout_kernel, gauss_seidel.cu:1977-2015), eight columns.
template <class T>
__global__ void blk_aout_kernel(int n, const int32_t* __restrict__ orp, const int32_t* __restrict__ oci,
                                const T* __restrict__ ov, const T* __restrict__ x, T* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V8<T> s;
#pragma unroll
  for (int j = 0; j < kBlock; j++) s.v[j] = (T)0;
  for (int e = orp[i]; e < orp[i + 1]; e++) {
    const T a = ov[e];
    const V8<T> xv = ld8(x + (int64_t)oci[e] * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) s.v[j] = fma(a, xv.v[j], s.v[j]);
  }
  V8<T> ri = ld8(r + (int64_t)i * kBlock);
#pragma unroll
  for (int j = 0; j < kBlock; j++) ri.v[j] = ri.v[j] - s.v[j];
  st8(r + (int64_t)i * kBlock, ri);
}

// y = M x (accumulate = 0) or y += M x, eight columns (restriction, prolongation).
template <class T>
__global__ void blk_spmm_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const T* __restrict__ v, const T* __restrict__ x, T* __restrict__ y, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V8<T> s;
#pragma unroll
  for (int j = 0; j < kBlock; j++) s.v[j] = (T)0;
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    const T a = v[e];
    const V8<T> xv = ld8(x + (int64_t)ci[e] * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) s.v[j] = fma(a, xv.v[j], s.v[j]);
  }
  if (accumulate) {
    const V8<T> yi = ld8(y + (int64_t)i * kBlock);
#pragma unroll
    for (int j = 0; j < kBlock; j++) s.v[j] = yi.v[j] + s.v[j];
  }
  st8(y + (int64_t)i * kBlock, s);
}

// Coarsest level, X = Ainv B for the eight columns on the FP64 tensor cores: warp w forms
// rows 8w .. 8w + 7 of X with mma.sync m8n8k4 f64 steps over the inner dimension (A tile =
// 8 x 4 of the explicit inverse, row-major; B tile = 4 x 8 of the block).  Rows and inner
// indices past n are zero.
template <class T>
__global__ void blk_coarse_kernel(int n, const double* __restrict__ inv, const T* __restrict__ b,
                                  T* __restrict__ x) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int r0 = w * 8;
  if (r0 >= n) return;  // the whole warp
  double d0 = 0.0, d1 = 0.0;
  const int arow = r0 + (lane >> 2), acol = lane & 3;  // A fragment: (lane / 4, lane % 4)
  const int brow = lane & 3, bcol = lane >> 2;         // B fragment: (lane % 4, lane / 4)
  for (int k0 = 0; k0 < n; k0 += 4) {
    const double a = (arow < n && k0 + acol < n) ? inv[(int64_t)arow * n + k0 + acol] : 0.0;
    const double bv = (k0 + brow < n) ? (double)b[(int64_t)(k0 + brow) * kBlock + bcol] : 0.0;
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(bv));
  }
  const int crow = r0 + (lane >> 2), ccol = (lane & 3) * 2;  // D fragment: (lane / 4, 2 (lane % 4) + i)
  if (crow < n) {
    x[(int64_t)crow * kBlock + ccol] = (T)d0;
    x[(int64_t)crow * kBlock + ccol + 1] = (T)d1;
  }
}

// ---- per-handle state -----------------------------------------------------------------------
template <class T>
struct BlockLevel {
  DBuf<T> b, x, r, xo, t;
};

template <class T>
struct BlockState : BlockStateBase {
  uint64_t gen = ~0ull;
  std::vector<BlockLevel<T>> lv;
  DBuf<double> vb, vx, vr, vz, vp, vy, vrold, part, sc;
  DBuf<unsigned> cnt;
  double* h_sc = nullptr;
  // the block PCG loop captured as a CUDA graph (conditional while node), per flexible flag
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int64_t nodes[2] = {0, 0};
  ~BlockState() override {
    for (cudaGraphExec_t e : exec)
      if (e) cudaGraphExecDestroy(e);
    if (h_sc) cudaFreeHost(h_sc);
  }
};

// Continue the device-side block loop while a column is still running.
__global__ void blk_check_kernel(const double* sc, cudaGraphConditionalHandle loop) {
  cudaGraphSetConditional(loop, sc[G_ANY] != 0.0 ? 1u : 0u);
}

// Shared memory of blk_smooth_kernel: x twice and the right-hand side (m x 8 each), plus
// the staged entries (values and 16-bit columns) when `ecap` > 0.
template <class T>
size_t blk_smooth_smem(int mcap, int ecap = 0) {
  return (size_t)mcap * kBlock * sizeof(T) * 3 + (size_t)ecap * (sizeof(T) + 2);
}

// Entries are staged in shared memory when they fit beside the vectors.
constexpr size_t kBlockStageLimit = 200 * 1024;
template <class T>
bool blk_staged(const Level<T>& L) {
  return L.max_group_rows < 65536 && blk_smooth_smem<T>(L.max_group_rows, L.max_group_ents) <= kBlockStageLimit;
}

template <class T, bool POST>
void launch_blk_smooth(cudaStream_t s, const Level<T>& L, const T* b, T w, int inner, const T* x_in, T* x_out,
                       T* r_out) {
  const int thr = std::min(512, std::max(32, (L.max_group_rows + 31) / 32 * 32));
  if (blk_staged(L)) {
    const size_t smem = blk_smooth_smem<T>(L.max_group_rows, L.max_group_ents);
    ensure_smem(blk_smooth_kernel<T, POST, true>, smem);
    FG_LAUNCH((blk_smooth_kernel<T, POST, true>), L.ngroups, thr, smem, s, L.grows.p, L.Ain.rp.p, L.Ain.ci.p,
              L.Ain.v.p, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, L.diag.p, L.dinv.p, b, w, inner, x_in, x_out, r_out,
              L.max_group_rows, L.max_group_ents);
  } else {
    const size_t smem = blk_smooth_smem<T>(L.max_group_rows);
    ensure_smem(blk_smooth_kernel<T, POST, false>, smem);
    FG_LAUNCH((blk_smooth_kernel<T, POST, false>), L.ngroups, thr, smem, s, L.grows.p, L.Ain.rp.p, L.Ain.ci.p,
              L.Ain.v.p, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, L.diag.p, L.dinv.p, b, w, inner, x_in, x_out, r_out,
              L.max_group_rows, 0);
  }
}

template <class T>
void block_vcycle(Ctx& c, Hierarchy<T>& H, BlockState<T>& S, int l, T* b_in, T* x_out) {
  cudaStream_t s = c.stream;
  Level<T>& L = *H.L[l];
  const int n = L.A.n;
  if (L.coarsest) {
    FG_LAUNCH(blk_coarse_kernel<T>, grid_for((int64_t)((n + 7) / 8) * 32, 128), 128, 0, s, n, L.Ainv.p, b_in, x_out);
    return;
  }
  BlockLevel<T>& W = S.lv[l];
  const T w = (T)c.cfg.smootherWeight;
  // pre relax: x, r = b - A_in x - d x, then r -= A_out x
  launch_blk_smooth<T, false>(s, L, b_in, w, c.cfg.preInnerIters, (const T*)nullptr, W.x.p, W.r.p);
  FG_LAUNCH(blk_aout_kernel<T>, grid_for(n, 128), 128, 0, s, n, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, W.x.p, W.r.p);
  BlockLevel<T>& NW = S.lv[l + 1];
  FG_LAUNCH(blk_spmm_kernel<T>, grid_for(L.R.n, 128), 128, 0, s, L.R.n, L.R.rp.p, L.R.ci.p, L.R.v.p, W.r.p, NW.t.p,
            0);
  block_vcycle(c, H, S, l + 1, NW.t.p, NW.xo.p);
  FG_LAUNCH(blk_spmm_kernel<T>, grid_for(n, 128), 128, 0, s, n, L.P.rp.p, L.P.ci.p, L.P.v.p, NW.xo.p, W.x.p, 1);
  T* src = W.x.p;
  for (int rl = 0; rl < c.cfg.postRelaxes; rl++) {
    T* dst = (rl + 1 == c.cfg.postRelaxes) ? x_out : (src == W.x.p ? W.r.p : W.x.p);
    launch_blk_smooth<T, true>(s, L, b_in, w, c.cfg.postInnerIters, src, dst, (T*)nullptr);
    src = dst;
  }
  if (c.cfg.postRelaxes == 0)
    FG_CUDA(cudaMemcpyAsync(x_out, W.x.p, (size_t)n * kBlock * sizeof(T), cudaMemcpyDeviceToDevice, s));
}

template <class T>
BlockState<T>& block_state(Ctx& c, Hierarchy<T>& H) {
  BlockState<T>* S = dynamic_cast<BlockState<T>*>(c.block.get());
  if (!S || S->gen != c.hier_gen) {
    auto fresh = std::make_unique<BlockState<T>>();
    S = fresh.get();
    c.block = std::move(fresh);
    cudaStream_t s = c.stream;
    const int64_t n = c.A.n;
    for (int l = 0; l < H.num_levels; l++) {
      const Level<T>& L = *H.L[l];
      BlockLevel<T> W;
      const int64_t m = (int64_t)L.A.n * kBlock;
      W.b.alloc(m, s);
      W.x.alloc(m, s);
      W.xo.alloc(m, s);
      W.t.alloc(m, s);
      if (!L.coarsest) {
        W.r.alloc(m, s);
        const size_t smem = blk_smooth_smem<T>(L.max_group_rows);
        FG_REQUIRE(smem <= 227 * 1024, FEMGPU_ERR_LIMIT,
                   "a smoother group is too large for the multi-right-hand-side smoother's shared memory");
      }
      S->lv.push_back(std::move(W));
    }
    for (DBuf<double>* v : {&S->vb, &S->vx, &S->vr, &S->vz, &S->vp, &S->vy, &S->vrold}) v->alloc(n * kBlock, s);
    S->part.alloc((size_t)2 * kBlock * kBG, s);
    S->sc.alloc(G_COUNT, s);
    S->cnt.alloc(4, s);
    S->cnt.zero();
    FG_CUDA(cudaMallocHost((void**)&S->h_sc, G_COUNT * sizeof(double)));
    S->gen = c.hier_gen;
  }
  return *S;
}

// z = M r for the block (permuted level-0 FP64 vectors).
template <class T>
void block_precondition(Ctx& c, Hierarchy<T>& H, BlockState<T>& S, const double* r, double* z) {
  cudaStream_t s = c.stream;
  const int64_t m = (int64_t)H.L[0]->A.n * kBlock;
  BlockLevel<T>& W = S.lv[0];
  if constexpr (std::is_same<T, double>::value) {
    block_vcycle(c, H, S, 0, const_cast<double*>(r), z);  // the V-cycle only reads its input
  } else {
    FG_LAUNCH(blk_cast_in_kernel<T>, grid_for(m, 256), 256, 0, s, m, r, W.b.p);
    block_vcycle(c, H, S, 0, W.b.p, W.xo.p);
    FG_LAUNCH(blk_cast_out_kernel<T>, grid_for(m, 256), 256, 0, s, m, W.xo.p, z);
  }
}

template <class T>
void block_solve_columns(Ctx& c, Hierarchy<T>& H, int kc, const double* B, int64_t ldb, double* X, int64_t ldx,
                         int* iters, double* relres, femgpu_status* status) {
  cudaStream_t s = c.stream;
  BlockState<T>& S = block_state(c, H);
  const int n = c.A.n;
  const int32_t* off = c.sliced ? c.s_off.p : nullptr;
  const int32_t* rp = c.sliced ? nullptr : c.A0p.rp.p;
  const int32_t* ci = c.sliced ? c.s_ci.p : c.A0p.ci.p;
  const double* v = c.sliced ? c.s_v.p : c.A0p.v.p;
  double* sc = S.sc.p;
  double* part = S.part.p;
  const int flexible = c.cfg.flexibleCG;
  FG_LAUNCH(blk_in_kernel, grid_for(n, 256), 256, 0, s, n, kc, c.perm0.p, B, ldb, S.vb.p);
  FG_LAUNCH(blk_in_kernel, grid_for(n, 256), 256, 0, s, n, kc, c.perm0.p, X, ldx, S.vx.p);
  // scalars: b.b, r = b - A x, r.r, active columns
  FG_CUDA(cudaMemsetAsync(sc, 0, G_COUNT * sizeof(double), s));
  FG_CUDA(cudaMemsetAsync(S.cnt.p, 0, S.cnt.n * sizeof(unsigned), s));
  FG_CUDA(cudaMemsetAsync(S.vp.p, 0, S.vp.n * sizeof(double), s));
  FG_LAUNCH(blk_dot_kernel, kBG, kBT, 0, s, n, S.vb.p, S.vb.p, (const double*)nullptr, part, sc, (int)B_BN, 0,
            S.cnt.p);
  FG_LAUNCH(blk_spmv_kernel, grid_for(n, 128), 128, 0, s, n, off, rp, ci, v, S.vx.p, S.vy.p);
  FG_LAUNCH(blk_sub_kernel, grid_for(n, 256), 256, 0, s, n, S.vb.p, S.vy.p, S.vr.p);
  FG_LAUNCH(blk_dot_kernel, kBG, kBT, 0, s, n, S.vr.p, S.vr.p, (const double*)nullptr, part, sc, (int)B_NR, 0,
            S.cnt.p);
  FG_CUDA(cudaMemcpyAsync(S.h_sc, sc, G_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  double* h = S.h_sc;
  const double tol = c.cfg.tolerance;
  bool any = false;
  for (int j = 0; j < kBlock; j++) {
    const double bn = sqrt(h[B_BN * kBlock + j]);
    const bool act = j < kc && !(sqrt(h[B_NR * kBlock + j]) / (bn > 0.0 ? bn : 1.0) <= tol);
    h[B_ACTIVE * kBlock + j] = act ? 1.0 : 0.0;
    any = any || act;
  }
  h[G_FIRST] = 1.0;
  h[G_IT] = 0.0;
  h[G_TOL] = tol;
  h[G_MAXIT] = (double)c.cfg.maxIters;
  h[G_FLEX] = flexible ? 1.0 : 0.0;
  h[G_ANY] = (any && c.cfg.maxIters > 0) ? 1.0 : 0.0;
  FG_CUDA(cudaMemcpyAsync(sc, h, G_COUNT * sizeof(double), cudaMemcpyHostToDevice, s));
  // one block PCG iteration (the last kernel decides whether another one runs)
  auto iteration = [&]() {
    block_precondition(c, H, S, S.vr.p, S.vz.p);
    FG_LAUNCH(blk_dot_kernel, kBG, kBT, 0, s, n, S.vz.p, S.vr.p, flexible ? (const double*)S.vrold.p : nullptr, part,
              sc, (int)B_RZNEW, (int)B_ZROLD, S.cnt.p);
    FG_LAUNCH(blk_beta_kernel, 1, kBlock, 0, s, sc);
    FG_LAUNCH(blk_pupdate_kernel, grid_for(n, 256), 256, 0, s, n, sc, S.vz.p, S.vp.p);
    FG_LAUNCH(blk_spmv_dot_kernel, kBG, kBT, 0, s, n, off, rp, ci, v, S.vp.p, S.vy.p, part, sc, S.cnt.p + 1);
    FG_LAUNCH(blk_update_kernel, kBG, kBT, 0, s, n, sc, S.vp.p, S.vy.p, S.vx.p, S.vr.p,
              flexible ? S.vrold.p : nullptr, part, S.cnt.p + 2);
  };
  if (h[G_ANY] != 0.0) {
    // the iterations run on the device as a CUDA graph with a conditional while node,
    // captured once per hierarchy (FEMGPU_HOST_LOOP: launched one by one from the host)
    cudaGraphExec_t& exec = S.exec[flexible ? 1 : 0];
    if (!exec && !getenv("FEMGPU_HOST_LOOP")) {
      const int64_t before = g_kernel_launches.load();
      cudaGraph_t g = nullptr;
      bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
      cudaGraphConditionalHandle loop;
      cudaGraphNodeParams cp = {};
      if (ok) ok = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
      if (ok) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = loop;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
      }
      if (ok)
        ok = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        try {
          iteration();
          FG_LAUNCH(blk_check_kernel, 1, 1, 0, s, sc, loop);
        } catch (...) {
          ok = false;
        }
        cudaGraph_t captured = nullptr;
        ok = cudaStreamEndCapture(s, &captured) == cudaSuccess && ok;
      }
      if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
      if (!ok) {
        (void)cudaGetLastError();
        exec = nullptr;
      }
      if (g) cudaGraphDestroy(g);
      S.nodes[flexible ? 1 : 0] = g_kernel_launches.load() - before;
      g_kernel_launches.store(before);  // counted per iteration after each run
    }
    if (exec) {
      FG_CUDA(cudaGraphLaunch(exec, s));
      FG_CUDA(cudaMemcpyAsync(h, sc, G_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaStreamSynchronize(s));
      g_kernel_launches.fetch_add(S.nodes[flexible ? 1 : 0] * (int64_t)h[G_IT]);
    } else {
      while (h[G_ANY] != 0.0) {
        iteration();
        FG_CUDA(cudaMemcpyAsync(h, sc, G_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaStreamSynchronize(s));
      }
    }
  }
  FG_LAUNCH(blk_out_kernel, grid_for(n, 256), 256, 0, s, n, kc, c.perm0.p, S.vx.p, X, ldx);
  for (int j = 0; j < kc; j++) {
    const double bn = sqrt(h[B_BN * kBlock + j]);
    const double rr = sqrt(h[B_NR * kBlock + j]) / (bn > 0.0 ? bn : 1.0);
    iters[j] = (int)h[B_ITS * kBlock + j];
    relres[j] = rr;
    status[j] = (h[B_FLAG * kBlock + j] != 0.0 || !std::isfinite(rr)) ? FEMGPU_ERR_BREAKDOWN
                : rr <= tol                                              ? FEMGPU_OK
                                                                         : FEMGPU_ERR_NOT_CONVERGED;
  }
}

}  // namespace

void block_solve_device(Ctx& c, int nrhs, const double* d_B, int64_t ldb, double* d_X, int64_t ldx, int* iters,
                        double* relres, femgpu_status* status) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  for (int j0 = 0; j0 < nrhs; j0 += kBlock) {
    const int kc = std::min(kBlock, nrhs - j0);
    if (c.cfg.precision == 1)
      block_solve_columns(c, static_cast<Hierarchy<double>&>(*c.H), kc, d_B + j0 * ldb, ldb, d_X + j0 * ldx, ldx,
                          iters + j0, relres + j0, status + j0);
    else
      block_solve_columns(c, static_cast<Hierarchy<float>&>(*c.H), kc, d_B + j0 * ldb, ldb, d_X + j0 * ldx, ldx,
                          iters + j0, relres + j0, status + j0);
  }
}

}  // namespace femgpu
