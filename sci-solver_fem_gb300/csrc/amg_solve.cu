// amg_solve.cu -- V-cycle and FP64 outer PCG on the device.
//
// Smoother (gauss_seidel.cu, dsType 0 "symmetric" path): partition-block Jacobi.
// Consecutive partitions are packed into groups; a group's x lives in shared memory,
// either of one persistent CTA with the entries in registers and the next group's
// entries staged by bulk copies (level 0), or of a thread-block cluster whose CTAs
// broadcast new values through distributed shared memory (coarse levels).  The inner
// weighted-Jacobi sweeps run over in-partition couplings; cross-partition couplings
// enter once per relax (pre: preRRSym_kernel + preAout_kernel, gauss_seidel.cu:1278-2015;
// post: postRelaxSym_kernel, :3626-3736).  In-partition row sums run in a fixed lane
// order with fused multiply-adds (the reference accumulates in shared-memory atomics in
// arbitrary order).  Every non-coarsest level works in its own permuted order.
//
// PCG (CG_Flex_Cycle, cgcycle.cu:6-69) runs in FP64 on the level-0 permuted
// numbering: b is permuted on entry and x back on exit, so the solved system is
// A x = b (the reference applies the permuted operator to unpermuted vectors).  The
// whole loop is one CUDA graph with a device-side conditional.  Reductions are
// two-stage with a fixed grid, so results are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <deque>
#include <map>
#include <mutex>
#include <string>

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#include "context.cuh"

namespace femgpu {

// Programmatic dependent launch of the solve kernels (on unless FEMGPU_NO_PDL is set, a
// diagnostic switch for timing the same kernels with plain stream ordering).
bool g_pdl_enabled = getenv("FEMGPU_NO_PDL") == nullptr;
thread_local bool t_pdl_scope = false;

namespace {

constexpr int kRedBlocks = 608;  // 4 x 152 SMs: fixed grid for deterministic reductions
constexpr int kRedThreads = 256;

// device scalar slots in Ctx::red (after the partials)
enum Slot {
  S_BN = 0, S_NR, S_YP, S_ALPHA, S_RZ, S_RZNEW, S_ZROLD, S_BETA, S_FLAG, S_FIRST, S_KERR,
  S_IT, S_BNORM, S_TOL, S_MAXIT, S_COUNT
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// ---- level kernels -----------------------------------------------------------------
template <class T>
__global__ void cast_in_kernel(int n, const double* in, T* out) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)in[i];
}

template <class T>
__global__ void cast_out_kernel(int n, const T* in, double* out) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

// Weighted Jacobi update x += w (b - sAx - d x) / d (gauss_seidel.cu:1333-1341) in the
// hierarchy's precision, dividing by d as a multiplication with the precomputed 1/d.
// The reference forms the correction in double because its weight is a double;
// on GB300 that FP64 division per row and sweep dominated the smoother, so the
// update is done in T (the CPU oracle uses the same expression).
template <class T>
__device__ __forceinline__ T relax(T x, T b, T sax, T d, T dinv, T w) {
  T t = b - sax;
  t = t - d * x;
  return x + (w * t) * dinv;
}

// Shared-memory layout of one CTA of the cluster smoother: the whole group's x
// (double-buffered), then for the CTA's own row slice the right-hand side, the
// diagonal and its reciprocal, local row offsets and (when they fit) the slice's
// in-partition entries with 16-bit column indices local to the group.
template <class T>
struct SliceSmem {
  T *xa, *xb, *sb, *sd, *sdi, *sval;
  int32_t* srp;
  uint16_t* scol;
};

template <class T>
__device__ __forceinline__ SliceSmem<T> carve(unsigned char* sm, int mcap, int scap, int ecap) {
  SliceSmem<T> L;
  L.xa = reinterpret_cast<T*>(sm);
  L.xb = L.xa + mcap;
  L.sb = L.xb + mcap;
  L.sd = L.sb + scap;
  L.sdi = L.sd + scap;
  L.sval = L.sdi + scap;
  L.srp = reinterpret_cast<int32_t*>(L.sval + ecap);
  L.scol = reinterpret_cast<uint16_t*>(L.srp + scap + 1);
  return L;
}

template <class T>
size_t slice_smem_bytes(int mcap, int scap, int ecap) {
  return (size_t)mcap * 2 * sizeof(T) + (size_t)scap * 3 * sizeof(T) + (size_t)ecap * sizeof(T) +
         (size_t)(scap + 1) * 4 + (size_t)ecap * 2 + 16;
}

// Sum over slice row t's in-partition entries with S lanes per row: lane j adds
// entries j, j+S, ... in order with fused multiply-adds (the reference adds them with
// shared-memory atomics in any order), then an xor butterfly combines the lanes.  Every lane of the warp must call it (the butterfly shuffles the warp).
template <class T, bool STAGED, int S>
__device__ __forceinline__ T slice_row_sum(const SliceSmem<T>& P, const T* x, int t, bool live, int j,
                                           const int32_t* __restrict__ ici, const T* __restrict__ iv, int es,
                                           int rs) {
  T s = 0;
  if (live) {
    const int q0 = P.srp[t], q1 = P.srp[t + 1];
    for (int q = q0 + j; q < q1; q += S) {
      if (STAGED) s = fma(P.sval[q], x[P.scol[q]], s);
      else s = fma(iv[es + q], x[ici[es + q] - rs], s);
    }
  }
#pragma unroll
  for (int off = S >> 1; off > 0; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off, S);
  return s;
}

// Partition-block Jacobi smoother on thread-block clusters.  A cluster of C CTAs
// runs one group of consecutive partitions (rows [grows[g], grows[g+1])): in-partition
// entries never leave their partition, so a group is smoothed exactly like each of
// its partitions alone.  CTA c of the cluster owns a slice of ceil(m / C) rows; every
// CTA keeps the whole group's x, and after each sweep a row's new value is stored
// into all C copies through distributed shared memory, then one cluster barrier
// ends the sweep (x is double-buffered).
// POST == false (preRRSym_kernel + the in-partition part of the residual,
//   gauss_seidel.cu:1278-1376): x0 = w b / d, `inner` sweeps, then x and
//   r = b - A_in x - d x are written;
// POST == true (postRelaxSym_kernel, gauss_seidel.cu:3626-3736): b' = b - A_out x_in
//   (precomputed by aout_rhs_kernel when orp == nullptr), `inner` sweeps from x_in,
//   result written to x_out.
template <class T, bool POST, bool STAGED, int S>
__global__ void __launch_bounds__(1024) smooth_cluster_kernel(
    const int32_t* __restrict__ grows, const int32_t* __restrict__ irp,
    const int32_t* __restrict__ ici, const T* __restrict__ iv, const int32_t* __restrict__ orp,
    const int32_t* __restrict__ oci, const T* __restrict__ ov, const T* __restrict__ diag,
    const T* __restrict__ dinv, const T* __restrict__ b, T w, int inner, const T* __restrict__ x_in,
    T* __restrict__ x_out, T* __restrict__ r_out, int mcap, int scap, int ecap) {
  pdl_enter();
  extern __shared__ __align__(128) unsigned char sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int c = (int)cl.block_rank();
  const int g = blockIdx.x / C;
  const int rs = grows[g], m = grows[g + 1] - rs;
  const int qs = (m + C - 1) / C;
  const int ss = min(m, c * qs), ns = min(m, ss + qs) - ss;  // own slice: group rows [ss, ss + ns)
  const int es = irp[rs + ss], ne = irp[rs + ss + ns] - es;
  SliceSmem<T> P = carve<T>(sm, mcap, scap, STAGED ? ecap : 0);
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    const int row = rs + t;
    P.xa[t] = POST ? x_in[row] : (w * b[row]) * dinv[row];
  }
  for (int t = threadIdx.x; t < ns; t += blockDim.x) {
    const int row = rs + ss + t;
    P.sd[t] = diag[row];
    P.sdi[t] = dinv[row];
    P.srp[t] = irp[row] - es;
    T acc = b[row];
    if (POST && orp)
      for (int e = orp[row]; e < orp[row + 1]; e++) acc = acc + (-ov[e]) * x_in[oci[e]];
    P.sb[t] = acc;
  }
  if (threadIdx.x == 0) P.srp[ns] = ne;
  if (STAGED)
    for (int q = threadIdx.x; q < ne; q += blockDim.x) {
      P.sval[q] = iv[es + q];
      P.scol[q] = (uint16_t)(ici[es + q] - rs);
    }
  cl.sync();  // every CTA of the cluster is running and holds x0
  const int j = threadIdx.x & (S - 1), per = blockDim.x / S;
  T* cur = P.xa;
  T* nxt = P.xb;
  for (int it = 0; it < inner; it++) {
    for (int base = 0; base < ns; base += per) {
      const int t = base + threadIdx.x / S;
      const bool live = t < ns;
      const T v = slice_row_sum<T, STAGED, S>(P, cur, t, live, j, ici, iv, es, rs);
      if (j == 0 && live) {
        const T xn = relax(cur[ss + t], P.sb[t], v, P.sd[t], P.sdi[t], w);
        for (int r = 0; r < C; r++) *cl.map_shared_rank(nxt + ss + t, r) = xn;
      }
    }
    cl.sync();  // all copies of the new x written; the old buffer is no longer read
    T* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (!POST) {
    for (int base = 0; base < ns; base += per) {
      const int t = base + threadIdx.x / S;
      const bool live = t < ns;
      const T v = slice_row_sum<T, STAGED, S>(P, cur, t, live, j, ici, iv, es, rs);
      if (j == 0 && live) {
        const T xv = cur[ss + t];
        x_out[rs + ss + t] = xv;
        T u = P.sb[t] - v;
        r_out[rs + ss + t] = u - P.sd[t] * xv;
      }
    }
  } else {
    for (int t = threadIdx.x; t < ns; t += blockDim.x) x_out[rs + ss + t] = cur[ss + t];
  }
}

// Cluster smoother with register-resident entries (groups split over a cluster as in
// smooth_cluster_kernel): thread (t, j) of a CTA owns lane j of slice row t and keeps
// that lane's entries j, j + S, ... (at most K, padded with zero values pointing at
// the zero slot mcap of x) in registers across the sweeps, so a sweep is K
// shared-memory loads and fused multiply-adds per lane, an xor butterfly, and the
// broadcast of the row's new x to every CTA of the cluster.  Same order as
// slice_row_sum.
template <class T, bool POST, int S, int K>
__global__ void __launch_bounds__(1024) smooth_creg_kernel(
    const int32_t* __restrict__ grows, const int32_t* __restrict__ irp, const int32_t* __restrict__ ici,
    const T* __restrict__ iv, const T* __restrict__ diag, const T* __restrict__ dinv, const T* __restrict__ b, T w,
    int inner, const T* __restrict__ x_in, T* __restrict__ x_out, T* __restrict__ r_out, int mcap) {
  extern __shared__ __align__(128) unsigned char sm[];
  T* const xa = reinterpret_cast<T*>(sm);
  T* const xb = xa + (mcap + 1);
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int c = (int)cl.block_rank();
  const int g = blockIdx.x / C;
  const int rs = grows[g], m = grows[g + 1] - rs;
  const int qs = (m + C - 1) / C;
  const int ss = min(m, c * qs), ns = min(m, ss + qs) - ss;  // own slice: group rows [ss, ss + ns)
  if (threadIdx.x == 0) {
    xa[mcap] = (T)0;
    xb[mcap] = (T)0;
  }
  const int t = threadIdx.x / S, j = threadIdx.x & (S - 1);
  const bool live = t < ns;
  const int row = rs + ss + t;
  // the operator's entries, diagonal and row bounds are constant: loaded before waiting
  // for the kernels that write b and x_in
  int e0 = 0, len = 0;
  T d = (T)1, di = (T)1, bb = (T)0, x = (T)0;
  if (live) {
    e0 = irp[row];
    len = irp[row + 1] - e0;
    d = diag[row];
    di = dinv[row];
  }
  T val[K];
  uint32_t offp[K / 2];  // two 16-bit local columns per register
#pragma unroll
  for (int k = 0; k < K; k += 2) {
    const int q0 = j + S * k, q1 = q0 + S;
    const bool a0 = live && q0 < len, a1 = live && q1 < len;
    val[k] = a0 ? iv[e0 + q0] : (T)0;
    val[k + 1] = a1 ? iv[e0 + q1] : (T)0;
    const uint32_t o0 = a0 ? (uint32_t)(ici[e0 + q0] - rs) : (uint32_t)mcap;
    const uint32_t o1 = a1 ? (uint32_t)(ici[e0 + q1] - rs) : (uint32_t)mcap;
    offp[k >> 1] = o0 | (o1 << 16);
  }
  pdl_enter();
  for (int tt = threadIdx.x; tt < m; tt += blockDim.x) {
    const int r = rs + tt;
    xa[tt] = POST ? x_in[r] : (w * b[r]) * dinv[r];
  }
  if (live) {
    bb = b[row];
    x = POST ? x_in[row] : (w * bb) * di;
  }
  cl.sync();  // every CTA of the cluster is running and holds x0
  const T* cur = xa;
  T* nxt = xb;
  for (int it = 0; it < inner; it++) {
    T sv = 0;
#pragma unroll
    for (int k = 0; k < K; k++) sv = fma(val[k], cur[(offp[k >> 1] >> ((k & 1) * 16)) & 0xffffu], sv);
#pragma unroll
    for (int off = S >> 1; off > 0; off >>= 1) sv = sv + __shfl_xor_sync(0xffffffffu, sv, off, S);
    if (live && j == 0) {
      x = relax(x, bb, sv, d, di, w);
      for (int r = 0; r < C; r++) *cl.map_shared_rank(nxt + ss + t, r) = x;
    }
    cl.sync();  // all copies of the new x written; the old buffer is no longer read
    T* tmp = const_cast<T*>(cur);
    cur = nxt;
    nxt = tmp;
  }
  if (!POST) {
    T sv = 0;
#pragma unroll
    for (int k = 0; k < K; k++) sv = fma(val[k], cur[(offp[k >> 1] >> ((k & 1) * 16)) & 0xffffu], sv);
#pragma unroll
    for (int off = S >> 1; off > 0; off >>= 1) sv = sv + __shfl_xor_sync(0xffffffffu, sv, off, S);
    if (live && j == 0) {
      x_out[row] = x;
      T u = bb - sv;
      r_out[row] = u - d * x;
    }
  } else if (live && j == 0) {
    x_out[row] = x;
  }
}

// PCG reduction helpers (defined with the PCG kernels below).
__device__ double ordered_total(const double* partial, int nparts, double* sh);
__device__ bool last_block_done(unsigned* counter);
__device__ void beta_update(double* sc, int flexible);

// Row sum s +/- v[q] x[ci[q]] over q = e, e + stride, ... < end, added in that order
// with separately rounded products; the first K entries' columns, values and x are
// all loaded before the first add, so a short row costs three dependent loads.
template <class T, int K, bool SUB>
__device__ __forceinline__ T gather_row(const int32_t* __restrict__ ci, const T* __restrict__ v,
                                        const T* __restrict__ x, int e, int end, int stride, T s) {
  int c[K];
  T a[K], xv[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int q = e + k * stride;
    c[k] = q < end ? ci[q] : 0;
    a[k] = q < end ? v[q] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < K; k++) xv[k] = e + k * stride < end ? x[c[k]] : (T)0;
#pragma unroll
  for (int k = 0; k < K; k++)
    if (e + k * stride < end) s = SUB ? s - a[k] * xv[k] : s + a[k] * xv[k];
  for (int q = e + K * stride; q < end; q += stride) s = SUB ? s - v[q] * x[ci[q]] : s + v[q] * x[ci[q]];
  return s;
}

// Shared memory of the register smoother: two mbarriers, x twice (each buffer holds
// kXCopies copies of the group's x, xcopy_stride<T>() elements apart), then two staging
// buffers for a group's in-partition values and 16-bit columns (ecap entries each, filled
// as 16-byte rounded ranges).
struct RegSmemLayout {
  size_t x0, x1, val0, col0, val1, col1, total;
};

template <class T>
__host__ __device__ constexpr size_t round16(size_t v) {
  return (v + 15) / 16 * 16;
}

template <class T>
__host__ __device__ inline RegSmemLayout reg_smem_layout(int ecap) {
  RegSmemLayout L{};
  constexpr size_t xbytes = (size_t)kXCopies * xcopy_stride<T>() * sizeof(T);
  L.x0 = 16;
  L.x1 = L.x0 + xbytes;
  L.val0 = round16<T>(L.x1 + xbytes);
  L.col0 = round16<T>(L.val0 + (size_t)ecap * sizeof(T));
  L.val1 = round16<T>(L.col0 + (size_t)ecap * 2);
  L.col1 = round16<T>(L.val1 + (size_t)ecap * sizeof(T));
  L.total = round16<T>(L.col1 + (size_t)ecap * 2);
  return L;
}

// One thread (thread 0) starts the bulk copies of a group's values and columns (entries
// [es, ee) of the jagged-diagonal arrays) into staging buffer `buf`; completion is counted
// on bar[buf].  A group's entries are one contiguous range (the reordering stays inside
// each 32-row block).  With orp (post relax), the group's cross-partition entries
// [o0, o1), also one contiguous range, are prefetched into L2 for the b - A_out x that
// opens the group.
template <class T>
__device__ __forceinline__ void stage_group(unsigned char* sm, const RegSmemLayout& Ls, uint64_t* bar, int buf,
                                            int es, int ee, const uint16_t* __restrict__ jc,
                                            const T* __restrict__ jv, const int32_t* __restrict__ oci = nullptr,
                                            const T* __restrict__ ov = nullptr, int o0 = 0, int o1 = 0) {
  constexpr int VA = 16 / (int)sizeof(T);
  if (oci) {
    bulk_prefetch_range_l2(oci + o0, oci + o1);
    bulk_prefetch_range_l2(ov + o0, ov + o1);
  }
  const int v0 = es & ~(VA - 1), c0 = es & ~7;
  const uint32_t vbytes = (uint32_t)((((ee + VA - 1) & ~(VA - 1)) - v0) * (int)sizeof(T));
  const uint32_t cbytes = (uint32_t)((((ee + 7) & ~7) - c0) * 2);
  mbar_arrive_expect_tx(bar + buf, vbytes + cbytes);
  if (vbytes) bulk_copy_g2s(sm + (buf ? Ls.val1 : Ls.val0), jv + v0, vbytes, bar + buf);
  if (cbytes) bulk_copy_g2s(sm + (buf ? Ls.col1 : Ls.col0), jc + c0, cbytes, bar + buf);
}

// Register-resident smoother for groups of at most 512 rows whose in-partition rows
// have at most K entries: one thread per row, persistent CTAs walking the groups.
// A group's values and 16-bit local columns are contiguous in HBM; thread 0 moves the
// NEXT group's ranges into the other staging buffer with bulk asynchronous copies
// (TMA) while the CTA smooths the current one.  Lane p of the warp that owns a 32-row
// block smooths the block's row at sorted position p (rows by decreasing length), and
// the entries are stored diagonal by diagonal, so the lanes read their k-th entries
// from consecutive shared-memory words.  Each thread keeps its row's entries in
// registers across the sweeps; x is double-buffered in shared memory, kXCopies copies
// per buffer, every entry's column pointing into the copy that setup chose to spread the
// warp's gathers over the banks (one barrier per sweep).  Row sums are the one-lane case
// of the shared-memory smoother: fused multiply-adds in entry order.  A copy that does
// not land within `wait_limit` polls sets *kerr and ends the CTA after waiting (with the
// full limit) for the copies it has in flight.
// Level-0 fusions (each off when its pointer is null):
// - pre relax, b64: the right-hand side is read in FP64 and rounded to T here (and
//   stored to b_store for the post relax) instead of by a separate cast;
// - post relax, orp/oci/ov: b' = b - A_out x_in is formed here, with the same
//   subtractions in the same order as aout_rhs_kernel;
// - z64: x is written widened to FP64 there instead of to x_out;
// - dot_part (with z64): the CTA's partial sums of z.dot_r (and z.dot_o) go to
//   dot_part[blockIdx.x] (and dot_part[gridDim.x + blockIdx.x]), each thread adding
//   its rows in the order it smooths them, then block_sum; the CTA that finishes last
//   (ticket dot_count) forms the ordered totals and the PCG beta in sc.
template <class T, bool POST, int K>
__global__ void __launch_bounds__(512, 2) smooth_reg_kernel(
    int ngroups, const int32_t* __restrict__ grows, const int32_t* __restrict__ irp,
    const uint16_t* __restrict__ jc, const T* __restrict__ jv, const uint8_t* __restrict__ jrow,
    const T* __restrict__ diag, const T* __restrict__ dinv, const T* __restrict__ b, T w, int inner,
    const T* __restrict__ x_in, T* __restrict__ x_out, T* __restrict__ r_out, int ecap, double* __restrict__ kerr,
    const double* __restrict__ b64, T* __restrict__ b_store, const int32_t* __restrict__ orp,
    const int32_t* __restrict__ oci, const T* __restrict__ ov, double* __restrict__ z64,
    const double* __restrict__ dot_r, const double* __restrict__ dot_o, double* __restrict__ dot_part,
    unsigned* dot_count, double* sc, int flexible, int wait_limit) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ double sh_dot[32];
  double dz1 = 0.0, dz2 = 0.0;
  const RegSmemLayout Ls = reg_smem_layout<T>(ecap);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm);
  T* const xa = reinterpret_cast<T*>(sm + Ls.x0);
  T* const xb = reinterpret_cast<T*>(sm + Ls.x1);
  constexpr int CS = xcopy_stride<T>();
  constexpr int VA = 16 / (int)sizeof(T);
  const int t = threadIdx.x, lane = t & 31;
  // Group bounds travel across iterations, so no warp waits on a dependent global load
  // at a group's start: rows [rs, re) of this group and [rsn, ren) of the next one; thread
  // 0 also holds the next group's entry range [esn, een) and cross-partition range
  // [osn, oen) for the staging it starts, and sh_es[buf] is the entry offset where the
  // group staged into buffer buf begins.
  __shared__ int sh_es[2];
  const int g0 = blockIdx.x;
  int rs = 0, re = 0, rsn = 0, ren = 0, esn = 0, een = 0, osn = 0, oen = 0;
  if (g0 < ngroups) {
    rs = grows[g0];
    re = grows[g0 + 1];
  }
  if (g0 + (int)gridDim.x < ngroups) {
    rsn = grows[g0 + gridDim.x];
    ren = grows[g0 + gridDim.x + 1];
  }
  if (t == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    if (g0 < ngroups) {
      const int es0 = irp[rs];
      sh_es[0] = es0;
      stage_group<T>(sm, Ls, bar, 0, es0, irp[re], jc, jv);
    }
    if (g0 + (int)gridDim.x < ngroups) {
      esn = irp[rsn];
      een = irp[ren];
      if (orp) {
        osn = orp[rsn];
        oen = orp[ren];
      }
    }
  }
  __syncthreads();
  // everything above reads constant data (group bounds, entry offsets) and writes only
  // this CTA's shared memory
  pdl_enter();
  int i = 0;
  for (int g = g0; g < ngroups; g += gridDim.x, i++) {
    const int buf = i & 1;
    const uint32_t parity = (uint32_t)(i >> 1) & 1u;
    const int gn = g + gridDim.x, gn2 = gn + gridDim.x;
    // buffer buf ^ 1 was last read before the barrier that ended the previous group
    if (t == 0 && gn < ngroups) {
      sh_es[buf ^ 1] = esn;
      stage_group<T>(sm, Ls, bar, buf ^ 1, esn, een, jc, jv, orp ? oci : nullptr, ov, osn, oen);
    }
    // the bounds of the group after next, used from the next iteration on
    int rsn2 = 0, ren2 = 0;
    if (gn2 < ngroups) {
      rsn2 = grows[gn2];
      ren2 = grows[gn2 + 1];
    }
    const int wb = rs + (t & ~31);  // first row of this warp's 32-row block
    const bool live = rs + t < re;
    // Every per-row input is loaded in the block's natural order (lane p loads row wb + p,
    // no dependence on the row order), then lane p takes the values of its sorted row
    // wb + jrow from the lane that loaded them: one memory round trip per group.
    const int nrow = rs + t;
    int jr = 0, ne0 = 0, ne1 = 0;
    T nd = (T)1, ndi = (T)1, nb = (T)0, nx = (T)0;
    double ndr = 0.0, ndor = 0.0;
    if (live) {
      jr = jrow[nrow];
      ne0 = irp[nrow];
      ne1 = irp[nrow + 1];
      nd = diag[nrow];
      ndi = dinv[nrow];
      if (POST && dot_part) {
        ndr = dot_r[nrow];
        if (dot_o) ndor = dot_o[nrow];
      }
      if (POST) {
        nb = b[nrow];
        if (orp) nb = gather_row<T, 8, true>(oci, ov, x_in, orp[nrow], orp[nrow + 1], 1, nb);
        nx = x_in[nrow];
      } else if (b64) {
        nb = (T)b64[nrow];
        b_store[nrow] = nb;
      } else {
        nb = b[nrow];
      }
    }
    // the next group's per-row inputs into L2 while this group is smoothed
    if (gn < ngroups) {
      const int nr2 = rsn + t;
      if (nr2 < ren) {
        prefetch_l2(jrow + nr2);
        prefetch_l2(irp + nr2);
        prefetch_l2(diag + nr2);
        prefetch_l2(dinv + nr2);
        if (POST) {
          prefetch_l2(b + nr2);
          prefetch_l2(x_in + nr2);
          if (orp) prefetch_l2(orp + nr2);
          if (dot_part) {
            prefetch_l2(dot_r + nr2);
            if (dot_o) prefetch_l2(dot_o + nr2);
          }
        } else if (b64) {
          prefetch_l2(b64 + nr2);
        } else {
          prefetch_l2(b + nr2);
        }
      }
    }
    const int row = wb + jr;
    const int loc = row - rs;
    // every lane of the warp executes every shuffle (none sits under a lane-dependent branch)
    const int e0 = __shfl_sync(0xffffffffu, ne0, jr);
    const int e1 = __shfl_sync(0xffffffffu, ne1, jr);
    const int len = live ? e1 - e0 : 0;
    const T d = __shfl_sync(0xffffffffu, nd, jr), di = __shfl_sync(0xffffffffu, ndi, jr);
    const T bb = __shfl_sync(0xffffffffu, nb, jr);
    const double dr = __shfl_sync(0xffffffffu, ndr, jr), dor = __shfl_sync(0xffffffffu, ndor, jr);
    const T xs = __shfl_sync(0xffffffffu, nx, jr);
    T x = POST ? xs : (w * bb) * di;
    if (live) {
#pragma unroll
      for (int c = 0; c < kXCopies; c++) xa[loc + c * CS] = x;
    }
    const int kmax = __shfl_sync(0xffffffffu, len, 0);  // lane 0 holds the block's longest row
    const bool ok = mbar_wait_bounded(bar + buf, parity, wait_limit);
    // Entry k of this lane's row: its value, and the index of the x it reads within an x
    // buffer (group-local column + copy stride: below 2^16), two per register.
    T val[K];
    uint32_t offp[K / 2];
    {
      const int es = sh_es[buf];
      // the block's entries start where its first row's do (the reordering stays in the
      // block): lane 0 loaded that row's offset
      const int eb = __shfl_sync(0xffffffffu, ne0, 0);
      const T* sval = reinterpret_cast<const T*>(sm + (buf ? Ls.val1 : Ls.val0)) + (eb - (es & ~(VA - 1)));
      const uint16_t* scol = reinterpret_cast<const uint16_t*>(sm + (buf ? Ls.col1 : Ls.col0)) + (eb - (es & ~7));
      int dk = lane;  // this lane's position on diagonal k
#pragma unroll
      for (int k = 0; k < K; k++) {
        const unsigned m = __ballot_sync(0xffffffffu, k < len);
        const bool a = ok && k < len;
        val[k] = a ? sval[dk] : (T)0;
        const uint32_t o = a ? (uint32_t)scol[dk] : 0u;
        if (k & 1) offp[k >> 1] |= o << 16;
        else offp[k >> 1] = o;
        dk += __popc(m);
      }
    }
    // thread 0: the entry and cross-partition ranges of the group after next (its row
    // bounds have arrived by now), for the staging it starts in the next iteration
    if (t == 0 && gn2 < ngroups) {
      esn = irp[rsn2];
      een = irp[ren2];
      if (orp) {
        osn = orp[rsn2];
        oen = orp[ren2];
      }
    }
    if (__syncthreads_or(!ok)) {
      if (t == 0) {
        *kerr = 1.0 + g;  // where: the first group whose copy did not land
        // let the copies in flight land before the CTA exits
        (void)mbar_wait_bounded(bar + buf, parity);
        if (gn < ngroups) (void)mbar_wait_bounded(bar + (buf ^ 1), (uint32_t)((i + 1) >> 1) & 1u);
      }
      return;
    }
    // Fused multiply-adds in entry order over the row's entries (lanes past their row's
    // end are predicated off and touch no shared memory).
    auto rowsum = [&](const T* src) {
      T sax = 0;
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k < kmax && k < len) sax = fma(val[k], src[(offp[k >> 1] >> ((k & 1) * 16)) & 0xffffu], sax);
      return sax;
    };
    auto sweep = [&](const T* src, T* dst) {
      if (live) {
        x = relax(x, bb, rowsum(src), d, di, w);
#pragma unroll
        for (int c = 0; c < kXCopies; c++) dst[loc + c * CS] = x;
      }
      __syncthreads();
    };
    int it = 0;
    for (; it + 1 < inner; it += 2) {
      sweep(xa, xb);
      sweep(xb, xa);
    }
    const T* last = xa;
    if (it < inner) {
      sweep(xa, xb);
      last = xb;
    }
    if (live) {
      if (POST && z64) {
        const double zr = (double)x;
        z64[row] = zr;
        if (dot_part) {
          dz1 = fma(zr, dr, dz1);
          if (dot_o) dz2 = fma(zr, dor, dz2);
        }
      } else {
        x_out[row] = x;
      }
      if (!POST) {
        T u = bb - rowsum(last);
        r_out[row] = u - d * x;
      }
    }
    __syncthreads();  // x buffers and this staging buffer are free for the next group
    rs = rsn;
    re = ren;
    rsn = rsn2;
    ren = ren2;
  }
  if (POST && dot_part && z64) {
    const double t1 = block_sum(dz1, sh_dot);
    if (threadIdx.x == 0) dot_part[blockIdx.x] = t1;
    if (dot_o) {
      const double t2 = block_sum(dz2, sh_dot);
      if (threadIdx.x == 0) dot_part[gridDim.x + blockIdx.x] = t2;
    }
    if (!last_block_done(dot_count)) return;
    const double rzn = ordered_total(dot_part, gridDim.x, sh_dot);
    const double zro = dot_o ? ordered_total(dot_part + gridDim.x, gridDim.x, sh_dot) : 0.0;
    if (threadIdx.x == 0) {
      sc[S_RZNEW] = rzn;
      if (dot_o) sc[S_ZROLD] = zro;
      beta_update(sc, flexible);
      *dot_count = 0u;
    }
  }
}

// r -= A_out x (preAout_kernel, gauss_seidel.cu:1977-2015).
template <class T>
__global__ void aout_residual_kernel(int n, const int32_t* __restrict__ orp, const int32_t* __restrict__ oci,
                                     const T* __restrict__ ov, const T* __restrict__ x, T* __restrict__ r) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T ri = r[i];
  const T s = gather_row<T, 8, false>(oci, ov, x, orp[i], orp[i + 1], 1, (T)0);
  r[i] = ri - s;
}

// y = M x (accumulate = 0) or y = y + M x (accumulate = 1) with S lanes per row:
// lane j sums entries j, j+S, ... in order, then an xor butterfly combines the lanes.
// S comes from lanes_for_rows(); the CPU oracle evaluates the same order.
template <class T, int S>
__global__ void spmv_lanes_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                  const T* __restrict__ v, const T* __restrict__ x, T* __restrict__ y, int accumulate) {
  constexpr int K = S == 1 ? 8 : 4;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) / S;
  const int j = threadIdx.x & (S - 1);
  const bool live = g < n;
  // the operator's row bounds and first K entries of this lane are constant: loaded
  // before waiting for the kernel that writes x
  int e = 0, end = 0, c[K];
  T a[K];
  if (live) {
    e = rp[g] + j;
    end = rp[g + 1];
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int q = e + k * S;
    c[k] = q < end ? ci[q] : 0;
    a[k] = q < end ? v[q] : (T)0;
  }
  pdl_enter();
  // the sum of gather_row: products rounded separately, added in entry order from 0
  T s = 0;
  if (live) {
    T xv[K];
#pragma unroll
    for (int k = 0; k < K; k++) xv[k] = e + k * S < end ? x[c[k]] : (T)0;
#pragma unroll
    for (int k = 0; k < K; k++)
      if (e + k * S < end) s = s + a[k] * xv[k];
    for (int q = e + K * S; q < end; q += S) s = s + v[q] * x[ci[q]];
  }
#pragma unroll
  for (int off = S >> 1; off > 0; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off, S);
  if (live && j == 0) y[g] = accumulate ? y[g] + s : s;
}

// Coarsest level: x = A^-1 b with the explicit FP64 inverse, one warp per row: lane j
// accumulates columns j, j+32, ... with fma, then an xor butterfly (the oracle uses
// the same order).
template <class T>
__global__ void coarse_solve_kernel(int n, const double* __restrict__ inv, const T* __restrict__ b, T* __restrict__ x) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  // the inverse is constant: this lane's first four entries are loaded before the wait
  double iv[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int j = lane + 32 * q;
    iv[q] = i < n && j < n ? inv[(int64_t)i * n + j] : 0.0;
  }
  pdl_enter();
  double s = 0.0;
  if (i < n) {
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (lane + 32 * q < n) s = fma(iv[q], (double)b[lane + 32 * q], s);
    for (int j = lane + 128; j < n; j += 32) s = fma(inv[(int64_t)i * n + j], (double)b[j], s);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off);
  if (i < n && lane == 0) x[i] = (T)s;
}

// ---- FP64 PCG kernels -----------------------------------------------------------------
// y = A p (rows in order, fused multiply-add) and a partial dot(y, p).
__global__ void spmv_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int e = rp[i]; e < rp[i + 1]; e++) s = fma(v[e], x[ci[e]], s);
  y[i] = s;
}


// partial dot(a, b) (and dot(a, c) when c != nullptr into partial2)
__global__ void dot_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                           const double* __restrict__ c, double* partial, double* partial2) {
  __shared__ double sh[32];
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    s1 = fma(a[i], b[i], s1);
    if (c) s2 = fma(a[i], c[i], s2);
  }
  double t = block_sum(s1, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (c) {
    double t2 = block_sum(s2, sh);
    if (threadIdx.x == 0) partial2[blockIdx.x] = t2;
  }
}

// Sum nparts partials (fixed order) into slot.
// Sum of partial[0 .. nparts) in the order of one 1024-thread block: virtual thread
// v adds partial[v], partial[v + 1024], ...; each virtual warp folds its 32 values
// with an xor butterfly and the 32 warp sums are folded the same way.  Any block
// whose size divides 1024 gets the same bits (valid in thread 0).
__device__ double ordered_total(const double* partial, int nparts, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // a warp stands in for up to 4 virtual warps per pass; their first partials are
  // loaded together (one L2 round trip) before the adds and butterflies
  for (int vw0 = w; vw0 < 32; vw0 += 4 * nw) {
    double v[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const int q = (vw0 + m * nw) * 32 + lane;
      v[m] = (vw0 + m * nw < 32 && q < nparts) ? 0.0 + partial[q] : 0.0;  // 0 + x: the sum's first add
    }
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const int vw = vw0 + m * nw;
      if (vw < 32) {
        for (int q = vw * 32 + lane + 1024; q < nparts; q += 1024) v[m] += partial[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[m] += __shfl_xor_sync(0xffffffffu, v[m], o);
        if (lane == 0) sh[vw] = v[m];
      }
    }
  }
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = sh[lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

__global__ void finalize_kernel(const double* partial, int nparts, double* slot) {
  __shared__ double sh[32];
  double t = ordered_total(partial, nparts, sh);
  if (threadIdx.x == 0) *slot = t;
}

// After every block wrote its partial: true in the block that finishes last, which
// then reads all partials (the fence orders the writes before the ticket).
__device__ bool last_block_done(unsigned* counter) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// r = b - y; partial ||r||^2
__global__ void residual_kernel(int n, const double* __restrict__ b, const double* __restrict__ y,
                                double* __restrict__ r, double* partial) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = b[i] - y[i];
    r[i] = v;
    acc = fma(v, v, acc);
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}



// x += alpha p; r -= alpha y (rold = r first when flexible); partial ||r||^2
__global__ void update_kernel(int n, double* __restrict__ sc, const double* __restrict__ p,
                              const double* __restrict__ y, double* __restrict__ x, double* __restrict__ r,
                              double* __restrict__ rold, double* partial, unsigned* counter) {
  pdl_enter();
  __shared__ double sh[32];
  const double alpha = sc[S_ALPHA];
  double acc = 0.0;
  // elements i, i + G, i + 2G, ... in order; four at a time with all loads issued first
  const int G = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * G < n; i += 4 * G) {
    double rr[4], pp[4], xx[4], yy[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      rr[u] = r[i + u * G];
      pp[u] = p[i + u * G];
      xx[u] = x[i + u * G];
      yy[u] = y[i + u * G];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if (rold) rold[i + u * G] = rr[u];
      x[i + u * G] = fma(alpha, pp[u], xx[u]);
      const double ri = fma(-alpha, yy[u], rr[u]);
      r[i + u * G] = ri;
      acc = fma(ri, ri, acc);
    }
  }
  for (; i < n; i += G) {
    double ri = r[i];
    if (rold) rold[i] = ri;
    x[i] = fma(alpha, p[i], x[i]);
    ri = fma(-alpha, y[i], ri);
    r[i] = ri;
    acc = fma(ri, ri, acc);
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  // r.r total by the last block (same sum as finalize_kernel)
  if (!last_block_done(counter)) return;
  const double nr = ordered_total(partial, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc[S_NR] = nr;
    *counter = 0u;
  }
}

// beta (cgcycle.cu:52-54; Polak-Ribiere when flexible); 0 on the first iteration,
// where p = z.
__device__ void beta_update(double* sc, int flexible) {
  double rz = sc[S_RZ], rzn = sc[S_RZNEW];
  if (sc[S_FIRST] != 0.0) {
    sc[S_BETA] = 0.0;
    sc[S_FIRST] = 0.0;
  } else {
    sc[S_BETA] = flexible ? (rzn - sc[S_ZROLD]) / rz : rzn / rz;
  }
  sc[S_RZ] = rzn;
}

__device__ void alpha_update(double* sc) {
  double yp = sc[S_YP];
  if (!(yp > 0.0) || !isfinite(yp)) sc[S_FLAG] = 1.0;
  sc[S_ALPHA] = sc[S_RZ] / yp;
}

// The outer PCG's y = A p and p.y, one thread per row over a fixed grid; the last
// block forms p.y and alpha (same sums as a separate finalize and alpha step).
__global__ void spmv_dot_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                      const double* __restrict__ v, const double* __restrict__ p,
                                      double* __restrict__ y, double* __restrict__ partial, double* sc,
                                      unsigned* counter) {
  pdl_enter();
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int a = rp[i], b = rp[i + 1];
    const double pi = p[i];
    double s = 0.0;
    // entries in groups of 8: all columns and values, then all gathers, then the
    // fused multiply-adds in entry order
    for (int e0 = a; e0 < b; e0 += 8) {
      int c[8];
      double w[8], x[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        c[k] = e0 + k < b ? ci[e0 + k] : 0;
        w[k] = e0 + k < b ? v[e0 + k] : 0.0;
      }
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = e0 + k < b ? p[c[k]] : 0.0;
#pragma unroll
      for (int k = 0; k < 8; k++)
        if (e0 + k < b) s = fma(w[k], x[k], s);
    }
    y[i] = s;
    acc = fma(s, pi, acc);
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (!last_block_done(counter)) return;
  const double yp = ordered_total(partial, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc[S_YP] = yp;
    alpha_update(sc);
    *counter = 0u;
  }
}

// Row i of the sliced operator: its entries in order (padding, column -1, comes after
// them and is skipped), in groups of 8 loads in flight; the same fused multiply-adds
// as the CSR loop.  The 32 rows of a slice are the 32 lanes of a warp, so each load
// instruction reads 32 consecutive columns or values.
__device__ __forceinline__ double sliced_row(int i, const int32_t* __restrict__ off, const int32_t* __restrict__ ci,
                                             const double* __restrict__ v, const double* __restrict__ p) {
  const int sl = i >> 5, e1 = off[sl + 1];
  double s = 0.0;
  for (int e0 = off[sl] + (i & 31); e0 < e1; e0 += 256) {
    int c[8];
    double w[8], x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int q = e0 + 32 * k;
      c[k] = q < e1 ? ci[q] : -1;
      w[k] = q < e1 ? v[q] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = c[k] >= 0 ? p[c[k]] : 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (c[k] >= 0) s = fma(w[k], x[k], s);
  }
  return s;
}

// spmv_dot_kernel on the sliced operator: the same rows per thread (the grid is a
// whole number of warps, so a warp's 32 rows are one slice) and the same sums.
__global__ void spmv_dot_sliced_kernel(int n, const int32_t* __restrict__ off, const int32_t* __restrict__ ci,
                                       const double* __restrict__ v, const double* __restrict__ p,
                                       double* __restrict__ y, double* __restrict__ partial, double* sc,
                                       unsigned* counter) {
  pdl_enter();
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double s = sliced_row(i, off, ci, v, p);
    y[i] = s;
    acc = fma(s, p[i], acc);
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (!last_block_done(counter)) return;
  const double yp = ordered_total(partial, gridDim.x, sh);
  if (threadIdx.x == 0) {
    sc[S_YP] = yp;
    alpha_update(sc);
    *counter = 0u;
  }
}

__global__ void spmv_sliced_kernel(int n, const int32_t* __restrict__ off, const int32_t* __restrict__ ci,
                                   const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = sliced_row(i, off, ci, v, x);
}

// z.r (and z.r_old for the flexible beta) with the totals and beta formed by the
// last block (same sums as dot_kernel + finalize_kernel + the beta step).
__global__ void dot_beta_kernel(int n, const double* __restrict__ z, const double* __restrict__ r,
                                const double* __restrict__ rold, double* partial, double* partial2, double* sc,
                                int flexible, unsigned* counter) {
  pdl_enter();
  __shared__ double sh[32];
  double s1 = 0.0, s2 = 0.0;
  // elements i, i + G, ... in order; four at a time with all loads issued first
  const int G = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * G < n; i += 4 * G) {
    double zz[4], rr[4], oo[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      zz[u] = z[i + u * G];
      rr[u] = r[i + u * G];
      oo[u] = rold ? rold[i + u * G] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      s1 = fma(zz[u], rr[u], s1);
      if (rold) s2 = fma(zz[u], oo[u], s2);
    }
  }
  for (; i < n; i += G) {
    s1 = fma(z[i], r[i], s1);
    if (rold) s2 = fma(z[i], rold[i], s2);
  }
  double t = block_sum(s1, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
  if (rold) {
    double t2 = block_sum(s2, sh);
    if (threadIdx.x == 0) partial2[blockIdx.x] = t2;
  }
  if (!last_block_done(counter)) return;
  const double rzn = ordered_total(partial, gridDim.x, sh);
  const double zro = rold ? ordered_total(partial2, gridDim.x, sh) : 0.0;
  if (threadIdx.x == 0) {
    sc[S_RZNEW] = rzn;
    if (rold) sc[S_ZROLD] = zro;
    beta_update(sc, flexible);
    *counter = 0u;
  }
}

// Continue the device-side PCG loop?  Stops on convergence (the host's test:
// sqrt(r.r) / |b| <= tol), breakdown, a non-finite residual, a smoother copy that
// timed out, or maxIters.
__global__ void pcg_check_kernel(double* sc, cudaGraphConditionalHandle loop) {
  pdl_enter();
  const double it = sc[S_IT] + 1.0;
  sc[S_IT] = it;
  const double nr = sqrt(sc[S_NR]);
  const bool stop = sc[S_FLAG] != 0.0 || sc[S_KERR] != 0.0 || !isfinite(nr) || nr / sc[S_BNORM] <= sc[S_TOL] ||
                    it >= sc[S_MAXIT];
  cudaGraphSetConditional(loop, stop ? 0u : 1u);
}

__global__ void set_slot_kernel(double* sc, int slot, double v) { sc[slot] = v; }

__global__ void pupdate_kernel(int n, const double* __restrict__ sc, const double* __restrict__ z,
                               double* __restrict__ p) {
  pdl_enter();
  const double beta = sc[S_BETA];
  const int G = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * G < n; i += 4 * G) {
    double pp[4], zz[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      pp[u] = p[i + u * G];
      zz[u] = z[i + u * G];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) p[i + u * G] = fma(beta, pp[u], zz[u]);
  }
  for (; i < n; i += G) p[i] = fma(beta, p[i], z[i]);
}

__global__ void perm_vec_in_kernel(int n, const int32_t* perm, const double* in, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[perm[i]] = in[i];
}

__global__ void perm_vec_out_kernel(int n, const int32_t* perm, const double* in, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}

// ---- V-cycle driver ------------------------------------------------------------------
constexpr size_t kStageLimit = 200 * 1024;  // staged smoother: one 1024-thread CTA per SM
constexpr size_t kSmemOptIn = 227 * 1024;   // largest dynamic shared memory of one CTA
constexpr int kMaxCluster = 8;              // portable thread-block cluster size

// Lanes per row for the R/P products: the same rule in the CPU oracle.
inline int lanes_for_rows(int64_t nnz, int n) {
  double avg = n > 0 ? (double)nnz / n : 0.0;
  int s = 1;
  while (s < 32 && s * 4 < avg) s <<= 1;
  return s;
}

template <class T>
void spmv_lanes(const DCsr<T>& M, const T* x, T* y, int accumulate, cudaStream_t st) {
  const int S = lanes_for_rows(M.nnz, M.n);
  const int64_t threads = (int64_t)M.n * S;
  const int g = grid_for(threads, 256);
  switch (S) {
    case 1: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 1>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
    case 2: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 2>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
    case 4: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 4>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
    case 8: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 8>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
    case 16: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 16>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
    default: FG_LAUNCH_PDL((spmv_lanes_kernel<T, 32>), g, 256, 0, st, M.n, M.rp.p, M.ci.p, M.v.p, x, y, accumulate); break;
  }
}

template <class T>
using ClusterSmoothFn = void (*)(const int32_t*, const int32_t*, const int32_t*, const T*, const int32_t*,
                                 const int32_t*, const T*, const T*, const T*, const T*, T, int, const T*, T*, T*, int,
                                 int, int);

template <class T>
ClusterSmoothFn<T> pick_cluster_kernel(bool post, bool staged, int S) {
#define FG_SMOOTH_PICK(SS)                                                                              \
  return post ? (staged ? smooth_cluster_kernel<T, true, true, SS> : smooth_cluster_kernel<T, true, false, SS>) \
              : (staged ? smooth_cluster_kernel<T, false, true, SS> : smooth_cluster_kernel<T, false, false, SS>)
  switch (S) {
    case 1: FG_SMOOTH_PICK(1);
    case 2: FG_SMOOTH_PICK(2);
    case 4: FG_SMOOTH_PICK(4);
    case 8: FG_SMOOTH_PICK(8);
    case 16: FG_SMOOTH_PICK(16);
    default: FG_SMOOTH_PICK(32);
  }
#undef FG_SMOOTH_PICK
}

template <class T>
using CregSmoothFn = void (*)(const int32_t*, const int32_t*, const int32_t*, const T*, const T*, const T*, const T*,
                              T, int, const T*, T*, T*, int);

template <class T, int S>
CregSmoothFn<T> pick_creg_k(bool post, int K) {
  if (K <= 8) return post ? smooth_creg_kernel<T, true, S, 8> : smooth_creg_kernel<T, false, S, 8>;
  return post ? smooth_creg_kernel<T, true, S, 16> : smooth_creg_kernel<T, false, S, 16>;
}

template <class T>
CregSmoothFn<T> pick_creg_kernel(bool post, int S, int K) {
  switch (S) {
    case 1: return pick_creg_k<T, 1>(post, K);
    case 2: return pick_creg_k<T, 2>(post, K);
    case 4: return pick_creg_k<T, 4>(post, K);
    case 8: return pick_creg_k<T, 8>(post, K);
    case 16: return pick_creg_k<T, 16>(post, K);
    default: return pick_creg_k<T, 32>(post, K);
  }
}

// Launch with a 1-D thread-block cluster of `cluster` CTAs (counted like FG_LAUNCH).
template <class... KArgs, class... Args>
void launch_clustered(void (*k)(KArgs...), int grid, int block, size_t smem, int cluster, cudaStream_t s,
                      Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  // both clustered smoothers call pdl_wait() before they touch memory other kernels write
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl_enabled && t_pdl_scope ? 2 : 1;
  g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
  FG_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...));
}

// Entries of each CTA's row slice when groups are split over `C` CTAs.
__global__ void slice_entries_kernel(int ngroups, int C, const int32_t* grows, const int32_t* irp, int32_t* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ngroups * C) return;
  const int g = i / C, c = i % C;
  const int rs = grows[g], m = grows[g + 1] - rs;
  const int qs = (m + C - 1) / C;
  const int ss = min(m, c * qs), se = min(m, ss + qs);
  out[i] = irp[rs + se] - irp[rs + ss];
}

// Cross-partition products with S lanes per row, for levels with long rows: lane j
// forms the products of entries j, j + S, ... (4 rounds of loads in flight), and lane 0
// of the row receives them through shuffles and adds them in entry order -- the same
// sums as the per-thread gathers.
// RHS == false: out_i = base_i - (sum of the row's products, from 0)   (the residual);
// RHS == true:  out_i = base_i - p_0 - p_1 - ...                        (b' = b - A_out x).
template <class T, bool RHS, int S>
__global__ void aout_lanes_kernel(int n, const int32_t* __restrict__ orp, const int32_t* __restrict__ oci,
                                  const T* __restrict__ ov, const T* base, const T* __restrict__ x, T* out) {
  pdl_enter();
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) / S, j = threadIdx.x & (S - 1);
  const bool live = g < n;
  int a = 0, b = 0;
  if (live) {
    a = orp[g];
    b = orp[g + 1];
  }
  T acc = live ? base[g] : (T)0, sum = (T)0;
  const int rounds = (b - a + S - 1) / S;
  const int wmax = __reduce_max_sync(0xffffffffu, rounds);  // warp-uniform trip count
  for (int m0 = 0; m0 < wmax; m0 += 4) {
    int c[4];
    T v[4], p[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int q = a + (m0 + k) * S + j;
      c[k] = q < b ? oci[q] : 0;
      v[k] = q < b ? ov[q] : (T)0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int q = a + (m0 + k) * S + j;
      p[k] = q < b ? v[k] * x[c[k]] : (T)0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int t = 0; t < S; t++) {
        const T pt = __shfl_sync(0xffffffffu, p[k], t, S);
        if (j == 0 && a + (m0 + k) * S + t < b) {
          if (RHS) acc = acc - pt;
          else sum = sum + pt;
        }
      }
  }
  if (live && j == 0) out[g] = RHS ? acc : acc - sum;
}

// Lanes per row of the cross-partition kernels: 1 (per-thread gather) below 8 entries
// per row on average, else a power of two near a quarter of the average row.
template <class T>
int aout_lanes(const Level<T>& L) {
  if (L.aout_lanes_tuned > 0) return L.aout_lanes_tuned;  // chosen by the autotuner (same sums)
  const double avg = L.n > 0 ? (double)L.Aout.nnz / L.n : 0.0;
  if (avg < 8.0) return 1;
  int s = 2;
  while (s < 32 && s * 4 < avg) s <<= 1;
  return s;
}

template <class T, bool RHS>
void launch_aout_lanes(cudaStream_t st, const Level<T>& L, int S, const T* base, const T* x, T* out) {
  const int g = grid_for((int64_t)L.n * S, 256);
#define FG_AOUT(SS)                                                                                   \
  FG_LAUNCH_PDL((aout_lanes_kernel<T, RHS, SS>), g, 256, 0, st, L.n, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, base, x, out)
  switch (S) {
    case 2: FG_AOUT(2); break;
    case 4: FG_AOUT(4); break;
    case 8: FG_AOUT(8); break;
    case 16: FG_AOUT(16); break;
    default: FG_AOUT(32); break;
  }
#undef FG_AOUT
}

template <class T>
void aout_rhs(cudaStream_t s, const Level<T>& L, const T* b, const T* x, T* bp);

// Post-smoother right-hand side b' = b - A_out x (the first loop of
// postRelaxSym_kernel, gauss_seidel.cu:3676-3684), one thread per row.
template <class T>
__global__ void aout_rhs_kernel(int n, const int32_t* __restrict__ orp, const int32_t* __restrict__ oci,
                                const T* __restrict__ ov, const T* __restrict__ b, const T* __restrict__ x,
                                T* __restrict__ bp) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // acc + (-v) x and acc - v x round identically: the negation is exact
  bp[i] = gather_row<T, 8, true>(oci, ov, x, orp[i], orp[i + 1], 1, b[i]);
}

template <class T>
void aout_rhs(cudaStream_t s, const Level<T>& L, const T* b, const T* x, T* bp) {
  const int S = aout_lanes(L);
  if (S > 1)
    launch_aout_lanes<T, true>(s, L, S, b, x, bp);
  else
    FG_LAUNCH_PDL(aout_rhs_kernel<T>, grid_for(L.n, 256), 256, 0, s, L.n, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, b, x,
              bp);
}

// r -= A_out x (preAout_kernel, gauss_seidel.cu:1977-2015).
template <class T>
void aout_residual(cudaStream_t s, const Level<T>& L, const T* x, T* r) {
  const int S = aout_lanes(L);
  if (S > 1)
    launch_aout_lanes<T, false>(s, L, S, r, x, r);
  else
    FG_LAUNCH_PDL(aout_residual_kernel<T>, grid_for(L.n, 256), 256, 0, s, L.n, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p, x,
              r);
}

// Fused level-0 inputs and outputs of the register smoother (all null: none).
template <class T>
struct RegFusion {
  const double* b64 = nullptr;  // pre relax: FP64 right-hand side, rounded to T in the kernel ...
  T* b_store = nullptr;         // ... and stored here
  bool aout = false;            // post relax: b' = b - A_out x_in formed in the kernel
  double* z64 = nullptr;        // result widened to FP64 here instead of xout
  const double* dot_r = nullptr;  // with z64: CTA partials of z.dot_r (and z.dot_o) to dot_part
  const double* dot_o = nullptr;
  double* dot_part = nullptr;
};

// The partition-block sweeps alone; a post relax reads its right-hand side b' =
// b - A_out x_in from b (as computed by aout_rhs_kernel) unless f.aout.
template <class T>
void smooth_sweeps(Ctx& c, Level<T>& L, bool post, const T* b, const T* xin, T* xout, T* rout,
                   const RegFusion<T>& f = RegFusion<T>()) {
  cudaStream_t s = c.stream;
  const int32_t* aorp = post ? nullptr : L.Aout.rp.p;
  const T w = (T)c.cfg.smootherWeight;
  const int inner = post ? c.cfg.postInnerIters : c.cfg.preInnerIters;
  if (smoother_in_registers(L.max_in_row, L.max_part_rows)) {
    auto k = post ? smooth_reg_kernel<T, true, kRegRow> : smooth_reg_kernel<T, false, kRegRow>;
    if (L.smooth_smem > 48 * 1024)
      ensure_smem(k, L.smooth_smem);
    FG_LAUNCH_PDL(k, L.smooth_grid, L.smooth_threads, L.smooth_smem, s, L.ngroups, L.grows.p, L.Ain.rp.p, L.jc16.p,
              L.jv.p, L.jrow.p, L.diag.p, L.dinv.p, b, w, inner, xin, xout, rout, L.max_group_ents + 16,
              c.red.p + 2 * kRedBlocks + S_KERR, f.b64, f.b_store, f.aout ? L.Aout.rp.p : nullptr,
              f.aout ? L.Aout.ci.p : nullptr, f.aout ? L.Aout.v.p : nullptr, f.z64, f.dot_r, f.dot_o, f.dot_part,
              c.rcount.p + 3, c.red.p + 2 * kRedBlocks, f.dot_o ? 1 : 0, c.copy_wait_limit);
    return;
  }
  if (L.smooth_k > 0) {
    CregSmoothFn<T> k = pick_creg_kernel<T>(post, L.smooth_lanes, L.smooth_k);
    if (L.smooth_smem > 48 * 1024)
      ensure_smem(k, L.smooth_smem);
    launch_clustered(k, L.ngroups * L.cluster, L.smooth_threads, L.smooth_smem, L.cluster, s,
                     (const int32_t*)L.grows.p, (const int32_t*)L.Ain.rp.p, (const int32_t*)L.Ain.ci.p,
                     (const T*)L.Ain.v.p, (const T*)L.diag.p, (const T*)L.dinv.p, b, w, inner, xin, xout, rout,
                     L.max_group_rows);
    return;
  }
  ClusterSmoothFn<T> k = pick_cluster_kernel<T>(post, L.smooth_staged, L.smooth_lanes);
  // the limit is a per-function attribute shared by every handle: set it per launch
  if (L.smooth_smem > 48 * 1024)
    ensure_smem(k, L.smooth_smem);
  launch_clustered(k, L.ngroups * L.cluster, L.smooth_threads, L.smooth_smem, L.cluster, s,
                   (const int32_t*)L.grows.p, (const int32_t*)L.Ain.rp.p, (const int32_t*)L.Ain.ci.p,
                   (const T*)L.Ain.v.p, aorp, (const int32_t*)L.Aout.ci.p, (const T*)L.Aout.v.p,
                   (const T*)L.diag.p, (const T*)L.dinv.p, b, w, inner, xin, xout, rout, L.max_group_rows,
                   L.slice_rows, L.slice_ents);
}

// Pre relax (post == false) or post relax: b' = b - A_out x_in, then the sweeps.
// b64 (pre relax): b is first rounded from this FP64 vector into b (b_store);
// z64: the result goes to z64 in FP64 instead of xout.  The register smoother does
// both (and b') inside its kernel; the other smoothers use separate kernels.
template <class T>
void smooth(Ctx& c, Level<T>& L, bool post, const T* b, const T* xin, T* xout, T* rout,
            const double* b64 = nullptr, T* b_store = nullptr, double* z64 = nullptr) {
  cudaStream_t s = c.stream;
  if (smoother_in_registers(L.max_in_row, L.max_part_rows)) {
    RegFusion<T> f;
    f.b64 = post ? nullptr : b64;
    f.b_store = post ? nullptr : b_store;
    f.aout = post && L.Aout.nnz > 0;
    f.z64 = z64;
    if (z64 && c.zdot && L.smooth_grid <= kRedBlocks / 2) {
      f.dot_r = c.zdot->r;
      f.dot_o = c.zdot->rold;
      f.dot_part = c.zdot->part;
      c.zdot->done = true;
    }
    smooth_sweeps<T>(c, L, post, b, xin, xout, rout, f);
    return;
  }
  if (!post && b64) {
    FG_LAUNCH_PDL(cast_in_kernel<T>, grid_for(L.n, 256), 256, 0, s, L.n, b64, b_store);
    b = b_store;
  }
  if (post) {
    aout_rhs<T>(s, L, b, xin, L.bp.p);
    b = L.bp.p;
  }
  smooth_sweeps<T>(c, L, post, b, xin, xout, rout);
  if (z64) FG_LAUNCH_PDL(cast_out_kernel<T>, grid_for(L.n, 256), 256, 0, s, L.n, xout, z64);
}

// Records a named event on the stream when stage timing is on (never during capture).
void stage_mark(Ctx& c, const char* what, int l) {
  if (!c.stage_marks) return;
  cudaEvent_t e;
  FG_CUDA(cudaEventCreate(&e));
  FG_CUDA(cudaEventRecord(e, c.stream));
  c.stage_marks->emplace_back(std::string(what) + " l" + std::to_string(l), e);
}

// r = b - M x with M's rows in their stored entry order, products rounded separately.
template <class T>
__global__ void residual_rows_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                     const T* __restrict__ v, const T* __restrict__ b, const T* __restrict__ x,
                                     T* __restrict__ r) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = gather_row<T, 8, true>(ci, v, x, rp[i], rp[i + 1], 1, b[i]);
}

template <class T>
__global__ void add_into_kernel(int n, const T* __restrict__ d, T* __restrict__ x) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] + d[i];
}

// ---- l1-Jacobi smoother (cfg.smoother == 1) ---------------------------------------------
// A point smoother on the level's whole permuted operator Ap (Baker, Falgout, Kolev and Yang,
// "Multigrid smoothers for ultraparallel computing", SISC 2011): x += w (b - A x) / l1 with
// l1_i = sum_j |a_ij|, convergent for any symmetric positive definite A without a damping
// estimate.  Row sums with fused multiply-adds in entry order (the oracle uses the same).
template <class T>
__global__ void l1_inverse_kernel(int n, const int32_t* __restrict__ rp, const T* __restrict__ v,
                                  T* __restrict__ l1inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T s = 0;
  for (int e = rp[i]; e < rp[i + 1]; e++) s = s + fabs(v[e]);
  l1inv[i] = (T)1 / s;
}

template <class T>
__device__ __forceinline__ T row_fma_sum(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                        const T* __restrict__ v, const T* __restrict__ x, int i) {
  const int a = rp[i], b = rp[i + 1];
  T s = 0;
  for (int e0 = a; e0 < b; e0 += 8) {
    int c[8];
    T w[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      c[k] = e0 + k < b ? ci[e0 + k] : 0;
      w[k] = e0 + k < b ? v[e0 + k] : (T)0;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) xv[k] = e0 + k < b ? x[c[k]] : (T)0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (e0 + k < b) s = fma(w[k], xv[k], s);
  }
  return s;
}

// xout = xin + (w (b - A xin)) l1inv
template <class T>
__global__ void l1_sweep_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const T* __restrict__ v, const T* __restrict__ b, const T* __restrict__ l1inv, T w,
                                const T* __restrict__ xin, T* __restrict__ xout) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T s = row_fma_sum(rp, ci, v, xin, i);
  xout[i] = xin[i] + (w * (b[i] - s)) * l1inv[i];
}

// The first sweep from x = 0: the row sums vanish (+0), so x = 0 + (w (b - 0)) l1inv with no
// pass over A (the same bits as the general sweep on a zero vector).
template <class T>
__global__ void l1_first_sweep_kernel(int n, const T* __restrict__ b, const T* __restrict__ l1inv, T w,
                                      T* __restrict__ x) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (T)0 + (w * (b[i] - (T)0)) * l1inv[i];
}

// r = b - A x
template <class T>
__global__ void full_residual_kernel(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                     const T* __restrict__ v, const T* __restrict__ b, const T* __restrict__ x,
                                     T* __restrict__ r) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = b[i] - row_fma_sum(rp, ci, v, x, i);
}

// `sweeps` l1-Jacobi sweeps from L.x (ping-pong with L.r; the result is left in L.x).
template <class T>
void l1_sweeps(Ctx& c, Level<T>& L, const T* b, int sweeps) {
  const T w = (T)c.cfg.smootherWeight;
  for (int it = 0; it < sweeps; it++) {
    FG_LAUNCH_PDL(l1_sweep_kernel<T>, grid_for(L.n, 256), 256, 0, c.stream, L.n, L.Ap.rp.p, L.Ap.ci.p, L.Ap.v.p, b,
              L.l1inv.p, w, L.x.p, L.r.p);
    std::swap(L.x.p, L.r.p);
  }
}

// Coarse visits of a cycle of type `type` (cycleType: 0 V, 1 W, 2 F) from a non-coarsest
// level: the first visit is a V-cycle for V and a W-cycle otherwise; W- and F-cycles visit
// a non-coarsest next level a second time (W: a W-cycle, F: a V-cycle), the visit pattern
// of the reference's W_Cycle / F_Cycle classes (cycles/wcycle.h, cycles/fcycle.h; its
// AMG_Level::cycle, amg_level.cu:51, always recurses with V_CYCLE and never reaches them).
// The second visit corrects the first: xc += cycle(bc - A_c xc), the residual formed with
// the coarse level's permuted operator (the oracle forms it the same way).
inline int cycle_first_visit(int type) { return type == 0 ? 0 : 1; }
inline int cycle_second_visit(int type) { return type == 1 ? 1 : 0; }

// b (level order for l > 0, already permuted for l == 0) -> x (same ordering).  At
// level 0 with z_out != nullptr the result goes to z_out in FP64 instead of x_out;
// with r64 != nullptr, b_in is first rounded from the FP64 vector r64 (by the
// pre-smoother when it can, which also writes the rounded copy to b_in).
template <class T>
void vcycle(Ctx& c, Hierarchy<T>& H, int l, T* b_in, T* x_out, double* z_out = nullptr,
            const double* r64 = nullptr, int type = 0) {
  cudaStream_t s = c.stream;
  Level<T>& L = *H.L[l];
  const int n = L.A.n;
  const PdlScope pdl_scope(n <= kPdlLevelRows);
  if (L.coarsest) {
    FG_LAUNCH_PDL(coarse_solve_kernel<T>, grid_for((int64_t)n * 32, 256), 256, 0, s, n, L.Ainv.p, b_in, x_out);
    stage_mark(c, "coarse", l);
    return;
  }
  const T* b = b_in;  // already in this level's order (the parent's restriction writes it so)
  const bool l1 = c.cfg.smoother == 1;
  if (l1) {
    // l1-Jacobi from x = 0, then r = b - A x
    if (r64) FG_LAUNCH_PDL(cast_in_kernel<T>, grid_for(n, 256), 256, 0, s, n, r64, b_in);
    if (c.cfg.preInnerIters > 0) {
      FG_LAUNCH_PDL(l1_first_sweep_kernel<T>, grid_for(n, 256), 256, 0, s, n, b, L.l1inv.p, (T)c.cfg.smootherWeight,
                L.x.p);
      l1_sweeps(c, L, b, c.cfg.preInnerIters - 1);
    } else {
      FG_CUDA(cudaMemsetAsync(L.x.p, 0, (size_t)n * sizeof(T), s));
    }
    FG_LAUNCH_PDL(full_residual_kernel<T>, grid_for(n, 256), 256, 0, s, n, L.Ap.rp.p, L.Ap.ci.p, L.Ap.v.p, b, L.x.p,
              L.r.p);
    stage_mark(c, "pre", l);
  } else {
    smooth<T>(c, L, false, b, nullptr, L.x.p, L.r.p, r64, b_in);
    stage_mark(c, "pre", l);
    aout_residual<T>(s, L, L.x.p, L.r.p);
    stage_mark(c, "residual", l);
  }
  // next level: input in its t (or b when coarsest), output in its xo (or x)
  Level<T>& N = *H.L[l + 1];
  T* bc = N.coarsest ? N.b.p : N.t.p;
  T* xc = N.coarsest ? N.x.p : N.xo.p;
  spmv_lanes(L.R, L.r.p, bc, 0, s);
  stage_mark(c, "restrict", l);
  vcycle(c, H, l + 1, bc, xc, nullptr, nullptr, cycle_first_visit(type));
  if (type != 0 && !N.coarsest) {
    FG_REQUIRE(N.wr.n == (size_t)N.n && N.wd.n == (size_t)N.n, FEMGPU_ERR_INVALID, "cycle work vectors missing");
    FG_LAUNCH_PDL(residual_rows_kernel<T>, grid_for(N.n, 256), 256, 0, s, N.n, N.Ap.rp.p, N.Ap.ci.p, N.Ap.v.p, bc, xc,
              N.wr.p);
    vcycle(c, H, l + 1, N.wr.p, N.wd.p, nullptr, nullptr, cycle_second_visit(type));
    FG_LAUNCH_PDL(add_into_kernel<T>, grid_for(N.n, 256), 256, 0, s, N.n, N.wd.p, xc);
  }
  spmv_lanes(L.P, xc, L.x.p, 1, s);
  stage_mark(c, "prolong", l);
  bool z_done = false, out_done = false;
  if (l1) {
    for (int rl = 0; rl < c.cfg.postRelaxes; rl++) l1_sweeps(c, L, b, c.cfg.postInnerIters);
  }
  for (int rl = 0; rl < (l1 ? 0 : c.cfg.postRelaxes); rl++) {
    const bool last = rl + 1 == c.cfg.postRelaxes;
    // the last post relax of level 0 writes z itself; of a coarser level, x_out (this
    // level's order, which the parent's prolongation reads)
    double* z64 = (l == 0 && z_out && last) ? z_out : nullptr;
    T* dst = (l > 0 && last) ? x_out : L.r.p;
    smooth<T>(c, L, true, b, L.x.p, dst, nullptr, nullptr, nullptr, z64);
    if (dst == L.r.p) std::swap(L.x.p, L.r.p);  // r is free after the restriction: the ping-pong buffer
    z_done = z64 != nullptr;
    out_done = dst == x_out;
  }
  stage_mark(c, "post", l);
  if (l > 0) {
    if (!out_done) FG_CUDA(cudaMemcpyAsync(x_out, L.x.p, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  } else if (z_out) {
    if (!z_done) FG_LAUNCH_PDL(cast_out_kernel<T>, grid_for(n, 256), 256, 0, s, n, L.x.p, z_out);
  } else {
    FG_CUDA(cudaMemcpyAsync(x_out, L.x.p, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
  }
  stage_mark(c, "output", l);
}

// z = M r on permuted level-0 FP64 vectors.
template <class T>
void precondition(Ctx& c, Hierarchy<T>& H, const double* r, double* z) {
  cudaStream_t s = c.stream;
  Level<T>& L = *H.L[0];
  const int n = L.A.n;
  T* b = L.coarsest ? L.b.p : L.t.p;
  T* x = L.coarsest ? L.x.p : L.xo.p;
  if (L.coarsest) {
    FG_LAUNCH_PDL(cast_in_kernel<T>, grid_for(n, 256), 256, 0, s, n, r, b);
    vcycle(c, H, 0, b, x);
    FG_LAUNCH_PDL(cast_out_kernel<T>, grid_for(n, 256), 256, 0, s, n, x, z);
  } else {
    vcycle(c, H, 0, b, x, z, r, c.cfg.cycleType);  // level 0 reads r and writes z itself
  }
}

void precondition_any(Ctx& c, const double* r, double* z) {
  if (c.cfg.precision == 1) precondition(c, static_cast<Hierarchy<double>&>(*c.H), r, z);
  else precondition(c, static_cast<Hierarchy<float>&>(*c.H), r, z);
}

// Work vectors of the second coarse visits of W- and F-cycles and the l1-Jacobi scaling
// (allocated before any capture).
template <class T>
void ensure_cycle_work(Ctx& c, Hierarchy<T>& H) {
  if (c.cfg.smoother == 1)
    for (int l = 0; l < H.num_levels; l++) {
      Level<T>& L = *H.L[l];
      if (L.coarsest || L.l1inv.n == (size_t)L.n) continue;
      L.l1inv.alloc(L.n, c.stream);
      FG_LAUNCH(l1_inverse_kernel<T>, grid_for(L.n, 256), 256, 0, c.stream, L.n, L.Ap.rp.p, L.Ap.v.p, L.l1inv.p);
    }
  if (c.cfg.cycleType == 0) return;
  for (int l = 1; l < H.num_levels; l++) {
    Level<T>& L = *H.L[l];
    if (L.coarsest || L.wr.n == (size_t)L.n) continue;
    L.wr.alloc(L.n, c.stream);
    L.wd.alloc(L.n, c.stream);
  }
}

void ensure_work(Ctx& c, int n) {
  cudaStream_t s = c.stream;
  if (c.H) {
    if (c.cfg.precision == 1) ensure_cycle_work(c, static_cast<Hierarchy<double>&>(*c.H));
    else ensure_cycle_work(c, static_cast<Hierarchy<float>&>(*c.H));
  }
  if (c.vb.n != (size_t)n) {
    c.vb.alloc(n, s);
    c.vx.alloc(n, s);
    c.vr.alloc(n, s);
    c.vz.alloc(n, s);
    c.vp.alloc(n, s);
    c.vy.alloc(n, s);
    c.vrold.alloc(n, s);
  }
  if (c.red.n == 0) {
    c.red.alloc(2 * kRedBlocks + 64, s);
    c.red.zero();
    c.rcount.alloc(8, s);
    c.rcount.zero();
  }
  if (!c.h_scalars) FG_CUDA(cudaMallocHost((void**)&c.h_scalars, 64 * sizeof(double)));
}

// The error slot holds 1 + the group whose staged copy a register-smoother CTA gave up on.
std::string copy_wait_message(double v) {
  return "smoother copy wait ran out (group " + std::to_string((long long)v - 1) + ")";
}

// Fails when a smoother CTA gave up waiting for its bulk copies (waits on the stream).
void check_kernel_error(Ctx& c) {
  double v = 0.0;
  FG_CUDA(cudaMemcpyAsync(&v, c.red.p + 2 * kRedBlocks + S_KERR, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  FG_CUDA(cudaStreamSynchronize(c.stream));
  FG_REQUIRE(v == 0.0, FEMGPU_ERR_LIMIT, copy_wait_message(v));
}

}  // namespace

// The register-resident cluster smoother with C CTAs per group: sets the plan and returns
// true when both its pre and post kernels have a resident configuration.
template <class T>
bool creg_plan(Ctx& c, Level<T>& L, int S, int K, int C) {
  const int mcap = L.max_group_rows;
  const int scap = (mcap + C - 1) / C;
  const int thr = (int)std::max<int64_t>(32, ((int64_t)scap * S + 31) / 32 * 32);
  if (thr > 1024) return false;
  const size_t sm = 2 * (size_t)(mcap + 1) * sizeof(T);
  for (int post = 0; post < 2; post++) {
    CregSmoothFn<T> k = pick_creg_kernel<T>(post != 0, S, K);
    if (sm > 48 * 1024) ensure_smem(k, sm);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(L.ngroups * C));
    cfg.blockDim = dim3((unsigned)thr);
    cfg.dynamicSmemBytes = sm;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, k, &cfg);
    if (e != cudaSuccess) (void)cudaGetLastError();
    if (e != cudaSuccess || clusters <= 0) return false;
  }
  L.smooth_lanes = S;
  L.smooth_k = K;
  L.cluster = C;
  L.slice_rows = scap;
  L.slice_ents = 0;
  L.smooth_staged = false;
  L.smooth_smem = sm;
  L.smooth_threads = thr;
  return true;
}

template <class T>
void plan_smoother(Ctx& c, Level<T>& L) {
  cudaStream_t s = c.stream;
  if (smoother_in_registers(L.max_in_row, L.max_part_rows)) {
    L.smooth_lanes = 1;
    L.cluster = 1;
    L.smooth_threads = std::max(32, ((L.max_group_rows + 31) / 32) * 32);
    L.smooth_smem = reg_smem_layout<T>(L.max_group_ents + 16).total;
    FG_REQUIRE(L.smooth_smem <= kSmemOptIn, FEMGPU_ERR_LIMIT, "register smoother staging exceeds shared memory");
    int per_sm = 0;
    for (int post = 0; post < 2; post++) {
      auto k = post ? smooth_reg_kernel<T, true, kRegRow> : smooth_reg_kernel<T, false, kRegRow>;
      if (L.smooth_smem > 48 * 1024)
        ensure_smem(k, L.smooth_smem);
      int nb = 0;
      FG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, L.smooth_threads, L.smooth_smem));
      per_sm = post ? std::min(per_sm, nb) : nb;
    }
    FG_REQUIRE(per_sm > 0, FEMGPU_ERR_LIMIT, "no resident configuration for the register smoother");
    int sms = 0;
    FG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
    L.smooth_grid = (int)std::min<int64_t>(L.ngroups, (int64_t)per_sm * sms);
    return;
  }
  const int S = smooth_lanes_for(L.n, L.Ain.nnz, L.max_in_row);
  const int mcap = L.max_group_rows;
  L.smooth_lanes = S;
  L.smooth_k = 0;
  // register-resident entries: at most 16 per lane, one row slice per CTA of <= 1024
  // threads, 16-bit group-local columns
  const int per_lane = (L.max_in_row + S - 1) / S;
  const int rows_per_cta = 1024 / S;
  const int creg_c = (mcap + rows_per_cta - 1) / rows_per_cta;
  if (per_lane <= kLaneEntries && creg_c <= kMaxCluster && mcap < 65535) {
    const int K = per_lane <= 8 ? 8 : 16;
    for (int C = std::max(1, creg_c); C <= kMaxCluster; C++)
      if (creg_plan(c, L, S, K, C)) return;
  }
  int C = (int)std::min<int64_t>(kMaxCluster, ((int64_t)mcap * S + 1023) / 1024);
  if (C < 1) C = 1;
  for (;; C--) {
    DBuf<int32_t> sent((size_t)L.ngroups * C, s);
    FG_LAUNCH(slice_entries_kernel, grid_for((int64_t)L.ngroups * C, 256), 256, 0, s, L.ngroups, C, L.grows.p,
              L.Ain.rp.p, sent.p);
    const int scap = (mcap + C - 1) / C;
    const int ecap = reduce_max(sent.p, (int64_t)L.ngroups * C, s);
    const bool st = mcap < 65536 && slice_smem_bytes<T>(mcap, scap, ecap) <= kStageLimit;
    const size_t sm = slice_smem_bytes<T>(mcap, scap, st ? ecap : 0);
    FG_REQUIRE(sm <= kSmemOptIn, FEMGPU_ERR_LIMIT, "partition too large for the shared-memory smoother");
    const int64_t want = ((int64_t)scap * S + 31) / 32 * 32;
    const int thr = (int)std::max<int64_t>(32, std::min<int64_t>(1024, want));
    bool fits = true;
    for (int post = 0; post < 2 && fits; post++) {
      ClusterSmoothFn<T> k = pick_cluster_kernel<T>(post != 0, st, S);
      if (sm > 48 * 1024) ensure_smem(k, sm);
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)(L.ngroups * C));
      cfg.blockDim = dim3((unsigned)thr);
      cfg.dynamicSmemBytes = sm;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)C;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int clusters = 0;
      const cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, k, &cfg);
      if (e != cudaSuccess) (void)cudaGetLastError();
      fits = e == cudaSuccess && clusters > 0;
    }
    if (fits || C == 1) {
      FG_REQUIRE(fits, FEMGPU_ERR_LIMIT, "no resident configuration for the shared-memory smoother");
      L.cluster = C;
      L.slice_rows = scap;
      L.slice_ents = ecap;
      L.smooth_staged = st;
      L.smooth_smem = sm;
      L.smooth_threads = thr;
      return;
    }
  }
}

template void plan_smoother<float>(Ctx&, Level<float>&);
template void plan_smoother<double>(Ctx&, Level<double>&);

// ---- autotuner ---------------------------------------------------------------------------
// Launch shapes that do not change any result are picked per level by timing the level's
// own kernels once: the lanes per row of the cross-partition products (every lane count
// adds the products in entry order), and the CTAs per cluster of the register-resident
// cluster smoother (a row's sums never cross CTAs).  Choices are cached per device and
// level shape for the life of the process, and in the file named by FEMGPU_TUNE_CACHE
// when it is set (one "key value" per line).
namespace {

std::mutex g_tune_mu;
std::map<std::string, int>* g_tune = nullptr;
bool g_tune_loaded = false;

std::string tune_path() {
  const char* p = getenv("FEMGPU_TUNE_CACHE");
  return p ? std::string(p) : std::string();
}

bool tune_lookup(const std::string& key, int* value) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (!g_tune) g_tune = new std::map<std::string, int>();
  if (!g_tune_loaded) {
    g_tune_loaded = true;
    const std::string path = tune_path();
    if (!path.empty()) {
      if (FILE* f = fopen(path.c_str(), "r")) {
        char k[512];
        int v = 0;
        while (fscanf(f, "%511s %d", k, &v) == 2) (*g_tune)[k] = v;
        fclose(f);
      }
    }
  }
  auto it = g_tune->find(key);
  if (it == g_tune->end()) return false;
  *value = it->second;
  return true;
}

void tune_store(const std::string& key, int value) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (!g_tune) g_tune = new std::map<std::string, int>();
  (*g_tune)[key] = value;
  const std::string path = tune_path();
  if (!path.empty())
    if (FILE* f = fopen(path.c_str(), "a")) {
      fprintf(f, "%s %d\n", key.c_str(), value);
      fclose(f);
    }
}

std::string device_tag(int device) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
    (void)cudaGetLastError();
    return "dev";
  }
  std::string n = p.name;
  for (char& ch : n)
    if (ch == ' ') ch = '_';
  return n + "_sm" + std::to_string(p.multiProcessorCount);
}

// average time of `reps` launches of fn (after one untimed launch)
template <class F>
float time_launches(cudaStream_t s, F&& fn, int reps = 3) {
  fn();
  cudaEvent_t e0, e1;
  FG_CUDA(cudaEventCreate(&e0));
  FG_CUDA(cudaEventCreate(&e1));
  FG_CUDA(cudaEventRecord(e0, s));
  for (int i = 0; i < reps; i++) fn();
  FG_CUDA(cudaEventRecord(e1, s));
  FG_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  FG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

}  // namespace

template <class T>
void autotune_level(Ctx& c, Level<T>& L) {
  if (!c.cfg.autotune || L.coarsest || L.n == 0) return;
  cudaStream_t s = c.stream;
  const std::string dev = device_tag(c.device);
  const std::string shape = std::to_string(sizeof(T)) + "_" + std::to_string(L.n) + "_" + std::to_string(L.Ain.nnz) +
                            "_" + std::to_string(L.Aout.nnz) + "_" + std::to_string(L.max_group_rows);
  const bool verbose = getenv("FEMGPU_PROFILE") != nullptr;
  // inputs of the timed launches: finite values in the level's work vectors
  FG_CUDA(cudaMemsetAsync(L.x.p, 0, L.x.n * sizeof(T), s));
  FG_CUDA(cudaMemsetAsync(L.r.p, 0, L.r.n * sizeof(T), s));
  FG_CUDA(cudaMemsetAsync(L.b.p, 0, L.b.n * sizeof(T), s));
  // cross-partition lanes
  if (L.Aout.nnz > 0) {
    const std::string key = dev + "|aout|" + shape;
    int best = 0;
    if (!tune_lookup(key, &best)) {
      float tbest = 1e30f;
      for (int S = 1; S <= 32; S <<= 1) {
        L.aout_lanes_tuned = S;
        const float t = time_launches(s, [&] { aout_residual<T>(s, L, L.x.p, L.r.p); });
        if (t < tbest) {
          tbest = t;
          best = S;
        }
      }
      tune_store(key, best);
    }
    L.aout_lanes_tuned = best;
    if (verbose) fprintf(stderr, "[femgpu tune] level n=%d cross-partition lanes %d\n", L.n, best);
  }
  // CTAs per cluster of the register-resident cluster smoother
  if (!smoother_in_registers(L.max_in_row, L.max_part_rows) && L.smooth_k > 0) {
    const std::string key = dev + "|creg|" + shape;
    const int S = L.smooth_lanes, K = L.smooth_k, C0 = L.cluster;
    int best = 0;
    if (!tune_lookup(key, &best)) {
      float tbest = 1e30f;
      for (int C = C0; C <= kMaxCluster; C++) {
        if (!creg_plan(c, L, S, K, C)) continue;
        const float t = time_launches(s, [&] { smooth_sweeps<T>(c, L, false, L.b.p, nullptr, L.x.p, L.r.p); });
        if (t < tbest) {
          tbest = t;
          best = C;
        }
      }
      tune_store(key, best);
    }
    if (best < C0 || !creg_plan(c, L, S, K, best))
      FG_REQUIRE(creg_plan(c, L, S, K, C0), FEMGPU_ERR_LIMIT, "no resident configuration for the cluster smoother");
    if (verbose) fprintf(stderr, "[femgpu tune] level n=%d cluster smoother CTAs per group %d\n", L.n, L.cluster);
  }
}

template void autotune_level<float>(Ctx&, Level<float>&);
template void autotune_level<double>(Ctx&, Level<double>&);

void spmv_original(Ctx& c, const double* d_x, double* d_y) {
  FG_REQUIRE(c.has_matrix, FEMGPU_ERR_NOT_READY, "no operator");
  cudaStream_t s = c.stream;
  FG_LAUNCH(spmv_kernel, grid_for(c.A.n, 256), 256, 0, s, c.A.n, c.A.rp.p, c.A.ci.p, c.A.v.p, d_x, d_y);
}

void amg_vcycle_device(Ctx& c, const double* d_r, double* d_z) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  const int n = c.A.n;
  cudaStream_t s = c.stream;
  ensure_work(c, n);
  std::vector<std::pair<std::string, cudaEvent_t>> marks;
  if (getenv("FEMGPU_PROFILE")) c.stage_marks = &marks;
  try {
    FG_LAUNCH(perm_vec_in_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, d_r, c.vr.p);
    stage_mark(c, "start", 0);
    precondition_any(c, c.vr.p, c.vz.p);
    FG_LAUNCH(perm_vec_out_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.vz.p, d_z);
  } catch (...) {
    c.stage_marks = nullptr;
    for (auto& m : marks) cudaEventDestroy(m.second);
    throw;
  }
  c.stage_marks = nullptr;
  if (!marks.empty()) {
    FG_CUDA(cudaEventSynchronize(marks.back().second));
    for (size_t i = 1; i < marks.size(); i++) {
      float ms = 0;
      cudaEventElapsedTime(&ms, marks[i - 1].second, marks[i].second);
      fprintf(stderr, "[femgpu vcycle] %-14s %8.1f us\n", marks[i].first.c_str(), ms * 1000.0f);
    }
    for (auto& m : marks) cudaEventDestroy(m.second);
  }
  check_kernel_error(c);
}

namespace {

// One PCG iteration after the residual check: z = M r, beta, p = z + beta p,
// y = A p, alpha, x += alpha p, r -= alpha y, ||r||^2, scalars to the host.
// y = A0p p with p.y and alpha.
void launch_spmv_dot(Ctx& c, int n, const double* p, double* y) {
  const DCsr<double>& A = c.A0p;
  if (c.sliced)
    FG_LAUNCH_PDL(spmv_dot_sliced_kernel, kRedBlocks, kRedThreads, 0, c.stream, n, c.s_off.p, c.s_ci.p, c.s_v.p, p, y,
              c.red.p, c.red.p + 2 * kRedBlocks, c.rcount.p + 1);
  else
    FG_LAUNCH_PDL(spmv_dot_kernel, kRedBlocks, kRedThreads, 0, c.stream, n, A.rp.p, A.ci.p, A.v.p, p, y, c.red.p,
              c.red.p + 2 * kRedBlocks, c.rcount.p + 1);
}

// y = A0p x.
void launch_spmv_a0(Ctx& c, int n, const double* x, double* y) {
  const DCsr<double>& A = c.A0p;
  if (c.sliced)
    FG_LAUNCH(spmv_sliced_kernel, grid_for(n, 256), 256, 0, c.stream, n, c.s_off.p, c.s_ci.p, c.s_v.p, x, y);
  else
    FG_LAUNCH(spmv_kernel, grid_for(n, 256), 256, 0, c.stream, n, A.rp.p, A.ci.p, A.v.p, x, y);
}

void pcg_iteration_body(Ctx& c, int n, int flexible, bool to_host) {
  cudaStream_t s = c.stream;
  double* part = c.red.p;
  double* part2 = c.red.p + kRedBlocks;
  double* sc = c.red.p + 2 * kRedBlocks;
  unsigned* cnt = c.rcount.p;
  Ctx::ZDot zd;
  zd.r = c.vr.p;
  zd.rold = flexible ? c.vrold.p : nullptr;
  zd.part = part;
  c.zdot = &zd;
  try {
    precondition_any(c, c.vr.p, c.vz.p);
  } catch (...) {
    c.zdot = nullptr;
    throw;
  }
  c.zdot = nullptr;
  if (!zd.done)  // else z.r (z.r_old) and beta came from the smoother that wrote z
    FG_LAUNCH_PDL(dot_beta_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vz.p, c.vr.p, flexible ? c.vrold.p : nullptr,
              part, part2, sc, flexible, cnt);
  FG_LAUNCH_PDL(pupdate_kernel, kRedBlocks, kRedThreads, 0, s, n, sc, c.vz.p, c.vp.p);
  launch_spmv_dot(c, n, c.vp.p, c.vy.p);
  FG_LAUNCH_PDL(update_kernel, kRedBlocks, kRedThreads, 0, s, n, sc, c.vp.p, c.vy.p, c.vx.p, c.vr.p,
            flexible ? c.vrold.p : nullptr, part, cnt + 2);
  if (to_host) FG_CUDA(cudaMemcpyAsync(c.h_scalars, sc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
}

// Captures the whole PCG loop once per hierarchy as a CUDA graph: a conditional while
// node whose body is one iteration followed by pcg_check_kernel, so the iterations
// run back to back on the device with no host round trip.
// Adds to `g` a while node on `loop` after `deps` and captures its body on c.stream: one
// PCG iteration followed by pcg_check_kernel.  Returns the node, or null when a graph call
// or the capture failed (the capture is ended either way).
cudaGraphNode_t add_pcg_loop(Ctx& c, int n, int flexible, cudaGraph_t g, cudaGraphConditionalHandle loop,
                             const cudaGraphNode_t* deps, size_t ndeps) {
  cudaStream_t s = c.stream;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = loop;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp) != cudaSuccess) return nullptr;
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return nullptr;
  try {
    pcg_iteration_body(c, n, flexible, false);
    FG_LAUNCH_PDL(pcg_check_kernel, 1, 1, 0, s, c.red.p + 2 * kRedBlocks, loop);
  } catch (...) {
    cudaGraph_t dummy = nullptr;
    cudaStreamEndCapture(s, &dummy);
    return nullptr;
  }
  cudaGraph_t captured = nullptr;
  if (cudaStreamEndCapture(s, &captured) != cudaSuccess) return nullptr;
  return node;
}

bool capture_iteration(Ctx& c, int n, int flexible) {
  if (c.pcg_exec && c.graph_gen == c.hier_gen && c.graph_flexible == flexible) return true;
  if (c.pcg_exec) {
    cudaGraphExecDestroy(c.pcg_exec);
    c.pcg_exec = nullptr;
  }
  int64_t before = g_kernel_launches.load();
  cudaGraph_t g = nullptr;
  // a failed capture leaves the solve on the host-driven loop (same kernels); with
  // FEMGPU_PROFILE the reason is printed
  auto fail = [&](const char* where) {
    const cudaError_t err = cudaGetLastError();
    if (getenv("FEMGPU_PROFILE"))
      fprintf(stderr, "[femgpu] PCG graph not used (%s: %s)\n", where, cudaGetErrorString(err));
    if (g) cudaGraphDestroy(g);
    g_kernel_launches.store(before);
    return false;
  };
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return fail("create");
  cudaGraphConditionalHandle loop;
  if (cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault) != cudaSuccess)
    return fail("conditional handle");
  if (!add_pcg_loop(c, n, flexible, g, loop, nullptr, 0)) return fail("capture");
  cudaError_t e = cudaGraphInstantiate(&c.pcg_exec, g, 0);
  cudaGraphDestroy(g);
  g = nullptr;
  if (e != cudaSuccess) {
    c.pcg_exec = nullptr;
    return fail("instantiate");
  }
  c.graph_nodes = g_kernel_launches.load() - before;  // kernels of one iteration
  g_kernel_launches.store(before);  // counted per iteration after each solve
  c.graph_gen = c.hier_gen;
  c.graph_flexible = flexible;
  return true;
}


}  // namespace

SolveResult amg_solve_device(Ctx& c, const double* d_b, double* d_x) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  const int n = c.A.n;
  cudaStream_t s = c.stream;
  ensure_work(c, n);
  SolveResult res;
  double* part = c.red.p;
  double* sc = c.red.p + 2 * kRedBlocks;
  FG_LAUNCH(perm_vec_in_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, d_b, c.vb.p);
  FG_LAUNCH(perm_vec_in_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, d_x, c.vx.p);
  if (c.cfg.solverType == 0) {
    // AMG_SOLVER: one V-cycle applied to b (amg.cu:150-160); x is overwritten
    precondition_any(c, c.vb.p, c.vx.p);
    FG_LAUNCH(perm_vec_out_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.vx.p, d_x);
    launch_spmv_a0(c, n, c.vx.p, c.vy.p);
    FG_LAUNCH(residual_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vy.p, c.vr.p, part);
    FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_NR);
    FG_LAUNCH(dot_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vb.p, nullptr, part, nullptr);
    FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_BN);
    FG_CUDA(cudaMemcpyAsync(c.h_scalars, sc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    double bn = sqrt(c.h_scalars[S_BN]);
    res.relres = sqrt(c.h_scalars[S_NR]) / (bn > 0 ? bn : 1.0);
    res.iterations = 1;
    return res;
  }
  const int flexible = c.cfg.flexibleCG;
  FG_LAUNCH(dot_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vb.p, nullptr, part, nullptr);
  FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_BN);
  launch_spmv_a0(c, n, c.vx.p, c.vy.p);
  FG_LAUNCH(residual_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vy.p, c.vr.p, part);
  FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_NR);
  FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_FLAG, 0.0);
  FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_FIRST, 1.0);
  FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_KERR, 0.0);
  // last-block tickets start at zero (a CTA that gave up on a copy leaves its ticket unset)
  FG_CUDA(cudaMemsetAsync(c.rcount.p, 0, c.rcount.n * sizeof(unsigned), s));
  FG_CUDA(cudaMemsetAsync(c.vp.p, 0, n * sizeof(double), s));
  FG_CUDA(cudaMemcpyAsync(c.h_scalars, sc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  double bnorm = sqrt(c.h_scalars[S_BN]);
  if (bnorm == 0.0) bnorm = 1.0;
  double nr = sqrt(c.h_scalars[S_NR]);
  const double tol = c.cfg.tolerance;
  int it = 0;
  res.status = FEMGPU_ERR_NOT_CONVERGED;
  if (nr / bnorm <= tol) {
    res.status = FEMGPU_OK;
  } else {
    // FEMGPU_HOST_LOOP selects the host-driven loop (same kernels, one launch each),
    // which profilers can list kernel by kernel
    const bool graph = c.cfg.maxIters > 0 && !getenv("FEMGPU_HOST_LOOP") && capture_iteration(c, n, flexible);
    if (graph) {
      // the device runs the iterations until pcg_check_kernel stops the loop
      FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_IT, 0.0);
      FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_BNORM, bnorm);
      FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_TOL, tol);
      FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_MAXIT, (double)c.cfg.maxIters);
      FG_CUDA(cudaGraphLaunch(c.pcg_exec, s));
      FG_CUDA(cudaMemcpyAsync(c.h_scalars, sc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaStreamSynchronize(s));
      it = (int)c.h_scalars[S_IT];
      g_kernel_launches.fetch_add(c.graph_nodes * it);
      nr = sqrt(c.h_scalars[S_NR]);
      FG_REQUIRE(c.h_scalars[S_KERR] == 0.0, FEMGPU_ERR_LIMIT, copy_wait_message(c.h_scalars[S_KERR]));
      if (c.h_scalars[S_FLAG] != 0.0 || !std::isfinite(nr)) res.status = FEMGPU_ERR_BREAKDOWN;
      else if (nr / bnorm <= tol) res.status = FEMGPU_OK;
    } else {
      while (it < c.cfg.maxIters) {
        pcg_iteration_body(c, n, flexible, true);
        FG_CUDA(cudaStreamSynchronize(s));
        it++;
        nr = sqrt(c.h_scalars[S_NR]);
        FG_REQUIRE(c.h_scalars[S_KERR] == 0.0, FEMGPU_ERR_LIMIT, copy_wait_message(c.h_scalars[S_KERR]));
        if (c.h_scalars[S_FLAG] != 0.0 || !std::isfinite(nr)) {
          res.status = FEMGPU_ERR_BREAKDOWN;
          break;
        }
        if (nr / bnorm <= tol) {
          res.status = FEMGPU_OK;
          break;
        }
      }
    }
  }
  FG_LAUNCH(perm_vec_out_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.vx.p, d_x);
  res.iterations = it;
  res.relres = nr / bnorm;
  return res;
}

// ---- the PCG solves of many meshes in one graph launch --------------------------------
namespace {

// Start of a batch branch's loop: b's norm (1 when b = 0) to S_BNORM, and the loop runs only
// when the initial residual is above the tolerance (the host check of amg_solve_device).
__global__ void batch_init_kernel(double* sc, cudaGraphConditionalHandle loop) {
  double bn = sqrt(sc[S_BN]);
  if (bn == 0.0) bn = 1.0;
  sc[S_BNORM] = bn;
  cudaGraphSetConditional(loop, sqrt(sc[S_NR]) / bn <= sc[S_TOL] ? 0u : 1u);
}

struct BatchGraph {
  std::vector<Ctx*> hs;
  std::vector<uint64_t> gens;         // each handle's hierarchy generation when captured
  std::vector<int64_t> body_kernels;  // kernels of one iteration of each mesh's loop
  int64_t fixed_kernels = 0;          // kernels outside the loops
  cudaGraphExec_t exec = nullptr;
  ~BatchGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

std::mutex g_batch_mu;
std::deque<std::unique_ptr<BatchGraph>> g_batch;  // most recently used first
constexpr size_t kBatchGraphsKept = 4;

// One independent branch per mesh: the kernels amg_solve_device runs before its loop (b and
// x read from c.bat_b and c.bat_x), the PCG while loop, then x back to c.bat_x and the
// scalars to the pinned host mirror.  Each branch is captured on its handle's stream into
// g in three parts, since a loop body is captured on the same stream.
bool add_batch_branch(Ctx& c, cudaGraph_t g, int64_t* body_kernels, int64_t* fixed_kernels) {
  const int n = c.A.n;
  cudaStream_t s = c.stream;
  double* part = c.red.p;
  double* sc = c.red.p + 2 * kRedBlocks;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaGraphConditionalHandle loop;
  if (cudaGraphConditionalHandleCreate(&loop, g, 0, 0) != cudaSuccess) return false;
  const int64_t k0 = g_kernel_launches.load();
  std::vector<cudaGraphNode_t> leaves;
  cudaGraph_t gg = nullptr;
  if (cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, mode) != cudaSuccess) return false;
  bool ok = true;
  try {
    FG_LAUNCH(perm_vec_in_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.bat_b.p, c.vb.p);
    FG_LAUNCH(perm_vec_in_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.bat_x.p, c.vx.p);
    FG_LAUNCH(dot_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vb.p, nullptr, part, nullptr);
    FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_BN);
    launch_spmv_a0(c, n, c.vx.p, c.vy.p);
    FG_LAUNCH(residual_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vb.p, c.vy.p, c.vr.p, part);
    FG_LAUNCH(finalize_kernel, 1, 1024, 0, s, part, kRedBlocks, sc + S_NR);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_FLAG, 0.0);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_FIRST, 1.0);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_KERR, 0.0);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_IT, 0.0);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_TOL, c.cfg.tolerance);
    FG_LAUNCH(set_slot_kernel, 1, 1, 0, s, sc, S_MAXIT, (double)c.cfg.maxIters);
    FG_CUDA(cudaMemsetAsync(c.rcount.p, 0, c.rcount.n * sizeof(unsigned), s));
    FG_CUDA(cudaMemsetAsync(c.vp.p, 0, n * sizeof(double), s));
    FG_LAUNCH(batch_init_kernel, 1, 1, 0, s, sc, loop);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* d = nullptr;
    size_t nd = 0;
    FG_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd));
    leaves.assign(d, d + nd);
  } catch (...) {
    ok = false;
  }
  if (cudaStreamEndCapture(s, &gg) != cudaSuccess || !ok) return false;
  const int64_t k1 = g_kernel_launches.load();
  cudaGraphNode_t ln = add_pcg_loop(c, n, c.cfg.flexibleCG, g, loop, leaves.data(), leaves.size());
  if (!ln) return false;
  const int64_t k2 = g_kernel_launches.load();
  if (cudaStreamBeginCaptureToGraph(s, g, &ln, nullptr, 1, mode) != cudaSuccess) return false;
  try {
    FG_LAUNCH(perm_vec_out_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, c.vx.p, c.bat_x.p);
    FG_CUDA(cudaMemcpyAsync(c.h_scalars, sc, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s));
  } catch (...) {
    ok = false;
  }
  if (cudaStreamEndCapture(s, &gg) != cudaSuccess || !ok) return false;
  *body_kernels = k2 - k1;
  *fixed_kernels += (k1 - k0) + (g_kernel_launches.load() - k2);
  return true;
}

}  // namespace

void batch_prepare(Ctx& c) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  const int n = c.A.n;
  ensure_work(c, n);
  if (c.bat_b.n != (size_t)n) {
    c.bat_b.alloc(n, c.stream);
    c.bat_x.alloc(n, c.stream);
  }
}

bool batch_solve_graph(const std::vector<Ctx*>& hs, std::vector<SolveResult>& res, float* ms) {
  if (hs.empty()) return true;
  cudaStream_t s = hs[0]->stream;
  std::lock_guard<std::mutex> lock(g_batch_mu);
  std::vector<uint64_t> gens(hs.size());
  for (size_t i = 0; i < hs.size(); i++) gens[i] = hs[i]->hier_gen;
  auto it = std::find_if(g_batch.begin(), g_batch.end(), [&](const std::unique_ptr<BatchGraph>& b) { return b->hs == hs; });
  std::unique_ptr<BatchGraph> bg;
  if (it != g_batch.end()) {
    bg = std::move(*it);
    g_batch.erase(it);
  }
  if (!bg || bg->gens != gens) {
    // capture the branches again (new hierarchies, new buffers); the executable graph is
    // updated in place when its topology is unchanged, else instantiated anew
    const int64_t before = g_kernel_launches.load();
    cudaGraph_t g = nullptr;
    std::vector<int64_t> body(hs.size(), 0);
    int64_t fixed = 0;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    for (size_t i = 0; ok && i < hs.size(); i++) ok = add_batch_branch(*hs[i], g, &body[i], &fixed);
    g_kernel_launches.store(before);
    if (ok && bg && bg->exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(bg->exec, g, &info) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(bg->exec);
        bg->exec = nullptr;
      }
    }
    if (ok && (!bg || !bg->exec)) {
      if (!bg) bg = std::make_unique<BatchGraph>();
      ok = cudaGraphInstantiate(&bg->exec, g, 0) == cudaSuccess;
      if (!ok) bg->exec = nullptr;
    }
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      (void)cudaGetLastError();
      return false;
    }
    bg->hs = hs;
    bg->gens = gens;
    bg->body_kernels = body;
    bg->fixed_kernels = fixed;
  }
  // the branches read what each handle's stream wrote (b, x, the hierarchy)
  cudaEvent_t e0, e1;
  FG_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDefault));
  FG_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDefault));
  for (Ctx* c : hs)
    if (c->stream != s) {
      cudaEvent_t w;
      FG_CUDA(cudaEventCreateWithFlags(&w, cudaEventDisableTiming));
      FG_CUDA(cudaEventRecord(w, c->stream));
      FG_CUDA(cudaStreamWaitEvent(s, w, 0));
      cudaEventDestroy(w);
    }
  FG_CUDA(cudaEventRecord(e0, s));
  FG_CUDA(cudaGraphLaunch(bg->exec, s));
  FG_CUDA(cudaEventRecord(e1, s));
  FG_CUDA(cudaEventSynchronize(e1));
  FG_CUDA(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  res.assign(hs.size(), SolveResult());
  int64_t kernels = bg->fixed_kernels;
  for (size_t i = 0; i < hs.size(); i++) {
    const double* h = hs[i]->h_scalars;
    SolveResult& r = res[i];
    r.iterations = (int)h[S_IT];
    const double nr = sqrt(h[S_NR]), bnorm = h[S_BNORM];
    r.relres = nr / bnorm;
    kernels += bg->body_kernels[i] * r.iterations;
    if (h[S_KERR] != 0.0) r.status = FEMGPU_ERR_LIMIT;
    else if (h[S_FLAG] != 0.0 || !std::isfinite(nr)) r.status = FEMGPU_ERR_BREAKDOWN;
    else if (r.relres <= hs[i]->cfg.tolerance) r.status = FEMGPU_OK;
    else r.status = FEMGPU_ERR_NOT_CONVERGED;
  }
  g_kernel_launches.fetch_add(kernels);
  g_batch.push_front(std::move(bg));
  while (g_batch.size() > kBatchGraphsKept) g_batch.pop_back();
  return true;
}

void batch_forget(Ctx* c) {
  std::lock_guard<std::mutex> lock(g_batch_mu);
  for (auto it = g_batch.begin(); it != g_batch.end();)
    if (std::find((*it)->hs.begin(), (*it)->hs.end(), c) != (*it)->hs.end()) it = g_batch.erase(it);
    else ++it;
}

namespace {

template <class T>
__global__ void fill_value_kernel(int64_t n, T* a, T v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

template <class T>
void profile_level0(Ctx& c, Hierarchy<T>& H, int which, int reps, double* ms, double* bytes) {
  cudaStream_t s = c.stream;
  Level<T>& L = *H.L[0];
  FG_REQUIRE(!L.coarsest, FEMGPU_ERR_INVALID, "level 0 is the coarsest level: no smoother to time");
  const int n = L.n;
  const double ts = sizeof(T);
  // well-defined inputs
  FG_LAUNCH(fill_value_kernel<T>, grid_for(n, 256), 256, 0, s, (int64_t)n, L.b.p, (T)1);
  FG_LAUNCH(fill_value_kernel<T>, grid_for(n, 256), 256, 0, s, (int64_t)n, L.x.p, (T)0.5);
  FG_LAUNCH(fill_value_kernel<T>, grid_for(n, 256), 256, 0, s, (int64_t)n, L.r.p, (T)0.25);
  FG_LAUNCH(fill_value_kernel<T>, grid_for(L.nagg, 256), 256, 0, s, (int64_t)L.nagg, L.t.p, (T)0.125);
  if (which == 5) {
    ensure_work(c, c.A.n);
    FG_LAUNCH(fill_value_kernel<double>, grid_for(n, 256), 256, 0, s, (int64_t)n, c.vr.p, 0.5);
    FG_LAUNCH(fill_value_kernel<double>, grid_for(n, 256), 256, 0, s, (int64_t)n, c.vrold.p, 0.25);
  }
  auto run = [&]() {
    switch (which) {
      case 1: smooth<T>(c, L, false, L.b.p, nullptr, L.x.p, L.r.p); break;
      case 2: smooth_sweeps<T>(c, L, true, L.bp.p, L.x.p, L.xo.p, nullptr); break;
      case 3: spmv_lanes(L.R, L.r.p, L.t.p, 0, s); break;
      case 5: {
        // the last post relax of a PCG iteration's V-cycle: b - A_out x, the sweeps, z
        // widened to FP64 and the z.r / z.r_old partials with beta from the last CTA
        Ctx::ZDot zd;
        zd.r = c.vr.p;
        zd.rold = c.vrold.p;
        zd.part = c.red.p;
        c.zdot = &zd;
        try {
          smooth<T>(c, L, true, L.b.p, L.x.p, L.xo.p, nullptr, nullptr, nullptr, c.vz.p);
        } catch (...) {
          c.zdot = nullptr;
          throw;
        }
        c.zdot = nullptr;
        if (!zd.done)
          FG_LAUNCH_PDL(dot_beta_kernel, kRedBlocks, kRedThreads, 0, s, n, c.vz.p, c.vr.p, c.vrold.p, c.red.p,
                    c.red.p + kRedBlocks, c.red.p + 2 * kRedBlocks, 1, c.rcount.p);
        break;
      }
      default: spmv_lanes(L.P, L.t.p, L.xo.p, 1, s); break;
    }
  };
  if (which == 2)  // the post relax's right-hand side, computed once outside the timing
    aout_rhs<T>(s, L, L.b.p, L.x.p, L.bp.p);
  // in-partition entries: value + 16-bit column on the register path (plus one byte per
  // row for its place in its block), value + 32-bit column otherwise
  const bool reg = smoother_in_registers(L.max_in_row, L.max_part_rows);
  const double ein = reg ? ts + 2 : ts + 4;
  const double rowb = reg ? 1.0 * n : 0.0;
  switch (which) {
    case 1:  // entries, row offsets, b, diag, 1/diag in; x, r out
      *bytes = L.Ain.nnz * ein + 4.0 * (n + 1) + 3 * ts * n + 2 * ts * n + rowb;
      break;
    case 2:  // entries, row offsets, b', diag, 1/diag, x in; x out
      *bytes = L.Ain.nnz * ein + 4.0 * (n + 1) + 4 * ts * n + ts * n + rowb;
      break;
    case 3:
      *bytes = L.R.nnz * (ts + 4) + 4.0 * (L.nagg + 1) + ts * n + ts * L.nagg;
      break;
    case 5:  // as case 2 plus A_out (entries, row offsets) for b - A_out x, z out in FP64, r and r_old in
      *bytes = L.Ain.nnz * ein + 4.0 * (n + 1) + 4 * ts * n + L.Aout.nnz * (ts + 4) + 4.0 * (n + 1) + 8.0 * n +
               16.0 * n + rowb;
      break;
    default:
      *bytes = L.P.nnz * (ts + 4) + 4.0 * (n + 1) + ts * L.nagg + 2 * ts * n;
      break;
  }
  for (int i = 0; i < 3; i++) run();
  cudaEvent_t e0, e1;
  FG_CUDA(cudaEventCreate(&e0));
  FG_CUDA(cudaEventCreate(&e1));
  FG_CUDA(cudaEventRecord(e0, s));
  for (int i = 0; i < reps; i++) run();
  FG_CUDA(cudaEventRecord(e1, s));
  FG_CUDA(cudaEventSynchronize(e1));
  float t = 0;
  FG_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / reps;
  check_kernel_error(c);
}

}  // namespace

// Times one hot kernel with CUDA events on the handle's stream (after 3 untimed
// launches) and reports its algorithmic bytes: 0 = the outer PCG's FP64 SpMV
// (CSR, fused dot), 1 = level-0 pre-smoother, 2 = level-0 post-smoother relax,
// 3 = level-0 restriction R r, 4 = level-0 prolongation x += P xc, 5 = the level-0
// post-smoother as a PCG iteration runs it (fused), 6 / 7 = the assembly's element and
// row-gather kernels.
void profile_kernel(Ctx& c, int which, int reps, double* ms, double* bytes) {
  FG_REQUIRE(reps > 0 && which >= 0 && which <= 7, FEMGPU_ERR_INVALID, "bad kernel selector");
  if (which == 6 || which == 7) {
    profile_assembly(c, which, reps, ms, bytes);
    return;
  }
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  cudaStream_t s = c.stream;
  if (which == 0) {
    const int n = c.A.n;
    ensure_work(c, n);
      FG_LAUNCH(fill_value_kernel<double>, grid_for(n, 256), 256, 0, s, (int64_t)n, c.vp.p, 1.0);
    auto run = [&]() {
      launch_spmv_dot(c, n, c.vp.p, c.vy.p);
    };
    for (int i = 0; i < 3; i++) run();
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    FG_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < reps; i++) run();
    FG_CUDA(cudaEventRecord(e1, s));
    FG_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    FG_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / reps;
    // entries (value + column), row (or slice) offsets, p read and y written
    *bytes = c.sliced ? 12.0 * c.A0p.nnz + 4.0 * ((n + 31) / 32 + 1) + 16.0 * n
                      : 12.0 * c.A0p.nnz + 4.0 * (n + 1) + 16.0 * n;
    return;
  }
  if (c.cfg.precision == 1) profile_level0(c, static_cast<Hierarchy<double>&>(*c.H), which, reps, ms, bytes);
  else profile_level0(c, static_cast<Hierarchy<float>&>(*c.H), which, reps, ms, bytes);
}

}  // namespace femgpu
