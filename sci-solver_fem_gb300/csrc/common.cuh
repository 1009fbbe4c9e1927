// common.cuh -- shared device infrastructure of libfemgpu (sm_103a).
//
// Conventions used by every kernel file:
//  * all work runs on the handle's stream; device memory comes from
//    cudaMallocAsync on that stream (stream-ordered, no device-wide syncs);
//  * the library is compiled with -fmad=false: no multiply-add is fused unless
//    the source says fma()/fmaf(), so rounding matches the CPU oracle exactly;
//  * every loop that waits for a convergence flag has an iteration cap and
//    reports FEMGPU_ERR_LIMIT instead of spinning forever.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/femgpu.h"

namespace femgpu {

// A named NVTX range over a scope: Nsight Systems and Nsight Compute show the library's
// calls and setup levels on the timeline when they run the program; without a tool
// attached the push and pop do nothing.  A null name opens no range.
struct TraceRange {
  bool on;
  explicit TraceRange(const char* name) : on(name != nullptr) {
    if (on) nvtxRangePushA(name);
  }
  ~TraceRange() {
    if (on) nvtxRangePop();
  }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

struct Error : std::runtime_error {
  femgpu_status status;
  Error(femgpu_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define FG_CUDA(call)                                                                        \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      throw ::femgpu::Error(FEMGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define FG_CHECK_LAUNCH() FG_CUDA(cudaGetLastError())

#define FG_REQUIRE(cond, status, msg)                     \
  do {                                                    \
    if (!(cond)) throw ::femgpu::Error((status), (msg));  \
  } while (0)

// Memory pool of the handle whose entry point is running on this thread (set by the
// C ABI around each call); null = the device's current pool.
extern thread_local cudaMemPool_t g_alloc_pool;

// Stream-ordered device buffer.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = 0;
  DBuf() = default;
  DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; s = o.s;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count) {
      cudaError_t e = g_alloc_pool ? cudaMallocFromPoolAsync((void**)&p, count * sizeof(T), g_alloc_pool, st)
                                   : cudaMallocAsync((void**)&p, count * sizeof(T), st);
      if (e != cudaSuccess) {
        p = nullptr;
        n = 0;
        (void)cudaGetLastError();
        throw Error(FEMGPU_ERR_ALLOC, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
      }
    }
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (n) FG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  void upload(const T* h, size_t count) {
    FG_REQUIRE(count <= n, FEMGPU_ERR_INVALID, "upload larger than buffer");
    if (count) FG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t count) const {
    FG_REQUIRE(count <= n, FEMGPU_ERR_INVALID, "download larger than buffer");
    if (count) FG_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  std::vector<T> to_host() const {
    std::vector<T> v(n);
    download(v.data(), n);
    FG_CUDA(cudaStreamSynchronize(s));
    return v;
  }
};

// CSR matrix in device memory.
template <class T>
struct DCsr {
  int n = 0, m = 0;
  int64_t nnz = 0;
  DBuf<int32_t> rp, ci;
  DBuf<T> v;
};

inline int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 2147483647LL) g = 2147483647LL;
  return (int)g;
}

// Raises a kernel's dynamic shared memory limit to at least `bytes` on the current
// device.  The runtime call is slow (about a millisecond on GB300), so the largest
// value set per (device, kernel) is remembered and the call is made only to raise it.
void ensure_dynamic_smem(const void* func, size_t bytes);
template <class F>
inline void ensure_smem(F* func, size_t bytes) {
  if (bytes > 48 * 1024) ensure_dynamic_smem(reinterpret_cast<const void*>(func), bytes);
}

// Host round trips of the setup (counted for its phase timer).
extern std::atomic<int64_t> g_host_syncs;

// Reads one device scalar synchronously (used only at setup-time loop checks).
template <class T>
inline T read_scalar(const T* d, cudaStream_t s) {
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  T h;
  FG_CUDA(cudaMemcpyAsync(&h, d, sizeof(T), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  return h;
}

// ---- device primitives (primitives.cu) --------------------------------------
// Exclusive scan of n int32 counts into out[0..n] (out[n] = total, int64 safe
// total returned).  out may alias in only if in has n+1 entries.
int64_t exclusive_scan(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s);
// The same scan with the total left on the device (out[n]); no host round trip.
void exclusive_scan_async(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s);
// Inclusive scan in place.
void inclusive_scan_inplace(int32_t* a, int64_t n, cudaStream_t s);
int32_t reduce_max(const int32_t* a, int64_t n, cudaStream_t s);
// The same maximum written to out[0] on the device (INT32_MIN when n == 0).
void reduce_max_async(const int32_t* a, int64_t n, int32_t* out, cudaStream_t s);
int64_t count_equal(const int32_t* a, int64_t n, int32_t value, cudaStream_t s);
void fill_i32(int32_t* a, int64_t n, int32_t v, cudaStream_t s);
void iota_i32(int32_t* a, int64_t n, cudaStream_t s);
// Segmented in-place ascending sort of int32 values; segment k spans
// [off[k], off[k+1]).  With unique != nullptr each segment is also deduplicated
// in place and its unique length written to unique[k].
void segmented_sort_i32(int32_t* vals, const int32_t* off, int nseg, int32_t* unique_counts, cudaStream_t s);

// ---- small device helpers -----------------------------------------------------
__device__ __forceinline__ int lower_bound_i32(const int32_t* a, int lo, int hi, int key) {
  // first index in [lo, hi) with a[i] >= key
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Bitonic sort of n (power of two) keys in shared memory by the threads
// [t0, t0 + nthreads) that call it; sync() is __syncwarp or __syncthreads.
template <class K, class Sync>
__device__ __forceinline__ void bitonic_sort_shared(K* s, int n, int tid, int nthreads, Sync sync) {
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < (n >> 1); i += nthreads) {
        int lo = 2 * i - (i & (stride - 1));
        int hi = lo + stride;
        bool asc = (lo & size) == 0;
        K a = s[lo], b = s[hi];
        if ((a > b) == asc) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      sync();
    }
  }
}

struct WarpSync {
  __device__ void operator()() const { __syncwarp(); }
};
struct BlockSync {
  __device__ void operator()() const { __syncthreads(); }
};

__host__ __device__ inline int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream-serialisation attribute (launch_pdl) may be scheduled before the kernel ahead
// of it in the stream has finished, once every CTA of that kernel has called
// pdl_trigger() (or exited).  It must call pdl_wait() before it reads anything an
// earlier kernel wrote and before it writes anything: pdl_wait() returns when the kernel
// ahead has completed and its memory operations are visible.  What it reads before
// pdl_wait() must be constant across the kernels of the stream (matrix entries, sizes).
// In a kernel launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// The start of a kernel that reads nothing before waiting: wait, then let the next
// kernel be scheduled.
__device__ __forceinline__ void pdl_enter() {
  pdl_wait();
  pdl_trigger();
}

// A hint to bring the line holding p into L2 (p must point into an allocation).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// A bulk asynchronous prefetch of the 16-byte units that lie wholly inside [b, e) into
// L2 (both ends rounded down to 16 bytes, so nothing past e is touched; b must point
// into an allocation, whose start is 16-byte aligned).  Nothing waits for it.
__device__ __forceinline__ void bulk_prefetch_range_l2(const void* b, const void* e) {
  const uintptr_t lo = (uintptr_t)b & ~(uintptr_t)15, hi = (uintptr_t)e & ~(uintptr_t)15;
  if (hi > lo)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((uint32_t)(hi - lo)) : "memory");
}

// ---- bulk asynchronous copies (TMA, 1-D) with an mbarrier -----------------------
// cp.async.bulk moves a contiguous global range into shared memory; source,
// destination and size must be multiples of 16 bytes.  Completion is counted in
// bytes on an mbarrier in shared memory.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the barrier phase with an iteration limit and a time limit; false when either
// ran out (a limit of 0 gives up without polling).  A try_wait may suspend the thread for
// a while before it reports an incomplete phase, so the poll count alone does not bound
// the time: the clock is read every 64 polls and the wait ends after kMbarWaitNs.
constexpr int kMbarWaitLimit = 1 << 22;
constexpr uint64_t kMbarWaitNs = 500ull * 1000 * 1000;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit = kMbarWaitLimit) {
  const uint64_t t0 = global_ns();
  for (int i = 0; i < limit; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && global_ns() - t0 > kMbarWaitNs) return false;
  }
  return false;
}

}  // namespace femgpu
