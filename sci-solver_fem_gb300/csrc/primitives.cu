// primitives.cu -- scans, reductions and segmented sorts written for this library
// (no Thrust/CUB on the product path).
#include <map>
#include <mutex>

#include "common.cuh"

namespace femgpu {

void ensure_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> set;
  int dev = 0;
  FG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = set[{dev, func}];
  if (bytes <= cur) return;
  FG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}


namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of ITEMS consecutive values per thread.
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* warp_sums, int32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
    int32_t ws = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    warp_sums[lane] = ws - w;  // exclusive warp offsets
    if (lane == 31) *total = ws;
  }
  __syncthreads();
  return warp_sums[warp] + x - v;
}

__global__ void scan_tiles_kernel(const int32_t* in, int32_t* out, int64_t n, int32_t* tile_sums) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t total;
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int64_t i = base + k;
    v[k] = (i < n) ? in[i] : 0;
    local += v[k];
  }
  int32_t off = block_exclusive_scan(local, warp_sums, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    int64_t i = base + k;
    if (i < n) out[i] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void add_tile_offsets_kernel(int32_t* out, int64_t n, const int32_t* tile_offsets) {
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int32_t add = tile_offsets[blockIdx.x];
  for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
    int64_t i = base + k;
    if (i < n) out[i] += add;
  }
}

__global__ void write_total_kernel(int32_t* out, int64_t n, const int32_t* last_in_copy, int32_t has_last) {
  // out[n] = out[n-1] + in[n-1] (in[n-1] saved before an in-place scan)
  if (threadIdx.x == 0 && blockIdx.x == 0) out[n] = (n > 0 ? out[n - 1] + (has_last ? *last_in_copy : 0) : 0);
}

// Recursive exclusive scan without the total entry.
void exclusive_scan_rec(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  DBuf<int32_t> sums(tiles + 1, s);
  scan_tiles_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, sums.p);
  FG_CHECK_LAUNCH();
  if (tiles > 1) {
    exclusive_scan_rec(sums.p, sums.p, tiles, s);
    add_tile_offsets_kernel<<<(unsigned)tiles, 256, 0, s>>>(out, n, sums.p);
    FG_CHECK_LAUNCH();
  }
}

__global__ void copy_one_kernel(const int32_t* src, int32_t* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = *src;
}

__global__ void reduce_max_kernel(const int32_t* a, int64_t n, int32_t* out) {
  int32_t m = INT32_MIN;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, a[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  // one atomic per block
  __shared__ int32_t wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : INT32_MIN;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) atomicMax(out, m);
  }
}

__global__ void count_equal_kernel(const int32_t* a, int64_t n, int32_t v, unsigned long long* out) {
  unsigned c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += (a[i] == v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  // one atomic per block
  __shared__ unsigned wc[32];
  if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    c = threadIdx.x < (blockDim.x >> 5) ? wc[threadIdx.x] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0 && c) atomicAdd(out, (unsigned long long)c);
  }
}

__global__ void fill_kernel(int32_t* a, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}
__global__ void iota_kernel(int32_t* a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = (int32_t)i;
}

int reduce_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

// ---- segmented sort ----------------------------------------------------------
constexpr int kWarpCap = 1024;   // per-warp shared-memory capacity (ints)
constexpr int kWarpsPerBlock = 4;
constexpr int kBlockCap = 8192;  // per-block capacity (ints)

// Compacts the sorted run s[0..len) to its unique values at dst; returns count.
template <class Sync>
__device__ int unique_write(const int32_t* s, int len, int32_t* dst, int tid, int nthr, int32_t* scratch_count,
                            Sync sync) {
  // sequential-by-chunk ballot compaction works only inside one warp; blocks use
  // a simple two-step approach on the scratch counter.
  int count = 0;
  if (nthr == 32) {
    for (int base = 0; base < len; base += 32) {
      int p = base + tid;
      bool keep = p < len && (p == 0 || s[p] != s[p - 1]);
      unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) dst[count + __popc(m & ((1u << tid) - 1u))] = s[p];
      count += __popc(m);
    }
    return count;
  }
  // block: one thread writes (blocks are only used for rare long segments)
  if (tid == 0) {
    int c = 0;
    for (int p = 0; p < len; p++)
      if (p == 0 || s[p] != s[p - 1]) dst[c++] = s[p];
    *scratch_count = c;
  }
  sync();
  return *scratch_count;
}

__global__ void segsort_warp_kernel(int32_t* vals, const int32_t* off, int nseg, int32_t* ucount) {
  __shared__ int32_t sm[kWarpsPerBlock][kWarpCap];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int seg = blockIdx.x * kWarpsPerBlock + w;
  if (seg >= nseg) return;
  int b = off[seg], e = off[seg + 1], len = e - b;
  if (len > kWarpCap) return;
  int32_t* s = sm[w];
  int np2 = next_pow2(len < 2 ? 2 : len);
  for (int i = lane; i < np2; i += 32) s[i] = (i < len) ? vals[b + i] : INT32_MAX;
  __syncwarp();
  bitonic_sort_shared(s, np2, lane, 32, WarpSync());
  if (ucount) {
    int c = unique_write(s, len, vals + b, lane, 32, nullptr, WarpSync());
    if (lane == 0) ucount[seg] = c;
  } else {
    for (int i = lane; i < len; i += 32) vals[b + i] = s[i];
  }
}

__global__ void segsort_block_kernel(int32_t* vals, const int32_t* off, int nseg, int32_t* ucount) {
  __shared__ int32_t s[kBlockCap];
  __shared__ int32_t cnt;
  const int seg = blockIdx.x;
  int b = off[seg], e = off[seg + 1], len = e - b;
  if (len <= kWarpCap || len > kBlockCap) return;
  int np2 = next_pow2(len);
  for (int i = threadIdx.x; i < np2; i += blockDim.x) s[i] = (i < len) ? vals[b + i] : INT32_MAX;
  __syncthreads();
  bitonic_sort_shared(s, np2, threadIdx.x, blockDim.x, BlockSync());
  if (ucount) {
    int c = unique_write(s, len, vals + b, threadIdx.x, blockDim.x, &cnt, BlockSync());
    if (threadIdx.x == 0) ucount[seg] = c;
  } else {
    for (int i = threadIdx.x; i < len; i += blockDim.x) vals[b + i] = s[i];
  }
}

// Heap sort in global memory for segments beyond the shared-memory tiers.
__device__ void sift_down(int32_t* a, int start, int end) {
  int root = start;
  while (2 * root + 1 <= end) {
    int child = 2 * root + 1, sw = root;
    if (a[sw] < a[child]) sw = child;
    if (child + 1 <= end && a[sw] < a[child + 1]) sw = child + 1;
    if (sw == root) return;
    int32_t t = a[root];
    a[root] = a[sw];
    a[sw] = t;
    root = sw;
  }
}

__global__ void segsort_serial_kernel(int32_t* vals, const int32_t* off, int nseg, int32_t* ucount) {
  for (int seg = blockIdx.x * blockDim.x + threadIdx.x; seg < nseg; seg += gridDim.x * blockDim.x) {
    int b = off[seg], e = off[seg + 1], len = e - b;
    if (len <= kBlockCap) continue;
    int32_t* a = vals + b;
    for (int st = (len - 2) / 2; st >= 0; st--) sift_down(a, st, len - 1);
    for (int end = len - 1; end > 0; end--) {
      int32_t t = a[0];
      a[0] = a[end];
      a[end] = t;
      sift_down(a, 0, end - 1);
    }
    if (ucount) {
      int c = 0;
      for (int p = 0; p < len; p++)
        if (p == 0 || a[p] != a[p - 1]) a[c++] = a[p];
      ucount[seg] = c;
    }
  }
}

__global__ void seg_len_kernel(const int32_t* off, int nseg, int32_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nseg; i += gridDim.x * blockDim.x) out[i] = off[i + 1] - off[i];
}

}  // namespace

void exclusive_scan_async(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
  DBuf<int32_t> last(1, s);
  if (n > 0) {
    copy_one_kernel<<<1, 32, 0, s>>>(in + (n - 1), last.p);
    FG_CHECK_LAUNCH();
  }
  exclusive_scan_rec(in, out, n, s);
  write_total_kernel<<<1, 32, 0, s>>>(out, n, last.p, n > 0);
  FG_CHECK_LAUNCH();
}

int64_t exclusive_scan(const int32_t* in, int32_t* out, int64_t n, cudaStream_t s) {
  exclusive_scan_async(in, out, n, s);
  return (int64_t)read_scalar(out + n, s);
}

void inclusive_scan_inplace(int32_t* a, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  DBuf<int32_t> tmp(n + 1, s);
  exclusive_scan_async(a, tmp.p, n, s);
  // inclusive[i] = exclusive[i+1]
  FG_CUDA(cudaMemcpyAsync(a, tmp.p + 1, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
}

void reduce_max_async(const int32_t* a, int64_t n, int32_t* out, cudaStream_t s) {
  fill_i32(out, 1, INT32_MIN, s);
  if (n > 0) {
    reduce_max_kernel<<<reduce_grid(n), 256, 0, s>>>(a, n, out);
    FG_CHECK_LAUNCH();
  }
}

int32_t reduce_max(const int32_t* a, int64_t n, cudaStream_t s) {
  DBuf<int32_t> out(1, s);
  fill_i32(out.p, 1, INT32_MIN, s);
  if (n > 0) {
    reduce_max_kernel<<<reduce_grid(n), 256, 0, s>>>(a, n, out.p);
    FG_CHECK_LAUNCH();
  }
  return read_scalar(out.p, s);
}

int64_t count_equal(const int32_t* a, int64_t n, int32_t value, cudaStream_t s) {
  DBuf<unsigned long long> out(1, s);
  out.zero();
  if (n > 0) {
    count_equal_kernel<<<reduce_grid(n), 256, 0, s>>>(a, n, value, out.p);
    FG_CHECK_LAUNCH();
  }
  return (int64_t)read_scalar(out.p, s);
}

void fill_i32(int32_t* a, int64_t n, int32_t v, cudaStream_t s) {
  if (n <= 0) return;
  fill_kernel<<<reduce_grid(n), 256, 0, s>>>(a, n, v);
  FG_CHECK_LAUNCH();
}

void iota_i32(int32_t* a, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  iota_kernel<<<reduce_grid(n), 256, 0, s>>>(a, n);
  FG_CHECK_LAUNCH();
}

void segmented_sort_i32(int32_t* vals, const int32_t* off, int nseg, int32_t* ucount, cudaStream_t s) {
  if (nseg <= 0) return;
  DBuf<int32_t> lens(nseg, s);
  seg_len_kernel<<<grid_for(nseg, 256), 256, 0, s>>>(off, nseg, lens.p);
  FG_CHECK_LAUNCH();
  int32_t maxlen = reduce_max(lens.p, nseg, s);
  segsort_warp_kernel<<<grid_for(nseg, kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(vals, off, nseg, ucount);
  FG_CHECK_LAUNCH();
  if (maxlen > kWarpCap) {
    segsort_block_kernel<<<nseg, 1024, 0, s>>>(vals, off, nseg, ucount);
    FG_CHECK_LAUNCH();
  }
  if (maxlen > kBlockCap) {
    segsort_serial_kernel<<<grid_for(nseg, 128), 128, 0, s>>>(vals, off, nseg, ucount);
    FG_CHECK_LAUNCH();
  }
}

}  // namespace femgpu
