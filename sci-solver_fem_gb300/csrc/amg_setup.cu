// amg_setup.cu -- smoothed-aggregation hierarchy built on the device.
//
// Per level (AMG::setup, src/core/cuda/amg.cu:80-144; createNextLevel,
// smoothedMG_amg_level.cu:403-494):
//   1. OldMIS two-level aggregation of the level graph (ComputePermutationMethods.cu:22-151):
//      seeded distance-2 randomized MIS -> aggregates (min size 9) -> distance-1 MIS on
//      the aggregate graph -> partitions of <= partitionMaxSize rows;
//   2. the permutation that makes aggregates and partitions contiguous;
//   3. Ap = perm(A), the in/out-of-partition split used by the smoother;
//   4. P = (I - omega D^-1 Ap) T, R = P^T;
//   5. A_next = R (Ap P), each product row accumulated in generation order by the
//      tier its size calls for: a per-thread column list (large levels), a warp hash
//      table, a block hash table or a dense accumulator;
//   6. each parent's R rows and P columns put in the child's order, and the FP64 outer
//      operator in level-0 order as 32-row slices.
// Integer results are bit-identical to the CPU oracle for the same seed; floating
// results use fixed summation orders (generation order, ascending column), so they are
// too.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <limits>
#include <vector>

#include "context.cuh"

namespace femgpu {

namespace {

constexpr int kCap = 100000;  // bound on every data-dependent loop (error, never spin)

// Setup phase timer (FEMGPU_PROFILE): stream-synchronised wall time per phase with
// the kernel launches and host reads it took.
struct PhaseTimer {
  bool on;
  cudaStream_t s;
  int level;
  std::chrono::steady_clock::time_point t0;
  int64_t syncs0 = 0, launches0 = 0;
  PhaseTimer(cudaStream_t st, int lvl) : on(getenv("FEMGPU_PROFILE") != nullptr), s(st), level(lvl) {
    if (on) {
      cudaStreamSynchronize(s);
      t0 = std::chrono::steady_clock::now();
      syncs0 = g_host_syncs.load();
      launches0 = g_kernel_launches.load();
    }
  }
  void mark(const char* what) {
    if (!on) return;
    cudaStreamSynchronize(s);
    auto t = std::chrono::steady_clock::now();
    const int64_t sy = g_host_syncs.load(), la = g_kernel_launches.load();
    fprintf(stderr, "[femgpu setup] level %d %-10s %8.3f ms  %5lld launches %4lld host reads\n", level, what,
            std::chrono::duration<double, std::milli>(t - t0).count(), (long long)(la - launches0),
            (long long)(sy - syncs0));
    t0 = t;
    syncs0 = sy;
    launches0 = la;
  }
};

// ---------------------------------------------------------------------------------
// glibc rand() stream (TYPE_3 additive feedback generator), host side: the
// reference draws 32768 seeds with rand() after srand() (randomizedMIS_GPU.cu:195-201).
void glibc_rand_stream(uint32_t seed, int count, std::vector<uint32_t>& out) {
  std::vector<uint32_t> st(344 + (size_t)count);
  int32_t s0 = (int32_t)(seed ? seed : 1u);
  st[0] = (uint32_t)s0;
  int64_t w = s0;
  for (int i = 1; i < 31; i++) {
    w = (16807LL * w) % 2147483647LL;
    if (w < 0) w += 2147483647LL;
    st[i] = (uint32_t)w;
  }
  for (int i = 31; i < 34; i++) st[i] = st[i - 31];
  for (size_t i = 34; i < st.size(); i++) st[i] = st[i - 31] + st[i - 3];
  out.resize(count);
  for (int k = 0; k < count; k++) out[k] = st[344 + (size_t)k] >> 1;
}

__device__ __forceinline__ uint32_t taus(uint32_t z) {
  uint32_t b = (((z << 13) ^ z) >> 19);
  return (z << 12) ^ b;
}

// ---- randomized MIS (randomizedMIS_GPU.cu:3-152) ---------------------------------
__global__ void mis_randoms_kernel(int n, int iterations, uint32_t* randoms, const uint32_t* seeds) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 32768) return;
  uint32_t z = seeds[t];
  int off = t;
  for (int i = 0; i < iterations; i++)
    if (off < n) {
      z = taus(z);
      randoms[off] = z;
      off += 32768;
    }
}

// A node's (value, origin) pair packed as value << 32 | origin: the reference's update
// (take a neighbour with a larger value, or the same positive value and a larger
// origin) is the maximum of the packed keys over the node and its neighbours with a
// positive value.
__device__ __forceinline__ uint64_t mis_key(int32_t best, int32_t origin) {
  return ((uint64_t)(uint32_t)best << 32) | (uint32_t)origin;
}

__global__ void mis_first_init_kernel(int n, const uint32_t* randoms, uint64_t* key) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) key[i] = mis_key((int32_t)(randoms[i] % 1000000u), i);
}

__global__ void mis_init_kernel(int n, uint32_t* randoms, uint64_t* key, const int32_t* mis) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    uint32_t z = taus(randoms[i]);
    int st = mis[i];
    key[i] = mis_key(st == -1 ? (int32_t)(z % 1000000u) : (st == 1 ? 1000001 : 0), i);
    randoms[i] = z;
  }
}

__global__ void mis_iterate_kernel(int n, const uint64_t* __restrict__ kin, uint64_t* __restrict__ kout,
                                   const int32_t* __restrict__ xadj, const int32_t* __restrict__ adj, int32_t* mis,
                                   int32_t* incomplete, int final_pass) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = kin[i];
  if ((k >> 32) < 1000001u) {
    // neighbours in groups of 8: all indices, then all keys, so the loads overlap
    const int e1 = xadj[i + 1];
    for (int e0 = xadj[i]; e0 < e1; e0 += 8) {
      int nb[8];
      uint64_t kn[8];
#pragma unroll
      for (int q = 0; q < 8; q++) nb[q] = e0 + q < e1 ? adj[e0 + q] : i;
#pragma unroll
      for (int q = 0; q < 8; q++) kn[q] = kin[nb[q]];
#pragma unroll
      for (int q = 0; q < 8; q++)
        if ((kn[q] >> 32) > 0u && kn[q] > k) k = kn[q];
    }
  }
  kout[i] = k;
  if (final_pass) {
    const int best = (int)(k >> 32), org = (int)(uint32_t)k;
    int st = -1;
    if (org == i) st = 1;
    else if (best == 1000001) st = 0;
    mis[i] = st;
    // one store per warp with an undecided node (a single flag address)
    const unsigned undecided = __ballot_sync(__activemask(), st == -1);
    if (undecided && (threadIdx.x & 31) == (__ffs(__activemask()) - 1)) *incomplete = 1;
  }
}

void random_mis(Ctx& c, int n, const int32_t* xadj, const int32_t* adj, int k, DBuf<int32_t>& mis) {
  cudaStream_t s = c.stream;
  PhaseTimer pt(s, -5);
  mis.alloc(n, s);
  fill_i32(mis.p, n, -1, s);
  std::vector<uint32_t> seeds;
  glibc_rand_stream(c.cfg.seed, 32768, seeds);
  DBuf<uint32_t> dseeds(32768, s), randoms(n, s);
  dseeds.upload(seeds.data(), 32768);
  DBuf<uint64_t> k0(n, s), k1(n, s);
  DBuf<int32_t> flag(1, s);
  FG_LAUNCH(mis_randoms_kernel, 128, 256, 0, s, n, (n + 32767) / 32768, randoms.p, dseeds.p);
  FG_LAUNCH(mis_first_init_kernel, grid_for(n, 256), 256, 0, s, n, randoms.p, k0.p);
  pt.mark("mis init");
  // Rounds are enqueued in batches and the flag of a batch's last round is read once:
  // a round after the one that completes the set changes nothing (decided nodes keep
  // their state), so the extra rounds only cost time.  Small levels, where a host
  // round trip costs more than a round, take larger batches.
  const int batch = n < (1 << 18) ? 4 : 2;
  for (int round = 0;; round++) {
    FG_REQUIRE(round < kCap, FEMGPU_ERR_LIMIT, "randomized MIS did not complete");
    if (round > 0) FG_LAUNCH(mis_init_kernel, grid_for(n, 256), 256, 0, s, n, randoms.p, k0.p, mis.p);
    flag.zero();
    uint64_t *ki = k0.p, *ko = k1.p;
    for (int it = 0; it < k; it++) {
      FG_LAUNCH(mis_iterate_kernel, grid_for(n, 256), 256, 0, s, n, ki, ko, xadj, adj, mis.p, flag.p, it == k - 1);
      std::swap(ki, ko);
    }
    if (ki != k0.p) std::swap(k0.p, k1.p);  // keep k0 as the next round's input
    if ((round + 1) % batch != 0) continue;
    if (read_scalar(flag.p, s) == 0) break;
    pt.mark("mis rounds");
  }
}

// ---- aggregation helpers (misHelpers.cu) ----------------------------------------------
__global__ void label_roots_kernel(int n, const int32_t* mis, const int32_t* incl, int32_t* part, int32_t* aggregated) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    aggregated[i] = mis[i];
    part[i] = mis[i] == 0 ? -1 : incl[i] - 1;  // ifLabelOne
  }
}

// allocateNodesKernel (misHelpers.cu:13-75): its candidate loop fills every free slot
// with the first aggregated neighbour seen and can never out-count it, so an
// unaggregated node joins the aggregate of its first aggregated neighbour in
// adjacency order.  Writes the full partOut so the buffers can be swapped.
__global__ void allocate_kernel(int n, const int32_t* __restrict__ xadj, const int32_t* __restrict__ adj,
                                const int32_t* __restrict__ pin, int32_t* __restrict__ pout, int32_t* aggregated,
                                int32_t* counters /* [0] unallocated after, [1] changed */) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool changed = false, left = false;
  if (i < n) {
    int p = pin[i];
    if (aggregated[i] == 0) {
      int add = -1;
      // first aggregated neighbour in adjacency order, neighbours loaded 8 at a time
      const int e1 = xadj[i + 1];
      for (int e0 = xadj[i]; e0 < e1 && add == -1; e0 += 8) {
        int nb[8], cnd[8];
#pragma unroll
        for (int q = 0; q < 8; q++) nb[q] = e0 + q < e1 ? adj[e0 + q] : -1;
#pragma unroll
        for (int q = 0; q < 8; q++) cnd[q] = nb[q] >= 0 ? pin[nb[q]] : -1;
#pragma unroll
        for (int q = 0; q < 8; q++)
          if (add == -1 && cnd[q] != -1) add = cnd[q];
      }
      p = add;
      if (add != -1) {
        aggregated[i] = 1;
        changed = true;
      } else {
        left = true;
      }
    }
    pout[i] = p;
  }
  // one atomic per block instead of one per node (a single counter address)
  const int nleft = __syncthreads_count(left);
  const int nchanged = __syncthreads_or(changed);
  if (threadIdx.x == 0) {
    if (nleft) atomicAdd(&counters[0], nleft);
    if (nchanged) atomicExch(&counters[1], 1);
  }
}

__global__ void histogram_kernel(int n, const int32_t* part, const int32_t* w, int32_t* sizes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int p = part[i];
    if (p >= 0) atomicAdd(&sizes[p], w ? w[i] : 1);
  }
}

__global__ void less_than_kernel(int np, const int32_t* sizes, int threshold, int32_t* flags) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np) flags[p] = sizes[p] < threshold ? 1 : 0;
}

__global__ void remove_parts_kernel(int n, int32_t* part, const int32_t* rm, const int32_t* sub, int32_t* aggregated) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int p = part[i];
    int q = rm[p] ? -1 : p - sub[p];
    part[i] = q;
    aggregated[i] = q == -1 ? 0 : 1;
  }
}

// findDesirabilityKernel (misHelpers.cu:297-382) with IEEE float steps spelled out.
__global__ void desirability_kernel(int n, int opt, const int32_t* __restrict__ xadj, const int32_t* __restrict__ adj,
                                    const int32_t* __restrict__ part, const int32_t* __restrict__ sizes,
                                    const int32_t* __restrict__ w, int32_t* to,
                                    unsigned long long* best /* per partition: (desirability bits, node) */) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  int cur = part[idx];
  int cs = sizes[cur];
  int nw = w[idx];
  int selfAdj = 0, addTo = -1;
  float bestD = 0.0f;
  float cwf = __fdiv_rn((float)abs(cs - opt), (float)opt);
  float selfImp = __fmul_rn((float)(abs(cs - opt) - abs((cs - nw) - opt)), cwf);
  if (selfImp > 0) {
    int cand[10], cnt[10];
#pragma unroll
    for (int q = 0; q < 10; q++) {
      cand[q] = -1;
      cnt[q] = 0;
    }
    for (int e = xadj[idx]; e < xadj[idx + 1]; e++) {
      int cc = part[adj[e]];
      if (cc == cur) {
        selfAdj++;
        continue;
      }
      // distinct candidates in first-seen order, at most 10 (junk counts of free
      // slots in the reference never reach a used slot)
#pragma unroll
      for (int q = 0; q < 10; q++) {
        if (cand[q] == cc) {
          cnt[q]++;
          break;
        }
        if (cand[q] == -1) {
          cand[q] = cc;
          cnt[q] = 1;
          break;
        }
      }
    }
    // the reference scans candidates 1..9 (its loop starts at 1)
#pragma unroll
    for (int q = 1; q < 10; q++) {
      if (cand[q] == -1) continue;
      int np_ = cand[q];
      int nsz = sizes[np_];
      float nwf = __fdiv_rn((float)abs(nsz - opt), (float)opt);
      float imp = __fmul_rn((float)(abs(nsz - opt) - abs((nsz + nw) - opt)), nwf);
      imp = __fadd_rn(imp, selfImp);
      float ratio = __fdiv_rn((float)cnt[q], (float)selfAdj);
      imp = __fmul_rn(imp, ratio);
      if (imp > bestD) {
        addTo = np_;
        bestD = imp;
      }
    }
  }
  to[idx] = addTo;
  unsigned long long key = ((unsigned long long)__float_as_uint(bestD) << 32) | (unsigned)idx;
  atomicMax(&best[cur], key);
}

// makeSwapsKernel (misHelpers.cu:384-412): per source partition, the node with the
// largest (desirability, index) moves when its desirability exceeds 0.1.
__global__ void swap_kernel(int np, unsigned long long* best, int32_t* part, const int32_t* to, const int32_t* w,
                            int32_t* sizes) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  unsigned long long key = best[p];
  best[p] = 0ull;
  float d = __uint_as_float((unsigned)(key >> 32));
  int idx = (int)(key & 0xffffffffu);
  if ((double)d > .1) {
    int t = to[idx];
    part[idx] = t;
    atomicAdd(&sizes[t], w[idx]);
    atomicAdd(&sizes[p], -w[idx]);
  }
}

// removeRuntyParts / removeRuntyPartitions (misHelpers.cu:744-820).  Returns the
// number of removed parts.  np: the number of parts (labels 0 .. np-1, none empty)
// when the caller tracks it, else -1 (then it is read from the labels).
int remove_small_parts(Ctx& c, int n, DBuf<int32_t>& part, const int32_t* weights, int threshold_mode, int min_size,
                       int full_size, DBuf<int32_t>& aggregated, int np = -1) {
  cudaStream_t s = c.stream;
  if (np < 0) np = reduce_max(part.p, n, s) + 1;
  DBuf<int32_t> sizes(np, s), rm(np + 1, s), sub(np + 1, s);
  sizes.zero();
  FG_LAUNCH(histogram_kernel, grid_for(n, 256), 256, 0, s, n, part.p, weights, sizes.p);
  int threshold = min_size;
  if (threshold_mode == 1) {
    double avg = (double)full_size / np;
    threshold = (int)(avg * .7);
  }
  FG_LAUNCH(less_than_kernel, grid_for(np, 256), 256, 0, s, np, sizes.p, threshold, rm.p);
  int64_t removed = exclusive_scan(rm.p, sub.p, np, s);
  if (removed == 0 && threshold_mode == 0) return 0;
  // subtractions = inclusive scan of the removal flags = exclusive scan shifted by one
  FG_LAUNCH(remove_parts_kernel, grid_for(n, 256), 256, 0, s, n, part.p, rm.p, sub.p + 1, aggregated.p);
  return (int)removed;
}

// np: the number of partitions (labels 0 .. np-1, none empty) when the caller tracks it,
// else -1 (then it is read from the labels).
int restrict_partitions(Ctx& c, int max_size, int full_size, int n, const int32_t* xadj, const int32_t* adj,
                        DBuf<int32_t>& part, const int32_t* w, int np = -1) {
  cudaStream_t s = c.stream;
  if (np < 0) np = reduce_max(part.p, n, s) + 1;
  DBuf<int32_t> sizes(np, s), to(n, s);
  sizes.zero();
  FG_LAUNCH(histogram_kernel, grid_for(n, 256), 256, 0, s, n, part.p, w, sizes.p);
  int avg = full_size / np;
  DBuf<unsigned long long> best(np, s);
  best.zero();
  int largest = reduce_max(sizes.p, np, s);
  int loops = 0;
  while (largest > max_size) {
    FG_REQUIRE(++loops < kCap, FEMGPU_ERR_LIMIT, "partition size restriction did not converge");
    FG_LAUNCH(desirability_kernel, grid_for(n, 256), 256, 0, s, n, avg, xadj, adj, part.p, sizes.p, w, to.p, best.p);
    FG_LAUNCH(swap_kernel, grid_for(np, 256), 256, 0, s, np, best.p, part.p, to.p, w, sizes.p);
    largest = reduce_max(sizes.p, np, s);
  }
  return np;
}

// aggregateGraph / aggregateWeightedGraph (misHelpers.cu:513-677).  Returns the number
// of parts for the unweighted graph (the parts are labelled 0 .. count-1), -1 for the
// weighted one (whose partition restriction may empty a part).
int aggregate(Ctx& c, int n, const int32_t* xadj, const int32_t* adj, int depth, bool weighted, int min_size,
              int max_size, int full_size, const int32_t* weights, DBuf<int32_t>& part) {
  cudaStream_t s = c.stream;
  PhaseTimer pt(s, -4);
  DBuf<int32_t> mis;
  random_mis(c, n, xadj, adj, depth, mis);
  pt.mark("mis");
  DBuf<int32_t> incl(n + 1, s), aggregated(n, s), pout(n, s), counters(2, s);
  FG_CUDA(cudaMemcpyAsync(incl.p, mis.p, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  inclusive_scan_inplace(incl.p, n, s);
  // the MIS size (= the number of parts, labelled 0 .. count-1 by label_roots_kernel)
  // comes back with the first allocation counters
  int mis_count = -1;
  part.alloc(n, s);
  FG_LAUNCH(label_roots_kernel, grid_for(n, 256), 256, 0, s, n, mis.p, incl.p, part.p, aggregated.p);
  bool first = true;
  for (int loop = 0;; loop++) {
    FG_REQUIRE(loop < kCap, FEMGPU_ERR_LIMIT, "aggregation did not complete");
    // two passes per host read: a pass after the one that leaves no node unallocated
    // changes nothing, and the counters describe the second pass
    for (int pass = 0; pass < 2; pass++) {
      counters.zero();
      FG_LAUNCH(allocate_kernel, grid_for(n, 256), 256, 0, s, n, xadj, adj, part.p, pout.p, aggregated.p,
                counters.p);
      std::swap(part.p, pout.p);
    }
    int32_t h[2];
    counters.download(h, 2);
    if (mis_count < 0 && n > 0) FG_CUDA(cudaMemcpyAsync(&mis_count, incl.p + (n - 1), sizeof(int32_t),
                                                       cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    g_host_syncs.fetch_add(1, std::memory_order_relaxed);
    if (mis_count < 0) mis_count = 0;
    pt.mark("allocate");
    if (h[0] == 0) {
      if (!weighted) {
        // unweighted parts are never emptied: their count is tracked, not read back
        const int removed = remove_small_parts(c, n, part, nullptr, 0, min_size, full_size, aggregated, mis_count);
        if (removed == 0) return mis_count;
        mis_count -= removed;
      } else {
        // the labels are still contiguous and non-empty here (the restriction below may
        // empty a partition, but nothing reads the count after it): tracked, not read
        if (!first || mis_count < 10) {
          restrict_partitions(c, max_size, full_size, n, xadj, adj, part, weights, mis_count);
          return -1;
        }
        first = false;
        mis_count -= remove_small_parts(c, n, part, weights, 1, 0, full_size, aggregated, mis_count);
      }
    } else if (h[1] == 0) {
      // also the case where every aggregate was removed as undersized (the reference
      // loops forever there)
      throw Error(FEMGPU_ERR_LIMIT,
                  "aggregation stalled: nodes unreachable from any aggregate, or every aggregate was removed "
                  "as undersized");
    }
  }
}

__global__ void scatter_bucket_kernel(int n, const int32_t* key, const int32_t* start, int32_t* cursor, int32_t* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int k = key[i];
    out[start[k] + atomicAdd(&cursor[k], 1)] = i;
  }
}

__global__ void node_degree_to_agg_kernel(int n, const int32_t* xadj, const int32_t* fine, int32_t* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[fine[i]], xadj[i + 1] - xadj[i]);
}

// Degree of each member node, in member order (aggregates in order, members ascending).
__global__ void member_degree_kernel(int n, const int32_t* members, const int32_t* xadj, int32_t* deg) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) deg[q] = xadj[members[q] + 1] - xadj[members[q]];
}

// Induced-graph rows by hashing: one warp per aggregate walks the flattened neighbour
// lists of its members 32 entries at a time (flat index f of member q starts at
// noff[q]), groups equal aggregate ids with __match_any_sync, inserts each new id once
// into a shared-memory set and finally sorts the set, so a row holds the sorted distinct
// neighbour aggregates (what sorting the candidate list and dropping duplicates gives).
// An aggregate with more than kIndCap - 32 distinct neighbours sets *overflow.
constexpr int kIndCap = 256;

__device__ __forceinline__ unsigned induced_hash(unsigned b) { return (b * 2654435761u) >> 9; }

__global__ void __launch_bounds__(256) induced_hash_kernel(int nagg, const int32_t* __restrict__ astart,
                                                           const int32_t* __restrict__ members,
                                                           const int32_t* __restrict__ noff,
                                                           const int32_t* __restrict__ xadj,
                                                           const int32_t* __restrict__ adj,
                                                           const int32_t* __restrict__ fine, int32_t* tmp,
                                                           int32_t* ucount, int32_t* overflow) {
  __shared__ int32_t hk[8][kIndCap];
  __shared__ int32_t sk[8][kIndCap];
  __shared__ int s_cnt[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int a = blockIdx.x * 8 + w; a < nagg; a += gridDim.x * 8) {
    for (int t = lane; t < kIndCap; t += 32) hk[w][t] = -1;
    if (lane == 0) s_cnt[w] = 0;
    __syncwarp();
    const int q0 = astart[a], q1 = astart[a + 1];
    const int f0 = noff[q0], f1 = noff[q1];
    bool over = false;
    for (int fb = f0; fb < f1 && !over; fb += 32) {
      const int f = fb + lane;
      int b = -1;
      if (f < f1) {
        int lo = q0, hi = q1 - 1;  // last member q with noff[q] <= f
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (noff[mid] <= f) lo = mid;
          else hi = mid - 1;
        }
        const int i = members[lo];
        b = fine[adj[xadj[i] + (f - noff[lo])]];
        if (b == a) b = -1;
      }
      const unsigned peers = __match_any_sync(0xffffffffu, b);
      if (b >= 0 && (__ffs(peers) - 1) == lane) {
        unsigned slot = induced_hash((unsigned)b) & (kIndCap - 1);
        for (int p = 0; p < kIndCap; p++) {
          const int prev = atomicCAS(&hk[w][slot], -1, b);
          if (prev == -1) {
            atomicAdd(&s_cnt[w], 1);
            break;
          }
          if (prev == b) break;
          slot = (slot + 1) & (kIndCap - 1);
        }
      }
      __syncwarp();
      over = s_cnt[w] > kIndCap - 32;  // the next chunk might not fit
    }
    if (over) {
      if (lane == 0) *overflow = 1;
      continue;
    }
    // compact the set, pad to a power of two, sort
    const int cnt = s_cnt[w];
    int base = 0;
    for (int t0 = 0; t0 < kIndCap; t0 += 32) {
      const int key = hk[w][t0 + lane];
      const unsigned m = __ballot_sync(0xffffffffu, key >= 0);
      if (key >= 0) sk[w][base + __popc(m & ((1u << lane) - 1u))] = key;
      base += __popc(m);
    }
    const int np2 = next_pow2(cnt < 2 ? 2 : cnt);
    for (int t = cnt + lane; t < np2; t += 32) sk[w][t] = INT32_MAX;
    __syncwarp();
    bitonic_sort_shared(sk[w], np2, lane, 32, WarpSync());
    for (int t = lane; t < cnt; t += 32) tmp[(int64_t)a * kIndCap + t] = sk[w][t];
    if (lane == 0) ucount[a] = cnt;
    __syncwarp();
  }
}

// Rows of fixed stride `stride` in src to their offsets doff in dst, one warp per row.
__global__ void compact_stride_kernel(int nseg, const int32_t* src, int stride, const int32_t* doff, int32_t* dst) {
  const int lane = threadIdx.x & 31;
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nseg; k += (gridDim.x * blockDim.x) >> 5) {
    const int len = doff[k + 1] - doff[k];
    for (int t = lane; t < len; t += 32) dst[doff[k] + t] = src[(int64_t)k * stride + t];
  }
}

// One thread per member node: the aggregates of its neighbours go to the node's slice
// of its aggregate's candidate list (its own aggregate as INT32_MAX padding), so every
// list holds the same multiset as a member-by-member walk.
__global__ void induced_candidates_nodes_kernel(int n, const int32_t* members, const int32_t* noff,
                                                const int32_t* __restrict__ xadj, const int32_t* __restrict__ adj,
                                                const int32_t* __restrict__ fine, int32_t* cand) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = members[q], a = fine[i];
  int o = noff[q];
  for (int e = xadj[i]; e < xadj[i + 1]; e++) {
    const int b = fine[adj[e]];
    cand[o++] = b != a ? b : INT32_MAX;
  }
}

__global__ void drop_padding_kernel(int nseg, const int32_t* off, int32_t* cnt, const int32_t* vals) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nseg && cnt[k] > 0 && vals[off[k] + cnt[k] - 1] == INT32_MAX) cnt[k]--;
}

__global__ void compact_segments_kernel(int nseg, const int32_t* src, const int32_t* soff, const int32_t* doff,
                                        int32_t* dst) {
  int lane = threadIdx.x & 31;
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < nseg; k += (gridDim.x * blockDim.x) >> 5) {
    int len = doff[k + 1] - doff[k];
    for (int t = lane; t < len; t += 32) dst[doff[k] + t] = src[soff[k] + t];
  }
}

__global__ void invert_kernel(int n, const int32_t* order, int32_t* inv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) inv[order[i]] = i;
}

__global__ void gather_len_kernel(int n, const int32_t* order, const int32_t* off, int32_t* len) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) len[q] = off[order[q] + 1] - off[order[q]];
}

__global__ void remap_graph_kernel(int nagg, const int32_t* old_of, const int32_t* ixadj, const int32_t* iadj,
                                   const int32_t* new_id, const int32_t* xo, int32_t* ao) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nagg) return;
  int a = old_of[q];
  int o = xo[q];
  for (int e = ixadj[a]; e < ixadj[a + 1]; e++) ao[o++] = new_id[iadj[e]];
}

__global__ void node_order_kernel(int nagg, const int32_t* old_of, const int32_t* astart, const int32_t* members,
                                  const int32_t* agg_idx, const int32_t* coarse, int32_t* iperm, int32_t* agg_of,
                                  int32_t* part_of_row) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nagg) return;
  int a = old_of[q];
  int o = agg_idx[q];
  int p = coarse[a];
  for (int t = astart[a]; t < astart[a + 1]; t++) {
    iperm[o] = members[t];
    agg_of[o] = q;
    part_of_row[o] = p;
    o++;
  }
}

// Opt-in setup phase timing (environment FEMGPU_PROFILE set): synchronizes between
// phases and prints the host wall time of each to stderr.

struct OldMisOut {
  int nagg = 0, npart = 0;
  DBuf<int32_t> perm, iperm, agg_idx, part_idx, agg_of, part_of_row, xadj_out, adj_out;
  int64_t nnz_out = 0;
};

// misHelpers::CP::OldMIS (ComputePermutationMethods.cu:22-151).
void old_mis(Ctx& c, int n, const int32_t* xadj, const int32_t* adj, OldMisOut& o) {
  cudaStream_t s = c.stream;
  const int params = c.cfg.randMisParameters;
  const int fine_depth = params % 100, coarse_depth = (params / 100) % 100, min_agg = (params / 10000) % 10;
  PhaseTimer pt(s, -1);
  DBuf<int32_t> fine;
  const int nagg = aggregate(c, n, xadj, adj, fine_depth, false, min_agg, 0, n, nullptr, fine);
  pt.mark("fine agg");
  // aggregate member lists, ascending node id
  DBuf<int32_t> acount(nagg + 1, s), astart(nagg + 1, s), cursor(nagg, s), members(n, s);
  acount.zero();
  FG_LAUNCH(histogram_kernel, grid_for(n, 256), 256, 0, s, n, fine.p, nullptr, acount.p);
  exclusive_scan_async(acount.p, astart.p, nagg, s);
  cursor.zero();
  FG_LAUNCH(scatter_bucket_kernel, grid_for(n, 256), 256, 0, s, n, fine.p, astart.p, cursor.p, members.p);
  segmented_sort_i32(members.p, astart.p, nagg, nullptr, s);
  // induced graph (getInducedGraph, misHelpers.cu:1078-1107): sorted unique neighbour aggregates
  DBuf<int32_t> ucount(nagg + 1, s), ixadj(nagg + 1, s), iadj;
  DBuf<int32_t> mdeg(n + 1, s), noff(n + 1, s);
  FG_LAUNCH(member_degree_kernel, grid_for(n, 256), 256, 0, s, n, members.p, xadj, mdeg.p);
  exclusive_scan_async(mdeg.p, noff.p, n, s);
  bool induced_done = false;
  int64_t induced_nnz = 0;
  {
    DBuf<int32_t> tmp((size_t)nagg * kIndCap, s), ovf(1, s);
    ovf.zero();
    FG_LAUNCH(induced_hash_kernel, (int)std::min<int64_t>((nagg + 7) / 8, 152 * 16), 256, 0, s, nagg, astart.p,
              members.p, noff.p, xadj, adj, fine.p, tmp.p, ucount.p, ovf.p);
    // the overflow flag and the total come back in one round trip
    exclusive_scan_async(ucount.p, ixadj.p, nagg, s);
    int32_t h_ovf = 0, h_tot = 0;
    FG_CUDA(cudaMemcpyAsync(&h_ovf, ovf.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaMemcpyAsync(&h_tot, ixadj.p + nagg, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    g_host_syncs.fetch_add(1, std::memory_order_relaxed);
    if (h_ovf == 0) {
      const int64_t innz = h_tot;
      induced_nnz = innz;
      iadj.alloc(innz > 0 ? innz : 1, s);
      FG_LAUNCH(compact_stride_kernel, grid_for((int64_t)nagg * 32, 256), 256, 0, s, nagg, tmp.p, kIndCap, ixadj.p,
                iadj.p);
      induced_done = true;
    }
  }
  if (!induced_done) {
    // an aggregate with more than kIndCap neighbour aggregates: sort every candidate list
    DBuf<int32_t> ccount(nagg + 1, s), coff(nagg + 1, s);
    ccount.zero();
    FG_LAUNCH(node_degree_to_agg_kernel, grid_for(n, 256), 256, 0, s, n, xadj, fine.p, ccount.p);
    int64_t ncand = exclusive_scan(ccount.p, coff.p, nagg, s);
    DBuf<int32_t> cand(ncand > 0 ? ncand : 1, s);
    FG_LAUNCH(induced_candidates_nodes_kernel, grid_for(n, 256), 256, 0, s, n, members.p, noff.p, xadj, adj, fine.p,
              cand.p);
    segmented_sort_i32(cand.p, coff.p, nagg, ucount.p, s);
    FG_LAUNCH(drop_padding_kernel, grid_for(nagg, 256), 256, 0, s, nagg, coff.p, ucount.p, cand.p);
    int64_t innz = exclusive_scan(ucount.p, ixadj.p, nagg, s);
    induced_nnz = innz;
    iadj.alloc(innz > 0 ? innz : 1, s);
    FG_LAUNCH(compact_segments_kernel, grid_for((int64_t)nagg * 32, 256), 256, 0, s, nagg, cand.p, coff.p, ixadj.p,
              iadj.p);
  }
  pt.mark("induced");
  // partitions of aggregates (aggregateWeightedGraph, weights = aggregate sizes)
  DBuf<int32_t> coarse;
  aggregate(c, nagg, ixadj.p, iadj.p, coarse_depth, true, 0, c.cfg.partitionMaxSize, n, acount.p, coarse);
  pt.mark("partitions");
  const int npart = reduce_max(coarse.p, nagg, s) + 1;
  // new aggregate ids: order (partition, old id)
  DBuf<int32_t> pcount(npart + 1, s), pcur(npart, s), old_of(nagg, s), new_id(nagg, s);
  pcount.zero();
  FG_LAUNCH(histogram_kernel, grid_for(nagg, 256), 256, 0, s, nagg, coarse.p, nullptr, pcount.p);
  o.part_idx.alloc(npart + 1, s);
  exclusive_scan_async(pcount.p, o.part_idx.p, npart, s);
  pcur.zero();
  FG_LAUNCH(scatter_bucket_kernel, grid_for(nagg, 256), 256, 0, s, nagg, coarse.p, o.part_idx.p, pcur.p, old_of.p);
  segmented_sort_i32(old_of.p, o.part_idx.p, npart, nullptr, s);
  FG_LAUNCH(invert_kernel, grid_for(nagg, 256), 256, 0, s, nagg, old_of.p, new_id.p);
  // next-level graph (remapInducedGraph, misHelpers.cu:1258-1280): rows in new order,
  // entries kept in their order and renamed
  DBuf<int32_t> rlen(nagg + 1, s);
  FG_LAUNCH(gather_len_kernel, grid_for(nagg, 256), 256, 0, s, nagg, old_of.p, ixadj.p, rlen.p);
  o.xadj_out.alloc(nagg + 1, s);
  exclusive_scan_async(rlen.p, o.xadj_out.p, nagg, s);
  o.nnz_out = induced_nnz;  // the same rows, reordered
  o.adj_out.alloc(o.nnz_out > 0 ? o.nnz_out : 1, s);
  FG_LAUNCH(remap_graph_kernel, grid_for(nagg, 256), 256, 0, s, nagg, old_of.p, ixadj.p, iadj.p, new_id.p,
            o.xadj_out.p, o.adj_out.p);
  // node order: aggregates in new order, members ascending
  DBuf<int32_t> asz(nagg + 1, s);
  FG_LAUNCH(gather_len_kernel, grid_for(nagg, 256), 256, 0, s, nagg, old_of.p, astart.p, asz.p);
  o.agg_idx.alloc(nagg + 1, s);
  exclusive_scan_async(asz.p, o.agg_idx.p, nagg, s);
  o.iperm.alloc(n, s);
  o.perm.alloc(n, s);
  o.agg_of.alloc(n, s);
  o.part_of_row.alloc(n, s);
  FG_LAUNCH(node_order_kernel, grid_for(nagg, 256), 256, 0, s, nagg, old_of.p, astart.p, members.p, o.agg_idx.p,
            coarse.p, o.iperm.p, o.agg_of.p, o.part_of_row.p);
  FG_LAUNCH(invert_kernel, grid_for(n, 256), 256, 0, s, n, o.iperm.p, o.perm.p);
  pt.mark("order");
  o.nagg = nagg;
  o.npart = npart;
}

// ---------------------------------------------------------------------------------
// Row-wise expand-sort-compress in shared memory.
//
// Each output row is generated as a list of (column, value) items in a fixed
// generation order, sorted stably by column, and every run of equal columns is
// summed left to right from its first item.  Modes:
//   PERMUTE  row i <- input row iperm[i], columns renamed by perm (no duplicates);
//   PROLONG  row i of Ap: items (agg_of[j], ((-omega) a_ij) / d_i), then (agg_of[i], 1)
//            (generateProlongatorFull_d, smoothedMG_amg_level.cu:321-387);
//   SPGEMM   row i of A*B: items (k, a_ij b_jk) for j ascending, then k ascending
//            (the product of generateNextLevelMatrixFull_d, :390-400).
// Pass 0 writes per-row item counts, pass 1 unique counts, pass 2 the row.
enum EscMode { ESC_PERMUTE = 0, ESC_PROLONG = 1, ESC_SPGEMM = 2 };

template <class T>
struct EscArgs {
  int n;
  const int32_t* arp;
  const int32_t* aci;
  const T* av;
  const int32_t* brp;
  const int32_t* bci;
  const T* bv;
  const int32_t* perm;   // PERMUTE: old->new column map (nullptr = identity)
  const int32_t* iperm;  // PERMUTE: output row -> input row (nullptr = identity)
  const int32_t* agg_of; // PROLONG
  const T* diag;         // PROLONG
  T neg_omega;           // PROLONG
  const int32_t* big_rows;  // block tier: list of rows
  int nbig;
  int32_t* counts;       // pass 0/1 output
  const int32_t* orp;    // pass 2: output row offsets
  int32_t* oci;
  T* ov;
  int32_t* overflow;
  int thread_cap;        // rows with at most this many items use the thread tier
  int64_t known_nnz;     // PERMUTE: the input's entry count (every entry is kept), else 0
};

constexpr int kEscWarpCap = 1024;
constexpr int kEscWarps = 4;
constexpr int kEscBlockCap = 8192;
constexpr int kEscBlockThreads = 512;

template <class T, int MODE>
__device__ __forceinline__ int esc_input_row(const EscArgs<T>& a, int i) {
  return (MODE == ESC_PERMUTE && a.iperm) ? a.iperm[i] : i;
}

// Number of items of row i.
template <class T, int MODE>
__device__ __forceinline__ int esc_row_items(const EscArgs<T>& a, int i) {
  int r = esc_input_row<T, MODE>(a, i);
  int b = a.arp[r], e = a.arp[r + 1];
  if (MODE == ESC_PERMUTE) return e - b;
  if (MODE == ESC_PROLONG) return e - b + 1;
  int s = 0;
  for (int q = b; q < e; q++) {
    int j = a.aci[q];
    s += a.brp[j + 1] - a.brp[j];
  }
  return s;
}

// Generates row i's items into keys (column << 32 | generation index) and vals.
// tid/nthr: cooperating threads; sync: their barrier.
template <class T, int MODE, class Sync>
__device__ void esc_generate(const EscArgs<T>& a, int i, unsigned long long* keys, T* vals, int tid, int nthr,
                             int* s_scan, Sync sync) {
  int r = esc_input_row<T, MODE>(a, i);
  int b = a.arp[r], e = a.arp[r + 1];
  if (MODE != ESC_SPGEMM) {
    for (int q = b + tid; q < e; q += nthr) {
      int g = q - b;
      int j = a.aci[q];
      int col;
      T v;
      if (MODE == ESC_PERMUTE) {
        col = a.perm ? a.perm[j] : j;
        v = a.av[q];
      } else {
        col = a.agg_of[j];
        T t = (a.neg_omega * a.av[q]) * (T)1;
        v = t / a.diag[i];
      }
      keys[g] = ((unsigned long long)(unsigned)col << 32) | (unsigned)g;
      vals[g] = v;
    }
    if (MODE == ESC_PROLONG && tid == 0) {
      int g = e - b;
      keys[g] = ((unsigned long long)(unsigned)a.agg_of[i] << 32) | (unsigned)g;
      vals[g] = (T)1;
    }
    return;
  }
  // SPGEMM: chunks of nthr A entries; offsets by an exclusive scan of B row lengths
  int base = 0;
  for (int c0 = b; c0 < e; c0 += nthr) {
    int q = c0 + tid;
    int len = 0, j = 0;
    if (q < e) {
      j = a.aci[q];
      len = a.brp[j + 1] - a.brp[j];
    }
    // block/warp exclusive scan of len via shared memory (nthr <= 512)
    s_scan[tid] = len;
    sync();
    for (int off = 1; off < nthr; off <<= 1) {
      int add = tid >= off ? s_scan[tid - off] : 0;
      sync();
      s_scan[tid] += add;
      sync();
    }
    int excl = s_scan[tid] - len;
    int total = s_scan[nthr - 1];
    sync();
    if (q < e) {
      T av = a.av[q];
      int jb = a.brp[j];
      for (int t = 0; t < len; t++) {
        int g = base + excl + t;
        keys[g] = ((unsigned long long)(unsigned)a.bci[jb + t] << 32) | (unsigned)g;
        vals[g] = av * a.bv[jb + t];
      }
    }
    base += total;
  }
}

// After sorting: count (pass 1) or write (pass 2) the reduced row.  Heads are the
// first item of each column run; each head's thread sums its run left to right.
// Heads are ranked by warp ballots plus an exclusive scan over the warps.
template <class T, class Sync>
__device__ int esc_reduce(const unsigned long long* keys, const T* vals_by_gen, int len, int tid, int nthr,
                          int* s_warp /* >= nthr/32 + 1 ints */, int32_t* oci, T* ov, bool write, Sync sync) {
  const int lane = tid & 31, w = tid >> 5, nw = (nthr + 31) >> 5;
  int total = 0;
  for (int c0 = 0; c0 < len; c0 += nthr) {
    const int p = c0 + tid;
    const bool head = p < len && (p == 0 || (keys[p] >> 32) != (keys[p - 1] >> 32));
    const unsigned m = __ballot_sync(0xffffffffu, head);
    int rank = __popc(m & ((1u << lane) - 1u)), chunk = __popc(m);
    if (nw > 1) {
      if (lane == 0) s_warp[w] = chunk;
      sync();
      if (tid == 0) {
        int t = 0;
        for (int k = 0; k < nw; k++) {
          int v = s_warp[k];
          s_warp[k] = t;
          t += v;
        }
        s_warp[nw] = t;
      }
      sync();
      rank += s_warp[w];
      chunk = s_warp[nw];
    }
    if (head && write) {
      const unsigned col = (unsigned)(keys[p] >> 32);
      T sum = vals_by_gen[(unsigned)(keys[p] & 0xffffffffu)];
      for (int q = p + 1; q < len && (unsigned)(keys[q] >> 32) == col; q++)
        sum = sum + vals_by_gen[(unsigned)(keys[q] & 0xffffffffu)];
      oci[total + rank] = (int32_t)col;
      ov[total + rank] = sum;
    }
    total += chunk;
    sync();
  }
  return total;
}

template <class T, int MODE>
__global__ void esc_count_items_kernel(EscArgs<T> a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) a.counts[i] = esc_row_items<T, MODE>(a, i);
}

__global__ void collect_big_rows_kernel(int n, const int32_t* items, int cap, int hard_cap, int32_t* list,
                                        int32_t* nlist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && items[i] > cap && items[i] <= hard_cap) list[atomicAdd(nlist, 1)] = i;
}

template <class T, int MODE, bool WRITE>
__global__ void esc_warp_kernel(EscArgs<T> a, const int32_t* items) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw) + (size_t)w * kEscWarpCap;
  T* vals = reinterpret_cast<T*>(reinterpret_cast<unsigned long long*>(smem_raw) + (size_t)kEscWarps * kEscWarpCap) +
            (size_t)w * kEscWarpCap;
  __shared__ int s_scan[kEscWarps][32];
  __shared__ int s_cnt[kEscWarps];
  for (int i = blockIdx.x * kEscWarps + w; i < a.n; i += gridDim.x * kEscWarps) {
    int len = items[i];
    if (len > kEscWarpCap || len <= a.thread_cap) continue;
    esc_generate<T, MODE>(a, i, keys, vals, lane, 32, s_scan[w], WarpSync());
    int np2 = next_pow2(len < 2 ? 2 : len);
    for (int p = len + lane; p < np2; p += 32) keys[p] = ~0ull;
    __syncwarp();
    bitonic_sort_shared(keys, np2, lane, 32, WarpSync());
    int out = WRITE ? a.orp[i] : 0;
    int cnt = esc_reduce<T>(keys, vals, len, lane, 32, &s_cnt[w], WRITE ? a.oci + out : nullptr,
                            WRITE ? a.ov + out : nullptr, WRITE, WarpSync());
    if (!WRITE && lane == 0) a.counts[i] = cnt;
    __syncwarp();
  }
}

template <class T, int MODE, bool WRITE>
__global__ void esc_block_kernel(EscArgs<T> a, const int32_t* items) {
  extern __shared__ unsigned char smem_raw[];
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem_raw);
  T* vals = reinterpret_cast<T*>(keys + kEscBlockCap);
  __shared__ int s_scan[kEscBlockThreads];
  __shared__ int s_cnt[kEscBlockThreads / 32 + 1];
  for (int b = blockIdx.x; b < a.nbig; b += gridDim.x) {
    int i = a.big_rows[b];
    int len = items[i];
    esc_generate<T, MODE>(a, i, keys, vals, threadIdx.x, blockDim.x, s_scan, BlockSync());
    int np2 = next_pow2(len);
    for (int p = len + threadIdx.x; p < np2; p += blockDim.x) keys[p] = ~0ull;
    __syncthreads();
    bitonic_sort_shared(keys, np2, threadIdx.x, blockDim.x, BlockSync());
    int out = WRITE ? a.orp[i] : 0;
    int cnt = esc_reduce<T>(keys, vals, len, threadIdx.x, blockDim.x, s_cnt, WRITE ? a.oci + out : nullptr,
                            WRITE ? a.ov + out : nullptr, WRITE, BlockSync());
    if (!WRITE && threadIdx.x == 0) a.counts[i] = cnt;
    __syncthreads();
  }
}

// Rows beyond the shared-memory sort capacity (they appear only on coarse levels,
// where the column count is small): one block per row, a dense accumulator over
// the output columns; thread 0 walks the items in generation order (so every
// column is summed left to right from its first item), then the block compacts
// the touched columns in ascending order.
template <class T, int MODE>
__device__ void esc_dense_row(const EscArgs<T>& a, int i, T* acc, unsigned char* mark, int ncols) {
  auto add = [&](int col, T v) {
    if (!mark[col]) {
      mark[col] = 1;
      acc[col] = v;
    } else {
      acc[col] = acc[col] + v;
    }
  };
  int r = esc_input_row<T, MODE>(a, i);
  int b = a.arp[r], e = a.arp[r + 1];
  for (int q = b; q < e; q++) {
    int j = a.aci[q];
    if (MODE == ESC_PERMUTE) {
      add(a.perm ? a.perm[j] : j, a.av[q]);
    } else if (MODE == ESC_PROLONG) {
      T t = (a.neg_omega * a.av[q]) * (T)1;
      add(a.agg_of[j], t / a.diag[i]);
    } else {
      T av = a.av[q];
      for (int f = a.brp[j]; f < a.brp[j + 1]; f++) add(a.bci[f], av * a.bv[f]);
    }
  }
  if (MODE == ESC_PROLONG) add(a.agg_of[i], (T)1);
}

template <class T, int MODE, bool WRITE>
__global__ void esc_dense_kernel(EscArgs<T> a, int ncols, T* gacc, unsigned char* gmark) {
  extern __shared__ unsigned char smem_raw[];
  const bool shared = gacc == nullptr;
  __shared__ int s_total;
  __shared__ int s_warp[32];
  for (int bi = blockIdx.x; bi < a.nbig; bi += gridDim.x) {
    int i = a.big_rows[bi];
    T* acc = shared ? reinterpret_cast<T*>(smem_raw) : gacc + (size_t)blockIdx.x * ncols;
    unsigned char* mark = shared ? smem_raw + (size_t)ncols * sizeof(T) : gmark + (size_t)blockIdx.x * ncols;
    for (int q = threadIdx.x; q < ncols; q += blockDim.x) mark[q] = 0;
    __syncthreads();
    if (threadIdx.x == 0) esc_dense_row<T, MODE>(a, i, acc, mark, ncols);
    __syncthreads();
    // ordered compaction of marked columns
    int base = 0;
    int out = WRITE ? a.orp[i] : 0;
    for (int c0 = 0; c0 < ncols; c0 += blockDim.x) {
      int q = c0 + threadIdx.x;
      int m = (q < ncols && mark[q]) ? 1 : 0;
      unsigned bal = __ballot_sync(0xffffffffu, m);
      int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      if (lane == 0) s_warp[w] = __popc(bal);
      __syncthreads();
      if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
          int v = s_warp[k];
          s_warp[k] = t;
          t += v;
        }
        s_total = t;
      }
      __syncthreads();
      if (m && WRITE) {
        int pos = base + s_warp[w] + __popc(bal & ((1u << lane) - 1u));
        a.oci[out + pos] = q;
        a.ov[out + pos] = acc[q];
      }
      base += s_total;
      __syncthreads();
    }
    if (!WRITE && threadIdx.x == 0) a.counts[i] = base;
    __syncthreads();
  }
}

__global__ void collect_dense_rows_kernel(int n, const int32_t* items, int cap, int32_t* list, int32_t* nlist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && items[i] > cap) list[atomicAdd(nlist, 1)] = i;
}

// ---- thread tier: short PERMUTE / PROLONG rows, one thread per row -----------------
// Items are generated in order and merged into a sorted local list; a repeated
// column adds to its running sum (left to right from the first item).
constexpr int kThreadRowCap = 16;

// Bitonic network on N register-resident (key, value) pairs; every index is a
// compile-time constant after unrolling, so nothing spills to local memory.
template <class T, int N>
__device__ __forceinline__ void sort_network(unsigned long long (&k)[N], T (&v)[N]) {
#pragma unroll
  for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
      for (int i = 0; i < N; i++) {
        const int j = i ^ stride;
        if (j > i) {
          const bool asc = (i & size) == 0;
          if ((k[i] > k[j]) == asc) {
            unsigned long long tk = k[i];
            k[i] = k[j];
            k[j] = tk;
            T tv = v[i];
            v[i] = v[j];
            v[j] = tv;
          }
        }
      }
    }
  }
}

template <class T, int MODE, bool WRITE>
__global__ void esc_thread_kernel(EscArgs<T> a, const int32_t* items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int len = items[i];
  if (len > kThreadRowCap) return;
  unsigned long long key[kThreadRowCap];
  T val[kThreadRowCap];
  const int r = esc_input_row<T, MODE>(a, i);
  const int rb = a.arp[r], re = a.arp[r + 1];
#pragma unroll
  for (int g = 0; g < kThreadRowCap; g++) {
    key[g] = ~0ull;
    val[g] = (T)0;
    const int q = rb + g;
    if (q < re) {
      const int j = a.aci[q];
      int col;
      T v;
      if (MODE == ESC_PERMUTE) {
        col = a.perm ? a.perm[j] : j;
        v = a.av[q];
      } else {
        col = a.agg_of[j];
        T t = (a.neg_omega * a.av[q]) * (T)1;
        v = t / a.diag[i];
      }
      key[g] = ((unsigned long long)(unsigned)col << 32) | (unsigned)g;
      val[g] = v;
    } else if (MODE == ESC_PROLONG && q == re) {
      key[g] = ((unsigned long long)(unsigned)a.agg_of[i] << 32) | (unsigned)g;
      val[g] = (T)1;
    }
  }
  sort_network<T, kThreadRowCap>(key, val);
  // runs of equal columns summed left to right (generation order within the run)
  const int o = WRITE ? a.orp[i] : 0;
  int u = 0;
  unsigned cur = 0xffffffffu;
  T sum = (T)0;
#pragma unroll
  for (int g = 0; g < kThreadRowCap; g++) {
    if (key[g] == ~0ull) continue;
    const unsigned col = (unsigned)(key[g] >> 32);
    if (col != cur) {
      if (cur != 0xffffffffu) {
        if (WRITE) {
          a.oci[o + u] = (int32_t)cur;
          a.ov[o + u] = sum;
        }
        u++;
      }
      cur = col;
      sum = val[g];
    } else {
      sum = sum + val[g];
    }
  }
  if (cur != 0xffffffffu) {
    if (WRITE) {
      a.oci[o + u] = (int32_t)cur;
      a.ov[o + u] = sum;
    }
    u++;
  }
  if (!WRITE) a.counts[i] = u;
}

template <class T, int MODE>
void run_esc_sort(Ctx& c, EscArgs<T> a, int nrows_out, int ncols_out, DCsr<T>& out) {
  cudaStream_t s = c.stream;
  a.n = nrows_out;
  DBuf<int32_t> items(nrows_out + 1, s), ucnt(nrows_out + 1, s), big(nrows_out + 1, s), nbig(1, s);
  DBuf<int32_t> dense(nrows_out + 1, s), ndense(1, s);
  nbig.zero();
  ndense.zero();
  a.counts = items.p;
  FG_LAUNCH((esc_count_items_kernel<T, MODE>), grid_for(nrows_out, 256), 256, 0, s, a);
  FG_LAUNCH(collect_big_rows_kernel, grid_for(nrows_out, 256), 256, 0, s, nrows_out, items.p, kEscWarpCap,
            kEscBlockCap, big.p, nbig.p);
  FG_LAUNCH(collect_dense_rows_kernel, grid_for(nrows_out, 256), 256, 0, s, nrows_out, items.p, kEscBlockCap,
            dense.p, ndense.p);
  int32_t h_big = 0, h_dense = 0;  // both counts in one round trip
  FG_CUDA(cudaMemcpyAsync(&h_big, nbig.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(&h_dense, ndense.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  a.nbig = h_big;
  a.big_rows = big.p;
  EscArgs<T> ad = a;  // dense tier: rows with more items than the sort capacity
  ad.nbig = h_dense;
  ad.big_rows = dense.p;
  const int dgrid = std::min(ad.nbig, 152 * 2);
  const size_t dsm = (size_t)ncols_out * (sizeof(T) + 1);
  const bool dense_shared = dsm <= 200 * 1024;
  DBuf<T> gacc;
  DBuf<unsigned char> gmark;
  if (ad.nbig > 0 && !dense_shared) {
    FG_REQUIRE((size_t)dgrid * ncols_out * (sizeof(T) + 1) <= ((size_t)8 << 30), FEMGPU_ERR_LIMIT,
               "dense accumulator for long SpGEMM rows exceeds 8 GB");
    gacc.alloc((size_t)dgrid * ncols_out, s);
    gmark.alloc((size_t)dgrid * ncols_out, s);
  }
  if (ad.nbig > 0 && dense_shared && dsm > 48 * 1024) {
    ensure_smem(esc_dense_kernel<T, MODE, false>, dsm);
    ensure_smem(esc_dense_kernel<T, MODE, true>, dsm);
  }
  const size_t wsm = (size_t)kEscWarps * kEscWarpCap * (sizeof(unsigned long long) + sizeof(T));
  const size_t bsm = (size_t)kEscBlockCap * (sizeof(unsigned long long) + sizeof(T));
  static bool attr_set = false;
  if (!attr_set) {
    ensure_smem(esc_warp_kernel<T, MODE, false>, wsm);
    ensure_smem(esc_warp_kernel<T, MODE, true>, wsm);
    ensure_smem(esc_block_kernel<T, MODE, false>, bsm);
    ensure_smem(esc_block_kernel<T, MODE, true>, bsm);
    attr_set = true;
  }
  const int wgrid = std::min<int64_t>((nrows_out + kEscWarps - 1) / kEscWarps, 152 * 64);
  a.counts = ucnt.p;
  a.thread_cap = kThreadRowCap;
  // a permuted row has no repeated column: its output length is its item count, so the
  // counting pass is needed only for the prolongator
  if (MODE != ESC_PERMUTE) {
    FG_LAUNCH((esc_thread_kernel<T, MODE, false>), grid_for(nrows_out, 128), 128, 0, s, a, items.p);
    FG_LAUNCH((esc_warp_kernel<T, MODE, false>), wgrid, 32 * kEscWarps, wsm, s, a, items.p);
    if (a.nbig > 0)
      FG_LAUNCH((esc_block_kernel<T, MODE, false>), std::min(a.nbig, 152 * 2), kEscBlockThreads, bsm, s, a,
                items.p);
    if (ad.nbig > 0) {
      ad.counts = ucnt.p;
      FG_LAUNCH((esc_dense_kernel<T, MODE, false>), dgrid, 256, dense_shared ? dsm : 0, s, ad, ncols_out, gacc.p,
                gmark.p);
    }
  }
  out.n = nrows_out;
  out.m = ncols_out;
  out.rp.alloc(nrows_out + 1, s);
  if (MODE == ESC_PERMUTE && a.known_nnz > 0) {  // a permutation keeps every entry: no read-back
    exclusive_scan_async(items.p, out.rp.p, nrows_out, s);
    out.nnz = a.known_nnz;
  } else {
    out.nnz = exclusive_scan(MODE == ESC_PERMUTE ? items.p : ucnt.p, out.rp.p, nrows_out, s);
  }
  out.ci.alloc(out.nnz > 0 ? out.nnz : 1, s);
  out.v.alloc(out.nnz > 0 ? out.nnz : 1, s);
  a.orp = out.rp.p;
  a.oci = out.ci.p;
  a.ov = out.v.p;
  FG_LAUNCH((esc_thread_kernel<T, MODE, true>), grid_for(nrows_out, 128), 128, 0, s, a, items.p);
  FG_LAUNCH((esc_warp_kernel<T, MODE, true>), wgrid, 32 * kEscWarps, wsm, s, a, items.p);
  if (a.nbig > 0)
    FG_LAUNCH((esc_block_kernel<T, MODE, true>), std::min(a.nbig, 152 * 2), kEscBlockThreads, bsm, s, a, items.p);
  if (ad.nbig > 0) {
    ad.orp = out.rp.p;
    ad.oci = out.ci.p;
    ad.ov = out.v.p;
    FG_LAUNCH((esc_dense_kernel<T, MODE, true>), dgrid, 256, dense_shared ? dsm : 0, s, ad, ncols_out, gacc.p,
              gmark.p);
  }
}


// ---- hash SpGEMM: C = A B, row by row ----------------------------------------------
// A row's products are visited one A entry at a time; the entries of one B row have
// distinct columns, so every column receives at most one product per step and the
// threads of a step never touch the same accumulator.  Steps run in order, so each
// column is summed left to right in generation order starting from its first
// product -- the same value as the sort-based expand-sort-compress.  The unique
// columns are then sorted (bitonic, in shared memory) and written to the row's slot
// of a temporary buffer; rows whose unique count exceeds the table go to a larger
// tier.
constexpr int kHashWarpCap = 256;
constexpr int kHashWarps = 8;
constexpr int kHashBlockCap = 4096;
constexpr int kHashBlockThreads = 256;

__device__ __forceinline__ unsigned hash_col(unsigned c) { return (c * 2654435761u) >> 7; }

template <class T, class Sync>
__device__ bool hash_row_accumulate(const EscArgs<T>& a, int i, int32_t* hk, T* hv, int cap, int tid, int nth,
                                    int* s_flag, Sync sync) {
  for (int q = tid; q < cap; q += nth) hk[q] = -1;
  if (tid == 0) *s_flag = 0;
  sync();
  for (int e = a.arp[i]; e < a.arp[i + 1]; e++) {
    const int j = a.aci[e];
    const T av = a.av[e];
    const int fb = a.brp[j], fe = a.brp[j + 1];
    for (int f0 = fb; f0 < fe; f0 += nth) {
      const int f = f0 + tid;
      if (f < fe && *s_flag == 0) {
        const int col = a.bci[f];
        const T v = av * a.bv[f];
        unsigned slot = hash_col((unsigned)col) & (unsigned)(cap - 1);
        for (int probes = 0;; probes++) {
          if (probes >= cap) {
            *s_flag = 1;
            break;
          }
          int k = hk[slot];
          if (k == -1) {
            int prev = atomicCAS(&hk[slot], -1, col);
            if (prev == -1) {
              hv[slot] = v;
              break;
            }
            k = prev;
          }
          if (k == col) {
            hv[slot] = hv[slot] + v;
            break;
          }
          slot = (slot + 1) & (unsigned)(cap - 1);
        }
      }
      sync();
    }
  }
  return *s_flag == 0;
}

// Collects the occupied slots as (column << 32 | slot) keys, sorts them and writes
// the row; returns the unique count.  nth threads, warp-ballot compaction.
template <class T, class Sync>
__device__ int hash_row_emit(const int32_t* hk, const T* hv, unsigned long long* lst, int cap, int tid, int nth,
                             int* s_warp, int32_t* oci, T* ov, Sync sync) {
  const int lane = tid & 31, w = tid >> 5, nw = (nth + 31) >> 5;
  int total = 0;
  for (int c0 = 0; c0 < cap; c0 += nth) {
    const int q = c0 + tid;
    const bool occ = q < cap && hk[q] != -1;
    const unsigned m = __ballot_sync(0xffffffffu, occ);
    int rank = __popc(m & ((1u << lane) - 1u)), chunk = __popc(m);
    if (nw > 1) {
      if (lane == 0) s_warp[w] = chunk;
      sync();
      if (tid == 0) {
        int t = 0;
        for (int k = 0; k < nw; k++) {
          int v = s_warp[k];
          s_warp[k] = t;
          t += v;
        }
        s_warp[nw] = t;
      }
      sync();
      rank += s_warp[w];
      chunk = s_warp[nw];
    }
    if (occ) lst[total + rank] = ((unsigned long long)(unsigned)hk[q] << 32) | (unsigned)q;
    total += chunk;
    sync();
  }
  const int np2 = next_pow2(total < 2 ? 2 : total);
  for (int p = total + tid; p < np2; p += nth) lst[p] = ~0ull;
  sync();
  bitonic_sort_shared(lst, np2, tid, nth, sync);
  for (int p = tid; p < total; p += nth) {
    oci[p] = (int32_t)(lst[p] >> 32);
    ov[p] = hv[(unsigned)(lst[p] & 0xffffffffu)];
  }
  sync();
  return total;
}

// Warp tier: 32 products per step in generation order (A entries of the row taken 32
// at a time, their B rows flattened by a warp scan).  Lanes holding the same column
// are grouped with __match_any_sync; the group's lowest lane adds the group's
// products to the accumulator in lane order, so each column is still summed left
// to right in generation order.
template <class T>
__device__ bool hash_row_accumulate_matched(const EscArgs<T>& a, int i, int32_t* hk, T* hv, T* sv, int cap,
                                            int lane, int* s_flag) {
  for (int q = lane; q < cap; q += 32) hk[q] = -1;
  if (lane == 0) *s_flag = 0;
  __syncwarp();
  const int rb = a.arp[i], re = a.arp[i + 1];
  for (int eb = rb; eb < re; eb += 32) {
    const int e = eb + lane;
    int j = 0, len = 0;
    T av = (T)0;
    if (e < re) {
      j = a.aci[e];
      av = a.av[e];
      len = a.brp[j + 1] - a.brp[j];
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int jb = e < re ? a.brp[j] : 0;
    for (int g0 = 0; g0 < total; g0 += 32) {
      const int g = g0 + lane;
      const bool live = g < total;
      int owner = 0;
#pragma unroll
      for (int st = 16; st > 0; st >>= 1) {
        int probe = __shfl_sync(0xffffffffu, incl, owner + st - 1);
        if (probe <= g) owner += st;
      }
      owner = owner > 31 ? 31 : owner;
      const int o_incl = __shfl_sync(0xffffffffu, incl, owner);
      const int o_len = __shfl_sync(0xffffffffu, len, owner);
      const int o_jb = __shfl_sync(0xffffffffu, jb, owner);
      const T o_av = __shfl_sync(0xffffffffu, av, owner);
      int col = -1;
      T v = (T)0;
      if (live) {
        const int f = o_jb + (g - (o_incl - o_len));
        col = a.bci[f];
        v = o_av * a.bv[f];
      }
      sv[lane] = v;
      const unsigned peers = __match_any_sync(0xffffffffu, col);
      __syncwarp();
      const bool leader = live && (__ffs(peers) - 1) == lane;
      if (leader && *s_flag == 0) {
        unsigned slot = hash_col((unsigned)col) & (unsigned)(cap - 1);
        int found = -1;
        bool fresh = false;
        for (int probes = 0; probes < cap; probes++) {
          int k = hk[slot];
          if (k == -1) {
            int prev = atomicCAS(&hk[slot], -1, col);
            if (prev == -1) {
              found = (int)slot;
              fresh = true;
              break;
            }
            k = prev;
          }
          if (k == col) {
            found = (int)slot;
            break;
          }
          slot = (slot + 1) & (unsigned)(cap - 1);
        }
        if (found < 0) {
          *s_flag = 1;
        } else {
          unsigned m = peers;
          T acc = fresh ? sv[__ffs(m) - 1] : hv[found] + sv[__ffs(m) - 1];
          m &= m - 1;
          while (m) {
            acc = acc + sv[__ffs(m) - 1];
            m &= m - 1;
          }
          hv[found] = acc;
        }
      }
      __syncwarp();
    }
  }
  return *s_flag == 0;
}

// Galerkin-product rows with few distinct columns: one thread per row keeps up to
// kRowSlots (column, value) pairs in shared memory and adds every product to its
// column's slot in generation order (entries of the left row in order, each times
// the right row in order), the first product of a column starting its slot; rows
// with more distinct columns are listed for the warp tier.  Same sums as the hash
// tiers, sorted by column on output.
constexpr int kRowSlots = 32;
constexpr int kRowThreads = 128;

template <class T>
__global__ void __launch_bounds__(kRowThreads) spgemm_row_kernel(EscArgs<T> a, const int32_t* toff, int32_t* tci,
                                                                 T* tv, int32_t* counts, int32_t* over,
                                                                 int32_t* nover) {
  __shared__ int32_t sc[kRowSlots][kRowThreads];
  __shared__ T sv[kRowSlots][kRowThreads];
  const int t = threadIdx.x;
  const int i = blockIdx.x * blockDim.x + t;
  if (i >= a.n) return;
  int u = 0;
  bool overflow = false;
  const int ea = a.arp[i], eb = a.arp[i + 1];
  for (int e0 = ea; e0 < eb && !overflow; e0 += 8) {
    // 8 left entries at a time: their columns, values and right-row ranges are loaded
    // before the products (which then run in generation order)
    int kk[8], fb[8], fe[8];
    T avv[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      kk[q] = e0 + q < eb ? a.aci[e0 + q] : 0;
      avv[q] = e0 + q < eb ? a.av[e0 + q] : (T)0;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      fb[q] = e0 + q < eb ? a.brp[kk[q]] : 0;
      fe[q] = e0 + q < eb ? a.brp[kk[q] + 1] : 0;
    }
    for (int m = 0; m < 8 && !overflow; m++)
    for (int f = fb[m]; f < fe[m]; f++) {
      const int j = a.bci[f];
      const T p = avv[m] * a.bv[f];
      int q = 0;
      while (q < u && sc[q][t] != j) q++;
      if (q < u) {
        sv[q][t] = sv[q][t] + p;
      } else if (u < kRowSlots) {
        sc[u][t] = j;
        sv[u][t] = p;
        u++;
      } else {
        overflow = true;
        break;
      }
    }
  }
  if (overflow) {
    over[atomicAdd(nover, 1)] = i;
    counts[i] = 0;
    return;
  }
  for (int q = 1; q < u; q++) {
    const int cj = sc[q][t];
    const T vj = sv[q][t];
    int p = q - 1;
    while (p >= 0 && sc[p][t] > cj) {
      sc[p + 1][t] = sc[p][t];
      sv[p + 1][t] = sv[p][t];
      p--;
    }
    sc[p + 1][t] = cj;
    sv[p + 1][t] = vj;
  }
  const int o = toff[i];
  for (int q = 0; q < u; q++) {
    tci[o + q] = sc[q][t];
    tv[o + q] = sv[q][t];
  }
  counts[i] = u;
}

// Rows `rows[0 .. *nrows)` (all rows when rows == nullptr), one warp per row.
template <class T>
__global__ void hash_warp_kernel(EscArgs<T> a, const int32_t* rows, const int32_t* nrows, const int32_t* toff,
                                 int32_t* tci, T* tv, int32_t* counts, int32_t* over, int32_t* nover) {
  __shared__ int32_t hk[kHashWarps][kHashWarpCap];
  __shared__ T hv[kHashWarps][kHashWarpCap];
  __shared__ unsigned long long lst[kHashWarps][kHashWarpCap];
  __shared__ T sv[kHashWarps][32];
  __shared__ int s_flag[kHashWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nr = rows ? *nrows : a.n;
  for (int ii = blockIdx.x * kHashWarps + w; ii < nr; ii += gridDim.x * kHashWarps) {
    const int i = rows ? rows[ii] : ii;
    bool ok = hash_row_accumulate_matched<T>(a, i, hk[w], hv[w], sv[w], kHashWarpCap, lane, &s_flag[w]);
    if (!ok) {
      if (lane == 0) {
        over[atomicAdd(nover, 1)] = i;
        counts[i] = 0;
      }
      __syncwarp();
      continue;
    }
    int u = hash_row_emit<T>(hk[w], hv[w], lst[w], kHashWarpCap, lane, 32, nullptr, tci + toff[i], tv + toff[i],
                             WarpSync());
    if (lane == 0) counts[i] = u;
    __syncwarp();
  }
}

template <class T>
__global__ void hash_block_kernel(EscArgs<T> a, const int32_t* rows, int nrows, const int32_t* toff, int32_t* tci,
                                  T* tv, int32_t* counts, int32_t* over, int32_t* nover) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* lst = reinterpret_cast<unsigned long long*>(smem_raw);
  T* hv = reinterpret_cast<T*>(lst + kHashBlockCap);
  int32_t* hk = reinterpret_cast<int32_t*>(hv + kHashBlockCap);
  __shared__ int s_flag;
  __shared__ int s_warp[kHashBlockThreads / 32 + 1];
  for (int b = blockIdx.x; b < nrows; b += gridDim.x) {
    const int i = rows[b];
    bool ok = hash_row_accumulate<T>(a, i, hk, hv, kHashBlockCap, threadIdx.x, blockDim.x, &s_flag, BlockSync());
    if (!ok) {
      if (threadIdx.x == 0) {
        over[atomicAdd(nover, 1)] = i;
        counts[i] = 0;
      }
      __syncthreads();
      continue;
    }
    int u = hash_row_emit<T>(hk, hv, lst, kHashBlockCap, threadIdx.x, blockDim.x, s_warp, tci + toff[i],
                             tv + toff[i], BlockSync());
    if (threadIdx.x == 0) counts[i] = u;
    __syncthreads();
  }
}

// Galerkin-product rows of a narrow product (at most kDenseCols output columns, few
// rows): one warp per row with a dense accumulator over the output columns in shared
// memory.  The left row's entries are taken in order, and for each of them the lanes take
// the right row's entries, whose columns are distinct; so every column is summed in
// generation order, its first product starting the sum -- the sums of the hash tiers,
// without their probing.  Columns are listed as they are first hit, the list is sorted,
// and the row is written in ascending column order into its temporary slots.
constexpr int kDenseCols = 4096;
template <class T>
__host__ __device__ inline size_t dense_warp_smem(int ncols) {
  const size_t acc = ((size_t)ncols * sizeof(T) + 15) / 16 * 16;
  const size_t list = (size_t)next_pow2(ncols < 2 ? 2 : ncols) * sizeof(int32_t);
  const size_t mark = ((size_t)ncols + 15) / 16 * 16;
  return acc + list + mark;
}

template <class T>
__global__ void spgemm_dense_warp_kernel(EscArgs<T> a, int ncols, const int32_t* __restrict__ toff,
                                         int32_t* __restrict__ tci, T* __restrict__ tv, int32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t per = dense_warp_smem<T>(ncols);
  unsigned char* base = smem_raw + (size_t)w * per;
  T* acc = reinterpret_cast<T*>(base);
  int32_t* list = reinterpret_cast<int32_t*>(base + ((size_t)ncols * sizeof(T) + 15) / 16 * 16);
  const int cap = next_pow2(ncols < 2 ? 2 : ncols);
  unsigned char* mark = reinterpret_cast<unsigned char*>(list + cap);
  for (int k = lane; k < ncols; k += 32) mark[k] = 0;
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
  // adds product v to column col (lanes hold distinct columns within one right row)
  int nt = 0;
  auto add = [&](bool live, int col, T v) {
    const bool fresh = live && mark[col] == 0;
    if (fresh) {
      mark[col] = 1;
      acc[col] = v;
    } else if (live) {
      acc[col] = acc[col] + v;
    }
    const unsigned m = __ballot_sync(0xffffffffu, fresh);
    if (fresh) list[nt + __popc(m & below)] = col;
    nt += __popc(m);
  };
  for (int i = blockIdx.x * nw + w; i < a.n; i += gridDim.x * nw) {
    nt = 0;
    const int qb = a.arp[i], qe = a.arp[i + 1];
    // the left row in chunks of 32 entries: lane t holds entry q0 + t's value and right
    // row bounds; each right row's first 32 entries are loaded one entry ahead
    for (int q0 = qb; q0 < qe; q0 += 32) {
      const int nq = min(32, qe - q0);
      T avq = (T)0;
      int bs = 0, be = 0;
      if (lane < nq) {
        const int j = a.aci[q0 + lane];
        avq = a.av[q0 + lane];
        bs = a.brp[j];
        be = a.brp[j + 1];
      }
      int b0 = __shfl_sync(0xffffffffu, bs, 0), b1 = __shfl_sync(0xffffffffu, be, 0);
      int ncol = b0 + lane < b1 ? a.bci[b0 + lane] : 0;
      T nval = b0 + lane < b1 ? a.bv[b0 + lane] : (T)0;
      for (int u = 0; u < nq; u++) {
        const T av = __shfl_sync(0xffffffffu, avq, u);
        const int c0 = ncol;
        const T v0 = nval;
        const int cb0 = b0, cb1 = b1;
        if (u + 1 < nq) {
          b0 = __shfl_sync(0xffffffffu, bs, u + 1);
          b1 = __shfl_sync(0xffffffffu, be, u + 1);
          ncol = b0 + lane < b1 ? a.bci[b0 + lane] : 0;
          nval = b0 + lane < b1 ? a.bv[b0 + lane] : (T)0;
        }
        add(cb0 + lane < cb1, c0, av * v0);
        __syncwarp();
        for (int f = cb0 + 32 + lane; f - lane < cb1; f += 32) {
          const bool live = f < cb1;
          add(live, live ? a.bci[f] : 0, live ? av * a.bv[f] : (T)0);
          __syncwarp();
        }
      }
    }
    const int np2 = next_pow2(nt < 2 ? 2 : nt);
    for (int t = nt + lane; t < np2; t += 32) list[t] = INT32_MAX;
    __syncwarp();
    bitonic_sort_shared(list, np2, lane, 32, WarpSync());
    const int o = toff[i];
    for (int t = lane; t < nt; t += 32) {
      const int col = list[t];
      tci[o + t] = col;
      tv[o + t] = acc[col];
      mark[col] = 0;
    }
    if (lane == 0) counts[i] = nt;
    __syncwarp();
  }
}

__global__ void spgemm_capacity_kernel(int n, const int32_t* items, int ncols, int32_t* cap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cap[i] = min(items[i], ncols);
}

// Rows from their capacity-spaced temporary slots to the compact CSR: G lanes per row
// (G near the average row length, so short rows do not leave most of a warp idle).
template <class T, int G>
__global__ void compact_rows_copy_kernel(int n, const int32_t* toff, const int32_t* tci, const T* tv,
                                         const int32_t* orp, int32_t* oci, T* ov) {
  const int lane = threadIdx.x & (G - 1);
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) / G; i < n; i += (gridDim.x * blockDim.x) / G) {
    const int o = orp[i], len = orp[i + 1] - o, src = toff[i];
    for (int t = lane; t < len; t += G) {
      oci[o + t] = tci[src + t];
      ov[o + t] = tv[src + t];
    }
  }
}

template <class T>
void run_spgemm_hash(Ctx& c, EscArgs<T> a, int nrows_out, int ncols_out, DCsr<T>& out) {
  cudaStream_t s = c.stream;
  PhaseTimer pt(s, -2);
  a.n = nrows_out;
  DBuf<int32_t> items(nrows_out + 1, s), capv(nrows_out + 1, s), toff(nrows_out + 1, s), cnt(nrows_out + 1, s);
  a.counts = items.p;
  FG_LAUNCH((esc_count_items_kernel<T, ESC_SPGEMM>), grid_for(nrows_out, 256), 256, 0, s, a);
  FG_LAUNCH(spgemm_capacity_kernel, grid_for(nrows_out, 256), 256, 0, s, nrows_out, items.p, ncols_out, capv.p);
  const int64_t tcap = exclusive_scan(capv.p, toff.p, nrows_out, s);
  FG_REQUIRE(tcap < INT32_MAX, FEMGPU_ERR_LIMIT, "SpGEMM temporary exceeds int32 indexing");
  DBuf<int32_t> tci(tcap > 0 ? tcap : 1, s);
  DBuf<T> tv(tcap > 0 ? tcap : 1, s);
  pt.mark("sp items");
  DBuf<int32_t> over1(nrows_out + 1, s), nover1(1, s), over2(nrows_out + 1, s), nover2(1, s);
  nover1.zero();
  nover2.zero();
  const int wgrid = std::min<int64_t>((nrows_out + kHashWarps - 1) / kHashWarps, 152 * 32);
  const size_t dper = dense_warp_smem<T>(ncols_out);
  if (nrows_out < 65536 && ncols_out <= kDenseCols) {
    // a narrow product: every row on the dense accumulator tier (no overflow rows)
    const int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (size_t)(200 * 1024) / dper));
    const size_t dsm = (size_t)wpb * dper;
    if (dsm > 48 * 1024) ensure_smem(spgemm_dense_warp_kernel<T>, dsm);
    FG_LAUNCH(spgemm_dense_warp_kernel<T>, (int)std::min<int64_t>((nrows_out + wpb - 1) / wpb, 152 * 4), 32 * wpb,
              dsm, s, a, ncols_out, toff.p, tci.p, tv.p, cnt.p);
  } else if (nrows_out >= 65536 && tcap <= (int64_t)nrows_out * 128) {
    // short rows on average: thread-per-row tier first, its overflow rows to the warp tier
    DBuf<int32_t> over0(nrows_out + 1, s), nover0(1, s);
    nover0.zero();
    FG_LAUNCH(spgemm_row_kernel<T>, grid_for(nrows_out, kRowThreads), kRowThreads, 0, s, a, toff.p, tci.p, tv.p,
              cnt.p, over0.p, nover0.p);
    FG_LAUNCH(hash_warp_kernel<T>, wgrid, 32 * kHashWarps, 0, s, a, over0.p, nover0.p, toff.p, tci.p, tv.p, cnt.p,
              over1.p, nover1.p);
  } else {
    FG_LAUNCH(hash_warp_kernel<T>, wgrid, 32 * kHashWarps, 0, s, a, (const int32_t*)nullptr,
              (const int32_t*)nullptr, toff.p, tci.p, tv.p, cnt.p, over1.p, nover1.p);
  }
  pt.mark("sp rows");
  // the output offsets are scanned before the overflow count is read, so when no row
  // overflowed (the usual case) both come back in one round trip
  out.n = nrows_out;
  out.m = ncols_out;
  out.rp.alloc(nrows_out + 1, s);
  exclusive_scan_async(cnt.p, out.rp.p, nrows_out, s);
  int32_t h_n1 = 0, h_tot = 0;
  FG_CUDA(cudaMemcpyAsync(&h_n1, nover1.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaMemcpyAsync(&h_tot, out.rp.p + nrows_out, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  const int n1 = h_n1;
  out.nnz = h_tot;
  if (n1 > 0) {
    const size_t bsm = (size_t)kHashBlockCap * (sizeof(unsigned long long) + sizeof(T) + sizeof(int32_t));
    ensure_smem(hash_block_kernel<T>, bsm);
    FG_LAUNCH(hash_block_kernel<T>, std::min(n1, 152 * 2), kHashBlockThreads, bsm, s, a, over1.p, n1, toff.p, tci.p,
              tv.p, cnt.p, over2.p, nover2.p);
    const int n2 = read_scalar(nover2.p, s);
    if (n2 > 0) {
      // more unique columns than the block table: dense accumulator over the columns
      const size_t dsm = (size_t)ncols_out * (sizeof(T) + 1);
      FG_REQUIRE(dsm <= 200 * 1024, FEMGPU_ERR_LIMIT, "SpGEMM row with more than 4096 unique columns");
      EscArgs<T> ad = a;
      ad.nbig = n2;
      ad.big_rows = over2.p;
      if (dsm > 48 * 1024) {
        ensure_smem(esc_dense_kernel<T, ESC_SPGEMM, false>, dsm);
        ensure_smem(esc_dense_kernel<T, ESC_SPGEMM, true>, dsm);
      }
      ad.counts = cnt.p;
      FG_LAUNCH((esc_dense_kernel<T, ESC_SPGEMM, false>), std::min(n2, 304), 256, dsm, s, ad, ncols_out, nullptr,
                nullptr);
      ad.orp = toff.p;
      ad.oci = tci.p;
      ad.ov = tv.p;
      FG_LAUNCH((esc_dense_kernel<T, ESC_SPGEMM, true>), std::min(n2, 304), 256, dsm, s, ad, ncols_out, nullptr,
                nullptr);
    }
    out.nnz = exclusive_scan(cnt.p, out.rp.p, nrows_out, s);  // the overflow rows' counts are in now
  }
  pt.mark("sp big");
  out.ci.alloc(out.nnz > 0 ? out.nnz : 1, s);
  out.v.alloc(out.nnz > 0 ? out.nnz : 1, s);
  {
    const double avg = nrows_out > 0 ? (double)out.nnz / nrows_out : 0.0;
    const int G = avg <= 6.0 ? 4 : avg <= 12.0 ? 8 : avg <= 24.0 ? 16 : 32;
    const int cgrid = grid_for((int64_t)nrows_out * G, 256);
#define FG_COMPACT(GG)                                                                                    \
  FG_LAUNCH((compact_rows_copy_kernel<T, GG>), cgrid, 256, 0, s, nrows_out, toff.p, tci.p, tv.p, out.rp.p, \
            out.ci.p, out.v.p)
    switch (G) {
      case 4: FG_COMPACT(4); break;
      case 8: FG_COMPACT(8); break;
      case 16: FG_COMPACT(16); break;
      default: FG_COMPACT(32); break;
    }
#undef FG_COMPACT
  }
  pt.mark("sp out");
}

template <class T, int MODE>
void run_esc(Ctx& c, EscArgs<T> a, int nrows_out, int ncols_out, DCsr<T>& out) {
  if (MODE == ESC_SPGEMM) run_spgemm_hash<T>(c, a, nrows_out, ncols_out, out);
  else run_esc_sort<T, MODE>(c, a, nrows_out, ncols_out, out);
}

// ---- level matrices -----------------------------------------------------------------
template <class T>
__global__ void diag_kernel(int n, const int32_t* rp, const int32_t* ci, const T* v, T* d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    int s = lower_bound_i32(ci, rp[i], rp[i + 1], i);
    d[i] = (s < rp[i + 1] && ci[s] == i) ? v[s] : (T)0;
  }
}

template <class T>
__global__ void reciprocal_kernel(int n, const T* d, T* dinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dinv[i] = (T)1 / d[i];
}

template <class T>
__global__ void split_count_kernel(int n, const int32_t* rp, const int32_t* ci, const int32_t* part, int32_t* cin,
                                   int32_t* cout) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pi = part[i], a = 0, b = 0;
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    int j = ci[e];
    if (j == i) continue;
    if (part[j] == pi) a++;
    else b++;
  }
  cin[i] = a;
  cout[i] = b;
}

template <class T>
__global__ void split_fill_kernel(int n, const int32_t* rp, const int32_t* ci, const T* v, const int32_t* part,
                                  const int32_t* irp, int32_t* ici, T* iv, const int32_t* orp, int32_t* oci, T* ov) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pi = part[i], qi = irp[i], qo = orp[i];
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    int j = ci[e];
    if (j == i) continue;
    if (part[j] == pi) {
      T val = v[e];
      if (j < i) {  // the symmetric smoother reads the upper entry (j, i) for both
        int u = lower_bound_i32(ci, rp[j], rp[j + 1], i);
        val = (u < rp[j + 1] && ci[u] == i) ? v[u] : (T)0;
      }
      ici[qi] = j;
      iv[qi] = val;
      qi++;
    } else {
      oci[qo] = j;
      ov[qo] = v[e];
      qo++;
    }
  }
}

template <class T>
__global__ void transpose_count_kernel(int64_t nnz, const int32_t* ci, int32_t* cnt) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[ci[e]], 1);
}

template <class T>
__global__ void transpose_fill_kernel(int n, const int32_t* rp, const int32_t* ci, const T* v, const int32_t* trp,
                                      int32_t* cur, int32_t* tci, T* tv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int e = rp[i]; e < rp[i + 1]; e++) {
    int k = ci[e];
    int q = trp[k] + atomicAdd(&cur[k], 1);
    tci[q] = i;
    tv[q] = v[e];
  }
}

template <class T>
__global__ void cast_kernel(int64_t n, const double* in, T* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (T)in[i];
}

template <class T>
__global__ void widen_kernel(int64_t n, const T* __restrict__ in, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

template <class T>
__global__ void narrow_kernel(int64_t n, const double* __restrict__ in, T* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)in[i];
}

template <class T>
__global__ void densify_kernel(int n, const int32_t* rp, const int32_t* ci, const T* v, double* F) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    for (int e = rp[i]; e < rp[i + 1]; e++) F[(int64_t)i * n + ci[e]] = (double)v[e];
}

// Dense LU with partial pivoting (first maximal |pivot| in row order), one block.
__global__ void dense_lu_kernel(int n, double* F, int32_t* piv, int32_t* status) {
  __shared__ double s_best[1024];
  __shared__ int s_idx[1024];
  for (int k = 0; k < n; k++) {
    double best = -1.0;
    int bi = n;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      double a = fabs(F[(int64_t)i * n + k]);
      if (a > best || (a == best && i < bi)) {
        best = a;
        bi = i;
      }
    }
    s_best[threadIdx.x] = best;
    s_idx[threadIdx.x] = bi;
    __syncthreads();
    for (int off = blockDim.x >> 1; off > 0; off >>= 1) {
      if (threadIdx.x < off) {
        double ob = s_best[threadIdx.x + off];
        int oi = s_idx[threadIdx.x + off];
        if (ob > s_best[threadIdx.x] || (ob == s_best[threadIdx.x] && oi < s_idx[threadIdx.x])) {
          s_best[threadIdx.x] = ob;
          s_idx[threadIdx.x] = oi;
        }
      }
      __syncthreads();
    }
    int p = s_idx[0];
    double pb = s_best[0];
    __syncthreads();
    if (pb == 0.0) {
      if (threadIdx.x == 0) *status = 1;
      return;
    }
    if (threadIdx.x == 0) piv[k] = p;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double t = F[(int64_t)k * n + j];
        F[(int64_t)k * n + j] = F[(int64_t)p * n + j];
        F[(int64_t)p * n + j] = t;
      }
    __syncthreads();
    double d = F[(int64_t)k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) F[(int64_t)i * n + k] = F[(int64_t)i * n + k] / d;
    __syncthreads();
    for (int64_t q = threadIdx.x; q < (int64_t)(n - k - 1) * (n - k - 1); q += blockDim.x) {
      int i = k + 1 + (int)(q / (n - k - 1));
      int j = k + 1 + (int)(q % (n - k - 1));
      F[(int64_t)i * n + j] = fma(-F[(int64_t)i * n + k], F[(int64_t)k * n + j], F[(int64_t)i * n + j]);
    }
    __syncthreads();
  }
}

// The same factorization with the matrix in shared memory (n * n doubles), one block:
// warp 0 finds the pivot (first maximal |a| in row order), every thread then swaps,
// scales and updates the trailing block.  Identical arithmetic to dense_lu_kernel.
__global__ void __launch_bounds__(1024) dense_lu_smem_kernel(int n, double* F, int32_t* piv, int32_t* status) {
  extern __shared__ double sf[];
  __shared__ int s_p;
  __shared__ double s_pb;
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) sf[q] = F[q];
  __syncthreads();
  for (int k = 0; k < n; k++) {
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = n;
      for (int i = k + (int)threadIdx.x; i < n; i += 32) {
        const double a = fabs(sf[i * n + k]);
        if (a > best) {  // rows visited in ascending order per lane
          best = a;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        s_p = bi;
        s_pb = best;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (s_pb == 0.0) {
      if (threadIdx.x == 0) *status = 1;
      return;
    }
    if (threadIdx.x == 0) piv[k] = p;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t = sf[k * n + j];
        sf[k * n + j] = sf[p * n + j];
        sf[p * n + j] = t;
      }
    __syncthreads();
    const double d = sf[k * n + k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) sf[i * n + k] = sf[i * n + k] / d;
    __syncthreads();
    const int m = n - k - 1;
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
      const int i = k + 1 + q / m, j = k + 1 + q % m;
      sf[i * n + j] = fma(-sf[i * n + k], sf[k * n + j], sf[i * n + j]);
    }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) F[q] = sf[q];
}

// Column j of the inverse (block j): solve L U x = P e_j column by column, so each
// step updates every remaining row in parallel.  Forward: row i takes the updates of
// columns 0, 1, ..., i-1 in that order; back: columns n-1, ..., i+1, then the division
// by U_ii (the CPU oracle uses the same orders).
__global__ void dense_inverse_kernel(int n, const double* __restrict__ F, const int32_t* __restrict__ piv,
                                     double* __restrict__ inv) {
  extern __shared__ double sb[];
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sb[i] = (i == j) ? 1.0 : 0.0;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < n; k++) {
      const double t = sb[k];
      sb[k] = sb[piv[k]];
      sb[piv[k]] = t;
    }
  __syncthreads();
  for (int q = 0; q < n; q++) {
    const double bq = sb[q];
    for (int i = q + 1 + threadIdx.x; i < n; i += blockDim.x) sb[i] = fma(-F[(int64_t)i * n + q], bq, sb[i]);
    __syncthreads();
  }
  for (int q = n - 1; q >= 0; q--) {
    if (threadIdx.x == 0) sb[q] = sb[q] / F[(int64_t)q * n + q];
    __syncthreads();
    const double bq = sb[q];
    for (int i = threadIdx.x; i < q; i += blockDim.x) sb[i] = fma(-F[(int64_t)i * n + q], bq, sb[i]);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) inv[(int64_t)i * n + j] = sb[i];
}

__global__ void partition_rows_kernel(int npart, const int32_t* part_idx, const int32_t* agg_idx, int32_t* rows) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npart) rows[p] = agg_idx[part_idx[p + 1]] - agg_idx[part_idx[p]];
}

// In-partition entries per partition (the shared-memory footprint of the smoother).
__global__ void partition_entries_kernel(int npart, const int32_t* part_idx, const int32_t* agg_idx,
                                         const int32_t* irp, int32_t* ent) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npart) ent[p] = irp[agg_idx[part_idx[p + 1]]] - irp[agg_idx[part_idx[p]]];
}

// First row and first in-partition entry of partitions 0..npart (npart = the end).
__global__ void partition_starts_kernel(int npart, const int32_t* part_idx, const int32_t* agg_idx,
                                        const int32_t* irp, int32_t* row0, int32_t* ent0) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p <= npart) {
    const int r = agg_idx[part_idx[p]];
    row0[p] = r;
    ent0[p] = irp[r];
  }
}

// The register smoother's entry layout, one CTA of 512 threads per group, warp w taking
// the group's rows [rs + 32w, rs + 32w + 32) (a block):
// * the block's rows are ranked by decreasing in-partition length (ties: lower row
//   first); jrow[block start + p] = offset in the block of the row ranked p;
// * entry k of the row ranked p goes to (block's first entry) + m_0 + ... + m_{k-1} + p,
//   m_j = rows of the block longer than j (a jagged-diagonal layout of the block);
// * each entry's column becomes (column - rs) + c * xcopy_stride<T>(): the copy c of x
//   is chosen greedily per diagonal, entries in lane order, each distinct column taking
//   the copy whose shared-memory bank has held the fewest distinct columns of that
//   diagonal so far (ties: the lowest copy); equal columns share the first one's copy.
// Entry values and the order of each row's entries are unchanged: only where they sit.
template <class T>
__global__ void __launch_bounds__(512) jds_build_kernel(const int32_t* __restrict__ grows,
                                                        const int32_t* __restrict__ irp,
                                                        const int32_t* __restrict__ ici, const T* __restrict__ iv,
                                                        T* __restrict__ jv, uint16_t* __restrict__ jc,
                                                        uint8_t* __restrict__ jrow) {
  constexpr unsigned kAll = 0xffffffffu;
  constexpr int CS = xcopy_stride<T>();
  constexpr int NB = sizeof(T) == 4 ? 32 : 16;  // bank slots of one element size
  constexpr int SHIFT = NB / kXCopies;          // bank slots between copies
  const int rs = grows[blockIdx.x], re = grows[blockIdx.x + 1];
  const int lane = threadIdx.x & 31;
  const int r0 = rs + (threadIdx.x & ~31);
  if (r0 >= re) return;  // the whole warp: its block is empty
  const int row = r0 + lane;
  const bool live = row < re;
  const int len = live ? irp[row + 1] - irp[row] : 0;
  const unsigned key = live ? ((unsigned)(len + 1) << 5) | (unsigned)(31 - lane) : 0u;
  int rank = 0;
  for (int j = 0; j < 32; j++) rank += __shfl_sync(kAll, key, j) > key;
  if (live) jrow[r0 + rank] = (uint8_t)lane;
  const int eb = irp[r0];
  const int mine = live ? irp[row] : 0;
  int dk = 0;  // entries on the diagonals before k
  for (int k = 0;; k++) {
    const bool act = k < len;
    const unsigned am = __ballot_sync(kAll, act);
    if (!am) break;
    const int a = act ? ici[mine + k] - rs : -1;
    const unsigned same = __match_any_sync(kAll, a);
    const int leader = __ffs(same) - 1;
    unsigned todo = __ballot_sync(kAll, act && leader == lane);
    int load = 0;  // lane b: distinct columns of this diagonal placed in bank slot b
    int copy = 0;
    while (todo) {
      const int q = __ffs(todo) - 1;
      todo &= todo - 1;
      const int aq = __shfl_sync(kAll, a, q);
      int best = 0, bc = 0;
      for (int c = 0; c < kXCopies; c++) {
        const int lb = __shfl_sync(kAll, load, (aq + c * SHIFT) % NB);
        if (c == 0 || lb < best) {
          best = lb;
          bc = c;
        }
      }
      if (lane == (aq + bc * SHIFT) % NB) load++;
      if (lane == q) copy = bc;
    }
    copy = __shfl_sync(kAll, copy, leader);
    if (act) {
      const int dst = eb + dk + rank;
      jv[dst] = iv[mine + k];
      jc[dst] = (uint16_t)(a + copy * CS);
    }
    dk += __popc(am);
  }
}

// Smoother work groups: consecutive partitions packed greedily into one CTA while
// the group stays within `max_rows` rows and `max_ents` in-partition entries.
template <class T>
void build_smoother_groups(Ctx& c, Level<T>& L, int max_rows, int max_ents) {
  cudaStream_t s = c.stream;
  DBuf<int32_t> row0(L.npart + 1, s), ent0(L.npart + 1, s);
  FG_LAUNCH(partition_starts_kernel, grid_for(L.npart + 1, 256), 256, 0, s, L.npart, L.part_idx.p, L.agg_idx.p,
            L.Ain.rp.p, row0.p, ent0.p);
  std::vector<int32_t> hr(L.npart + 1), he(L.npart + 1);
  row0.download(hr.data(), L.npart + 1);
  ent0.download(he.data(), L.npart + 1);
  FG_CUDA(cudaStreamSynchronize(s));
  g_host_syncs.fetch_add(1, std::memory_order_relaxed);
  std::vector<int32_t> g{hr[0]};
  int gp = 0, mx = 0, mxe = 0;
  for (int p = 1; p <= L.npart; p++) {
    const bool last = p == L.npart;
    if (last || hr[p + 1] - hr[gp] > max_rows || he[p + 1] - he[gp] > max_ents) {
      g.push_back(hr[p]);
      mx = std::max(mx, hr[p] - hr[gp]);
      mxe = std::max(mxe, he[p] - he[gp]);
      gp = p;
    }
  }
  L.ngroups = (int)g.size() - 1;
  L.max_group_rows = mx;
  L.max_group_ents = mxe;
  L.grows.alloc(g.size(), s);
  L.grows.upload(g.data(), g.size());
}

// ci[e] = map[ci[e]]
__global__ void map_columns_kernel(int64_t nnz, const int32_t* __restrict__ map, int32_t* ci) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) ci[e] = map[ci[e]];
}

// len[i] = length of row src[i] of rp
__global__ void gather_row_lengths_kernel(int m, const int32_t* __restrict__ src, const int32_t* __restrict__ rp,
                                          int32_t* __restrict__ len) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) len[i] = rp[src[i] + 1] - rp[src[i]];
}

// Row i of the output is row src[i] of the input (one warp per row, entries in order).
template <class T>
__global__ void gather_rows_kernel(int m, const int32_t* __restrict__ src, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ ci, const T* __restrict__ v,
                                   const int32_t* __restrict__ orp, int32_t* __restrict__ oci, T* __restrict__ ov) {
  const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (i >= m) return;
  const int a = rp[src[i]], len = rp[src[i] + 1] - a, o = orp[i];
  for (int t = lane; t < len; t += 32) {
    oci[o + t] = ci[a + t];
    ov[o + t] = v[a + t];
  }
}

template <class T>
void build_levels(Ctx& c, Hierarchy<T>& H) {
  cudaStream_t s = c.stream;
  const int n0 = c.A.n;
  // level 0: the operator converted to T
  {
    auto L0 = std::make_unique<Level<T>>();
    L0->n = n0;
    L0->A.n = L0->A.m = n0;
    L0->A.nnz = c.A.nnz;
    L0->A.rp.alloc(n0 + 1, s);
    L0->A.ci.alloc(c.A.nnz, s);
    L0->A.v.alloc(c.A.nnz, s);
    FG_CUDA(cudaMemcpyAsync(L0->A.rp.p, c.A.rp.p, (n0 + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    FG_CUDA(cudaMemcpyAsync(L0->A.ci.p, c.A.ci.p, c.A.nnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    FG_LAUNCH(cast_kernel<T>, grid_for(c.A.nnz, 256), 256, 0, s, c.A.nnz, c.A.v.p, L0->A.v.p);
    L0->gnnz = c.graph_nnz;
    L0->gxadj.alloc(n0 + 1, s);
    L0->gadj.alloc(c.graph_nnz > 0 ? c.graph_nnz : 1, s);
    FG_CUDA(cudaMemcpyAsync(L0->gxadj.p, c.gxadj.p, (n0 + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    if (c.graph_nnz > 0)
      FG_CUDA(cudaMemcpyAsync(L0->gadj.p, c.gadj.p, c.graph_nnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    H.L.push_back(std::move(L0));
  }
  int num_levels = 1;
  while (true) {
    Level<T>& L = *H.L.back();
    const int N = L.A.n;
    if (N < c.cfg.topSize || num_levels >= c.cfg.maxLevels) {
      FG_REQUIRE(N <= 8192, FEMGPU_ERR_LIMIT, "coarsest level too large for the dense solve (raise maxLevels)");
      L.coarsest = true;
      DBuf<double> F((size_t)N * N, s);
      DBuf<int32_t> piv(N, s), st(1, s);
      F.zero();
      st.zero();
      if (L.A64v.n)  // formed in FP64: the dense factorisation takes those values
        FG_LAUNCH(densify_kernel<double>, grid_for(N, 128), 128, 0, s, N, L.A.rp.p, L.A.ci.p, L.A64v.p, F.p);
      else
        FG_LAUNCH(densify_kernel<T>, grid_for(N, 128), 128, 0, s, N, L.A.rp.p, L.A.ci.p, L.A.v.p, F.p);
      const size_t fbytes = (size_t)N * N * sizeof(double);
      if (fbytes <= 200 * 1024) {
        if (fbytes > 48 * 1024)
          ensure_smem(dense_lu_smem_kernel, fbytes);
        FG_LAUNCH(dense_lu_smem_kernel, 1, 1024, fbytes, s, N, F.p, piv.p, st.p);
      } else {
        FG_LAUNCH(dense_lu_kernel, 1, 1024, 0, s, N, F.p, piv.p, st.p);
      }
      FG_REQUIRE(read_scalar(st.p, s) == 0, FEMGPU_ERR_BREAKDOWN, "coarsest matrix is singular");
      L.Ainv.alloc((size_t)N * N, s);
      const size_t bbytes = (size_t)N * sizeof(double);
      if (bbytes > 48 * 1024)
        ensure_smem(dense_inverse_kernel, bbytes);
      FG_LAUNCH(dense_inverse_kernel, N, std::min(1024, std::max(32, (N + 31) / 32 * 32)), bbytes, s, N, F.p, piv.p,
                L.Ainv.p);
      L.b.alloc(N, s);
      L.x.alloc(N, s);
      break;
    }
    PhaseTimer pt(s, num_levels - 1);
    const TraceRange level_range("femgpu setup: level");
    OldMisOut o;
    old_mis(c, N, L.gxadj.p, L.gadj.p, o);
    pt.mark("aggregate");
    L.nagg = o.nagg;
    L.npart = o.npart;
    L.perm = std::move(o.perm);
    L.iperm = std::move(o.iperm);
    L.agg_idx = std::move(o.agg_idx);
    L.part_idx = std::move(o.part_idx);
    L.agg_of = std::move(o.agg_of);
    // permuted operator
    {
      EscArgs<T> a{};
      a.arp = L.A.rp.p;
      a.aci = L.A.ci.p;
      a.av = L.A.v.p;
      a.perm = L.perm.p;
      a.iperm = L.iperm.p;
      a.known_nnz = L.A.nnz;
      run_esc<T, ESC_PERMUTE>(c, a, N, N, L.Ap);
    }
    pt.mark("permute");
    L.diag.alloc(N, s);
    FG_LAUNCH(diag_kernel<T>, grid_for(N, 256), 256, 0, s, N, L.Ap.rp.p, L.Ap.ci.p, L.Ap.v.p, L.diag.p);
    L.dinv.alloc(N, s);
    FG_LAUNCH(reciprocal_kernel<T>, grid_for(N, 256), 256, 0, s, N, L.diag.p, L.dinv.p);
    // in/out-of-partition split; the two entry counts and the three maxima the smoother
    // plan needs come back in one round trip
    {
      DBuf<int32_t> cin(N + 1, s), cout(N + 1, s), prow(L.npart + 1, s), pent(L.npart + 1, s), mx(3, s);
      FG_LAUNCH(split_count_kernel<T>, grid_for(N, 256), 256, 0, s, N, L.Ap.rp.p, L.Ap.ci.p, o.part_of_row.p, cin.p,
                cout.p);
      L.Ain.n = L.Ain.m = L.Aout.n = L.Aout.m = N;
      L.Ain.rp.alloc(N + 1, s);
      L.Aout.rp.alloc(N + 1, s);
      reduce_max_async(cin.p, N, mx.p + 2, s);  // longest in-partition row
      exclusive_scan_async(cin.p, L.Ain.rp.p, N, s);
      exclusive_scan_async(cout.p, L.Aout.rp.p, N, s);
      FG_LAUNCH(partition_rows_kernel, grid_for(L.npart, 256), 256, 0, s, L.npart, L.part_idx.p, L.agg_idx.p, prow.p);
      reduce_max_async(prow.p, L.npart, mx.p, s);
      FG_LAUNCH(partition_entries_kernel, grid_for(L.npart, 256), 256, 0, s, L.npart, L.part_idx.p, L.agg_idx.p,
                L.Ain.rp.p, pent.p);
      reduce_max_async(pent.p, L.npart, mx.p + 1, s);
      int32_t h_in = 0, h_out = 0, h_mx[3] = {0, 0, 0};
      FG_CUDA(cudaMemcpyAsync(&h_in, L.Ain.rp.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaMemcpyAsync(&h_out, L.Aout.rp.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaMemcpyAsync(h_mx, mx.p, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      FG_CUDA(cudaStreamSynchronize(s));
      g_host_syncs.fetch_add(1, std::memory_order_relaxed);
      L.Ain.nnz = h_in;
      L.Aout.nnz = h_out;
      L.max_part_rows = h_mx[0];
      L.max_part_entries = h_mx[1];
      L.max_in_row = h_mx[2];
      L.Ain.ci.alloc(L.Ain.nnz > 0 ? L.Ain.nnz : 1, s);
      L.Ain.v.alloc(L.Ain.nnz + 16, s);  // slack for 16-byte rounded bulk copies
      L.Ain.v.zero();
      L.Aout.ci.alloc(L.Aout.nnz > 0 ? L.Aout.nnz : 1, s);
      L.Aout.v.alloc(L.Aout.nnz > 0 ? L.Aout.nnz : 1, s);
      FG_LAUNCH(split_fill_kernel<T>, grid_for(N, 256), 256, 0, s, N, L.Ap.rp.p, L.Ap.ci.p, L.Ap.v.p,
                o.part_of_row.p, L.Ain.rp.p, L.Ain.ci.p, L.Ain.v.p, L.Aout.rp.p, L.Aout.ci.p, L.Aout.v.p);
    }
    {
      pt.mark("split rows");
      if (smoother_in_registers(L.max_in_row, L.max_part_rows)) {
        build_smoother_groups(c, L, kRegGroupRows, std::numeric_limits<int>::max());
        L.jv.alloc(L.Ain.nnz + 16, s);
        L.jv.zero();
        L.jc16.alloc(L.Ain.nnz + 16, s);
        L.jc16.zero();
        L.jrow.alloc(N, s);
        if (L.ngroups > 0)
          FG_LAUNCH(jds_build_kernel<T>, L.ngroups, kRegGroupRows, 0, s, L.grows.p, L.Ain.rp.p, L.Ain.ci.p,
                    L.Ain.v.p, L.jv.p, L.jc16.p, L.jrow.p);
      } else
        build_smoother_groups(c, L, L.max_part_rows, L.max_part_entries);
      pt.mark("groups");
      plan_smoother(c, L);
      pt.mark("plan");
      if (pt.on)
        fprintf(stderr,
                "[femgpu setup] level %d smoother: %s, groups %d (max %d rows), lanes %d, cluster %d, "
                "slice %d rows / %d entries, %d threads, %zu B shared%s\n",
                num_levels - 1,
                smoother_in_registers(L.max_in_row, L.max_part_rows) ? "registers"
                : L.smooth_k > 0                                      ? "cluster, entries in registers"
                                                                      : "cluster",
                L.ngroups, L.max_group_rows, L.smooth_lanes, L.cluster, L.slice_rows, L.slice_ents,
                L.smooth_threads, L.smooth_smem, L.smooth_staged ? ", staged" : "");
    }
    pt.mark("split");
    // prolongator and restrictor
    {
      EscArgs<T> a{};
      a.arp = L.Ap.rp.p;
      a.aci = L.Ap.ci.p;
      a.av = L.Ap.v.p;
      a.agg_of = L.agg_of.p;
      a.diag = L.diag.p;
      a.neg_omega = -(T)c.cfg.proOmega;
      run_esc<T, ESC_PROLONG>(c, a, N, L.nagg, L.P);
    }
    {
      pt.mark("P");
      DCsr<T> Ru;  // unsorted transpose, then rows sorted by column
      Ru.n = L.nagg;
      Ru.m = N;
      Ru.nnz = L.P.nnz;
      DBuf<int32_t> cnt(L.nagg + 1, s), cur(L.nagg, s);
      cnt.zero();
      cur.zero();
      FG_LAUNCH(transpose_count_kernel<T>, grid_for(L.P.nnz, 256), 256, 0, s, L.P.nnz, L.P.ci.p, cnt.p);
      Ru.rp.alloc(L.nagg + 1, s);
      exclusive_scan_async(cnt.p, Ru.rp.p, L.nagg, s);
      Ru.ci.alloc(L.P.nnz, s);
      Ru.v.alloc(L.P.nnz, s);
      FG_LAUNCH(transpose_fill_kernel<T>, grid_for(N, 256), 256, 0, s, N, L.P.rp.p, L.P.ci.p, L.P.v.p, Ru.rp.p, cur.p,
                Ru.ci.p, Ru.v.p);
      EscArgs<T> a{};
      a.arp = Ru.rp.p;
      a.aci = Ru.ci.p;
      a.av = Ru.v.p;
      a.known_nnz = L.P.nnz;
      run_esc<T, ESC_PERMUTE>(c, a, L.nagg, N, L.R);
    }
    // Galerkin product A_next = R (Ap P)
    auto nx = std::make_unique<Level<T>>();
    if (sizeof(T) == 4 && (int64_t)L.nagg <= (int64_t)kFp64GalerkinPerTop * c.cfg.topSize) {
      // the coarse end of a mixed hierarchy: the product in FP64 on widened operands
      DBuf<double> apv(L.Ap.nnz > 0 ? L.Ap.nnz : 1, s), pv(L.P.nnz > 0 ? L.P.nnz : 1, s),
          rv(L.R.nnz > 0 ? L.R.nnz : 1, s);
      FG_LAUNCH(widen_kernel<T>, grid_for(L.Ap.nnz, 256), 256, 0, s, L.Ap.nnz, L.Ap.v.p, apv.p);
      FG_LAUNCH(widen_kernel<T>, grid_for(L.P.nnz, 256), 256, 0, s, L.P.nnz, L.P.v.p, pv.p);
      FG_LAUNCH(widen_kernel<T>, grid_for(L.R.nnz, 256), 256, 0, s, L.R.nnz, L.R.v.p, rv.p);
      DCsr<double> AP, A64;
      EscArgs<double> a{};
      a.arp = L.Ap.rp.p;
      a.aci = L.Ap.ci.p;
      a.av = apv.p;
      a.brp = L.P.rp.p;
      a.bci = L.P.ci.p;
      a.bv = pv.p;
      run_esc<double, ESC_SPGEMM>(c, a, N, L.nagg, AP);
      EscArgs<double> r{};
      r.arp = L.R.rp.p;
      r.aci = L.R.ci.p;
      r.av = rv.p;
      r.brp = AP.rp.p;
      r.bci = AP.ci.p;
      r.bv = AP.v.p;
      run_esc<double, ESC_SPGEMM>(c, r, L.nagg, L.nagg, A64);
      nx->A.n = A64.n;
      nx->A.m = A64.m;
      nx->A.nnz = A64.nnz;
      nx->A.rp = std::move(A64.rp);
      nx->A.ci = std::move(A64.ci);
      nx->A.v.alloc(A64.nnz > 0 ? A64.nnz : 1, s);
      FG_LAUNCH(narrow_kernel<T>, grid_for(A64.nnz, 256), 256, 0, s, A64.nnz, A64.v.p, nx->A.v.p);
      nx->A64v = std::move(A64.v);
      pt.mark("RAP");
    } else {
      DCsr<T> AP;
      EscArgs<T> a{};
      a.arp = L.Ap.rp.p;
      a.aci = L.Ap.ci.p;
      a.av = L.Ap.v.p;
      a.brp = L.P.rp.p;
      a.bci = L.P.ci.p;
      a.bv = L.P.v.p;
      pt.mark("R");
      run_esc<T, ESC_SPGEMM>(c, a, N, L.nagg, AP);
      pt.mark("AP");
      EscArgs<T> r{};
      r.arp = L.R.rp.p;
      r.aci = L.R.ci.p;
      r.av = L.R.v.p;
      r.brp = AP.rp.p;
      r.bci = AP.ci.p;
      r.bv = AP.v.p;
      run_esc<T, ESC_SPGEMM>(c, r, L.nagg, L.nagg, nx->A);
      pt.mark("RAP");
    }
    nx->n = L.nagg;
    nx->gxadj = std::move(o.xadj_out);
    nx->gadj = std::move(o.adj_out);
    nx->gnnz = o.nnz_out;
    // work vectors
    L.b.alloc(N, s);
    L.x.alloc(N, s);
    L.r.alloc(N, s);
    L.xo.alloc(N, s);
    L.t.alloc(N, s);
    L.bp.alloc(N, s);
    autotune_level(c, L);  // result-neutral launch choices, timed on this level's data
    H.L.push_back(std::move(nx));
    num_levels++;
  }
  H.num_levels = num_levels;
  // The V-cycle keeps every non-coarsest level's vectors in that level's own (permuted)
  // order: each parent's restriction writes its rows in the child's order and its
  // prolongation reads the child's vector by the child's new indices, so no separate
  // permutation runs per cycle.  Entry order within each row is kept (same sums).
  for (size_t l = 0; l + 1 < H.L.size(); l++) {
    Level<T>& L = *H.L[l];
    const Level<T>& N = *H.L[l + 1];
    if (L.coarsest || N.coarsest) continue;
    if (L.P.nnz > 0)
      FG_LAUNCH(map_columns_kernel, grid_for(L.P.nnz, 256), 256, 0, s, L.P.nnz, N.perm.p, L.P.ci.p);
    const int m = L.R.n;
    DCsr<T> Rp;
    Rp.n = m;
    Rp.m = L.R.m;
    Rp.nnz = L.R.nnz;
    DBuf<int32_t> len(m + 1, s);
    Rp.rp.alloc(m + 1, s);
    FG_LAUNCH(gather_row_lengths_kernel, grid_for(m, 256), 256, 0, s, m, N.iperm.p, L.R.rp.p, len.p);
    exclusive_scan_async(len.p, Rp.rp.p, m, s);
    Rp.ci.alloc(L.R.nnz > 0 ? L.R.nnz : 1, s);
    Rp.v.alloc(L.R.nnz > 0 ? L.R.nnz : 1, s);
    FG_LAUNCH(gather_rows_kernel<T>, grid_for((int64_t)m * 32, 256), 256, 0, s, m, N.iperm.p, L.R.rp.p, L.R.ci.p,
              L.R.v.p, Rp.rp.p, Rp.ci.p, Rp.v.p);
    L.R = std::move(Rp);
  }
}

__global__ void identity_kernel(int n, int32_t* p) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = i;
}

}  // namespace

std::atomic<int64_t> g_kernel_launches{0};
std::atomic<int64_t> g_host_syncs{0};
thread_local cudaMemPool_t g_alloc_pool = nullptr;

// Values of perm(A) on its (sorted) pattern: row i' and column j' of the permuted
// matrix are row iperm[i'] and column iperm[j'] of A, found by binary search.
__global__ void permuted_values_kernel(int n, const int32_t* __restrict__ prp, const int32_t* __restrict__ pci,
                                       const int32_t* __restrict__ iperm, const int32_t* __restrict__ arp,
                                       const int32_t* __restrict__ aci, const double* __restrict__ av,
                                       double* __restrict__ pv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = iperm[i], a0 = arp[r], a1 = arp[r + 1];
  for (int e = prp[i]; e < prp[i + 1]; e++) {
    const int q = lower_bound_i32(aci, a0, a1, iperm[pci[e]]);
    pv[e] = av[q];
  }
}

// Entries of each 32-row slice (32 x its longest row), for the sliced layout of the
// permuted FP64 operator.
__global__ void slice_width_kernel(int n, int nslices, const int32_t* __restrict__ prp, int32_t* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((i >> 5) >= nslices) return;  // whole warps: nslices * 32 threads are live
  const int len = i < n ? prp[i + 1] - prp[i] : 0;
  const int w = __reduce_max_sync(0xffffffffu, len);
  if ((i & 31) == 0) cnt[i >> 5] = 32 * w;
}

// The permuted operator written as slices: row i's entry k (in the sorted pattern's
// order) goes to off[i / 32] + 32 k + i % 32, its value looked up in A as in
// permuted_values_kernel; the slice's remaining slots get column -1 and value 0.
__global__ void sliced_values_kernel(int n, int nslices, const int32_t* __restrict__ prp,
                                     const int32_t* __restrict__ pci, const int32_t* __restrict__ iperm,
                                     const int32_t* __restrict__ arp, const int32_t* __restrict__ aci,
                                     const double* __restrict__ av, const int32_t* __restrict__ off,
                                     int32_t* __restrict__ sci, double* __restrict__ sv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int sl = i >> 5;
  if (sl >= nslices) return;
  const int base = off[sl] + (i & 31), w = (off[sl + 1] - off[sl]) >> 5;
  int k = 0;
  if (i < n) {
    const int r = iperm[i], a0 = arp[r], a1 = arp[r + 1], e0 = prp[i], e1 = prp[i + 1];
    for (; k < e1 - e0; k++) {
      const int col = pci[e0 + k];
      sci[base + 32 * k] = col;
      sv[base + 32 * k] = av[lower_bound_i32(aci, a0, a1, iperm[col])];
    }
  }
  for (; k < w; k++) {
    sci[base + 32 * k] = -1;
    sv[base + 32 * k] = 0.0;
  }
}

void amg_setup(Ctx& c) {
  cudaStream_t s = c.stream;
  FG_REQUIRE(c.has_matrix, FEMGPU_ERR_NOT_READY, "no operator: call femgpu_set_mesh + femgpu_assemble or femgpu_set_matrix_csr");
  FG_REQUIRE(c.cfg.aggregatorType == 0, FEMGPU_ERR_INVALID, "only aggregatorType 0 (OldMIS) is implemented");
  cudaEvent_t e0, e1;
  FG_CUDA(cudaEventCreate(&e0));
  FG_CUDA(cudaEventCreate(&e1));
  FG_CUDA(cudaEventRecord(e0, s));
  c.H.reset();
  c.has_hierarchy = false;
  const int n = c.A.n;
  const int32_t* perm0 = nullptr;
  if (c.cfg.precision == 1) {
    auto H = std::make_unique<Hierarchy<double>>();
    build_levels(c, *H);
    if (!H->L[0]->coarsest) perm0 = H->L[0]->perm.p;
    c.H = std::move(H);
  } else {
    auto H = std::make_unique<Hierarchy<float>>();
    build_levels(c, *H);
    if (!H->L[0]->coarsest) perm0 = H->L[0]->perm.p;
    c.H = std::move(H);
  }
  c.perm0.alloc(n, s);
  if (perm0)
    FG_CUDA(cudaMemcpyAsync(c.perm0.p, perm0, n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
  else
    FG_LAUNCH(identity_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p);
  // FP64 outer operator in level-0 order: the pattern of the level-0 permuted operator
  // (already built, rows sorted by column), values looked up in the FP64 matrix
  {
    DBuf<int32_t> iperm(n, s);
    FG_LAUNCH(invert_kernel, grid_for(n, 256), 256, 0, s, n, c.perm0.p, iperm.p);
    const int32_t *prp, *pci;
    int64_t pnnz;
    if (c.cfg.precision == 1) {
      const Level<double>& L0 = *static_cast<Hierarchy<double>&>(*c.H).L[0];
      prp = L0.coarsest ? c.A.rp.p : L0.Ap.rp.p;
      pci = L0.coarsest ? c.A.ci.p : L0.Ap.ci.p;
      pnnz = L0.coarsest ? c.A.nnz : L0.Ap.nnz;
    } else {
      const Level<float>& L0 = *static_cast<Hierarchy<float>&>(*c.H).L[0];
      prp = L0.coarsest ? c.A.rp.p : L0.Ap.rp.p;
      pci = L0.coarsest ? c.A.ci.p : L0.Ap.ci.p;
      pnnz = L0.coarsest ? c.A.nnz : L0.Ap.nnz;
    }
    c.A0p.n = c.A0p.m = n;
    c.A0p.nnz = pnnz;
    c.A0p.rp.alloc(n + 1, s);
    FG_CUDA(cudaMemcpyAsync(c.A0p.rp.p, prp, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    // Slices of 32 rows when they pad the operator by at most 1/8 (mesh operators,
    // whose neighbouring rows have similar lengths); otherwise CSR.
    const int nslices = (n + 31) / 32;
    c.sliced = false;
    c.s_off.release();
    c.s_ci.release();
    c.s_v.release();
    c.A0p.ci.release();
    c.A0p.v.release();
    if (n > 0) {
      c.s_off.alloc(nslices + 1, s);
      FG_LAUNCH(slice_width_kernel, grid_for((int64_t)nslices * 32, 256), 256, 0, s, n, nslices, c.A0p.rp.p,
                c.s_off.p);
      const int64_t padded = exclusive_scan(c.s_off.p, c.s_off.p, nslices, s);
      if (padded <= INT32_MAX && padded <= pnnz + pnnz / 8) {
        c.sliced = true;
        c.s_padded = padded;
        c.s_ci.alloc(padded > 0 ? padded : 1, s);
        c.s_v.alloc(padded > 0 ? padded : 1, s);
        FG_LAUNCH(sliced_values_kernel, grid_for((int64_t)nslices * 32, 128), 128, 0, s, n, nslices, c.A0p.rp.p,
                  pci, iperm.p, c.A.rp.p, c.A.ci.p, c.A.v.p, c.s_off.p, c.s_ci.p, c.s_v.p);
      } else {
        c.s_off.release();
      }
    }
    if (!c.sliced) {
      c.A0p.ci.alloc(pnnz > 0 ? pnnz : 1, s);
      c.A0p.v.alloc(pnnz > 0 ? pnnz : 1, s);
      if (pnnz > 0)
        FG_CUDA(cudaMemcpyAsync(c.A0p.ci.p, pci, pnnz * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
      FG_LAUNCH(permuted_values_kernel, grid_for(n, 128), 128, 0, s, n, c.A0p.rp.p, c.A0p.ci.p, iperm.p, c.A.rp.p,
                c.A.ci.p, c.A.v.p, c.A0p.v.p);
    }
  }
  FG_CUDA(cudaEventRecord(e1, s));
  FG_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  FG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c.setup_ms = ms;
  c.has_hierarchy = true;
  c.hier_gen++;  // invalidates the captured PCG iteration graph
}

}  // namespace femgpu
