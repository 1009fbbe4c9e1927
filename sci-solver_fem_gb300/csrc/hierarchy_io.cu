// hierarchy_io.cu -- the AMG hierarchy of a handle written to / read from a file, so a
// process holding the same operator can skip femgpu_setup.
//
// Layout (native byte order, for the machine that wrote it): an 8-byte magic, a version,
// the hierarchy precision, the operator's size and fingerprint, then every level's
// persistent state in a fixed order (scalars as raw values, device arrays as a 64-bit
// element count followed by the elements), then the level-0 permutation and the outer
// FP64 operator.  The smoother launch plan is not stored: it depends on the device and
// is planned again on load.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "context.cuh"

namespace femgpu {

namespace {

constexpr char kMagic[8] = {'F', 'E', 'M', 'G', 'P', 'U', 'H', '1'};
constexpr uint32_t kVersion = 1;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // splitmix64 finaliser (Steele, Lea, Flood 2014)
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Order-independent fingerprint of a CSR operator: the wrapping sum of a hash of every
// (position, row offset) and (position, column, value bits), so any thread order gives
// the same 64 bits.
__global__ void fingerprint_kernel(int n, int64_t nnz, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ ci, const double* __restrict__ v,
                                   unsigned long long* out) {
  uint64_t h = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride)
    h += mix64(((uint64_t)i << 1) ^ ((uint64_t)(uint32_t)rp[i] << 32));
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
    const uint64_t bits = (uint64_t)__double_as_longlong(v[e]);
    h += mix64(mix64(((uint64_t)e << 1) | 1ull) ^ ((uint64_t)(uint32_t)ci[e] << 17) ^ bits);
  }
  atomicAdd(out, (unsigned long long)h);
}

uint64_t operator_fingerprint(Ctx& c) {
  DBuf<unsigned long long> out(1, c.stream);
  out.zero();
  FG_LAUNCH(fingerprint_kernel, 152 * 4, 256, 0, c.stream, c.A.n, c.A.nnz, c.A.rp.p, c.A.ci.p, c.A.v.p, out.p);
  return (uint64_t)read_scalar(out.p, c.stream);
}

struct FileCloser {
  void operator()(FILE* f) const {
    if (f) fclose(f);
  }
};
using File = std::unique_ptr<FILE, FileCloser>;

// Writes scalars and device arrays in visiting order.
struct Writer {
  FILE* f;
  cudaStream_t s;
  std::string path;
  void raw(const void* p, size_t bytes) {
    FG_REQUIRE(bytes == 0 || fwrite(p, 1, bytes, f) == bytes, FEMGPU_ERR_IO, "cannot write " + path);
  }
  template <class V>
  void scalar(V& v) {
    raw(&v, sizeof(V));
  }
  template <class E>
  void buf(DBuf<E>& b) {
    const uint64_t count = b.n;
    raw(&count, sizeof(count));
    if (!count) return;
    std::vector<E> h(count);
    b.download(h.data(), count);
    FG_CUDA(cudaStreamSynchronize(s));
    raw(h.data(), count * sizeof(E));
  }
  template <class E>
  void csr(DCsr<E>& m) {
    scalar(m.n);
    scalar(m.m);
    scalar(m.nnz);
    buf(m.rp);
    buf(m.ci);
    buf(m.v);
  }
};

// Reads them back in the same order, allocating each array on the handle's stream.
struct Reader {
  FILE* f;
  cudaStream_t s;
  std::string path;
  int64_t remaining;  // bytes left in the file: bounds every array before it is allocated
  void raw(void* p, size_t bytes) {
    FG_REQUIRE((int64_t)bytes <= remaining && (bytes == 0 || fread(p, 1, bytes, f) == bytes), FEMGPU_ERR_IO,
               "truncated hierarchy file " + path);
    remaining -= (int64_t)bytes;
  }
  template <class V>
  void scalar(V& v) {
    raw(&v, sizeof(V));
  }
  template <class E>
  void buf(DBuf<E>& b) {
    uint64_t count = 0;
    raw(&count, sizeof(count));
    FG_REQUIRE(count <= (uint64_t)remaining / sizeof(E), FEMGPU_ERR_IO, "corrupt array length in " + path);
    b.release();
    if (!count) return;
    std::vector<E> h(count);
    raw(h.data(), count * sizeof(E));
    b.alloc(count, s);
    b.upload(h.data(), count);
    FG_CUDA(cudaStreamSynchronize(s));
  }
  template <class E>
  void csr(DCsr<E>& m) {
    scalar(m.n);
    scalar(m.m);
    scalar(m.nnz);
    buf(m.rp);
    buf(m.ci);
    buf(m.v);
  }
};

// Every persistent field of a level, in file order.
template <class T, class IO>
void visit_level(Level<T>& L, IO& io) {
  io.scalar(L.n);
  io.scalar(L.nagg);
  io.scalar(L.npart);
  io.scalar(L.coarsest);
  io.csr(L.A);
  io.buf(L.gxadj);
  io.buf(L.gadj);
  io.scalar(L.gnnz);
  io.buf(L.perm);
  io.buf(L.iperm);
  io.buf(L.agg_idx);
  io.buf(L.part_idx);
  io.buf(L.agg_of);
  io.csr(L.Ap);
  io.csr(L.Ain);
  io.csr(L.Aout);
  io.csr(L.P);
  io.csr(L.R);
  io.buf(L.diag);
  io.buf(L.dinv);
  io.scalar(L.max_part_rows);
  io.scalar(L.max_part_entries);
  io.scalar(L.max_in_row);
  io.buf(L.grows);
  io.scalar(L.ngroups);
  io.scalar(L.max_group_rows);
  io.scalar(L.max_group_ents);
  io.buf(L.ci16);
  io.buf(L.Ainv);
}

template <class IO>
void visit_outer(Ctx& c, IO& io) {
  io.buf(c.perm0);
  io.csr(c.A0p);
  io.scalar(c.sliced);
  io.scalar(c.s_padded);
  io.buf(c.s_off);
  io.buf(c.s_ci);
  io.buf(c.s_v);
}

template <class T>
void save_levels(Ctx& c, Writer& w) {
  auto& H = static_cast<Hierarchy<T>&>(*c.H);
  int32_t nl = (int32_t)H.L.size();
  w.scalar(nl);
  for (auto& L : H.L) visit_level(*L, w);
}

template <class T>
void load_levels(Ctx& c, Reader& r) {
  int32_t nl = 0;
  r.scalar(nl);
  FG_REQUIRE(nl >= 1 && nl <= 100, FEMGPU_ERR_IO, "corrupt level count in " + r.path);
  auto H = std::make_unique<Hierarchy<T>>();
  for (int l = 0; l < nl; l++) {
    auto L = std::make_unique<Level<T>>();
    visit_level(*L, r);
    FG_REQUIRE(L->n >= 0 && L->A.n == L->n, FEMGPU_ERR_IO, "corrupt level in " + r.path);
    FG_REQUIRE(l + 1 < nl ? !L->coarsest : L->coarsest, FEMGPU_ERR_IO, "corrupt level order in " + r.path);
    // work vectors (level numbering); the coarsest level uses b and x only
    L->b.alloc(L->n, c.stream);
    L->x.alloc(L->n, c.stream);
    if (!L->coarsest) {
      L->r.alloc(L->n, c.stream);
      L->xo.alloc(L->n, c.stream);
      L->t.alloc(L->n, c.stream);
      L->bp.alloc(L->n, c.stream);
      plan_smoother(c, *L);
    }
    H->L.push_back(std::move(L));
  }
  H->num_levels = nl;
  c.H = std::move(H);
}

}  // namespace

void save_hierarchy(Ctx& c, const char* path) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  File f(fopen(path, "wb"));
  FG_REQUIRE(f != nullptr, FEMGPU_ERR_IO, std::string("cannot open ") + path + " for writing");
  Writer w{f.get(), c.stream, path};
  w.raw(kMagic, sizeof(kMagic));
  uint32_t version = kVersion;
  int32_t precision = c.cfg.precision;
  int64_t n = c.A.n, nnz = c.A.nnz;
  uint64_t fp = operator_fingerprint(c);
  w.scalar(version);
  w.scalar(precision);
  w.scalar(n);
  w.scalar(nnz);
  w.scalar(fp);
  if (precision == 1) save_levels<double>(c, w);
  else save_levels<float>(c, w);
  visit_outer(c, w);
  FG_REQUIRE(fflush(f.get()) == 0, FEMGPU_ERR_IO, std::string("cannot write ") + path);
}

void load_hierarchy(Ctx& c, const char* path) {
  FG_REQUIRE(c.has_matrix, FEMGPU_ERR_NOT_READY, "no operator: the hierarchy belongs to an operator, set it first");
  File f(fopen(path, "rb"));
  FG_REQUIRE(f != nullptr, FEMGPU_ERR_IO, std::string("cannot open ") + path);
  FG_REQUIRE(fseek(f.get(), 0, SEEK_END) == 0, FEMGPU_ERR_IO, std::string("cannot read ") + path);
  const long size = ftell(f.get());
  FG_REQUIRE(size >= 0 && fseek(f.get(), 0, SEEK_SET) == 0, FEMGPU_ERR_IO, std::string("cannot read ") + path);
  Reader r{f.get(), c.stream, path, (int64_t)size};
  char magic[8];
  r.raw(magic, sizeof(magic));
  FG_REQUIRE(memcmp(magic, kMagic, sizeof(kMagic)) == 0, FEMGPU_ERR_IO, std::string(path) + " is not a hierarchy file");
  uint32_t version = 0;
  int32_t precision = -1;
  int64_t n = -1, nnz = -1;
  uint64_t fp = 0;
  r.scalar(version);
  r.scalar(precision);
  r.scalar(n);
  r.scalar(nnz);
  r.scalar(fp);
  FG_REQUIRE(version == kVersion, FEMGPU_ERR_IO, std::string("unsupported hierarchy file version in ") + path);
  FG_REQUIRE(precision == c.cfg.precision, FEMGPU_ERR_INVALID,
             "the hierarchy was built with another precision setting than the handle's");
  FG_REQUIRE(n == c.A.n && nnz == c.A.nnz && fp == operator_fingerprint(c), FEMGPU_ERR_INVALID,
             "the hierarchy was built for another operator");
  c.H.reset();
  c.has_hierarchy = false;
  try {
    if (precision == 1) load_levels<double>(c, r);
    else load_levels<float>(c, r);
    visit_outer(c, r);
    FG_REQUIRE(c.perm0.n == (size_t)n, FEMGPU_ERR_IO, std::string("corrupt permutation in ") + path);
    FG_REQUIRE(c.sliced ? (c.s_off.n == (size_t)(n + 31) / 32 + 1 && c.s_ci.n == c.s_v.n)
                        : (c.A0p.rp.n == (size_t)n + 1 && c.A0p.ci.n == c.A0p.v.n),
               FEMGPU_ERR_IO, std::string("corrupt outer operator in ") + path);
  } catch (...) {
    c.H.reset();
    throw;
  }
  c.setup_ms = 0.0;
  c.has_hierarchy = true;
  c.hier_gen++;  // a new hierarchy: the captured PCG loop is rebuilt
}

}  // namespace femgpu
