// hierarchy_io.cu -- the AMG hierarchy of a handle written to / read from a file, so a
// process holding the same operator can skip femgpu_setup.
//
// Layout (native byte order, for the machine that wrote it): an 8-byte magic, a version,
// the hierarchy precision, the operator's size and fingerprint, then every level's
// persistent state in a fixed order (scalars as raw values, device arrays as a 64-bit
// element count followed by the elements), then the level-0 permutation and the outer
// FP64 operator, and last a 64-bit checksum of every byte before it.  The smoother
// launch plan is not stored: it depends on the device and is planned again on load.
//
// Loading reads the whole file, checks the checksum, and checks the structure of every
// array on the host (offsets monotone and ending at the entry count, indices inside
// their range, level sizes that chain, smoother groups that hold their rows' columns)
// before anything is uploaded, so a damaged or foreign file is an FEMGPU_ERR_IO and
// never reaches a kernel.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>

#include "context.cuh"

namespace femgpu {

namespace {

constexpr char kMagic[8] = {'F', 'E', 'M', 'G', 'P', 'U', 'H', '1'};
constexpr uint32_t kVersion = 2;

// 64-bit checksum of a byte range: four interleaved multiply-xor lanes over 8-byte words
// (FNV-1a's prime and offset basis per lane, so long files hash at memory speed), the
// tail bytes folded into lane 0, and the lanes combined with the length.
uint64_t payload_checksum(const unsigned char* p, size_t n) {
  constexpr uint64_t kPrime = 0x100000001b3ull;
  uint64_t h[4] = {0xcbf29ce484222325ull, 0xcbf29ce484222325ull ^ 1, 0xcbf29ce484222325ull ^ 2,
                   0xcbf29ce484222325ull ^ 3};
  size_t i = 0;
  for (; i + 32 <= n; i += 32)
    for (int l = 0; l < 4; l++) {
      uint64_t w;
      memcpy(&w, p + i + 8 * l, 8);
      h[l] = (h[l] ^ w) * kPrime;
    }
  for (; i < n; i++) h[0] = (h[0] ^ p[i]) * kPrime;
  uint64_t out = (uint64_t)n * kPrime;
  for (int l = 0; l < 4; l++) out = ((out ^ h[l]) * kPrime) ^ (h[l] >> 29);
  return out;
}

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

// Writes scalars and device arrays in visiting order (kept in memory for the checksum,
// written out at the end).
struct Writer {
  FILE* f;
  cudaStream_t s;
  std::string path;
  std::vector<unsigned char> out;
  void raw(const void* p, size_t bytes) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    out.insert(out.end(), b, b + bytes);
  }
  void finish() {
    const uint64_t sum = payload_checksum(out.data(), out.size());
    raw(&sum, sizeof(sum));
    FG_REQUIRE(fwrite(out.data(), 1, out.size(), f) == out.size() && fflush(f) == 0, FEMGPU_ERR_IO,
               "cannot write " + path);
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

// Reads them back in the same order from the file's bytes in memory.  Every array is
// kept as a host copy until the whole hierarchy has been checked; nothing is uploaded
// before that (upload_all).
struct Reader {
  const unsigned char* data;
  size_t size;  // payload bytes (the checksum excluded)
  std::string path;
  size_t pos = 0;
  struct Pending {
    void* dst;       // the DBuf
    std::vector<unsigned char> bytes;
    size_t elem;
    void (*upload)(void* dst, const std::vector<unsigned char>& bytes, size_t elem, cudaStream_t s);
  };
  std::vector<Pending> pending;
  std::unordered_map<const void*, size_t> index;  // DBuf address -> pending slot
  void raw(void* p, size_t bytes) {
    FG_REQUIRE(bytes <= size - pos, FEMGPU_ERR_IO, "truncated hierarchy file " + path);
    memcpy(p, data + pos, bytes);
    pos += bytes;
  }
  template <class V>
  void scalar(V& v) {
    raw(&v, sizeof(V));
  }
  template <class E>
  static void upload_fn(void* dst, const std::vector<unsigned char>& bytes, size_t elem, cudaStream_t s) {
    DBuf<E>& b = *static_cast<DBuf<E>*>(dst);
    const size_t count = bytes.size() / elem;
    b.release();
    if (!count) return;
    b.alloc(count, s);
    b.upload(reinterpret_cast<const E*>(bytes.data()), count);
  }
  template <class E>
  void buf(DBuf<E>& b) {
    uint64_t count = 0;
    raw(&count, sizeof(count));
    FG_REQUIRE(count <= (uint64_t)(size - pos) / sizeof(E), FEMGPU_ERR_IO, "corrupt array length in " + path);
    b.release();
    Pending pd;
    pd.dst = &b;
    pd.elem = sizeof(E);
    pd.bytes.resize(count * sizeof(E));
    raw(pd.bytes.data(), pd.bytes.size());
    pd.upload = &upload_fn<E>;
    index[&b] = pending.size();
    pending.push_back(std::move(pd));
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
  // host copy of an array read by buf()
  template <class E>
  std::vector<E> host(const DBuf<E>& b) const {
    auto it = index.find(&b);
    FG_REQUIRE(it != index.end(), FEMGPU_ERR_IO, "internal: array not read from " + path);
    const auto& bytes = pending[it->second].bytes;
    std::vector<E> v(bytes.size() / sizeof(E));
    if (!v.empty()) memcpy(v.data(), bytes.data(), bytes.size());
    return v;
  }
  template <class E>
  size_t count(const DBuf<E>& b) const {
    auto it = index.find(&b);
    return it == index.end() ? 0 : pending[it->second].bytes.size() / sizeof(E);
  }
  void upload_all(cudaStream_t s) {
    for (auto& pd : pending) pd.upload(pd.dst, pd.bytes, pd.elem, s);
    FG_CUDA(cudaStreamSynchronize(s));
    pending.clear();
    index.clear();
  }
};

// ---- structural checks of a read hierarchy (host) ------------------------------------
void check(bool ok, const Reader& r, const char* what) {
  FG_REQUIRE(ok, FEMGPU_ERR_IO, std::string("corrupt hierarchy file ") + r.path + ": " + what);
}

// Offsets of `rows` rows: start at 0, never decrease, end at `total`.
void check_offsets(const std::vector<int32_t>& off, int64_t rows, int64_t total, const Reader& r, const char* what) {
  check(rows >= 0 && off.size() == (size_t)rows + 1, r, what);
  check(off[0] == 0 && off[rows] == total, r, what);
  for (int64_t i = 0; i < rows; i++) check(off[i] <= off[i + 1], r, what);
}

// A CSR matrix of n x m whose stored arrays hold its entries (values may carry slack).
template <class E>
void check_csr(const DCsr<E>& M, int64_t n, int64_t m, const Reader& r, const char* what) {
  check(M.n == n && M.m == m && M.nnz >= 0, r, what);
  check_offsets(r.host(M.rp), n, M.nnz, r, what);
  const std::vector<int32_t> ci = r.host(M.ci);
  check(ci.size() >= (size_t)M.nnz && r.count(M.v) >= (size_t)M.nnz, r, what);
  for (int64_t e = 0; e < M.nnz; e++) check(ci[e] >= 0 && ci[e] < m, r, what);
}

bool is_permutation(const std::vector<int32_t>& p, int64_t n) {
  if (p.size() != (size_t)n) return false;
  std::vector<char> seen(n, 0);
  for (int32_t v : p) {
    if (v < 0 || v >= n || seen[v]) return false;
    seen[v] = 1;
  }
  return true;
}

template <class T>
void check_level(const Level<T>& L, int64_t next_n, const Reader& r) {
  const int64_t n = L.n;
  check(n >= 1 && n < INT32_MAX, r, "level size");
  check_csr(L.A, n, n, r, "level operator");
  if (L.coarsest) {
    check(r.count(L.Ainv) == (size_t)(n * n), r, "coarsest inverse size");
    return;
  }
  check(L.nagg >= 1 && L.nagg <= n && L.nagg == next_n && L.npart >= 1 && L.npart <= L.nagg, r,
        "aggregate and partition counts");
  const std::vector<int32_t> perm = r.host(L.perm), iperm = r.host(L.iperm);
  check(is_permutation(perm, n) && iperm.size() == (size_t)n, r, "permutation");
  for (int64_t i = 0; i < n; i++) check(iperm[perm[i]] == i, r, "inverse permutation");
  check_offsets(r.host(L.agg_idx), L.nagg, n, r, "aggregate offsets");
  check_offsets(r.host(L.part_idx), L.npart, L.nagg, r, "partition offsets");
  const std::vector<int32_t> agg_of = r.host(L.agg_of);
  check(agg_of.size() == (size_t)n, r, "aggregate of row");
  for (int32_t a : agg_of) check(a >= 0 && a < L.nagg, r, "aggregate of row");
  check_csr(L.Ap, n, n, r, "permuted operator");
  check_csr(L.Ain, n, n, r, "in-partition entries");
  check_csr(L.Aout, n, n, r, "cross-partition entries");
  check_csr(L.P, n, L.nagg, r, "prolongator");
  check_csr(L.R, L.nagg, n, r, "restriction");
  check(r.count(L.diag) == (size_t)n && r.count(L.dinv) == (size_t)n, r, "diagonal");
  // smoother groups: consecutive row ranges whose in-partition columns stay inside them
  const std::vector<int32_t> grows = r.host(L.grows), irp = r.host(L.Ain.rp), ici = r.host(L.Ain.ci);
  check(L.ngroups >= 1, r, "smoother groups");
  check_offsets(grows, L.ngroups, n, r, "smoother groups");
  int mx = 0, mxe = 0, mrow = 0;
  for (int g = 0; g < L.ngroups; g++) {
    check(grows[g] < grows[g + 1], r, "empty smoother group");
    mx = std::max(mx, grows[g + 1] - grows[g]);
    mxe = std::max(mxe, irp[grows[g + 1]] - irp[grows[g]]);
    for (int i = grows[g]; i < grows[g + 1]; i++) {
      mrow = std::max(mrow, irp[i + 1] - irp[i]);
      for (int e = irp[i]; e < irp[i + 1]; e++)
        check(ici[e] >= grows[g] && ici[e] < grows[g + 1], r, "in-partition column");
    }
  }
  check(L.max_group_rows == mx && L.max_group_ents == mxe && L.max_in_row == mrow && L.max_part_rows >= 1 &&
            L.max_part_rows <= mx,
        r, "smoother group maxima");
  if (smoother_in_registers(L.max_in_row, L.max_part_rows)) {
    // the jagged-diagonal layout: per 32-row block, rows ranked by decreasing length and
    // every entry where that ranking puts it, with its column into one of the x copies
    check(mx <= kRegGroupRows && L.max_part_entries >= 0, r, "register smoother group size");
    constexpr int CS = xcopy_stride<T>();
    const std::vector<uint16_t> jc = r.host(L.jc16);
    const std::vector<uint8_t> jrow = r.host(L.jrow);
    const std::vector<T> jv = r.host(L.jv), iv = r.host(L.Ain.v);
    check(jc.size() >= (size_t)L.Ain.nnz + 16 && jv.size() >= (size_t)L.Ain.nnz + 16 && jrow.size() == (size_t)n &&
              iv.size() >= (size_t)L.Ain.nnz,
          r, "register smoother arrays");
    for (int g = 0; g < L.ngroups; g++)
      for (int b0 = grows[g]; b0 < grows[g + 1]; b0 += 32) {
        const int m = std::min(32, grows[g + 1] - b0);
        int rlen[32], used = 0, prev = INT32_MAX;
        for (int p = 0; p < m; p++) {
          const int o = jrow[b0 + p];
          check(o < m && !(used >> o & 1), r, "register smoother row order");
          used |= 1 << o;
          rlen[p] = irp[b0 + o + 1] - irp[b0 + o];
          check(rlen[p] <= prev, r, "register smoother row order");
          prev = rlen[p];
        }
        int dk = 0;
        for (int k = 0; k < kRegRow; k++) {
          int mk = 0;
          for (int p = 0; p < m; p++) {
            if (k >= rlen[p]) continue;
            const int src = irp[b0 + jrow[b0 + p]] + k, dst = irp[b0] + dk + p;
            check(jc[dst] % CS == ici[src] - grows[g] && jc[dst] / CS < kXCopies &&
                      memcmp(&jv[dst], &iv[src], sizeof(T)) == 0,
                  r, "register smoother entries");
            mk++;
          }
          dk += mk;
        }
      }
  }
}

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
  io.buf(L.jv);
  io.buf(L.jc16);
  io.buf(L.jrow);
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

// Reads every level, checks the whole hierarchy and the outer operator on the host, then
// uploads, allocates the work vectors and plans the smoothers.
template <class T>
void load_levels(Ctx& c, Reader& r, int64_t n0) {
  int32_t nl = 0;
  r.scalar(nl);
  check(nl >= 1 && nl <= 100, r, "level count");
  auto H = std::make_unique<Hierarchy<T>>();
  for (int l = 0; l < nl; l++) {
    auto L = std::make_unique<Level<T>>();
    visit_level(*L, r);
    check(l + 1 < nl ? !L->coarsest : L->coarsest, r, "level order");
    H->L.push_back(std::move(L));
  }
  visit_outer(c, r);
  check(r.pos == r.size, r, "trailing bytes");
  check(H->L[0]->n == n0, r, "level-0 size");
  for (int l = 0; l < nl; l++) check_level(*H->L[l], l + 1 < nl ? H->L[l + 1]->n : 0, r);
  check(is_permutation(r.host(c.perm0), n0), r, "level-0 permutation");
  if (c.sliced) {
    const int64_t ns = (n0 + 31) / 32;
    const std::vector<int32_t> off = r.host(c.s_off), sci = r.host(c.s_ci);
    check(off.size() == (size_t)ns + 1 && off[0] == 0 && off[ns] == c.s_padded && c.s_padded >= 0 &&
              sci.size() >= (size_t)c.s_padded && r.count(c.s_v) >= (size_t)c.s_padded,
          r, "sliced outer operator");
    for (int64_t q = 0; q < ns; q++) check(off[q] <= off[q + 1] && (off[q + 1] - off[q]) % 32 == 0, r, "slice offsets");
    for (int64_t e = 0; e < c.s_padded; e++) check(sci[e] >= -1 && sci[e] < n0, r, "slice columns");
    check(c.A0p.n == n0 && c.A0p.m == n0, r, "outer operator size");
    check_offsets(r.host(c.A0p.rp), n0, c.A0p.nnz, r, "outer operator offsets");
  } else {
    check_csr(c.A0p, n0, n0, r, "outer operator");
  }
  r.upload_all(c.stream);
  for (auto& L : H->L) {
    // work vectors (level numbering); the coarsest level uses b and x only
    L->b.alloc(L->n, c.stream);
    L->x.alloc(L->n, c.stream);
    if (!L->coarsest) {
      L->r.alloc(L->n, c.stream);
      L->xo.alloc(L->n, c.stream);
      L->t.alloc(L->n, c.stream);
      L->bp.alloc(L->n, c.stream);
      plan_smoother(c, *L);
      autotune_level(c, *L);
    }
  }
  H->num_levels = nl;
  c.H = std::move(H);
}

}  // namespace

void save_hierarchy(Ctx& c, const char* path) {
  FG_REQUIRE(c.has_hierarchy, FEMGPU_ERR_NOT_READY, "call femgpu_setup first");
  File f(fopen(path, "wb"));
  FG_REQUIRE(f != nullptr, FEMGPU_ERR_IO, std::string("cannot open ") + path + " for writing");
  Writer w{f.get(), c.stream, path, {}};
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
  w.finish();
}

void load_hierarchy(Ctx& c, const char* path) {
  FG_REQUIRE(c.has_matrix, FEMGPU_ERR_NOT_READY, "no operator: the hierarchy belongs to an operator, set it first");
  std::vector<unsigned char> bytes;
  {
    File f(fopen(path, "rb"));
    FG_REQUIRE(f != nullptr, FEMGPU_ERR_IO, std::string("cannot open ") + path);
    FG_REQUIRE(fseek(f.get(), 0, SEEK_END) == 0, FEMGPU_ERR_IO, std::string("cannot read ") + path);
    const long size = ftell(f.get());
    FG_REQUIRE(size >= 0 && fseek(f.get(), 0, SEEK_SET) == 0, FEMGPU_ERR_IO, std::string("cannot read ") + path);
    bytes.resize((size_t)size);
    FG_REQUIRE(size == 0 || fread(bytes.data(), 1, bytes.size(), f.get()) == bytes.size(), FEMGPU_ERR_IO,
               std::string("cannot read ") + path);
  }
  FG_REQUIRE(bytes.size() >= sizeof(kMagic) + sizeof(uint64_t) && memcmp(bytes.data(), kMagic, sizeof(kMagic)) == 0,
             FEMGPU_ERR_IO, std::string(path) + " is not a hierarchy file");
  const size_t payload = bytes.size() - sizeof(uint64_t);
  uint64_t stored = 0;
  memcpy(&stored, bytes.data() + payload, sizeof(stored));
  Reader r{bytes.data(), payload, path};
  r.pos = sizeof(kMagic);
  uint32_t version = 0;
  r.scalar(version);
  FG_REQUIRE(version == kVersion, FEMGPU_ERR_IO, std::string("unsupported hierarchy file version in ") + path);
  FG_REQUIRE(payload_checksum(bytes.data(), payload) == stored, FEMGPU_ERR_IO,
             std::string("checksum mismatch: damaged hierarchy file ") + path);
  int32_t precision = -1;
  int64_t n = -1, nnz = -1;
  uint64_t fp = 0;
  r.scalar(precision);
  r.scalar(n);
  r.scalar(nnz);
  r.scalar(fp);
  FG_REQUIRE(precision == c.cfg.precision, FEMGPU_ERR_INVALID,
             "the hierarchy was built with another precision setting than the handle's");
  FG_REQUIRE(n == c.A.n && nnz == c.A.nnz && fp == operator_fingerprint(c), FEMGPU_ERR_INVALID,
             "the hierarchy was built for another operator");
  c.H.reset();
  c.has_hierarchy = false;
  try {
    if (precision == 1) load_levels<double>(c, r, n);
    else load_levels<float>(c, r, n);
  } catch (...) {
    c.H.reset();
    c.perm0.release();
    c.A0p = DCsr<double>();
    c.s_off.release();
    c.s_ci.release();
    c.s_v.release();
    c.sliced = false;
    throw;
  }
  c.setup_ms = 0.0;
  c.has_hierarchy = true;
  c.hier_gen++;  // a new hierarchy: the captured PCG loop is rebuilt
}

}  // namespace femgpu
