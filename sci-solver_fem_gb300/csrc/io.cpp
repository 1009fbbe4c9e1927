// io.cpp -- host-side file formats of the FEMSolver API: TetGen .node/.ele, PLY,
// MAT v5 (uncompressed) sparse matrices and double arrays, legacy ASCII VTK.
// Every reader validates its input and returns FEMGPU_ERR_IO instead of exiting.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/femgpu.h"

namespace {

bool is_skip_line(const std::string& l) {
  size_t p = l.find_first_not_of(" \t\r");
  return p == std::string::npos || l[p] == '#';
}

struct TetFile {
  std::vector<double> xyz;
  std::vector<int32_t> conn, labels;
};

// TetMesh::read (src/core/cuda/tetmesh.cu:251-376): coordinates parsed as float,
// indices 1-based unless a 0 appears (then 0-based), optional material label.
femgpu_status read_tetgen(const char* node, const char* ele, TetFile& out) {
  std::ifstream nf(node), ef(ele);
  if (!nf.is_open() || !ef.is_open()) return FEMGPU_ERR_IO;
  std::string line;
  int nv = -1, t1, t2, t3;
  while (std::getline(nf, line)) {
    if (is_skip_line(line)) continue;
    if (sscanf(line.c_str(), "%d %d %d %d", &nv, &t1, &t2, &t3) != 4 || nv <= 0) return FEMGPU_ERR_IO;
    break;
  }
  if (nv <= 0) return FEMGPU_ERR_IO;
  out.xyz.assign((size_t)nv * 3, 0.0);
  int i = 0;
  while (i < nv && std::getline(nf, line)) {
    if (is_skip_line(line)) continue;
    int id;
    float x, y, z;
    if (sscanf(line.c_str(), "%d %f %f %f", &id, &x, &y, &z) != 4) return FEMGPU_ERR_IO;
    out.xyz[(size_t)i * 3] = x;
    out.xyz[(size_t)i * 3 + 1] = y;
    out.xyz[(size_t)i * 3 + 2] = z;
    i++;
  }
  if (i != nv) return FEMGPU_ERR_IO;
  int ne = -1, npe = 0, haslabel = 0;
  while (std::getline(ef, line)) {
    if (is_skip_line(line)) continue;
    if (sscanf(line.c_str(), "%d %d %d", &ne, &npe, &haslabel) != 3 || ne <= 0) return FEMGPU_ERR_IO;
    break;
  }
  if (ne <= 0) return FEMGPU_ERR_IO;
  out.conn.assign((size_t)ne * 4, 0);
  out.labels.assign(ne, 0);
  bool zero_based = false;
  int e = 0;
  while (e < ne && std::getline(ef, line)) {
    if (is_skip_line(line)) continue;
    int id, v[4], mat = 0;
    if (haslabel == 0) {
      if (sscanf(line.c_str(), "%d %d %d %d %d", &id, &v[0], &v[1], &v[2], &v[3]) != 5) return FEMGPU_ERR_IO;
    } else {
      if (sscanf(line.c_str(), "%d %d %d %d %d %d", &id, &v[0], &v[1], &v[2], &v[3], &mat) != 6) return FEMGPU_ERR_IO;
      out.labels[e] = mat;
    }
    for (int a = 0; a < 4; a++) {
      out.conn[(size_t)e * 4 + a] = v[a];
      if (v[a] == 0) zero_based = true;
    }
    e++;
  }
  if (e != ne) return FEMGPU_ERR_IO;
  if (!zero_based)
    for (auto& v : out.conn) v--;
  int minidx = *std::min_element(out.conn.begin(), out.conn.end());
  if (minidx == 1)  // tetmesh.cu:350-366 shifts once more
    for (auto& v : out.conn) v--;
  for (int32_t v : out.conn)
    if (v < 0 || v >= nv) return FEMGPU_ERR_IO;
  return FEMGPU_OK;
}

// PLY (ascii, binary_little_endian): vertex x/y/z and polygon faces (fan-split).
// Coordinates are kept in double as parsed: the reference's TriMesh reader scans ASCII
// values with "%lf" into its double vertices (src/core/aggmis/cuda/TriMesh_io.cu,
// read_verts_asc), and binary values keep their stored precision.
struct PlyProp {
  std::string name, type, count_type;
  bool list = false;
};

int type_size(const std::string& t) {
  if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
  if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
  if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
  if (t == "double" || t == "float64") return 8;
  return 0;
}

double read_bin(const unsigned char* p, const std::string& t) {
  if (t == "char" || t == "int8") return (double)*(const int8_t*)p;
  if (t == "uchar" || t == "uint8") return (double)*(const uint8_t*)p;
  int16_t s; uint16_t us; int32_t i; uint32_t u; float f; double d;
  if (t == "short" || t == "int16") { memcpy(&s, p, 2); return s; }
  if (t == "ushort" || t == "uint16") { memcpy(&us, p, 2); return us; }
  if (t == "int" || t == "int32") { memcpy(&i, p, 4); return i; }
  if (t == "uint" || t == "uint32") { memcpy(&u, p, 4); return u; }
  if (t == "float" || t == "float32") { memcpy(&f, p, 4); return f; }
  memcpy(&d, p, 8);
  return d;
}

femgpu_status read_ply(const char* file, std::vector<double>& xyz, std::vector<int32_t>& tri) {
  std::ifstream in(file, std::ios::binary);
  if (!in.is_open()) return FEMGPU_ERR_IO;
  std::string line;
  if (!std::getline(in, line) || line.compare(0, 3, "ply") != 0) return FEMGPU_ERR_IO;
  bool binary = false;
  int64_t nv = 0, nf = 0;
  std::vector<PlyProp> vprops, fprops;
  std::vector<std::pair<std::string, int64_t>> elems;
  std::vector<std::vector<PlyProp>> eprops;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ss(line);
    std::string kw;
    ss >> kw;
    if (kw == "format") {
      std::string f;
      ss >> f;
      if (f == "binary_little_endian") binary = true;
      else if (f != "ascii") return FEMGPU_ERR_IO;
    } else if (kw == "element") {
      std::string name;
      int64_t cnt;
      ss >> name >> cnt;
      elems.push_back({name, cnt});
      eprops.emplace_back();
    } else if (kw == "property") {
      if (eprops.empty()) return FEMGPU_ERR_IO;
      PlyProp p;
      std::string t;
      ss >> t;
      if (t == "list") {
        p.list = true;
        ss >> p.count_type >> p.type >> p.name;
      } else {
        p.type = t;
        ss >> p.name;
      }
      eprops.back().push_back(p);
    } else if (kw == "end_header") {
      break;
    }
  }
  xyz.clear();
  tri.clear();
  for (size_t ei = 0; ei < elems.size(); ei++) {
    const std::string& name = elems[ei].first;
    int64_t cnt = elems[ei].second;
    const std::vector<PlyProp>& props = eprops[ei];
    bool is_v = name == "vertex", is_f = name == "face";
    if (is_v) nv = cnt;
    if (is_f) nf = cnt;
    for (int64_t r = 0; r < cnt; r++) {
      double pos[3] = {0, 0, 0};
      std::vector<int64_t> poly;
      if (!binary) {
        if (!std::getline(in, line)) return FEMGPU_ERR_IO;
        std::istringstream ss(line);
        for (const PlyProp& p : props) {
          if (p.list) {
            int64_t k;
            if (!(ss >> k)) return FEMGPU_ERR_IO;
            for (int64_t q = 0; q < k; q++) {
              double v;
              if (!(ss >> v)) return FEMGPU_ERR_IO;
              poly.push_back((int64_t)v);
            }
          } else {
            double v;
            if (!(ss >> v)) return FEMGPU_ERR_IO;
            if (is_v && p.name == "x") pos[0] = v;
            if (is_v && p.name == "y") pos[1] = v;
            if (is_v && p.name == "z") pos[2] = v;
          }
        }
      } else {
        for (const PlyProp& p : props) {
          unsigned char buf[8];
          if (p.list) {
            int cs = type_size(p.count_type), vs = type_size(p.type);
            if (!cs || !vs || !in.read((char*)buf, cs)) return FEMGPU_ERR_IO;
            int64_t k = (int64_t)read_bin(buf, p.count_type);
            for (int64_t q = 0; q < k; q++) {
              if (!in.read((char*)buf, vs)) return FEMGPU_ERR_IO;
              poly.push_back((int64_t)read_bin(buf, p.type));
            }
          } else {
            int sz = type_size(p.type);
            if (!sz || !in.read((char*)buf, sz)) return FEMGPU_ERR_IO;
            double v = read_bin(buf, p.type);
            if (is_v && p.name == "x") pos[0] = v;
            if (is_v && p.name == "y") pos[1] = v;
            if (is_v && p.name == "z") pos[2] = v;
          }
        }
      }
      if (is_v) xyz.insert(xyz.end(), pos, pos + 3);
      if (is_f) {
        if (poly.size() < 3) return FEMGPU_ERR_IO;
        for (size_t q = 1; q + 1 < poly.size(); q++) {
          tri.push_back((int32_t)poly[0]);
          tri.push_back((int32_t)poly[q]);
          tri.push_back((int32_t)poly[q + 1]);
        }
      }
    }
  }
  if (nv <= 0 || nf <= 0) return FEMGPU_ERR_IO;
  for (int32_t v : tri)
    if (v < 0 || v >= nv) return FEMGPU_ERR_IO;
  return FEMGPU_OK;
}

// MAT v5 sparse (FEMSolver::readMatlabSparseMatrix, src/FEMSolver.cu:177-356):
// 128-byte header, miMATRIX, array flags (class 5 = sparse), dimensions, name
// (short or long tag), int32 row indices, int32 column offsets, double values.
struct MatSparse {
  int64_t rows = 0, cols = 0;
  std::vector<int32_t> rp, ci;
  std::vector<double> v;
};

bool rd(std::ifstream& in, void* p, size_t n) { return (bool)in.read((char*)p, n); }

femgpu_status read_mat_header(std::ifstream& in, uint32_t* mclass, int32_t* xdim, int32_t* ydim, bool sparse_ok) {
  char buf[128];
  if (!rd(in, buf, 128)) return FEMGPU_ERR_IO;
  int32_t type;
  uint32_t size;
  if (!rd(in, &type, 4) || type != 14) return FEMGPU_ERR_IO;  // 15 = compressed: unsupported
  if (!rd(in, &size, 4)) return FEMGPU_ERR_IO;
  int32_t ftype, fsize;
  if (!rd(in, &ftype, 4) || (ftype != 6 && ftype != 5) || !rd(in, &fsize, 4)) return FEMGPU_ERR_IO;
  uint32_t flags, nzmax;
  if (!rd(in, &flags, 4) || !rd(in, &nzmax, 4)) return FEMGPU_ERR_IO;
  *mclass = flags & 0xFF;
  if (!sparse_ok && *mclass == 5) return FEMGPU_ERR_IO;
  int32_t dtype, dbytes;
  if (!rd(in, &dtype, 4) || !rd(in, &dbytes, 4) || (dtype != 6 && dtype != 5) || dbytes != 8) return FEMGPU_ERR_IO;
  if (!rd(in, xdim, 4) || !rd(in, ydim, 4)) return FEMGPU_ERR_IO;
  uint16_t ntype = 0, nlen16 = 0;
  if (!rd(in, &ntype, 2) || !rd(in, &nlen16, 2)) return FEMGPU_ERR_IO;
  uint32_t nlen = nlen16;
  uint32_t align = 4;
  if (nlen16 == 0) {  // long-form tag: 4-byte type, 4-byte length, 8-byte padding
    if (!rd(in, &nlen, 4)) return FEMGPU_ERR_IO;
    align = 8;
  }
  if (ntype != 1 && ntype != 2) return FEMGPU_ERR_IO;
  if (nlen % align) nlen += align - nlen % align;
  std::vector<char> name(nlen);
  if (nlen && !rd(in, name.data(), nlen)) return FEMGPU_ERR_IO;
  return FEMGPU_OK;
}

femgpu_status read_mat_sparse(const char* file, MatSparse& M) {
  std::ifstream in(file, std::ios::binary);
  if (!in.is_open()) return FEMGPU_ERR_IO;
  uint32_t mclass;
  int32_t xdim, ydim;
  femgpu_status st = read_mat_header(in, &mclass, &xdim, &ydim, true);
  if (st != FEMGPU_OK || mclass != 5 || xdim <= 0 || ydim <= 0) return FEMGPU_ERR_IO;
  auto read_int_block = [&](std::vector<int32_t>& out) -> bool {
    int32_t type, bytes;
    if (!rd(in, &type, 4) || (type != 6 && type != 5) || !rd(in, &bytes, 4) || bytes < 0) return false;
    out.resize(bytes / 4);
    if (bytes && !rd(in, out.data(), bytes)) return false;
    char pad[8];
    if (bytes % 8 && !rd(in, pad, 8 - bytes % 8)) return false;
    return true;
  };
  std::vector<int32_t> ir, jc;
  if (!read_int_block(ir) || !read_int_block(jc)) return FEMGPU_ERR_IO;
  if ((int64_t)jc.size() < (int64_t)ydim + 1) return FEMGPU_ERR_IO;
  int32_t type, bytes;
  if (!rd(in, &type, 4) || type != 9 || !rd(in, &bytes, 4) || bytes < 0) return FEMGPU_ERR_IO;
  std::vector<double> val(bytes / 8);
  if (bytes && !rd(in, val.data(), bytes)) return FEMGPU_ERR_IO;
  int64_t nnz = jc[ydim];
  if (nnz > (int64_t)ir.size() || nnz > (int64_t)val.size()) return FEMGPU_ERR_IO;
  // column-compressed -> CSR with sorted columns
  M.rows = xdim;
  M.cols = ydim;
  M.rp.assign(xdim + 1, 0);
  for (int64_t e = 0; e < nnz; e++) {
    if (ir[e] < 0 || ir[e] >= xdim) return FEMGPU_ERR_IO;
    M.rp[ir[e] + 1]++;
  }
  for (int i = 0; i < xdim; i++) M.rp[i + 1] += M.rp[i];
  M.ci.resize(nnz);
  M.v.resize(nnz);
  std::vector<int32_t> cur(M.rp.begin(), M.rp.end() - 1);
  for (int32_t j = 0; j < ydim; j++)
    for (int32_t e = jc[j]; e < jc[j + 1]; e++) {
      int32_t q = cur[ir[e]]++;
      M.ci[q] = j;
      M.v[q] = val[e];
    }
  return FEMGPU_OK;
}

femgpu_status read_mat_array(const char* file, std::vector<double>& out) {
  std::ifstream in(file, std::ios::binary);
  if (!in.is_open()) return FEMGPU_ERR_IO;
  uint32_t mclass;
  int32_t xdim, ydim;
  femgpu_status st = read_mat_header(in, &mclass, &xdim, &ydim, false);
  if (st != FEMGPU_OK) return st;
  int32_t type;
  uint32_t bytes;
  if (!rd(in, &type, 4) || type != 9 || !rd(in, &bytes, 4)) return FEMGPU_ERR_IO;
  out.resize(bytes / 8);
  if (bytes && !rd(in, out.data(), bytes)) return FEMGPU_ERR_IO;
  return FEMGPU_OK;
}

}  // namespace

extern "C" {

femgpu_status femgpu_read_tetgen(const char* node_file, const char* ele_file, int64_t* nverts, int64_t* nelems,
                                 double* xyz, int32_t* conn, int32_t* labels) {
  if (!node_file || !ele_file || !nverts || !nelems) return FEMGPU_ERR_INVALID;
  TetFile t;
  femgpu_status st = read_tetgen(node_file, ele_file, t);
  if (st != FEMGPU_OK) return st;
  *nverts = (int64_t)t.xyz.size() / 3;
  *nelems = (int64_t)t.labels.size();
  if (xyz) std::copy(t.xyz.begin(), t.xyz.end(), xyz);
  if (conn) std::copy(t.conn.begin(), t.conn.end(), conn);
  if (labels) std::copy(t.labels.begin(), t.labels.end(), labels);
  return FEMGPU_OK;
}

femgpu_status femgpu_read_ply(const char* file, int64_t* nverts, int64_t* nfaces, double* xyz, int32_t* conn) {
  if (!file || !nverts || !nfaces) return FEMGPU_ERR_INVALID;
  std::vector<double> v;
  std::vector<int32_t> f;
  femgpu_status st = read_ply(file, v, f);
  if (st != FEMGPU_OK) return st;
  *nverts = (int64_t)v.size() / 3;
  *nfaces = (int64_t)f.size() / 3;
  if (xyz) std::copy(v.begin(), v.end(), xyz);
  if (conn) std::copy(f.begin(), f.end(), conn);
  return FEMGPU_OK;
}

femgpu_status femgpu_read_mat_sparse(const char* file, int64_t* rows, int64_t* cols, int64_t* nnz, int32_t* rowptr,
                                     int32_t* colidx, double* vals) {
  if (!file || !rows || !cols || !nnz) return FEMGPU_ERR_INVALID;
  MatSparse M;
  femgpu_status st = read_mat_sparse(file, M);
  if (st != FEMGPU_OK) return st;
  *rows = M.rows;
  *cols = M.cols;
  *nnz = (int64_t)M.ci.size();
  if (rowptr) std::copy(M.rp.begin(), M.rp.end(), rowptr);
  if (colidx) std::copy(M.ci.begin(), M.ci.end(), colidx);
  if (vals) std::copy(M.v.begin(), M.v.end(), vals);
  return FEMGPU_OK;
}

femgpu_status femgpu_read_mat_array(const char* file, int64_t* n, double* vals) {
  if (!file || !n) return FEMGPU_ERR_INVALID;
  std::vector<double> v;
  femgpu_status st = read_mat_array(file, v);
  if (st != FEMGPU_OK) return st;
  *n = (int64_t)v.size();
  if (vals) std::copy(v.begin(), v.end(), vals);
  return FEMGPU_OK;
}

// FEMSolver::writeMatlabArray (src/FEMSolver.cu:451-517): a column vector x_h.
femgpu_status femgpu_write_mat_array(const char* file, int64_t n, const double* vals) {
  if (!file || n < 0 || (n && !vals)) return FEMGPU_ERR_INVALID;
  std::ofstream f(file, std::ios::binary);
  if (!f.is_open()) return FEMGPU_ERR_IO;
  std::string desc = "MATLAB 5.0 MAT-file, Platform: GLNXA64, Created by femgpu.";
  desc.resize(116, ' ');
  f.write(desc.data(), 116);
  char zeros[8] = {0};
  f.write(zeros, 8);
  int16_t version = 0x0100;
  f.write((char*)&version, 2);
  f.write("IM", 2);
  int32_t miMATRIX = 14;
  int32_t total = (int32_t)(16 + 16 + 8 + 8 + 8 + n * 8);
  f.write((char*)&miMATRIX, 4);
  f.write((char*)&total, 4);
  int32_t hdr[4] = {6, 8, 6, 0};  // array flags: miUINT32, 8 bytes, class double
  f.write((char*)hdr, 16);
  int32_t dims[4] = {5, 8, (int32_t)n, 1};
  f.write((char*)dims, 16);
  int16_t ntag[2] = {1, 3};
  f.write((char*)ntag, 4);
  f.write("x_h\0", 4);
  int32_t dt[2] = {9, (int32_t)(n * 8)};
  f.write((char*)dt, 8);
  f.write((const char*)vals, n * 8);
  return f.good() ? FEMGPU_OK : FEMGPU_ERR_IO;
}

// FEMSolver::writeVTK (src/FEMSolver.cu:519-582): legacy ASCII unstructured grid.
femgpu_status femgpu_write_vtk(const char* file, int dim, int64_t nverts, const double* xyz, int64_t nelems,
                               const int32_t* conn, const double* values) {
  if (!file || !xyz || !conn || (dim != 2 && dim != 3)) return FEMGPU_ERR_INVALID;
  FILE* f = fopen(file, "w");
  if (!f) return FEMGPU_ERR_IO;
  int k = dim + 1;
  fprintf(f, "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  fprintf(f, "POINTS %lld float\n", (long long)nverts);
  for (int64_t i = 0; i < nverts; i++) fprintf(f, "%.12f %.12f %.12f\n", xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]);
  fprintf(f, "CELLS %lld %lld\n", (long long)nelems, (long long)(nelems * (k + 1)));
  for (int64_t e = 0; e < nelems; e++) {
    fprintf(f, "%d", k);
    for (int a = 0; a < k; a++) fprintf(f, " %d", conn[e * k + a]);
    fprintf(f, "\n");
  }
  fprintf(f, "CELL_TYPES %lld\n", (long long)nelems);
  for (int64_t e = 0; e < nelems; e++) fprintf(f, "%d\n", dim == 3 ? 10 : 5);
  if (values) {
    fprintf(f, "POINT_DATA %lld\nSCALARS traveltime float 1\nLOOKUP_TABLE default\n", (long long)nverts);
    for (int64_t i = 0; i < nverts; i++) fprintf(f, "%.12f\n", values[i]);
  }
  fclose(f);
  return FEMGPU_OK;
}

}  // extern "C"
