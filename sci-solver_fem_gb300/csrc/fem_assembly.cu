// fem_assembly.cu -- mesh pattern and P1 element assembly on the device.
//
// Pattern: vertex -> (element, local vertex) incidence lists, sorted, then each
// row's column set is the sorted union of the vertices of its incident elements
// (the row of tetmesh2ell / trimesh2ell, src/core/cuda/cutil.cu:168-230,297-348,
// with the diagonal in its sorted place).
//
// Assembly: one thread per element computes the element's upper-triangle
// entries (perform_element_loop_3D.cuh:480-627 / perform_element_loop_2D.cuh:287-372)
// into a per-element table; one thread per row then gathers its entries from the
// incident elements in element order.  No floating-point atomics: the sum at
// every slot is taken in element order, so results are bitwise reproducible and
// equal to a sequential element loop.  Tetrahedra use a fused multiply-add gradient
// formulation (tet_gradients), within a few units in the last place of the reference's
// cofactor inverse; triangles follow the reference's arithmetic.
#include "context.cuh"
#include "quadrature.h"

namespace femgpu {

namespace {

__constant__ double c_tet_mass[10];
__constant__ double c_tri_q[24];  // zx[6], wx[6], zy[6], wy[6]

// Index of entry (a, b) in the packed upper triangle of a k x k element matrix.
__device__ __forceinline__ int upper_index(int a, int b, int k) {
  int i = a < b ? a : b, j = a < b ? b : a;
  return i * k - (i * (i - 1)) / 2 + (j - i);
}

__device__ __forceinline__ double label_coef(int label) {
  // co of element_loop_3d_kernel (perform_element_loop_3D.cuh:585-612)
  return label == 2 ? 2.0 : label == 3 ? 3.0 : label == 4 ? 4.0 : label == 5 ? 5.0 : label == 6 ? 6.0 : 1.0;
}

// ---- pattern ----------------------------------------------------------------------
__global__ void incidence_count_kernel(const int32_t* conn, int64_t nslots, int32_t* deg, int nv, int32_t* bad) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nslots; q += (int64_t)gridDim.x * blockDim.x) {
    int v = conn[q];
    if (v < 0 || v >= nv) {
      atomicExch(bad, 1);
      continue;
    }
    atomicAdd(&deg[v], 1);
  }
}

__global__ void incidence_fill_kernel(const int32_t* conn, int64_t nslots, const int32_t* vstart, int32_t* cursor,
                                      int32_t* inc) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nslots; q += (int64_t)gridDim.x * blockDim.x) {
    int v = conn[q];
    int pos = atomicAdd(&cursor[v], 1);
    inc[vstart[v] + pos] = (int32_t)q;  // q = e * k + a
  }
}

__global__ void times_k_kernel(const int32_t* deg, int nv, int k, int32_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) out[i] = deg[i] * k;
}

__global__ void candidates_kernel(const int32_t* conn, const int32_t* vstart, const int32_t* inc, const int32_t* coff,
                                  int nv, int k, int32_t* cand) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    int o = coff[v];
    for (int q = vstart[v]; q < vstart[v + 1]; q++) {
      int e = inc[q] / k;
      for (int b = 0; b < k; b++) cand[o++] = conn[(int64_t)e * k + b];
    }
  }
}

__global__ void compact_rows_kernel(const int32_t* cand, const int32_t* coff, const int32_t* rowptr, int nv,
                                    int32_t* cols) {
  // warp per row
  int lane = threadIdx.x & 31;
  for (int v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nv; v += (gridDim.x * blockDim.x) >> 5) {
    int len = rowptr[v + 1] - rowptr[v];
    for (int t = lane; t < len; t += 32) cols[rowptr[v] + t] = cand[coff[v] + t];
  }
}

__global__ void graph_from_pattern_kernel(const int32_t* rowptr, const int32_t* cols, int n, int32_t* xadj,
                                          int32_t* adj) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int o = rowptr[i] - i;  // one diagonal entry per earlier row
    if (i == 0) xadj[0] = 0;
    int c = 0;
    for (int e = rowptr[i]; e < rowptr[i + 1]; e++)
      if (cols[e] != i) adj[o + c++] = cols[e];
    xadj[i + 1] = o + c;
  }
}

// ---- assembly --------------------------------------------------------------------
// P1 basis gradients of tetrahedron e from its edge vectors (a fused multiply-add
// formulation; the CPU oracle evaluates the same operations in the same order):
// with a = p1 - p0, b = p2 - p0, c = p3 - p0 and det = a . (b x c),
// grad l1 = (b x c) / det, grad l2 = (c x a) / det, grad l3 = (a x b) / det,
// grad l0 = -((grad l1 + grad l2) + grad l3); the volume is |det| / 6.  About a quarter of
// the floating-point work of the 4x4 cofactor inverse (perform_element_loop_3D.cuh:
// 525-583), which it matches to a few units in the last place.
__device__ __forceinline__ void cross_fma(const double u[3], const double v[3], double w[3]) {
  w[0] = fma(u[1], v[2], -(u[2] * v[1]));
  w[1] = fma(u[2], v[0], -(u[0] * v[2]));
  w[2] = fma(u[0], v[1], -(u[1] * v[0]));
}

__device__ __forceinline__ void tet_gradients(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                                              int64_t e, double& det, double g[4][3]) {
  double p[4][3];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int64_t v = conn[e * 4 + q];
#pragma unroll
    for (int d = 0; d < 3; d++) p[q][d] = xyz[v * 3 + d];
  }
  double a[3], b[3], c[3], bc[3], ca[3], ab[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    a[d] = p[1][d] - p[0][d];
    b[d] = p[2][d] - p[0][d];
    c[d] = p[3][d] - p[0][d];
  }
  cross_fma(b, c, bc);
  cross_fma(c, a, ca);
  cross_fma(a, b, ab);
  det = fma(a[0], bc[0], fma(a[1], bc[1], a[2] * bc[2]));
  const double inv = 1.0 / det;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    g[1][d] = bc[d] * inv;
    g[2][d] = ca[d] * inv;
    g[3][d] = ab[d] * inv;
    g[0][d] = -((g[1][d] + g[2][d]) + g[3][d]);
  }
}

// Element matrices of P1 tetrahedra: the 10 upper-triangle entries of co K_e + lambda M_e
// (perform_element_loop_3D.cuh:28-116,480-627): K_ab = vol grad l_a . grad l_b, the mass
// from the reference-element integrand table times |det| / 8.
__global__ void element3d_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                                 const int32_t* __restrict__ labels, const double* __restrict__ coef, int64_t ne,
                                 double lambda, double* __restrict__ ev) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double det, g[4][3];
    tet_gradients(xyz, conn, e, det, g);
    const double co = coef ? coef[e] : (labels ? label_coef(labels[e]) : 1.0);
    const double wk = (fabs(det) / 6.0) * co;
    const double jac = fabs(det) * 0.125;
    int c = 0;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
#pragma unroll
      for (int q = kk; q < 4; q++) {
        const double st = fma(g[kk][0], g[q][0], fma(g[kk][1], g[q][1], g[kk][2] * g[q][2])) * wk;
        ev[(int64_t)c * ne + e] = fma(lambda, c_tet_mass[c] * jac, st);  // SoA: entry-major stores
        c++;
      }
    }
  }
}

__global__ void element2d_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                                 const double* __restrict__ coef, int64_t ne, double lambda, double* __restrict__ ev) {
  const double* zx = c_tri_q;
  const double* wx = c_tri_q + 6;
  const double* zy = c_tri_q + 12;
  const double* wy = c_tri_q + 18;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double x[3], y[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      int v = conn[e * 3 + a];
      x[a] = xyz[(int64_t)v * 3];
      y[a] = xyz[(int64_t)v * 3 + 1];
    }
    double area = fabs(x[0] * y[2] - x[0] * y[1] + x[1] * y[0] - x[1] * y[2] + x[2] * y[1] - x[2] * y[0]) / 2.0;
    double a11 = x[0], a12 = y[0], a13 = 1.0, a21 = x[1], a22 = y[1], a23 = 1.0, a31 = x[2], a32 = y[2], a33 = 1.0;
    double det = a11 * a22 * a33 + a21 * a32 * a13 + a31 * a12 * a23 - a11 * a32 * a23 - a31 * a22 * a13 - a21 * a12 * a33;
    double cf[9] = {(a22 * a33 - a23 * a32) / det, (a23 * a31 - a21 * a33) / det, (a21 * a32 - a22 * a31) / det,
                    (a13 * a32 - a12 * a33) / det, (a11 * a33 - a13 * a31) / det, (a12 * a31 - a11 * a32) / det,
                    (a12 * a23 - a13 * a22) / det, (a13 * a21 - a11 * a23) / det, (a11 * a22 - a12 * a21) / det};
    double jacobi = (x[0] * y[1] - x[1] * y[0] - x[0] * y[2] + x[2] * y[0] + x[1] * y[2] - x[2] * y[1]) / 8;
    double co = coef ? coef[e] : 1.0;
    int c = 0;
    for (int k = 0; k < 3; k++)
      for (int q = k; q < 3; q++) {
        double A1 = cf[3 * k], B1 = cf[3 * k + 1], C1 = cf[3 * k + 2];
        double A2 = cf[3 * q], B2 = cf[3 * q + 1], C2 = cf[3 * q + 2];
        double st = (A1 * A2 + B1 * B2) * area * co;
        double integral = 0;
        for (int i = 0; i < 6; i++) {
          double ty = 0.0;
          for (int j = 0; j < 6; j++) {
            double px = x[0] * (1 - zx[i]) * 0.5 * (1 - zy[j]) * 0.5 + x[1] * (1 + zx[i]) * 0.5 * (1 - zy[j]) * 0.5 +
                        x[2] * (1 + zy[j]) * 0.5;
            double py = y[0] * (1 - zx[i]) * 0.5 * (1 - zy[j]) * 0.5 + y[1] * (1 + zx[i]) * 0.5 * (1 - zy[j]) * 0.5 +
                        y[2] * (1 + zy[j]) * 0.5;
            double f = (A1 * px + B1 * py + C1) * (A2 * px + B2 * py + C2) * jacobi;
            ty += f * wy[j];
          }
          integral += ty * wx[i];
        }
        ev[(int64_t)c * ne + e] = st + lambda * integral;
        c++;
      }
  }
}

// Positions within its row of every (incidence, element vertex) pair, for the gather
// below (one binary search each, once per mesh).
__global__ void slot_map_kernel(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
                                const int32_t* __restrict__ vstart, const int32_t* __restrict__ inc,
                                const int32_t* __restrict__ conn, int nv, int k, uint8_t* __restrict__ slot,
                                int32_t* bad) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    const int rb = rowptr[v], re = rowptr[v + 1];
    for (int q = vstart[v]; q < vstart[v + 1]; q++) {
      const int e = inc[q] / k;
      for (int b = 0; b < k; b++) {
        const int col = conn[(int64_t)e * k + b];
        const int s = lower_bound_i32(cols, rb, re, col);
        if (s >= re || cols[s] != col) {
          atomicExch(bad, 1);
          slot[(int64_t)q * k + b] = 0;
          continue;
        }
        slot[(int64_t)q * k + b] = (uint8_t)(s - rb);
      }
    }
  }
}

// One thread per row with its row's sums in shared memory (at most kSlotRowMax entries,
// kSlotRowMax + 1 doubles apart per thread): the incident elements' contributions added
// in element order at the positions the slot map gives, then the row written out.
__global__ void gather_rows_slot_kernel(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ vstart,
                                        const int32_t* __restrict__ inc, const uint8_t* __restrict__ slot,
                                        const double* __restrict__ ev, int64_t ne, int nv, int k,
                                        double* __restrict__ vals) {
  extern __shared__ double acc_all[];
  double* acc = acc_all + threadIdx.x * (kSlotRowMax + 1);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    const int rb = rowptr[v], len = rowptr[v + 1] - rb;
    for (int s = 0; s < len; s++) acc[s] = 0.0;
    for (int q = vstart[v]; q < vstart[v + 1]; q++) {
      const int code = inc[q];
      const int e = code / k, a = code - e * k;
      for (int b = 0; b < k; b++) acc[slot[(int64_t)q * k + b]] += ev[(int64_t)upper_index(a, b, k) * ne + e];
    }
    for (int s = 0; s < len; s++) vals[rb + s] = acc[s];
  }
}

// One thread per row: contributions of the incident elements, in element order.
__global__ void gather_rows_kernel(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
                                   const int32_t* __restrict__ vstart, const int32_t* __restrict__ inc,
                                   const int32_t* __restrict__ conn, const double* __restrict__ ev, int64_t ne, int nv,
                                   int k, double* __restrict__ vals, int32_t* bad) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    int rb = rowptr[v], re = rowptr[v + 1];
    for (int s = rb; s < re; s++) vals[s] = 0.0;
    for (int q = vstart[v]; q < vstart[v + 1]; q++) {
      int code = inc[q];
      int e = code / k, a = code - e * k;
      for (int b = 0; b < k; b++) {
        int col = conn[(int64_t)e * k + b];
        int s = lower_bound_i32(cols, rb, re, col);
        if (s >= re || cols[s] != col) {
          atomicExch(bad, 1);
          continue;
        }
        vals[s] += ev[(int64_t)upper_index(a, b, k) * ne + e];
      }
    }
  }
}

__global__ void element_load_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                                    const double* __restrict__ f, int64_t ne, int k, double* __restrict__ scale,
                                    double* __restrict__ fsum) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double meas;
    if (k == 4) {
      double x[4], y[4], z[4];
      for (int a = 0; a < 4; a++) {
        int v = conn[e * 4 + a];
        x[a] = xyz[(int64_t)v * 3];
        y[a] = xyz[(int64_t)v * 3 + 1];
        z[a] = xyz[(int64_t)v * 3 + 2];
      }
      double a1 = x[1] - x[3], a2 = y[1] - y[3], a3 = z[1] - z[3];
      double b1 = x[2] - x[3], b2 = y[2] - y[3], b3 = z[2] - z[3];
      double c1 = x[0] - x[3], c2 = y[0] - y[3], c3 = z[0] - z[3];
      meas = fabs(c1 * (a2 * b3 - a3 * b2) + c2 * (a3 * b1 - a1 * b3) + c3 * (a1 * b2 - a2 * b1)) / 6.0;
    } else {
      int v0 = conn[e * 3], v1 = conn[e * 3 + 1], v2 = conn[e * 3 + 2];
      double x0 = xyz[(int64_t)v0 * 3], y0 = xyz[(int64_t)v0 * 3 + 1];
      double x1 = xyz[(int64_t)v1 * 3], y1 = xyz[(int64_t)v1 * 3 + 1];
      double x2 = xyz[(int64_t)v2 * 3], y2 = xyz[(int64_t)v2 * 3 + 1];
      meas = fabs(x0 * y2 - x0 * y1 + x1 * y0 - x1 * y2 + x2 * y1 - x2 * y0) / 2.0;
    }
    double fs = 0;
    for (int a = 0; a < k; a++) fs += f[conn[e * k + a]];
    scale[e] = meas / (double)(k * (k + 1));
    fsum[e] = fs;
  }
}

__global__ void gather_load_kernel(const int32_t* vstart, const int32_t* inc, const double* scale, const double* fsum,
                                   const double* f, int nv, int k, double* b) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    double s = 0.0;
    double fv = f[v];
    for (int q = vstart[v]; q < vstart[v + 1]; q++) {
      int e = inc[q] / k;
      s += scale[e] * (fsum[e] + fv);
    }
    b[v] = s;
  }
}

__global__ void dirichlet_kernel(const int32_t* rowptr, const int32_t* cols, double* vals, const uint8_t* mask, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool mi = mask[i] != 0;
    for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
      int j = cols[e];
      if (mi || mask[j]) vals[e] = (i == j) ? 1.0 : 0.0;
    }
  }
}

// dL/dtheta_e = -c_e * vol_e * grad(lambda)_e . grad(u)_e for P1 tetrahedra: the
// derivative of lambda^T A(theta) u through the stiffness term c_e K_e with
// c_e = exp(theta_e) (the mass term does not depend on theta).
__global__ void grad3d_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                              const int32_t* __restrict__ labels, const double* __restrict__ coef, int64_t ne,
                              const double* __restrict__ lam, const double* __restrict__ u,
                              double* __restrict__ grad) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double det, g[4][3];
    tet_gradients(xyz, conn, e, det, g);
    const double vol = fabs(det) / 6.0;
    double gl[3] = {0.0, 0.0, 0.0}, gu[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int v = conn[e * 4 + a];
      const double la = lam[v], ua = u[v];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        gl[d] = fma(la, g[a][d], gl[d]);
        gu[d] = fma(ua, g[a][d], gu[d]);
      }
    }
    const double co = coef ? coef[e] : (labels ? label_coef(labels[e]) : 1.0);
    grad[e] = -co * vol * (gl[0] * gu[0] + gl[1] * gu[1] + gl[2] * gu[2]);
  }
}

// The same for P1 triangles (basis gradients from the 3x3 cofactor inverse).
__global__ void grad2d_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ conn,
                              const double* __restrict__ coef, int64_t ne, const double* __restrict__ lam,
                              const double* __restrict__ u, double* __restrict__ grad) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    double x[3], y[3], la[3], ua[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int v = conn[e * 3 + a];
      x[a] = xyz[(int64_t)v * 3];
      y[a] = xyz[(int64_t)v * 3 + 1];
      la[a] = lam[v];
      ua[a] = u[v];
    }
    const double area = fabs(x[0] * y[2] - x[0] * y[1] + x[1] * y[0] - x[1] * y[2] + x[2] * y[1] - x[2] * y[0]) / 2.0;
    const double det = x[0] * y[1] + x[1] * y[2] + x[2] * y[0] - x[0] * y[2] - x[2] * y[1] - x[1] * y[0];
    // gradient of basis a: ((y[b] - y[c]) / det, (x[c] - x[b]) / det) with (a, b, c) cyclic
    double gl[2] = {0.0, 0.0}, gu[2] = {0.0, 0.0};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int b = (a + 1) % 3, c = (a + 2) % 3;
      const double gx = (y[b] - y[c]) / det, gy = (x[c] - x[b]) / det;
      gl[0] = fma(la[a], gx, gl[0]);
      gl[1] = fma(la[a], gy, gl[1]);
      gu[0] = fma(ua[a], gx, gu[0]);
      gu[1] = fma(ua[a], gy, gu[1]);
    }
    const double co = coef ? coef[e] : 1.0;
    grad[e] = -co * area * (gl[0] * gu[0] + gl[1] * gu[1]);
  }
}

__global__ void mask_rows_kernel(int n, const uint8_t* __restrict__ mask, const double* __restrict__ in,
                                 double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (mask && mask[i]) ? 0.0 : in[i];
}

__global__ void row_length_kernel(const int32_t* rowptr, int n, int32_t* len) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) len[i] = rowptr[i + 1] - rowptr[i];
}

// Longest row of the level-0 pattern.
int reduce_max_row_length(Ctx& c) {
  DBuf<int32_t> len(c.A.n > 0 ? c.A.n : 1, c.stream);
  FG_LAUNCH(row_length_kernel, grid_for(c.A.n, 256), 256, 0, c.stream, c.A.rp.p, c.A.n, len.p);
  return reduce_max(len.p, c.A.n, c.stream);
}

// Row gather of the element entries into the operator's values (slot map when built).
void gather_rows(Ctx& c, const double* ev, double* vals) {
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  if (M.slot.n) {
    const size_t smem = (size_t)128 * (kSlotRowMax + 1) * sizeof(double);
    FG_LAUNCH(gather_rows_slot_kernel, grid_for(M.nv, 128), 128, smem, s, c.A.rp.p, M.vstart.p, M.inc.p, M.slot.p,
              ev, M.ne, (int)M.nv, M.k, vals);
    return;
  }
  DBuf<int32_t> bad(1, s);
  bad.zero();
  FG_LAUNCH(gather_rows_kernel, grid_for(M.nv, 128), 128, 0, s, c.A.rp.p, c.A.ci.p, M.vstart.p, M.inc.p, M.conn.p,
            ev, M.ne, (int)M.nv, M.k, vals, bad.p);
  FG_REQUIRE(read_scalar(bad.p, s) == 0, FEMGPU_ERR_INVALID, "element entry outside the pattern");
}

}  // namespace

void build_mesh_pattern(Ctx& c) {
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  const int nv = (int)M.nv, k = M.k;
  const int64_t nslots = M.ne * k;
  DBuf<int32_t> deg(nv + 1, s), bad(1, s);
  deg.zero();
  bad.zero();
  FG_LAUNCH(incidence_count_kernel, grid_for(nslots, 256), 256, 0, s, M.conn.p, nslots, deg.p, nv, bad.p);
  FG_REQUIRE(read_scalar(bad.p, s) == 0, FEMGPU_ERR_INVALID, "element connectivity references a vertex out of range");
  M.vstart.alloc(nv + 1, s);
  int64_t total = exclusive_scan(deg.p, M.vstart.p, nv, s);
  FG_REQUIRE(total == nslots, FEMGPU_ERR_INVALID, "incidence count mismatch");
  M.inc.alloc(nslots, s);
  DBuf<int32_t> cursor(nv, s);
  cursor.zero();
  FG_LAUNCH(incidence_fill_kernel, grid_for(nslots, 256), 256, 0, s, M.conn.p, nslots, M.vstart.p, cursor.p, M.inc.p);
  segmented_sort_i32(M.inc.p, M.vstart.p, nv, nullptr, s);
  // candidate columns: all vertices of every incident element (includes the row itself)
  DBuf<int32_t> ccount(nv + 1, s), coff(nv + 1, s);
  FG_LAUNCH(times_k_kernel, grid_for(nv, 256), 256, 0, s, deg.p, nv, k, ccount.p);
  int64_t ncand = exclusive_scan(ccount.p, coff.p, nv, s);
  FG_REQUIRE(ncand < INT32_MAX, FEMGPU_ERR_LIMIT, "pattern candidate count exceeds int32");
  DBuf<int32_t> cand(ncand > 0 ? ncand : 1, s);
  FG_LAUNCH(candidates_kernel, grid_for(nv, 128), 128, 0, s, M.conn.p, M.vstart.p, M.inc.p, coff.p, nv, k, cand.p);
  DBuf<int32_t> ucount(nv + 1, s);
  segmented_sort_i32(cand.p, coff.p, nv, ucount.p, s);
  // isolated vertices still get their diagonal
  c.A.n = c.A.m = nv;
  c.A.rp.alloc(nv + 1, s);
  int64_t nnz = exclusive_scan(ucount.p, c.A.rp.p, nv, s);
  c.A.nnz = nnz;
  c.A.ci.alloc(nnz, s);
  c.A.v.alloc(nnz, s);
  c.A.v.zero();
  FG_LAUNCH(compact_rows_kernel, grid_for((int64_t)nv * 32, 256), 256, 0, s, cand.p, coff.p, c.A.rp.p, nv, c.A.ci.p);
  // slot map for the assembly's row gather, when every row fits its shared-memory sums
  M.slot.release();
  if (reduce_max_row_length(c) <= kSlotRowMax) {
    M.slot.alloc((size_t)nslots * k, s);
    DBuf<int32_t> bad2(1, s);
    bad2.zero();
    FG_LAUNCH(slot_map_kernel, grid_for(nv, 128), 128, 0, s, c.A.rp.p, c.A.ci.p, M.vstart.p, M.inc.p, M.conn.p, nv,
              k, M.slot.p, bad2.p);
    FG_REQUIRE(read_scalar(bad2.p, s) == 0, FEMGPU_ERR_INVALID, "element vertex outside the pattern");
  }
  // level-0 aggregation graph: the pattern without self loops
  c.gxadj.alloc(nv + 1, s);
  c.gadj.alloc(nnz - nv > 0 ? nnz - nv : 1, s);
  FG_LAUNCH(graph_from_pattern_kernel, grid_for(nv, 256), 256, 0, s, c.A.rp.p, c.A.ci.p, nv, c.gxadj.p, c.gadj.p);
  c.graph_nnz = nnz - nv;
}

void assemble_operator(Ctx& c, const double* coef_host, double lambda, bool coef_on_device) {
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  const int64_t ne = M.ne;
  const int k = M.k;
  const int nup = k == 4 ? 10 : 6;
  if (k == 4) {
    double t[10];
    tet_mass_table(t);
    FG_CUDA(cudaMemcpyToSymbolAsync(c_tet_mass, t, sizeof(t), 0, cudaMemcpyHostToDevice, s));
  } else {
    double zx[6], wx[6], zy[6], wy[6], q[24];
    tri_quadrature_table(zx, wx, zy, wy);
    for (int i = 0; i < 6; i++) {
      q[i] = zx[i];
      q[6 + i] = wx[i];
      q[12 + i] = zy[i];
      q[18 + i] = wy[i];
    }
    FG_CUDA(cudaMemcpyToSymbolAsync(c_tri_q, q, sizeof(q), 0, cudaMemcpyHostToDevice, s));
  }
  DBuf<double>& coef = c.coef;  // kept for the adjoint gradient
  c.lambda_mass = lambda;
  coef.release();
  if (coef_host) {
    coef.alloc(ne, s);
    if (coef_on_device)
      FG_CUDA(cudaMemcpyAsync(coef.p, coef_host, ne * sizeof(double), cudaMemcpyDeviceToDevice, s));
    else
      coef.upload(coef_host, ne);
  }
  DBuf<double> ev((size_t)ne * nup, s);
  if (k == 4)
    FG_LAUNCH(element3d_kernel, grid_for(ne, 128), 128, 0, s, M.xyz.p, M.conn.p, M.has_labels ? M.labels.p : nullptr,
              coef.p, ne, lambda, ev.p);
  else
    FG_LAUNCH(element2d_kernel, grid_for(ne, 128), 128, 0, s, M.xyz.p, M.conn.p, coef.p, ne, lambda, ev.p);
  gather_rows(c, ev.p, c.A.v.p);
}

void load_vector(Ctx& c, const double* f_host, double* b_host) {
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  DBuf<double> f(M.nv, s), b(M.nv, s), sc(M.ne, s), fs(M.ne, s);
  f.upload(f_host, M.nv);
  FG_LAUNCH(element_load_kernel, grid_for(M.ne, 256), 256, 0, s, M.xyz.p, M.conn.p, f.p, M.ne, M.k, sc.p, fs.p);
  FG_LAUNCH(gather_load_kernel, grid_for(M.nv, 256), 256, 0, s, M.vstart.p, M.inc.p, sc.p, fs.p, f.p, (int)M.nv, M.k,
            b.p);
  b.download(b_host, M.nv);
  FG_CUDA(cudaStreamSynchronize(s));
}

void load_vector_enqueue(Ctx& c, const double* d_f, double* d_b, double* scale, double* fsum) {
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  FG_LAUNCH(element_load_kernel, grid_for(M.ne, 256), 256, 0, s, M.xyz.p, M.conn.p, d_f, M.ne, M.k, scale, fsum);
  FG_LAUNCH(gather_load_kernel, grid_for(M.nv, 256), 256, 0, s, M.vstart.p, M.inc.p, scale, fsum, d_f, (int)M.nv,
            M.k, d_b);
}

void zero_dirichlet_rows(Ctx& c, const double* d_in, double* d_out) {
  const int n = c.A.n;
  FG_LAUNCH(mask_rows_kernel, grid_for(n, 256), 256, 0, c.stream, n, c.dmask.n ? c.dmask.p : nullptr, d_in, d_out);
}

void element_log_coef_gradient(Ctx& c, const double* d_lam, const double* d_u, double* d_grad) {
  Mesh& M = c.mesh;
  const double* coef = c.coef.n ? c.coef.p : nullptr;
  if (M.k == 4)
    FG_LAUNCH(grad3d_kernel, grid_for(M.ne, 128), 128, 0, c.stream, M.xyz.p, M.conn.p,
              M.has_labels ? M.labels.p : nullptr, coef, M.ne, d_lam, d_u, d_grad);
  else
    FG_LAUNCH(grad2d_kernel, grid_for(M.ne, 128), 128, 0, c.stream, M.xyz.p, M.conn.p, coef, M.ne, d_lam, d_u,
              d_grad);
}

void profile_assembly(Ctx& c, int which, int reps, double* ms, double* bytes) {
  FG_REQUIRE(c.has_mesh && c.assembled_from_mesh, FEMGPU_ERR_NOT_READY, "no operator assembled from the mesh");
  cudaStream_t s = c.stream;
  Mesh& M = c.mesh;
  const int64_t ne = M.ne, nv = M.nv, nnz = c.A.nnz;
  const int k = M.k, nup = k == 4 ? 10 : 6;
  DBuf<double> ev((size_t)ne * nup, s), vals(nnz, s);
  const double* coef = c.coef.n ? c.coef.p : nullptr;
  auto element = [&]() {
    if (k == 4)
      FG_LAUNCH(element3d_kernel, grid_for(ne, 128), 128, 0, s, M.xyz.p, M.conn.p,
                M.has_labels ? M.labels.p : nullptr, coef, ne, c.lambda_mass, ev.p);
    else
      FG_LAUNCH(element2d_kernel, grid_for(ne, 128), 128, 0, s, M.xyz.p, M.conn.p, coef, ne, c.lambda_mass, ev.p);
  };
  auto gather = [&]() { gather_rows(c, ev.p, vals.p); };
  element();
  auto run = [&]() {
    if (which == 6) element();
    else gather();
  };
  if (which == 6)  // connectivity, coefficient and entries per element, coordinates once per vertex
    *bytes = (double)ne * (4.0 * k + (coef ? 8.0 : 0.0) + 8.0 * nup) + 24.0 * nv;
  else if (M.slot.n)  // row and incidence offsets, incidence lists, slot map, element entries, values out
    *bytes = 8.0 * (nv + 1) + 4.0 * k * ne + 1.0 * k * k * ne + 8.0 * nup * ne + 8.0 * nnz;
  else  // row offsets, columns, incidence offsets and lists, the incident elements' vertices and entries, values out
    *bytes = 8.0 * (nv + 1) + 4.0 * nnz + 4.0 * k * ne + 4.0 * k * ne + 8.0 * nup * ne + 8.0 * nnz;
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
}

void apply_dirichlet(Ctx& c, const uint8_t* mask_host) {
  cudaStream_t s = c.stream;
  DBuf<uint8_t>& mask = c.dmask;  // kept for the adjoint right-hand side
  mask.alloc(c.A.n, s);
  mask.upload(mask_host, c.A.n);
  FG_LAUNCH(dirichlet_kernel, grid_for(c.A.n, 256), 256, 0, s, c.A.rp.p, c.A.ci.p, c.A.v.p, mask.p, c.A.n);
  FG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace femgpu
