/*
 * fem_oracle.cpp -- CPU restatement of SCI-Solver_FEM's P1 FEM -> SA-AMG -> PCG path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA implementation and the
 * timed CPU baseline.  The product path never links or calls this file.
 *
 * Build: oracle/Makefile (g++ -O3 -fopenmp -ffp-contract=off).  FP contraction is
 * off so that every multiply and add rounds exactly where the CUDA kernels (built
 * with -fmad=false) round; fused operations are written as explicit fma() on both
 * sides.  Summation orders are fixed (element order, ascending column, generation
 * order) so that integer outputs are bit-exact and most floating outputs are too.
 */
#include "fem_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ===================================================================== */
/* A. glibc rand()                                                        */
/* ===================================================================== */
/* glibc's TYPE_3 additive generator (published algorithm): r[0] = seed,
 * r[i] = 16807 r[i-1] mod (2^31-1) for i < 31, r[i] = r[i-31] for 31..33,
 * r[i] = r[i-31] + r[i-3] (mod 2^32) afterwards; output k is r[k+344] >> 1.
 * randomizedMIS_GPU.cu:195-201 draws 32768 of these after srand(). */
void glibc_rand_seq(uint32_t seed, int n, int32_t* out) {
  std::vector<uint32_t> r(344 + (size_t)n);
  int32_t s0 = (int32_t)(seed == 0 ? 1u : seed);
  r[0] = (uint32_t)s0;
  int64_t w = s0;
  for (int i = 1; i < 31; i++) {
    w = (16807LL * w) % 2147483647LL;
    if (w < 0) w += 2147483647LL;
    r[i] = (uint32_t)w;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (size_t i = 34; i < 344 + (size_t)n; i++) r[i] = r[i - 31] + r[i - 3];
  for (int k = 0; k < n; k++) out[k] = (int32_t)(r[344 + (size_t)k] >> 1);
}

/* ===================================================================== */
/* B. Gauss-Jacobi quadrature (FEM3D.cu:58-368, FEM2D.cu:120-340)          */
/* ===================================================================== */
const double kPI = 3.1415927;  /* FEM2D.cu:5 / TriMesh.h:27 */

/* compute_gamma_3d (FEM3D.cu:58-136) is only ever called with positive integers,
 * where it returns (x-1)! by a product loop. */
double gamma_int(int x) {
  double ga = 1.0;
  for (int i = 2; i < x; i++) ga *= i;
  return ga;
}

/* JacobiPoly (FEM3D.cu:138-190): three-term recurrence. */
std::vector<double> jacobi_poly(int degree, const std::vector<double>& x, int alpha, int beta) {
  size_t s = x.size();
  std::vector<double> y(s);
  if (degree == 0) {
    for (size_t i = 0; i < s; i++) y[i] = 1.0;
  } else if (degree == 1) {
    for (size_t i = 0; i < s; i++) y[i] = 0.5 * ((alpha - beta) + (alpha + beta + 2.0) * x[i]);
  } else {
    double degm1 = degree - 1.0;
    double tmp = 2.0 * degm1 + alpha + beta;
    double a1 = 2.0 * (degm1 + 1) * (degm1 + alpha + beta + 1) * tmp;
    double a2 = (tmp + 1) * (alpha * alpha - beta * beta);
    double a3 = tmp * (tmp + 1.0) * (tmp + 2.0);
    double a4 = 2.0 * (degm1 + alpha) * (degm1 + beta) * (tmp + 2.0);
    std::vector<double> p1 = jacobi_poly(degree - 1, x, alpha, beta);
    std::vector<double> p2 = jacobi_poly(degree - 2, x, alpha, beta);
    for (size_t i = 0; i < s; i++) y[i] = ((a2 + a3 * x[i]) * p1[i] - a4 * p2[i]) / a1;
  }
  return y;
}

/* JacobiPolyDerivative (FEM3D.cu:192-216). */
std::vector<double> jacobi_poly_der(int degree, const std::vector<double>& x, int alpha, int beta) {
  std::vector<double> y(x.size());
  if (degree == 0) {
    for (auto& v : y) v = 0.0;
    return y;
  }
  std::vector<double> p = jacobi_poly(degree - 1, x, alpha + 1, beta + 1);
  for (size_t i = 0; i < p.size(); i++) y[i] = 0.5 * (alpha + beta + degree + 1) * p[i];
  return y;
}

/* JacobiGZeros (FEM3D.cu:218-270): Newton with deflation, EPS 1e-6, 60 iterations. */
std::vector<double> jacobi_zeros(int degree, int alpha, int beta) {
  std::vector<double> z(degree, 0.0);
  if (degree == 0) return z;
  const int maxit = 60;
  const double EPS = 1.0e-6;
  double dth = double(kPI) / (2.0 * degree);
  double rlast = 0.0;
  std::vector<double> r(1);
  for (int k = 0; k < degree; k++) {
    r[0] = -cos((2.0 * k + 1.0) * dth);
    if (k) r[0] = 0.5 * (r[0] + rlast);
    for (int j = 0; j < maxit; j++) {
      std::vector<double> poly = jacobi_poly(degree, r, alpha, beta);
      std::vector<double> pder = jacobi_poly_der(degree, r, alpha, beta);
      double sum = 0.0;
      for (int i = 0; i < k; i++) sum = sum + 1.0 / (r[0] - z[i]);
      double delr = -poly[0] / (pder[0] - sum * poly[0]);
      r[0] = r[0] + delr;
      if (fabs(delr) < EPS) break;
    }
    z[k] = r[0];
    rlast = r[0];
  }
  return z;
}

/* JacobiGLZW (FEM3D.cu:272-316): Gauss-Lobatto zeros and weights. */
void jacobi_glzw(std::vector<double>& Z, std::vector<double>& W, int degree, int alpha, int beta) {
  Z.assign(degree, 0.0);
  W.assign(degree, 0.0);
  if (degree == 1) return;
  int apb = alpha + beta;
  Z[0] = -1;
  Z[degree - 1] = 1;
  std::vector<double> t = jacobi_zeros(degree - 2, alpha + 1, beta + 1);
  for (int i = 1; i < degree - 1; i++) Z[i] = t[i - 1];
  W = jacobi_poly(degree - 1, Z, alpha, beta);
  double tmp1 = pow(2.0, (double)(apb + 1));
  double tmp2 = gamma_int(alpha + degree);
  double fac = tmp1 * tmp2 * gamma_int(beta + degree);
  fac = fac / ((degree - 1) * gamma_int(degree) * gamma_int(alpha + beta + degree + 1));
  for (int j = 0; j < degree; j++) W[j] = fac / (W[j] * W[j]);
  W[0] = W[0] * (beta + 1);
  W[degree - 1] = W[degree - 1] * (alpha + 1);
}

/* JacobiGRZW (FEM3D.cu:318-366): Gauss-Radau zeros and weights. */
void jacobi_grzw(std::vector<double>& Z, std::vector<double>& W, int degree, int alpha, int beta) {
  Z.assign(degree, 0.0);
  W.assign(degree, 0.0);
  if (degree == 1) {
    W[0] = 2.0;
    return;
  }
  int apb = alpha + beta;
  Z[0] = -1;
  std::vector<double> t = jacobi_zeros(degree - 1, alpha, beta + 1);
  for (int i = 1; i < degree; i++) Z[i] = t[i - 1];
  W = jacobi_poly(degree - 1, Z, alpha, beta);
  double tmp = gamma_int(alpha + degree);
  double fac = pow(2.0, (double)apb) * tmp * gamma_int(beta + degree);
  fac = fac / (gamma_int(degree) * (beta + degree) * gamma_int(apb + degree + 1));
  for (int j = 0; j < degree; j++) W[j] = fac * (1 - Z[j]) / (W[j] * W[j]);
  W[0] = W[0] * (beta + 1);
}

/* FEM3D::assemble quadrature set-up + IntegrationInTet (FEM3D.cu:377-475,501-549). */
void tet_mass_integrand(double out[10]) {
  const int D = 4;
  std::vector<double> zx, wx, zy, wy, zz, wz;
  jacobi_glzw(zx, wx, D, 0, 0);
  jacobi_grzw(zy, wy, D, 1, 0);
  jacobi_grzw(zz, wz, D, 2, 0);
  for (int i = 0; i < D; i++) {
    wy[i] /= 2;
    wz[i] /= 4;
  }
  /* Collapsed-coordinate map (Transform2StdTetSpace) and the basis of the unit tet
   * (EvalBasisTet with rows {1,-1,-1,-1},{0,1,0,0},{0,0,1,0},{0,0,0,1}). */
  static const double coef[4][4] = {{1, -1, -1, -1}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  double phi[4][D][D][D];
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++)
      for (int k = 0; k < D; k++) {
        double cx = (1 + zx[i]) * 0.5 * (1 - zy[j]) * 0.5 * (1 - zz[k]) * 0.5;
        double cy = (1 + zy[j]) * 0.5 * (1 - zz[k]) * 0.5;
        double cz = (1 + zz[k]) * 0.5;
        for (int s = 0; s < 4; s++)
          phi[s][i][j][k] = coef[s][0] + coef[s][1] * cx + coef[s][2] * cy + coef[s][3] * cz;
      }
  int cnt = 0;
  for (int a = 0; a < 4; a++)
    for (int b = a; b < 4; b++) {
      double integral = 0;
      for (int i = 0; i < D; i++) {
        double ty = 0.0;
        for (int j = 0; j < D; j++) {
          double tz = 0.0;
          for (int k = 0; k < D; k++) tz += (phi[a][i][j][k] * phi[b][i][j][k]) * wz[k];
          ty += tz * wy[j];
        }
        integral += ty * wx[i];
      }
      out[cnt++] = integral;
    }
}

/* FEM2D::assemble (FEM2D.cu:340-378): degree 6, GL in x, GR(1,0) in y. */
void tri_quadrature(double zx[6], double wx[6], double zy[6], double wy[6]) {
  std::vector<double> a, b, c, d;
  jacobi_glzw(a, b, 6, 0, 0);
  jacobi_grzw(c, d, 6, 1, 0);
  for (int i = 0; i < 6; i++) {
    zx[i] = a[i];
    wx[i] = b[i];
    zy[i] = c[i];
    wy[i] = d[i];
  }
}

/* ===================================================================== */
/* C. Element matrices                                                    */
/* ===================================================================== */
/* The 4x4 cofactor inverse of perform_element_loop_3D.cuh:525-583.  Each cofactor
 * b_rc is a sum of six signed triple products a_{..}a_{..}a_{..}; the terms are
 * evaluated in the reference's order ((t0 + t1 + t2) - t3 - t4 - t5) so that the
 * FP64 result is bit-identical.  Encoding: entry = row*4 + col of the 0-based
 * 4x4 matrix [x y z 1] per vertex. */
struct Tri3 { unsigned char a, b, c; };
#define E(r, c) (unsigned char)(((r) - 1) * 4 + ((c) - 1))
static const Tri3 kCof[16][6] = {
  /* b11 */ {{E(2,2),E(3,3),E(4,4)},{E(2,3),E(3,4),E(4,2)},{E(2,4),E(3,2),E(4,3)},{E(2,2),E(3,4),E(4,3)},{E(2,3),E(3,2),E(4,4)},{E(2,4),E(3,3),E(4,2)}},
  /* b12 */ {{E(1,2),E(3,4),E(4,3)},{E(1,3),E(3,2),E(4,4)},{E(1,4),E(3,3),E(4,2)},{E(1,2),E(3,3),E(4,4)},{E(1,3),E(3,4),E(4,2)},{E(1,4),E(3,2),E(4,3)}},
  /* b13 */ {{E(1,2),E(2,3),E(4,4)},{E(1,3),E(2,4),E(4,2)},{E(1,4),E(2,2),E(4,3)},{E(1,2),E(2,4),E(4,3)},{E(1,3),E(2,2),E(4,4)},{E(1,4),E(2,3),E(4,2)}},
  /* b14 */ {{E(1,2),E(2,4),E(3,3)},{E(1,3),E(2,2),E(3,4)},{E(1,4),E(2,3),E(3,2)},{E(1,2),E(2,3),E(3,4)},{E(1,3),E(2,4),E(3,2)},{E(1,4),E(2,2),E(3,3)}},
  /* b21 */ {{E(2,1),E(3,4),E(4,3)},{E(2,3),E(3,1),E(4,4)},{E(2,4),E(3,3),E(4,1)},{E(2,1),E(3,3),E(4,4)},{E(2,3),E(3,4),E(4,1)},{E(2,4),E(3,1),E(4,3)}},
  /* b22 */ {{E(1,1),E(3,3),E(4,4)},{E(1,3),E(3,4),E(4,1)},{E(1,4),E(3,1),E(4,3)},{E(1,1),E(3,4),E(4,3)},{E(1,3),E(3,1),E(4,4)},{E(1,4),E(3,3),E(4,1)}},
  /* b23 */ {{E(1,1),E(2,4),E(4,3)},{E(1,3),E(2,1),E(4,4)},{E(1,4),E(2,3),E(4,1)},{E(1,1),E(2,3),E(4,4)},{E(1,3),E(2,4),E(4,1)},{E(1,4),E(2,1),E(4,3)}},
  /* b24 */ {{E(1,1),E(2,3),E(3,4)},{E(1,3),E(2,4),E(3,1)},{E(1,4),E(2,1),E(3,3)},{E(1,1),E(2,4),E(3,3)},{E(1,3),E(2,1),E(3,4)},{E(1,4),E(2,3),E(3,1)}},
  /* b31 */ {{E(2,1),E(3,2),E(4,4)},{E(2,2),E(3,4),E(4,1)},{E(2,4),E(3,1),E(4,2)},{E(2,1),E(3,4),E(4,2)},{E(2,2),E(3,1),E(4,4)},{E(2,4),E(3,2),E(4,1)}},
  /* b32 */ {{E(1,1),E(3,4),E(4,2)},{E(1,2),E(3,1),E(4,4)},{E(1,4),E(3,2),E(4,1)},{E(1,1),E(3,2),E(4,4)},{E(1,2),E(3,4),E(4,1)},{E(1,4),E(3,1),E(4,2)}},
  /* b33 */ {{E(1,1),E(2,2),E(4,4)},{E(1,2),E(2,4),E(4,1)},{E(1,4),E(2,1),E(4,2)},{E(1,1),E(2,4),E(4,2)},{E(1,2),E(2,1),E(4,4)},{E(1,4),E(2,2),E(4,1)}},
  /* b34 */ {{E(1,1),E(2,4),E(3,2)},{E(1,2),E(2,1),E(3,4)},{E(1,4),E(2,2),E(3,1)},{E(1,1),E(2,2),E(3,4)},{E(1,2),E(2,4),E(3,1)},{E(1,4),E(2,1),E(3,2)}},
  /* b41 */ {{E(2,1),E(3,3),E(4,2)},{E(2,2),E(3,1),E(4,3)},{E(2,3),E(3,2),E(4,1)},{E(2,1),E(3,2),E(4,3)},{E(2,2),E(3,3),E(4,1)},{E(2,3),E(3,1),E(4,2)}},
  /* b42 */ {{E(1,1),E(3,2),E(4,3)},{E(1,2),E(3,3),E(4,1)},{E(1,3),E(3,1),E(4,2)},{E(1,1),E(3,3),E(4,2)},{E(1,2),E(3,1),E(4,3)},{E(1,3),E(3,2),E(4,1)}},
  /* b43 */ {{E(1,1),E(2,3),E(4,2)},{E(1,2),E(2,1),E(4,3)},{E(1,3),E(2,2),E(4,1)},{E(1,1),E(2,2),E(4,3)},{E(1,2),E(2,3),E(4,1)},{E(1,3),E(2,1),E(4,2)}},
  /* b44 */ {{E(1,1),E(2,2),E(3,3)},{E(1,2),E(2,3),E(3,1)},{E(1,3),E(2,1),E(3,2)},{E(1,1),E(2,3),E(3,2)},{E(1,2),E(2,1),E(3,3)},{E(1,3),E(2,2),E(3,1)}},
};
/* Determinant: 24 signed quadruple products, first 12 positive (cuh:535-544). */
struct Quad4 { unsigned char a, b, c, d; };
static const Quad4 kDet[24] = {
  {E(1,1),E(2,2),E(3,3),E(4,4)},{E(1,1),E(2,3),E(3,4),E(4,2)},{E(1,1),E(2,4),E(3,2),E(4,3)},
  {E(1,2),E(2,1),E(3,4),E(4,3)},{E(1,2),E(2,3),E(3,1),E(4,4)},{E(1,2),E(2,4),E(3,3),E(4,1)},
  {E(1,3),E(2,1),E(3,2),E(4,4)},{E(1,3),E(2,2),E(3,4),E(4,1)},{E(1,3),E(2,4),E(3,1),E(4,2)},
  {E(1,4),E(2,1),E(3,3),E(4,2)},{E(1,4),E(2,2),E(3,1),E(4,3)},{E(1,4),E(2,3),E(3,2),E(4,1)},
  {E(1,1),E(2,2),E(3,4),E(4,3)},{E(1,1),E(2,3),E(3,2),E(4,4)},{E(1,1),E(2,4),E(3,3),E(4,2)},
  {E(1,2),E(2,1),E(3,3),E(4,4)},{E(1,2),E(2,3),E(3,4),E(4,1)},{E(1,2),E(2,4),E(3,1),E(4,3)},
  {E(1,3),E(2,1),E(3,4),E(4,2)},{E(1,3),E(2,2),E(3,1),E(4,4)},{E(1,3),E(2,4),E(3,2),E(4,1)},
  {E(1,4),E(2,1),E(3,2),E(4,3)},{E(1,4),E(2,2),E(3,3),E(4,1)},{E(1,4),E(2,3),E(3,1),E(4,2)},
};
#undef E

/* Element 3D: returns the 10 upper-triangle entries coef*K + lambda*M in the order
 * (0,0),(0,1),(0,2),(0,3),(1,1),(1,2),(1,3),(2,2),(2,3),(3,3)
 * (perform_element_loop_3D.cuh:28-116,505-617). */
void element3d(const double x[4], const double y[4], const double z[4], double co,
               double lambda, const double integrand[10], double out[10]) {
  double a1 = x[1] - x[3], a2 = y[1] - y[3], a3 = z[1] - z[3];
  double b1 = x[2] - x[3], b2 = y[2] - y[3], b3 = z[2] - z[3];
  double c1 = x[0] - x[3], c2 = y[0] - y[3], c3 = z[0] - z[3];
  double Tvol = fabs(c1 * (a2 * b3 - a3 * b2) + c2 * (a3 * b1 - a1 * b3) + c3 * (a1 * b2 - a2 * b1)) / 6.0;
  double m[16];
  for (int r = 0; r < 4; r++) {
    m[r * 4 + 0] = x[r];
    m[r * 4 + 1] = y[r];
    m[r * 4 + 2] = z[r];
    m[r * 4 + 3] = 1.0;
  }
  double det = 0.0;
  for (int t = 0; t < 24; t++) {
    double p = m[kDet[t].a] * m[kDet[t].b] * m[kDet[t].c] * m[kDet[t].d];
    det = (t == 0) ? p : (t < 12 ? det + p : det - p);
  }
  double cof[16];
  for (int q = 0; q < 16; q++) {
    const Tri3* T = kCof[q];
    double s = m[T[0].a] * m[T[0].b] * m[T[0].c];
    s = s + m[T[1].a] * m[T[1].b] * m[T[1].c];
    s = s + m[T[2].a] * m[T[2].b] * m[T[2].c];
    s = s - m[T[3].a] * m[T[3].b] * m[T[3].c];
    s = s - m[T[4].a] * m[T[4].b] * m[T[4].c];
    s = s - m[T[5].a] * m[T[5].b] * m[T[5].c];
    cof[q] = s; /* cof[(r-1)*4+(c-1)] = b_rc */
  }
  /* coeffs[4k+m] = b_{m+1,k+1} / det: gradient of basis k is coeffs[4k+0..2]. */
  double g[4][3];
  for (int k = 0; k < 4; k++)
    for (int mm = 0; mm < 3; mm++) g[k][mm] = cof[mm * 4 + k] / det;
  /* mass Jacobian (cuh:88-96) */
  double x1 = x[0], y1 = y[0], z1 = z[0], x2 = x[1], y2 = y[1], z2 = z[1];
  double x3 = x[2], y3 = y[2], z3 = z[2], x4 = x[3], y4 = y[3], z4 = z[3];
  double mdet = 0.125 * ((-x1 + x2) * (-y1 + y3) * (-z1 + z4) + (-y1 + y2) * (-z1 + z3) * (-x1 + x4) +
                         (-z1 + z2) * (-x1 + x3) * (-y1 + y4) - (-x1 + x2) * (-z1 + z3) * (-y1 + y4) -
                         (-z1 + z2) * (-y1 + y3) * (-x1 + x4) - (-y1 + y2) * (-x1 + x3) * (-z1 + z4));
  double jac = fabs(mdet);
  int cnt = 0;
  for (int k = 0; k < 4; k++)
    for (int q = k; q < 4; q++) {
      double st = (g[k][0] * g[q][0] + g[k][1] * g[q][1] + g[k][2] * g[q][2]) * Tvol * co;
      double ms = integrand[cnt] * jac;
      out[cnt] = st + lambda * ms;
      cnt++;
    }
}

/* Element 3D in the library's fused multiply-add formulation (fem_assembly.cu
 * tet_gradients / element3d_kernel, restated operation for operation): edge vectors
 * a = p1 - p0, b = p2 - p0, c = p3 - p0, det = a . (b x c), grad l1..3 = (b x c, c x a,
 * a x b) / det, grad l0 = -((grad l1 + grad l2) + grad l3), K_ab = (|det| / 6) co grad
 * l_a . grad l_b, mass integrand * |det| / 8.  It agrees with element3d (the
 * reference's cofactor inverse) to a few units in the last place. */
static void cross_fma(const double u[3], const double v[3], double w[3]) {
  w[0] = std::fma(u[1], v[2], -(u[2] * v[1]));
  w[1] = std::fma(u[2], v[0], -(u[0] * v[2]));
  w[2] = std::fma(u[0], v[1], -(u[1] * v[0]));
}

void element3d_fma(const double x[4], const double y[4], const double z[4], double co, double lambda,
                   const double integrand[10], double out[10]) {
  double p[4][3];
  for (int q = 0; q < 4; q++) {
    p[q][0] = x[q];
    p[q][1] = y[q];
    p[q][2] = z[q];
  }
  double a[3], b[3], c[3], bc[3], ca[3], ab[3], g[4][3];
  for (int d = 0; d < 3; d++) {
    a[d] = p[1][d] - p[0][d];
    b[d] = p[2][d] - p[0][d];
    c[d] = p[3][d] - p[0][d];
  }
  cross_fma(b, c, bc);
  cross_fma(c, a, ca);
  cross_fma(a, b, ab);
  const double det = std::fma(a[0], bc[0], std::fma(a[1], bc[1], a[2] * bc[2]));
  const double inv = 1.0 / det;
  for (int d = 0; d < 3; d++) {
    g[1][d] = bc[d] * inv;
    g[2][d] = ca[d] * inv;
    g[3][d] = ab[d] * inv;
    g[0][d] = -((g[1][d] + g[2][d]) + g[3][d]);
  }
  const double wk = (fabs(det) / 6.0) * co;
  const double jac = fabs(det) * 0.125;
  int cnt = 0;
  for (int k = 0; k < 4; k++)
    for (int q = k; q < 4; q++) {
      const double st = std::fma(g[k][0], g[q][0], std::fma(g[k][1], g[q][1], g[k][2] * g[q][2])) * wk;
      out[cnt] = std::fma(lambda, integrand[cnt] * jac, st);
      cnt++;
    }
}

/* Element 2D (perform_element_loop_2D.cuh:29-147,287-372): 6 upper entries
 * (0,0),(0,1),(0,2),(1,1),(1,2),(2,2). */
void element2d(const double x[3], const double y[3], double co, double lambda, const double zx[6],
               const double wx[6], const double zy[6], const double wy[6], double out[6]) {
  double TArea = fabs(x[0] * y[2] - x[0] * y[1] + x[1] * y[0] - x[1] * y[2] + x[2] * y[1] - x[2] * y[0]) / 2.0;
  double a11 = x[0], a12 = y[0], a13 = 1.0, a21 = x[1], a22 = y[1], a23 = 1.0, a31 = x[2], a32 = y[2], a33 = 1.0;
  double det = a11 * a22 * a33 + a21 * a32 * a13 + a31 * a12 * a23 - a11 * a32 * a23 - a31 * a22 * a13 - a21 * a12 * a33;
  double b11 = a22 * a33 - a23 * a32, b12 = a13 * a32 - a12 * a33, b13 = a12 * a23 - a13 * a22;
  double b21 = a23 * a31 - a21 * a33, b22 = a11 * a33 - a13 * a31, b23 = a13 * a21 - a11 * a23;
  double b31 = a21 * a32 - a22 * a31, b32 = a12 * a31 - a11 * a32, b33 = a11 * a22 - a12 * a21;
  double cf[9] = {b11 / det, b21 / det, b31 / det, b12 / det, b22 / det, b32 / det, b13 / det, b23 / det, b33 / det};
  double px[6][6], py[6][6];
  for (int mm = 0; mm < 6; mm++)
    for (int j = 0; j < 6; j++) {
      px[mm][j] = x[0] * (1 - zx[mm]) * 0.5 * (1 - zy[j]) * 0.5 + x[1] * (1 + zx[mm]) * 0.5 * (1 - zy[j]) * 0.5 + x[2] * (1 + zy[j]) * 0.5;
      py[mm][j] = y[0] * (1 - zx[mm]) * 0.5 * (1 - zy[j]) * 0.5 + y[1] * (1 + zx[mm]) * 0.5 * (1 - zy[j]) * 0.5 + y[2] * (1 + zy[j]) * 0.5;
    }
  double jacobi = (x[0] * y[1] - x[1] * y[0] - x[0] * y[2] + x[2] * y[0] + x[1] * y[2] - x[2] * y[1]) / 8;
  int cnt = 0;
  for (int k = 0; k < 3; k++)
    for (int g = k; g < 3; g++) {
      double A1 = cf[3 * k], B1 = cf[3 * k + 1], C1 = cf[3 * k + 2];
      double A2 = cf[3 * g], B2 = cf[3 * g + 1], C2 = cf[3 * g + 2];
      double st = (A1 * A2 + B1 * B2) * TArea * co;
      double integral = 0;
      for (int i = 0; i < 6; i++) {
        double ty = 0.0;
        for (int j = 0; j < 6; j++) {
          double f = (A1 * px[i][j] + B1 * py[i][j] + C1) * (A2 * px[i][j] + B2 * py[i][j] + C2) * jacobi;
          ty += f * wy[j];
        }
        integral += ty * wx[i];
      }
      out[cnt++] = st + lambda * integral;
    }
}

/* co table of the device kernel (perform_element_loop_3D.cuh:585-612). */
double label_coefficient(int label) {
  static const double tab[7] = {1.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0};
  return (label >= 0 && label < 7) ? tab[label] : 1.0;
}

int64_t find_col(const int32_t* rowptr, const int32_t* cols, int r, int c) {
  int lo = rowptr[r], hi = rowptr[r + 1] - 1;
  while (lo <= hi) {
    int mid = lo + (hi - lo) / 2;
    if (cols[mid] < c) lo = mid + 1;
    else if (cols[mid] > c) hi = mid - 1;
    else return mid;
  }
  return -1;
}

/* ===================================================================== */
/* D. Sparse helpers                                                      */
/* ===================================================================== */
template <class T>
struct Csr {
  int n = 0, m = 0;
  std::vector<int32_t> rp, ci;
  std::vector<T> v;
  int64_t nnz() const { return (int64_t)ci.size(); }
};

/* ===================================================================== */
/* E. Randomized MIS + OldMIS aggregation                                 */
/* ===================================================================== */
inline uint32_t taus_step(uint32_t z) {
  uint32_t b = (((z << 13) ^ z) >> 19);
  return ((z & 0xFFFFFFFFu) << 12) ^ b;
}

const int kLoopCap = 100000;

/* misHelpers::randomizedMIS (randomizedMIS_GPU.cu:154-272) and its kernels (:3-152).
 * The reference seeds with srand(time(NULL)) on every call; a seed is passed here. */
int random_mis(int n, const int32_t* xadj, const int32_t* adj, int k, uint32_t seed, std::vector<int32_t>& mis) {
  mis.assign(n, -1);
  if (n == 0) return 0;
  std::vector<int32_t> seeds(32768);
  glibc_rand_seq(seed, 32768, seeds.data());
  std::vector<uint32_t> randoms(n);
  int iterations = (n + 32767) / 32768;
  for (int t = 0; t < 32768; t++) { /* Generate_Randoms_Kernel */
    uint32_t z = (uint32_t)seeds[t];
    int off = t;
    for (int i = 0; i < iterations; i++)
      if (off < n) {
        z = taus_step(z);
        randoms[off] = z;
        off += 32768;
      }
  }
  std::vector<int32_t> bsA(n), bsB(n), orA(n), orB(n);
  for (int i = 0; i < n; i++) { /* First_Initialize_Kernel */
    orA[i] = i;
    bsA[i] = (int32_t)(randoms[i] % 1000000u);
  }
  int rounds = 0;
  bool first = true;
  while (true) {
    if (!first) {
      for (int i = 0; i < n; i++) { /* Initialize_Kernel */
        uint32_t z = taus_step(randoms[i]);
        orA[i] = i;
        int v = (mis[i] == 1) ? 1000001 : 0;
        bsA[i] = (mis[i] == -1) ? (int32_t)(z % 1000000u) : v;
        randoms[i] = z;
      }
    }
    first = false;
    int32_t *bin = bsA.data(), *bout = bsB.data(), *oin = orA.data(), *oout = orB.data();
    bool incomplete = false;
    for (int it = 0; it < k; it++) { /* Iterate_Kernel x (k-1), Final_Iterate_Kernel */
      for (int i = 0; i < n; i++) {
        int best = bin[i], org = oin[i];
        if (best < 1000001) {
          for (int e = xadj[i]; e < xadj[i + 1]; e++) {
            int nb = adj[e];
            int ch = bin[nb], cho = oin[nb];
            if (ch > 0 && ch == best && cho > org) org = cho;
            if (ch > best) {
              best = ch;
              org = cho;
            }
          }
        }
        bout[i] = best;
        oout[i] = org;
        if (it == k - 1) {
          int st = -1;
          if (org == i) st = 1;
          else if (best == 1000001) st = 0;
          mis[i] = st;
          if (st == -1) incomplete = true;
        }
      }
      std::swap(bin, bout);
      std::swap(oin, oout);
    }
    /* the swapped buffers become the next round's inputs; Initialize overwrites them */
    if (bin != bsA.data()) {
      std::swap(bsA, bsB);
      std::swap(orA, orB);
    }
    if (!incomplete) break;
    if (++rounds > kLoopCap) return 6;
  }
  return 0;
}

/* allocateNodesKernel (misHelpers.cu:13-75), Jacobi over partIn -> partOut. */
void allocate_nodes(int n, const int32_t* xadj, const int32_t* adj, const std::vector<int32_t>& partIn,
                    std::vector<int32_t>& partOut, std::vector<int32_t>& aggregated) {
  for (int idx = 0; idx < n; idx++) {
    if (aggregated[idx] != 0) continue;
    int cand[10], cnt[10];
    for (int i = 0; i < 10; i++) {
      cand[i] = -1;
      cnt[i] = 0;
    }
    for (int e = xadj[idx]; e < xadj[idx + 1]; e++) {
      int c = partIn[adj[e]];
      if (c != -1) {
        for (int j = 0; j < 10 && c != -1; j++) {
          if (cand[j] == -1) {
            cand[j] = c;
            cnt[j] = 1;
          } else if (cand[j] == c) {
            cnt[j] += 1;
            c = -1;
          }
        }
      }
    }
    int addTo = cand[0], count = cnt[0];
    for (int i = 1; i < 10; i++)
      if (cnt[i] > count) {
        count = cnt[i];
        addTo = cand[i];
      }
    partOut[idx] = addTo;
    if (addTo != -1) aggregated[idx] = 1;
  }
}

/* removeRuntyParts (misHelpers.cu:744-781). Returns true when nothing was removed. */
bool remove_runty_parts(int minSize, std::vector<int32_t>& part) {
  int maxp = -1;
  for (int p : part) maxp = std::max(maxp, p);
  std::vector<int32_t> sizes(maxp + 1, 0);
  for (int p : part) sizes[p]++;
  std::vector<int32_t> rm(maxp + 1), sub(maxp + 1);
  int removed = 0, acc = 0;
  for (int p = 0; p <= maxp; p++) {
    rm[p] = sizes[p] < minSize ? 1 : 0;
    removed += rm[p];
    acc += rm[p];
    sub[p] = acc;
  }
  if (removed == 0) return true;
  for (auto& p : part) p = rm[p] ? -1 : p - sub[p];
  return false;
}

/* getWeightedPartSizes (misHelpers.cu:1109-1142). */
std::vector<int32_t> weighted_sizes(const std::vector<int32_t>& part, const std::vector<int32_t>& w) {
  int maxp = -1;
  for (int p : part) maxp = std::max(maxp, p);
  std::vector<int32_t> s(maxp + 1, 0);
  for (size_t i = 0; i < part.size(); i++) s[part[i]] += w[i];
  return s;
}

/* removeRuntyPartitions (misHelpers.cu:783-820). */
void remove_runty_partitions(int fullSize, std::vector<int32_t>& part, const std::vector<int32_t>& w) {
  std::vector<int32_t> sizes = weighted_sizes(part, w);
  double avg = (double)fullSize / sizes.size();
  int threshold = (int)(avg * .7);
  std::vector<int32_t> rm(sizes.size()), sub(sizes.size());
  int acc = 0;
  for (size_t p = 0; p < sizes.size(); p++) {
    rm[p] = sizes[p] < threshold ? 1 : 0;
    acc += rm[p];
    sub[p] = acc;
  }
  for (auto& p : part) p = rm[p] ? -1 : p - sub[p];
}

/* findDesirabilityKernel (misHelpers.cu:297-382): returns desirability, sets addTo. */
float desirability(int idx, int opt, const int32_t* xadj, const int32_t* adj, const std::vector<int32_t>& part,
                   const std::vector<int32_t>& sizes, const std::vector<int32_t>& w, int* addToOut) {
  int cur = part[idx];
  int cs = sizes[cur];
  int ns_ = w[idx];
  int selfAdj = 0, addTo = -1;
  float best = 0;
  float cwf = (float)abs(cs - opt) / (float)opt;
  float selfImp = (float)(abs(cs - opt) - abs((cs - ns_) - opt)) * cwf;
  if (selfImp > 0) {
    int cand[10], cnt[10];
    for (int i = 0; i < 10; i++) {
      cand[i] = -1;
      cnt[i] = 0;
    }
    for (int e = xadj[idx]; e < xadj[idx + 1]; e++) {
      int c = part[adj[e]];
      if (c == cur) selfAdj++;
      else
        for (int j = 0; j < 10; j++) {
          if (c != -1 && cand[j] == -1) {
            cand[j] = c;
            cnt[j] = 1;
            c = -1;
          } else if (cand[j] == c) {
            cnt[j] += 1;
            c = -1;
          }
        }
    }
    for (int i = 1; i < 10; i++) {
      if (cand[i] == -1) continue;
      int np = cand[i];
      int nsz = sizes[np];
      float nwf = (float)abs(nsz - opt) / (float)opt;
      float imp = (float)(abs(nsz - opt) - abs((nsz + ns_) - opt)) * nwf;
      imp = imp + selfImp;
      float ratio = (float)cnt[i] / (float)selfAdj;
      imp = imp * ratio;
      if (imp > best) {
        addTo = np;
        best = imp;
      }
    }
  }
  *addToOut = addTo;
  return best;
}

/* restrictPartitionSize (misHelpers.cu:679-727) with makeSwapsKernel (:384-412):
 * per source partition the node of largest (desirability, index) moves when its
 * desirability exceeds 0.1. */
int restrict_partition_size(int maxSize, int fullSize, const int32_t* xadj, const int32_t* adj,
                            std::vector<int32_t>& part, const std::vector<int32_t>& w) {
  int n = (int)part.size();
  std::vector<int32_t> sizes = weighted_sizes(part, w);
  int np = (int)sizes.size();
  int avg = fullSize / np;
  int largest = 0;
  for (int s : sizes) largest = std::max(largest, s);
  std::vector<float> des(n);
  std::vector<int32_t> to(n), bestNode(np);
  int loops = 0;
  while (largest > maxSize) {
    if (++loops > kLoopCap) return 6;
    for (int i = 0; i < n; i++) des[i] = desirability(i, avg, xadj, adj, part, sizes, w, &to[i]);
    std::fill(bestNode.begin(), bestNode.end(), -1);
    for (int i = 0; i < n; i++) {
      int p = part[i];
      int b = bestNode[p];
      if (b < 0 || des[i] >= des[b]) bestNode[p] = i; /* ties -> larger index (stable sort) */
    }
    std::vector<int32_t> oldpart = part;
    for (int p = 0; p < np; p++) {
      int i = bestNode[p];
      if (i < 0) continue;
      if ((double)des[i] > .1) {
        part[i] = to[i];
        sizes[to[i]] += w[i];
        sizes[oldpart[i]] -= w[i];
      }
    }
    largest = 0;
    for (int s : sizes) largest = std::max(largest, s);
  }
  return 0;
}

/* aggregateGraph (misHelpers.cu:513-601). */
int aggregate_graph(int minSize, int depth, int n, const int32_t* xadj, const int32_t* adj, uint32_t seed,
                    std::vector<int32_t>& partIn) {
  std::vector<int32_t> mis;
  int st = random_mis(n, xadj, adj, depth, seed, mis);
  if (st) return st;
  std::vector<int32_t> aggregated = mis;
  partIn.resize(n);
  int acc = 0;
  for (int i = 0; i < n; i++) {
    acc += mis[i];
    partIn[i] = aggregated[i] == 0 ? -1 : acc - 1;
  }
  std::vector<int32_t> partOut = partIn;
  int loops = 0;
  while (true) {
    if (++loops > kLoopCap) return 6;
    allocate_nodes(n, xadj, adj, partIn, partOut, aggregated);
    bool changed = partIn != partOut;
    partIn = partOut;
    int unalloc = 0;
    for (int a : aggregated) unalloc += (a == 0);
    if (unalloc == 0) {
      if (remove_runty_parts(minSize, partIn)) break;
      for (int i = 0; i < n; i++) aggregated[i] = partIn[i] == -1 ? 0 : 1;
      bool any = false;
      for (int p : partIn) any |= (p != -1);
      if (!any) return 6; /* every aggregate was a runt: the reference loops forever */
      partOut = partIn;
    } else if (!changed) {
      return 6; /* unreachable nodes: the reference loops forever */
    }
  }
  return 0;
}

/* aggregateWeightedGraph (misHelpers.cu:603-677). */
int aggregate_weighted_graph(int maxSize, int fullSize, int depth, int n, const int32_t* xadj, const int32_t* adj,
                             const std::vector<int32_t>& weights, uint32_t seed, std::vector<int32_t>& partIn) {
  std::vector<int32_t> mis;
  int st = random_mis(n, xadj, adj, depth, seed, mis);
  if (st) return st;
  std::vector<int32_t> aggregated = mis;
  partIn.resize(n);
  int acc = 0;
  for (int i = 0; i < n; i++) {
    acc += mis[i];
    partIn[i] = aggregated[i] == 0 ? -1 : acc - 1;
  }
  int misCount = acc;
  std::vector<int32_t> partOut = partIn;
  bool firstTime = true;
  int loops = 0;
  while (true) {
    if (++loops > kLoopCap) return 6;
    allocate_nodes(n, xadj, adj, partIn, partOut, aggregated);
    bool changed = partIn != partOut;
    partIn = partOut;
    int unalloc = 0;
    for (int a : aggregated) unalloc += (a == 0);
    if (unalloc == 0) {
      if (!firstTime || misCount < 10) {
        return restrict_partition_size(maxSize, fullSize, xadj, adj, partIn, weights);
      }
      firstTime = false;
      remove_runty_partitions(fullSize, partIn, weights);
      bool any = false;
      for (int i = 0; i < n; i++) {
        aggregated[i] = partIn[i] == -1 ? 0 : 1;
        any |= partIn[i] != -1;
      }
      if (!any) return 6;
      partOut = partIn;
    } else if (!changed) {
      return 6;
    }
  }
}

struct OldMisOut {
  std::vector<int32_t> perm, iperm, aggIdx, partIdx, partLabel, xadjOut, adjOut;
};

/* misHelpers::CP::OldMIS (ComputePermutationMethods.cu:22-151). */
int old_mis(int n, const int32_t* xadj, const int32_t* adj, int params, int partMax, uint32_t seed, OldMisOut& o) {
  int fineDepth = params % 100;
  int coarseDepth = (params / 100) % 100;
  int minAgg = (params / 10000) % 10;
  std::vector<int32_t> fine;
  int st = aggregate_graph(minAgg, fineDepth, n, xadj, adj, seed, fine);
  if (st) return st;
  /* sort_by_key(fineAggregateSort, permutation): stable by aggregate id */
  int nagg = 0;
  for (int a : fine) nagg = std::max(nagg, a + 1);
  std::vector<int32_t> cnt(nagg + 1, 0);
  for (int a : fine) cnt[a + 1]++;
  std::vector<int32_t> aggStart(nagg + 1, 0);
  for (int a = 0; a < nagg; a++) aggStart[a + 1] = aggStart[a] + cnt[a + 1];
  std::vector<int32_t> perm1(n), fill(aggStart.begin(), aggStart.end() - 1);
  for (int i = 0; i < n; i++) perm1[fill[fine[i]]++] = i;
  std::vector<int32_t> weights(nagg);
  for (int a = 0; a < nagg; a++) weights[a] = aggStart[a + 1] - aggStart[a];
  /* getInducedGraph (misHelpers.cu:1078-1107): sorted unique neighbour aggregates */
  std::vector<int32_t> ixadj(nagg + 1, 0), iadj;
  {
    std::vector<int32_t> tmp;
    for (int a = 0; a < nagg; a++) {
      tmp.clear();
      for (int q = aggStart[a]; q < aggStart[a + 1]; q++) {
        int i = perm1[q];
        for (int e = xadj[i]; e < xadj[i + 1]; e++) {
          int b = fine[adj[e]];
          if (b != a) tmp.push_back(b);
        }
      }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      iadj.insert(iadj.end(), tmp.begin(), tmp.end());
      ixadj[a + 1] = (int32_t)iadj.size();
    }
  }
  std::vector<int32_t> coarse;
  st = aggregate_weighted_graph(partMax, n, coarseDepth, nagg, ixadj.data(), iadj.data(), weights, seed, coarse);
  if (st) return st;
  int npart = 0;
  for (int p : coarse) npart = std::max(npart, p + 1);
  /* new aggregate ids: stable order by (partition, old id) -- remapInducedGraph
   * (misHelpers.cu:1258-1280) and the aggregate remap of OldMIS agree on it */
  std::vector<int32_t> pcnt(npart + 1, 0);
  for (int p : coarse) pcnt[p + 1]++;
  o.partIdx.assign(npart + 1, 0);
  for (int p = 0; p < npart; p++) o.partIdx[p + 1] = o.partIdx[p] + pcnt[p + 1];
  std::vector<int32_t> newId(nagg), oldOf(nagg), pf(o.partIdx.begin(), o.partIdx.end() - 1);
  for (int a = 0; a < nagg; a++) {
    int id = pf[coarse[a]]++;
    newId[a] = id;
    oldOf[id] = a;
  }
  o.xadjOut.assign(nagg + 1, 0);
  o.adjOut.clear();
  o.adjOut.reserve(iadj.size());
  for (int id = 0; id < nagg; id++) {
    int a = oldOf[id];
    for (int e = ixadj[a]; e < ixadj[a + 1]; e++) o.adjOut.push_back(newId[iadj[e]]);
    o.xadjOut[id + 1] = (int32_t)o.adjOut.size();
  }
  /* node order: (partition, old aggregate id, node id) == new aggregate id order */
  o.aggIdx.assign(nagg + 1, 0);
  o.iperm.resize(n);
  o.perm.resize(n);
  o.partLabel.resize(n);
  int pos = 0;
  for (int id = 0; id < nagg; id++) {
    int a = oldOf[id];
    for (int q = aggStart[a]; q < aggStart[a + 1]; q++) {
      o.iperm[pos] = perm1[q];
      o.partLabel[pos] = coarse[a];
      pos++;
    }
    o.aggIdx[id + 1] = pos;
  }
  for (int i = 0; i < n; i++) o.perm[o.iperm[i]] = i;
  return 0;
}

/* ===================================================================== */
/* F. Hierarchy                                                           */
/* ===================================================================== */
struct LevelBase {
  virtual ~LevelBase() {}
};

int lanes_for_rows(int64_t nnz, int n);

template <class T>
struct Level {
  int n = 0;
  int smooth_lanes = 1; /* lanes per row of the in-partition sums (device layout rule) */
  Csr<T> A;          /* level matrix, level's own numbering */
  bool coarsest = false;
  /* aggregation (non-coarsest) */
  std::vector<int32_t> perm, iperm, aggIdx, partIdx, partLabel, aggOf;
  std::vector<int32_t> gxadj, gadj; /* this level's graph */
  Csr<T> Ap;         /* permuted matrix */
  std::vector<T> diag, dinv;
  Csr<T> Ain, Aout;  /* in-partition off-diagonal (upper values mirrored), cross-partition */
  Csr<T> P, R;
  /* coarsest: dense factor */
  std::vector<double> F;
  std::vector<int32_t> piv;
  bool chol = true;
  /* work vectors */
  std::vector<T> b, x, r, bc, xc, xo;
  /* mixed precision: the FP64 values of A when its Galerkin product was formed in FP64 */
  std::vector<double> A64v;
};

/* Mixed precision forms the Galerkin products whose result has at most
 * kFp64GalerkinPerTop x top_size rows in FP64: the FP32 operands are widened exactly, the
 * products and sums run in double in the usual generation order, and the result is rounded
 * to FP32 for the level (its FP64 values feed the coarsest dense factorisation).  At the
 * benchmark configurations these are the two coarsest levels' products. */
constexpr int kFp64GalerkinPerTop = 32;

template <class T>
Csr<double> widen(const Csr<T>& A) {
  Csr<double> B;
  B.n = A.n;
  B.m = A.m;
  B.rp = A.rp;
  B.ci = A.ci;
  B.v.assign(A.v.begin(), A.v.end());
  return B;
}

template <class T>
Csr<T> permute(const Csr<T>& A, const std::vector<int32_t>& perm, const std::vector<int32_t>& iperm) {
  Csr<T> B;
  B.n = A.n;
  B.m = A.m;
  B.rp.assign(A.n + 1, 0);
  for (int i = 0; i < A.n; i++) B.rp[i + 1] = B.rp[i] + (A.rp[iperm[i] + 1] - A.rp[iperm[i]]);
  B.ci.resize(A.nnz());
  B.v.resize(A.nnz());
#pragma omp parallel for schedule(static)
  for (int i = 0; i < A.n; i++) {
    int o = iperm[i];
    std::vector<std::pair<int32_t, T>> row;
    for (int e = A.rp[o]; e < A.rp[o + 1]; e++) row.push_back({perm[A.ci[e]], A.v[e]});
    std::sort(row.begin(), row.end(), [](const std::pair<int32_t, T>& a, const std::pair<int32_t, T>& b) { return a.first < b.first; });
    for (size_t q = 0; q < row.size(); q++) {
      B.ci[B.rp[i] + q] = row[q].first;
      B.v[B.rp[i] + q] = row[q].second;
    }
  }
  return B;
}

template <class T>
Csr<T> transpose(const Csr<T>& P) {
  Csr<T> R;
  R.n = P.m;
  R.m = P.n;
  R.rp.assign(P.m + 1, 0);
  for (int32_t c : P.ci) R.rp[c + 1]++;
  for (int k = 0; k < P.m; k++) R.rp[k + 1] += R.rp[k];
  R.ci.resize(P.nnz());
  R.v.resize(P.nnz());
  std::vector<int32_t> f(R.rp.begin(), R.rp.end() - 1);
  for (int i = 0; i < P.n; i++)
    for (int e = P.rp[i]; e < P.rp[i + 1]; e++) {
      int q = f[P.ci[e]]++;
      R.ci[q] = i;
      R.v[q] = P.v[e];
    }
  return R;
}

/* Expand-sort-compress SpGEMM C = A*B: products of row i in generation order
 * (A entries ascending, then B row entries ascending), grouped stably by column,
 * each group summed left to right starting from its first product.  This is the
 * fixed-order reading of the CUSP multiply used by generateNextLevelMatrixFull_d
 * (smoothedMG_amg_level.cu:390-400). */
template <class T>
Csr<T> spgemm(const Csr<T>& A, const Csr<T>& B) {
  Csr<T> C;
  C.n = A.n;
  C.m = B.m;
  std::vector<std::vector<int32_t>> cols(A.n);
  std::vector<std::vector<T>> vals(A.n);
#pragma omp parallel
  {
    std::vector<std::pair<int32_t, int32_t>> key;
    std::vector<T> pv;
#pragma omp for schedule(dynamic, 256)
    for (int i = 0; i < A.n; i++) {
      key.clear();
      pv.clear();
      for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
        T a = A.v[e];
        int j = A.ci[e];
        for (int f = B.rp[j]; f < B.rp[j + 1]; f++) {
          key.push_back({B.ci[f], (int32_t)pv.size()});
          pv.push_back(a * B.v[f]);
        }
      }
      std::sort(key.begin(), key.end());
      for (size_t q = 0; q < key.size();) {
        size_t r = q;
        T s = pv[key[q].second];
        while (++r < key.size() && key[r].first == key[q].first) s = s + pv[key[r].second];
        cols[i].push_back(key[q].first);
        vals[i].push_back(s);
        q = r;
      }
    }
  }
  C.rp.assign(A.n + 1, 0);
  for (int i = 0; i < A.n; i++) C.rp[i + 1] = C.rp[i] + (int32_t)cols[i].size();
  C.ci.resize(C.rp[A.n]);
  C.v.resize(C.rp[A.n]);
  for (int i = 0; i < A.n; i++) {
    std::copy(cols[i].begin(), cols[i].end(), C.ci.begin() + C.rp[i]);
    std::copy(vals[i].begin(), vals[i].end(), C.v.begin() + C.rp[i]);
  }
  return C;
}

/* generateProlongatorFull_d (smoothedMG_amg_level.cu:321-387):
 * P = T - omega D^-1 A T with per-entry value ((-omega) * a_ij) / d_i, the (i,k)
 * group summed in ascending j order and the tentative 1 added last. */
template <class T>
Csr<T> build_prolongator(const Csr<T>& Ap, const std::vector<T>& diag, const std::vector<int32_t>& aggOf, int nagg,
                         double omega) {
  Csr<T> P;
  P.n = Ap.n;
  P.m = nagg;
  std::vector<std::vector<int32_t>> cols(Ap.n);
  std::vector<std::vector<T>> vals(Ap.n);
  const T lam = -(T)omega;
#pragma omp parallel
  {
    std::vector<std::pair<int32_t, int32_t>> key;
    std::vector<T> pv;
#pragma omp for schedule(static)
    for (int i = 0; i < Ap.n; i++) {
      key.clear();
      pv.clear();
      for (int e = Ap.rp[i]; e < Ap.rp[i + 1]; e++) {
        T t = (lam * Ap.v[e]) * (T)1;
        key.push_back({aggOf[Ap.ci[e]], (int32_t)pv.size()});
        pv.push_back(t / diag[i]);
      }
      key.push_back({aggOf[i], (int32_t)pv.size()});
      pv.push_back((T)1);
      std::sort(key.begin(), key.end());
      for (size_t q = 0; q < key.size();) {
        size_t r = q;
        T s = pv[key[q].second];
        while (++r < key.size() && key[r].first == key[q].first) s = s + pv[key[r].second];
        cols[i].push_back(key[q].first);
        vals[i].push_back(s);
        q = r;
      }
    }
  }
  P.rp.assign(Ap.n + 1, 0);
  for (int i = 0; i < Ap.n; i++) P.rp[i + 1] = P.rp[i] + (int32_t)cols[i].size();
  P.ci.resize(P.rp[Ap.n]);
  P.v.resize(P.rp[Ap.n]);
  for (int i = 0; i < Ap.n; i++) {
    std::copy(cols[i].begin(), cols[i].end(), P.ci.begin() + P.rp[i]);
    std::copy(vals[i].begin(), vals[i].end(), P.v.begin() + P.rp[i]);
  }
  return P;
}

/* generateMatrixSymmetric_d (smoothedMG_amg_level.cu:200-304): the smoother reads
 * the strictly-upper in-partition entries for both (i,j) and (j,i), and every
 * cross-partition entry as stored.  Ain here holds both triangles with the upper
 * value, Aout the cross entries, both in ascending column order. */
template <class T>
void split_partitions(Level<T>& L) {
  const Csr<T>& A = L.Ap;
  int n = A.n;
  L.Ain.n = L.Aout.n = n;
  L.Ain.m = L.Aout.m = n;
  L.Ain.rp.assign(n + 1, 0);
  L.Aout.rp.assign(n + 1, 0);
  for (int i = 0; i < n; i++) {
    int pi = L.partLabel[i];
    int ci = 0, co = 0;
    for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
      int j = A.ci[e];
      if (j == i) continue;
      if (L.partLabel[j] == pi) ci++;
      else co++;
    }
    L.Ain.rp[i + 1] = L.Ain.rp[i] + ci;
    L.Aout.rp[i + 1] = L.Aout.rp[i] + co;
  }
  L.Ain.ci.resize(L.Ain.rp[n]);
  L.Ain.v.resize(L.Ain.rp[n]);
  L.Aout.ci.resize(L.Aout.rp[n]);
  L.Aout.v.resize(L.Aout.rp[n]);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    int pi = L.partLabel[i];
    int qi = L.Ain.rp[i], qo = L.Aout.rp[i];
    for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
      int j = A.ci[e];
      if (j == i) continue;
      if (L.partLabel[j] == pi) {
        T v = A.v[e];
        if (j < i) { /* mirror the upper entry (j,i) */
          int64_t u = find_col(A.rp.data(), A.ci.data(), j, i);
          v = u >= 0 ? A.v[u] : (T)0;
        }
        L.Ain.ci[qi] = j;
        L.Ain.v[qi] = v;
        qi++;
      } else {
        L.Aout.ci[qo] = j;
        L.Aout.v[qo] = A.v[e];
        qo++;
      }
    }
  }
}

/* Dense LU with partial pivoting in FP64 (coarsest level). */
int dense_factor(int n, std::vector<double>& F, std::vector<int32_t>& piv) {
  piv.resize(n);
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = fabs(F[(size_t)k * n + k]);
    for (int i = k + 1; i < n; i++)
      if (fabs(F[(size_t)i * n + k]) > best) {
        best = fabs(F[(size_t)i * n + k]);
        p = i;
      }
    piv[k] = p;
    if (best == 0.0) return 4;
    if (p != k)
      for (int j = 0; j < n; j++) std::swap(F[(size_t)k * n + j], F[(size_t)p * n + j]);
    double d = F[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      double l = F[(size_t)i * n + k] / d;
      F[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; j++) F[(size_t)i * n + j] = fma(-l, F[(size_t)k * n + j], F[(size_t)i * n + j]);
    }
  }
  return 0;
}

void dense_solve(int n, const std::vector<double>& F, const std::vector<int32_t>& piv, std::vector<double>& b) {
  for (int k = 0; k < n; k++) std::swap(b[k], b[piv[k]]);
  for (int i = 0; i < n; i++) {
    double s = b[i];
    for (int j = 0; j < i; j++) s = fma(-F[(size_t)i * n + j], b[j], s);
    b[i] = s;
  }
  /* back substitution column by column (the device's order): row i takes the
   * updates of columns n-1, n-2, ..., i+1, then the division */
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int j = n - 1; j > i; j--) s = fma(-F[(size_t)i * n + j], b[j], s);
    b[i] = s / F[(size_t)i * n + i];
  }
}

}  // namespace

/* ===================================================================== */
/* AMG object                                                             */
/* ===================================================================== */
struct orc_amg {
  orc_config cfg;
  int n0 = 0;
  Csr<double> A0p; /* FP64 level-0 matrix in level-0 permuted order (outer PCG) */
  std::vector<int32_t> perm0, iperm0;
  std::vector<Level<float>> Lf;
  std::vector<Level<double>> Ld;
  int nlev() const { return cfg.fp64_hierarchy ? (int)Ld.size() : (int)Lf.size(); }
};

namespace {

template <class T>
int setup_levels(orc_amg* h, std::vector<Level<T>>& L, const Csr<double>& A, const int32_t* gx, const int32_t* ga) {
  const orc_config& c = h->cfg;
  Level<T> L0;
  L0.n = A.n;
  L0.A.n = A.n;
  L0.A.m = A.m;
  L0.A.rp = A.rp;
  L0.A.ci = A.ci;
  L0.A.v.resize(A.v.size());
  for (size_t i = 0; i < A.v.size(); i++) L0.A.v[i] = (T)A.v[i];
  L0.gxadj.assign(gx, gx + A.n + 1);
  L0.gadj.assign(ga, ga + gx[A.n]);
  L.push_back(std::move(L0));
  int num_levels = 1;
  while (true) {
    Level<T>& lv = L.back();
    int N = lv.A.n;
    if (N < c.top_size || num_levels >= c.max_levels) { /* amg.cu:99-108 */
      lv.coarsest = true;
      lv.F.assign((size_t)N * N, 0.0);
      for (int i = 0; i < N; i++)
        for (int e = lv.A.rp[i]; e < lv.A.rp[i + 1]; e++)
          lv.F[(size_t)i * N + lv.A.ci[e]] = lv.A64v.empty() ? (double)lv.A.v[e] : lv.A64v[e];
      int st = dense_factor(N, lv.F, lv.piv);
      if (st) return st;
      /* explicit inverse, column j = LU solve of e_j; the coarse solve is then x = inv b */
      std::vector<double> inv((size_t)N * N), col(N);
      for (int j = 0; j < N; j++) {
        for (int i = 0; i < N; i++) col[i] = (i == j) ? 1.0 : 0.0;
        dense_solve(N, lv.F, lv.piv, col);
        for (int i = 0; i < N; i++) inv[(size_t)i * N + j] = col[i];
      }
      lv.F.swap(inv);
      lv.x.resize(N);
      break;
    }
    OldMisOut o;
    int st = old_mis(N, lv.gxadj.data(), lv.gadj.data(), c.rand_mis_params, c.partition_max, c.seed, o);
    if (st) return st;
    lv.perm = o.perm;
    lv.iperm = o.iperm;
    lv.aggIdx = o.aggIdx;
    lv.partIdx = o.partIdx;
    lv.partLabel = o.partLabel;
    int nagg = (int)o.aggIdx.size() - 1;
    lv.aggOf.resize(N);
    for (int a = 0; a < nagg; a++)
      for (int q = o.aggIdx[a]; q < o.aggIdx[a + 1]; q++) lv.aggOf[q] = a;
    lv.Ap = permute(lv.A, lv.perm, lv.iperm);
    lv.diag.assign(N, (T)0);
    for (int i = 0; i < N; i++) {
      int64_t d = find_col(lv.Ap.rp.data(), lv.Ap.ci.data(), i, i);
      lv.diag[i] = d >= 0 ? lv.Ap.v[d] : (T)0;
    }
    lv.dinv.resize(N);
    for (int i = 0; i < N; i++) lv.dinv[i] = (T)1 / lv.diag[i];
    split_partitions(lv);
    {
      /* the device keeps rows of <= 16 in-partition entries in registers (one lane per
       * row) when partitions have <= 512 rows, else sums rows with S lanes */
      int max_row = 0, max_part = 0;
      for (int i = 0; i < N; i++) max_row = std::max(max_row, lv.Ain.rp[i + 1] - lv.Ain.rp[i]);
      for (size_t q = 0; q + 1 < lv.partIdx.size(); q++)
        max_part = std::max(max_part, lv.aggIdx[lv.partIdx[q + 1]] - lv.aggIdx[lv.partIdx[q]]);
      /* S lanes per row: doubled while every lane still adds >= 3 entries of an average
       * row (ceil(in-partition nnz / N)) and N x lanes stays within 152 x 2048 */
      const int64_t in_nnz = lv.Ain.rp[N];
      const int64_t avg = N > 0 ? (in_nnz + N - 1) / N : 0;
      int sl = 1;
      while (sl < 32 && 3 * (2 * sl) <= avg && (int64_t)N * (2 * sl) <= 152LL * 2048) sl <<= 1;
      /* then while the longest row leaves a lane more than 16 entries */
      while (sl < 32 && (max_row + sl - 1) / sl > 16) sl <<= 1;
      lv.smooth_lanes = (max_row <= 16 && max_part <= 512) ? 1 : sl;
    }
    lv.P = build_prolongator(lv.Ap, lv.diag, lv.aggOf, nagg, c.pro_omega);
    lv.R = transpose(lv.P);
    Level<T> nx;
    if (sizeof(T) == 4 && nagg <= kFp64GalerkinPerTop * c.top_size) {
      const Csr<double> AP64 = spgemm(widen(lv.Ap), widen(lv.P));
      Csr<double> A64 = spgemm(widen(lv.R), AP64);
      nx.A.n = A64.n;
      nx.A.m = A64.m;
      nx.A.rp = A64.rp;
      nx.A.ci = A64.ci;
      nx.A.v.resize(A64.v.size());
      for (size_t q = 0; q < A64.v.size(); q++) nx.A.v[q] = (T)A64.v[q];
      nx.A64v.swap(A64.v);
    } else {
      Csr<T> AP = spgemm(lv.Ap, lv.P);
      nx.A = spgemm(lv.R, AP);
    }
    nx.n = nagg;
    nx.gxadj = o.xadjOut;
    nx.gadj = o.adjOut;
    lv.b.resize(N);
    lv.x.resize(N);
    lv.r.resize(N);
    lv.xo.resize(N);
    lv.bc.resize(nagg);
    lv.xc.resize(nagg);
    L.push_back(std::move(nx));
    num_levels++;
  }
  return 0;
}

/* gauss_seidel in-partition sweep update x += w (b - sAx - d x) / d
 * (gauss_seidel.cu:1333-1341), evaluated in T with the precomputed reciprocal of
 * the diagonal.  (The reference forms it in double because its weight is a double;
 * the device does the same T arithmetic as here.) */
template <class T>
inline T relax_update(T x, T b, T sAx, T d, T dinv, T w) {
  T t = b - sAx;
  t = t - d * x;
  return x + (w * t) * dinv;
}

/* Row sum of in-partition entries in the device's lane order: S lanes, lane j takes
 * entries j, j+S, ... with fused multiply-adds, then an xor butterfly. */
template <class T>
inline T part_row_sum(const Csr<T>& M, int i, const T* x, int xoff, int S) {
  T p[32], q[32];
  for (int j = 0; j < S; j++) p[j] = 0;
  for (int e = M.rp[i]; e < M.rp[i + 1]; e++) {
    int j = (e - M.rp[i]) % S;
    p[j] = std::fma(M.v[e], x[M.ci[e] - xoff], p[j]);
  }
  for (int off = S >> 1; off > 0; off >>= 1) {
    for (int j = 0; j < S; j++) q[j] = p[j] + p[j ^ off];
    for (int j = 0; j < S; j++) p[j] = q[j];
  }
  return p[0];
}

template <class T>
void pre_smooth(Level<T>& L, const orc_config& c) {
  int np = (int)L.partIdx.size() - 1;
  const T w = (T)c.smoother_weight;
#pragma omp parallel
  {
    std::vector<T> sAx;
#pragma omp for schedule(dynamic, 1)
    for (int p = 0; p < np; p++) {
      int rs = L.aggIdx[L.partIdx[p]], re = L.aggIdx[L.partIdx[p + 1]];
      sAx.assign(re - rs, (T)0);
      for (int i = rs; i < re; i++) L.x[i] = (w * L.b[i]) * L.dinv[i];
      for (int it = 0; it < c.pre_inner; it++) {
        for (int i = rs; i < re; i++) sAx[i - rs] = part_row_sum(L.Ain, i, L.x.data(), 0, L.smooth_lanes);
        for (int i = rs; i < re; i++) L.x[i] = relax_update(L.x[i], L.b[i], sAx[i - rs], L.diag[i], L.dinv[i], w);
      }
      for (int i = rs; i < re; i++) {
        T s = part_row_sum(L.Ain, i, L.x.data(), 0, L.smooth_lanes);
        T t = L.b[i] - s;
        L.r[i] = t - L.diag[i] * L.x[i];
      }
    }
    /* preAout_kernel (gauss_seidel.cu:1977-2015) */
#pragma omp for schedule(static)
    for (int i = 0; i < L.n; i++) {
      T s = 0;
      for (int e = L.Aout.rp[i]; e < L.Aout.rp[i + 1]; e++) s = s + L.Aout.v[e] * L.x[L.Aout.ci[e]];
      L.r[i] = L.r[i] - s;
    }
  }
}

template <class T>
void post_smooth(Level<T>& L, const orc_config& c) {
  int np = (int)L.partIdx.size() - 1;
  const T w = (T)c.smoother_weight;
  for (int rl = 0; rl < c.post_relaxes; rl++) {
#pragma omp parallel
    {
      std::vector<T> sb, sx, sAx;
#pragma omp for schedule(dynamic, 1)
      for (int p = 0; p < np; p++) {
        int rs = L.aggIdx[L.partIdx[p]], re = L.aggIdx[L.partIdx[p + 1]];
        int m = re - rs;
        sb.resize(m);
        sx.resize(m);
        sAx.resize(m);
        for (int i = rs; i < re; i++) {
          T s = L.b[i];
          for (int e = L.Aout.rp[i]; e < L.Aout.rp[i + 1]; e++) s = s + (-L.Aout.v[e]) * L.x[L.Aout.ci[e]];
          sb[i - rs] = s;
          sx[i - rs] = L.x[i];
        }
        for (int it = 0; it < c.post_inner; it++) {
          for (int i = rs; i < re; i++) sAx[i - rs] = part_row_sum(L.Ain, i, sx.data(), rs, L.smooth_lanes);
          for (int i = rs; i < re; i++) sx[i - rs] = relax_update(sx[i - rs], sb[i - rs], sAx[i - rs], L.diag[i], L.dinv[i], w);
        }
        for (int i = rs; i < re; i++) L.xo[i] = sx[i - rs];
      }
    }
    std::swap(L.x, L.xo);
  }
}

/* Row products of the transfer operators in the device's lane order: S lanes per row
 * (S from the average row length), lane j sums entries j, j+S, ... in order, then
 * an xor butterfly (p_j + p_{j^off}, off = S/2 .. 1) combines them; lane 0's value is
 * the result.  The reference's CUSP SpMV order is unpinned. */
int lanes_for_rows(int64_t nnz, int n) {
  double avg = n > 0 ? (double)nnz / n : 0.0;
  int s = 1;
  while (s < 32 && s * 4 < avg) s <<= 1;
  return s;
}

template <class T>
void spmv_rows(const Csr<T>& A, const std::vector<T>& x, std::vector<T>& y) {
  const int S = lanes_for_rows(A.nnz(), A.n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < A.n; i++) {
    T p[32], q[32];
    for (int j = 0; j < S; j++) p[j] = 0;
    for (int e = A.rp[i]; e < A.rp[i + 1]; e++) {
      int j = (e - A.rp[i]) % S;
      p[j] = p[j] + A.v[e] * x[A.ci[e]];
    }
    for (int off = S >> 1; off > 0; off >>= 1) {
      for (int j = 0; j < S; j++) q[j] = p[j] + p[j ^ off];
      for (int j = 0; j < S; j++) p[j] = q[j];
    }
    y[i] = p[0];
  }
}

/* l1-Jacobi (smoother 1, the library's performance option): x += w (b - Ap x) / l1 with
 * l1_i = sum_j |a_ij| in entry order; row sums with fused multiply-adds in entry order. */
template <class T>
T ap_row_sum(const Csr<T>& A, int i, const std::vector<T>& x) {
  T s = 0;
  for (int e = A.rp[i]; e < A.rp[i + 1]; e++) s = std::fma(A.v[e], x[A.ci[e]], s);
  return s;
}

template <class T>
void l1_sweeps(Level<T>& L, const orc_config& c, int sweeps) {
  const T w = (T)c.smoother_weight;
  std::vector<T> l1inv(L.n), xn(L.n);
  for (int i = 0; i < L.n; i++) {
    T s = 0;
    for (int e = L.Ap.rp[i]; e < L.Ap.rp[i + 1]; e++) s = s + std::fabs(L.Ap.v[e]);
    l1inv[i] = (T)1 / s;
  }
  for (int it = 0; it < sweeps; it++) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < L.n; i++) xn[i] = L.x[i] + (w * (L.b[i] - ap_row_sum(L.Ap, i, L.x))) * l1inv[i];
    L.x.swap(xn);
  }
}

/* Coarse visits of a cycle of type `type` (0 V, 1 W, 2 F) at a non-coarsest level: the
 * first visit has type V for a V-cycle and W otherwise; W- and F-cycles visit a
 * non-coarsest next level a second time (W: a W-cycle, F: a V-cycle), as the reference's
 * W_Cycle / F_Cycle classes do (cycles/wcycle.h, cycles/fcycle.h; AMG_Level::cycle,
 * amg_level.cu:51, never reaches them).  The second visit corrects the first:
 * xc += cycle(bc - A_c xc), the residual formed row by row in the permuted coarse
 * operator's entry order with separately rounded products, as the device does. */
inline int first_visit(int type) { return type == 0 ? 0 : 1; }
inline int second_visit(int type) { return type == 1 ? 1 : 0; }

template <class T>
void vcycle(std::vector<Level<T>>& L, int l, const orc_config& c, int type = 0);

template <class T>
void coarse_visits(std::vector<Level<T>>& L, int l, const orc_config& c, int type) {
  Level<T>& lv = L[l];
  Level<T>& nx = L[l + 1];
  nx.b = lv.bc;
  vcycle(L, l + 1, c, first_visit(type));
  lv.xc = nx.x;
  if (type == 0 || nx.coarsest) return;
  const int N = nx.n;
  std::vector<T> bp(N), xp(N), rc(N);
  for (int i = 0; i < N; i++) {
    bp[i] = lv.bc[nx.iperm[i]];
    xp[i] = lv.xc[nx.iperm[i]];
  }
  for (int i = 0; i < N; i++) {
    T s = bp[i];
    for (int e = nx.Ap.rp[i]; e < nx.Ap.rp[i + 1]; e++) s = s - nx.Ap.v[e] * xp[nx.Ap.ci[e]];
    rc[nx.iperm[i]] = s;
  }
  nx.b = rc;
  vcycle(L, l + 1, c, second_visit(type));
  for (int i = 0; i < N; i++) lv.xc[i] = lv.xc[i] + nx.x[i];
}

/* AMG_Level::cycle (amg_level.cu:22-71).  Input L[l].b in the level's own order for
 * l > 0 (permuted in, as permutation_kernel1), already permuted for l == 0. */
template <class T>
void vcycle(std::vector<Level<T>>& L, int l, const orc_config& c, int type) {
  Level<T>& lv = L[l];
  if (lv.coarsest) { /* lv.F holds the explicit inverse */
    const int N = lv.A.n;
    for (int i = 0; i < N; i++) { /* the device's warp-per-row order: 32 fma lanes, butterfly */
      double p[32], q[32];
      for (int j = 0; j < 32; j++) p[j] = 0.0;
      for (int j = 0; j < N; j++) p[j & 31] = fma(lv.F[(size_t)i * N + j], (double)lv.b[j], p[j & 31]);
      for (int off = 16; off > 0; off >>= 1) {
        for (int j = 0; j < 32; j++) q[j] = p[j] + p[j ^ off];
        for (int j = 0; j < 32; j++) p[j] = q[j];
      }
      lv.x[i] = (T)p[0];
    }
    return;
  }
  if (l > 0) {
    std::vector<T> tmp(lv.n);
    for (int i = 0; i < lv.n; i++) tmp[i] = lv.b[lv.iperm[i]];
    lv.b.swap(tmp);
  }
  if (c.smoother == 1) {
    lv.x.assign(lv.n, (T)0);
    l1_sweeps(lv, c, c.pre_inner);
    lv.r.resize(lv.n);
    for (int i = 0; i < lv.n; i++) lv.r[i] = lv.b[i] - ap_row_sum(lv.Ap, i, lv.x);
  } else {
    pre_smooth(lv, c);
  }
  spmv_rows(lv.R, lv.r, lv.bc);
  coarse_visits(L, l, c, type);
  /* x += P xc (postPCRFullSymmetric, gauss_seidel.cu:4425-4427) */
  std::vector<T> dx(lv.n);
  spmv_rows(lv.P, lv.xc, dx);
  for (int i = 0; i < lv.n; i++) lv.x[i] = lv.x[i] + dx[i];
  if (c.smoother == 1) {
    for (int rl = 0; rl < c.post_relaxes; rl++) l1_sweeps(lv, c, c.post_inner);
  } else {
    post_smooth(lv, c);
  }
  if (l > 0) {
    std::vector<T> tmp(lv.n);
    for (int i = 0; i < lv.n; i++) tmp[lv.iperm[i]] = lv.x[i];
    lv.x.swap(tmp);
  }
}

/* cycle_level0 on permuted level-0 vectors: FP64 in, FP64 out. */
template <class T>
void precond(std::vector<Level<T>>& L, const orc_config& c, const std::vector<double>& r, std::vector<double>& z) {
  Level<T>& l0 = L[0];
  int n = (int)r.size();
  l0.b.resize(n);
  for (int i = 0; i < n; i++) l0.b[i] = (T)r[i];
  vcycle(L, 0, c, c.cycle_type);
  for (int i = 0; i < n; i++) z[i] = (double)l0.x[i];
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); i++) s = fma(a[i], b[i], s);
  return s;
}

void spmv64(const Csr<double>& A, const std::vector<double>& x, std::vector<double>& y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < A.n; i++) {
    double s = 0;
    for (int e = A.rp[i]; e < A.rp[i + 1]; e++) s = fma(A.v[e], x[A.ci[e]], s);
    y[i] = s;
  }
}

template <class T>
int pcg(orc_amg* h, std::vector<Level<T>>& L, const double* b_in, double* x_inout, double tol, int maxit, int flexible,
        int* iters, double* relres) {
  int n = h->n0;
  const std::vector<int32_t>& perm = h->perm0;
  std::vector<double> b(n), x(n), y(n), r(n), z(n), p(n), rold(n);
  for (int i = 0; i < n; i++) {
    b[perm[i]] = b_in[i];
    x[perm[i]] = x_inout[i];
  }
  double bnorm = sqrt(dot(b, b));
  spmv64(h->A0p, x, y);
  for (int i = 0; i < n; i++) r[i] = b[i] - y[i];
  int status = 5, it = 0;
  double nr = sqrt(dot(r, r));
  if (bnorm == 0.0) bnorm = 1.0;
  if (nr / bnorm <= tol) {
    status = 0;
  } else {
    precond(L, h->cfg, r, z);
    p = z;
    double rz = dot(r, z);
    while (it < maxit) {
      spmv64(h->A0p, p, y);
      double yp = dot(y, p);
      if (!(yp > 0.0) || !std::isfinite(yp)) {
        status = 4;
        break;
      }
      double alpha = rz / yp;
      if (flexible) rold = r;
      for (int i = 0; i < n; i++) {
        x[i] = fma(alpha, p[i], x[i]);
        r[i] = fma(-alpha, y[i], r[i]);
      }
      nr = sqrt(dot(r, r));
      it++;
      if (!std::isfinite(nr)) {
        status = 4;
        break;
      }
      if (nr / bnorm <= tol) {
        status = 0;
        break;
      }
      precond(L, h->cfg, r, z);
      double rznew = dot(z, r);
      double beta;
      if (flexible) {
        double zro = 0;
        for (int i = 0; i < n; i++) zro = fma(z[i], rold[i], zro);
        beta = (rznew - zro) / rz;
      } else {
        beta = rznew / rz;
      }
      for (int i = 0; i < n; i++) p[i] = fma(beta, p[i], z[i]);
      rz = rznew;
    }
  }
  for (int i = 0; i < n; i++) x_inout[i] = x[perm[i]];
  if (iters) *iters = it;
  if (relres) *relres = nr / bnorm;
  return status;
}

template <class T>
void level_info(const std::vector<Level<T>>& L, int l, int64_t* o) {
  const Level<T>& lv = L[l];
  o[0] = lv.A.n;
  o[1] = lv.A.nnz();
  o[2] = lv.coarsest ? 0 : (int64_t)lv.aggIdx.size() - 1;
  o[3] = lv.coarsest ? 0 : (int64_t)lv.partIdx.size() - 1;
  o[4] = lv.coarsest ? 0 : lv.P.nnz();
}

template <class T>
void level_get(const std::vector<Level<T>>& L, int l, int32_t* Arp, int32_t* Aci, double* Av, int32_t* perm,
               int32_t* aggIdx, int32_t* partIdx, int32_t* Prp, int32_t* Pci, double* Pv) {
  const Level<T>& lv = L[l];
  if (Arp) std::copy(lv.A.rp.begin(), lv.A.rp.end(), Arp);
  if (Aci) std::copy(lv.A.ci.begin(), lv.A.ci.end(), Aci);
  if (Av)
    for (size_t i = 0; i < lv.A.v.size(); i++) Av[i] = (double)lv.A.v[i];
  if (lv.coarsest) return;
  if (perm) std::copy(lv.perm.begin(), lv.perm.end(), perm);
  if (aggIdx) std::copy(lv.aggIdx.begin(), lv.aggIdx.end(), aggIdx);
  if (partIdx) std::copy(lv.partIdx.begin(), lv.partIdx.end(), partIdx);
  if (Prp) std::copy(lv.P.rp.begin(), lv.P.rp.end(), Prp);
  if (Pci) std::copy(lv.P.ci.begin(), lv.P.ci.end(), Pci);
  if (Pv)
    for (size_t i = 0; i < lv.P.v.size(); i++) Pv[i] = (double)lv.P.v[i];
}

}  // namespace

/* ===================================================================== */
/* extern "C" API                                                         */
/* ===================================================================== */
extern "C" {

void orc_glibc_rand(uint32_t seed, int n, int32_t* out) { glibc_rand_seq(seed, n, out); }
void orc_tet_mass_integrand(double out[10]) { tet_mass_integrand(out); }
void orc_tri_quadrature(double zx[6], double wx[6], double zy[6], double wy[6]) { tri_quadrature(zx, wx, zy, wy); }

int64_t orc_build_pattern(int nv, int ne, int nvpe, const int32_t* conn, int32_t* rowptr, int32_t* cols, int64_t cap) {
  std::vector<std::vector<int32_t>> nb(nv);
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < nvpe; a++) {
      int v = conn[(size_t)e * nvpe + a];
      if (v < 0 || v >= nv) return -1;
      for (int b = 0; b < nvpe; b++) nb[v].push_back(conn[(size_t)e * nvpe + b]);
    }
  int64_t nnz = 0;
  rowptr[0] = 0;
  for (int i = 0; i < nv; i++) {
    nb[i].push_back(i);
    std::sort(nb[i].begin(), nb[i].end());
    nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
    if (nnz + (int64_t)nb[i].size() > cap) return -1;
    std::copy(nb[i].begin(), nb[i].end(), cols + nnz);
    nnz += nb[i].size();
    rowptr[i + 1] = (int32_t)nnz;
  }
  return nnz;
}

int orc_assemble(int dim, int nv, const double* xyz, int ne, const int32_t* conn, const int32_t* labels,
                 const double* coef, double lambda_mass, const int32_t* rowptr, const int32_t* cols, double* vals,
                 int reference_formula) {
  int64_t nnz = rowptr[nv];
  std::fill(vals, vals + nnz, 0.0);
  if (dim == 3) {
    double integ[10];
    tet_mass_integrand(integ);
    static const int pr[10][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 3}, {1, 1}, {1, 2}, {1, 3}, {2, 2}, {2, 3}, {3, 3}};
    for (int e = 0; e < ne; e++) {
      const int32_t* id = conn + (size_t)e * 4;
      double x[4], y[4], z[4];
      for (int a = 0; a < 4; a++) {
        x[a] = xyz[(size_t)id[a] * 3];
        y[a] = xyz[(size_t)id[a] * 3 + 1];
        z[a] = xyz[(size_t)id[a] * 3 + 2];
      }
      double co = coef ? coef[e] : (labels ? label_coefficient(labels[e]) : 1.0);
      double ev[10];
      if (reference_formula) element3d(x, y, z, co, lambda_mass, integ, ev);
      else element3d_fma(x, y, z, co, lambda_mass, integ, ev);
      for (int q = 0; q < 10; q++) {
        int i = id[pr[q][0]], j = id[pr[q][1]];
        int64_t s = find_col(rowptr, cols, i, j);
        if (s < 0) return 1;
        vals[s] += ev[q];
        if (i != j) {
          s = find_col(rowptr, cols, j, i);
          if (s < 0) return 1;
          vals[s] += ev[q];
        }
      }
    }
  } else {
    double zx[6], wx[6], zy[6], wy[6];
    tri_quadrature(zx, wx, zy, wy);
    static const int pr[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    for (int e = 0; e < ne; e++) {
      const int32_t* id = conn + (size_t)e * 3;
      double x[3], y[3];
      for (int a = 0; a < 3; a++) {
        x[a] = xyz[(size_t)id[a] * 3];
        y[a] = xyz[(size_t)id[a] * 3 + 1];
      }
      double co = coef ? coef[e] : 1.0;
      double ev[6];
      element2d(x, y, co, lambda_mass, zx, wx, zy, wy, ev);
      for (int q = 0; q < 6; q++) {
        int i = id[pr[q][0]], j = id[pr[q][1]];
        int64_t s = find_col(rowptr, cols, i, j);
        if (s < 0) return 1;
        vals[s] += ev[q];
        if (i != j) {
          s = find_col(rowptr, cols, j, i);
          if (s < 0) return 1;
          vals[s] += ev[q];
        }
      }
    }
  }
  return 0;
}

int orc_load_vector(int dim, int nv, const double* xyz, int ne, const int32_t* conn, const double* f, double* b) {
  std::fill(b, b + nv, 0.0);
  int k = dim == 3 ? 4 : 3;
  for (int e = 0; e < ne; e++) {
    const int32_t* id = conn + (size_t)e * k;
    double meas;
    if (dim == 3) {
      double x[4], y[4], z[4];
      for (int a = 0; a < 4; a++) {
        x[a] = xyz[(size_t)id[a] * 3];
        y[a] = xyz[(size_t)id[a] * 3 + 1];
        z[a] = xyz[(size_t)id[a] * 3 + 2];
      }
      double a1 = x[1] - x[3], a2 = y[1] - y[3], a3 = z[1] - z[3];
      double b1 = x[2] - x[3], b2 = y[2] - y[3], b3 = z[2] - z[3];
      double c1 = x[0] - x[3], c2 = y[0] - y[3], c3 = z[0] - z[3];
      meas = fabs(c1 * (a2 * b3 - a3 * b2) + c2 * (a3 * b1 - a1 * b3) + c3 * (a1 * b2 - a2 * b1)) / 6.0;
    } else {
      double x0 = xyz[(size_t)id[0] * 3], y0 = xyz[(size_t)id[0] * 3 + 1];
      double x1 = xyz[(size_t)id[1] * 3], y1 = xyz[(size_t)id[1] * 3 + 1];
      double x2 = xyz[(size_t)id[2] * 3], y2 = xyz[(size_t)id[2] * 3 + 1];
      meas = fabs(x0 * y2 - x0 * y1 + x1 * y0 - x1 * y2 + x2 * y1 - x2 * y0) / 2.0;
    }
    /* exact P1 mass: M_ij = meas (1 + delta_ij) / ((k)(k+1)) */
    double fs = 0;
    for (int a = 0; a < k; a++) fs += f[id[a]];
    double scale = meas / (double)(k * (k + 1));
    for (int a = 0; a < k; a++) b[id[a]] += scale * (fs + f[id[a]]);
  }
  return 0;
}

void orc_apply_dirichlet(int n, const int32_t* rowptr, const int32_t* cols, double* vals, const uint8_t* mask,
                         double* b) {
  for (int i = 0; i < n; i++)
    for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
      int j = cols[e];
      if (mask[i] || mask[j]) vals[e] = (i == j) ? 1.0 : 0.0;
    }
  if (b)
    for (int i = 0; i < n; i++)
      if (mask[i]) b[i] = 0.0;
}

int orc_random_mis(int n, const int32_t* xadj, const int32_t* adj, int k, uint32_t seed, int32_t* mis) {
  std::vector<int32_t> m;
  int st = random_mis(n, xadj, adj, k, seed, m);
  std::copy(m.begin(), m.end(), mis);
  return st;
}

int orc_oldmis(int n, const int32_t* xadj, const int32_t* adj, int params, int part_max, uint32_t seed,
               int32_t* permutation, int32_t* ipermutation, int32_t* aggregate_idx, int32_t* n_agg,
               int32_t* partition_idx, int32_t* n_part, int32_t* partition_label, int32_t* xadj_out, int32_t* adj_out,
               int32_t* nnz_out) {
  OldMisOut o;
  int st = old_mis(n, xadj, adj, params, part_max, seed, o);
  if (st) return st;
  std::copy(o.perm.begin(), o.perm.end(), permutation);
  std::copy(o.iperm.begin(), o.iperm.end(), ipermutation);
  std::copy(o.aggIdx.begin(), o.aggIdx.end(), aggregate_idx);
  *n_agg = (int32_t)o.aggIdx.size() - 1;
  std::copy(o.partIdx.begin(), o.partIdx.end(), partition_idx);
  *n_part = (int32_t)o.partIdx.size() - 1;
  std::copy(o.partLabel.begin(), o.partLabel.end(), partition_label);
  std::copy(o.xadjOut.begin(), o.xadjOut.end(), xadj_out);
  std::copy(o.adjOut.begin(), o.adjOut.end(), adj_out);
  *nnz_out = (int32_t)o.adjOut.size();
  return 0;
}

void orc_config_default(orc_config* c) {
  c->max_levels = 100;
  c->top_size = 256;
  c->rand_mis_params = 90102;
  c->partition_max = 512;
  c->pre_inner = 5;
  c->post_inner = 5;
  c->post_relaxes = 1;
  c->smoother_weight = 1.0;
  c->pro_omega = 0.67;
  c->seed = 1;
  c->fp64_hierarchy = 0;
  c->threads = 0;
  c->cycle_type = 0;
  c->smoother = 0;
}

orc_amg* orc_amg_setup(const orc_config* cfg, int n, const int32_t* rowptr, const int32_t* cols, const double* vals,
                       const int32_t* gxadj, const int32_t* gadj, int* status) {
  orc_amg* h = new orc_amg();
  h->cfg = *cfg;
#ifdef _OPENMP
  if (cfg->threads > 0) omp_set_num_threads(cfg->threads);
#endif
  h->n0 = n;
  Csr<double> A;
  A.n = A.m = n;
  A.rp.assign(rowptr, rowptr + n + 1);
  A.ci.assign(cols, cols + rowptr[n]);
  A.v.assign(vals, vals + rowptr[n]);
  int st = cfg->fp64_hierarchy ? setup_levels(h, h->Ld, A, gxadj, gadj) : setup_levels(h, h->Lf, A, gxadj, gadj);
  if (st) {
    if (status) *status = st;
    delete h;
    return nullptr;
  }
  bool coarse0 = cfg->fp64_hierarchy ? h->Ld[0].coarsest : h->Lf[0].coarsest;
  if (coarse0) {
    h->perm0.resize(n);
    std::iota(h->perm0.begin(), h->perm0.end(), 0);
    h->iperm0 = h->perm0;
  } else {
    h->perm0 = cfg->fp64_hierarchy ? h->Ld[0].perm : h->Lf[0].perm;
    h->iperm0 = cfg->fp64_hierarchy ? h->Ld[0].iperm : h->Lf[0].iperm;
  }
  h->A0p = permute(A, h->perm0, h->iperm0);
  if (status) *status = 0;
  return h;
}

void orc_amg_free(orc_amg* h) { delete h; }
int orc_amg_num_levels(const orc_amg* h) { return h->nlev(); }

int orc_amg_level_info(const orc_amg* h, int level, int64_t* info5) {
  if (level < 0 || level >= h->nlev()) return 1;
  if (h->cfg.fp64_hierarchy) level_info(h->Ld, level, info5);
  else level_info(h->Lf, level, info5);
  return 0;
}

int orc_amg_level_get(const orc_amg* h, int level, int32_t* A_rowptr, int32_t* A_cols, double* A_vals, int32_t* perm,
                      int32_t* agg_idx, int32_t* part_idx, int32_t* P_rowptr, int32_t* P_cols, double* P_vals) {
  if (level < 0 || level >= h->nlev()) return 1;
  if (h->cfg.fp64_hierarchy) level_get(h->Ld, level, A_rowptr, A_cols, A_vals, perm, agg_idx, part_idx, P_rowptr, P_cols, P_vals);
  else level_get(h->Lf, level, A_rowptr, A_cols, A_vals, perm, agg_idx, part_idx, P_rowptr, P_cols, P_vals);
  return 0;
}

int orc_amg_vcycle(orc_amg* h, const double* r, double* z) {
  int n = h->n0;
  std::vector<double> rp(n), zp(n);
  for (int i = 0; i < n; i++) rp[h->perm0[i]] = r[i];
  if (h->cfg.fp64_hierarchy) precond(h->Ld, h->cfg, rp, zp);
  else precond(h->Lf, h->cfg, rp, zp);
  for (int i = 0; i < n; i++) z[i] = zp[h->perm0[i]];
  return 0;
}

int orc_amg_pcg(orc_amg* h, const double* b, double* x, double tol, int max_iters, int flexible, int* iters,
                double* relres) {
  if (h->cfg.fp64_hierarchy) return pcg(h, h->Ld, b, x, tol, max_iters, flexible, iters, relres);
  return pcg(h, h->Lf, b, x, tol, max_iters, flexible, iters, relres);
}

int orc_cg(int n, const int32_t* rowptr, const int32_t* cols, const double* vals, const double* b, double* x, double tol,
           int max_iters, int* iters, double* relres) {
  Csr<double> A;
  A.n = A.m = n;
  A.rp.assign(rowptr, rowptr + n + 1);
  A.ci.assign(cols, cols + rowptr[n]);
  A.v.assign(vals, vals + rowptr[n]);
  std::vector<double> bb(b, b + n), xx(x, x + n), r(n), p(n), y(n), z(n), dinv(n, 1.0);
  for (int i = 0; i < n; i++) {
    int64_t d = find_col(rowptr, cols, i, i);
    if (d >= 0 && vals[d] != 0.0) dinv[i] = 1.0 / vals[d];
  }
  double bn = sqrt(dot(bb, bb));
  if (bn == 0) bn = 1;
  spmv64(A, xx, y);
  for (int i = 0; i < n; i++) r[i] = bb[i] - y[i];
  for (int i = 0; i < n; i++) z[i] = dinv[i] * r[i];
  p = z;
  double rz = dot(r, z), nr = sqrt(dot(r, r));
  int it = 0, st = 5;
  while (it < max_iters) {
    if (nr / bn <= tol) {
      st = 0;
      break;
    }
    spmv64(A, p, y);
    double yp = dot(y, p);
    if (!(yp > 0)) {
      st = 4;
      break;
    }
    double al = rz / yp;
    for (int i = 0; i < n; i++) {
      xx[i] = fma(al, p[i], xx[i]);
      r[i] = fma(-al, y[i], r[i]);
    }
    for (int i = 0; i < n; i++) z[i] = dinv[i] * r[i];
    double rzn = dot(r, z);
    double be = rzn / rz;
    for (int i = 0; i < n; i++) p[i] = fma(be, p[i], z[i]);
    rz = rzn;
    nr = sqrt(dot(r, r));
    it++;
  }
  if (nr / bn <= tol) st = 0;
  std::copy(xx.begin(), xx.end(), x);
  if (iters) *iters = it;
  if (relres) *relres = nr / bn;
  return st;
}

}  // extern "C"
