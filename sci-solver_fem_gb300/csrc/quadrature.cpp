// quadrature.cpp -- host-side Gauss-Jacobi tables of the P1 element kernels.
//
// The reference builds these once per assembly on the host (FEM3D::assemble,
// src/core/cuda/FEM3D.cu:501-549; FEM2D::assemble, FEM2D.cu:340-356) and copies
// them to constant memory.  The same recurrences, Newton iteration (EPS 1e-6,
// 60 steps, PI = 3.1415927) and collapsed-coordinate map are used here so the
// tables agree bit for bit with the reference's.
#include <cmath>
#include <vector>

#include "quadrature.h"

namespace femgpu {
namespace {

double factorial_gamma(int x) {  // Gamma(x) for positive integers (FEM3D.cu:58-136)
  double g = 1.0;
  for (int i = 2; i < x; i++) g *= i;
  return g;
}

std::vector<double> poly(int deg, const std::vector<double>& x, int al, int be) {
  std::vector<double> y(x.size());
  if (deg == 0) {
    for (auto& v : y) v = 1.0;
    return y;
  }
  if (deg == 1) {
    for (size_t i = 0; i < x.size(); i++) y[i] = 0.5 * ((al - be) + (al + be + 2.0) * x[i]);
    return y;
  }
  const double dm = deg - 1.0;
  const double t = 2.0 * dm + al + be;
  const double c1 = 2.0 * (dm + 1) * (dm + al + be + 1) * t;
  const double c2 = (t + 1) * (al * al - be * be);
  const double c3 = t * (t + 1.0) * (t + 2.0);
  const double c4 = 2.0 * (dm + al) * (dm + be) * (t + 2.0);
  std::vector<double> pm1 = poly(deg - 1, x, al, be), pm2 = poly(deg - 2, x, al, be);
  for (size_t i = 0; i < x.size(); i++) y[i] = ((c2 + c3 * x[i]) * pm1[i] - c4 * pm2[i]) / c1;
  return y;
}

std::vector<double> dpoly(int deg, const std::vector<double>& x, int al, int be) {
  std::vector<double> y(x.size(), 0.0);
  if (deg == 0) return y;
  std::vector<double> p = poly(deg - 1, x, al + 1, be + 1);
  for (size_t i = 0; i < p.size(); i++) y[i] = 0.5 * (al + be + deg + 1) * p[i];
  return y;
}

std::vector<double> zeros(int deg, int al, int be) {
  std::vector<double> z(deg, 0.0);
  if (deg == 0) return z;
  const double dth = double(3.1415927) / (2.0 * deg);
  double prev = 0.0;
  std::vector<double> r(1);
  for (int k = 0; k < deg; k++) {
    r[0] = -cos((2.0 * k + 1.0) * dth);
    if (k) r[0] = 0.5 * (r[0] + prev);
    for (int it = 0; it < 60; it++) {
      double p = poly(deg, r, al, be)[0];
      double dp = dpoly(deg, r, al, be)[0];
      double defl = 0.0;
      for (int i = 0; i < k; i++) defl = defl + 1.0 / (r[0] - z[i]);
      double step = -p / (dp - defl * p);
      r[0] = r[0] + step;
      if (fabs(step) < 1.0e-6) break;
    }
    z[k] = r[0];
    prev = r[0];
  }
  return z;
}

void lobatto(std::vector<double>& Z, std::vector<double>& W, int deg, int al, int be) {
  Z.assign(deg, 0.0);
  W.assign(deg, 0.0);
  if (deg == 1) return;
  Z[0] = -1;
  Z[deg - 1] = 1;
  std::vector<double> inner = zeros(deg - 2, al + 1, be + 1);
  for (int i = 1; i < deg - 1; i++) Z[i] = inner[i - 1];
  W = poly(deg - 1, Z, al, be);
  double fac = pow(2.0, (double)(al + be + 1)) * factorial_gamma(al + deg) * factorial_gamma(be + deg);
  fac = fac / ((deg - 1) * factorial_gamma(deg) * factorial_gamma(al + be + deg + 1));
  for (int j = 0; j < deg; j++) W[j] = fac / (W[j] * W[j]);
  W[0] = W[0] * (be + 1);
  W[deg - 1] = W[deg - 1] * (al + 1);
}

void radau(std::vector<double>& Z, std::vector<double>& W, int deg, int al, int be) {
  Z.assign(deg, 0.0);
  W.assign(deg, 0.0);
  if (deg == 1) {
    W[0] = 2.0;
    return;
  }
  Z[0] = -1;
  std::vector<double> inner = zeros(deg - 1, al, be + 1);
  for (int i = 1; i < deg; i++) Z[i] = inner[i - 1];
  W = poly(deg - 1, Z, al, be);
  double fac = pow(2.0, (double)(al + be)) * factorial_gamma(al + deg) * factorial_gamma(be + deg);
  fac = fac / (factorial_gamma(deg) * (be + deg) * factorial_gamma(al + be + deg + 1));
  for (int j = 0; j < deg; j++) W[j] = fac * (1 - Z[j]) / (W[j] * W[j]);
  W[0] = W[0] * (be + 1);
}

}  // namespace

void tet_mass_table(double out[10]) {
  const int D = 4;
  std::vector<double> zx, wx, zy, wy, zz, wz;
  lobatto(zx, wx, D, 0, 0);
  radau(zy, wy, D, 1, 0);
  radau(zz, wz, D, 2, 0);
  for (int i = 0; i < D; i++) {
    wy[i] /= 2;
    wz[i] /= 4;
  }
  // P1 basis of the unit tet at the collapsed quadrature points.
  double phi[4][D][D][D];
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++)
      for (int k = 0; k < D; k++) {
        double u = (1 + zx[i]) * 0.5 * (1 - zy[j]) * 0.5 * (1 - zz[k]) * 0.5;
        double v = (1 + zy[j]) * 0.5 * (1 - zz[k]) * 0.5;
        double w = (1 + zz[k]) * 0.5;
        phi[0][i][j][k] = 1 + -1 * u + -1 * v + -1 * w;
        phi[1][i][j][k] = 0 + 1 * u + 0 * v + 0 * w;
        phi[2][i][j][k] = 0 + 0 * u + 1 * v + 0 * w;
        phi[3][i][j][k] = 0 + 0 * u + 0 * v + 1 * w;
      }
  int c = 0;
  for (int a = 0; a < 4; a++)
    for (int b = a; b < 4; b++) {
      double sum = 0;
      for (int i = 0; i < D; i++) {
        double sy = 0.0;
        for (int j = 0; j < D; j++) {
          double sz = 0.0;
          for (int k = 0; k < D; k++) sz += (phi[a][i][j][k] * phi[b][i][j][k]) * wz[k];
          sy += sz * wy[j];
        }
        sum += sy * wx[i];
      }
      out[c++] = sum;
    }
}

void tri_quadrature_table(double zx[6], double wx[6], double zy[6], double wy[6]) {
  std::vector<double> a, b, c, d;
  lobatto(a, b, 6, 0, 0);
  radau(c, d, 6, 1, 0);
  for (int i = 0; i < 6; i++) {
    zx[i] = a[i];
    wx[i] = b[i];
    zy[i] = c[i];
    wy[i] = d[i];
  }
}

}  // namespace femgpu
