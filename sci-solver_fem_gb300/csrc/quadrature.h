// quadrature.h -- host-side quadrature tables for the element kernels.
#pragma once

namespace femgpu {
// Reference-tet P1 mass integrand, 10 upper-triangle entries (FEM3D.cu:452-475).
void tet_mass_table(double out[10]);
// 6-point Gauss-Lobatto (x) and Gauss-Radau(1,0) (y) zeros/weights (FEM2D.cu:358-378).
void tri_quadrature_table(double zx[6], double wx[6], double zy[6], double wy[6]);
}  // namespace femgpu
