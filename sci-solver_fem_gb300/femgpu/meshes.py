"""Synthetic meshes and problem data for the P1 FEM path.

All generators are seeded and return plain numpy arrays:
  xyz  float64 (nv, 3)   vertex coordinates (z = 0 for triangle meshes)
  conn int32   (ne, 4|3) element connectivity, 0-based

The 3D generator splits each cube of an n^3 grid into 6 tetrahedra sharing the
(0,0,0)-(1,1,1) diagonal (Kuhn split); vertex id = (i*(n+1) + j)*(n+1) + k.
The 2D generator splits each square of an n^2 grid along its (i,j)-(i+1,j+1)
diagonal and jitters interior vertices by U[-0.2h, 0.2h]^2.
"""
from __future__ import annotations

import numpy as np

# The six Kuhn tetrahedra of the unit cube, as corner bit masks (x=4, y=2, z=1):
# each is a monotone lattice path 000 -> 111 through one permutation of the axes.
_KUHN_PATHS = (
    (0, 4, 6, 7), (0, 4, 5, 7), (0, 2, 6, 7),
    (0, 2, 3, 7), (0, 1, 5, 7), (0, 1, 3, 7),
)


def kuhn_cube(n: int, length: float = 1.0):
    """Unit cube with n^3 cells, 6 tets per cell: (n+1)^3 vertices, 6 n^3 tets."""
    m = n + 1
    g = np.arange(m, dtype=np.float64) * (length / n)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    xyz = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()

    def vid(dx, dy, dz):
        return ((ci + dx) * m + (cj + dy)) * m + (ck + dz)

    corner = {}
    for mask in range(8):
        corner[mask] = vid((mask >> 2) & 1, (mask >> 1) & 1, mask & 1)
    tets = []
    for path in _KUHN_PATHS:
        tets.append(np.stack([corner[c] for c in path], axis=1))
    conn = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return xyz, conn


def jittered_square(n: int, seed: int = 1, jitter: float = 0.2):
    """Unit square with n^2 cells split into 2 triangles, interior vertices jittered."""
    m = n + 1
    h = 1.0 / n
    g = np.arange(m, dtype=np.float64) * h
    I, J = np.meshgrid(g, g, indexing="ij")
    xy = np.stack([I.ravel(), J.ravel()], axis=1)
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, size=xy.shape)
    ii, jj = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    interior = ((ii > 0) & (ii < n) & (jj > 0) & (jj < n)).ravel()
    xy[interior] += d[interior]
    ci, cj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    v00 = ci * m + cj
    v10 = (ci + 1) * m + cj
    v01 = ci * m + cj + 1
    v11 = (ci + 1) * m + cj + 1
    t1 = np.stack([v00, v10, v11], axis=1)
    t2 = np.stack([v00, v11, v01], axis=1)
    conn = np.stack([t1, t2], axis=1).reshape(-1, 3).astype(np.int32)
    xyz = np.zeros((m * m, 3))
    xyz[:, :2] = xy
    return xyz, conn


def boundary_mask_2d(n: int):
    m = n + 1
    ii, jj = np.meshgrid(np.arange(m), np.arange(m), indexing="ij")
    return (((ii == 0) | (ii == n) | (jj == 0) | (jj == n)).ravel()).astype(np.uint8)


def bottom_face_mask(n: int):
    """Dirichlet mask for the z = 0 face of the Kuhn cube."""
    m = n + 1
    k = np.arange(m ** 3) % m
    return (k == 0).astype(np.uint8)


def poisson3d_problem(n: int, sigma: float = 1.0, kappa_seed: int = 2, f_seed: int = 3):
    """3D Poisson benchmark data: kappa_e = exp(sigma * g_e), g ~ N(0,1);
    f_v ~ U[-1,1]; Dirichlet u = 0 on z = 0, Neumann elsewhere."""
    xyz, conn = kuhn_cube(n)
    g = np.random.default_rng(kappa_seed).standard_normal(conn.shape[0])
    kappa = np.exp(sigma * g)
    f = np.random.default_rng(f_seed).uniform(-1.0, 1.0, size=xyz.shape[0])
    mask = bottom_face_mask(n)
    return xyz, conn, kappa, f, mask


def poisson2d_problem(n: int = 64, seed: int = 1):
    """2D Poisson: kappa = 1, f = 1, homogeneous Dirichlet on the whole boundary."""
    xyz, conn = jittered_square(n, seed=seed)
    kappa = np.ones(conn.shape[0])
    f = np.ones(xyz.shape[0])
    mask = boundary_mask_2d(n)
    return xyz, conn, kappa, f, mask


def adjacency_from_pattern(rowptr: np.ndarray, cols: np.ndarray):
    """Mesh graph (no self loops) from a CSR pattern that includes the diagonal."""
    n = rowptr.shape[0] - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rowptr))
    keep = cols != rows
    counts = np.bincount(rows[keep], minlength=n)
    xadj = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(counts, out=xadj[1:])
    return xadj, cols[keep].astype(np.int32)
