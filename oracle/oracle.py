"""ctypes wrapper of the CPU oracle (libfem_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg.  The product path never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfem_oracle.so")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class OrcConfig(C.Structure):
    _fields_ = [
        ("max_levels", C.c_int), ("top_size", C.c_int), ("rand_mis_params", C.c_int),
        ("partition_max", C.c_int), ("pre_inner", C.c_int), ("post_inner", C.c_int),
        ("post_relaxes", C.c_int), ("smoother_weight", C.c_double), ("pro_omega", C.c_double),
        ("seed", C.c_uint32), ("fp64_hierarchy", C.c_int), ("threads", C.c_int), ("cycle_type", C.c_int),
        ("smoother", C.c_int),
    ]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_glibc_rand.argtypes = [C.c_uint32, C.c_int, _i32p]
        L.orc_tet_mass_integrand.argtypes = [_f64p]
        L.orc_tri_quadrature.argtypes = [_f64p, _f64p, _f64p, _f64p]
        L.orc_build_pattern.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _i32p, _i32p, C.c_int64]
        L.orc_build_pattern.restype = C.c_int64
        L.orc_assemble.argtypes = [C.c_int, C.c_int, _f64p, C.c_int, _i32p, C.c_void_p, C.c_void_p,
                                   C.c_double, _i32p, _i32p, _f64p, C.c_int]
        L.orc_load_vector.argtypes = [C.c_int, C.c_int, _f64p, C.c_int, _i32p, _f64p, _f64p]
        L.orc_apply_dirichlet.argtypes = [C.c_int, _i32p, _i32p, _f64p, _u8p, C.c_void_p]
        L.orc_random_mis.argtypes = [C.c_int, _i32p, _i32p, C.c_int, C.c_uint32, _i32p]
        L.orc_oldmis.argtypes = [C.c_int, _i32p, _i32p, C.c_int, C.c_int, C.c_uint32] + [_i32p] * 3 + \
            [C.POINTER(C.c_int32), _i32p, C.POINTER(C.c_int32), _i32p, _i32p, _i32p, C.POINTER(C.c_int32)]
        L.orc_config_default.argtypes = [C.POINTER(OrcConfig)]
        L.orc_amg_setup.argtypes = [C.POINTER(OrcConfig), C.c_int, _i32p, _i32p, _f64p, _i32p, _i32p,
                                    C.POINTER(C.c_int)]
        L.orc_amg_setup.restype = C.c_void_p
        L.orc_amg_free.argtypes = [C.c_void_p]
        L.orc_amg_num_levels.argtypes = [C.c_void_p]
        L.orc_amg_level_info.argtypes = [C.c_void_p, C.c_int, _i64p]
        L.orc_amg_level_get.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 9
        L.orc_amg_vcycle.argtypes = [C.c_void_p, _f64p, _f64p]
        L.orc_amg_pcg.argtypes = [C.c_void_p, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                  C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_cg.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_double, C.c_int,
                             C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def glibc_rand(seed: int, n: int):
    out = np.zeros(n, np.int32)
    lib().orc_glibc_rand(seed, n, out)
    return out


def tet_mass_integrand():
    out = np.zeros(10)
    lib().orc_tet_mass_integrand(out)
    return out


def tri_quadrature():
    a, b, c, d = (np.zeros(6) for _ in range(4))
    lib().orc_tri_quadrature(a, b, c, d)
    return a, b, c, d


def build_pattern(nv: int, conn: np.ndarray):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    ne, k = conn.shape
    rowptr = np.zeros(nv + 1, np.int32)
    cap = int(ne) * k * k + nv
    cols = np.zeros(cap, np.int32)
    nnz = lib().orc_build_pattern(nv, ne, k, conn.ravel(), rowptr, cols, cap)
    if nnz < 0:
        raise ValueError("pattern build failed")
    return rowptr, cols[:nnz].copy()


def assemble(xyz, conn, rowptr, cols, labels=None, coef=None, lambda_mass=1.0, reference_formula=False):
    """A = sum_e coef_e K_e + lambda_mass M_e on the pattern.  Tetrahedra: the library's
    fused multiply-add gradients by default (what the GPU computes, bit for bit); with
    reference_formula the reference's 4x4 cofactor inverse."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    dim = 3 if conn.shape[1] == 4 else 2
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    labels = None if labels is None else np.ascontiguousarray(labels, dtype=np.int32)
    coef = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
    vals = np.zeros(cols.shape[0])
    st = lib().orc_assemble(dim, xyz.shape[0], xyz.ravel(), conn.shape[0], conn.ravel(), _ptr(labels),
                            _ptr(coef), float(lambda_mass), rowptr, cols, vals, int(bool(reference_formula)))
    if st:
        raise ValueError("assembly failed")
    return vals


def load_vector(xyz, conn, f):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    dim = 3 if conn.shape[1] == 4 else 2
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    b = np.zeros(xyz.shape[0])
    lib().orc_load_vector(dim, xyz.shape[0], xyz.ravel(), conn.shape[0], conn.ravel(),
                          np.ascontiguousarray(f, dtype=np.float64), b)
    return b


def apply_dirichlet(rowptr, cols, vals, mask, b=None):
    vals = vals.copy()
    bb = None if b is None else b.copy()
    lib().orc_apply_dirichlet(rowptr.shape[0] - 1, rowptr, cols, vals,
                              np.ascontiguousarray(mask, dtype=np.uint8), _ptr(bb))
    return vals, bb


def random_mis(xadj, adj, k, seed):
    n = xadj.shape[0] - 1
    mis = np.zeros(n, np.int32)
    st = lib().orc_random_mis(n, xadj, adj, k, seed, mis)
    if st:
        raise RuntimeError(f"random_mis status {st}")
    return mis


def oldmis(xadj, adj, params=90102, part_max=512, seed=1):
    n = xadj.shape[0] - 1
    perm, iperm, plabel = (np.zeros(n, np.int32) for _ in range(3))
    agg_idx = np.zeros(n + 1, np.int32)
    part_idx = np.zeros(n + 1, np.int32)
    xo = np.zeros(n + 1, np.int32)
    ao = np.zeros(max(1, adj.shape[0]), np.int32)
    na, npart, nnz = C.c_int32(), C.c_int32(), C.c_int32()
    st = lib().orc_oldmis(n, xadj, adj, params, part_max, seed, perm, iperm, agg_idx, C.byref(na),
                          part_idx, C.byref(npart), plabel, xo, ao, C.byref(nnz))
    if st:
        raise RuntimeError(f"oldmis status {st}")
    na, npart = na.value, npart.value
    return dict(perm=perm, iperm=iperm, agg_idx=agg_idx[:na + 1], part_idx=part_idx[:npart + 1],
                part_label=plabel, xadj_out=xo[:na + 1], adj_out=ao[:nnz.value])


def default_config(**kw):
    c = OrcConfig()
    lib().orc_config_default(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class OracleAMG:
    """Oracle hierarchy; vectors are in the original (unpermuted) numbering."""

    def __init__(self, rowptr, cols, vals, gxadj, gadj, **cfg):
        self.cfg = default_config(**cfg)
        st = C.c_int(0)
        self.n = rowptr.shape[0] - 1
        self.h = lib().orc_amg_setup(C.byref(self.cfg), self.n, rowptr, cols, np.ascontiguousarray(vals),
                                     gxadj, gadj, C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle setup failed with status {st.value}")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_amg_free(self.h)
            self.h = None

    @property
    def num_levels(self):
        return lib().orc_amg_num_levels(self.h)

    def level_info(self, level):
        o = np.zeros(5, np.int64)
        lib().orc_amg_level_info(self.h, level, o)
        return dict(n=int(o[0]), nnz=int(o[1]), n_agg=int(o[2]), n_part=int(o[3]), nnz_p=int(o[4]))

    def level(self, level):
        info = self.level_info(level)
        n, nnz = info["n"], info["nnz"]
        rp, ci, v = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
        out = dict(info, A_rowptr=rp, A_cols=ci, A_vals=v)
        args = [_ptr(rp), _ptr(ci), _ptr(v)] + [None] * 6
        if info["n_agg"] > 0:
            perm = np.zeros(n, np.int32)
            agg = np.zeros(info["n_agg"] + 1, np.int32)
            part = np.zeros(info["n_part"] + 1, np.int32)
            prp = np.zeros(n + 1, np.int32)
            pci = np.zeros(info["nnz_p"], np.int32)
            pv = np.zeros(info["nnz_p"])
            out.update(perm=perm, agg_idx=agg, part_idx=part, P_rowptr=prp, P_cols=pci, P_vals=pv)
            args[3:] = [_ptr(perm), _ptr(agg), _ptr(part), _ptr(prp), _ptr(pci), _ptr(pv)]
        lib().orc_amg_level_get(self.h, level, *args)
        return out

    def vcycle(self, r):
        z = np.zeros(self.n)
        lib().orc_amg_vcycle(self.h, np.ascontiguousarray(r, dtype=np.float64), z)
        return z

    def pcg(self, b, x0=None, tol=1e-8, max_iters=100, flexible=False):
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        it, rr = C.c_int(), C.c_double()
        st = lib().orc_amg_pcg(self.h, np.ascontiguousarray(b, dtype=np.float64), x, tol, max_iters,
                               int(flexible), C.byref(it), C.byref(rr))
        return x, dict(status=st, iters=it.value, relres=rr.value)


def cg(rowptr, cols, vals, b, tol=1e-12, max_iters=100000):
    n = rowptr.shape[0] - 1
    x = np.zeros(n)
    it, rr = C.c_int(), C.c_double()
    st = lib().orc_cg(n, rowptr, cols, np.ascontiguousarray(vals), np.ascontiguousarray(b), x, tol, max_iters,
                      C.byref(it), C.byref(rr))
    return x, dict(status=st, iters=it.value, relres=rr.value)
