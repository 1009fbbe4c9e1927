"""ctypes declarations of include/femgpu.h and the Solver wrapper."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_i64 = C.c_int64
_pi64 = C.POINTER(C.c_int64)

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "not ready", 4: "breakdown",
          5: "not converged", 6: "limit reached", 7: "I/O error", 8: "allocation failed", 9: "no CUDA device"}

# every symbol include/femgpu.h declares
EXPORTS = [
    "femgpu_config_default", "femgpu_create", "femgpu_destroy", "femgpu_set_config", "femgpu_status_string",
    "femgpu_last_error",
    "femgpu_set_mesh", "femgpu_assemble", "femgpu_assemble_device", "femgpu_load_vector", "femgpu_set_dirichlet", "femgpu_set_matrix_csr",
    "femgpu_setup", "femgpu_solve", "femgpu_solve_device", "femgpu_spmv_device", "femgpu_get_matrix",
    "femgpu_num_levels", "femgpu_get_level_info", "femgpu_level_get", "femgpu_vcycle", "femgpu_kernel_launches",
    "femgpu_profile_kernel", "femgpu_load_vector_device_noalloc", "femgpu_adjoint_grad",
    "femgpu_adjoint_grad_device", "femgpu_solve_multi", "femgpu_solve_multi_device", "femgpu_solve_batch",
    "femgpu_save_hierarchy", "femgpu_load_hierarchy", "femgpu_test_copy_wait_limit",
    "femgpu_read_tetgen", "femgpu_read_ply", "femgpu_read_mat_sparse", "femgpu_read_mat_array",
    "femgpu_write_mat_array", "femgpu_write_vtk",
]


class Config(C.Structure):
    _fields_ = [
        ("verbose", C.c_int), ("maxLevels", C.c_int), ("maxIters", C.c_int), ("preInnerIters", C.c_int),
        ("postInnerIters", C.c_int), ("postRelaxes", C.c_int), ("cycleIters", C.c_int), ("dsType", C.c_int),
        ("topSize", C.c_int), ("randMisParameters", C.c_int), ("partitionMaxSize", C.c_int),
        ("aggregatorType", C.c_int), ("convergeType", C.c_int), ("tolerance", C.c_double), ("cycleType", C.c_int),
        ("solverType", C.c_int), ("smootherWeight", C.c_double), ("proOmega", C.c_double), ("device", C.c_int),
        ("blockSize", C.c_int), ("seed", C.c_uint32), ("precision", C.c_int), ("flexibleCG", C.c_int),
        ("stream", C.c_void_p),
        ("mem_pool", C.c_void_p),
        ("autotune", C.c_int),
        ("smoother", C.c_int),
    ]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("relative_residual", C.c_double), ("setup_ms", C.c_double),
                ("solve_ms", C.c_double), ("num_levels", C.c_int)]


class LevelInfo(C.Structure):
    _fields_ = [("rows", C.c_int64), ("nnz", C.c_int64), ("aggregates", C.c_int64), ("partitions", C.c_int64),
                ("nnz_p", C.c_int64)]


class FemgpuError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"femgpu: {STATUS.get(status, status)}" + (f": {msg}" if msg else ""))


_lib = None


def native_library_path(build_if_missing: bool = True) -> str:
    if build_if_missing:
        return _build.build_library()
    return _build.LIB_PATH


def lib():
    """Loads libfemgpu.so (building it in-tree when the sources changed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = native_library_path()
    if not os.path.exists(path):
        raise ImportError(f"libfemgpu.so not found at {path}; the CUDA extension is required")
    L = C.CDLL(path)
    L.femgpu_config_default.argtypes = [C.POINTER(Config)]
    L.femgpu_config_default.restype = None
    L.femgpu_create.argtypes = [C.POINTER(_vp), C.POINTER(Config)]
    L.femgpu_destroy.argtypes = [_vp]
    L.femgpu_set_config.argtypes = [_vp, C.POINTER(Config)]
    L.femgpu_status_string.argtypes = [C.c_int]
    L.femgpu_status_string.restype = C.c_char_p
    L.femgpu_last_error.argtypes = [_vp]
    L.femgpu_last_error.restype = C.c_char_p
    L.femgpu_set_mesh.argtypes = [_vp, C.c_int, _i64, _f64p, _i64, _i32p, _vp]
    L.femgpu_assemble.argtypes = [_vp, _vp, C.c_double]
    L.femgpu_assemble_device.argtypes = [_vp, _vp, C.c_double]
    L.femgpu_load_vector.argtypes = [_vp, _f64p, _f64p]
    L.femgpu_set_dirichlet.argtypes = [_vp, _u8p]
    L.femgpu_set_matrix_csr.argtypes = [_vp, _i64, _i32p, _i32p, _f64p]
    L.femgpu_setup.argtypes = [_vp]
    L.femgpu_solve.argtypes = [_vp, _f64p, _f64p, C.POINTER(SolveStats)]
    L.femgpu_solve_device.argtypes = [_vp, _vp, _vp, C.POINTER(SolveStats)]
    L.femgpu_spmv_device.argtypes = [_vp, _vp, _vp]
    L.femgpu_load_vector_device_noalloc.argtypes = [_vp, _vp, _vp]
    L.femgpu_adjoint_grad.argtypes = [_vp, _f64p, _f64p, _f64p, C.POINTER(SolveStats)]
    L.femgpu_solve_multi.argtypes = [_vp, C.c_int, _f64p, _f64p, C.POINTER(SolveStats)]
    L.femgpu_solve_multi_device.argtypes = [_vp, C.c_int, _vp, _i64, _vp, _i64, C.POINTER(SolveStats)]
    L.femgpu_save_hierarchy.argtypes = [_vp, C.c_char_p]
    L.femgpu_load_hierarchy.argtypes = [_vp, C.c_char_p]
    L.femgpu_solve_batch.argtypes = [C.c_int, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.c_int, C.c_int,
                                     C.POINTER(SolveStats)]
    L.femgpu_adjoint_grad_device.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(SolveStats)]
    L.femgpu_get_matrix.argtypes = [_vp, _pi64, _pi64, _vp, _vp, _vp]
    L.femgpu_num_levels.argtypes = [_vp, C.POINTER(C.c_int)]
    L.femgpu_get_level_info.argtypes = [_vp, C.c_int, C.POINTER(LevelInfo)]
    L.femgpu_level_get.argtypes = [_vp, C.c_int] + [_vp] * 9
    L.femgpu_vcycle.argtypes = [_vp, _f64p, _f64p]
    L.femgpu_kernel_launches.argtypes = [_vp, _pi64]
    L.femgpu_test_copy_wait_limit.argtypes = [_vp, C.c_int]
    L.femgpu_profile_kernel.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.femgpu_read_tetgen.argtypes = [C.c_char_p, C.c_char_p, _pi64, _pi64, _vp, _vp, _vp]
    L.femgpu_read_ply.argtypes = [C.c_char_p, _pi64, _pi64, _vp, _vp]
    L.femgpu_read_mat_sparse.argtypes = [C.c_char_p, _pi64, _pi64, _pi64, _vp, _vp, _vp]
    L.femgpu_read_mat_array.argtypes = [C.c_char_p, _pi64, _vp]
    L.femgpu_write_mat_array.argtypes = [C.c_char_p, _i64, _f64p]
    L.femgpu_write_vtk.argtypes = [C.c_char_p, C.c_int, _i64, _f64p, _i64, _i32p, _vp]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _check(st, h=None):
    if st != 0:
        msg = lib().femgpu_last_error(h).decode(errors="replace")
        raise FemgpuError(st, msg)


def kernel_launches() -> int:
    c = C.c_int64()
    lib().femgpu_kernel_launches(None, C.byref(c))
    return c.value


class Solver:
    """One solver context (femgpu_handle).  Keyword options are the FEMSolver members
    (maxLevels, tolerance, solverType, ...) plus seed, precision, flexibleCG, stream, mem_pool."""

    def __init__(self, **options):
        L = lib()
        self.cfg = Config()
        L.femgpu_config_default(C.byref(self.cfg))
        for k, v in options.items():
            if not hasattr(self.cfg, k):
                raise AttributeError(f"unknown option {k}")
            setattr(self.cfg, k, v)
        h = _vp()
        _check(L.femgpu_create(C.byref(h), C.byref(self.cfg)))
        self.h = h
        self.n = 0
        self.dim = 0

    def set_config(self, **options):
        """Changes options of this context (femgpu_set_config); the next setup / solve uses them."""
        for k, v in options.items():
            if not hasattr(self.cfg, k):
                raise AttributeError(f"unknown option {k}")
            setattr(self.cfg, k, v)
        _check(lib().femgpu_set_config(self.h, C.byref(self.cfg)), self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().femgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- operator ---------------------------------------------------------------------
    def set_mesh(self, xyz, conn, labels=None):
        conn = np.ascontiguousarray(conn, dtype=np.int32)
        dim = 3 if conn.shape[1] == 4 else 2
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        if xyz.shape[1] == 2:
            xyz = np.ascontiguousarray(np.concatenate([xyz, np.zeros((xyz.shape[0], 1))], axis=1))
        labels = None if labels is None else np.ascontiguousarray(labels, dtype=np.int32)
        _check(lib().femgpu_set_mesh(self.h, dim, xyz.shape[0], xyz.ravel(), conn.shape[0], conn.ravel(),
                                     _ptr(labels)), self.h)
        self.n = xyz.shape[0]
        self.nelems = conn.shape[0]
        self.dim = dim
        self._labels_keep = labels

    def assemble(self, coef=None, lambda_mass=1.0):
        coef = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        _check(lib().femgpu_assemble(self.h, _ptr(coef), float(lambda_mass)), self.h)

    def assemble_device(self, coef_ptr: int, lambda_mass=0.0):
        """Per-element coefficients in device memory (e.g. tensor.data_ptr())."""
        _check(lib().femgpu_assemble_device(self.h, _vp(coef_ptr), float(lambda_mass)), self.h)

    def load_vector(self, f):
        b = np.zeros(self.n)
        _check(lib().femgpu_load_vector(self.h, np.ascontiguousarray(f, dtype=np.float64), b), self.h)
        return b

    def set_dirichlet(self, mask):
        _check(lib().femgpu_set_dirichlet(self.h, np.ascontiguousarray(mask, dtype=np.uint8)), self.h)

    def set_matrix_csr(self, rowptr, cols, vals):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        _check(lib().femgpu_set_matrix_csr(self.h, rowptr.shape[0] - 1, rowptr,
                                           np.ascontiguousarray(cols, dtype=np.int32),
                                           np.ascontiguousarray(vals, dtype=np.float64)), self.h)
        self.n = rowptr.shape[0] - 1

    def matrix(self):
        n, nnz = C.c_int64(), C.c_int64()
        _check(lib().femgpu_get_matrix(self.h, C.byref(n), C.byref(nnz), None, None, None), self.h)
        rp = np.zeros(n.value + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        v = np.zeros(nnz.value)
        _check(lib().femgpu_get_matrix(self.h, C.byref(n), C.byref(nnz), _ptr(rp), _ptr(ci), _ptr(v)), self.h)
        return rp, ci, v

    # ---- hierarchy ----------------------------------------------------------------------
    def setup(self):
        _check(lib().femgpu_setup(self.h), self.h)

    @property
    def num_levels(self):
        n = C.c_int()
        _check(lib().femgpu_num_levels(self.h, C.byref(n)), self.h)
        return n.value

    def level_info(self, level):
        info = LevelInfo()
        _check(lib().femgpu_get_level_info(self.h, level, C.byref(info)), self.h)
        return dict(n=info.rows, nnz=info.nnz, n_agg=info.aggregates, n_part=info.partitions, nnz_p=info.nnz_p)

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
        _check(lib().femgpu_level_get(self.h, level, *args), self.h)
        return out

    # ---- solve --------------------------------------------------------------------------
    def vcycle(self, r):
        z = np.zeros(self.n)
        _check(lib().femgpu_vcycle(self.h, np.ascontiguousarray(r, dtype=np.float64), z), self.h)
        return z

    def solve(self, b, x0=None, check=True, out=None):
        """Solves A x = b.  x0 is the initial guess (zeros when None); with `out` (a
        contiguous float64 array of n entries holding the initial guess) the solve runs in
        place there, as femgpu_solve does, instead of on a copy."""
        if out is not None:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                    and out.shape == (self.n,)):
                raise ValueError("out must be a C-contiguous float64 array of the operator's size")
            x = out
        else:
            x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        st = SolveStats()
        status = lib().femgpu_solve(self.h, np.ascontiguousarray(b, dtype=np.float64), x, C.byref(st))
        if check and status not in (0,):
            _check(status, self.h)
        return x, dict(status=status, iterations=st.iterations, relres=st.relative_residual,
                       setup_ms=st.setup_ms, solve_ms=st.solve_ms, levels=st.num_levels)

    def solve_device(self, b_ptr: int, x_ptr: int, check=True):
        """Device pointers (e.g. torch tensor.data_ptr()) on the handle's stream."""
        st = SolveStats()
        status = lib().femgpu_solve_device(self.h, _vp(b_ptr), _vp(x_ptr), C.byref(st))
        if check and status != 0:
            _check(status, self.h)
        return dict(status=status, iterations=st.iterations, relres=st.relative_residual,
                    setup_ms=st.setup_ms, solve_ms=st.solve_ms, levels=st.num_levels)

    KERNELS = {0: "spmv_dot_sliced_kernel (FP64 outer SpMV + dot, 32-row slices)", 1: "smooth pre (level 0)",
               2: "smooth post sweeps alone (level 0)", 3: "spmv_lanes R (level 0)", 4: "spmv_lanes P (level 0)",
               5: "smooth post as in the V-cycle (level 0: b - A_out x, sweeps, z, z.r)",
               6: "element kernel (assembly)", 7: "gather_rows_kernel (assembly)"}

    def test_copy_wait_limit(self, polls: int):
        """Failure-detection testing: polls of the smoother's copy wait (negative: default)."""
        _check(lib().femgpu_test_copy_wait_limit(self.h, int(polls)), self.h)

    def profile_kernel(self, which: int, reps: int = 20):
        ms, nb = C.c_double(), C.c_double()
        _check(lib().femgpu_profile_kernel(self.h, which, reps, C.byref(ms), C.byref(nb)), self.h)
        return ms.value, nb.value

    def solve_multi(self, B, X0=None, check=True):
        """Columns of B (n x k, host) with one hierarchy; returns X (n x k) and stats."""
        B = np.asarray(B, dtype=np.float64)
        k = B.shape[1]
        Bc = np.ascontiguousarray(B.T)  # column j contiguous
        Xc = np.zeros_like(Bc) if X0 is None else np.ascontiguousarray(np.asarray(X0, dtype=np.float64).T)
        st = SolveStats()
        status = lib().femgpu_solve_multi(self.h, k, Bc.ravel(), Xc.ravel(), C.byref(st))
        if check and status != 0:
            _check(status, self.h)
        return Xc.T.copy(), dict(status=status, iterations=st.iterations, relres=st.relative_residual,
                                 solve_ms=st.solve_ms)

    def solve_multi_device(self, nrhs: int, b_ptr: int, ldb: int, x_ptr: int, ldx: int, check=True):
        """Device arrays (column j at ptr + j * ld doubles) on the handle's stream."""
        st = SolveStats()
        status = lib().femgpu_solve_multi_device(self.h, nrhs, _vp(b_ptr), ldb, _vp(x_ptr), ldx, C.byref(st))
        if check and status != 0:
            _check(status, self.h)
        return dict(status=status, iterations=st.iterations, relres=st.relative_residual, solve_ms=st.solve_ms)

    def adjoint_grad(self, dLdu, u, check=True):
        """dL/dtheta per element for theta = log(coefficients) (host arrays)."""
        ne = self.nelems
        out = np.zeros(ne)
        st = SolveStats()
        status = lib().femgpu_adjoint_grad(self.h, np.ascontiguousarray(dLdu, dtype=np.float64),
                                           np.ascontiguousarray(u, dtype=np.float64), out, C.byref(st))
        if check and status != 0:
            _check(status, self.h)
        return out, dict(status=status, iterations=st.iterations, relres=st.relative_residual,
                         solve_ms=st.solve_ms)

    def adjoint_grad_device(self, dLdu_ptr: int, u_ptr: int, grad_ptr: int, check=False):
        """Device pointers on the handle's stream; returns the status with the statistics."""
        st = SolveStats()
        status = lib().femgpu_adjoint_grad_device(self.h, _vp(dLdu_ptr), _vp(u_ptr), _vp(grad_ptr), C.byref(st))
        if check and status != 0:
            _check(status, self.h)
        return dict(status=status, iterations=st.iterations, relres=st.relative_residual, solve_ms=st.solve_ms)

    def spmv_device(self, x_ptr: int, y_ptr: int):
        _check(lib().femgpu_spmv_device(self.h, _vp(x_ptr), _vp(y_ptr)), self.h)

    def save_hierarchy(self, path: str):
        """Writes the AMG hierarchy of the last setup to `path`."""
        _check(lib().femgpu_save_hierarchy(self.h, os.fsencode(path)), self.h)

    def load_hierarchy(self, path: str, check=True):
        """Reads a hierarchy written for this same operator, in place of setup()."""
        status = lib().femgpu_load_hierarchy(self.h, os.fsencode(path))
        if check:
            _check(status, self.h)
        return status

    def load_vector_device_noalloc(self, f_ptr: int, b_ptr: int, check=True):
        """Device f -> device b on the handle's stream; allocates no device memory."""
        status = lib().femgpu_load_vector_device_noalloc(self.h, _vp(f_ptr), _vp(b_ptr))
        if check:
            _check(status, self.h)
        return status


# ---- file IO -----------------------------------------------------------------------------
def solve_batch(solvers, bs, x0s=None, setup=True, threads=0, check=True):
    """Independent problems at once (femgpu_solve_batch): solvers[i] (distinct handles,
    each with its operator) solves bs[i]; returns the solutions and per-problem stats."""
    k = len(solvers)
    xs = [np.zeros(s.n) if x0s is None else np.array(x0s[i], dtype=np.float64) for i, s in enumerate(solvers)]
    bs = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
    hs = (_vp * k)(*[s.h for s in solvers])
    pb = (_vp * k)(*[b.ctypes.data for b in bs])
    px = (_vp * k)(*[x.ctypes.data for x in xs])
    st = (SolveStats * k)()
    status = lib().femgpu_solve_batch(k, hs, pb, px, 1 if setup else 0, threads, st)
    if check and status != 0:
        bad = next((s.h for s in solvers if lib().femgpu_last_error(s.h)), None)
        _check(status, bad)
    stats = [dict(iterations=t.iterations, relres=t.relative_residual, setup_ms=t.setup_ms, solve_ms=t.solve_ms,
                  levels=t.num_levels) for t in st]
    return xs, stats, status


def read_tetgen(base: str):
    node, ele = (base + ".node").encode(), (base + ".ele").encode()
    nv, ne = C.c_int64(), C.c_int64()
    _check(lib().femgpu_read_tetgen(node, ele, C.byref(nv), C.byref(ne), None, None, None))
    xyz = np.zeros(nv.value * 3)
    conn = np.zeros(ne.value * 4, np.int32)
    lab = np.zeros(ne.value, np.int32)
    _check(lib().femgpu_read_tetgen(node, ele, C.byref(nv), C.byref(ne), _ptr(xyz), _ptr(conn), _ptr(lab)))
    return xyz.reshape(-1, 3), conn.reshape(-1, 4), lab


def read_ply(path: str):
    nv, nf = C.c_int64(), C.c_int64()
    _check(lib().femgpu_read_ply(path.encode(), C.byref(nv), C.byref(nf), None, None))
    xyz = np.zeros(nv.value * 3)
    conn = np.zeros(nf.value * 3, np.int32)
    _check(lib().femgpu_read_ply(path.encode(), C.byref(nv), C.byref(nf), _ptr(xyz), _ptr(conn)))
    return xyz.reshape(-1, 3), conn.reshape(-1, 3)


def read_mat_sparse(path: str):
    r, c, nnz = C.c_int64(), C.c_int64(), C.c_int64()
    _check(lib().femgpu_read_mat_sparse(path.encode(), C.byref(r), C.byref(c), C.byref(nnz), None, None, None))
    rp = np.zeros(r.value + 1, np.int32)
    ci = np.zeros(nnz.value, np.int32)
    v = np.zeros(nnz.value)
    _check(lib().femgpu_read_mat_sparse(path.encode(), C.byref(r), C.byref(c), C.byref(nnz), _ptr(rp), _ptr(ci),
                                        _ptr(v)))
    return rp, ci, v, (r.value, c.value)


def read_mat_array(path: str):
    n = C.c_int64()
    _check(lib().femgpu_read_mat_array(path.encode(), C.byref(n), None))
    v = np.zeros(n.value)
    _check(lib().femgpu_read_mat_array(path.encode(), C.byref(n), _ptr(v)))
    return v


def write_mat_array(path: str, v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    _check(lib().femgpu_write_mat_array(path.encode(), v.shape[0], v))


def write_vtk(path: str, xyz, conn, values=None):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    values = None if values is None else np.ascontiguousarray(values, dtype=np.float64)
    dim = 3 if conn.shape[1] == 4 else 2
    _check(lib().femgpu_write_vtk(path.encode(), dim, xyz.shape[0], xyz.ravel(), conn.shape[0], conn.ravel(),
                                  _ptr(values)))
