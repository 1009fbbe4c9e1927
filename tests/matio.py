"""Independent numpy reader of the MAT v5 files in tests/golden/reference_data.

Test utility: pins the library's C++ reader and feeds the oracle.  It follows the
layout the reference reads (src/FEMSolver.cu:177-449): 128-byte header, miMATRIX
element, array flags, dimensions, array name (short or long tag), then either
int32 row indices + int32 column offsets + double values (sparse) or doubles.
"""
import struct

import numpy as np


def _tag(buf, off):
    t, n = struct.unpack_from("<II", buf, off)
    if t >> 16:  # small data element: (bytes << 16) | type
        return t & 0xFFFF, t >> 16, off + 4, 4
    return t, n, off + 8, 8


def read(path):
    buf = open(path, "rb").read()
    off = 128
    t, n, off, _ = _tag(buf, off)
    assert t == 14, "not an uncompressed miMATRIX"
    t, n, off, _ = _tag(buf, off)  # array flags
    flags = struct.unpack_from("<I", buf, off)[0]
    off += n
    mclass = flags & 0xFF
    t, n, off, _ = _tag(buf, off)  # dimensions
    dims = struct.unpack_from(f"<{n // 4}i", buf, off)
    off += n + (-n % 8)
    t, n, off, hdr = _tag(buf, off)  # name
    off += n + (-n % hdr if hdr == 4 else -n % 8)
    if mclass == 5:
        t, n, off, _ = _tag(buf, off)
        ir = np.frombuffer(buf, np.int32, n // 4, off)
        off += n + (-n % 8)
        t, n, off, _ = _tag(buf, off)
        jc = np.frombuffer(buf, np.int32, n // 4, off)
        off += n + (-n % 8)
        t, n, off, _ = _tag(buf, off)
        pr = np.frombuffer(buf, np.float64, n // 8, off)
        import scipy.sparse as sp
        nnz = jc[dims[1]]
        A = sp.csc_matrix((pr[:nnz], ir[:nnz], jc[:dims[1] + 1]), shape=(dims[0], dims[1])).tocsr()
        A.sort_indices()
        return A
    t, n, off, _ = _tag(buf, off)
    return np.frombuffer(buf, np.float64, n // 8, off).copy()
