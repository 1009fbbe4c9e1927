"""AMG hierarchy written to a file and read back in place of setup (needs a GB300).

A handle that loads the hierarchy of another handle with the same operator must solve
bit-identically to it; a file for another operator, another precision, or a damaged file
is refused."""
import numpy as np
import pytest

import femgpu
from femgpu import meshes

pytestmark = pytest.mark.gpu


def make(n=10, sigma=2.0, precision=0, kappa_seed=2):
    xyz, conn, kappa, f, mask = meshes.poisson3d_problem(n, sigma=sigma, kappa_seed=kappa_seed)
    s = femgpu.Solver(solverType=1, tolerance=1e-10, maxIters=500, flexibleCG=1, seed=4, precision=precision)
    s.set_mesh(xyz, conn)
    s.assemble(kappa, 0.0)
    s.set_dirichlet(mask)
    b = np.where(mask.astype(bool), 0.0, s.load_vector(f))
    return s, b


@pytest.mark.parametrize("precision", [0, 1])
def test_loaded_hierarchy_solves_identically(tmp_path, precision):
    path = str(tmp_path / "h.bin")
    a, b = make(precision=precision)
    a.setup()
    xa, sta = a.solve(b)
    a.save_hierarchy(path)
    c, b2 = make(precision=precision)
    c.load_hierarchy(path)
    assert c.num_levels == a.num_levels
    xc, stc = c.solve(b2)
    assert np.array_equal(xa, xc) and sta["iterations"] == stc["iterations"]
    for l in range(a.num_levels - 1):
        la, lc = a.level(l), c.level(l)
        for k in ("perm", "agg_idx", "part_idx", "P_rowptr", "P_cols", "P_vals", "A_vals"):
            assert np.array_equal(la[k], lc[k]), (l, k)


def test_load_refuses_other_operator_precision_and_damage(tmp_path):
    path = str(tmp_path / "h.bin")
    a, b = make(n=8)
    a.setup()
    a.save_hierarchy(path)
    other, _ = make(n=8, kappa_seed=3)  # same pattern, other coefficients
    assert other.load_hierarchy(path, check=False) == 1  # FEMGPU_ERR_INVALID
    fp64, _ = make(n=8, precision=1)
    assert fp64.load_hierarchy(path, check=False) == 1
    data = open(path, "rb").read()
    cut = tmp_path / "cut.bin"
    cut.write_bytes(data[: len(data) // 2])
    same, b2 = make(n=8)
    assert same.load_hierarchy(str(cut), check=False) == 7  # FEMGPU_ERR_IO
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"not a hierarchy" * 10)
    assert same.load_hierarchy(str(junk), check=False) == 7
    assert same.load_hierarchy(str(tmp_path / "missing.bin"), check=False) == 7
    # the handle is still usable: a good file, then a solve equal to the writer's
    same.load_hierarchy(path)
    x1, _ = same.solve(b2)
    x0, _ = a.solve(b)
    assert np.array_equal(x0, x1)


def file_checksum(payload: bytes) -> int:
    """The file's trailing checksum (hierarchy_io.cu payload_checksum), restated."""
    P, M = 0x100000001B3, (1 << 64) - 1
    h = [0xCBF29CE484222325 ^ l for l in range(4)]
    n = len(payload)
    words = np.frombuffer(payload[: n // 32 * 32], dtype=np.uint64).reshape(-1, 4)
    for row in words:
        for l in range(4):
            h[l] = ((h[l] ^ int(row[l])) * P) & M
    for c in payload[n // 32 * 32:]:
        h[0] = ((h[0] ^ c) * P) & M
    out = (n * P) & M
    for l in range(4):
        out = (((out ^ h[l]) * P) & M) ^ (h[l] >> 29)
    return out


def level0_in_partition_columns(data: bytes, value_size: int):
    """Byte offset and count of level 0's in-partition column array: the fields before it
    in the file's order (magic, header, level scalars, A, graph, permutations, Ap, Ain)."""
    pos = 8 + 4 + 4 + 8 + 8 + 8 + 4  # magic, version, precision, n, nnz, fingerprint, level count
    pos += 4 + 4 + 4 + 1  # n, nagg, npart, coarsest

    def buf(pos, elem):
        count = int(np.frombuffer(data[pos:pos + 8], dtype=np.uint64)[0])
        return pos + 8 + count * elem, pos + 8, count

    def csr(pos):
        pos += 4 + 4 + 8
        pos, _, _ = buf(pos, 4)
        ci_end, ci_at, ci_n = buf(pos, 4)
        end, _, _ = buf(ci_end, value_size)
        return end, ci_at, ci_n

    pos, _, _ = csr(pos)  # A
    pos, _, _ = buf(pos, 4)  # gxadj
    pos, _, _ = buf(pos, 4)  # gadj
    pos += 8  # gnnz
    for _ in range(5):  # perm, iperm, agg_idx, part_idx, agg_of
        pos, _, _ = buf(pos, 4)
    pos, _, _ = csr(pos)  # Ap
    _, ci_at, ci_n = csr(pos)  # Ain
    return ci_at, ci_n


def test_load_refuses_damaged_payload_before_any_upload(tmp_path):
    path = tmp_path / "h.bin"
    a, b = make(n=8)
    a.setup()
    a.save_hierarchy(str(path))
    data = bytearray(path.read_bytes())
    assert file_checksum(bytes(data[:-8])) == int(np.frombuffer(bytes(data[-8:]), dtype=np.uint64)[0])
    same, b2 = make(n=8)
    # one flipped byte behind a valid header: the checksum refuses it
    flipped = bytearray(data)
    flipped[len(data) // 2] ^= 0x40
    bad = tmp_path / "flipped.bin"
    bad.write_bytes(bytes(flipped))
    assert same.load_hierarchy(str(bad), check=False) == 7  # FEMGPU_ERR_IO
    # a column index out of range with a recomputed checksum: the structure check refuses it
    at, count = level0_in_partition_columns(bytes(data), 4)
    assert count > 0
    broken = bytearray(data)
    broken[at:at + 4] = np.array([10**9], dtype=np.int32).tobytes()
    broken[-8:] = np.array([file_checksum(bytes(broken[:-8]))], dtype=np.uint64).tobytes()
    bad2 = tmp_path / "structure.bin"
    bad2.write_bytes(bytes(broken))
    assert same.load_hierarchy(str(bad2), check=False) == 7
    assert "corrupt hierarchy file" in femgpu.capi.lib().femgpu_last_error(same.h).decode()
    # nothing of the refused files stayed: the good file loads and solves as the writer does
    same.load_hierarchy(str(path))
    x1, _ = same.solve(b2)
    x0, _ = a.solve(b)
    assert np.array_equal(x0, x1)
