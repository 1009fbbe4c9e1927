"""The C++ FEMSolver drop-in, compiled against include/ and libfemgpu.so, running the
reference's own end-to-end tests (src/test/*.cc) unchanged in form."""
import os
import subprocess

import pytest

from conftest import REF_DATA, ROOT
from femgpu import capi

pytestmark = pytest.mark.gpu


def test_reference_sanity_programs(tmp_path):
    lib = capi.native_library_path()
    exe = str(tmp_path / "reference_sanity")
    src = os.path.join(ROOT, "tests", "cpp", "reference_sanity.cpp")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, lib, "-o", exe,
           f"-Wl,-rpath,{os.path.dirname(lib)}"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe, REF_DATA], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
