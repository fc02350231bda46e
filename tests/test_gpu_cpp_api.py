"""The C++ mirror of the reference's API, exercised by tests/cpp/
test_krylov_api.cc (written like the reference's own cg.cc / gmres.cc /
bicgstab.cc / flecsi_vector.cc tests) against the device library."""
import os
import subprocess
from pathlib import Path

import pytest

from flecsolve_gb300 import build

pytestmark = pytest.mark.gpu


def test_cpp_api_program():
    exe = build.build_cpp_tests()
    env = dict(os.environ, FS_MM_FIXTURE=str(Path(__file__).resolve().parent / "golden" / "mm" /
                                             "diffusion3d-6.mtx"))
    r = subprocess.run([str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600, env=env)
    print(r.stdout)
    assert "FAIL" not in r.stdout
    assert r.returncode == 0, r.stdout
    assert r.stdout.count("PASS") >= 20
