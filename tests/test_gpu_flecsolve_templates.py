"""flecsolve's own, unmodified solver templates (cg.hh with the flexible CG,
bicgstab.hh, gmres.hh) running on the GPU over the device Data/Operations
policy and device CSR operator of include/flecsolve_gb300/flecsolve_device.hh
(tests/cpp/test_flecsolve_templates.cc), against the fixtures the same
templates produced over the reference's serial vectors.

The program is built where a flecsolve checkout is staged (baseline/_ref);
without one these tests are skipped.  Bars: the same status, iterations
within +-2, the first residual norms handed to the diagnostic within 1e-10,
the CG solution within 1e-10 of the reference's; the flexible CG, BiCGSTAB
and GMRES forward error within 2x the reference's own (the flexible CG's
one-step truncation amplifies the rounding of its dot products: without a
preconditioner two correct runs that differ only in summation order end
1.5e-9 apart at 16^3)."""
import json
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

import pyoracle as O
from flecsolve_gb300 import build
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "golden.json").read_text())


@pytest.fixture(scope="module")
def program():
    build.build_gpu()
    exe = build.build_template_test()
    if exe is None:
        pytest.skip("no flecsolve checkout staged in baseline/_ref")
    return exe


def _run(exe, A, b, x0, method, maxiter, rtol, zero_guess, precond, gm=None):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        O.write_problem(fin, A, b, np.zeros(A.nrows) if x0 is None else x0)
        args = [str(exe), fin, fout, method, str(maxiter), repr(float(rtol)),
                str(int(bool(zero_guess))), precond]
        if gm:
            args += [str(gm[0]), gm[1], str(int(gm[2]))]
        r = subprocess.run(args, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        raw = open(fout, "rb").read()
    head = np.frombuffer(raw, np.int32, 3, 0)
    nh = int(np.frombuffer(raw, np.int64, 1, 32)[0])
    hist = np.frombuffer(raw, np.float64, nh, 40).copy()
    x = np.frombuffer(raw, np.float64, A.nrows, 40 + 8 * nh).copy()
    return O.STATUS.get(int(head[0]), str(head[0])), int(head[1]), int(head[2]), hist, x


@pytest.mark.parametrize("name", sorted(META["cases"]))
def test_reference_templates_on_device(program, name):
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    kw = dict(c["kwargs"])
    x0 = P.uniform(int(c["x0"][1]), A.nrows, 0.0, 1.0) if c["x0"] else None
    inner = kw.pop("inner_iters", 0)
    precond = f"cg{inner}" if inner else kw.pop("precond", "jacobi")
    gm = None
    if c["method"] == "gmres":
        gm = (kw.get("krylov_dim", 30), kw.get("side", "right"), kw.get("restart", True))
    status, iters, restarts, hist, x = _run(
        program, A, b, x0, c["method"], kw.get("maxiter", 2000), kw.get("rtol", 1e-8),
        kw.get("use_zero_guess", True), precond, gm)
    g = np.load(GOLD / f"{name}.npz")
    assert status == c["status"]
    assert abs(iters - c["iters"]) <= 2
    k = min(5, hist.size, g["hist"].size)
    assert np.allclose(hist[:k], g["hist"][:k], rtol=1e-10, atol=0)
    if c["status"] != "converged_rtol":
        return
    if c["method"] == "cg":
        assert np.linalg.norm(x - g["x"]) <= 1e-10 * np.linalg.norm(g["x"])
    else:
        import scipy.sparse.linalg as spla
        xs = spla.spsolve(A.to_scipy().tocsc(), b)
        e = np.linalg.norm(x - xs) / np.linalg.norm(xs)
        e_ref = np.linalg.norm(g["x"] - xs) / np.linalg.norm(xs)
        assert e <= 2.0 * e_ref + 1e-12
