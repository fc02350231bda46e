"""NKA (flecsolve/solvers/nka.hh) on device vectors against the reference's
own NKA, run by tests/golden/make_nka_golden.py with its CG solver as the
preconditioner (solvers/test/nka.cc:72-80: b = 1, x0 = 3, nka.cfg settings).

Bars: the same stop reason; iteration counts within +-2 (the device dots are
tree reductions, the reference's are serial); the residual history handed to
the diagnostic follows the reference's to 1e-6 relative over its first ten
iterations; converged solutions within 1e-6 of the reference's; a run that
exhausts maxiter reports status unknown and iters 0, as the reference's does."""
import json
from pathlib import Path

import numpy as np
import pytest

import flecsolve_gb300 as fs
from flecsolve_gb300 import _lib
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "nka_golden.json").read_text())["cases"]


def _solve(ctx, c, diag=None):
    A, _ = P.workload(c["workload"])
    b = np.ones(A.nrows)
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, np.full(A.nrows, 3.0))
    pc_maxiter, pc_rtol = c["pc"]
    pre = fs.cg.solver(fs.cg.settings(maxiter=pc_maxiter, rtol=pc_rtol, atol=pc_rtol,
                                      use_zero_guess=True), fs.cg.make_work(vb))(dA)
    maxiter, atol, max_dim, angle_tol = c["nka"]
    damp = c["damping"] or (0, 0, 1.0)
    s = fs.nka.settings(maxiter=maxiter, atol=atol, max_dim=max_dim, angle_tol=angle_tol,
                        use_zero_guess=False, use_damping=bool(damp[0]),
                        adaptive_damping=bool(damp[1]), damping_factor=damp[2])
    slv = fs.nka.solver(s, fs.nka.make_work(vb, 10))(dA, pre, diag)
    info = slv(vb, vx)
    return A, b, info, vx.numpy()


@pytest.mark.parametrize("name", sorted(META))
def test_nka_against_reference(ctx, name):
    c = META[name]
    g = np.load(GOLD / f"nka_{name}.npz")
    hist = []
    A, b, info, x = _solve(ctx, c, lambda xv, r: hist.append(r) or False)
    ref_status = _lib.STOP_REASONS[c["status"]]
    assert info.status == ref_status
    hist = np.array(hist)
    k = min(10, len(g["hist"]))
    assert np.allclose(hist[:k], g["hist"][:k], rtol=1e-6, atol=0), (hist[:k], g["hist"][:k])
    if ref_status == "unknown":
        assert info.iters == 0 and len(hist) == c["nka"][0]
        return
    assert abs(info.iters - c["iters"]) <= 2, (info.iters, c["iters"])
    true_res = np.linalg.norm(A.to_scipy() @ x - b)
    assert true_res < c["nka"][1] * 1.001
    assert np.linalg.norm(x - g["x"]) <= 1e-6 * np.linalg.norm(g["x"])


def test_nka_settings_validation(ctx):
    A, _ = P.workload("poisson2d-16")
    dA = fs.CSR(ctx, A)
    for kw, status in ((dict(max_dim=0), _lib.ERR_BREAKDOWN),
                       (dict(max_dim=3, angle_tol=0.0), _lib.ERR_BREAKDOWN),
                       (dict(max_dim=3, adaptive_damping=True), _lib.ERR_BREAKDOWN),
                       (dict(max_dim=3, use_qr=True), _lib.ERR_UNSUPPORTED)):
        with pytest.raises(_lib.FsError) as ei:
            fs.nka.solver(fs.nka.settings(maxiter=10, atol=1e-6, **kw))(dA)
        assert ei.value.status == status, kw


def test_nka_nonlinear_residual(ctx):
    """A nonlinear F(u) = M u + u^3 / 10 (M = the 2-D Laplacian + 2 I) through
    the residual callback, with Jacobi-CG on M as a fixed preconditioner (the
    Jacobian at u = 0)."""
    import scipy.sparse as sp
    A, _ = P.workload("poisson2d-32")
    n = A.nrows
    S = (A.to_scipy() + 2.0 * sp.identity(n)).tocsr()
    S.sort_indices()
    M = P.CSR(n, n, S.indptr.astype(np.int64), S.indices.astype(np.int32), S.data.copy())
    dM = fs.CSR(ctx, M)
    f = np.linspace(-1.0, 1.0, n)

    def residual(fv, uv, rv):  # r = f - F(u)
        u = uv.numpy()
        rv.upload(fv.numpy() - (S @ u + 0.1 * u ** 3))

    vf, vu = fs.Vector(ctx, f), fs.Vector(ctx, n)
    pre = fs.cg.solver(fs.cg.settings(maxiter=30, rtol=1e-6, use_zero_guess=True),
                       fs.cg.make_work(vf))(dM, fs.op.jacobi)
    s = fs.nka.settings(maxiter=60, atol=1e-8, max_dim=6, angle_tol=0.2)
    slv = fs.nka.solver(s)(None, pre, residual=residual, ctx=ctx)
    info = slv(vf, vu)
    assert info.status == "converged_atol" and info.iters < 30
    u = vu.numpy()
    assert np.linalg.norm(f - (S @ u + 0.1 * u ** 3)) < 1e-8
    # the subspace persists across applies (as the reference's does); reset
    # empties it and the same solve repeats exactly
    slv.reset()
    vu2 = fs.Vector(ctx, n)
    info2 = slv(vf, vu2)
    assert info2.iters == info.iters and np.array_equal(vu2.numpy(), u)
