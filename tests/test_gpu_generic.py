"""Solvers over any operator and any preconditioner: caller-defined shell
operators (op::make_shell, flecsolve/operators/shell.hh:26-95) as A and as
P, a general (non-diagonal) CSR preconditioner, a bound solver as the
preconditioner, and the flexible CG (flecsolve/solvers/cg.hh:145-244).

These run the host-stepped loops, which restate the reference's loops over
device vectors.  Bars: against the fixtures the reference produced
(tests/golden/golden.json) and the oracle -- the same status, iterations
within +-2, the CG/FCG solution within 1e-10 of the reference's, BiCGSTAB
and GMRES within the forward-error bar of the fused loops' tests."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "golden.json").read_text())
ITER_TOL = 2


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case(name):
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    g = np.load(GOLD / f"{name}.npz")
    return c, A, b, g


def _dinv(ctx, dA, n):
    d = fs.Vector(ctx, n)
    fs.api.lib().fs_csr_diag_inv(dA.h, d.h)
    return d


def _shell_of(ctx, dA):
    """A shell operator whose callback applies the stored matrix with the
    reference's row arithmetic."""
    calls = []

    def f(x, y):
        calls.append(1)
        dA.apply(x, y, exact=True)
    return fs.op.make_shell(ctx, f, dA.nrows), calls


@pytest.mark.parametrize("name,ns", [("poisson2d-128_cg", fs.cg),
                                     ("diffusion3d-16_cg", fs.cg),
                                     ("diffusion3d-16_bicgstab", fs.bicgstab),
                                     ("convdiff3d-16_gmres30", fs.gmres),
                                     ("diffusion3d-16_gmres_left", fs.gmres)])
def test_shell_operator_as_A(ctx, name, ns):
    c, A, b, g = _case(name)
    dA = fs.CSR(ctx, A)
    shell, calls = _shell_of(ctx, dA)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    kw = dict(maxiter=c["kwargs"].get("maxiter", 2000), rtol=c["kwargs"].get("rtol", 1e-8))
    if ns is fs.gmres:
        kw.update(max_krylov_dim=c["kwargs"].get("krylov_dim", 30), restart=True,
                  pre_side=c["kwargs"].get("side", "right"))
    # D^-1 of A as a diagonal vector (a shell stores no diagonal for Jacobi)
    slv = ns.solver(ns.settings(**kw))(shell, _dinv(ctx, dA, A.nrows))
    info = slv(vb, vx)
    x = vx.numpy()
    assert info.status == c["status"]
    assert abs(info.iters - c["iters"]) <= ITER_TOL
    assert len(calls) >= info.iters
    relres = np.linalg.norm(b - A.to_scipy() @ x) / np.linalg.norm(b)
    if c["kwargs"].get("side") == "left":
        # left preconditioning stops on the preconditioned residual: the
        # true residual is bounded by the reference's own
        ref_relres = np.linalg.norm(b - A.to_scipy() @ g["x"]) / np.linalg.norm(b)
        assert relres <= 2.0 * ref_relres
    else:
        assert relres <= 1e-8 * 1.01
    if ns is fs.cg:
        assert _rel(x, g["x"]) <= 1e-10
    else:
        import scipy.sparse.linalg as spla
        xs = spla.spsolve(A.to_scipy().tocsc(), b)
        assert _rel(x, xs) <= 2.0 * _rel(g["x"], xs) + 1e-12


def _neumann_preconditioner(A):
    """M = 2 D^-1 - D^-1 A D^-1, the first-order Neumann-series approximate
    inverse: symmetric positive definite for these operators and not
    diagonal."""
    S = A.to_scipy()
    Di = sp.diags(1.0 / S.diagonal())
    M = (2.0 * Di - Di @ S @ Di).tocsr()
    M.sort_indices()
    return P.CSR(M.shape[0], M.shape[1], M.indptr.astype(np.int64), M.indices.astype(np.int32),
                 M.data.astype(np.float64))


@pytest.mark.parametrize("wl", ["poisson2d-64", "diffusion3d-12"])
def test_general_csr_preconditioner(ctx, wl):
    A, b = P.workload(wl)
    M = _neumann_preconditioner(A)
    r = O.solve("cg", A, b, maxiter=2000, rtol=1e-8, pmat=M)
    dA, dM = fs.CSR(ctx, A), fs.CSR(ctx, M)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    info = fs.cg.solver(fs.cg.settings(maxiter=2000, rtol=1e-8))(dA, dM)(vb, vx)
    assert info.status == r.status == "converged_rtol"
    assert abs(info.iters - r.iters) <= ITER_TOL
    assert _rel(vx.numpy(), r.x) <= 1e-10
    # and fewer iterations than Jacobi alone (the operator is applied)
    assert info.iters < O.solve("cg", A, b, maxiter=2000, rtol=1e-8).iters


@pytest.mark.parametrize("name", ["poisson2d-128_fcg", "diffusion3d-16_fcg_noprec"])
def test_fcg_against_reference_fixture(ctx, name):
    c, A, b, g = _case(name)
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    prec = fs.op.I if c["kwargs"].get("precond") == "none" else fs.op.jacobi
    info = fs.fcg.solver(fs.fcg.settings(maxiter=2000, rtol=1e-8))(dA, prec)(vb, vx)
    assert info.status == c["status"]
    assert abs(info.iters - c["iters"]) <= ITER_TOL
    # the one-step truncation amplifies the rounding of the dot products
    # (without a preconditioner two runs that differ only in summation order
    # end 1.5e-9 apart): forward error within 2x the reference's own
    import scipy.sparse.linalg as spla
    xs = spla.spsolve(A.to_scipy().tocsc(), b)
    assert _rel(vx.numpy(), xs) <= 2.0 * _rel(g["x"], xs) + 1e-12


def test_fcg_with_a_bound_cg_as_preconditioner(ctx):
    """The nested-solver pattern: a bound Jacobi-PCG (5 iterations, rtol 0,
    zero guess) as FCG's preconditioner, against the reference's fcg over its
    own cg::solver."""
    c, A, b, g = _case("diffusion3d-16_fcg_cg5")
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    inner = fs.cg.solver(fs.cg.settings(maxiter=5, rtol=0.0, use_zero_guess=True))(dA, fs.op.jacobi)
    info = fs.fcg.solver(fs.fcg.settings(maxiter=2000, rtol=1e-8))(dA, inner)(vb, vx)
    assert info.status == c["status"]
    assert abs(info.iters - c["iters"]) <= ITER_TOL
    assert _rel(vx.numpy(), g["x"]) <= 1e-10
    hist = fs.fcg.solver(fs.fcg.settings(maxiter=2000, rtol=1e-8))(dA, inner)
    hist(vb, vx)
    h = hist.history()
    assert h.size == info.iters
    assert np.allclose(h[:5], g["hist"][:5], rtol=1e-9, atol=0)


def test_shell_preconditioner_and_user_diagnostic(ctx):
    """A shell as P (here z = D^-1 r written by the callback) and a user
    diagnostic that stops the solve: the reference's converged_user."""
    A, b = P.workload("poisson2d-64")
    dA = fs.CSR(ctx, A)
    d = _dinv(ctx, dA, A.nrows)

    def pc(r, z):
        z.multiply(d, r)
    Pshell = fs.op.make_shell(ctx, pc, A.nrows)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    seen = []

    def diag(x, res):
        seen.append(res)
        return len(seen) == 7
    slv = fs.cg.solver(fs.cg.settings(maxiter=2000, rtol=1e-8))(dA, Pshell, diag)
    info = slv(vb, vx)
    assert info.status == "converged_user" and info.iters == 7 and len(seen) == 7
    r = O.solve("cg", A, b, maxiter=7, rtol=1e-30)
    assert np.allclose(seen, r.hist[:7], rtol=1e-12, atol=0)


def test_generic_path_errors(ctx):
    A, b = P.workload("poisson2d-16")
    dA = fs.CSR(ctx, A)

    def bad(x, y):
        raise RuntimeError("boom")
    shell = fs.op.make_shell(ctx, bad, A.nrows)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.cg.solver(fs.cg.settings(maxiter=10, rtol=1e-8))(shell)(vb, vx)
    assert ei.value.status == fs.api._lib.ERR_CALLBACK
    assert isinstance(shell.error, RuntimeError)
    good, _ = _shell_of(ctx, dA)
    # Jacobi needs a stored diagonal
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.cg.solver(fs.cg.settings(maxiter=10, rtol=1e-8))(good, fs.op.jacobi)
    assert ei.value.status == fs.api._lib.ERR_INVALID_ARG
    # the mixed-precision loops take stored operators only
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=10, rtol=1e-8))(good)
    assert ei.value.status == fs.api._lib.ERR_UNSUPPORTED
    # the calls that need stored values refuse a shell
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.batch_cg(good, [0, A.nrows], vb, vx, maxiter=10, rtol=1e-8)
    assert ei.value.status == fs.api._lib.ERR_INVALID_ARG
