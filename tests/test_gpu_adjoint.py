"""Adjoint of the device solve: transpose SpMV / transpose solve parity, the
gradient kernels, the torch.autograd binding, and differentiation through
backward-Euler heat stepping with checkpoints.

Finite differences.  The bar is agreement with central finite differences to
<= 1e-6 relative, with step h = 1e-6 |theta_i|.  At these sizes one face
coefficient moves the loss by ~1e-7 of its value, so L(theta + h) - L(theta
- h) formed by subtracting two solved losses would be swamped by the solver
tolerance.  The difference of the two solutions is therefore solved for
directly: A(theta+) x+ = b+ and A(theta-) x- = b- give
    A(theta+) (x+ - x-) = (b+ - b-) - K(c+ - c-) x-
(K is linear in the face coefficients), and then exactly
    L(theta+) - L(theta-) = d . (2 x- + d - 2 t),   d = x+ - x-.
This is the same central difference, evaluated without cancellation."""
import numpy as np
import pytest

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import adjoint as ad
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-6


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _host_transpose(A):
    T = A.to_scipy().T.tocsr()
    T.sort_indices()
    return P.CSR(A.ncols, A.nrows, T.indptr.astype(np.int64), T.indices.astype(np.int32),
                 T.data.astype(np.float64), A.name + "^T")


# ------------------------------------------------------ kernels / views ---

def test_transpose_materialised_and_value_grad_exact(ctx):
    A = P.convdiff3d(12, seed=4)
    dA = fs.CSR(ctx, A)
    T = _host_transpose(A)
    dT = dA.transpose()
    assert (dT.nrows, dT.ncols, dT.nnz()) == (T.nrows, T.ncols, T.nnz)
    assert np.array_equal(dT.values(), T.val)
    x = P.uniform(21, A.nrows)
    y = fs.Vector(ctx, A.nrows)
    dT.apply(fs.Vector(ctx, x), y, exact=True)
    np.testing.assert_array_equal(y.numpy(), O.spmv(T, x))
    # dL/dA_ij = -lam_i x_j on the pattern, bit for bit
    lam = P.uniform(22, A.nrows)
    g = fs.Vector(ctx, A.nnz)
    dA.value_grad(fs.Vector(ctx, lam), fs.Vector(ctx, x), g)
    rows = np.repeat(np.arange(A.nrows), np.diff(A.rowptr))
    np.testing.assert_array_equal(g.numpy(), -lam[rows] * x[A.col])


@pytest.mark.parametrize("dim,n", [(2, 33), (3, 17)])
def test_fv_assemble_matches_generator(ctx, dim, n):
    c = P.faces_lognormal(dim, n, seed=2)
    A = P.assemble_diffusion(dim, n, c)
    dA = fs.CSR(ctx, P.assemble_diffusion(dim, n, P.faces_const(dim, n, 1.0)))
    vc = fs.Vector(ctx, c)
    dA.fv_assemble(dim, n, vc)
    np.testing.assert_array_equal(dA.values(), A.val)
    # backward-Euler operator I + dt K
    dt = 1e-3
    dA.fv_assemble(dim, n, vc, scale=dt, shift=1.0)
    want = dt * A.val
    want[A.col == np.repeat(np.arange(A.nrows), np.diff(A.rowptr))] += 1.0
    np.testing.assert_allclose(dA.values(), want, rtol=4e-16, atol=0)
    # the solver picks up the new values (diagonal and FP32 copy refreshed)
    b = P.uniform(3, A.nrows)
    for ns in (fs.cg, fs.mixed_cg):
        dA.fv_assemble(dim, n, fs.Vector(ctx, P.faces_const(dim, n, 1.0)))
        slv = ns.solver(ns.settings(maxiter=5000, rtol=1e-10))(dA, fs.op.jacobi)
        vx = fs.Vector(ctx, A.nrows)
        slv(fs.Vector(ctx, b), vx)
        dA.fv_assemble(dim, n, vc)
        info = slv(fs.Vector(ctx, b), vx)
        assert info.status == "converged_rtol"
        xs = np.linalg.norm(b - A.to_scipy() @ vx.numpy()) / np.linalg.norm(b)
        assert xs < 1e-9


@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_transpose_solve_nonsymmetric_matches_oracle(ctx, method):
    """A^T x = b through the bound solver on the convection-diffusion
    operator, against the oracle solving the host-transposed matrix."""
    A = P.convdiff3d(16, seed=4)
    T = _host_transpose(A)
    b = P.uniform(3, A.nrows)
    ns = fs.bicgstab if method == "bicgstab" else fs.gmres
    kw = dict(max_krylov_dim=30, restart=True) if method == "gmres" else {}
    slv = ns.solver(ns.settings(maxiter=4000, rtol=1e-10, **kw))(fs.CSR(ctx, A), fs.op.jacobi)
    vx = fs.Vector(ctx, A.nrows)
    info = slv.apply_transpose(fs.Vector(ctx, b), vx)
    assert info.status == "converged_rtol"
    x = vx.numpy()
    ref = O.solve(method, T, b, maxiter=4000, rtol=1e-10, krylov_dim=30, restart=True)
    assert ref.status == "converged_rtol"
    import scipy.sparse.linalg as sla
    exact = sla.spsolve(T.to_scipy().tocsc(), b)
    assert _rel(x, exact) <= max(2 * _rel(ref.x, exact), 1e-11)
    assert np.linalg.norm(b - T.to_scipy() @ x) / np.linalg.norm(b) < 1e-9
    # the forward solve on the same bound solver is unaffected
    info2 = slv(fs.Vector(ctx, b), vx)
    assert info2.status == "converged_rtol"
    assert np.linalg.norm(b - A.to_scipy() @ vx.numpy()) / np.linalg.norm(b) < 1e-9


# -------------------------------------------------------- linear solve ---

def _setup(ctx, n, rtol=1e-13):
    c = P.faces_lognormal(3, n, seed=2)
    b = P.uniform(3, n ** 3)
    system = ad.DiffusionSolve(ctx, 3, n, rtol=rtol)
    system.set_faces(P.faces_lognormal(3, n, seed=7))       # ground-truth field
    xt = fs.Vector(ctx, n ** 3)
    system.solve(fs.Vector(ctx, b), xt)
    return system, c, b, xt.numpy()


def _fd_linear(ctx, system, c, b, t, i):
    """Central difference of L = ||x - t||^2 in coordinate i of (c, b)."""
    nf, n, N = c.size, system.n, b.size
    cm, cp, bm, bp = c, c, b, b
    if i < nf:
        h = 1e-6 * abs(c[i])
        cm, cp = c.copy(), c.copy()
        cm[i] -= h
        cp[i] += h
        step = cp[i] - cm[i]
    else:
        j = i - nf
        h = 1e-6 * abs(b[j])
        bm, bp = b.copy(), b.copy()
        bm[j] -= h
        bp[j] += h
        step = bp[j] - bm[j]
    system.set_faces(cm)
    xm = fs.Vector(ctx, N)
    system.solve(fs.Vector(ctx, bm), xm)
    xm = xm.numpy()
    r = bp - bm
    if i < nf:
        r = r - ad.face_delta_apply(3, n, [i], step, xm)
    system.set_faces(cp)
    d = fs.Vector(ctx, N)
    system.solve(fs.Vector(ctx, r), d)
    d = d.numpy()
    return float(d @ (2 * xm + d - 2 * t)) / step


def _adjoint_grad(ctx, system, c, b, t):
    system.set_faces(c)
    x = fs.Vector(ctx, b.size)
    system.solve(fs.Vector(ctx, b), x)
    xh = x.numpy()
    lam = system.adjoint(fs.Vector(ctx, 2 * (xh - t)), x)
    return np.concatenate([system.gfaces.numpy(), lam.numpy()]), xh


def test_adjoint_gradient_vs_central_fd_128(ctx):
    """128^3 log-normal diffusion, L = ||x - x_target||^2 with x_target from
    the ground-truth field: the gradient in all face coefficients and in b,
    checked on 64 random coordinates (seed 8)."""
    n = 128
    system, c, b, t = _setup(ctx, n)
    g, _ = _adjoint_grad(ctx, system, c, b, t)
    coords = P.randint(8, 64, 0, c.size + b.size - 1)
    errs = []
    for i in coords:
        fd = _fd_linear(ctx, system, c, b, t, int(i))
        errs.append(abs(g[i] - fd) / abs(fd))
    errs = np.array(errs)
    assert (coords >= c.size).any() and (coords < c.size).any()
    assert errs.max() <= FD_RTOL, (errs.max(), np.median(errs))


def test_adjoint_lambda_matches_oracle_solve(ctx):
    """The adjoint vector against the oracle's CPU PCG on A^T (24^3)."""
    n = 24
    system, c, b, t = _setup(ctx, n)
    g, x = _adjoint_grad(ctx, system, c, b, t)
    lam = g[c.size:]
    A = P.assemble_diffusion(3, n, c)
    T = _host_transpose(A)
    ref = O.solve("cg", T, 2 * (x - t), maxiter=20000, rtol=1e-12)
    assert ref.status == "converged_rtol"
    import scipy.sparse.linalg as sla
    exact = sla.spsolve(T.to_scipy().tocsc(), 2 * (x - t))
    assert _rel(lam, exact) <= max(2 * _rel(ref.x, exact), 1e-11)
    # the face gradient from the oracle's lambda
    fa, fb = ad.face_cells(3, n, np.arange(c.size))
    inner = (fa >= 0) & (fb >= 0)
    cc = np.where(fa >= 0, fa, fb)
    gref = np.where(inner, -(ref.x[fa] - ref.x[fb]) * (x[fa] - x[fb]), -ref.x[cc] * x[cc])
    assert _rel(g[: c.size], gref) < 1e-8


def test_torch_autograd_binding(ctx):
    torch = pytest.importorskip("torch")
    n = 16
    system, c, b, t = _setup(ctx, n)
    faces = torch.tensor(c, device="cuda", dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, device="cuda", dtype=torch.float64, requires_grad=True)
    tt = torch.tensor(t, device="cuda", dtype=torch.float64)
    x = ad.LinearSolve().apply(faces, bt, system)
    loss = ((x - tt) ** 2).sum()
    loss.backward()
    g, xh = _adjoint_grad(ctx, system, c, b, t)
    np.testing.assert_allclose(x.detach().cpu().numpy(), xh, rtol=0, atol=1e-14)
    np.testing.assert_allclose(faces.grad.cpu().numpy(), g[: c.size], rtol=1e-10, atol=1e-18)
    np.testing.assert_allclose(bt.grad.cpu().numpy(), g[c.size:], rtol=1e-10, atol=1e-18)
    for i in P.randint(81, 6, 0, c.size + b.size - 1):
        fd = _fd_linear(ctx, system, c, b, t, int(i))
        gt = faces.grad[i].item() if i < c.size else bt.grad[i - c.size].item()
        assert abs(gt - fd) <= FD_RTOL * abs(fd)


# ------------------------------------------------------- heat equation ---

def _heat_fd(ctx, sm, sp, c, u0, target, nsteps, i, dt):
    """Central difference of L = ||u_N - target||^2 in coordinate i of
    (c, u0) by propagating the solution difference through the steps:
    M+ d_{k+1} = d_k - dt K(c+ - c-) u-_{k+1}."""
    nf, n, N = c.size, sm.n, u0.size
    cm, cp, um, up = c, c, u0, u0
    if i < nf:
        h = 1e-6 * abs(c[i])
        cm, cp = c.copy(), c.copy()
        cm[i] -= h
        cp[i] += h
        step = cp[i] - cm[i]
    else:
        j = i - nf
        h = 1e-6 * abs(u0[j])
        um, up = u0.copy(), u0.copy()
        um[j] -= h
        up[j] += h
        step = up[j] - um[j]
    sm.set_faces(cm)
    sp.set_faces(cp)
    u = fs.Vector(ctx, um)
    un = fs.Vector(ctx, N)
    d = fs.Vector(ctx, up - um)
    dn = fs.Vector(ctx, N)
    for _ in range(nsteps):
        sm.solve(u, un)
        u, un = un, u
        if i < nf:
            r = d.numpy() - ad.face_delta_apply(3, n, [i], dt * step, u.numpy())
            d.upload(r)
        sp.solve(d, dn)
        d, dn = dn, d
    uh, dh = u.numpy(), d.numpy()
    return float(dh @ (2 * uh + dh - 2 * target)) / step


def test_heat_backward_euler_adjoint_64(ctx):
    """Backward Euler (I + dt K(c)) u_{k+1} = u_k on 64^3, dt = 1e-3, 200
    steps, differentiated through every step with checkpoints every 20:
    gradients in c and u0 against central differences, and the checkpoint
    interval does not change a bit of the result."""
    n, dt, nsteps = 64, 1e-3, 200
    N = n ** 3
    mk = lambda: ad.DiffusionSolve(ctx, 3, n, rtol=1e-13, scale=dt, shift=1.0)
    system = mk()
    c = P.faces_lognormal(3, n, seed=2)
    u0 = P.uniform(9, N)
    system.set_faces(P.faces_lognormal(3, n, seed=7))
    target = ad.heat_forward(system, u0, nsteps)[0].numpy()
    L, gc, gu = ad.heat_loss_and_grad(system, c, u0, target, nsteps, checkpoint=20)
    L2, gc2, gu2 = ad.heat_loss_and_grad(system, c, u0, target, nsteps, checkpoint=7)
    assert L == L2 and np.array_equal(gc, gc2) and np.array_equal(gu, gu2)
    uN = ad.heat_forward(system, u0, nsteps)[0].numpy()
    assert L == float((uN - target) @ (uN - target))
    g = np.concatenate([gc, gu])
    sm, sp = mk(), mk()
    coords = np.concatenate([P.randint(8, 6, 0, c.size - 1), c.size + P.randint(18, 3, 0, N - 1)])
    for i in coords:
        fd = _heat_fd(ctx, sm, sp, c, u0, target, nsteps, int(i), dt)
        assert abs(g[i] - fd) <= FD_RTOL * abs(fd), (int(i), g[i], fd)
