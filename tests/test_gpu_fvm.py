"""Finite-volume physics operators on the device against the reference.

* The operators on fields (boundary operators, face-coefficient setters,
  diffusion) give the reference's fields bit for bit on every golden case
  (tests/golden/fvm_*.npz, from the reference's own operators).
* The matrix-free operator (the expression on vectors of logical cells)
  gives the reference's v bit for bit in FP64 (golden cases with a boundary
  operator on every face and a linear coefficient, and a 128^3 mesh against
  the oracle), FP32 within 2e-6 relative.
* CG over the matrix-free operator against the reference's CG over the
  reference's expression (the equilibrium-diffusion example and a 3-D
  field-coefficient case): status, iteration count within +-2, the first
  residuals of the history to 1e-9, the solution to 1e-6.
* Jacobi PCG and the mixed-precision CG over the matrix-free operator
  against the same solves over the operator assembled as a CSR matrix; the
  Jacobi diagonal against the assembled diagonal.
* Calls that need stored values refuse the matrix-free operator."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

import flecsolve_gb300 as fs
import fvm_oracle as O
from flecsolve_gb300 import physics as ph
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "fvm_golden.json").read_text())
ITER_TOL = 2


def _bits(x):
    return np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)


def _spec(kind, value):
    return ph.dirichlet(value) if kind == O.DIRICHLET else ph.neumann(value)


def _build(ctx, m, z):
    mesh = ph.fvm_mesh(ctx, m["n"], m["box"])
    u, a = mesh.cell_field(z["u"]), mesh.cell_field(z["a"])
    faces = mesh.face_fields([z["bx"], z["by"], z["bz"]])
    bcs = [ph.bc(_spec(k, val), f // 2, f % 2) for f, (k, val) in enumerate(zip(m["bc_kind"], m["bc_value"]))
           if k != 0]
    ops = [ph.op_expr(*bcs)]
    if m["coef_kind"] == 1:
        ops.append(ph.coefficient(ph.constant_coefficient(m["coef_value"]), faces))
    elif m["coef_kind"] == 2:
        ops.append(ph.coefficient(ph.average_coefficient(), faces))
    ops.append(ph.diffusion(mesh, a, faces, m["beta"], m["alpha"]))
    return mesh, u, a, faces, ph.op_expr(*ops)


@pytest.mark.parametrize("name", sorted(META["apply"]))
def test_field_operators_match_reference(ctx, name):
    m = META["apply"][name]
    z = np.load(GOLD / f"fvm_{name}.npz")
    mesh, u, _, faces, expr = _build(ctx, m, z)
    v = mesh.cell_field(z["v"])
    expr.apply(u, v)
    shp_c, shp_f = mesh.cell_shape, mesh.face_shape
    assert np.array_equal(_bits(u.numpy().reshape(shp_c)), _bits(z["u_out"]))
    for k, ax in enumerate("xyz"):
        assert np.array_equal(_bits(faces[k].numpy().reshape(shp_f)), _bits(z[f"b{ax}_out"]))
    assert np.array_equal(_bits(v.numpy().reshape(shp_c)), _bits(z["v_out"]))


MF_CASES = [n for n, m in sorted(META["apply"].items()) if all(m["bc_kind"]) and m["coef_kind"] != 2]


@pytest.mark.parametrize("name", MF_CASES)
def test_matrix_free_matches_reference(ctx, name):
    m = META["apply"][name]
    z = np.load(GOLD / f"fvm_{name}.npz")
    mesh, _, _, _, expr = _build(ctx, m, z)
    A = expr.matrix_free()
    x = O.logical(z["u"])
    want = O.logical(z["v_out"])
    y = fs.Vector(ctx, x.size)
    A.apply(fs.Vector(ctx, x), y)
    assert np.array_equal(_bits(y.numpy()), _bits(want))
    # the packed field gives the same vector
    assert np.array_equal(mesh.pack(mesh.cell_field(z["u"])).numpy(), x)
    # FP32
    y32 = fs.Vector(ctx, x.size, "f32")
    A.apply(fs.Vector(ctx, x.astype(np.float32), "f32"), y32)
    err = np.linalg.norm(y32.numpy().astype(np.float64) - want) / np.linalg.norm(want)
    assert err < 2e-6
    aff, n = ph.operator_info(A)
    assert n == tuple(m["n"]) and aff == any(v != 0.0 for v in m["bc_value"])


def test_matrix_free_full_size_against_oracle(ctx):
    """a 128^3 mesh with log-normal face coefficients, mixed boundaries and a
    cell term: identical bit for bit to the oracle"""
    n = (128, 128, 128)
    box = [[0.0, 1.0], [0.0, 2.0], [0.0, 0.5]]
    rng = np.random.default_rng(7)
    b = [np.exp(rng.normal(size=O.face_fields(n)[0].shape)) for _ in range(3)]
    a = np.exp(rng.normal(size=O.cell_field(n).shape))
    kinds = [O.DIRICHLET, O.NEUMANN, O.NEUMANN, O.DIRICHLET, O.DIRICHLET, O.NEUMANN]
    vals = [0.5, -1.0, 0.25, 2.0, -0.75, 1.5]
    x = rng.normal(size=n[0] * n[1] * n[2])
    want = O.matrix_free_apply(n, box, 0.9, 1.1, kinds, vals, a, b, x)
    mesh = ph.fvm_mesh(ctx, n, box)
    faces = mesh.face_fields(b)
    expr = ph.op_expr(*[ph.bc(_spec(k, v), f // 2, f % 2) for f, (k, v) in enumerate(zip(kinds, vals))],
                      ph.diffusion(mesh, mesh.cell_field(a), faces, 0.9, 1.1))
    A = expr.matrix_free()
    y = fs.Vector(ctx, x.size)
    A.apply(fs.Vector(ctx, x), y)
    assert np.array_equal(_bits(y.numpy()), _bits(want))


@pytest.mark.parametrize("n", [(40, 9, 17), (33, 8, 1), (64, 3, 20)])
@pytest.mark.parametrize("faces_as_fields", [True, False])
def test_matrix_free_plane_marching_against_oracle(ctx, n, faces_as_fields):
    """meshes at least a warp wide take the plane-marching kernel: partial x
    and y tiles, a partial last z chunk, one-plane meshes, every boundary kind,
    face fields or a constant, a cell term; FP64 bit for bit, FP32 to 2e-6"""
    box = [[0.0, 2.0], [0.0, 1.0], [-1.0, 1.0]]
    rng = np.random.default_rng(sum(n))
    b = [np.exp(rng.normal(size=O.face_fields(n)[0].shape)) for _ in range(3)] if faces_as_fields else None
    a = np.exp(rng.normal(size=O.cell_field(n).shape))
    kinds = [O.NEUMANN, O.DIRICHLET, O.DIRICHLET, O.NEUMANN, O.NEUMANN, O.DIRICHLET]
    vals = [0.25, -0.5, 1.0, 0.0, 2.0, -1.5]
    x = rng.normal(size=n[0] * n[1] * n[2])
    want = O.matrix_free_apply(n, box, 1.2, 0.3, kinds, vals, a, b, x, b_value=2.5)
    mesh = ph.fvm_mesh(ctx, n, box)
    faces = mesh.face_fields(b if faces_as_fields else 0.0)
    ops = [ph.bc(_spec(k, v), f // 2, f % 2) for f, (k, v) in enumerate(zip(kinds, vals))]
    if not faces_as_fields:
        ops.append(ph.coefficient(ph.constant_coefficient(2.5), faces))
    ops.append(ph.diffusion(mesh, mesh.cell_field(a), faces, 1.2, 0.3))
    A = ph.op_expr(*ops).matrix_free()
    y = fs.Vector(ctx, x.size)
    A.apply(fs.Vector(ctx, x), y)
    assert np.array_equal(_bits(y.numpy()), _bits(want))
    y32 = fs.Vector(ctx, x.size, "f32")
    A.apply(fs.Vector(ctx, x.astype(np.float32), "f32"), y32)
    assert np.linalg.norm(y32.numpy() - want) / np.linalg.norm(want) < 2e-6
    # the residual epilogue through the same kernel
    bb = rng.normal(size=x.size)
    vb, vx, rv = fs.Vector(ctx, bb), fs.Vector(ctx, x), fs.Vector(ctx, x.size)
    fs.api.check(fs.api.lib().fs_csr_residual(A.h, vb.h, vx.h, rv.h), ctx.h)
    assert np.allclose(rv.numpy(), bb - want, rtol=0, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("name", sorted(META["cg"]))
def test_cg_matches_reference(ctx, name):
    m = META["cg"][name]
    z = np.load(GOLD / f"fvm_{name}.npz")
    _, _, _, _, expr = _build(ctx, m, z)
    A = expr.matrix_free()
    hist = []

    def diag(x, r):
        hist.append(r)
        return False

    vb, vx = fs.Vector(ctx, z["rhs"]), fs.Vector(ctx, z["x0"])
    s = fs.cg.settings(maxiter=m["maxiter"], rtol=m["rtol"], use_zero_guess=m["zero_guess"])
    info = fs.cg.solver(s, fs.cg.make_work(vb))(fs.op.ref(A), fs.op.I, diag)(vb, vx)
    assert info.status == "converged_rtol"
    assert abs(info.iters - m["iters"]) <= ITER_TOL
    k = min(5, len(hist), len(z["hist"]))
    assert np.allclose(hist[:k], z["hist"][:k], rtol=1e-9, atol=0)
    x = vx.numpy()
    if np.linalg.norm(z["rhs"]) > 0:
        assert np.linalg.norm(x - z["x"]) / np.linalg.norm(z["x"]) < 1e-6
    else:
        # the example's homogeneous right-hand side: both solutions are within
        # the stopping tolerance of the boundary value
        assert np.abs(x - z["x"]).max() < 1e-5


def _assembled(n, box, beta, alpha, kinds, a, b):
    N = n[0] * n[1] * n[2]
    cols = [O.matrix_free_apply(n, box, beta, alpha, kinds, [0.0] * 6, a, b, e) for e in np.eye(N)]
    return sp.csr_matrix(np.stack(cols, 1))


def test_pcg_and_mixed_cg_matrix_free_vs_assembled(ctx):
    n = (12, 10, 9)
    box = [[0.0, 1.0]] * 3
    rng = np.random.default_rng(9)
    b = [np.exp(rng.normal(size=O.face_fields(n)[0].shape)) for _ in range(3)]
    a = np.exp(rng.normal(size=O.cell_field(n).shape))
    kinds = [O.DIRICHLET, O.DIRICHLET, O.NEUMANN, O.NEUMANN, O.DIRICHLET, O.NEUMANN]
    beta, alpha = 1.0, 0.05
    M = _assembled(n, box, beta, alpha, kinds, a, b)
    M.eliminate_zeros()
    M.sort_indices()
    mesh = ph.fvm_mesh(ctx, n, box)
    expr = ph.op_expr(*[ph.bc(_spec(k, 0.0), f // 2, f % 2) for f, k in enumerate(kinds)],
                      ph.diffusion(mesh, mesh.cell_field(a), mesh.face_fields(b), beta, alpha))
    A = expr.matrix_free()
    dC = fs.CSR(ctx, P.CSR(M.shape[0], M.shape[1], M.indptr.astype(np.int64), M.indices.astype(np.int32),
                           M.data.astype(np.float64)))
    N = M.shape[0]
    # the Jacobi diagonal
    d_mf, d_csr = fs.Vector(ctx, N), fs.Vector(ctx, N)
    fs.api.lib().fs_csr_diag_inv(A.h, d_mf.h)
    fs.api.lib().fs_csr_diag_inv(dC.h, d_csr.h)
    assert np.allclose(d_mf.numpy(), d_csr.numpy(), rtol=1e-13, atol=0)
    rhs = rng.uniform(-1.0, 1.0, N)
    vb = fs.Vector(ctx, rhs)
    out = {}
    for key, op in (("mf", A), ("csr", dC)):
        for name, ns in (("cg", fs.cg), ("mixed", fs.mixed_cg)):
            vx = fs.Vector(ctx, N)
            slv = ns.solver(ns.settings(maxiter=2000, rtol=1e-8), ns.make_work(vb))(fs.op.ref(op), fs.op.jacobi)
            info = slv(vb, vx)
            out[key, name] = (info, vx.numpy())
    xs = sp.linalg.spsolve(M.tocsc(), rhs)
    iters = {k: v[0].iters for k, v in out.items()}
    for k, (info, x) in out.items():
        assert info.status == "converged_rtol", k
        assert np.linalg.norm(M @ x - rhs) / np.linalg.norm(rhs) <= 1e-8 * 1.01, k
        assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-6, k
    vals = list(iters.values())
    assert max(vals) - min(vals) <= ITER_TOL, iters


def test_matrix_free_refuses_matrix_calls(ctx):
    mesh = ph.fvm_mesh(ctx, (4, 4, 4))
    faces = mesh.face_fields(1.0)
    expr = ph.op_expr(*[ph.bc(ph.dirichlet(0.0), f // 2, f % 2) for f in range(6)],
                      ph.diffusion(mesh, mesh.cell_field(1.0), faces))
    A = expr.matrix_free()
    for call in (lambda: A.index_coding("colids"),
                 lambda: fs.api.check(fs.api.lib().fs_csr_spmv_transpose(A.h, fs.Vector(ctx, 64).h,
                                                                          fs.Vector(ctx, 64).h), ctx.h)):
        with pytest.raises(Exception):
            call()
    # an expression without a boundary operator on every face, or with an
    # average coefficient, has no matrix-free form
    with pytest.raises(ValueError):
        ph.op_expr(ph.bc(ph.dirichlet(0.0), 0, 0), ph.diffusion(mesh, mesh.cell_field(1.0), faces)).matrix_free()
    with pytest.raises(ValueError):
        ph.op_expr(*[ph.bc(ph.dirichlet(0.0), f // 2, f % 2) for f in range(6)],
                   ph.coefficient(ph.average_coefficient(), faces),
                   ph.diffusion(mesh, mesh.cell_field(1.0), faces)).matrix_free()
