"""The numpy restatement of the finite-volume physics operators
(oracle/fvm_oracle.py) against the reference.

* The golden fixtures (tests/golden/fvm_*.npz, made by make_fvm_golden.py
  from the reference's own operators compiled as oracle/_ref/ref_fvm): the
  restatement gives the same fields bit for bit.
* The closed forms the reference's own physics tests check
  (physics/test/fvm_diffusion.cc:174-212, fvm_coeff.cc:79-112,
  boundaries.cc:58-80).
* The matrix-free form (the expression on vectors of logical cells) against
  the expression on fields, and its linearity with zero boundary values."""
import json
from pathlib import Path

import numpy as np
import pytest

import fvm_oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "fvm_golden.json").read_text())
UNIT = [[0.0, 1.0]] * 3
TOL = 1.0e-8  # DEFAULT_TOL of physics/test/test_setup.hh:40


def _bits(x):
    return np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", sorted(META["apply"]))
def test_restatement_matches_reference_fixture(name):
    m = META["apply"][name]
    z = np.load(GOLD / f"fvm_{name}.npz")
    u, v, b = z["u"].copy(), z["v"].copy(), [z["bx"].copy(), z["by"].copy(), z["bz"].copy()]
    O.apply_expr(tuple(m["n"]), m["box"], m["beta"], m["alpha"], m["bc_kind"], m["bc_value"],
                 m["coef_kind"], m["coef_value"], u, z["a"], v, b)
    assert np.array_equal(_bits(u), _bits(z["u_out"]))
    for k, ax in enumerate("xyz"):
        assert np.array_equal(_bits(b[k]), _bits(z[f"b{ax}_out"]))
    assert np.array_equal(_bits(v), _bits(z["v_out"]))


def _vol_op(n, beta, alpha, bc_kind, bc_value, coef=1.0, u=1.0):
    uu, a, v, b = O.cell_field(n), O.cell_field(n, 1.0), O.cell_field(n), O.face_fields(n)
    uu[...] = u
    O.apply_expr(n, UNIT, beta, alpha, bc_kind, bc_value, 1, coef, uu, a, v, b)
    return uu, b, v


def test_reference_closed_forms_diffusion():
    n = (8, 8, 8)
    D, N = O.DIRICHLET, O.NEUMANN
    # zero-flux Neumann, x = 1: no flux anywhere
    _, _, v = _vol_op(n, 1.0, 0.0, [N] * 6, [0.0] * 6)
    assert np.abs(v[1:-1, 1:-1, 1:-1]).max() < TOL
    # beta = 0, alpha = 1: the source alpha vol
    _, _, v = _vol_op(n, 0.0, 1.0, [N] * 6, [0.0] * 6)
    vol = O.geometry(n, UNIT)[2]
    assert np.abs(v[1:-1, 1:-1, 1:-1] - vol).max() < TOL
    # Dirichlet 1e-9 sink, x = 1 on the logical cells
    u = O.cell_field(n)
    u[1:-1, 1:-1, 1:-1] = 1.0
    _, _, v = _vol_op(n, 1.0, 0.0, [D] * 6, [1e-9] * 6, u=u)
    L = v[1:-1, 1:-1, 1:-1]
    assert np.abs(L[1:-1, 1:-1, 1:-1]).max() < TOL
    edge = np.ones(L.shape, bool)
    edge[1:-1, 1:-1, 1:-1] = False
    assert (L[edge] < 1.0).all()


def test_reference_closed_forms_coefficients_and_boundaries():
    n = (8, 8, 8)
    u = O.cell_field(n, 1.0)
    for f in range(6):
        O.boundary(u, n, UNIT, f, O.DIRICHLET, 1.0)
    bc_, ba = O.coef_constant(O.face_fields(n), 3.14), O.coef_average(O.face_fields(n), u)
    ranges = [(slice(1, None), slice(1, None), slice(None)), (slice(1, None), slice(None), slice(1, None)),
              (slice(None), slice(1, None), slice(1, None))]
    for k in range(3):
        assert np.all(bc_[k][ranges[k]] == 3.14)
        assert np.all(ba[k][ranges[k]] == 1.0)
    # boundaries.cc: Dirichlet -1 / 1 on x, zero-flux Neumann on y, x = 1
    n = (6, 5, 1)
    u = O.cell_field(n, 1.0)
    O.boundary(u, n, UNIT, 0, O.DIRICHLET, -1.0)
    O.boundary(u, n, UNIT, 1, O.DIRICHLET, 1.0)
    O.boundary(u, n, UNIT, 2, O.NEUMANN, 0.0)
    O.boundary(u, n, UNIT, 3, O.NEUMANN, 0.0)
    assert np.all(u[1:-1, 1:-1, 0] == -1.0) and np.all(u[1:-1, 1:-1, -1] == 1.0)
    assert np.all(u[1:-1, 0, 1:-1] == 1.0) and np.all(u[1:-1, -1, 1:-1] == 1.0)


def test_neumann_flux_matches_a_linear_field():
    """u = s x (x the cell centre along x) with Neumann flux s on both x faces
    and zero flux on the others: the boundary cells continue the line
    (neumann.hh:59-72: u_ghost = u_next - (nd dx) q, nd = +1 low, -1 high),
    so every cell's net flux is zero"""
    n, box, slope = (7, 4, 3), [[0.0, 2.0], [0.0, 1.0], [0.0, 1.0]], 1.75
    dx = O.geometry(n, box)[0][0]
    u = O.cell_field(n)
    u[...] = slope * dx * np.arange(n[0] + 2)[None, None, :]
    kinds, vals = [O.NEUMANN] * 6, [slope, slope, 0.0, 0.0, 0.0, 0.0]
    v = O.cell_field(n)
    b = O.face_fields(n)
    u_in = u.copy()
    O.apply_expr(n, box, 1.0, 0.0, kinds, vals, 1, 2.0, u, O.cell_field(n, 1.0), v, b)
    assert np.allclose(u[1:-1, 1:-1, 0], u_in[1:-1, 1:-1, 0], rtol=0, atol=1e-14)
    assert np.allclose(u[1:-1, 1:-1, -1], u_in[1:-1, 1:-1, -1], rtol=0, atol=1e-14)
    assert np.abs(v[1:-1, 1:-1, 1:-1]).max() < 1e-12


def test_geometry_follows_the_specialization():
    dx, dA, vol, c = O.geometry((8, 4, 2), [[0.0, 1.0], [0.0, 2.0], [-1.0, 1.0]])
    assert dx == [1.0 / 9, 2.0 / 5, 2.0 / 3]
    assert dA[0] == dx[1] * dx[2] and vol == dx[0] * (dx[1] * dx[2])
    assert c[2] == dA[2] * (1.0 / dx[2])


def test_matrix_free_form_and_linearity():
    rng = np.random.default_rng(3)
    n = (5, 4, 3)
    b = [np.exp(rng.normal(size=O.face_fields(n)[0].shape)) for _ in range(3)]
    a = np.exp(rng.normal(size=O.cell_field(n).shape))
    kinds = [O.DIRICHLET, O.NEUMANN, O.DIRICHLET, O.DIRICHLET, O.NEUMANN, O.NEUMANN]
    x, y = rng.normal(size=60), rng.normal(size=60)
    # on a field whose boundary cells hold anything, the boundary operators
    # overwrite them: the same v as from a field of NaN boundary cells
    u = rng.normal(size=O.cell_field(n).shape)
    u[1:-1, 1:-1, 1:-1] = x.reshape(3, 4, 5)
    v = O.cell_field(n)
    O.apply_expr(n, UNIT, 1.5, 0.5, kinds, [0.0] * 6, 0, 0.0, u, a, v, [f.copy() for f in b])
    mf = O.matrix_free_apply(n, UNIT, 1.5, 0.5, kinds, [0.0] * 6, a, b, x)
    assert np.array_equal(mf, O.logical(v))
    # zero boundary values: a linear, symmetric operator
    A = np.stack([O.matrix_free_apply(n, UNIT, 1.5, 0.5, kinds, [0.0] * 6, a, b, e) for e in np.eye(60)], 1)
    assert np.allclose(A @ x, mf, rtol=1e-13, atol=1e-13)
    assert np.allclose(A, A.T, rtol=0, atol=1e-14 * np.abs(A).max())
    assert np.all(np.linalg.eigvalsh(A) > 0)
    mfy = O.matrix_free_apply(n, UNIT, 1.5, 0.5, kinds, [0.0] * 6, a, b, y)
    assert np.allclose(A @ y, mfy, rtol=1e-13, atol=1e-13)


def test_cg_fixtures_are_converged():
    for name, m in META["cg"].items():
        z = np.load(GOLD / f"fvm_{name}.npz")
        assert m["status"] == 1, name
        assert len(z["hist"]) == m["iters"]
        assert z["hist"][-1] < m["rtol"] * max(np.linalg.norm(z["rhs"]), 1.0)
