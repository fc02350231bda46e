"""ORACLE -- test infrastructure only.

numpy restatement of flecsolve's finite-volume physics operators on one
structured mesh (flecsolve/physics/), and a runner for the reference's own
operators compiled as ``oracle/_ref/ref_fvm`` (``make -C oracle ref``).  Only
``tests/`` and the fixture script under ``tests/golden/`` use this module,
and only as the checker.

Mesh layout (the reference's fvm_narray with boundary depth 1, one color):
a cell field is a (nz+2, ny+2, nx+2) array ([k][j][i]), logical cells 1..n
per axis; a face field (one per axis) is (nz+1, ny+1, nx+1), face f of an
axis between cells f and f+1 of it.  numpy rounds every elementwise
operation on its own (no fused multiply-add), so each function below gives
the reference's values bit for bit when it performs the same operations in
the same order, which the docstrings cite.
"""
from __future__ import annotations

import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_FVM = HERE / "_ref" / "ref_fvm"

DIRICHLET, NEUMANN = 1, 2
FACES = ("x_low", "x_high", "y_low", "y_high", "z_low", "z_high")


def geometry(n, box):
    """Spacing, face areas, volume and flux factors dA * (1 / dx)
    (physics/specializations/fvm_narray.hh:233-289): dx = |hi - lo| /
    (n + 2 - 1); dA and the volume are products folded from the right onto
    1.0."""
    dx = [abs(float(box[a][1]) - float(box[a][0])) / float(int(n[a]) + 2 - 1) for a in range(3)]
    dA = [dx[1] * (dx[2] * 1.0), dx[0] * (dx[2] * 1.0), dx[0] * (dx[1] * 1.0)]
    vol = dx[0] * (dx[1] * (dx[2] * 1.0))
    c = [dA[a] * (1.0 / dx[a]) for a in range(3)]
    return dx, dA, vol, c


def cell_field(n, value=0.0):
    nx, ny, nz = n
    return np.full((nz + 2, ny + 2, nx + 2), value, dtype=np.float64)


def face_fields(n, value=0.0):
    nx, ny, nz = n
    return [np.full((nz + 1, ny + 1, nx + 1), value, dtype=np.float64) for _ in range(3)]


def _face_slices(face):
    """(boundary cells, neighbouring logical cells) of a face, as index tuples
    of a cell field: the other two axes over their logical cells
    (fvm_narray.hh:163-229, full_range with the face axis' boundary range)."""
    inner = slice(1, -1)
    axis, high = face // 2, face % 2 == 1
    b, nb = (-1, -2) if high else (0, 1)
    idx_b, idx_n = [inner, inner, inner], [inner, inner, inner]
    dim = 2 - axis  # array dims are (z, y, x)
    idx_b[dim], idx_n[dim] = b, nb
    return tuple(idx_b), tuple(idx_n)


def boundary(u, n, box, face, kind, value):
    """bc<dirichlet>::apply (physics/boundary/dirichlet.hh:49-63): the
    boundary cells beyond the face get the value; bc<neumann>::apply
    (physics/boundary/neumann.hh:49-74): they get the neighbouring cell's
    value minus (nd dx) q, nd = +1 on a low face and -1 on a high one.  In
    place on the cell field u."""
    ib, inn = _face_slices(face)
    if kind == DIRICHLET:
        u[ib] = value
    elif kind == NEUMANN:
        dx = geometry(n, box)[0][face // 2]
        nd = 1.0 if face % 2 == 0 else -1.0
        u[ib] = u[inn] - (nd * dx) * value
    return u


def coef_constant(b, value):
    """coefficient<constant_coefficient>::apply (volume_diffusion/
    coefficient.hh:84-113): every face of the coefficient range gets the
    value (x faces: logical y, z cells and faces 0..nx, and so on)."""
    b[0][1:, 1:, :] = value
    b[1][1:, :, 1:] = value
    b[2][:, 1:, 1:] = value
    return b


def coef_average(b, u):
    """coefficient<average_coefficient>::apply (coefficient.hh:134-177):
    0.5 * (u_hi + u_lo) of the two cells either side of each face."""
    c = u[1:-1, 1:-1, :]
    b[0][1:, 1:, :] = 0.5 * (c[:, :, 1:] + c[:, :, :-1])
    c = u[1:-1, :, 1:-1]
    b[1][1:, :, 1:] = 0.5 * (c[:, 1:, :] + c[:, :-1, :])
    c = u[:, 1:-1, 1:-1]
    b[2][:, 1:, 1:] = 0.5 * (c[1:, :, :] + c[:-1, :, :])
    return b


def diffusion(n, box, beta, alpha, a, b, u, v):
    """diffusion::apply (volume_diffusion/diffusion.hh:83-193): face fluxes
    (b (dA * (1/dx))) (u_hi - u_lo) (update_flux, :109-161), their
    differences summed x + y then + z (sum_cell_flux, :163-180), and
    v = (-beta) du + (alpha vol a) u on the logical cells (operate,
    :182-192).  v's boundary cells are left as they are."""
    _, _, vol, c = geometry(n, box)
    L = (slice(1, -1),) * 3
    uc = u[L]
    bx, by, bz = b
    fx_hi = bx[1:, 1:, 1:] * c[0] * (u[1:-1, 1:-1, 2:] - uc)
    fx_lo = bx[1:, 1:, :-1] * c[0] * (uc - u[1:-1, 1:-1, :-2])
    fy_hi = by[1:, 1:, 1:] * c[1] * (u[1:-1, 2:, 1:-1] - uc)
    fy_lo = by[1:, :-1, 1:] * c[1] * (uc - u[1:-1, :-2, 1:-1])
    fz_hi = bz[1:, 1:, 1:] * c[2] * (u[2:, 1:-1, 1:-1] - uc)
    fz_lo = bz[:-1, 1:, 1:] * c[2] * (uc - u[:-2, 1:-1, 1:-1])
    du = ((fx_hi - fx_lo) + (fy_hi - fy_lo)) + (fz_hi - fz_lo)
    v[L] = (-beta * du) + (alpha * vol * a[L] * uc)
    return v


def apply_expr(n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a, v, b):
    """op_expr(six boundary operators, coefficient, diffusion).apply(u, v)
    (expressions/operator_expression.hh:68-71): the operators in that order;
    returns (u, b, v) after the apply (all three are updated in place)."""
    for f in range(6):
        boundary(u, n, box, f, bc_kind[f], bc_value[f])
    if coef_kind == 1:
        coef_constant(b, coef_value)
    elif coef_kind == 2:
        coef_average(b, u)
    diffusion(n, box, beta, alpha, a, b, u, v)
    return u, b, v


def logical(field):
    """the logical cells of a cell field as a vector, i fastest"""
    return np.ascontiguousarray(field[1:-1, 1:-1, 1:-1]).reshape(-1)


def matrix_free_apply(n, box, beta, alpha, bc_kind, bc_value, a, b, x, b_value=None, a_value=None):
    """The expression as an operator on a vector of logical cells: x in the
    logical cells of a field, the six boundary operators, the face
    coefficient (fields b, or the constant b_value), diffusion; v's logical
    cells.  ``a`` is a cell field or None with the constant ``a_value``."""
    u = cell_field(n, np.nan)
    u[1:-1, 1:-1, 1:-1] = np.asarray(x, dtype=np.float64).reshape(n[2], n[1], n[0])
    bb = face_fields(n) if b is None else [f.copy() for f in b]
    aa = cell_field(n, a_value) if a is None else a
    v = cell_field(n)
    apply_expr(n, box, beta, alpha, bc_kind, bc_value, 1 if b is None else 0, b_value, u, aa, v, bb)
    return logical(v)


# ---- the reference's own operators (fixture generation only)

def ref_available() -> bool:
    return REF_FVM.exists()


def _write_case(f, n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a, v, b):
    f.write(struct.pack("<3q", *[int(k) for k in n]))
    f.write(np.asarray(box, "<f8").reshape(6).tobytes())
    f.write(struct.pack("<2d", beta, alpha))
    f.write(struct.pack("<6i", *[int(k) for k in bc_kind]))
    f.write(struct.pack("<6d", *[float(k) for k in bc_value]))
    f.write(struct.pack("<i", int(coef_kind)))
    f.write(struct.pack("<d", float(coef_value)))
    for x in (u, a, v):
        f.write(np.asarray(x, "<f8").tobytes())
    for x in b:
        f.write(np.asarray(x, "<f8").tobytes())


def ref_apply(n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a, v, b):
    """(u, b, v) after the reference's own operators (oracle/_ref/ref_fvm)"""
    nx, ny, nz = n
    C, F = (nz + 2) * (ny + 2) * (nx + 2), (nz + 1) * (ny + 1) * (nx + 1)
    with tempfile.TemporaryDirectory() as d:
        i, o = Path(d) / "in", Path(d) / "out"
        with open(i, "wb") as f:
            _write_case(f, n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a, v, b)
        subprocess.run([str(REF_FVM), str(i), str(o)], check=True)
        r = np.fromfile(o, "<f8")
    shp_c, shp_f = (nz + 2, ny + 2, nx + 2), (nz + 1, ny + 1, nx + 1)
    uo = r[:C].reshape(shp_c)
    bo = [r[C + k * F:C + (k + 1) * F].reshape(shp_f) for k in range(3)]
    vo = r[C + 3 * F:].reshape(shp_c)
    return uo, bo, vo


def ref_cg(n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a, b, rhs, x0, *,
           maxiter, rtol, zero_guess=False):
    """The reference's CG (solvers/cg.hh, no preconditioner) over the
    reference's operator expression: (status, iters, norms, hist, x)"""
    nx, ny, nz = n
    N = nx * ny * nz
    with tempfile.TemporaryDirectory() as d:
        i, o = Path(d) / "in", Path(d) / "out"
        with open(i, "wb") as f:
            _write_case(f, n, box, beta, alpha, bc_kind, bc_value, coef_kind, coef_value, u, a,
                        cell_field(n), b)
            f.write(np.asarray(rhs, "<f8").tobytes())
            f.write(np.asarray(x0, "<f8").tobytes())
        subprocess.run([str(REF_FVM), str(i), str(o), "cg", str(maxiter), repr(float(rtol)),
                        str(int(zero_guess))], check=True)
        d = o.read_bytes()
    st, it, _ = struct.unpack_from("<3i", d, 0)
    norms = struct.unpack_from("<5f", d, 12)
    nh = struct.unpack_from("<q", d, 32)[0]
    hist = np.frombuffer(d, "<f8", nh, 40).copy()
    x = np.frombuffer(d, "<f8", N, 40 + 8 * nh).copy()
    return st, it, norms, hist, x
