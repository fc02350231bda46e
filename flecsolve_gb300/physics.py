"""Finite-volume physics operators on the device (flecsolve/physics/).

Python mirror of the reference's structured-mesh physics layer over the
``fs_fvm_*`` C ABI of ``include/fsgpu.h``:

==============================================================  =====================================
reference (C++)                                                 here
==============================================================  =====================================
``init_mesh(s, m, {nx, ny, nz})`` (physics/test/test_setup.hh)   ``fvm_mesh(ctx, (nx, ny, nz), box)``
``bc<dirichlet<Vec>, msh::x_axis,                                ``bc(dirichlet(v), x_axis,
msh::domain::boundary_low>::create({{v}})``                      boundary_low)``
``bc<neumann<Vec>, axis, boundary>::create({{q}})``              ``bc(neumann(q), axis, boundary)``
``coefficient<constant_coefficient<Vec>, Vec>::create(           ``coefficient(constant_coefficient(c),
{{c}, faces})``                                                  faces)``
``coefficient<average_coefficient<Vec>, Vec>::create(            ``coefficient(average_coefficient(),
{{}, faces})``                                                   faces)``
``diffusion<Vec>::create({a, faces, beta, alpha}, m)``           ``diffusion(m, a, faces, beta, alpha)``
``op_expr(multivariable<...>, ops...)``                          ``op_expr(*ops)``
==============================================================  =====================================

Fields are device vectors of a mesh (``fvm_mesh.cell_field`` /
``face_fields``) laid out as the reference's: cells with one boundary layer,
``[k][j][i]``, i fastest.  ``op.apply(u, v)`` runs the operators in order as
the reference's expression does (boundary operators write u's boundary
cells, coefficient setters the face fields, diffusion v's logical cells),
with the same values bit for bit.  ``op_expr(...).matrix_free()`` turns an
expression of six boundary operators, a face coefficient and the diffusion
operator into the matrix-free operator the Krylov solvers take, on vectors
of the logical cells.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib
from .api import CSR, Context, Vector

x_axis, y_axis, z_axis = 0, 1, 2
boundary_low, boundary_high = 0, 1


class fvm_mesh:
    """The structured mesh (the reference's ``fvm_narray`` with boundary depth
    1 on one color): ``extents`` logical cells per axis (x, y, z) on ``box``
    ((lo, hi) per axis)."""

    x_axis, y_axis, z_axis = x_axis, y_axis, z_axis
    boundary_low, boundary_high = boundary_low, boundary_high

    def __init__(self, ctx: Context, extents, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))):
        self.ctx = ctx
        self.n = tuple(int(e) for e in extents)
        self.box = tuple((float(lo), float(hi)) for lo, hi in box)
        m = _lib.FvmMesh()
        for a in range(3):
            m.n[a] = self.n[a]
            m.box[a][0], m.box[a][1] = self.box[a]
        self._m = m
        dx, dA, vol = (C.c_double * 3)(), (C.c_double * 3)(), C.c_double()
        check(lib().fs_fvm_geometry(C.byref(m), dx, dA, C.byref(vol)), ctx.h, "fs_fvm_geometry")
        self._dx, self._dA, self._vol = list(dx), list(dA), vol.value

    # sizes and geometry (fvm_narray.hh:233-289)
    @property
    def cell_shape(self):
        nx, ny, nz = self.n
        return (nz + 2, ny + 2, nx + 2)

    @property
    def face_shape(self):
        nx, ny, nz = self.n
        return (nz + 1, ny + 1, nx + 1)

    def dofs(self) -> int:
        return self.n[0] * self.n[1] * self.n[2]

    def dx(self, axis: int) -> float:
        return self._dx[axis]

    def normal_dA(self, axis: int) -> float:
        return self._dA[axis]

    def volume(self) -> float:
        return self._vol

    # fields
    def cell_field(self, value=0.0) -> Vector:
        arr = np.broadcast_to(np.asarray(value, dtype=np.float64), self.cell_shape)
        v = Vector(self.ctx, np.ascontiguousarray(arr).reshape(-1))
        v.mesh = self
        return v

    def face_fields(self, value=0.0):
        out = []
        for k in range(3):
            val = value[k] if isinstance(value, (list, tuple)) else value
            arr = np.broadcast_to(np.asarray(val, dtype=np.float64), self.face_shape)
            v = Vector(self.ctx, np.ascontiguousarray(arr).reshape(-1))
            v.mesh = self
            out.append(v)
        return out

    def pack(self, field: Vector, x: Vector | None = None) -> Vector:
        """the logical cells of a cell field as a vector (i fastest)"""
        if x is None:
            x = Vector(self.ctx, self.dofs())
        check(lib().fs_fvm_pack(self.ctx.h, C.byref(self._m), field.h, x.h), self.ctx.h, "fs_fvm_pack")
        return x

    def unpack(self, x: Vector, field: Vector) -> Vector:
        """write a vector of logical cells into a cell field's logical cells"""
        check(lib().fs_fvm_unpack(self.ctx.h, C.byref(self._m), x.h, field.h), self.ctx.h, "fs_fvm_unpack")
        return field


def _mesh_of(*vs):
    for v in vs:
        m = getattr(v, "mesh", None)
        if m is not None:
            return m
    raise ValueError("the field is not a field of an fvm_mesh (make it with fvm_mesh.cell_field)")


class dirichlet:
    """``operator_parameters<dirichlet<Vec>>`` (boundary/dirichlet.hh:35-38)"""
    kind = _lib.BC_DIRICHLET

    def __init__(self, boundary_value: float = 0.0):
        self.value = float(boundary_value)


class neumann:
    """``operator_parameters<neumann<Vec>>`` (boundary/neumann.hh:31-34)"""
    kind = _lib.BC_NEUMANN

    def __init__(self, flux_value: float = 0.0):
        self.value = float(flux_value)


class bc:
    """``bc<Spec, Axis, Boundary>`` (boundary/bc_base.hh:29-57): applied to
    (u, v) it sets u's boundary cells beyond one face of the mesh."""

    def __init__(self, spec, axis: int, boundary: int):
        if axis not in (0, 1, 2) or boundary not in (0, 1):
            raise ValueError("axis must be x/y/z_axis and boundary boundary_low/high")
        self.spec, self.axis, self.boundary = spec, axis, boundary
        self.face = 2 * axis + boundary

    def apply(self, u: Vector, v=None):
        m = _mesh_of(u)
        check(lib().fs_fvm_boundary(m.ctx.h, C.byref(m._m), self.face, self.spec.kind, self.spec.value, u.h),
              m.ctx.h, "fs_fvm_boundary")

    def flat(self):
        return [self]


class constant_coefficient:
    """``operator_parameters<constant_coefficient<Vec>>`` (coefficient.hh:66-71)"""

    def __init__(self, coeff_value: float = 1.0):
        self.value = float(coeff_value)


class average_coefficient:
    """``operator_parameters<average_coefficient<Vec>>`` (coefficient.hh:119-123)"""

    def __init__(self, dummy_value: float = 1.0):
        self.value = float(dummy_value)


class coefficient:
    """``coefficient<Spec, Vec>`` (coefficient.hh:47-61): applied to (u, v) it
    sets the face fields from its parameters (a constant) or from u (the
    average of the cells either side of each face)."""

    def __init__(self, spec, faces):
        self.spec, self.faces = spec, list(faces)
        if len(self.faces) != 3:
            raise ValueError("faces: one face field per axis")

    def apply(self, u: Vector, v=None):
        m = _mesh_of(*self.faces)
        bx, by, bz = (f.h for f in self.faces)
        if isinstance(self.spec, average_coefficient):
            check(lib().fs_fvm_coef_average(m.ctx.h, C.byref(m._m), u.h, bx, by, bz), m.ctx.h,
                  "fs_fvm_coef_average")
        else:
            check(lib().fs_fvm_coef_constant(m.ctx.h, C.byref(m._m), self.spec.value, bx, by, bz), m.ctx.h,
                  "fs_fvm_coef_constant")

    def flat(self):
        return [self]


class diffusion:
    """``diffusion<Vec>`` (volume_diffusion/diffusion.hh:209-250): applied to
    (u, v), v = -beta div(b grad u) + alpha vol a u on the logical cells.
    ``a`` is a cell field or a number (a field of that value)."""

    def __init__(self, mesh: fvm_mesh, a, faces, beta: float = 1.0, alpha: float = 0.0):
        self.mesh, self.faces = mesh, list(faces)
        self.a = a if isinstance(a, Vector) else None
        self.a_value = 1.0 if isinstance(a, Vector) or a is None else float(a)
        self.beta, self.alpha = float(beta), float(alpha)

    def apply(self, u: Vector, v: Vector):
        m = self.mesh
        if self.a is None:
            self.a = m.cell_field(self.a_value)
        bx, by, bz = (f.h for f in self.faces)
        check(lib().fs_fvm_diffusion(m.ctx.h, C.byref(m._m), self.beta, self.alpha, self.a.h, bx, by, bz, u.h,
                                     v.h), m.ctx.h, "fs_fvm_diffusion")

    def flat(self):
        return [self]


class op_expr:
    """``op_expr(multivariable<...>, ops...)`` (expressions/
    operator_expression.hh:55-143): ``apply(u, v)`` applies each operator in
    order; nested expressions are flattened."""

    def __init__(self, *ops):
        self.ops = list(ops)

    def flat(self):
        out = []
        for o in self.ops:
            out.extend(o.flat())
        return out

    def apply(self, u: Vector, v: Vector):
        for o in self.ops:
            o.apply(u, v)

    def matrix_free(self) -> CSR:
        """The expression as an operator on vectors of the logical cells, for
        the Krylov solvers: six boundary operators (one per face), at most
        one coefficient setter with a constant (or none: the diffusion
        operator's face fields are used as they are) and one diffusion
        operator.  Returns a :class:`CSR`-compatible operator that stores no
        matrix; it copies the face and cell coefficients at creation, so later
        changes to those fields need a new operator."""
        ops = self.flat()
        bcs = {o.face: o for o in ops if isinstance(o, bc)}
        coefs = [o for o in ops if isinstance(o, coefficient)]
        diffs = [o for o in ops if isinstance(o, diffusion)]
        if len(bcs) != 6 or sum(isinstance(o, bc) for o in ops) != 6:
            raise ValueError("matrix_free: one boundary operator per face is needed")
        if len(diffs) != 1 or len(coefs) > 1 or len(bcs) + len(coefs) + len(diffs) != len(ops):
            raise ValueError("matrix_free: boundary operators, at most one coefficient and one diffusion")
        d = diffs[0]
        m = d.mesh
        s = _lib.FvmOperatorSettings()
        s.mesh = m._m
        s.beta, s.alpha = d.beta, d.alpha
        s.a_value = d.a_value
        for f in range(6):
            s.bc_kind[f] = bcs[f].spec.kind
            s.bc_value[f] = bcs[f].spec.value
        faces = d.faces
        if coefs:
            c = coefs[0]
            if isinstance(c.spec, average_coefficient):
                raise ValueError("matrix_free: an average coefficient makes the operator nonlinear")
            if [f.h.value for f in c.faces] != [f.h.value for f in d.faces]:
                raise ValueError("matrix_free: the coefficient must set the diffusion operator's faces")
            s.b_value = c.spec.value
            faces = None
        h = C.c_void_p()
        fh = [None, None, None] if faces is None else [f.h for f in faces]
        ah = d.a.h if d.a is not None else None
        check(lib().fs_fvm_operator_create(m.ctx.h, C.byref(s), ah, fh[0], fh[1], fh[2], C.byref(h)),
              m.ctx.h, "fs_fvm_operator_create")
        A = CSR(m.ctx, None, _handle=h)
        A.mesh = m
        return A


def operator_info(A: CSR):
    """(affine, logical cells per axis) of a matrix-free operator"""
    aff, n = C.c_int(), (C.c_int64 * 3)()
    check(lib().fs_fvm_operator_info(A.h, C.byref(aff), n), A.ctx.h, "fs_fvm_operator_info")
    return bool(aff.value), tuple(n)
