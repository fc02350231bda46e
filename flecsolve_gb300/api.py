"""Python mirror of flecsolve's Krylov-path API over the C ABI.

Names, argument order and meaning follow the reference so that code written
against it reads the same:

=====================================  =========================================
reference (C++)                        here
=====================================  =========================================
``vec::core`` ops (core.hh:59-310)     :class:`Vector` methods
``op::ref(A)`` / ``op::I``             :func:`op.ref`, :data:`op.I`
``mat::csr`` apply (seq.hh:50-60)      :class:`CSR` ``apply`` / ``residual``
``cg::settings{maxiter, rtol, ...}``   :func:`cg.settings`
``cg::make_work(b)``                   :func:`cg.make_work`
``cg::solver(s, w)(A, P, diag)(b, x)`` ``cg.solver(s, w)(A, P, diag)(b, x)``
``solve_info``                         :class:`SolveInfo`
=====================================  =========================================

Everything runs on the GPU through ``libfsgpu.so``; reductions synchronise
and return a :class:`Future` whose ``get()`` gives the value, like the
reference's futures (flecsolve/util/future.hh:23-59).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np

from . import _lib
from ._lib import check, lib

__all__ = ["Context", "Vector", "Multi", "CSR", "SolveInfo", "Future", "op", "vec", "mat",
           "batch_cg", "batch_tuning", "block_cg",
           "cg", "bicgstab", "gmres", "fcg", "pipelined_cg", "mixed_cg", "mixed_bicgstab", "mixed_gmres",
           "Shell"]


class Context:
    """One CUDA device + stream (``fs_ctx``)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().fs_ctx_create(device, C.byref(h)), None, "fs_ctx_create")
        self.h = h
        self.device = device

    def sync(self):
        check(lib().fs_ctx_sync(self.h), self.h)

    @property
    def sm_count(self) -> int:
        n = C.c_int()
        check(lib().fs_ctx_sm_count(self.h, C.byref(n)), self.h)
        return n.value

    @property
    def launches(self) -> int:
        n = C.c_int64()
        check(lib().fs_ctx_launch_count(self.h, C.byref(n)), self.h)
        return n.value

    @property
    def stream(self) -> int:
        p = C.c_void_p()
        check(lib().fs_ctx_stream(self.h, C.byref(p)), self.h)
        return p.value or 0

    def record(self, slot: int):
        """Record CUDA event `slot` on the context stream."""
        check(lib().fs_ctx_event_record(self.h, slot), self.h)

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        check(lib().fs_ctx_event_elapsed(self.h, a, b, C.byref(ms)), self.h)
        return ms.value

    def close(self):
        if getattr(self, "h", None):
            lib().fs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Future:
    """Value of a reduction (``.get()``, flecsolve/util/future.hh)."""

    def __init__(self, v):
        self._v = v

    def get(self):
        return self._v


class Vector:
    """Device vector: ``vec::core`` over the device Data/Operations policy."""

    def __init__(self, ctx: Context, n_or_array, dtype: str = "f64", *, _handle=None):
        self.ctx = ctx
        if _handle is not None:
            self.h = _handle
            return
        arr = None
        if isinstance(n_or_array, (int, np.integer)):
            n = int(n_or_array)
        else:
            arr = np.asarray(n_or_array)
            n = arr.size
            if dtype is None:
                dtype = "f32" if arr.dtype == np.float32 else "f64"
        self.dtype = dtype
        h = C.c_void_p()
        check(lib().fs_vec_create(ctx.h, n, _lib.F32 if dtype == "f32" else _lib.F64, C.byref(h)),
              ctx.h, "fs_vec_create")
        self.h = h
        if arr is not None:
            self.upload(arr)

    @classmethod
    def wrap(cls, ctx: Context, n: int, dptr: int, dtype: str = "f64") -> "Vector":
        h = C.c_void_p()
        check(lib().fs_vec_wrap(ctx.h, n, _lib.F32 if dtype == "f32" else _lib.F64,
                                C.c_void_p(dptr), C.byref(h)), ctx.h, "fs_vec_wrap")
        return cls(ctx, 0, dtype, _handle=h)

    # -- data
    def __len__(self):
        n = C.c_int64()
        check(lib().fs_vec_size(self.h, C.byref(n)), self.ctx.h)
        return n.value

    @property
    def np_dtype(self):
        d = C.c_int()
        check(lib().fs_vec_dtype(self.h, C.byref(d)), self.ctx.h)
        return np.float32 if d.value == _lib.F32 else np.float64

    @property
    def device_ptr(self) -> int:
        p = C.c_void_p()
        check(lib().fs_vec_device_ptr(self.h, C.byref(p)), self.ctx.h)
        return p.value or 0

    def upload(self, arr):
        a = np.ascontiguousarray(arr, dtype=self.np_dtype)
        check(lib().fs_vec_upload(self.h, a.ctypes.data_as(C.c_void_p), a.size), self.ctx.h, "upload")

    def numpy(self) -> np.ndarray:
        out = np.empty(len(self), dtype=self.np_dtype)
        check(lib().fs_vec_download(self.h, out.ctypes.data_as(C.c_void_p), out.size), self.ctx.h,
              "download")
        return out

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().fs_vec_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # -- elementwise ops (flecsolve/vectors/core.hh:59-221); `self` is the output
    def copy(self, src: "Vector"):
        check(lib().fs_vec_copy(src.h, self.h), self.ctx.h, "copy")

    def zero(self):
        check(lib().fs_vec_zero(self.h), self.ctx.h)

    def set_scalar(self, val: float):
        check(lib().fs_vec_set_scalar(self.h, float(val)), self.ctx.h)

    def scale(self, alpha: float, x: "Vector" = None):
        if x is None:
            check(lib().fs_vec_scale_self(float(alpha), self.h), self.ctx.h)
        else:
            check(lib().fs_vec_scale(float(alpha), x.h, self.h), self.ctx.h)

    def add(self, x, y):
        check(lib().fs_vec_add(x.h, y.h, self.h), self.ctx.h)

    def subtract(self, x, y):
        check(lib().fs_vec_subtract(x.h, y.h, self.h), self.ctx.h)

    def multiply(self, x, y):
        check(lib().fs_vec_multiply(x.h, y.h, self.h), self.ctx.h)

    def divide(self, x, y):
        check(lib().fs_vec_divide(x.h, y.h, self.h), self.ctx.h)

    def reciprocal(self, x):
        check(lib().fs_vec_reciprocal(x.h, self.h), self.ctx.h)

    def linear_sum(self, alpha, x, beta, y):
        check(lib().fs_vec_linear_sum(float(alpha), x.h, float(beta), y.h, self.h), self.ctx.h)

    def axpy(self, alpha, x, y):
        check(lib().fs_vec_axpy(float(alpha), x.h, y.h, self.h), self.ctx.h)

    def axpby(self, alpha, beta, x):
        check(lib().fs_vec_axpby(float(alpha), float(beta), x.h, self.h), self.ctx.h)

    def abs(self, x):
        check(lib().fs_vec_abs(x.h, self.h), self.ctx.h)

    def add_scalar(self, x, alpha):
        check(lib().fs_vec_add_scalar(x.h, float(alpha), self.h), self.ctx.h)

    def set_random(self, seed: int = 0):
        check(lib().fs_vec_set_random(self.h, int(seed)), self.ctx.h)

    # -- reductions (core.hh:229-290)
    def _red(self, fn, *args):
        out = C.c_double()
        check(fn(*args, C.byref(out)), self.ctx.h)
        return Future(out.value)

    def dot(self, x):
        return self._red(lib().fs_vec_dot, self.h, x.h)

    def l1norm(self):
        return self._red(lib().fs_vec_l1norm, self.h)

    def l2norm(self):
        return self._red(lib().fs_vec_l2norm, self.h)

    def inf_norm(self):
        return self._red(lib().fs_vec_inf_norm, self.h)

    def min(self):
        return self._red(lib().fs_vec_min, self.h)

    def max(self):
        return self._red(lib().fs_vec_max, self.h)

    def global_size(self):
        return Future(len(self))

    def local_size(self):
        return len(self)


def _dtype_code(dtype) -> int:
    """FS_F32 for float32 / "f32", FS_F64 otherwise."""
    if isinstance(dtype, str):
        return _lib.F32 if dtype == "f32" else _lib.F64
    return _lib.F32 if np.dtype(dtype) == np.float32 else _lib.F64


class CSR:
    """Device CSR operator (``op::core<mat::csr<double>>``).  ``var`` is the
    operator's input/output variable (``op::base<Params, ivar, ovar>``,
    operators/core.hh:29-34): applied to a :class:`Multi` the operator acts on
    that component (``op::core::apply`` subsets, core.hh:107-116)."""

    def __init__(self, ctx: Context, A, var=None, *, _handle=None):
        self.ctx = ctx
        self.var = var
        if _handle is not None:
            r, c = C.c_int64(), C.c_int64()
            check(lib().fs_csr_shape(_handle, C.byref(r), C.byref(c), None), ctx.h)
            self.nrows, self.ncols, self.h = r.value, c.value, _handle
            return
        self.nrows, self.ncols = int(A.nrows), int(A.ncols)
        rp = np.ascontiguousarray(A.rowptr, dtype=np.int64)
        col = np.ascontiguousarray(A.col)
        ib = 4 if col.dtype == np.int32 else 8
        if ib == 8:
            col = col.astype(np.int64, copy=False)
        val = np.ascontiguousarray(A.val, dtype=np.float64)
        h = C.c_void_p()
        check(lib().fs_csr_create(ctx.h, self.nrows, self.ncols, int(rp[-1]),
                                  rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                                  ib, val.ctypes.data_as(C.c_void_p), C.byref(h)),
              ctx.h, "fs_csr_create")
        self.h = h

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().fs_csr_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def rows(self):
        return self.nrows

    def cols(self):
        return self.ncols

    def nnz(self):
        n = C.c_int64()
        check(lib().fs_csr_shape(self.h, None, None, C.byref(n)), self.ctx.h)
        return n.value

    def _sub(self, v):
        return v.subset(self.var) if isinstance(v, Multi) else v

    def apply(self, x: Vector, y: Vector, exact: bool = False):
        """y = A x (op::core::apply, operators/core.hh:107-116)."""
        x, y = self._sub(x), self._sub(y)
        check(lib().fs_csr_spmv(self.h, x.h, y.h, _lib.SPMV_EXACT if exact else _lib.SPMV_FMA),
              self.ctx.h, "spmv")

    __call__ = apply

    def residual(self, b: Vector, x: Vector, r: Vector):
        """r = b - A x (op::core::residual, operators/core.hh:129-142)."""
        b, x, r = self._sub(b), self._sub(x), self._sub(r)
        check(lib().fs_csr_residual(self.h, b.h, x.h, r.h), self.ctx.h, "residual")

    def apply_transpose(self, x: Vector, y: Vector):
        check(lib().fs_csr_spmv_transpose(self.h, x.h, y.h), self.ctx.h, "spmv^T")

    def parcsr_apply(self, parts: int, x: Vector, y: Vector):
        check(lib().fs_parcsr_spmv(self.h, int(parts), x.h, y.h), self.ctx.h, "parcsr spmv")

    def update_values(self, val: np.ndarray):
        v = np.ascontiguousarray(val, dtype=np.float64)
        check(lib().fs_csr_update_values(self.h, v.ctypes.data_as(C.c_void_p)), self.ctx.h)

    def nblk(self) -> int:
        """Number of SpMV row blocks."""
        n = C.c_int64()
        check(lib().fs_csr_row_blocks(self.h, C.byref(n)), self.ctx.h)
        return n.value

    CODINGS = {"colids": 0, "patterns": 1, "symmetric": 2, "grid": 3}

    def index_coding(self, enable=None) -> int:
        """The index format the FP64 SpMV uses: 0 = column ids, 1 = row
        patterns (stencil operators: one pattern id per row, no column ids or
        row offsets read), 2 = row patterns with symmetric storage (the
        diagonal and upper diagonals of a matrix that is symmetric bit for
        bit), 3 = the symmetric storage of a grid stencil addressed by grid
        coordinates (no pattern ids, 16-byte loads), 4 = the general grid
        storage that format 3 uses for a grid stencil whose values are not
        symmetric (the lower diagonals at their own rows; not requestable by
        itself).  `enable` switches it:
        True = the best format the matrix supports, False = column ids, or a
        mode number / name; a format the matrix (or its current values) does
        not support falls back to the next one down."""
        if enable is None:
            req = -1
        elif isinstance(enable, bool):
            req = 3 if enable else 0
        elif isinstance(enable, str):
            req = self.CODINGS[enable]
        else:
            req = int(enable)
        a = C.c_int()
        check(lib().fs_csr_index_coding(self.h, req, C.byref(a)), self.ctx.h)
        return a.value

    def grid_dims(self):
        """(nx, ny, nz) of a grid-stencil matrix, (0, 0, 0) otherwise."""
        d = (C.c_int64 * 3)()
        check(lib().fs_csr_grid_dims(self.h, d), self.ctx.h)
        return tuple(int(v) for v in d)

    def tune(self, dtype=np.float64) -> int:
        """Time the column-id SpMV schedules for values of `dtype` and keep
        the fastest: 0 (one thread per row), 4 / 8 / 16 / 32 lanes per row,
        or 1 (lanes per row by row-length class).  Returns the choice."""
        lanes = C.c_int()
        check(lib().fs_csr_tune(self.h, _dtype_code(dtype), C.byref(lanes)), self.ctx.h, "fs_csr_tune")
        return lanes.value

    def set_lanes(self, lanes: int, dtype=np.float64) -> None:
        """Fix the column-id SpMV schedule (-1: tune again on the next SpMV)."""
        check(lib().fs_csr_set_lanes(self.h, _dtype_code(dtype), int(lanes)), self.ctx.h,
              "fs_csr_set_lanes")

    def values(self) -> np.ndarray:
        """The current values (row order) copied to the host."""
        p = C.c_void_p()
        check(lib().fs_csr_values_device_ptr(self.h, C.byref(p)), self.ctx.h)
        v = Vector.wrap(self.ctx, self.nnz(), p.value)
        return v.numpy()

    def transpose(self) -> "CSR":
        """A^T materialised as a new device CSR matrix."""
        h = C.c_void_p()
        check(lib().fs_csr_transpose(self.h, C.byref(h)), self.ctx.h, "fs_csr_transpose")
        return CSR(self.ctx, None, _handle=h)

    def value_grad(self, lam: Vector, x: Vector, g: Vector):
        """g = dL/dA on the pattern for x = A^-1 b and lam = A^-T dL/dx:
        g_k = -lam_i x_j for entry k = (i, j)."""
        check(lib().fs_csr_value_grad(self.h, lam.h, x.h, g.h), self.ctx.h, "value grad")

    def fv_assemble(self, dim: int, n: int, faces: Vector, scale: float = 1.0,
                    shift: float = 0.0):
        """Values = scale K(faces) + shift I for the finite-volume diffusion
        pattern of an n^dim grid (the generator's face layout and row order)."""
        check(lib().fs_fv_assemble(self.h, dim, n, faces.h, scale, shift), self.ctx.h,
              "fs_fv_assemble")

    def Dinv(self) -> Vector:
        """Diagonal inverse as a vector (util/test/mesh.hh:123-140)."""
        d = Vector(self.ctx, self.nrows)
        check(lib().fs_csr_diag_inv(self.h, d.h), self.ctx.h, "diag_inv")
        return d


class Multi:
    """``vec::multi``: a tuple of component vectors tagged with variables
    (flecsolve/vectors/multi.hh:74-160, operations/multi.hh:27-277).

    The components are views into one contiguous device allocation, so the
    multivector is also one :class:`Vector` (``whole``) for solvers bound to
    an operator on all components.  Elementwise operations act on every
    component; reductions combine the per-component reductions the way the
    reference's multi ops do (sum of dots, sqrt of the summed squares, max /
    min over components, in component order)."""

    def __init__(self, ctx: Context, parts, vars=None, dtype: str = "f64"):
        arrays = [np.asarray(p) if not isinstance(p, (int, np.integer)) else None for p in parts]
        sizes = [int(p) if a is None else int(a.size) for p, a in zip(parts, arrays)]
        self.ctx = ctx
        self.vars = list(vars) if vars is not None else list(range(len(sizes)))
        self.whole = Vector(ctx, sum(sizes), dtype)
        es = 4 if dtype == "f32" else 8
        base = self.whole.device_ptr
        self.components, off = [], 0
        for n, a in zip(sizes, arrays):
            c = Vector.wrap(ctx, n, base + off * es, dtype)
            c._owner = self.whole  # keep the allocation alive
            if a is not None:
                c.upload(a)
            self.components.append(c)
            off += n

    # -- access (multi.hh:94-159)
    def get(self, i: int) -> Vector:
        return self.components[i]

    def subset(self, var) -> Vector:
        return self.components[self.vars.index(var)]

    def __len__(self):
        return len(self.whole)

    def numpy(self):
        return [c.numpy() for c in self.components]

    # -- elementwise: the same operation on each component
    def _each(self, name, *args):
        for i, c in enumerate(self.components):
            a = [x.components[i] if isinstance(x, Multi) else x for x in args]
            getattr(c, name)(*a)

    def copy(self, src): self._each("copy", src)
    def zero(self): self._each("zero")
    def set_scalar(self, v): self._each("set_scalar", v)
    def scale(self, a, x=None): self._each("scale", a) if x is None else self._each("scale", a, x)
    def add(self, x, y): self._each("add", x, y)
    def subtract(self, x, y): self._each("subtract", x, y)
    def multiply(self, x, y): self._each("multiply", x, y)
    def divide(self, x, y): self._each("divide", x, y)
    def reciprocal(self, x): self._each("reciprocal", x)
    def linear_sum(self, a, x, b, y): self._each("linear_sum", a, x, b, y)
    def axpy(self, a, x, y): self._each("axpy", a, x, y)
    def axpby(self, a, b, x): self._each("axpby", a, b, x)
    def abs(self, x): self._each("abs", x)
    def add_scalar(self, x, a): self._each("add_scalar", x, a)

    # -- reductions combined over components (operations/multi.hh:179-253)
    def dot(self, x):
        return Future(sum(c.dot(xc).get() for c, xc in zip(self.components, x.components)))

    def l1norm(self):
        return Future(sum(c.l1norm().get() for c in self.components))

    def l2norm(self):
        return Future(float(np.sqrt(sum(c.dot(c).get() for c in self.components))))

    def inf_norm(self):
        return Future(max(c.inf_norm().get() for c in self.components))

    def min(self):
        return Future(min(c.min().get() for c in self.components))

    def max(self):
        return Future(max(c.max().get() for c in self.components))


# ------------------------------------------------------------- op:: ----

class Shell(CSR):
    """``op::make_shell(f)`` (operators/shell.hh:26-95): a caller-defined
    operator ``f(x, y)`` that writes ``y = Op(x)`` on FP64 device vectors of
    ``ctx`` (through any Vector / CSR / solver call).  Usable wherever an
    operator goes: ``apply``, residuals, and every solver as A or as the
    preconditioner.  An exception in ``f`` stops the solve with
    ``FsError`` (FS_ERR_CALLBACK)."""

    def __init__(self, ctx: Context, f, nrows: int, ncols: int = None, var=None):
        self.ctx = ctx
        self.var = var
        self.nrows = int(nrows)
        self.ncols = int(nrows if ncols is None else ncols)
        self.error = None

        def _cb(user, xh, yh):
            xv, yv = (Vector.__new__(Vector) for _ in range(2))
            for v, hnd in ((xv, xh), (yv, yh)):
                v.ctx = ctx
                v.h = C.c_void_p(hnd)
            try:
                f(xv, yv)
                return 0
            except Exception as e:  # reported through the status code
                self.error = e
                return 1
            finally:
                xv.h = yv.h = None  # borrowed handles

        self._cb = _lib.OP_FN(_cb)
        h = C.c_void_p()
        check(lib().fs_shell_create(ctx.h, self.nrows, self.ncols, self._cb, None, C.byref(h)),
              ctx.h, "fs_shell_create")
        self.h = h


class _Identity:
    """``op::I`` (operators/shell.hh:317-318)."""


class _Jacobi:
    """The D^-1 operator of A (util/test/mesh.hh:123-140)."""


op = SimpleNamespace(I=_Identity(), jacobi=_Jacobi(), ref=lambda A: A, cref=lambda A: A,
                     make_shared=lambda A: A, make_shell=Shell)
vec = SimpleNamespace(make=lambda ctx, a, dtype="f64": Vector(ctx, a, dtype), Vector=Vector,
                      multi=Multi)
mat = SimpleNamespace(csr=CSR)


# ---------------------------------------------------------- solvers ----

@dataclass
class SolveInfo:
    """solve_info (flecsolve/solvers/solver_settings.hh:61-85)."""
    status: str
    iters: int
    restarts: int
    res_norm_initial: float
    res_norm_final: float
    sol_norm_initial: float
    sol_norm_final: float
    rhs_norm: float

    def success(self) -> bool:
        return self.status in ("converged_atol", "converged_rtol", "converged_user")


def _settings(method, maxiter, rtol, atol, use_zero_guess, **kw):
    s = _lib.KrylovSettings()
    lib().fs_krylov_settings_default(C.byref(s))
    s.base.maxiter = int(maxiter)
    s.base.rtol = float(rtol)
    s.base.atol = float(atol)
    s.base.use_zero_guess = int(bool(use_zero_guess))
    for k, v in kw.items():
        if k == "pre_side":
            v = _lib.LEFT if v in ("left", _lib.LEFT) else _lib.RIGHT
        elif k == "ortho":
            v = {"mgs": _lib.ORTHO_MGS, "cgs2": _lib.ORTHO_CGS2, "auto": _lib.ORTHO_AUTO,
                 "dcgs2": _lib.ORTHO_DCGS2}.get(v, v)
        elif k == "refine":
            v = _lib.REFINE_RELIABLE if v in ("reliable", _lib.REFINE_RELIABLE) else _lib.REFINE_RESTART
        setattr(s, k, v)
    s._method = method
    return s


@dataclass
class Work:
    """Work vectors: the solver allocates them on the device on bind."""
    n: int
    nwork: int


class BoundSolver:
    """``op::core<op::X<krylov_parameters>>``: apply(b, x) -> SolveInfo."""

    def __init__(self, method, settings, work, A: CSR, P=None, diag=None):
        self.A = A
        self.ctx = A.ctx
        pc = _lib.Precond()
        self._keep = []
        if P is None or isinstance(P, _Identity):
            pc.kind = _lib.PRECOND_NONE
        elif isinstance(P, _Jacobi) or P == "jacobi":
            pc.kind = _lib.PRECOND_JACOBI
        elif isinstance(P, Vector):
            pc.kind = _lib.PRECOND_DIAG
            pc.diag = P.h
            self._keep.append(P)
        elif isinstance(P, CSR):
            # any operator: a stored or matrix-free CSR, or a shell
            pc.kind = _lib.PRECOND_CSR
            pc.op = P.h
            self._keep.append(P)
        elif isinstance(P, BoundSolver):
            # a nested solver (the NKA / flexible-CG pattern)
            pc.kind = _lib.PRECOND_SOLVER
            pc.solver = P.h
            self._keep.append(P)
        else:
            raise TypeError(f"unsupported preconditioner {P!r}")
        h = C.c_void_p()
        check(lib().fs_krylov_create(self.ctx.h, method, C.byref(settings), A.h, C.byref(pc),
                                     C.byref(h)), self.ctx.h, "fs_krylov_create")
        self.h = h
        self._diag_cb = None
        if diag is not None:
            self.set_diagnostic(diag)

    def set_diagnostic(self, fn):
        ctx = self.ctx

        def _cb(user, xh, res):
            v = Vector.__new__(Vector)
            v.ctx = ctx
            v.h = C.c_void_p(xh) if xh else None
            try:
                return 1 if fn(v, res) else 0
            finally:
                v.h = None  # borrowed handle

        self._diag_cb = _lib.DIAG_FN(_cb)
        check(lib().fs_krylov_set_diagnostic(self.h, self._diag_cb, None), self.ctx.h)

    @property
    def settings(self):
        s = _lib.KrylovSettings()
        check(lib().fs_krylov_settings_get(self.h, C.byref(s)), self.ctx.h)
        return s

    @settings.setter
    def settings(self, s):
        check(lib().fs_krylov_settings_set(self.h, C.byref(s)), self.ctx.h)

    def apply(self, b: Vector, x: Vector, _fn="fs_krylov_apply") -> SolveInfo:
        # op::core::apply subsets by the operator's variables (core.hh:107-116)
        if isinstance(b, Multi):
            b = b.subset(self.A.var) if self.A.var is not None else b.whole
        if isinstance(x, Multi):
            x = x.subset(self.A.var) if self.A.var is not None else x.whole
        info = _lib.SolveInfo()
        st = getattr(lib(), _fn)(self.h, b.h, x.h, C.byref(info))
        out = SolveInfo(_lib.STOP_REASONS.get(info.status, str(info.status)), info.iters,
                        info.restarts, info.res_norm_initial, info.res_norm_final,
                        info.sol_norm_initial, info.sol_norm_final, info.rhs_norm)
        if st != _lib.OK:
            err = _lib.FsError(st, (lib().fs_last_error(self.ctx.h) or b"").decode())
            err.info = out
            raise err
        return out

    __call__ = apply

    def apply_transpose(self, b: Vector, x: Vector) -> SolveInfo:
        """Solve A^T x = b with the same method, settings and preconditioner
        (the adjoint solve; A^T is a device view of A's current values)."""
        return self.apply(b, x, _fn="fs_krylov_apply_transpose")

    def history(self) -> np.ndarray:
        n = C.c_int64(1 << 30)
        check(lib().fs_krylov_history(self.h, None, C.byref(n)), self.ctx.h)
        out = np.empty(n.value)
        m = C.c_int64(out.size)
        check(lib().fs_krylov_history(self.h, out.ctypes.data_as(_lib._dp), C.byref(m)), self.ctx.h)
        return out[: m.value]

    def mixed_stats(self):
        o, i = C.c_int(), C.c_int()
        check(lib().fs_krylov_mixed_stats(self.h, C.byref(o), C.byref(i)), self.ctx.h)
        return o.value, i.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().fs_krylov_destroy(self.h)
                self.h = None
        except Exception:
            pass


def _info(i) -> "SolveInfo":
    return SolveInfo(_lib.STOP_REASONS.get(i.status, str(i.status)), i.iters, i.restarts,
                     i.res_norm_initial, i.res_norm_final, i.sol_norm_initial, i.sol_norm_final,
                     i.rhs_norm)


def batch_cg(A: CSR, offsets, b: Vector, x: Vector, maxiter: int, rtol: float,
             use_zero_guess: bool = True, delta: float = 0.0, cluster: int = 0,
             threads: int = 0, fp64_head: float = None, cluster_systems: int = None):
    """Solve the independent systems on the diagonal blocks of ``A`` (system
    s = rows offsets[s]:offsets[s+1]) in one persistent launch, one thread-
    block cluster per system; returns one :class:`SolveInfo` per system.
    ``cluster``/``threads`` = 0 lets the autotuner choose; ``fp64_head``: FP64
    iterations until each system's residual is below that fraction of its
    ||b|| (None: the library default, 3e-3; 0: FP32 from the start).
    ``cluster_systems`` (with explicit sizes): that many of the largest
    systems own a cluster, every other system one CTA."""
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nsys = off.size - 1
    st = _settings(_lib.CG_MIXED, maxiter, rtol, 0.0, use_zero_guess, inner_rtol=delta)
    if fp64_head is not None:
        st.fp64_head = float(fp64_head)
    infos = (_lib.SolveInfo * nsys)()
    offp = off.ctypes.data_as(C.POINTER(C.c_int64))
    if cluster_systems is None:
        check(lib().fs_batch_cg_solve(A.ctx.h, C.byref(st), A.h, nsys, offp, b.h, x.h, int(cluster),
                                      int(threads), infos), A.ctx.h, "fs_batch_cg_solve")
    else:
        check(lib().fs_batch_cg_solve_split(A.ctx.h, C.byref(st), A.h, nsys, offp, b.h, x.h,
                                            int(cluster), int(threads), int(cluster_systems), infos),
              A.ctx.h, "fs_batch_cg_solve_split")
    return [_info(i) for i in infos]


def block_cg(A: CSR, B: Vector, X: Vector, nrhs: int, maxiter: int, rtol: float,
             use_zero_guess: bool = True, jacobi: bool = True, k_readback: int = 16,
             mixed: bool = False, delta: float = 0.0):
    """Block Jacobi-PCG on ``nrhs`` right-hand sides stored N x nrhs row-major
    in ``B`` / ``X``; returns one :class:`SolveInfo` per column.  ``mixed``:
    FP32 block recurrences with FP64 residual replacement every ``delta``
    reduction (0 = library default)."""
    st = _settings(_lib.CG, maxiter, rtol, 0.0, use_zero_guess, k_readback=k_readback,
                   inner_rtol=delta)
    pc = _lib.Precond(_lib.PRECOND_JACOBI if jacobi else _lib.PRECOND_NONE, None, None)
    infos = (_lib.SolveInfo * nrhs)()
    fn = lib().fs_block_cg_solve_mixed if mixed else lib().fs_block_cg_solve
    check(fn(A.ctx.h, C.byref(st), A.h, C.byref(pc), nrhs, B.h, X.h, infos),
          A.ctx.h, "fs_block_cg_solve")
    return [_info(i) for i in infos]


def batch_tuning(A: CSR, offsets):
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    c, t = C.c_int(), C.c_int()
    check(lib().fs_batch_tuning(A.ctx.h, A.h, off.size - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                C.byref(c), C.byref(t)), A.ctx.h, "fs_batch_tuning")
    return c.value, t.value


def batch_schedule(A: CSR, offsets):
    """(cluster size, threads per CTA, systems that own a cluster) the
    autotuner chose for this partition."""
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    c, t, nb = C.c_int(), C.c_int(), C.c_int()
    check(lib().fs_batch_schedule(A.ctx.h, A.h, off.size - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                  C.byref(c), C.byref(t), C.byref(nb)), A.ctx.h, "fs_batch_schedule")
    return c.value, t.value, nb.value


def batch_format(A: CSR, offsets) -> str:
    """The storage the batched kernel reads for this partition (checked on
    the first solve after the values change): "grid" (every system a
    symmetric 5-point square-grid stencil: diagonal and upper diagonals) or
    "csr" (the column ids)."""
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    f = C.c_int()
    check(lib().fs_batch_format(A.ctx.h, A.h, off.size - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                C.byref(f)), A.ctx.h, "fs_batch_format")
    return "grid" if f.value == 1 else "csr"


class _SolverFactory:
    """``X::solver(settings, work)``; calling it with (A[, P[, diag]]) binds."""

    def __init__(self, method, settings, work):
        self.method = method
        self.settings = settings
        self.work = work

    def __call__(self, A, P=None, diag=None) -> BoundSolver:
        return BoundSolver(self.method, self.settings, self.work, A, P, diag)

    bind = __call__


def _namespace(method, nwork, **defaults):
    def settings(maxiter, rtol=0.0, atol=0.0, use_zero_guess=True, **kw):
        merged = dict(defaults)
        merged.update(kw)
        return _settings(method, maxiter, rtol, atol, use_zero_guess, **merged)

    def make_work(b: Vector) -> Work:
        return Work(len(b), nwork)

    def solver(settings, work=None):
        return _SolverFactory(method, settings, work)

    return SimpleNamespace(settings=settings, make_work=make_work, solver=solver, nwork=nwork)


cg = _namespace(_lib.CG, 4)                 # flecsolve/solvers/cg.hh:250-270
bicgstab = _namespace(_lib.BICGSTAB, 8)     # bicgstab.hh:193-216
gmres = _namespace(_lib.GMRES, 104, max_krylov_dim=-1, pre_side="right", restart=False)  # gmres.hh:366-438
fcg = _namespace(_lib.FCG, 5)               # cg.hh:145-244, 272-290 (flexible CG)
pipelined_cg = _namespace(_lib.CG_PIPELINED, 6)  # cg.hh:43-139, one reduction per iteration
mixed_cg = _namespace(_lib.CG_MIXED, 4)     # FP32 inner PCG in FP64 refinement
mixed_bicgstab = _namespace(_lib.BICGSTAB_MIXED, 8)
mixed_gmres = _namespace(_lib.GMRES_MIXED, 104, max_krylov_dim=-1, pre_side="right", restart=False)


# ---------------------------------------------------------------- NKA --

class NkaSolver:
    """``op::core<op::nka<...>>`` (flecsolve/solvers/nka.hh:31-605):
    apply(f, u) -> SolveInfo.  ``F`` is the CSR operator (or ``None`` with
    ``residual(f, u, r)`` computing r = f - F(u) on device vectors for a
    nonlinear operator); ``P`` a bound Krylov solver used as the
    preconditioner (solvers/test/nka.cc:72-80 uses a CG solver), or ``None``.
    The acceleration subspace persists across applies, as the reference's
    does; :meth:`reset` empties it."""

    def __init__(self, settings, F=None, P=None, diag=None, residual=None, ctx=None):
        self.ctx = ctx or (F.ctx if F is not None else P.ctx)
        self._keep = [F, P]
        self._res_cb = None
        if residual is not None:
            ctxr = self.ctx

            def _rcb(user, fh, uh, rh):
                vs = []
                for hnd in (fh, uh, rh):
                    v = Vector.__new__(Vector)
                    v.ctx = ctxr
                    v.h = C.c_void_p(hnd)
                    vs.append(v)
                try:
                    residual(*vs)
                    return 0
                except Exception:
                    return _lib.ERR_INVALID_ARG
                finally:
                    for v in vs:
                        v.h = None  # borrowed handles

            self._res_cb = _lib.RESIDUAL_FN(_rcb)
        h = C.c_void_p()
        check(lib().fs_nka_create(self.ctx.h, C.byref(settings), F.h if F is not None else None,
                                  self._res_cb or _lib.RESIDUAL_FN(), None,
                                  P.h if P is not None else None, C.byref(h)),
              self.ctx.h, "fs_nka_create")
        self.h = h
        self._diag_cb = None
        if diag is not None:
            ctx = self.ctx

            def _cb(user, xh, res):
                v = Vector.__new__(Vector)
                v.ctx = ctx
                v.h = C.c_void_p(xh)
                try:
                    return 1 if diag(v, res) else 0
                finally:
                    v.h = None

            self._diag_cb = _lib.DIAG_FN(_cb)
            check(lib().fs_nka_set_diagnostic(self.h, self._diag_cb, None), self.ctx.h)

    def apply(self, f: Vector, u: Vector) -> SolveInfo:
        info = _lib.SolveInfo()
        st = lib().fs_nka_apply(self.h, f.h, u.h, C.byref(info))
        out = _info(info)
        if st != _lib.OK:
            err = _lib.FsError(st, (lib().fs_last_error(self.ctx.h) or b"").decode())
            err.info = out
            raise err
        return out

    __call__ = apply

    def reset(self):
        check(lib().fs_nka_reset(self.h), self.ctx.h)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().fs_nka_destroy(self.h)
                self.h = None
        except Exception:
            pass


def _nka_settings(maxiter=100, rtol=0.0, atol=0.0, use_zero_guess=False, max_dim=0,
                  angle_tol=0.9, max_fun_evals=0, freeze_pc=True, use_qr=False,
                  use_damping=False, adaptive_damping=False, damping_factor=1.0):
    """nka::settings with the reference's option defaults (nka.hh:536-552)."""
    s = _lib.NkaSettings()
    check(lib().fs_nka_settings_default(C.byref(s)))
    s.base = _lib.SolverSettings(int(maxiter), float(rtol), float(atol), int(bool(use_zero_guess)))
    s.max_dim, s.angle_tol, s.max_fun_evals = int(max_dim), float(angle_tol), int(max_fun_evals)
    s.freeze_pc, s.use_qr = int(bool(freeze_pc)), int(bool(use_qr))
    s.use_damping, s.adaptive_damping = int(bool(use_damping)), int(bool(adaptive_damping))
    s.damping_factor = float(damping_factor)
    return s


class _NkaFactory:
    def __init__(self, settings, work):
        self.settings = settings
        self.work = work

    def __call__(self, F, P=None, diag=None, residual=None, ctx=None) -> NkaSolver:
        return NkaSolver(self.settings, F, P, diag, residual, ctx)

    bind = __call__


# nka::settings / make_work / solver (nka.hh:514-597); the work vectors
# ((dim_bound + 1) * 2 + nwork) are owned by the bound solver
nka = SimpleNamespace(
    settings=_nka_settings,
    make_work=lambda b, dim_bound=10: Work(len(b), 3 + 2 * (dim_bound + 1)),
    solver=lambda settings, work=None: _NkaFactory(settings, work),
    nwork=3)

