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

__all__ = ["Context", "Vector", "CSR", "SolveInfo", "Future", "op", "vec", "mat",
           "cg", "bicgstab", "gmres", "mixed_cg", "mixed_bicgstab", "mixed_gmres"]


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


class CSR:
    """Device CSR operator (``op::core<mat::csr<double>>``)."""

    def __init__(self, ctx: Context, A):
        self.ctx = ctx
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

    def apply(self, x: Vector, y: Vector, exact: bool = False):
        """y = A x (op::core::apply, operators/core.hh:107-116)."""
        check(lib().fs_csr_spmv(self.h, x.h, y.h, _lib.SPMV_EXACT if exact else _lib.SPMV_FMA),
              self.ctx.h, "spmv")

    __call__ = apply

    def residual(self, b: Vector, x: Vector, r: Vector):
        """r = b - A x (op::core::residual, operators/core.hh:129-142)."""
        check(lib().fs_csr_residual(self.h, b.h, x.h, r.h), self.ctx.h, "residual")

    def apply_transpose(self, x: Vector, y: Vector):
        check(lib().fs_csr_spmv_transpose(self.h, x.h, y.h), self.ctx.h, "spmv^T")

    def parcsr_apply(self, parts: int, x: Vector, y: Vector):
        check(lib().fs_parcsr_spmv(self.h, int(parts), x.h, y.h), self.ctx.h, "parcsr spmv")

    def update_values(self, val: np.ndarray):
        v = np.ascontiguousarray(val, dtype=np.float64)
        check(lib().fs_csr_update_values(self.h, v.ctypes.data_as(C.c_void_p)), self.ctx.h)

    def Dinv(self) -> Vector:
        """Diagonal inverse as a vector (util/test/mesh.hh:123-140)."""
        d = Vector(self.ctx, self.nrows)
        check(lib().fs_csr_diag_inv(self.h, d.h), self.ctx.h, "diag_inv")
        return d


# ------------------------------------------------------------- op:: ----

class _Identity:
    """``op::I`` (operators/shell.hh:317-318)."""


class _Jacobi:
    """The D^-1 operator of A (util/test/mesh.hh:123-140)."""


op = SimpleNamespace(I=_Identity(), jacobi=_Jacobi(), ref=lambda A: A, cref=lambda A: A,
                     make_shared=lambda A: A)
vec = SimpleNamespace(make=lambda ctx, a, dtype="f64": Vector(ctx, a, dtype), Vector=Vector)
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
            v = {"mgs": _lib.ORTHO_MGS, "cgs2": _lib.ORTHO_CGS2, "auto": _lib.ORTHO_AUTO}.get(v, v)
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
            pc.kind = _lib.PRECOND_CSR
            pc.op = P.h
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

    def apply(self, b: Vector, x: Vector) -> SolveInfo:
        info = _lib.SolveInfo()
        st = lib().fs_krylov_apply(self.h, b.h, x.h, C.byref(info))
        out = SolveInfo(_lib.STOP_REASONS.get(info.status, str(info.status)), info.iters,
                        info.restarts, info.res_norm_initial, info.res_norm_final,
                        info.sol_norm_initial, info.sol_norm_final, info.rhs_norm)
        if st != _lib.OK:
            err = _lib.FsError(st, (lib().fs_last_error(self.ctx.h) or b"").decode())
            err.info = out
            raise err
        return out

    __call__ = apply

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
mixed_cg = _namespace(_lib.CG_MIXED, 4)     # FP32 inner PCG in FP64 refinement
mixed_bicgstab = _namespace(_lib.BICGSTAB_MIXED, 8)
mixed_gmres = _namespace(_lib.GMRES_MIXED, 104, max_krylov_dim=-1, pre_side="right", restart=False)
