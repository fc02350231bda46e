"""ORACLE -- test infrastructure only.

ctypes wrapper over ``oracle/_build/libkrylov_oracle.so`` (the C restatement
of flecsolve's serial Krylov path in ``krylov_oracle.c``) and over the
reference driver ``oracle/_ref/ref_driver`` when it has been built.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from dataclasses import dataclass
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libkrylov_oracle.so"
REF_DRIVER = HERE / "_ref" / "ref_driver"

# solve_info::stop_reason, flecsolve/solvers/solver_settings.hh:64-72
STATUS = {0: "converged_atol", 1: "converged_rtol", 2: "converged_user",
          3: "diverged_dtol", 4: "diverged_iters", 5: "diverged_breakdown",
          6: "unknown", 100: "assert_failed"}


class _Settings(C.Structure):
    _fields_ = [("maxiter", C.c_int), ("rtol", C.c_float), ("atol", C.c_float),
                ("use_zero_guess", C.c_int)]


class _GmresSettings(C.Structure):
    _fields_ = [("base", _Settings), ("max_krylov_dim", C.c_int),
                ("pre_side", C.c_int), ("restart", C.c_int)]


class _Info(C.Structure):
    _fields_ = [("status", C.c_int), ("iters", C.c_int), ("restarts", C.c_int),
                ("res_norm_initial", C.c_float), ("res_norm_final", C.c_float),
                ("sol_norm_initial", C.c_float), ("sol_norm_final", C.c_float),
                ("rhs_norm", C.c_float)]


class _Csr(C.Structure):
    _fields_ = [("nrows", C.c_int64), ("rowptr", C.POINTER(C.c_int64)),
                ("col", C.POINTER(C.c_int32)), ("val", C.POINTER(C.c_double))]


_DIAG_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_int64,
                       C.c_double)


class _Diag(C.Structure):
    _fields_ = [("fn", _DIAG_FN), ("user", C.c_void_p),
                ("hist", C.POINTER(C.c_double)), ("cap", C.c_int64),
                ("count", C.c_int64)]


@dataclass
class Result:
    status: str
    iters: int
    restarts: int
    res_norm_initial: float
    res_norm_final: float
    sol_norm_initial: float
    sol_norm_final: float
    rhs_norm: float
    hist: np.ndarray
    x: np.ndarray


def available() -> bool:
    return LIB.exists()


@lru_cache(maxsize=1)
def lib() -> C.CDLL:
    if not LIB.exists():
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    L = C.CDLL(str(LIB))
    pc = C.POINTER(_Csr)
    dp = C.POINTER(C.c_double)
    L.or_spmv.argtypes = [pc, dp, dp]
    L.or_parcsr_spmv.argtypes = [pc, C.c_int, dp, dp]
    L.or_residual.argtypes = [pc, dp, dp, dp]
    L.or_diag_inv.argtypes = [pc, dp]
    L.or_dot.restype = C.c_double
    L.or_dot.argtypes = [C.c_int64, dp, dp]
    for f in (L.or_cg, L.or_bicgstab):
        f.argtypes = [C.POINTER(_Settings), pc, pc, dp, dp, C.POINTER(_Diag),
                      C.POINTER(_Info)]
    L.or_gmres.argtypes = [C.POINTER(_GmresSettings), pc, pc, dp, dp,
                           C.POINTER(_Diag), C.POINTER(_Info)]
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Mat:
    """Keeps the numpy arrays alive behind an or_csr struct."""

    def __init__(self, A):
        self.rp = np.ascontiguousarray(A.rowptr, dtype=np.int64)
        self.col = np.ascontiguousarray(A.col, dtype=np.int32)
        self.val = np.ascontiguousarray(A.val, dtype=np.float64)
        self.s = _Csr(int(A.nrows), self.rp.ctypes.data_as(C.POINTER(C.c_int64)),
                      self.col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(self.val))


class _DinvMat:
    """D^-1 as a 1-nnz-per-row CSR (flecsolve/util/test/mesh.hh:123-140)."""

    def __init__(self, A):
        n = int(A.nrows)
        d = np.zeros(n)
        m = _Mat(A)  # keeps the converted arrays alive during the call
        lib().or_diag_inv(C.byref(m.s), _dp(d))
        self.rp = np.arange(n + 1, dtype=np.int64)
        self.col = np.arange(n, dtype=np.int32)
        self.val = d
        self.s = _Csr(n, self.rp.ctypes.data_as(C.POINTER(C.c_int64)),
                      self.col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(self.val))


def spmv(A, x):
    m = _Mat(A)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(A.nrows)
    lib().or_spmv(C.byref(m.s), _dp(x), _dp(y))
    return y


def parcsr_spmv(A, parts, x):
    m = _Mat(A)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(A.nrows)
    lib().or_parcsr_spmv(C.byref(m.s), int(parts), _dp(x), _dp(y))
    return y


def residual(A, b, x):
    m = _Mat(A)
    r = np.empty(A.nrows)
    lib().or_residual(C.byref(m.s), _dp(np.ascontiguousarray(b, np.float64)),
                      _dp(np.ascontiguousarray(x, np.float64)), _dp(r))
    return r


def dinv(A):
    return _DinvMat(A).val.copy()


def serial_dot(x, y):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    return lib().or_dot(x.size, _dp(x), _dp(y))


def solve(method, A, b, x0=None, *, maxiter=2000, rtol=1e-8,
          use_zero_guess=True, precond="jacobi", krylov_dim=30,
          side="right", restart=True, diag=None, inner_iters=0, pmat=None) -> Result:
    """Run the oracle solver.  ``diag(x, res) -> bool`` is the optional user
    diagnostic; the residual history is always recorded.  ``pmat``: a CSR
    preconditioner operator (instead of ``precond``).  ``inner_iters`` (FCG
    only): the preconditioner is that many Jacobi-PCG iterations on A."""
    L = lib()
    n = A.nrows
    m = _Mat(A)
    P = _Mat(pmat) if pmat is not None else (_DinvMat(A) if precond == "jacobi" else None)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    hist = np.zeros(maxiter + 1)
    if diag is not None:
        def _fn(user, xp, nn, res):
            return 1 if diag(np.ctypeslib.as_array(xp, shape=(nn,)), res) else 0
        cb = _DIAG_FN(_fn)
    else:
        cb = _DIAG_FN()
    d = _Diag(cb, None, _dp(hist), hist.size, 0)
    info = _Info()
    base = _Settings(int(maxiter), C.c_float(rtol), C.c_float(0.0), int(bool(use_zero_guess)))
    Pp = C.byref(P.s) if P is not None else None
    if method == "cg":
        L.or_cg(C.byref(base), C.byref(m.s), Pp, _dp(b), _dp(x), C.byref(d), C.byref(info))
    elif method == "bicgstab":
        L.or_bicgstab(C.byref(base), C.byref(m.s), Pp, _dp(b), _dp(x), C.byref(d), C.byref(info))
    elif method == "gmres":
        gs = _GmresSettings(base, int(krylov_dim), 0 if side == "left" else 1, int(bool(restart)))
        L.or_gmres(C.byref(gs), C.byref(m.s), Pp, _dp(b), _dp(x), C.byref(d), C.byref(info))
    elif method == "fcg":
        L.or_fcg(C.byref(base), C.byref(m.s), Pp, int(inner_iters), _dp(b), _dp(x), C.byref(d),
                 C.byref(info))
    else:
        raise ValueError(method)
    return Result(STATUS[info.status], info.iters, info.restarts,
                  info.res_norm_initial, info.res_norm_final,
                  info.sol_norm_initial, info.sol_norm_final, info.rhs_norm,
                  hist[: min(d.count, hist.size)].copy(), x)


# ------------------------------------------------------ reference driver --

def ref_available() -> bool:
    return REF_DRIVER.exists()


def write_problem(path, A, b, x0):
    with open(path, "wb") as f:
        np.array([A.nrows, A.nnz], dtype=np.int64).tofile(f)
        np.ascontiguousarray(A.rowptr, np.int64).tofile(f)
        np.ascontiguousarray(A.col, np.int32).tofile(f)
        np.ascontiguousarray(A.val, np.float64).tofile(f)
        np.ascontiguousarray(b, np.float64).tofile(f)
        np.ascontiguousarray(x0, np.float64).tofile(f)


def ref_solve(method, A, b, x0=None, *, maxiter=2000, rtol=1e-8,
              use_zero_guess=True, precond="jacobi", krylov_dim=30,
              side="right", restart=True, inner_iters=0) -> Result:
    """Run the reference's own templates (compiled from its headers)."""
    if not ref_available():
        raise RuntimeError("reference driver not built (oracle/_ref/ref_driver)")
    n = A.nrows
    x0 = np.zeros(n) if x0 is None else x0
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_problem(fin, A, b, x0)
        pname = f"cg{int(inner_iters)}" if inner_iters > 0 else precond
        args = [str(REF_DRIVER), fin, fout, method, str(maxiter), repr(float(rtol)),
                str(int(bool(use_zero_guess))), pname]
        if method == "gmres":
            args += [str(krylov_dim), side, str(int(bool(restart)))]
        subprocess.run(args, check=True, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
        raw = open(fout, "rb").read()
    head = np.frombuffer(raw, np.int32, 3, 0)
    norms = np.frombuffer(raw, np.float32, 5, 12)
    nh = int(np.frombuffer(raw, np.int64, 1, 32)[0])
    hist = np.frombuffer(raw, np.float64, nh, 40).copy()
    x = np.frombuffer(raw, np.float64, n, 40 + 8 * nh).copy()
    return Result(STATUS[int(head[0])], int(head[1]), int(head[2]),
                  float(norms[0]), float(norms[1]), float(norms[2]),
                  float(norms[3]), float(norms[4]), hist, x)


def solve_orders(method, A, b, x0=None, **kw):
    """The oracle solve with its dot products summed in the reference's
    serial order and in two other valid orders (blocks of 4096 then the block
    sums; right to left).  The spread of their iteration counts is the part
    of a count difference that comes from summation order alone (BiCGSTAB
    and GMRES amplify it)."""
    L = lib()
    out = []
    try:
        for order in (0, 1, 2):
            L.or_set_dot_order(order)
            out.append(solve(method, A, b, x0, **kw))
    finally:
        L.or_set_dot_order(0)
    return out

