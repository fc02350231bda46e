"""BDF time integration over device vectors (flecsolve/time-integrators/).

Python mirror of ``time_integrator::bdf`` over the ``fs_bdf_*`` C ABI of
``include/fsgpu.h``:

=========================================================  ==============================================
reference (C++)                                            here
=========================================================  ==============================================
``bdf::options("bdf-2")`` + ``read_config`` keys           ``bdf.settings(**{"initial-time": 0, ...})``
``bdf::integrator(bdf::parameters(s, F, make_work(x),      ``bdf.integrator(bdf.parameters(s, F, x,
solver))``                                                 solver))``
``ti.advance(dt, first_step, x, xnew)``                    ``ti.advance(dt, first_step, x, xnew)``
``ti.check_solution()`` / ``update()`` / ``get_next_dt``   the same names
=========================================================  ==============================================

``F`` is the time operator (``apply_rhs(u, f)`` computes f(u),
``set_scaling(gamma)`` is called before each solve) and ``solver.apply(b,
x)`` solves u - gamma f(u) = b and returns an object with ``success()`` or
``status``, as in the reference's test (time-integrators/test/
implicit.cc:14-73).  For a linear f(u) = J u, ``bdf.linear(s, J,
krylov_settings, P)`` keeps the time operator I - gamma J on the device and
solves it with a bound device Krylov solver.
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from ._lib import check, lib
from .api import CSR, Vector

# the reference's option parsers (bdf_parameters.cc:6-105)
_METHOD = {"CN": 0, "BE": 1, "BDF2": 2, "BDF3": 3, "BDF4": 4, "BDF5": 5, "BDF6": 6}
_PREDICTOR = {"ab2": 0, "leapfrog": 1}
_STRATEGY = {"truncation-error": 0, "constant": 1, "final-constant": 2, "limit-relative-change": 3}
_CONTROLLER = {"H211b": 0, "PC.4.7": 1, "PC11": 2, "Deadbeat": 3}
_SCALING = {"fixed-resolution": 0, "fixed-scaling": 1}
_NORM = {"inf": 0, "l2": 1, "l1": 2}

_KEYS = {
    "initial-time": "initial_time", "final-time": "final_time", "max-steps": "max_steps",
    "max-dt": "max_dt", "min-dt": "min_dt", "initial-dt": "initial_dt",
    "use-predictor": "use_predictor", "has-source-term": "has_source_term",
    "use-initial-predictor": "use_initial_predictor", "predictor": "predictor",
    "timestep-selection-strategy": "timestep_strategy", "dt-cut-lower-bound": "dt_cut_lower_bound",
    "dt-growth-upper-bound": "dt_growth_upper_bound",
    "number-of-time-intervals": "number_of_time_intervals", "integrator": "integrator",
    "starting-integrator": "starting_integrator",
    "calculate-time-trunc-error": "calculate_time_trunc_error",
    "time-trunc-error-norm": "time_trunc_err_norm", "target-relative-change": "target_relative_change",
    "use-pi-controller": "use_pi_controller", "pi-controller-type": "pi_controller_type",
    "control-timestep-variation": "control_timestep_variation",
    "time-error-scaling": "time_error_scaling", "trunc-error-rtol": "time_rtol",
    "trunc-error-atol": "time_atol", "combine-timestep-estimators": "combine_timestep_estimators",
    "problem-scales": "problem_scales",
}


def _enum(table, v, lower=False):
    if isinstance(v, int):
        return v
    key = v.lower() if lower else v
    if key not in table:
        raise ValueError(f"unknown value {v!r}")
    return table[key]


def _bool(v):
    if isinstance(v, str):
        return v.strip().lower() in ("1", "true", "yes", "on")
    return bool(v)


class _Bdf:
    """``time_integrator::bdf``"""

    @staticmethod
    def settings(**kw) -> _lib.BdfSettings:
        """bdf::settings from option names (``"initial-dt"`` or
        ``initial_dt``) with the reference's defaults (bdf_parameters.hh:
        121-156)."""
        s = _lib.BdfSettings()
        check(lib().fs_bdf_settings_default(C.byref(s)))
        for k, v in kw.items():
            f = _KEYS.get(k, _KEYS.get(k.replace("_", "-"), k))
            if f in ("integrator", "starting_integrator"):
                v = _enum(_METHOD, v)
            elif f == "predictor":
                v = _enum(_PREDICTOR, v, lower=True)
            elif f == "timestep_strategy":
                v = _enum(_STRATEGY, v, lower=True)
            elif f == "pi_controller_type":
                v = _enum(_CONTROLLER, v)
            elif f == "time_error_scaling":
                v = _enum(_SCALING, v)
            elif f == "time_trunc_err_norm":
                v = _enum(_NORM, v)
            elif f == "problem_scales":
                vals = [float(x) for x in (v if isinstance(v, (list, tuple)) else [v])]
                if len(vals) > 1:
                    raise ValueError("problem-scales: one component")
                s.num_problem_scales = len(vals)
                s.problem_scale = vals[0] if vals else 0.0
                continue
            elif f in ("use_predictor", "use_initial_predictor", "has_source_term",
                       "calculate_time_trunc_error", "use_pi_controller", "control_timestep_variation",
                       "combine_timestep_estimators"):
                v = int(_bool(v))
            if not hasattr(s, f):
                raise KeyError(k)
            setattr(s, f, v)
        return s

    class parameters:
        """bdf::parameters(settings, op, work, solver) (bdf_parameters.hh:
        158-176); ``work`` is the exemplar vector (``make_work(x)``)."""

        def __init__(self, settings, op, work, solver):
            self.settings, self.op, self.work, self.solver = settings, op, work, solver

    @staticmethod
    def make_work(x: Vector) -> Vector:
        return x

    class integrator:
        """bdf::integrator (bdf.hh:49-777) on the device."""

        def __init__(self, params, *, _linear=None):
            self.ctx = params.work.ctx if _linear is None else _linear[0].ctx
            h = C.c_void_p()
            if _linear is not None:
                J, method, ks, P = _linear
                check(lib().fs_bdf_create_linear(self.ctx.h, C.byref(params.settings), J.h, method,
                                                 C.byref(ks), C.byref(P), C.byref(h)),
                      self.ctx.h, "fs_bdf_create_linear")
                self._cbs = ()
                self._J = J  # the integrator reads J's values at every step
            else:
                op, solver, ctx = params.op, params.solver, self.ctx

                def borrow(hnd):
                    v = Vector.__new__(Vector)
                    v.ctx = ctx
                    v.h = C.c_void_p(hnd)
                    return v

                def rhs_cb(user, uh, fh):
                    u, f = borrow(uh), borrow(fh)
                    try:
                        op.apply_rhs(u, f)
                        return 0
                    except Exception:
                        return _lib.ERR_INVALID_ARG
                    finally:
                        u.h = f.h = None

                def solve_cb(user, gamma, bh, xh, succ):
                    b, x = borrow(bh), borrow(xh)
                    try:
                        op.set_scaling(gamma)
                        info = solver.apply(b, x)
                        ok = info.success() if hasattr(info, "success") and callable(info.success) \
                            else getattr(info, "status", "") in ("converged_atol", "converged_rtol",
                                                                  "converged_user")
                        succ[0] = 1 if ok else 0
                        return 0
                    except Exception:
                        return _lib.ERR_INVALID_ARG
                    finally:
                        b.h = x.h = None

                self._cbs = (_lib.RHS_FN(rhs_cb), _lib.TIME_SOLVE_FN(solve_cb))
                n = len(params.work)
                check(lib().fs_bdf_create(self.ctx.h, C.byref(params.settings), n, self._cbs[0], None,
                                          self._cbs[1], None, C.byref(h)), self.ctx.h, "fs_bdf_create")
            self.h = h

        def __del__(self):
            try:
                if getattr(self, "h", None):
                    lib().fs_bdf_destroy(self.h)
                    self.h = None
            except Exception:
                pass

        def _state(self):
            st = _lib.BdfState()
            check(lib().fs_bdf_state_get(self.h, C.byref(st)), self.ctx.h)
            return st

        def advance(self, dt: float, first_step: bool, curr: Vector, out: Vector):
            check(lib().fs_bdf_advance(self.h, float(dt), int(bool(first_step)), curr.h, out.h),
                  self.ctx.h, "bdf advance")

        def check_solution(self) -> bool:
            ok = C.c_int()
            check(lib().fs_bdf_check_solution(self.h, C.byref(ok)), self.ctx.h)
            return bool(ok.value)

        def update(self):
            check(lib().fs_bdf_update(self.h), self.ctx.h)

        def get_next_dt(self, good_solution: bool) -> float:
            dt = C.c_double()
            check(lib().fs_bdf_get_next_dt(self.h, int(bool(good_solution)), C.byref(dt)), self.ctx.h)
            return dt.value

        def get_current_time(self) -> float:
            return self._state().current_time

        def get_final_time(self) -> float:
            return self._state().final_time

        def get_current_dt(self) -> float:
            return self._state().current_dt

        def get_current_step(self) -> int:
            return self._state().current_step

        def num_step_rejects(self) -> int:
            return self._state().num_step_rejects

        def get_time_operator_scaling(self) -> float:
            return self._state().gamma

        def last_solver_iters(self) -> int:
            return self._state().solver_iters

    @classmethod
    def linear(cls, settings, J: CSR, krylov_settings, P=None):
        """The integrator for f(u) = J u with the time operator I - gamma J on
        the device, solved by a Krylov solver bound to it: ``krylov_settings``
        from a solver namespace's ``settings(...)`` (``fs.cg``,
        ``fs.mixed_cg``, ``fs.bicgstab``, ``fs.gmres``, ...; its method is the
        solver's), ``P`` ``fs.op.jacobi`` or None."""
        from . import api
        if P is None or P is api.op.I:
            pc = _lib.Precond(_lib.PRECOND_NONE, None, None)
        elif P is api.op.jacobi:
            pc = _lib.Precond(_lib.PRECOND_JACOBI, None, None)
        else:
            raise ValueError("P: fs.op.jacobi or None")
        params = cls.parameters(settings, J, None, None)
        return cls.integrator(params, _linear=(J, krylov_settings._method, krylov_settings, pc))


bdf = _Bdf()
