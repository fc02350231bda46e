"""ORACLE -- test infrastructure only.

numpy restatement of flecsolve's BDF time integrator
(flecsolve/time-integrators/bdf.hh:49-948, bdf.cc:5-21, the settings rules of
bdf_parameters.hh:57-110) for checking, on the CPU, the step controller that
the device integrator runs on its host side.  Only ``tests/`` uses it.

Vectors are numpy arrays and every vector operation is an elementwise numpy
expression with one rounding per operation, in the reference's order, so with
the same time solver the restatement follows the reference's accept / reject
decisions and step sizes bit for bit.  The reference's quirks are kept (BDF6's
coefficient, alpha overwritten by the BDF source term, the relative-change
norm taken from the scratch function vector); the step-reject counters start
at 0 / false, the values its test's expectations correspond to.
"""
from __future__ import annotations

import math
import sys

import numpy as np

CN, BE = 0, 1
AB2, LEAPFROG = 0, 1
TRUNCATION_ERROR, CONSTANT, FINAL_CONSTANT, LIMIT_RELATIVE_CHANGE = 0, 1, 2, 3
H211B, PC4_7, PC11, DEADBEAT = 0, 1, 2, 3
FIXED_RESOLUTION, FIXED_SCALING = 0, 1
NORM_INF = 0
EPS = sys.float_info.epsilon


def memory_size(m):  # bdf.cc:5-8
    return 1 if m == CN else m


def order(m):  # bdf.cc:10-21
    return 2 if m == CN else (1 if m == BE else m)


class Integrator:
    """bdf::integrator over numpy vectors.  ``rhs(u)`` returns f(u);
    ``solve(gamma, b, x0)`` returns (x, success) for x - gamma f(x) = b."""

    def __init__(self, s: dict, n: int, rhs, solve):
        self.s = dict(s)
        self._validate()
        self.n, self.rhs, self.solve = n, rhs, solve
        z = lambda: np.zeros(n)  # noqa: E731
        self.w = {k: z() for k in ("rhs", "source", "sol", "scratch", "prev_fn", "curr_fn", "scratch_fn",
                                   "old_td", "predict", "td")}
        self.len = memory_size(self.s["integrator"])
        self.hist = [z() for _ in range(self.len)]
        self.hist_dt = [0.0] * self.len
        self.pos = 0
        self.current_time = self.s["initial_time"]
        self.current_dt = self.old_dt = self.s["initial_dt"]
        self.step = 0
        self.prev_successive_rejects, self.current_steprejects = False, 0
        self.tte = self.prev_tte = self.alpha = self.ratio = 0.0
        self.first_step, self.gamma, self.solver_success = False, 0.0, False
        self.total_steprejects, self.fc_interval = 0, 1

    # settings::validate, bdf_parameters.hh:57-110 (asserts become ValueError)
    def _validate(self):
        s = self.s
        if memory_size(s["starting_integrator"]) != 1:
            raise ValueError("Starting integrator must be CN or BE")
        if s["use_predictor"]:
            s["calculate_time_trunc_error"] = True
        if s["timestep_strategy"] == TRUNCATION_ERROR:
            s["calculate_time_trunc_error"] = True
            s["use_predictor"] = True
        else:
            s["control_timestep_variation"] = False
            s["use_pi_controller"] = False
        if s["calculate_time_trunc_error"]:
            s["use_predictor"] = True
        if s["use_predictor"]:
            if memory_size(s["integrator"]) > 1 and s["predictor"] != LEAPFROG:
                raise ValueError("Only the leapfrog predictor is supported for BDF2-6")
            if s["integrator"] == CN and s["predictor"] != AB2:
                raise ValueError("CN supports only ab2")

    def prev(self, i):
        return self.hist[(self.pos - 1 - i) % self.len]

    def prev_dt(self, i):
        return self.hist_dt[(self.pos - 1 - i) % self.len]

    def current_integrator(self):  # bdf.hh:216-226
        if self.step == 0:
            return self.s["starting_integrator"]
        if self.step + 1 < memory_size(self.s["integrator"]):
            return self.step + 1
        return self.s["integrator"]

    def _norm(self, v):
        if self.s["time_trunc_err_norm"] == NORM_INF:
            return float(np.max(np.abs(v)))
        # the serial vectors' dot: products summed left to right
        # (vectors/seq.hh:282-304), then the square root
        acc = 0.0
        for e in v.tolist():
            acc += e * e
        return math.sqrt(acc)

    # predictors (bdf.hh:542-600)
    def _forward_euler(self):
        w = self.w
        if self.first_step:
            w["scratch"][:] = self.prev(0)
            w["curr_fn"][:] = self.rhs(w["scratch"])
            w["td"][:] = w["curr_fn"]
        w["predict"][:] = self.prev(0)
        w["predict"][:] = self.current_dt * w["td"] + w["predict"]

    def _ab2(self):
        w = self.w
        r = self.current_dt / self.old_dt
        a = self.current_dt * (2. + r) / 2.
        b = -self.current_dt * r / 2.
        w["predict"][:] = a * w["curr_fn"] + b * w["old_td"]
        w["predict"][:] = w["predict"] + self.prev(0)

    def _leapfrog(self):
        w = self.w
        r = self.current_dt / self.old_dt
        a = r * r
        b = 1. - a
        g = (1. + r) * self.current_dt
        w["predict"][:] = a * self.prev(1) + b * self.prev(0)
        w["predict"][:] = g * w["td"] + w["predict"]

    def _evaluate_predictor(self):  # bdf.hh:504-540
        integ = self.s["integrator"]
        if integ == CN:
            if self.s["predictor"] == AB2:
                self._ab2()
        elif integ == BE or self.first_step:
            self._forward_euler()
        elif self.s["predictor"] == LEAPFROG:
            self._leapfrog()

    # time derivative (bdf.hh:449-502)
    def _estimate_td(self):
        w, ci = self.w, self.current_integrator()
        if ci == CN:
            w["td"][:] = -1. * self.prev(0) + w["sol"]
            w["td"][:] = (2. / self.current_dt) * w["td"] + (-1.) * w["prev_fn"]
        elif ci == BE:
            w["td"][:] = -1. * self.prev(0) + w["sol"]
            w["td"][:] = w["td"] * (1. / self.current_dt)
        else:
            dtt = self.current_dt / self.old_dt
            a = (2. * dtt + 1.) / ((dtt + 1.) * self.current_dt)
            b = -(dtt + 1.) / self.current_dt
            g = (dtt * dtt) / ((dtt + 1.) * self.current_dt)
            w["td"][:] = a * w["sol"] + b * self.prev(0)
            w["td"][:] = g * self.prev(1) + w["td"]

    # source term and gamma (bdf.hh:264-447)
    def _source(self):
        w, ci = self.w, self.current_integrator()
        m = memory_size(ci)
        h = [self.current_dt]
        for i in range(1, m):
            h.append(h[i - 1] + self.prev_dt(i - 1))
        f = w["source"]
        if ci == BE:
            f[:] = -1. * self.prev(0)
            self.gamma = self.current_dt
        elif ci == CN:
            eps = 0.0
            a, b = 0.5 * self.current_dt + eps, 0.5 * self.current_dt - eps
            f[:] = b * w["prev_fn"] + self.prev(0)
            f[:] = f * -1.
            self.gamma = a
        else:
            k = m
            nn = []
            for i in range(k):
                p = None
                for c in range(1, k):
                    hv = h[(i + c) % k]
                    p = hv if p is None else p * hv
                nn.append(p)
            ssum = nn[0]
            for i in range(1, k):
                ssum = ssum + nn[i]
            self.alpha = ssum
            prod = h[0]
            for i in range(1, k):
                prod = prod * h[i]
            a0 = prod / self.alpha
            for i in range(k):
                den = self.alpha
                for j in range(k):
                    if j != i:
                        hj, hi = (h[0], h[4]) if (k == 6 and i == 5 and j == 0) else (h[j], h[i])
                        den = den * (hj - hi)
                ai = -(nn[i] * nn[i]) / den
                if i == 0:
                    f[:] = ai * self.prev(0)
                else:
                    f[:] = ai * self.prev(i) + f
            self.gamma = a0

    def _initial_guess(self, first):  # bdf.hh:228-262
        w = self.w
        self.first_step = first
        if self.current_integrator() == CN:
            w["scratch"][:] = self.prev(0)
            w["prev_fn"][:] = self.rhs(w["scratch"])
        if self.s["use_predictor"]:
            if first and not self.s["use_initial_predictor"]:
                w["predict"][:] = self.prev(0)
            else:
                self._evaluate_predictor()
            w["sol"][:] = w["predict"]
        else:
            w["sol"][:] = self.prev(0)
        self._source()

    def advance(self, dt, first, curr):  # bdf.hh:74-94
        if not (self.step < self.s["max_steps"] and self.current_time < self.s["final_time"]):
            raise RuntimeError("already finished integrating")
        w = self.w
        self.prev(0)[:] = curr
        self.current_dt = dt
        self._initial_guess(first)
        w["rhs"][:] = -1. * w["source"]
        x, ok = self.solve(self.gamma, w["rhs"].copy(), w["sol"].copy())
        w["sol"][:] = x
        self.solver_success = bool(ok)
        return w["sol"].copy()

    # truncation error (bdf.hh:689-746)
    def _lte_factor(self):
        s = self.s
        if self.first_step:
            if s["starting_integrator"] == BE:
                return 0.5
            if s["starting_integrator"] == CN:
                ef = 1.5
                return ef * self.current_dt
            return 0.
        if s["predictor"] == LEAPFROG:
            return (1. + self.alpha) / (2. + 3. * self.alpha)
        return 2. / (6. - 1. / ((self.alpha + 1) * (self.alpha + 1)))

    def _scaled_norm(self, x, y):
        s, w = self.s, self.w
        if s["time_error_scaling"] == FIXED_RESOLUTION:
            w["scratch"][:] = s["time_rtol"] * x + s["time_atol"]
        else:
            w["scratch"][:] = (x + s["problem_scale"]) * s["time_rtol"]
        w["scratch_fn"][:] = (x - y) / w["scratch"]
        return self._norm(w["scratch_fn"])

    def _tte(self):
        s = self.s
        if self.step > 0 or (self.first_step and s["use_initial_predictor"]):
            self.alpha = self.current_dt / self.old_dt
            ef = self._lte_factor()
            y = self.prev(0) if (self.first_step and s["starting_integrator"] == CN) else self.w["predict"]
            est = self._scaled_norm(self.w["sol"], y) * ef
            self.prev_tte = self.tte
            self.tte = max(EPS, est)
            self.ratio = self.prev_tte / self.tte
        else:
            self.prev_tte = self.tte = self.ratio = 1.

    def check_solution(self):  # bdf.hh:98-130
        ok = False
        if self.solver_success:
            if self.s["calculate_time_trunc_error"]:
                self._tte()
            if self.s["timestep_strategy"] == TRUNCATION_ERROR:
                ok = self.tte <= 1.0
                if ok:
                    self.prev_successive_rejects = self.current_steprejects > 1
                    self.current_steprejects = 0
                else:
                    self.current_steprejects += 1
            else:
                ok = True
        else:
            self.current_steprejects += 1
        if not ok:
            self.total_steprejects += 1
        return ok

    def update(self):  # bdf.hh:132-146
        self.current_time += self.current_dt
        if self.s["use_predictor"]:
            if self.s["predictor"] == AB2:
                self.w["old_td"], self.w["curr_fn"] = self.w["curr_fn"], self.w["old_td"]
            self._estimate_td()
        self.hist[self.pos][:] = self.w["sol"]
        self.hist_dt[self.pos] = self.current_dt
        self.pos = (self.pos + 1) % self.len
        self.step += 1

    # step sizes (bdf.hh:148-211, 602-687)
    def _dynamical(self, dt):
        w = self.w
        w["scratch"][:] = self.prev(0) + EPS
        w["scratch"][:] = self.prev(1) / w["scratch"]
        w["scratch"][:] = w["scratch"] + -1
        w["scratch"][:] = np.abs(w["scratch"])
        change = self._norm(w["scratch_fn"])
        factor = 1.05 if dt > 0.5 else 1.1
        factor = 1.03 if dt > 10. else factor
        with np.errstate(divide="ignore"):
            cfl = math.sqrt(self.s["target_relative_change"] / change) * dt if change > 0 else math.inf
        return min(cfl, factor * dt)

    def _from_tte(self, dt, good):
        s = self.s
        p = float(order(self.current_integrator()))
        if s["use_pi_controller"] and good and not self.prev_successive_rejects:
            sf = 0.8
            t = s["pi_controller_type"]
            if t == H211B:
                b = 4.
                f = math.pow(sf / max(self.tte, EPS), 1. / (b * (p + 1.)))
                f *= math.pow(sf / max(self.prev_tte, EPS), 1. / (b * (p + 1.)))
                f *= math.pow(self.alpha, -0.25)
            elif t == PC4_7:
                f = math.pow(sf / max(self.tte, EPS), 0.4 / (p + 1.))
                f *= math.pow(self.ratio, 0.7 / (p + 1.)) * self.alpha
            elif t == PC11:
                f = math.pow(sf / max(self.tte, EPS), 1.0 / (p + 1.))
                f *= math.pow(self.ratio, 1. / (p + 1.)) * self.alpha
            else:
                f = math.pow(sf / max(self.tte, EPS), 1. / (p + 1.))
        else:
            f = math.pow(0.8 / max(self.tte, EPS), 1. / (p + 1.))
        if s["control_timestep_variation"] and not s["use_pi_controller"]:
            if abs(1. - f) < 0.1:
                f = 1.
        return dt * f

    def get_next_dt(self, good):
        s = self.s
        tmp = self.current_dt
        if s["timestep_strategy"] == TRUNCATION_ERROR:
            if good:
                self.current_dt = self._from_tte(self.current_dt, good)
                if s["max_dt"] < self.current_dt:
                    self.current_dt = s["max_dt"]
            elif self.solver_success:
                self.current_dt = self._from_tte(self.current_dt, good)
            else:
                self.current_dt = s["dt_cut_lower_bound"] * self.current_dt
            self._evaluate_predictor()
        else:
            if good:
                if s["timestep_strategy"] == CONSTANT:
                    self.current_dt = s["initial_dt"]
                elif s["timestep_strategy"] == FINAL_CONSTANT:
                    if self.fc_interval < s["number_of_time_intervals"]:
                        self.current_dt = s["initial_dt"] + float(self.fc_interval) / float(
                            s["number_of_time_intervals"]) * (s["max_dt"] - s["initial_dt"])
                        self.fc_interval += 1
                    else:
                        self.current_dt = s["max_dt"]
                elif s["timestep_strategy"] == LIMIT_RELATIVE_CHANGE:
                    self.current_dt = self._dynamical(self.current_dt)
            else:
                self.current_dt = 0.
        if good:
            self.old_dt = tmp
        self.current_dt = min(min(self.current_dt, s["max_dt"]), s["final_time"] - self.current_time)
        return self.current_dt


def settings(**kw) -> dict:
    """bdf::settings with the option defaults (bdf_parameters.hh:121-156)"""
    s = dict(use_predictor=True, use_initial_predictor=True, predictor=LEAPFROG,
             timestep_strategy=TRUNCATION_ERROR, dt_cut_lower_bound=0.58754407, number_of_time_intervals=100,
             integrator=2, starting_integrator=CN, calculate_time_trunc_error=False,
             time_trunc_err_norm=NORM_INF, target_relative_change=0.0, use_pi_controller=True,
             pi_controller_type=PC4_7, control_timestep_variation=False, time_error_scaling=FIXED_SCALING,
             time_rtol=1e-9, time_atol=1e-15, problem_scale=0.0, max_dt=sys.float_info.max,
             min_dt=sys.float_info.min, initial_dt=0.0)
    s.update(kw)
    return s
