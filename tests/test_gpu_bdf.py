"""The device BDF integrator against the reference's own integrator.

Fixtures (tests/golden/bdf_*.npz, make_bdf_golden.py) hold, per attempted
step, the reference's time, dt and acceptance, and its final solution:
* the scalar decay of time-integrators/test/implicit.cc (its rate operator
  and exact time solver, here on device vectors through the callback
  interface) at implicit.cfg's two settings and at settings covering BE, CN,
  BDF2-6, the AB2 / leapfrog / forward-Euler predictors, the H211b / PC.4.7 /
  PC11 / deadbeat controllers, both error scalings, both norms and the
  constant / final-constant / limit-relative-change strategies: the same
  accept / reject sequence,
  steps and rejects, times, steps and the solution to 1e-6; CN reaching
  max_steps (where the reference asserts) the same attempts up to that
  point; BDF6, whose coefficient typo makes the reference reject every step
  until dt underflows, the same first 20 attempts and the same collapse;
* the heat equation u' = -A u with the time operator I + gamma A on the
  device solved by device CG (the linear form): the same steps and rejects,
  dt to 1e-6, the solution to 1e-8; the mixed-precision CG as the time
  solver reaches the same final time within the same error bar."""
import json
from pathlib import Path

import numpy as np
import pytest

import flecsolve_gb300 as fs
from flecsolve_gb300 import problems as P
from flecsolve_gb300._lib import FsError
from flecsolve_gb300.time_integrator import bdf

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "bdf_golden.json").read_text())
# the device vector kernels fuse a x + b y into one rounding where the
# reference rounds twice; the error estimate divides the small difference of
# the solution and its prediction, so those last-bit differences reach the
# step sizes at about 1e-8 over a run
TOL = 1e-6


def _settings(c):
    return bdf.settings(**{
        "initial-time": c["initial_time"], "final-time": c["final_time"], "initial-dt": c["initial_dt"],
        "max-steps": c["max_steps"], "min-dt": c["min_dt"], "max-dt": c["max_dt"],
        "timestep-selection-strategy": c["strategy"], "integrator": c["method"],
        "starting-integrator": c["starting"], "calculate-time-trunc-error": False,
        "time-trunc-error-norm": c["norm"], "predictor": c["predictor"], "use-predictor": True,
        "problem-scales": [c["problem_scale"]], "trunc-error-rtol": c["rtol"], "trunc-error-atol": c["atol"],
        "time-error-scaling": c["scaling"], "pi-controller-type": c["controller"],
        "use-pi-controller": c["pi"], "control-timestep-variation": c["control_var"],
        "dt-cut-lower-bound": c["dt_cut"], "target-relative-change": c.get("target", 0.0)})


class Rate:
    """implicit.cc:14-51: f(u) = lambda u with the time operator's scaling"""

    def __init__(self, lam):
        self.lam, self.gamma = lam, 1.0

    def apply_rhs(self, u, f):
        f.scale(self.lam, u)

    def set_scaling(self, g):
        self.gamma = g


class RateSolver:
    """implicit.cc:55-73: the exact solve of u - gamma lambda u = b"""

    def __init__(self, F):
        self.F = F

    def apply(self, b, x):
        rhs = b.min().get()
        x.set_scalar(rhs / (1. - self.F.lam * self.F.gamma))
        return fs.SolveInfo("converged_atol", 0, 0, 0., 0., 0., 0., 0.)


def _drive(ti, x, xnew, limit):
    """the loop of implicit.cc:90-113, recording every attempt"""
    rec = []
    dt = ti.get_current_dt()
    first = True
    aborted = False
    while ti.get_current_time() < ti.get_final_time() and len(rec) < limit:
        t = ti.get_current_time()
        try:
            ti.advance(dt, first, x, xnew)
        except FsError:
            aborted = True
            break
        good = ti.check_solution()
        rec.append((t, dt, int(good)))
        if good:
            ti.update()
            x, xnew = xnew, x
            first = False
        dt = ti.get_next_dt(good)
    return rec, x, aborted


RATE_CASES = sorted(n for n, c in META["cases"].items() if c["problem"] == "rate")


@pytest.mark.parametrize("name", RATE_CASES)
def test_rate_problem_matches_reference(ctx, name):
    c = META["cases"][name]
    z = np.load(GOLD / f"bdf_{name}.npz")
    r = META["rate"]
    F = Rate(r["lam"])
    x, xnew = fs.Vector(ctx, r["n"]), fs.Vector(ctx, r["n"])
    ti = bdf.integrator(bdf.parameters(_settings(c), F, bdf.make_work(x), RateSolver(F)))
    x.set_scalar(r["ic"])
    rec, x, aborted = _drive(ti, x, xnew, c["attempts"])
    rec = np.array(rec)
    assert len(rec) == c["attempts"]
    if name == "rate_bdf6":
        # the reference's BDF6 coefficient typo: every step fails the error
        # test and dt collapses; the rejections are chaotic, so the first
        # attempts agree and both runs end with dt underflowing
        k = 20
        assert np.array_equal(rec[:k, 2].astype(int), z["accepted"][:k])
        assert np.allclose(rec[:k, 1], z["dt"][:k], rtol=TOL)
        assert rec[-1, 1] < 1e-20 and z["dt"][-1] < 1e-20
        return
    assert np.array_equal(rec[:, 2].astype(int), z["accepted"])
    assert np.allclose(rec[:, 0], z["t"], rtol=TOL, atol=1e-300)
    assert np.allclose(rec[:, 1], z["dt"], rtol=TOL, atol=1e-300)
    if not c["aborted"]:
        assert not aborted
        assert ti.get_current_step() == c["steps"] and ti.num_step_rejects() == c["rejects"]
        assert np.allclose(x.numpy(), z["x"], rtol=TOL, atol=0)


HEAT_CASES = sorted(n for n, c in META["cases"].items() if c["problem"] == "heat")


def _heat(ctx, c, solver_ns=fs.cg, rtol=None):
    h = META["heat"]
    A, _ = P.workload(h["workload"])
    J = fs.CSR(ctx, P.CSR(A.nrows, A.ncols, A.rowptr, A.col, -A.val))  # f(u) = -A u
    ks = solver_ns.settings(maxiter=h["cg_maxiter"], rtol=rtol or h["cg_rtol"], use_zero_guess=False)
    ti = bdf.linear(_settings(c), J, ks, P=None)
    x, xnew = fs.Vector(ctx, A.nrows), fs.Vector(ctx, A.nrows)
    x.upload(P.uniform(h["seed"], A.nrows, 0.0, 1.0))
    rec, x, aborted = _drive(ti, x, xnew, 100000)
    return ti, np.array(rec), x.numpy(), aborted


@pytest.mark.parametrize("name", HEAT_CASES)
def test_heat_linear_form_matches_reference(ctx, name):
    c = META["cases"][name]
    z = np.load(GOLD / f"bdf_{name}.npz")
    ti, rec, x, aborted = _heat(ctx, c)
    assert not aborted
    assert ti.get_current_step() == c["steps"] and ti.num_step_rejects() == c["rejects"]
    assert np.array_equal(rec[:, 2].astype(int), z["accepted"])
    assert np.allclose(rec[:, 1], z["dt"], rtol=1e-6, atol=0)
    assert np.linalg.norm(x - z["x"]) / np.linalg.norm(z["x"]) < 1e-8


def test_heat_with_mixed_precision_time_solver(ctx):
    c = META["cases"]["heat_bdf2"]
    z = np.load(GOLD / "bdf_heat_bdf2.npz")
    ti, rec, x, aborted = _heat(ctx, c, fs.mixed_cg, rtol=1e-10)
    assert not aborted
    assert ti.get_current_time() == pytest.approx(c["final_time"], rel=1e-12)
    assert abs(ti.get_current_step() - c["steps"]) <= 2
    assert np.linalg.norm(x - z["x"]) / np.linalg.norm(z["x"]) < 1e-6


def test_invalid_settings_and_misuse(ctx):
    c = dict(META["cases"]["rate_bdf2"])
    F = Rate(-1.0)
    x = fs.Vector(ctx, 4)
    # BDF2-6 with the AB2 predictor: the reference asserts
    with pytest.raises(Exception):
        bdf.integrator(bdf.parameters(_settings(dict(c, predictor="ab2")), F, x, RateSolver(F)))
    # a starting integrator with history
    with pytest.raises(Exception):
        bdf.integrator(bdf.parameters(_settings(dict(c, starting="BDF2")), F, x, RateSolver(F)))
    ti = bdf.integrator(bdf.parameters(_settings(c), F, x, RateSolver(F)))
    with pytest.raises(Exception):
        ti.advance(0.1, True, x, x)
