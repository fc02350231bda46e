"""The numpy restatement of the BDF integrator (oracle/bdf_oracle.py)
against the reference's own integrator (tests/golden/bdf_*.npz, made by
make_bdf_golden.py from oracle/_ref/ref_bdf).

* Decay problems with the reference test's exact time solver
  (time-integrators/test/implicit.cc:55-73): the same attempts, acceptance,
  times and steps bit for bit, and the same solution; where the reference
  aborted, the same attempts up to that point.
* Heat problems: the restatement with an exact sparse solve of the time
  operator against the reference with its CG at rtol 1e-12: the same
  accept / reject sequence, steps to 1e-6 (the error estimate divides the
  small difference of solution and prediction, which magnifies the CG's
  residual)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import bdf_oracle as B
from flecsolve_gb300 import problems as P

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "bdf_golden.json").read_text())
METHOD = {"CN": 0, "BE": 1, "BDF2": 2, "BDF3": 3, "BDF4": 4, "BDF5": 5, "BDF6": 6}


def _settings(c):
    return B.settings(
        initial_time=c["initial_time"], final_time=c["final_time"], initial_dt=c["initial_dt"],
        max_steps=c["max_steps"], min_dt=c["min_dt"], max_dt=c["max_dt"],
        timestep_strategy={"truncation-error": 0, "constant": 1, "final-constant": 2,
                           "limit-relative-change": 3}[c["strategy"]],
        integrator=METHOD[c["method"]], starting_integrator=METHOD[c["starting"]],
        predictor={"ab2": 0, "leapfrog": 1}[c["predictor"]],
        pi_controller_type={"H211b": 0, "PC.4.7": 1, "PC11": 2, "Deadbeat": 3}[c["controller"]],
        time_error_scaling={"fixed-resolution": 0, "fixed-scaling": 1}[c["scaling"]],
        time_trunc_err_norm={"inf": 0, "l2": 1, "l1": 2}[c["norm"]],
        use_pi_controller=c["pi"], control_timestep_variation=c["control_var"], time_rtol=c["rtol"],
        time_atol=c["atol"], problem_scale=c["problem_scale"], dt_cut_lower_bound=c["dt_cut"],
        target_relative_change=c.get("target", 0.0))


def _drive(ti, x, limit):
    rec, dt, first, aborted = [], ti.current_dt, True, False
    while ti.current_time < ti.s["final_time"] and len(rec) < limit:
        t = ti.current_time
        try:
            xnew = ti.advance(dt, first, x)
        except RuntimeError:
            aborted = True
            break
        good = ti.check_solution()
        rec.append((t, dt, int(good)))
        if good:
            ti.update()
            x = xnew
            first = False
        dt = ti.get_next_dt(good)
    return np.array(rec), x, aborted


@pytest.mark.parametrize("name", sorted(n for n, c in META["cases"].items() if c["problem"] == "rate"))
def test_rate_restatement_matches_reference(name):
    c, r = META["cases"][name], META["rate"]
    z = np.load(GOLD / f"bdf_{name}.npz")
    lam = r["lam"]

    def solve(gamma, b, x0):
        # implicit.cc:61-64: the minimum of b over (1 - lambda gamma), everywhere
        return np.full_like(b, b.min() / (1. - lam * gamma)), True

    ti = B.Integrator(_settings(c), r["n"], lambda u: lam * u, solve)
    rec, x, aborted = _drive(ti, np.full(r["n"], r["ic"]), c["attempts"])
    assert len(rec) == c["attempts"]
    assert np.array_equal(rec[:, 2].astype(int), z["accepted"])
    assert np.array_equal(rec[:, 0], z["t"]) and np.array_equal(rec[:, 1], z["dt"])
    if not c["aborted"]:
        assert ti.step == c["steps"] and ti.total_steprejects == c["rejects"]
        assert np.array_equal(x, z["x"])


@pytest.mark.parametrize("name", sorted(n for n, c in META["cases"].items() if c["problem"] == "heat"))
def test_heat_restatement_matches_reference(name):
    c, h = META["cases"][name], META["heat"]
    z = np.load(GOLD / f"bdf_{name}.npz")
    A, _ = P.workload(h["workload"])
    S = A.to_scipy().tocsc()
    I = sp.identity(A.nrows, format="csc")

    def solve(gamma, b, x0):
        return spla.spsolve(I + gamma * S, b), True

    ti = B.Integrator(_settings(c), A.nrows, lambda u: -(S @ u), solve)
    rec, x, aborted = _drive(ti, P.uniform(h["seed"], A.nrows, 0.0, 1.0), 100000)
    assert not aborted
    assert ti.step == c["steps"] and ti.total_steprejects == c["rejects"]
    assert np.array_equal(rec[:, 2].astype(int), z["accepted"])
    assert np.allclose(rec[:, 1], z["dt"], rtol=1e-6, atol=0)
    assert np.linalg.norm(x - z["x"]) / np.linalg.norm(z["x"]) < 1e-9


def test_invalid_settings_raise():
    with pytest.raises(ValueError):
        B.Integrator(B.settings(initial_time=0., final_time=1., max_steps=10, predictor=0, integrator=3), 2,
                     lambda u: u, lambda g, b, x: (b, True))
    with pytest.raises(ValueError):
        B.Integrator(B.settings(initial_time=0., final_time=1., max_steps=10, starting_integrator=2), 2,
                     lambda u: u, lambda g, b, x: (b, True))
    assert math.isclose(B.order(0), 2) and B.memory_size(0) == 1 and B.memory_size(5) == 5
