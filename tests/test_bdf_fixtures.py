"""The BDF fixtures (tests/golden/bdf_*.npz, made by make_bdf_golden.py from
the reference's own integrator) against the reference test's expectations
(time-integrators/test/implicit.cc:114-131) and for internal consistency."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "bdf_golden.json").read_text())


def test_reference_test_expectations():
    c2, c5 = META["cases"]["rate_bdf2"], META["cases"]["rate_bdf5"]
    exact = 3.0 * math.exp(-1.0)
    x2 = np.load(GOLD / "bdf_rate_bdf2.npz")["x"]
    x5 = np.load(GOLD / "bdf_rate_bdf5.npz")["x"]
    # implicit.cc: BDF2 error < 1e-3 in <= 49 steps with <= 7 rejects;
    # BDF5 error < 1e-7 in exactly 48 steps with 14 rejects
    assert abs(x2[0] - exact) < 1e-3 and c2["steps"] <= 49 and c2["rejects"] <= 7
    assert abs(x5[0] - exact) < 1e-7 and c5["steps"] == 48 and c5["rejects"] == 14


@pytest.mark.parametrize("name", sorted(META["cases"]))
def test_fixture_consistency(name):
    c = META["cases"][name]
    z = np.load(GOLD / f"bdf_{name}.npz")
    acc = z["accepted"]
    assert len(acc) == c["attempts"]
    assert int(acc.sum()) == c["steps"]
    assert c["attempts"] - c["steps"] == c["rejects"] or c["aborted"]
    # time advances exactly by the accepted steps
    t = z["t"]
    for k in range(1, len(t)):
        want = t[k - 1] + (z["dt"][k - 1] if acc[k - 1] else 0.0)
        assert t[k] == want
    if not c["aborted"]:
        assert t[-1] + z["dt"][-1] == pytest.approx(c["final_time"], rel=1e-12)
