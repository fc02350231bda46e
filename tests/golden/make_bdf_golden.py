"""Generate the BDF time-integrator fixtures in this directory from the
reference.

Runs the reference's own, unmodified BDF integrator
(flecsolve/time-integrators/bdf.hh, bdf.cc, bdf_parameters.cc), compiled with
``make -C oracle ref`` as ``oracle/_ref/ref_bdf``, driven as its test drives
it (time-integrators/test/implicit.cc:90-113), on
* the scalar decay u' = -u, u(0) = 3 of that test with its exact time
  solver, at its two configurations (implicit.cfg [bdf-2] and [bdf-5]) and
  at settings that exercise the other methods, predictors, controllers,
  error scalings, norms and step strategies;
* the heat equation u' = -A u (A the 2-D Poisson matrix) with the time
  operator solved by the reference's CG.
Stores, per attempted step, the time, dt, acceptance and solver iterations,
and the final solution, in ``bdf_<case>.npz``; ``bdf_golden.json`` lists
the cases with their settings, step and reject counts.

Usage (needs the reference headers and sources, i.e. only where they are
mounted):
    python tests/golden/make_bdf_golden.py
"""
from __future__ import annotations

import json
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from flecsolve_gb300 import problems as P  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "ref_bdf"

M = {"CN": 0, "BE": 1, "BDF2": 2, "BDF3": 3, "BDF4": 4, "BDF5": 5, "BDF6": 6}
PRED = {"ab2": 0, "leapfrog": 1}
STRAT = {"truncation-error": 0, "constant": 1, "final-constant": 2, "limit-relative-change": 3}
CTRL = {"H211b": 0, "PC.4.7": 1, "PC11": 2, "Deadbeat": 3}
SCAL = {"fixed-resolution": 0, "fixed-scaling": 1}
NORM = {"inf": 0, "l2": 1, "l1": 2}

# implicit.cfg, both sections
IMPLICIT = dict(initial_time=0.0, final_time=1.0, initial_dt=0.5, max_steps=1000, min_dt=0.001, max_dt=0.5,
                strategy="truncation-error", starting="CN", norm="inf", predictor="leapfrog", problem_scale=1.0,
                rtol=1e-7, atol=1e-5, scaling="fixed-resolution", controller="PC.4.7", pi=True,
                control_var=False, dt_cut=0.58754407)

CASES = {
    "rate_bdf2": dict(IMPLICIT, problem="rate", method="BDF2"),
    "rate_bdf5": dict(IMPLICIT, problem="rate", method="BDF5"),
    "rate_bdf3_pc11_l2": dict(IMPLICIT, problem="rate", method="BDF3", controller="PC11", norm="l2"),
    "rate_bdf4_deadbeat_scaling": dict(IMPLICIT, problem="rate", method="BDF4", controller="Deadbeat",
                                       scaling="fixed-scaling", rtol=1e-5),
    # BDF6's coefficient typo (bdf.hh:431) makes every step fail the error
    # test until dt underflows and advance asserts: the run aborts
    "rate_bdf6": dict(IMPLICIT, problem="rate", method="BDF6"),
    "rate_bdf3_h211b": dict(IMPLICIT, problem="rate", method="BDF3", controller="H211b"),
    "rate_cn_ab2": dict(IMPLICIT, problem="rate", method="CN", predictor="ab2", starting="CN"),
    "rate_be_fe": dict(IMPLICIT, problem="rate", method="BE", starting="BE", rtol=1e-4, atol=1e-4),
    "rate_be_constant": dict(IMPLICIT, problem="rate", method="BE", starting="BE", strategy="constant",
                             initial_dt=0.05, max_dt=0.05),
    "rate_bdf2_final_constant": dict(IMPLICIT, problem="rate", method="BDF2", strategy="final-constant",
                                     initial_dt=0.01, max_dt=0.1),
    "rate_bdf2_nopi": dict(IMPLICIT, problem="rate", method="BDF2", pi=False, control_var=True),
    "rate_bdf2_relchange": dict(IMPLICIT, problem="rate", method="BDF2", strategy="limit-relative-change",
                                initial_dt=0.01, target=1e-2),
    "heat_bdf2": dict(IMPLICIT, problem="heat", method="BDF2", final_time=0.2, initial_dt=1e-3, max_dt=0.05,
                      rtol=1e-4, atol=1e-6),
    "heat_be_constant": dict(IMPLICIT, problem="heat", method="BE", starting="BE", strategy="constant",
                             final_time=0.1, initial_dt=0.01, max_dt=0.01),
}
RATE = dict(lam=-1.0, ic=3.0, n=4)
HEAT = dict(workload="poisson2d-16", seed=17, cg_maxiter=1000, cg_rtol=1e-12)


def run(c):
    with tempfile.TemporaryDirectory() as d:
        i, o = Path(d) / "in", Path(d) / "out"
        with open(i, "wb") as f:
            f.write(struct.pack("<10i", 0 if c["problem"] == "rate" else 1, M[c["method"]], M[c["starting"]],
                                PRED[c["predictor"]], STRAT[c["strategy"]], CTRL[c["controller"]],
                                SCAL[c["scaling"]], NORM[c["norm"]], int(c["pi"]), int(c["control_var"])))
            f.write(struct.pack("<10d", c["initial_time"], c["final_time"], c["initial_dt"], c["max_dt"],
                                c["min_dt"], c["rtol"], c["atol"], c["problem_scale"], c["dt_cut"],
                                c.get("target", 0.0)))
            f.write(struct.pack("<i", c["max_steps"]))
            if c["problem"] == "rate":
                f.write(struct.pack("<2dq", RATE["lam"], RATE["ic"], RATE["n"]))
                n = RATE["n"]
            else:
                A, _ = P.workload(HEAT["workload"])
                n = A.nrows
                u0 = P.uniform(HEAT["seed"], n, 0.0, 1.0)
                f.write(struct.pack("<2q", A.nrows, A.nnz))
                f.write(np.asarray(A.rowptr, "<i8").tobytes())
                f.write(np.asarray(A.col, "<i4").tobytes())
                f.write(np.asarray(A.val, "<f8").tobytes())
                f.write(np.asarray(u0, "<f8").tobytes())
                f.write(struct.pack("<id", HEAT["cg_maxiter"], HEAT["cg_rtol"]))
        subprocess.run([str(REF), str(i), str(o)], check=True)
        b = o.read_bytes()
    steps, rejects, nrec, aborted = struct.unpack_from("<4i", b, 0)
    rec = np.frombuffer(b, np.dtype([("t", "<f8"), ("dt", "<f8"), ("accepted", "<i4"), ("iters", "<i4")]),
                        nrec, 16)
    x = np.frombuffer(b, "<f8", n, 16 + 24 * nrec).copy()
    return steps, rejects, rec, x, bool(aborted)


def main():
    if not REF.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    meta = {"rate": RATE, "heat": HEAT, "cases": {}}
    for name, c in CASES.items():
        steps, rejects, rec, x, aborted = run(c)
        np.savez_compressed(HERE / f"bdf_{name}.npz", t=rec["t"], dt=rec["dt"], accepted=rec["accepted"],
                            iters=rec["iters"], x=x)
        meta["cases"][name] = dict(c, steps=steps, rejects=rejects, attempts=int(len(rec)), aborted=aborted)
        print(f"{name}: steps {steps} rejects {rejects} attempts {len(rec)} aborted {aborted} x[0] {x[0]:.10g}")
    (HERE / "bdf_golden.json").write_text(json.dumps(meta, indent=1) + "\n")


if __name__ == "__main__":
    main()
