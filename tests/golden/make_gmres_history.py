"""The reference's GMRES(30) residual estimates on convdiff3d-192.

Runs the reference's own serial GMRES(30) (oracle/_ref/ref_driver: gmres.hh
over vec::seq_vec and mat::csr<double>, right Jacobi, restart, rtol 1e-8) on
the 192^3 convection-diffusion workload and records the residual estimate
|dw[k+1]| that its diagnostic sees at every step (gmres.hh:193-196): every
100th step and the last 66 (two restart cycles), in
tests/golden/gmres_history_convdiff3d-192.json.  Over 70 minutes on one core.

    python tests/golden/make_gmres_history.py
    python tests/golden/make_gmres_history.py --npz run.npz   # the `hist`,
        `iters`, `restarts` and `bnorm` arrays of an earlier run of the same
        pyoracle.ref_solve call, saved with numpy.savez
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

from flecsolve_gb300 import problems as P  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--npz", default=None)
    a = ap.parse_args()
    if a.npz:
        d = np.load(a.npz)
        hist, iters, restarts, bnorm = d["hist"], int(d["iters"]), int(d["restarts"]), float(d["bnorm"])
    else:
        import pyoracle as O
        A, b = P.workload("convdiff3d-192")
        r = O.ref_solve("gmres", A, b, maxiter=20000, rtol=1e-8, krylov_dim=30, side="right",
                        restart=True)
        hist, iters, restarts, bnorm = r.hist, r.iters, r.restarts, float(np.linalg.norm(b))
    tol = float(np.float32(1e-8)) * bnorm
    sampled = {str(k): float(hist[k - 1]) for k in range(100, len(hist) + 1, 100)}
    last = {str(k): float(hist[k - 1]) for k in range(max(1, len(hist) - 65), len(hist) + 1)}
    out = {"workload": "convdiff3d-192", "method": "gmres(30), right Jacobi, restart, rtol 1e-8",
           "iters": iters, "restarts": restarts, "rhs_norm": bnorm, "tol": tol,
           "estimate_every_100": sampled, "estimate_last_66": last}
    (HERE / "gmres_history_convdiff3d-192.json").write_text(json.dumps(out, indent=1))
    print(iters, restarts, tol)


if __name__ == "__main__":
    main()
