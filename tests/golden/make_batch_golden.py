"""Per-system reference results for the 512-system batched workload.

Runs the reference's own serial Jacobi-PCG (oracle/_ref/ref_driver, built
from the reference's headers) on each of the 512 independent 2-D
log-normal diffusion systems of ``problems.batch_diffusion2d()`` (sides
U{32..256}, seed 5) separately, rtol 1e-8, zero guess, and records each
system's size, status, iteration count and final residual norm in
tests/golden/batch512.json.  A few minutes on one core.

    python tests/golden/make_batch_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

from flecsolve_gb300 import problems as P  # noqa: E402
import pyoracle as O  # noqa: E402


def system(A, off, k):
    lo, hi = int(off[k]), int(off[k + 1])
    return P.CSR(hi - lo, hi - lo, A.rowptr[lo:hi + 1] - A.rowptr[lo],
                 A.col[A.rowptr[lo]:A.rowptr[hi]] - lo, A.val[A.rowptr[lo]:A.rowptr[hi]])


def main():
    A, off, b, sides = P.batch_diffusion2d()
    out = {"workload": "batch512-diffusion2d-32-256 (seed 5)", "rtol": 1e-8, "maxiter": 20000,
           "sides": [int(s) for s in sides], "rows": [], "status": [], "iters": [],
           "res_norm_final": []}
    for k in range(len(sides)):
        Ak = system(A, off, k)
        r = O.ref_solve("cg", Ak, b[off[k]:off[k + 1]], maxiter=20000, rtol=1e-8)
        out["rows"].append(Ak.nrows)
        out["status"].append(r.status)
        out["iters"].append(r.iters)
        out["res_norm_final"].append(r.res_norm_final)
    (HERE / "batch512.json").write_text(json.dumps(out))
    print("systems", len(sides), "iterations", sum(out["iters"]))


if __name__ == "__main__":
    main()
