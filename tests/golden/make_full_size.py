"""Full-size reference results (run where the reference headers are mounted).

Runs the reference's own serial Krylov templates (oracle/_ref/ref_driver) on
the full benchmark workloads and records status, iteration count, final
residual norm, and the solution at 1024 evenly spaced rows plus its norm, in
tests/golden/full_size.json.  Minutes per solve on one core.

    python tests/golden/make_full_size.py diffusion3d-256:cg convdiff3d-192:bicgstab
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

from flecsolve_gb300 import problems as P  # noqa: E402
import pyoracle as O  # noqa: E402

SETTINGS = {"cg": {}, "bicgstab": {}, "gmres": {"krylov_dim": 30, "side": "right",
                                                 "restart": True}}


def main(specs):
    out_path = HERE / "full_size.json"
    data = json.loads(out_path.read_text()) if out_path.exists() else {}
    cache = {}
    for spec in specs:
        wl, method = spec.split(":")
        if wl not in cache:
            cache[wl] = P.workload(wl)
        A, b = cache[wl]
        t0 = time.time()
        r = O.ref_solve(method, A, b, maxiter=20000, rtol=1e-8, **SETTINGS[method])
        idx = np.linspace(0, A.nrows - 1, 1024).astype(np.int64)
        data.setdefault(wl, {})[method] = {
            "status": r.status, "iters": r.iters, "restarts": r.restarts,
            "res_norm_final": r.res_norm_final, "x_norm": float(np.linalg.norm(r.x)),
            "x_sample_index": idx.tolist(), "x_sample": r.x[idx].tolist(),
            "settings": {"maxiter": 20000, "rtol": 1e-8, **SETTINGS[method]},
            "reference_seconds_one_core": time.time() - t0}
        out_path.write_text(json.dumps(data, indent=1, sort_keys=True))
        print(wl, method, r.status, r.iters, flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
