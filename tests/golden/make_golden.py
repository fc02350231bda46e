"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's unmodified serial Krylov templates (flecsolve/solvers/
{cg,bicgstab,gmres}.hh over vec::seq_vec and mat::csr<double>, compiled by
``make -C oracle ref`` into ``oracle/_ref/ref_driver``) on seeded problems
from ``flecsolve_gb300.problems`` and stores solve_info, the residual history
handed to the diagnostic, and the solution.  Also stores SHA-256 digests of
the generated matrices and right-hand sides so that generator drift on
another host is caught.

Usage (needs the reference headers, i.e. only where they are mounted):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from flecsolve_gb300 import build, problems as P  # noqa: E402
import pyoracle as O  # noqa: E402

# (name, workload, method, kwargs)
CASES = [
    ("poisson2d-128_cg", "poisson2d-128", "cg", {}),
    ("poisson2d-128_bicgstab", "poisson2d-128", "bicgstab", {}),
    ("poisson2d-128_gmres30", "poisson2d-128", "gmres", {"krylov_dim": 30}),
    ("poisson2d-128_cg_noprec_x0", "poisson2d-128", "cg",
     {"precond": "none", "use_zero_guess": False, "x0": ("uniform", 11)}),
    ("diffusion3d-16_cg", "diffusion3d-16", "cg", {}),
    ("diffusion3d-16_bicgstab", "diffusion3d-16", "bicgstab", {}),
    ("diffusion3d-16_gmres_left", "diffusion3d-16", "gmres", {"side": "left"}),
    ("convdiff3d-16_bicgstab", "convdiff3d-16", "bicgstab", {}),
    ("convdiff3d-16_gmres30", "convdiff3d-16", "gmres", {"krylov_dim": 30}),
    ("convdiff3d-16_gmres10_x0", "convdiff3d-16", "gmres",
     {"krylov_dim": 10, "use_zero_guess": False, "x0": ("uniform", 12), "rtol": 1e-10}),
    ("convdiff3d-16_gmres_norestart", "convdiff3d-16", "gmres",
     {"krylov_dim": 60, "restart": False, "maxiter": 60, "precond": "none"}),
    # flexible CG (cg.hh:145-244): Jacobi, none, and a nested reference CG
    # (5 Jacobi-PCG iterations, rtol 0, zero guess) bound as the preconditioner
    ("poisson2d-128_fcg", "poisson2d-128", "fcg", {}),
    ("diffusion3d-16_fcg_noprec", "diffusion3d-16", "fcg", {"precond": "none"}),
    ("diffusion3d-16_fcg_cg5", "diffusion3d-16", "fcg", {"inner_iters": 5}),
]


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def x0_of(spec, n):
    if spec is None:
        return None
    kind, seed = spec
    assert kind == "uniform"
    return P.uniform(seed, n, 0.0, 1.0)


def main() -> None:
    build.build_problems()
    build.build_oracle()
    if not O.ref_available():
        raise SystemExit("reference driver not built: the reference headers are needed")
    meta = {"problems": {}, "cases": {}}
    cache = {}
    for name, wl, method, kw in CASES:
        if wl not in cache:
            A, b = P.workload(wl)
            cache[wl] = (A, b)
            meta["problems"][wl] = {"nrows": A.nrows, "nnz": A.nnz,
                                    "matrix_sha256": digest(A.rowptr, A.col, A.val),
                                    "rhs_sha256": digest(b)}
        A, b = cache[wl]
        kw = dict(kw)
        spec = kw.pop("x0", None)
        x0 = x0_of(spec, A.nrows)
        r = O.ref_solve(method, A, b, x0, **kw)
        np.savez_compressed(HERE / f"{name}.npz", hist=r.hist, x=r.x)
        meta["cases"][name] = {"workload": wl, "method": method, "kwargs": kw,
                               "x0": list(spec) if spec else None, "status": r.status,
                               "iters": r.iters, "restarts": r.restarts,
                               "res_norm_final": r.res_norm_final,
                               "sol_norm_final": r.sol_norm_final, "rhs_norm": r.rhs_norm}
        print(f"{name:34s} {r.status:16s} iters={r.iters:5d} restarts={r.restarts}")
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
