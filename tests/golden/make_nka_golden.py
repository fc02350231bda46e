"""Generate the NKA golden fixtures in this directory from the reference.

Runs the reference's unmodified NKA (flecsolve/solvers/nka.hh) over
vec::seq_vec and mat::csr<double>, preconditioned by its CG solver as
solvers/test/nka.cc:72-80 does (``make -C oracle ref`` builds
``oracle/_ref/ref_nka``), on seeded problems with b = 1 and x0 = 3 as in that
test, and stores solve_info, the residual history handed to the diagnostic
and the solution in ``nka_<case>.npz``; ``nka_golden.json`` lists the cases.

Usage (needs the reference headers, i.e. only where they are mounted):
    python tests/golden/make_nka_golden.py
"""
from __future__ import annotations

import json
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from flecsolve_gb300 import problems as P  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "ref_nka"

# name, workload, nka (maxiter, atol, max_dim, angle_tol), cg (maxiter, rtol),
# damping (use, adaptive, factor) or None.  The first two are nka.cfg's
# settings (solvers/test/nka.cfg); the third runs out of iterations.
CASES = [
    ("poisson2d-64_pc11", "poisson2d-64", (100, 1e-6, 5, 0.2), (11, 1e-9), None),
    ("diffusion3d-16_pc11", "diffusion3d-16", (100, 1e-6, 5, 0.2), (11, 1e-9), None),
    ("diffusion3d-16_pc5", "diffusion3d-16", (100, 1e-6, 5, 0.2), (5, 1e-9), None),
    ("poisson2d-64_pc5_stalls", "poisson2d-64", (100, 1e-6, 5, 0.2), (5, 1e-9), None),
    ("diffusion3d-16_dim10", "diffusion3d-16", (100, 1e-6, 10, 0.05), (8, 1e-9), None),
    ("diffusion3d-16_damped", "diffusion3d-16", (100, 1e-6, 5, 0.2), (11, 1e-9), (1, 0, 0.8)),
    ("diffusion3d-16_adaptive", "diffusion3d-16", (100, 1e-6, 5, 0.2), (11, 1e-9), (1, 1, 1.0)),
]


def run(A, b, x0, nka, pc, damp):
    inp, out = HERE / "_nka.in", HERE / "_nka.out"
    with open(inp, "wb") as f:
        f.write(struct.pack("<qq", A.nrows, A.nnz))
        f.write(np.asarray(A.rowptr, "<i8").tobytes())
        f.write(np.asarray(A.col, "<i4").tobytes())
        f.write(np.asarray(A.val, "<f8").tobytes())
        f.write(np.asarray(b, "<f8").tobytes())
        f.write(np.asarray(x0, "<f8").tobytes())
    args = [str(v) for v in (*nka, *pc)] + ([str(v) for v in damp] if damp else [])
    subprocess.run([str(REF), str(inp), str(out)] + args, check=True)
    d = out.read_bytes()
    inp.unlink()
    out.unlink()
    st, it = struct.unpack_from("<ii", d, 0)
    r0, r1, s1 = struct.unpack_from("<fff", d, 8)
    nh = struct.unpack_from("<q", d, 20)[0]
    hist = np.frombuffer(d, "<f8", nh, 28).copy()
    x = np.frombuffer(d, "<f8", A.nrows, 28 + 8 * nh).copy()
    return st, it, r0, r1, s1, hist, x


def main():
    if not REF.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    meta = {}
    for name, wl, nka, pc, damp in CASES:
        A, _ = P.workload(wl)
        b = np.ones(A.nrows)
        x0 = np.full(A.nrows, 3.0)
        st, it, r0, r1, s1, hist, x = run(A, b, x0, nka, pc, damp)
        np.savez_compressed(HERE / f"nka_{name}.npz", hist=hist, x=x)
        meta[name] = {"workload": wl, "nka": list(nka), "pc": list(pc),
                      "damping": list(damp) if damp else None, "status": st, "iters": it,
                      "res_norm_initial": r0, "res_norm_final": r1, "sol_norm_final": s1}
        print(name, "status", st, "iters", it, "res", r1)
    (HERE / "nka_golden.json").write_text(json.dumps({"cases": meta}, indent=1) + "\n")


if __name__ == "__main__":
    main()
