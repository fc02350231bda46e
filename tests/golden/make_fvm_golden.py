"""Generate the finite-volume physics fixtures in this directory from the
reference.

Runs the reference's own, unmodified physics operators (flecsolve/physics/:
Dirichlet and Neumann boundary operators, constant / average face
coefficients, volume diffusion), compiled with ``make -C oracle ref`` as
``oracle/_ref/ref_fvm``, on seeded meshes, and the reference's CG
(solvers/cg.hh) over that operator expression as the equilibrium-diffusion
example solves it (examples/equilibrium_diffusion/include/
equilibrium_diffusion.hh:267-345, diffusion.cfg).  Stores inputs and outputs
in ``fvm_<case>.npz``; ``fvm_golden.json`` lists the cases and their
settings.

Usage (needs the reference headers, i.e. only where they are mounted):
    python tests/golden/make_fvm_golden.py
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import fvm_oracle as O  # noqa: E402

D, N_ = O.DIRICHLET, O.NEUMANN
UNIT = [[0.0, 1.0]] * 3

# name: mesh, box, beta, alpha, boundary kinds and values, coefficient kind
# (0 the face fields as given, 1 constant, 2 average) and value, seed
APPLY = {
    # physics/test/fvm_diffusion.cc:200-210: Dirichlet 1e-9 everywhere, x = 1
    "sink8": dict(n=(8, 8, 8), box=UNIT, beta=1.0, alpha=0.0, bc=[D] * 6, bcv=[1e-9] * 6, ck=1, cv=1.0,
                  seed=None),
    "mixed7x5x4": dict(n=(7, 5, 4), box=[[0.0, 2.0], [-1.0, 1.0], [0.0, 0.5]], beta=1.3, alpha=0.7,
                       bc=[D, N_, N_, D, D, N_], bcv=[0.25, -0.5, 1.5, -2.0, 0.75, 0.125], ck=0, cv=0.0,
                       seed=11),
    "average6": dict(n=(6, 6, 6), box=UNIT, beta=1.0, alpha=0.5, bc=[D] * 6,
                     bcv=[1.0, 2.0, 0.5, 1.5, 1.25, 0.75], ck=2, cv=0.0, seed=12),
    "neumann9x4x3": dict(n=(9, 4, 3), box=[[0.0, 3.0], [0.0, 1.0], [0.0, 2.0]], beta=0.8, alpha=2.0,
                         bc=[N_] * 6, bcv=[0.5, -0.25, 1.0, 0.0, -1.5, 2.0], ck=1, cv=3.14, seed=13),
    "flat16x12x1": dict(n=(16, 12, 1), box=UNIT, beta=1.0, alpha=0.0, bc=[D, D, D, D, N_, N_],
                        bcv=[1e-9] * 4 + [0.0, 0.0], ck=1, cv=1.0, seed=14),
    # faces without a boundary operator keep their cells' values
    "partial5x3x2": dict(n=(5, 3, 2), box=[[0.0, 1.0], [0.0, 2.0], [0.0, 1.0]], beta=1.0, alpha=1.0,
                         bc=[D, 0, N_, 0, 0, D], bcv=[0.5, 0.0, 0.25, 0.0, 0.0, -1.0], ck=0, cv=0.0, seed=15),
}

# CG cases: the apply settings plus the right-hand side, initial guess and
# the solver settings
CG = {
    # the equilibrium-diffusion example: Dirichlet 1e-9 on x and y, zero-flux
    # z, constant coefficient 1, RHS 0, X = 2, diffusion.cfg's CG settings
    "cg_example32x32x1": dict(n=(32, 32, 1), box=UNIT, beta=1.0, alpha=0.0, bc=[D, D, D, D, N_, N_],
                              bcv=[1e-9] * 4 + [0.0, 0.0], ck=1, cv=1.0, seed=None, rhs=0.0, x0=2.0,
                              maxiter=500, rtol=1e-6, zero_guess=False),
    "cg_field12x10x8": dict(n=(12, 10, 8), box=[[0.0, 1.0], [0.0, 1.0], [0.0, 0.8]], beta=1.0, alpha=0.5,
                            bc=[D, D, N_, N_, N_, N_], bcv=[0.0] * 6, ck=0, cv=0.0, seed=21, rhs="random",
                            x0=0.0, maxiter=2000, rtol=1e-8, zero_guess=False),
}


def inputs(c):
    n = c["n"]
    u, a, v, b = O.cell_field(n), O.cell_field(n, 1.0), O.cell_field(n), O.face_fields(n)
    if c["seed"] is None:
        u[1:-1, 1:-1, 1:-1] = 1.0
    else:
        rng = np.random.default_rng(c["seed"])
        u = rng.normal(size=u.shape) + (2.0 if c["ck"] == 2 else 0.0)
        a = np.exp(rng.normal(size=a.shape))
        v = rng.normal(size=v.shape)
        b = [np.exp(rng.normal(size=f.shape)) for f in b]
    return u, a, v, b


def meta(c):
    return {"n": list(c["n"]), "box": c["box"], "beta": c["beta"], "alpha": c["alpha"], "bc_kind": c["bc"],
            "bc_value": c["bcv"], "coef_kind": c["ck"], "coef_value": c["cv"]}


def main():
    if not O.ref_available():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    out = {"apply": {}, "cg": {}}
    for name, c in APPLY.items():
        u, a, v, b = inputs(c)
        args = (c["n"], c["box"], c["beta"], c["alpha"], c["bc"], c["bcv"], c["ck"], c["cv"])
        uo, bo, vo = O.ref_apply(*args, u, a, v, b)
        np.savez_compressed(HERE / f"fvm_{name}.npz", u=u, a=a, v=v, bx=b[0], by=b[1], bz=b[2], u_out=uo,
                            bx_out=bo[0], by_out=bo[1], bz_out=bo[2], v_out=vo)
        out["apply"][name] = meta(c)
        print(name, "max |v|", float(np.abs(vo[1:-1, 1:-1, 1:-1]).max()))
    for name, c in CG.items():
        u, a, _, b = inputs(c)
        n = c["n"]
        N = n[0] * n[1] * n[2]
        if c["rhs"] == "random":
            rhs = np.random.default_rng(c["seed"] + 100).uniform(-1.0, 1.0, N)
        else:
            rhs = np.full(N, float(c["rhs"]))
        x0 = np.full(N, float(c["x0"]))
        args = (n, c["box"], c["beta"], c["alpha"], c["bc"], c["bcv"], c["ck"], c["cv"])
        st, it, norms, hist, x = O.ref_cg(*args, u, a, b, rhs, x0, maxiter=c["maxiter"], rtol=c["rtol"],
                                          zero_guess=c["zero_guess"])
        np.savez_compressed(HERE / f"fvm_{name}.npz", u=u, a=a, bx=b[0], by=b[1], bz=b[2], rhs=rhs, x0=x0,
                            hist=hist, x=x)
        m = meta(c)
        m.update(maxiter=c["maxiter"], rtol=c["rtol"], zero_guess=c["zero_guess"], status=st, iters=it,
                 res_norm_initial=norms[0], res_norm_final=norms[1], sol_norm_final=norms[3])
        out["cg"][name] = m
        print(name, "status", st, "iters", it, "res", norms[1])
    (HERE / "fvm_golden.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
