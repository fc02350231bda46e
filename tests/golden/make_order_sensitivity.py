"""Iteration counts of the reference's solvers under other summation orders.

The reference sums every dot product serially left to right
(flecsolve/vectors/seq.hh:282-295); a device reduction sums the same products
in another order.  This script runs the oracle -- the reference's solvers
restated in C and pinned to them bit for bit -- on the full-size workloads
with its reductions taken in two other valid orders (blocks of 4096 then the
block sums; right to left) and records status and iteration count for each,
in tests/golden/order_sensitivity.json, with the solution at the rows that
tests/golden/full_size.json samples.  The spread is the part of an
iteration-count (and forward-error) difference that comes from summation
order alone.  Hours of
CPU per GMRES run; each spec can run in its own process:

    python tests/golden/make_order_sensitivity.py convdiff3d-192:gmres:1

The variant "fma" keeps the serial order and fuses every product into the sum
or update it feeds (convdiff3d-192:gmres:fma): the rounding of the device's
FMA kernels, which a change of summation order does not show.
"""
from __future__ import annotations

import fcntl
import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent.parent / "oracle"))

from flecsolve_gb300 import problems as P  # noqa: E402
import pyoracle as O  # noqa: E402

SETTINGS = {"cg": {}, "bicgstab": {}, "gmres": {"krylov_dim": 30, "side": "right",
                                                 "restart": True}}
ORDERS = {"1": "blocks of 4096, then the block sums", "2": "right to left",
          "fma": "serial, every product fused into its sum or update (one rounding, as in "
                 "the device's FMA kernels)"}


def run(spec: str) -> None:
    wl, method, order = spec.split(":")
    A, b = P.workload(wl)
    if order == "fma":
        O.lib().or_set_contract(1)
    else:
        O.lib().or_set_dot_order(int(order))
    t0 = time.time()
    r = O.solve(method, A, b, maxiter=20000, rtol=1e-8, **SETTINGS[method])
    O.lib().or_set_dot_order(0)
    O.lib().or_set_contract(0)
    full = json.loads((HERE / "full_size.json").read_text())
    idx = full[wl][method]["x_sample_index"]
    out = HERE / "order_sensitivity.json"
    # several processes may finish at once: read and write under a lock
    with open(HERE / ".order_sensitivity.lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        data = json.loads(out.read_text()) if out.exists() else {}
        data.setdefault(wl, {}).setdefault(method, {})[order] = {
            "order": ORDERS[order], "status": r.status, "iters": r.iters,
            "restarts": r.restarts, "res_norm_final": r.res_norm_final,
            "x_sample": r.x[idx].tolist(), "seconds_one_core": time.time() - t0}
        out.write_text(json.dumps(data, indent=1, sort_keys=True))
    print(spec, r.status, r.iters, flush=True)


if __name__ == "__main__":
    for s in sys.argv[1:]:
        run(s)
