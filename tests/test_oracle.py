"""CPU tests: the oracle (C restatement of the reference's serial Krylov path)
against the golden fixtures produced by the reference itself, and the
generators against their recorded digests."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle as O
from flecsolve_gb300 import problems as P

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "golden.json").read_text())


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("wl", sorted(META["problems"]))
def test_generator_digests(wl):
    """The seeded generators give the same bits as when the fixtures were made."""
    A, b = P.workload(wl)
    m = META["problems"][wl]
    assert (A.nrows, A.nnz) == (m["nrows"], m["nnz"])
    assert _digest(A.rowptr, A.col, A.val) == m["matrix_sha256"]
    assert _digest(b) == m["rhs_sha256"]


def _case_args(c, A):
    kw = dict(c["kwargs"])
    x0 = None
    if c["x0"]:
        kind, seed = c["x0"]
        x0 = P.uniform(int(seed), A.nrows, 0.0, 1.0)
    return kw, x0


@pytest.mark.parametrize("name", sorted(META["cases"]))
def test_oracle_matches_reference_fixture(name):
    """Bit-exact: status, iteration count, restart count, every residual norm
    handed to the diagnostic, and the solution."""
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    kw, x0 = _case_args(c, A)
    r = O.solve(c["method"], A, b, x0, **kw)
    g = np.load(GOLD / f"{name}.npz")
    assert r.status == c["status"]
    assert r.iters == c["iters"]
    assert r.restarts == c["restarts"]
    assert r.res_norm_final == c["res_norm_final"]
    assert np.array_equal(r.hist, g["hist"])
    assert np.array_equal(r.x, g["x"])


@pytest.mark.skipif(not O.ref_available(), reason="reference driver not built on this host")
@pytest.mark.parametrize("method,kw", [
    ("cg", {"rtol": 1e-6}),
    ("bicgstab", {"precond": "none"}),
    ("gmres", {"krylov_dim": 7, "side": "left"}),
    ("fcg", {"inner_iters": 3}),
])
def test_oracle_matches_reference_live(method, kw):
    """Where the reference compiles (this container), compare live on a fresh
    seeded problem not used for the fixtures."""
    A = P.diffusion(3, 10, seed=77, sigma=0.5)
    b = P.uniform(78, A.nrows)
    r1 = O.solve(method, A, b, **kw)
    r2 = O.ref_solve(method, A, b, **kw)
    assert (r1.status, r1.iters, r1.restarts) == (r2.status, r2.iters, r2.restarts)
    assert np.array_equal(r1.hist, r2.hist) and np.array_equal(r1.x, r2.x)


def test_oracle_spmv_is_reference_row_loop():
    A, _ = P.workload("diffusion3d-12")
    x = P.uniform(5, A.nrows)
    y = O.spmv(A, x)
    # same products, same left-to-right order, no fused multiply-add
    y2 = np.zeros(A.nrows)
    for i in range(A.nrows):
        s = 0.0
        for k in range(A.rowptr[i], A.rowptr[i + 1]):
            s = s + A.val[k] * x[A.col[k]]
        y2[i] = s
    assert np.array_equal(y, y2)


def test_oracle_parcsr_single_part_equals_csr():
    A, _ = P.workload("convdiff3d-8")
    x = P.uniform(6, A.nrows)
    assert np.array_equal(O.parcsr_spmv(A, 1, x), O.spmv(A, x))
    y3 = O.parcsr_spmv(A, 3, x)
    assert np.allclose(y3, O.spmv(A, x), rtol=1e-14, atol=1e-14)


def test_oracle_parcsr_blocks_follow_equal_map():
    """rows split as flecsi::util::equal_map (parcsr.hh:149-151): blocks of
    N // parts rows, the first N % parts one row longer; each row sums its
    owned and its ghost columns separately, in CSR order"""
    A, _ = P.workload("convdiff3d-8")  # 512 rows: 3 parts of 171, 171, 170
    x = P.uniform(7, A.nrows)
    for parts in (3, 5, 512):
        q, r = divmod(A.nrows, parts)
        starts = [c * q + min(c, r) for c in range(parts + 1)]
        assert starts[-1] == A.nrows
        want = np.empty(A.nrows)
        for c in range(parts):
            lo, hi = starts[c], starts[c + 1]
            for i in range(lo, hi):
                yd = yo = 0.0
                for k in range(A.rowptr[i], A.rowptr[i + 1]):
                    j = A.col[k]
                    if lo <= j < hi:
                        yd += A.val[k] * x[j]
                    else:
                        yo += A.val[k] * x[j]
                want[i] = yd + yo
        assert np.array_equal(O.parcsr_spmv(A, parts, x), want)


def test_oracle_edge_cases():
    A, b = P.workload("poisson2d-8")
    # zero right-hand side with zero guess: converged immediately (cg.hh:77-82)
    r = O.solve("cg", A, np.zeros_like(b))
    assert r.status == "converged_rtol" and r.iters == 0
    # maxiter exhausted: iters stays 0 and the status is diverged_iters
    r = O.solve("cg", A, b, maxiter=3)
    assert r.status == "diverged_iters" and r.iters == 0 and r.hist.size == 3
    # user diagnostic stops the solve (converged_user, iters = iteration)
    r = O.solve("bicgstab", A, b, diag=lambda x, res: True)
    assert r.status == "converged_user" and r.iters == 1
    # GMRES validate(): restart = false needs maxiter <= max_krylov_dim
    r = O.solve("gmres", A, b, krylov_dim=5, restart=False, maxiter=10)
    assert r.status == "assert_failed"


def test_summation_order_moves_bicgstab_not_cg():
    """The reference algorithms with their dot products summed in other valid
    orders (oracle order switch; order 0 is the reference's serial sum): CG's
    iteration count does not move, BiCGSTAB's does -- the basis of the
    order-range bars of the BiCGSTAB / GMRES parity tests."""
    A, b = P.workload("poisson2d-128")
    cg = [r.iters for r in O.solve_orders("cg", A, b, maxiter=2000, rtol=1e-8)]
    bi = [r.iters for r in O.solve_orders("bicgstab", A, b, maxiter=2000, rtol=1e-8)]
    assert cg == [389, 389, 389]
    assert bi == [259, 300, 285]
    # order 0 is the reference's own run, bit for bit
    assert bi[0] == META["cases"]["poisson2d-128_bicgstab"]["iters"]
