"""Parity at the full sizes of the benchmark workloads.

The reference's own runs of these workloads are committed fixtures:
tests/golden/full_size.json (its serial CG on the 256^3 diffusion system,
BiCGSTAB and GMRES(30) on the 192^3 convection-diffusion system: status,
iterations, the solution at 1024 rows and its norm) and
tests/golden/batch512.json (its CG on each of the 512 batched systems
separately).  tests/golden/order_sensitivity.json holds the iteration counts
of the same algorithms with their dot products summed in two other orders
and, for GMRES, with every product fused into its sum or update.

Bars:
* FP64 CG: iterations within +-2 of the reference's, the solution within
  1e-10 of the reference's (sampled rows and norm).
* Mixed CG with its FP64 head (the benchmark's solver): iterations +-2, true
  residual <= rtol, and within 1e-8 of the FP64 iterate.  With FP32
  recurrences from the first iteration the result is as accurate as the
  FP64 one: its forward error against a tight FP64 solve (rtol 1e-12) is
  within 1 % of the FP64 iterate's own.
* BiCGSTAB / GMRES: iterations within the reference's own spread over
  summation orders (+-2 beyond it); forward error on the sampled rows,
  against a tight FP64 solve, within 2x the largest of the reference's own
  runs under the three summation orders.  GMRES(30) at 192^3 stagnates near
  the tolerance, so its bar also allows the steps that a 1 % drift of the
  residual estimate is worth at the reference's final rate, with the drift
  itself checked against the reference's estimates every 100 steps.
* Batched (512 systems, the default FP64 head to 3e-3 ||b||): every system
  converged with true residual <= rtol, iterations within +-2 of the
  reference's CG on that system alone.
* Block CG (128^3, 16 right-hand sides): every column's true residual <=
  rtol, and its forward error within 2x that of the single-vector FP64 CG.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import flecsolve_gb300 as fs
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
FULL = json.loads((GOLD / "full_size.json").read_text())
ORDERS = json.loads((GOLD / "order_sensitivity.json").read_text())
ITER_TOL = 2
FP64_HEAD = 3e-3


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _iter_bar(wl, method):
    """+-2 around the reference's count, widened to the spread of the
    reference's own count over summation orders."""
    ref = FULL[wl][method]["iters"]
    spread = max([abs(v["iters"] - ref) for v in ORDERS.get(wl, {}).get(method, {}).values()],
                 default=0)
    return ref, spread + ITER_TOL


def _solve(ctx, ns, dA, vb, vx, P_=fs.op.jacobi, **kw):
    args = dict(maxiter=20000, rtol=1e-8, use_zero_guess=True)
    args.update(kw)
    slv = ns.solver(ns.settings(**args), ns.make_work(vb))(fs.op.ref(dA), P_)
    info = slv(vb, vx)
    return info, vx.numpy()


@pytest.fixture(scope="module")
def c2(ctx):
    A, b = P.workload("diffusion3d-256")
    S = A.to_scipy()
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    _, x_tight = _solve(ctx, fs.cg, dA, vb, vx, rtol=1e-12)
    info64, x64 = _solve(ctx, fs.cg, dA, vb, vx)
    yield dict(A=A, b=b, S=S, dA=dA, vb=vb, vx=vx, x_tight=x_tight, info64=info64, x64=x64)


def _relres(S, b, x):
    return float(np.linalg.norm(b - S @ x) / np.linalg.norm(b))


def test_diffusion3d_256_fp64_cg_matches_reference(c2):
    ref = FULL["diffusion3d-256"]["cg"]
    info, x = c2["info64"], c2["x64"]
    assert info.status == ref["status"]
    assert abs(info.iters - ref["iters"]) <= ITER_TOL
    assert _relres(c2["S"], c2["b"], x) <= 1e-8
    idx = np.asarray(ref["x_sample_index"])
    assert _rel(x[idx], np.asarray(ref["x_sample"])) <= 1e-10
    assert abs(np.linalg.norm(x) - ref["x_norm"]) / ref["x_norm"] <= 1e-10


def test_diffusion3d_256_mixed_cg_meets_fp64_bar(ctx, c2):
    """The benchmark's mixed solver (FP64 head to 3e-3 ||b||, then FP32
    recurrences with FP64 replacement) at the timed tolerance."""
    info, x = _solve(ctx, fs.mixed_cg, c2["dA"], c2["vb"], c2["vx"], fp64_head=FP64_HEAD)
    assert info.status == "converged_rtol"
    assert abs(info.iters - FULL["diffusion3d-256"]["cg"]["iters"]) <= ITER_TOL
    assert _relres(c2["S"], c2["b"], x) <= 1e-8
    assert _rel(x, c2["x64"]) <= 1e-8


def test_diffusion3d_256_mixed_cg_fp32_from_start_is_as_accurate(ctx, c2):
    """FP32 recurrences from the first iteration: the same iterations and
    stopping test, and a forward error (against a tight FP64 solve) within
    1 % of the FP64 iterate's own; the distance between the two iterates is
    a small fraction of that error."""
    info, x = _solve(ctx, fs.mixed_cg, c2["dA"], c2["vb"], c2["vx"], fp64_head=0.0)
    assert info.status == "converged_rtol"
    assert abs(info.iters - c2["info64"].iters) <= ITER_TOL
    assert _relres(c2["S"], c2["b"], x) <= 1e-8
    e64 = _rel(c2["x64"], c2["x_tight"])
    assert _rel(x, c2["x_tight"]) <= 1.01 * e64
    assert _rel(x, c2["x64"]) <= 0.1 * e64


@pytest.fixture(scope="module")
def c3(ctx):
    A, b = P.workload("convdiff3d-192")
    S = A.to_scipy()
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    info_t, x_tight = _solve(ctx, fs.bicgstab, dA, vb, vx, rtol=1e-12)
    assert info_t.status == "converged_rtol"
    yield dict(A=A, b=b, S=S, dA=dA, vb=vb, vx=vx, x_tight=x_tight)


def _sampled_accuracy(wl, method, x, x_tight):
    """Forward error of x on the sampled rows against a tight FP64 solve, and
    the largest forward error among the reference's own runs: its serial
    order (full_size.json) and the two other summation orders of the same
    algorithm (order_sensitivity.json)."""
    ref = FULL[wl][method]
    idx = np.asarray(ref["x_sample_index"])
    samples = [ref["x_sample"]] + [v["x_sample"] for v in ORDERS.get(wl, {}).get(method, {}).values()
                                   if "x_sample" in v]
    e_ref = max(_rel(np.asarray(xs), x_tight[idx]) for xs in samples)
    return _rel(x[idx], x_tight[idx]), e_ref


def test_convdiff3d_192_bicgstab_against_reference(ctx, c3):
    ref = FULL["convdiff3d-192"]["bicgstab"]
    info, x = _solve(ctx, fs.bicgstab, c3["dA"], c3["vb"], c3["vx"])
    assert info.status == ref["status"]
    it_ref, bar = _iter_bar("convdiff3d-192", "bicgstab")
    assert abs(info.iters - it_ref) <= bar
    assert _relres(c3["S"], c3["b"], x) <= 1e-8
    e, e_ref = _sampled_accuracy("convdiff3d-192", "bicgstab", x, c3["x_tight"])
    assert e <= 2.0 * e_ref + 1e-12


def test_convdiff3d_192_mixed_bicgstab(ctx, c3):
    info, x = _solve(ctx, fs.mixed_bicgstab, c3["dA"], c3["vb"], c3["vx"])
    assert info.status == "converged_rtol"
    assert info.iters <= 1.3 * FULL["convdiff3d-192"]["bicgstab"]["iters"] + 5
    assert _relres(c3["S"], c3["b"], x) <= 1e-8


HIST = json.loads((GOLD / "gmres_history_convdiff3d-192.json").read_text())
DRIFT = 0.01


def _gmres_drift_bar():
    """Steps over which the reference's own residual estimate falls by a
    factor 1 + DRIFT at the end of its run: what a relative drift of DRIFT in
    the estimate is worth in iterations at the final convergence rate."""
    last = {int(k): v for k, v in HIST["estimate_last_66"].items()}
    kend = HIST["iters"]
    j = 0
    while kend - j - 1 in last and last[kend - j - 1] < last[kend] * (1 + DRIFT):
        j += 1
    return j + 1


@pytest.mark.parametrize("ortho", ["mgs", "cgs2"])
def test_convdiff3d_192_gmres30_against_reference(ctx, c3, ortho):
    """GMRES(30) at 192^3 stagnates near the tolerance: its residual estimate
    falls 0.1 % per step at the end.  Two correct runs whose roundings differ
    therefore stop several steps apart: the reference's algorithm with fused
    multiply-adds (order_sensitivity.json, "fma") stops at 10230, the serial
    run at 10236.  The reference's estimate and this one agree to 1e-13
    after 100 steps and drift apart slowly over the 341 restarts.  Bars: the
    count within that spread +2; the estimates within DRIFT (1 %) of the
    reference's at every 100th step (tests/golden/gmres_history_convdiff3d-
    192.json), and the count within the steps that a DRIFT difference is
    worth at the reference's final rate, +2."""
    ref = FULL["convdiff3d-192"]["gmres"]
    slv = fs.gmres.solver(fs.gmres.settings(maxiter=20000, rtol=1e-8, use_zero_guess=True,
                                            max_krylov_dim=30, restart=True, ortho=ortho))(
        fs.op.ref(c3["dA"]), fs.op.jacobi)
    info = slv(c3["vb"], c3["vx"])
    x = c3["vx"].numpy()
    h = slv.history()
    assert info.status == ref["status"]
    assert h.size == info.iters
    drift = max(abs(h[int(k) - 1] - v) / v for k, v in HIST["estimate_every_100"].items()
                if int(k) <= h.size)
    assert drift <= DRIFT, drift
    it_ref, bar = _iter_bar("convdiff3d-192", "gmres")
    assert abs(info.iters - it_ref) <= bar
    assert abs(info.iters - it_ref) <= _gmres_drift_bar() + ITER_TOL
    assert _relres(c3["S"], c3["b"], x) <= 1e-8
    e, e_ref = _sampled_accuracy("convdiff3d-192", "gmres", x, c3["x_tight"])
    assert e <= 2.0 * e_ref + 1e-12


@pytest.mark.parametrize("ortho", ["auto", "cgs2"])
def test_convdiff3d_192_mixed_gmres30(ctx, c3, ortho):
    # auto: the delayed CGS2
    info, x = _solve(ctx, fs.mixed_gmres, c3["dA"], c3["vb"], c3["vx"], max_krylov_dim=30,
                     restart=True, ortho=ortho)
    assert info.status == "converged_rtol"
    assert info.iters <= 1.2 * FULL["convdiff3d-192"]["gmres"]["iters"] + 30
    assert _relres(c3["S"], c3["b"], x) <= 1e-8


def test_batched_512_systems_against_reference(ctx):
    gold = json.loads((GOLD / "batch512.json").read_text())
    A, off, b, sides = P.batch_diffusion2d()
    assert [int(s) for s in sides] == gold["sides"]
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    infos = fs.batch_cg(dA, off, vb, vx, maxiter=20000, rtol=1e-8)
    x = vx.numpy()
    S = A.to_scipy()
    for k, inf in enumerate(infos):
        lo, hi = off[k], off[k + 1]
        assert inf.status == gold["status"][k] == "converged_rtol", (k, inf)
        rr = np.linalg.norm(b[lo:hi] - S[lo:hi] @ x) / np.linalg.norm(b[lo:hi])
        assert rr <= 1e-8, (k, rr)
        assert abs(inf.iters - gold["iters"][k]) <= ITER_TOL, (k, inf.iters, gold["iters"][k])


@pytest.mark.parametrize("mixed", [False, True])
def test_block_cg_128_16_rhs(ctx, mixed):
    A, _ = P.workload("laplace3d-128")
    n = A.nrows
    B = np.stack([P.uniform(6 + j, n) for j in range(16)], axis=1)
    S = A.to_scipy()
    dA = fs.CSR(ctx, A)
    vB, vX = fs.Vector(ctx, B.ravel()), fs.Vector(ctx, n * 16)
    infos = fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8, mixed=mixed)
    X = vX.numpy().reshape(n, 16)
    vb, vx = fs.Vector(ctx, n), fs.Vector(ctx, n)
    for j in range(16):
        assert infos[j].status == "converged_rtol", (j, infos[j])
        assert _relres(S, B[:, j], X[:, j]) <= 1e-8, j
        vb.upload(B[:, j])
        _, x_tight = _solve(ctx, fs.cg, dA, vb, vx, rtol=1e-12)
        _, x64 = _solve(ctx, fs.cg, dA, vb, vx)
        assert _rel(X[:, j], x_tight) <= 2.0 * _rel(x64, x_tight), j
