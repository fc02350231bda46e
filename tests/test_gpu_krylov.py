"""Device CG / BiCGSTAB / mixed-precision CG against the reference.

Bars (from the specification of this path): iteration counts within +-2 of
the reference's, relative residual <= rtol, solution relative error vs the
FP64 oracle <= 1e-10 for the FP64 path and <= 1e-8 after refinement for the
mixed path.  The reference numbers come from the golden fixtures produced by
the reference's own templates (tests/golden/) or from the oracle on the same
seeded inputs."""
import json
from pathlib import Path

import numpy as np
import pytest

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "golden.json").read_text())
ITER_TOL = 2
X_RTOL_F64 = 1e-10
X_RTOL_MIXED = 1e-8


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _true_relres(A, b, x):
    return np.linalg.norm(O.residual(A, b, x)) / np.linalg.norm(b)


def _run(ctx, ns, A, b, x0=None, P_="jacobi", diag=None, **kw):
    dA = fs.CSR(ctx, A)
    vb = fs.Vector(ctx, b)
    vx = fs.Vector(ctx, np.zeros(A.nrows) if x0 is None else x0)
    s = ns.settings(**kw)
    prec = fs.op.jacobi if P_ == "jacobi" else fs.op.I
    slv = ns.solver(s, ns.make_work(vb))(fs.op.ref(dA), prec, diag)
    info = slv(vb, vx)
    return info, vx.numpy(), slv


GOLD_CASES = [n for n, c in sorted(META["cases"].items()) if c["method"] in ("cg", "bicgstab")]


@pytest.mark.parametrize("name", GOLD_CASES)
def test_against_reference_fixture(ctx, name):
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    kw = dict(c["kwargs"])
    x0 = P.uniform(int(c["x0"][1]), A.nrows, 0.0, 1.0) if c["x0"] else None
    prec = kw.pop("precond", "jacobi")
    ns = fs.cg if c["method"] == "cg" else fs.bicgstab
    info, x, _ = _run(ctx, ns, A, b, x0, prec, maxiter=kw.pop("maxiter", 2000),
                      rtol=kw.pop("rtol", 1e-8), use_zero_guess=kw.pop("use_zero_guess", True))
    g = np.load(GOLD / f"{name}.npz")
    assert info.status == c["status"]
    assert _true_relres(A, b, x) <= 1e-8 * 1.01
    if c["method"] == "cg":
        assert abs(info.iters - c["iters"]) <= ITER_TOL
        assert _rel(x, g["x"]) <= X_RTOL_F64
    else:
        _order_bar("bicgstab", A, b, info.iters, x0, maxiter=2000, rtol=1e-8, precond=prec,
                   use_zero_guess=x0 is None)
        rs = O.solve_orders("bicgstab", A, b, x0, maxiter=2000, rtol=1e-8, precond=prec,
                            use_zero_guess=x0 is None)
        _bicgstab_accuracy_bar(A, b, x, [g["x"]] + [q.x for q in rs])


def _order_bar(method, A, b, iters, x0=None, **kw):
    """BiCGSTAB and GMRES amplify the rounding of their dot products: the
    reference's own iteration count moves with the summation order (on the
    128^2 Poisson system its BiCGSTAB takes 259, 300 or 285 iterations for
    three valid orders).  The bar: within the range of the reference
    algorithm's counts over summation orders (the oracle, pinned bit for bit
    to the reference in its serial order), +-2."""
    rs = O.solve_orders(method, A, b, x0, **kw)
    lo, hi = min(r.iters for r in rs), max(r.iters for r in rs)
    assert lo - ITER_TOL <= iters <= hi + ITER_TOL, (iters, [r.iters for r in rs])


def _bicgstab_accuracy_bar(A, b, x, x_ref):
    """BiCGSTAB amplifies the rounding of its dot products: two correct FP64
    runs whose reductions are summed in different orders follow the same
    residual history for ~25 iterations and then separate, ending at
    different points of the rtol ball.  The bar is therefore that the device
    solution is as accurate as the reference's: its forward error against
    the direct solution is within 2x the reference's own (+ 1e-12).
    `x_ref` may be a list: the reference algorithm's solutions under several
    summation orders, whose largest forward error is the reference's."""
    import scipy.sparse.linalg as spla
    xs = spla.spsolve(A.to_scipy().tocsc(), b)
    refs = x_ref if isinstance(x_ref, list) else [x_ref]
    assert _rel(x, xs) <= 2.0 * max(_rel(xr, xs) for xr in refs) + 1e-12


def test_cg_history_tracks_reference(ctx):
    A, b = P.workload("poisson2d-128")
    info, x, slv = _run(ctx, fs.cg, A, b, maxiter=2000, rtol=1e-8)
    g = np.load(GOLD / "poisson2d-128_cg.npz")
    h = slv.history()
    m = min(h.size, g["hist"].size)
    assert h.size == info.iters
    # residual norms agree to rounding until the very end of the run
    assert np.allclose(h[: m - 5], g["hist"][: m - 5], rtol=1e-6)


def test_cg_diagnostic_called_every_iteration(ctx):
    """cg.cc:85-89: the diagnostic runs once per iteration and sees x."""
    A, b = P.workload("poisson2d-64")
    calls = []

    def diag(xv, res):
        calls.append((res, float(xv.l2norm().get())))
        return False

    info, x, _ = _run(ctx, fs.cg, A, b, diag=diag, maxiter=2000, rtol=1e-8)
    assert info.iters == len(calls)
    assert calls[-1][1] == pytest.approx(np.linalg.norm(x), rel=1e-12)
    # user stop
    info, _, _ = _run(ctx, fs.cg, A, b, diag=lambda xv, r: True, maxiter=2000, rtol=1e-8)
    assert info.status == "converged_user" and info.iters == 1


def test_cg_edge_cases(ctx):
    A, b = P.workload("poisson2d-32")
    info, x, _ = _run(ctx, fs.cg, A, np.zeros_like(b), maxiter=100, rtol=1e-8)
    assert info.status == "converged_rtol" and info.iters == 0 and not x.any()
    info, _, _ = _run(ctx, fs.cg, A, b, maxiter=5, rtol=1e-8)
    assert info.status == "diverged_iters" and info.iters == 0
    r = O.solve("cg", A, b, maxiter=5)
    assert (r.status, r.iters) == (info.status, info.iters)
    bad = b.copy()
    bad[7] = np.nan
    with pytest.raises(fs.api._lib.FsError) as ei:
        _run(ctx, fs.cg, A, bad, maxiter=50, rtol=1e-8)
    assert ei.value.status == fs.api._lib.ERR_NON_FINITE


def test_cg_readback_interval_does_not_change_result(ctx):
    A, b = P.workload("diffusion3d-24")
    res = []
    for k in (1, 7, 32):
        info, x, _ = _run(ctx, fs.cg, A, b, maxiter=2000, rtol=1e-8, k_readback=k)
        res.append((info.iters, x))
    assert res[0][0] == res[1][0] == res[2][0]
    assert np.array_equal(res[0][1], res[1][1]) and np.array_equal(res[0][1], res[2][1])


@pytest.mark.parametrize("wl", ["diffusion3d-40", "diffusion2d-96"])
def test_cg_vs_oracle(ctx, wl):
    A, b = P.workload(wl)
    r = O.solve("cg", A, b, maxiter=4000, rtol=1e-8)
    info, x, _ = _run(ctx, fs.cg, A, b, maxiter=4000, rtol=1e-8)
    assert info.status == r.status == "converged_rtol"
    assert abs(info.iters - r.iters) <= ITER_TOL
    assert _rel(x, r.x) <= X_RTOL_F64


@pytest.mark.parametrize("wl,prec", [("convdiff3d-24", "jacobi"), ("convdiff3d-16", "none"),
                                     ("diffusion3d-24", "jacobi")])
def test_bicgstab_vs_oracle(ctx, wl, prec):
    A, b = P.workload(wl)
    r = O.solve("bicgstab", A, b, maxiter=4000, rtol=1e-8, precond=prec)
    info, x, _ = _run(ctx, fs.bicgstab, A, b, P_=prec, maxiter=4000, rtol=1e-8)
    assert info.status == r.status
    _order_bar("bicgstab", A, b, info.iters, maxiter=4000, rtol=1e-8, precond=prec)
    assert _true_relres(A, b, x) <= 1e-8 * 1.01
    rs = O.solve_orders("bicgstab", A, b, maxiter=4000, rtol=1e-8, precond=prec)
    _bicgstab_accuracy_bar(A, b, x, [q.x for q in rs])


def test_bicgstab_early_exit_quirk(ctx):
    """bicgstab.hh:136-142: ||s|| < rtol (unscaled) exits with iters = iter;
    with iters == 0 the status becomes diverged_iters (bicgstab.hh:183)."""
    A, b = P.workload("poisson2d-16")
    b = b * 1e-12  # tiny rhs: ||s|| below rtol after the first half-step
    r = O.solve("bicgstab", A, b, maxiter=100, rtol=1e-8)
    info, x, _ = _run(ctx, fs.bicgstab, A, b, maxiter=100, rtol=1e-8)
    assert (info.status, info.iters) == (r.status, r.iters)
    assert _rel(x, r.x) <= 1e-9


@pytest.mark.parametrize("wl", ["diffusion3d-40", "poisson2d-128"])
def test_mixed_cg_refinement(ctx, wl):
    """FP32-inner / FP64-refined CG reaches the FP64 stopping test, and its
    error against the FP64 direct solution is <= 1e-8 when the stopping test
    asks for it (rtol 1e-11 bounds the forward error by cond(A) * 1e-11)."""
    A, b = P.workload(wl)
    ref64 = O.solve("cg", A, b, maxiter=20000, rtol=1e-8)
    # FP64 solution to rtol 1e-14 by the oracle (a sparse LU of the 3-D
    # operator takes half a minute on the test host); its forward error is
    # <= cond(A) * 1e-14, far inside the 1e-8 bar
    xs = O.solve("cg", A, b, maxiter=20000, rtol=1e-14).x
    # default: FP32 recurrences with FP64 residual replacement -- the search
    # direction survives a replacement, so the iteration count is the FP64 one
    info, x, slv = _run(ctx, fs.mixed_cg, A, b, maxiter=20000, rtol=1e-8)
    assert info.status == "converged_rtol"
    assert _true_relres(A, b, x) <= 1e-8
    outer, inner = slv.mixed_stats()
    assert outer >= 1 and inner == info.iters
    assert abs(info.iters - ref64.iters) <= ITER_TOL
    info2, x2, _ = _run(ctx, fs.mixed_cg, A, b, maxiter=20000, rtol=1e-11)
    assert info2.status == "converged_rtol"
    assert _rel(x2, xs) <= X_RTOL_MIXED
    # classic restarted refinement: converges, at a higher iteration cost
    info3, x3, _ = _run(ctx, fs.mixed_cg, A, b, maxiter=20000, rtol=1e-11, refine="restart",
                        inner_rtol=1e-4)
    assert info3.status == "converged_rtol"
    assert _rel(x3, xs) <= X_RTOL_MIXED


@pytest.mark.parametrize("eps", [1e-2, 1e-4, 1e-6])
@pytest.mark.parametrize("head", [0.0, 3e-3, 1e-2])
def test_mixed_cg_warm_start(ctx, eps, head):
    """A guess near the solution (initial residual above, near or below the
    FP64 head's tolerance): the mixed CG takes the oracle's FP64 CG count
    +-2 from the same guess, whether the head runs or not."""
    A, b = P.workload("diffusion3d-24")
    xs = O.solve("cg", A, b, maxiter=20000, rtol=1e-13).x
    x0 = xs + eps * P.uniform(5, A.nrows)
    ref = O.solve("cg", A, b, x0, maxiter=20000, rtol=1e-8, use_zero_guess=False)
    info, x, _ = _run(ctx, fs.mixed_cg, A, b, x0=x0, maxiter=20000, rtol=1e-8,
                      use_zero_guess=False, fp64_head=head)
    assert info.status == ref.status == "converged_rtol"
    assert abs(info.iters - ref.iters) <= ITER_TOL, (info.iters, ref.iters)
    assert _true_relres(A, b, x) <= 1e-8


@pytest.mark.parametrize("wl", ["diffusion3d-40", "poisson2d-127", "diffusion3d-23"])
def test_mixed_cg_index_formats(ctx, wl):
    """The mixed CG on a stencil matrix with each SpMV format (symmetric
    storage, row patterns, column ids): the same recurrences, the same
    stopping test, iteration counts within one of each other and of the FP64
    reference count, the same accuracy bar; a user stop folds the pending
    solution step into x."""
    A, b = P.workload(wl)
    ref64 = O.solve("cg", A, b, maxiter=20000, rtol=1e-8)
    xs = O.solve("cg", A, b, maxiter=20000, rtol=1e-14).x
    dA = fs.CSR(ctx, A)
    vb = fs.Vector(ctx, b)
    res = {}
    for coding in ("grid", "symmetric", "patterns", "colids"):
        dA.index_coding(coding)
        for rtol in (1e-8, 1e-11):
            vx = fs.Vector(ctx, A.nrows)
            slv = fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=20000, rtol=rtol),
                                     fs.mixed_cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi)
            info = slv(vb, vx)
            res[coding, rtol] = (info, vx.numpy(), slv.mixed_stats())
    for coding in ("grid", "symmetric", "patterns", "colids"):
        info, x, (outer, inner) = res[coding, 1e-8]
        assert info.status == "converged_rtol"
        assert _true_relres(A, b, x) <= 1e-8
        assert abs(info.iters - ref64.iters) <= ITER_TOL
        info2, x2, _ = res[coding, 1e-11]
        assert info2.status == "converged_rtol"
        assert _rel(x2, xs) <= X_RTOL_MIXED
    assert abs(res["patterns", 1e-8][0].iters - res["colids", 1e-8][0].iters) <= 1
    assert abs(res["symmetric", 1e-8][0].iters - res["colids", 1e-8][0].iters) <= 1
    assert abs(res["grid", 1e-8][0].iters - res["colids", 1e-8][0].iters) <= 1
    # with a diagnostic the loop reads back every iteration and a user stop
    # folds the pending solution step into x
    dA.index_coding("symmetric")
    seen = []

    def stop_at_5(x, r):
        seen.append(r)
        return len(seen) >= 5

    vx = fs.Vector(ctx, A.nrows)
    slv = fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=20000, rtol=1e-8),
                             fs.mixed_cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi, stop_at_5)
    info = slv(vb, vx)
    assert info.status == "converged_user" and info.iters == 5
    dA.index_coding("colids")
    seen.clear()
    vx2 = fs.Vector(ctx, A.nrows)
    slv2 = fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=20000, rtol=1e-8),
                              fs.mixed_cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi, stop_at_5)
    slv2(vb, vx2)
    assert _rel(vx.numpy(), vx2.numpy()) <= 1e-5


# ------------------------------------------------------------------ GMRES --

GMRES_CASES = [n for n, c in sorted(META["cases"].items()) if c["method"] == "gmres"]


def _run_gmres(ctx, A, b, x0=None, prec="jacobi", diag=None, **kw):
    return _run(ctx, fs.gmres, A, b, x0, prec, diag, **kw)


@pytest.mark.parametrize("ortho", ["cgs2", "mgs", "dcgs2"])
@pytest.mark.parametrize("name", GMRES_CASES)
def test_gmres_against_reference_fixture(ctx, name, ortho):
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    kw = dict(c["kwargs"])
    x0 = P.uniform(int(c["x0"][1]), A.nrows, 0.0, 1.0) if c["x0"] else None
    prec = kw.pop("precond", "jacobi")
    rtol = kw.pop("rtol", 1e-8)
    info, x, _ = _run_gmres(ctx, A, b, x0, prec, maxiter=kw.pop("maxiter", 2000), rtol=rtol,
                            use_zero_guess=x0 is None, max_krylov_dim=kw.pop("krylov_dim", 30),
                            pre_side=kw.pop("side", "right"), restart=kw.pop("restart", True),
                            ortho=ortho)
    g = np.load(GOLD / f"{name}.npz")
    assert info.status == c["status"]
    assert abs(info.iters - c["iters"]) <= ITER_TOL
    if c["status"] == "converged_rtol":
        assert abs(info.restarts - c["restarts"]) <= 1
        # GMRES stops on its Arnoldi residual estimate, which for left
        # preconditioning is the preconditioned residual: the bar is the
        # reference's own true residual (or rtol, whichever is larger)
        ref_rr = _true_relres(A, b, g["x"])
        assert _true_relres(A, b, x) <= 1.5 * max(rtol, ref_rr)
        _bicgstab_accuracy_bar(A, b, x, g["x"])
    else:
        # no convergence: the same number of Krylov steps gives the same
        # minimal-residual iterate up to rounding
        assert _rel(x, g["x"]) <= 1e-8


def test_gmres_restart_consistency(ctx):
    """gmres.cc:186-208: a restarted run equals 50 steps + a fresh run
    started from their result (same iteration total, same final residual)."""
    A, b = P.workload("convdiff3d-12")  # restarted run converges in 74 (> 50)
    x0 = P.uniform(1, A.nrows, 0.0, 1.0)
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, x0)
    mk = lambda **kw: fs.gmres.solver(fs.gmres.settings(rtol=1e-4, use_zero_guess=False, **kw))(dA, fs.op.I)
    info_restart = mk(maxiter=100, max_krylov_dim=50, restart=True)(vb, vx)
    vx.upload(x0)
    mk(maxiter=50, max_krylov_dim=50, restart=True)(vb, vx)
    info = mk(maxiter=100, max_krylov_dim=100, restart=False)(vb, vx)
    assert info_restart.status == "converged_rtol"
    assert 50 + info.iters == info_restart.iters
    assert info.res_norm_final == info_restart.res_norm_final


@pytest.mark.parametrize("ortho", ["auto", "dcgs2"])
def test_gmres_diagnostic_every_iteration(ctx, ortho):
    A, b = P.workload("convdiff3d-12")
    calls = []
    info, x, _ = _run_gmres(ctx, A, b, diag=lambda xv, r: calls.append(r) or False,
                            maxiter=500, rtol=1e-8, max_krylov_dim=10, restart=True, ortho=ortho)
    assert info.status == "converged_rtol" and len(calls) == info.iters
    r = O.solve("gmres", A, b, maxiter=500, rtol=1e-8, krylov_dim=10)
    assert abs(info.iters - r.iters) <= ITER_TOL
    info2, _, _ = _run_gmres(ctx, A, b, diag=lambda xv, r: len(calls) > 10**9 or r < 1e3,
                             maxiter=500, rtol=1e-8, max_krylov_dim=10, restart=True, ortho=ortho)
    assert info2.status == "converged_user" and info2.iters >= 1


def test_gmres_validate_rejects_reference_asserts(ctx):
    A, b = P.workload("poisson2d-8")
    with pytest.raises(fs.api._lib.FsError) as ei:
        _run_gmres(ctx, A, b, maxiter=10, max_krylov_dim=5, restart=False)
    assert ei.value.status == fs.api._lib.ERR_BREAKDOWN
    with pytest.raises(fs.api._lib.FsError):
        _run_gmres(ctx, A, b, maxiter=1000, max_krylov_dim=101, restart=True)


@pytest.mark.parametrize("ortho", ["auto", "dcgs2"])
@pytest.mark.parametrize("wl", ["convdiff3d-24", "diffusion3d-20", "convdiff3d-13", "convdiff3d-7"])
def test_gmres_cgs2_vs_oracle(ctx, wl, ortho):
    # odd sizes: a last tile of the staged passes that ends inside an element
    # pair (FP32) and a problem smaller than one tile
    A, b = P.workload(wl)
    r = O.solve("gmres", A, b, maxiter=5000, rtol=1e-8, krylov_dim=30)
    info, x, _ = _run_gmres(ctx, A, b, maxiter=5000, rtol=1e-8, max_krylov_dim=30, restart=True,
                            ortho=ortho)
    assert info.status == r.status == "converged_rtol"
    _order_bar("gmres", A, b, info.iters, maxiter=5000, rtol=1e-8, krylov_dim=30)
    _bicgstab_accuracy_bar(A, b, x, r.x)


# ------------------------------------------------- mixed BiCGSTAB / GMRES --

@pytest.mark.parametrize("wl", ["convdiff3d-24", "diffusion3d-24"])
def test_mixed_bicgstab(ctx, wl):
    """FP32 BiCGSTAB with FP64 residual replacement: the stopping test is on
    the FP64 residual and the iteration count stays near the FP64 one."""
    A, b = P.workload(wl)
    r = O.solve("bicgstab", A, b, maxiter=4000, rtol=1e-8)
    info, x, slv = _run(ctx, fs.mixed_bicgstab, A, b, maxiter=4000, rtol=1e-8)
    assert info.status == "converged_rtol"
    assert _true_relres(A, b, x) <= 1e-8
    assert info.iters <= 1.3 * r.iters + 5


@pytest.mark.parametrize("ortho", ["auto", "mgs", "cgs2", "dcgs2"])
@pytest.mark.parametrize("wl", ["convdiff3d-24", "diffusion3d-20", "convdiff3d-13", "convdiff3d-7"])
def test_mixed_gmres(ctx, wl, ortho):
    """FP32 Arnoldi cycles re-anchored on the FP64 residual at every restart:
    converges on the FP64 residual with the FP64 iteration count +- a few."""
    A, b = P.workload(wl)
    r = O.solve("gmres", A, b, maxiter=5000, rtol=1e-8, krylov_dim=30)
    info, x, slv = _run(ctx, fs.mixed_gmres, A, b, maxiter=5000, rtol=1e-8, max_krylov_dim=30,
                        restart=True, ortho=ortho)
    assert info.status == "converged_rtol"
    assert _true_relres(A, b, x) <= 1e-8
    assert info.iters <= 1.2 * r.iters + 30


@pytest.mark.parametrize("name", ["poisson2d-128_cg", "diffusion3d-16_cg", "poisson2d-128_cg_noprec_x0"])
def test_pipelined_cg_against_reference_fixture(ctx, name):
    """The single-reduction CG (the reference's recurrences rearranged,
    Chronopoulos & Gear): the same iterations (+-2), the same stopping test,
    and the solution within 1e-10 of the reference's CG."""
    c = META["cases"][name]
    A, b = P.workload(c["workload"])
    kw = dict(c["kwargs"])
    x0 = P.uniform(int(c["x0"][1]), A.nrows, 0.0, 1.0) if c["x0"] else None
    prec = kw.pop("precond", "jacobi")
    info, x, slv = _run(ctx, fs.pipelined_cg, A, b, x0, prec, maxiter=kw.pop("maxiter", 2000),
                        rtol=kw.pop("rtol", 1e-8), use_zero_guess=kw.pop("use_zero_guess", True))
    g = np.load(GOLD / f"{name}.npz")
    assert info.status == c["status"]
    assert abs(info.iters - c["iters"]) <= ITER_TOL
    assert _true_relres(A, b, x) <= 1e-8 * 1.01
    assert _rel(x, g["x"]) <= X_RTOL_F64
    h = slv.history()
    assert h.size == info.iters
    assert np.allclose(h[:20], g["hist"][:20], rtol=1e-9, atol=0)
