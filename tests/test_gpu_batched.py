"""Batched solves in one persistent launch (one thread-block cluster per
system) against the oracle's CG on every system separately."""
import numpy as np
import pytest

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    return P.batch_diffusion2d(nsys=24, side_lo=6, side_hi=48, seed=11)


@pytest.mark.parametrize("cluster,threads,cluster_systems",
                         [(0, 0, None), (1, 256, None), (2, 512, None), (8, 1024, None),
                          (8, 1024, 0), (8, 512, 6), (4, 1024, 23), (2, 256, 24)])
def test_batch_cg_each_system(ctx, batch, cluster, threads, cluster_systems):
    """Every schedule: every system a whole cluster, or the largest
    `cluster_systems` a whole cluster and the others one CTA each (24
    systems: 0, 6 and 23 own a cluster; a last cluster only partly used)."""
    A, off, b, sides = batch
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    infos = fs.batch_cg(dA, off, vb, vx, maxiter=4000, rtol=1e-8, cluster=cluster,
                        threads=threads, cluster_systems=cluster_systems)
    x = vx.numpy()
    S = A.to_scipy()
    for k, inf in enumerate(infos):
        lo, hi = off[k], off[k + 1]
        Ak = P.CSR(hi - lo, hi - lo, A.rowptr[lo:hi + 1] - A.rowptr[lo],
                   A.col[A.rowptr[lo]:A.rowptr[hi]] - lo, A.val[A.rowptr[lo]:A.rowptr[hi]])
        ref = O.solve("cg", Ak, b[lo:hi], maxiter=4000, rtol=1e-8)
        assert inf.status == "converged_rtol", (k, inf)
        rr = np.linalg.norm(b[lo:hi] - S[lo:hi] @ x) / np.linalg.norm(b[lo:hi])
        assert rr <= 1e-8, (k, rr)
        # FP32 recurrences with FP64 residual replacement keep the FP64 count
        assert abs(inf.iters - ref.iters) <= 3, (k, inf.iters, ref.iters)
    if cluster == 0:
        c, t = fs.batch_tuning(dA, off)
        assert c in (1, 2, 4, 8) and t in (256, 512, 1024)
        c2, t2, nb = fs.batch_schedule(dA, off)
        assert (c2, t2) == (c, t) and 1 <= nb <= len(infos)


def _extend(A, off, b, M, bm):
    """The batch (A, off, b) with one more system M (rhs bm) at the end."""
    rp = np.concatenate([A.rowptr, A.rowptr[-1] + M.rowptr[1:]])
    col = np.concatenate([A.col, M.col + A.nrows])
    val = np.concatenate([A.val, M.val])
    n = A.nrows + M.nrows
    return (P.CSR(n, n, rp, col, val, "block-diagonal"), np.append(off, n),
            np.concatenate([b, bm]))


def test_batch_grid_storage_matches_csr(ctx, batch):
    """A batch of square 2-D grids runs on the grid-stencil storage; the
    same systems with one non-grid system appended (a 27-row 3-D Laplacian)
    run on the column ids.  With one CTA per system the arithmetic of each
    system is independent of the rest of the batch, so the two paths must
    agree bit for bit, iteration counts included."""
    A, off, b, sides = batch
    M, _ = P.workload("laplace3d-3")
    A2, off2, b2 = _extend(A, off, b, M, P.uniform(77, M.nrows))
    out = []
    for Am, om, bm in ((A, off, b), (A2, off2, b2)):
        dA = fs.CSR(ctx, Am)
        vb, vx = fs.Vector(ctx, bm), fs.Vector(ctx, Am.nrows)
        infos = fs.batch_cg(dA, om, vb, vx, maxiter=4000, rtol=1e-8, cluster=1, threads=256,
                            cluster_systems=0)
        out.append((fs.batch_format(dA, om), infos, vx.numpy()))
    assert out[0][0] == "grid" and out[1][0] == "csr"
    n = A.nrows
    assert np.array_equal(out[0][2], out[1][2][:n])
    for k in range(len(off) - 1):
        assert out[0][1][k].iters == out[1][1][k].iters, k
        assert out[0][1][k].res_norm_final == out[1][1][k].res_norm_final, k
    assert out[1][1][-1].status == "converged_rtol"


def test_batch_grid_storage_follows_values(ctx, batch):
    """The storage is re-checked when the values change: one lower entry
    moved by one ulp (no longer equal to its partner) sends the batch to the
    column ids, the original values bring the grid storage back, and both
    solves converge."""
    A, off, b, sides = batch
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    kw = dict(maxiter=4000, rtol=1e-8, cluster=1, threads=256, cluster_systems=0)
    fs.batch_cg(dA, off, vb, vx, **kw)
    assert fs.batch_format(dA, off) == "grid"
    val = A.val.copy()
    r = int(off[3]) + sides[3] + 1  # an interior row of system 3
    k = next(q for q in range(A.rowptr[r], A.rowptr[r + 1]) if A.col[q] == r - 1)
    val[k] = np.nextafter(val[k], np.inf)
    dA.update_values(val)
    infos = fs.batch_cg(dA, off, vb, vx, **kw)
    assert fs.batch_format(dA, off) == "csr"
    assert all(i.status == "converged_rtol" for i in infos)
    dA.update_values(A.val)
    infos = fs.batch_cg(dA, off, vb, vx, **kw)
    assert fs.batch_format(dA, off) == "grid"
    assert all(i.status == "converged_rtol" for i in infos)


def test_batch_rejects_coupled_systems(ctx):
    A, _ = P.workload("poisson2d-10")
    dA = fs.CSR(ctx, A)
    vb, vx = fs.Vector(ctx, np.ones(A.nrows)), fs.Vector(ctx, A.nrows)
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.batch_cg(dA, [0, 50, 100], vb, vx, maxiter=10, rtol=1e-8, cluster=1, threads=256)
    assert ei.value.status == fs.api._lib.ERR_INVALID_ARG


def test_block_cg_16_rhs(ctx):
    """Block CG on 16 right-hand sides: every column converges to rtol on its
    own true residual, no later than single-vector PCG on that column, and
    matches the direct solve."""
    import scipy.sparse.linalg as spla
    A, _ = P.workload("laplace3d-24")
    n = A.nrows
    B = np.stack([P.uniform(6 + j, n) for j in range(16)], axis=1)  # N x 16
    dA = fs.CSR(ctx, A)
    vB, vX = fs.Vector(ctx, B.ravel()), fs.Vector(ctx, n * 16)
    infos = fs.block_cg(dA, vB, vX, 16, maxiter=2000, rtol=1e-8)
    X = vX.numpy().reshape(n, 16)
    S = A.to_scipy()
    lu = spla.splu(S.tocsc())
    for j, inf in enumerate(infos):
        assert inf.status == "converged_rtol", (j, inf)
        rr = np.linalg.norm(B[:, j] - S @ X[:, j]) / np.linalg.norm(B[:, j])
        assert rr <= 1e-8 * 1.5, (j, rr)
        single = O.solve("cg", A, B[:, j], maxiter=2000, rtol=1e-8)
        assert inf.iters <= single.iters + 2, (j, inf.iters, single.iters)
        xs = lu.solve(B[:, j])
        assert np.linalg.norm(X[:, j] - xs) / np.linalg.norm(xs) <= 1e-6


@pytest.mark.parametrize("wl,jacobi", [("laplace3d-24", True), ("diffusion3d-20", True),
                                       ("poisson2d-40", False)])
def test_block_cg_16_rhs_mixed(ctx, wl, jacobi):
    """FP32 block recurrences with FP64 residual replacement: every column
    converges on its own FP64 residual (checked here on the host) and a
    tighter rtol gives the direct solution to the forward-error bound.  On
    the 3-D operators the block iteration count is the FP64 one; on the small
    2-D system the 16-column block Krylov space reaches half the dimension
    (49 FP64 block iterations x 16 columns of 1600 unknowns), where FP64 block
    CG gains from near-finite termination that FP32 recurrences lose (60)."""
    import scipy.sparse.linalg as spla
    A, _ = P.workload(wl)
    n = A.nrows
    B = np.stack([P.uniform(60 + j, n) for j in range(16)], axis=1)
    dA = fs.CSR(ctx, A)
    S = A.to_scipy()
    vB = fs.Vector(ctx, B.ravel())
    vX64, vXm = fs.Vector(ctx, n * 16), fs.Vector(ctx, n * 16)
    i64 = fs.block_cg(dA, vB, vX64, 16, maxiter=4000, rtol=1e-8, jacobi=jacobi)
    imx = fs.block_cg(dA, vB, vXm, 16, maxiter=4000, rtol=1e-8, jacobi=jacobi, mixed=True)
    X = vXm.numpy().reshape(n, 16)

    def slack(it):
        return 3 if wl.startswith(("laplace3d", "diffusion3d")) else 0.25 * it + 3

    for j, inf in enumerate(imx):
        assert inf.status == "converged_rtol", (j, inf)
        rr = np.linalg.norm(B[:, j] - S @ X[:, j]) / np.linalg.norm(B[:, j])
        assert rr < 1e-8, (j, rr)
        assert inf.iters <= i64[j].iters + slack(i64[j].iters), (j, inf.iters, i64[j].iters)
    assert imx[0].restarts <= i64[0].restarts + slack(i64[0].restarts)
    imx2 = fs.block_cg(dA, vB, vXm, 16, maxiter=4000, rtol=1e-12, jacobi=jacobi, mixed=True)
    assert all(i.status == "converged_rtol" for i in imx2)
    X = vXm.numpy().reshape(n, 16)
    lu = spla.splu(S.tocsc())
    for j in range(16):
        xs = lu.solve(B[:, j])
        assert np.linalg.norm(X[:, j] - xs) / np.linalg.norm(xs) <= 1e-8


def test_block_cg_rejects_bad_arguments(ctx):
    A, _ = P.workload("poisson2d-10")
    dA = fs.CSR(ctx, A)
    vB, vX = fs.Vector(ctx, A.nrows * 16), fs.Vector(ctx, A.nrows * 8)
    for mixed in (False, True):
        with pytest.raises(fs.api._lib.FsError) as ei:
            fs.block_cg(dA, vB, vX, 16, maxiter=10, rtol=1e-8, mixed=mixed)
        assert ei.value.status == fs.api._lib.ERR_SIZE_MISMATCH
        with pytest.raises(fs.api._lib.FsError) as ei:
            fs.block_cg(dA, vB, vB, 8, maxiter=10, rtol=1e-8, mixed=mixed)
        assert ei.value.status == fs.api._lib.ERR_UNSUPPORTED
