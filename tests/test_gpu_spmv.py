"""CSR operator on the GPU against the oracle's reference row loop
(flecsolve/matrices/seq.hh:177-193): bit-exact in EXACT mode, within a few
ulps of the row sum in FMA mode; the index formats (column ids, row
patterns, symmetric storage) identical bit for bit; ragged, empty and long
rows; FP32 values; residual; parcsr split; transpose."""
import numpy as np
import pytest

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _bound(A, x):
    # |y_fma - y_exact| <= 2 * nnz_row * eps * sum |a x|
    S = A.to_scipy()
    return 2 * 8 * np.finfo(np.float64).eps * (abs(S) @ np.abs(x))


@pytest.mark.parametrize("wl", ["poisson2d-128", "diffusion3d-24", "convdiff3d-20"])
def test_spmv_exact_mode_is_bit_exact(ctx, wl):
    A, _ = P.workload(wl)
    x = P.uniform(42, A.ncols)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.apply(vx, vy, exact=True)
    assert np.array_equal(vy.numpy(), O.spmv(A, x))
    dA.apply(vx, vy)
    y = vy.numpy()
    assert (np.abs(y - O.spmv(A, x)) <= _bound(A, x)).all()


def _pattern_rect(n2, rows, cols):
    """Rows [0, rows) of the 2-D Poisson operator on an n2 x n2 grid, with the
    entries of columns >= cols dropped: a rectangular stencil matrix."""
    A = P.poisson2d(n2)
    S = A.to_scipy()[:rows, :cols].tocsr()
    S.sort_indices()
    return P.CSR(rows, cols, S.indptr.astype(np.int64), S.indices.astype(np.int32),
                 S.data.astype(np.float64), "poisson-rect")


PATTERN_CASES = ["poisson2d-128", "poisson2d-127", "diffusion3d-24", "diffusion3d-23",
                 "convdiff3d-20", "convdiff3d-21", "rect-wide", "rect-tall", "line-1000",
                 "box-12x5x7", "asym-line-1000", "asym-box-16x9x1", "asym-box-12x5x7"]


def _grid_stencil(nx, ny, nz, seed, asym=False):
    """A symmetric diffusion-like stencil on an nx x ny x nz grid (1-D when
    ny = nz = 1, 2-D when nz = 1) with seeded off-diagonals; `asym`: the lower
    entries drawn separately (the same structure, values not symmetric)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    dims = [d for d in (nx, ny, nz)]
    offs = [1, nx, nx * ny]
    K = 1 if ny == nz == 1 else (2 if nz == 1 else 3)
    r = np.arange(n)
    c = np.stack([r % nx, (r // nx) % ny, r // (nx * ny)])
    rows, cols, vals = [r], [r], [np.full(n, 8.0)]
    for d in range(K):
        keep = c[d] < dims[d] - 1
        v = rng.uniform(-1.0, -0.1, int(keep.sum()))
        vl = rng.uniform(-1.0, -0.1, int(keep.sum())) if asym else v
        rows += [r[keep], r[keep] + offs[d]]
        cols += [r[keep] + offs[d], r[keep]]
        vals += [v, vl]
    M = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    M.sort_indices()
    return P.CSR(n, n, M.indptr.astype(np.int64), M.indices.astype(np.int32), M.data)


def _pattern_matrix(name):
    if name == "line-1000":
        return _grid_stencil(1000, 1, 1, 5)
    if name == "box-12x5x7":
        return _grid_stencil(12, 5, 7, 6)
    if name == "asym-line-1000":
        return _grid_stencil(1000, 1, 1, 7, asym=True)
    if name == "asym-box-16x9x1":
        return _grid_stencil(16, 9, 1, 8, asym=True)
    if name == "asym-box-12x5x7":
        return _grid_stencil(12, 5, 7, 9, asym=True)
    if name == "rect-wide":
        return _pattern_rect(61, 3001, 61 * 61)   # ncols > nrows, odd sizes
    if name == "rect-tall":
        return _pattern_rect(61, 61 * 61, 3003)   # ncols < nrows
    return P.workload(name)[0]


@pytest.mark.parametrize("wl", PATTERN_CASES)
def test_row_pattern_spmv_matches_column_ids(ctx, wl):
    """Stencil matrices carry row patterns.  The grid-stencil kernel (coding
    3: the symmetric storage addressed by grid coordinates, 16-byte loads),
    the symmetric storage (coding 2: diagonal and upper diagonals, lower
    entries read from their partners) and the row-pattern SpMV (coding 1,
    warp-specialised, row offsets from pattern lengths) give the same bits as
    the one reading column ids (coding 0), in every mode and type, on odd
    sizes, 1-, 2- and 3-D grids and rectangular matrices.  A grid stencil with
    nx a multiple of 4 whose values are not symmetric reads the general grid
    storage (active coding 4: the lower diagonals stored at their own rows);
    another matrix that is not symmetric bit for bit falls back to coding 1, a
    symmetric one that is not a grid stencil with nx a multiple of 4 to
    coding 2."""
    A = _pattern_matrix(wl)
    x = P.uniform(43, A.ncols)
    dA = fs.CSR(ctx, A)
    S = A.to_scipy()
    symmetric = A.nrows == A.ncols and (S != S.T).nnz == 0
    nx, ny, nz = dA.grid_dims()
    if wl.startswith(("poisson2d", "diffusion3d", "convdiff3d", "line", "box", "asym")):
        side = int(wl.split("-")[-1].split("x")[0])
        assert nx == side and nx * ny * nz == A.nrows
    grid_ok = nx > 0 and nx % 4 == 0

    def expect(req):
        if req == 0:
            return 0
        if req >= 3 and grid_ok:
            return 3 if symmetric else 4
        return 2 if req >= 2 and symmetric else 1

    assert dA.index_coding() == expect(3)
    out = {}
    for coding in (3, 2, 1, 0):
        assert dA.index_coding(coding) == expect(coding)
        for dt in ("f64", "f32"):
            vx, vy = fs.Vector(ctx, x.astype(np.float32) if dt == "f32" else x, dt), fs.Vector(ctx, A.nrows, dt)
            for exact in (True, False):
                dA.apply(vx, vy, exact=exact)
                out[coding, dt, exact] = vy.numpy()
        if A.nrows == A.ncols:
            b = fs.Vector(ctx, P.uniform(44, A.nrows))
            r = fs.Vector(ctx, A.nrows)
            dA.residual(b, fs.Vector(ctx, x), r)
            out[coding, "res"] = r.numpy()
    for key in [k for k in out if k[0] != 0]:
        assert np.array_equal(out[key], out[(0,) + key[1:]]), key
    assert np.array_equal(out[2, "f64", True], O.spmv(A, x))


def test_symmetric_storage_follows_value_changes(ctx):
    """The symmetric storage is derived from the current values: a value
    change that breaks the symmetry switches the operator (and a bound
    solver's captured iterations) to the general grid storage (coding 4);
    restoring it switches back.  Results follow the values every time."""
    A, b = P.workload("diffusion3d-24")
    x = P.uniform(46, A.ncols)
    dA = fs.CSR(ctx, A)
    assert dA.index_coding() == 3
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    vb = fs.Vector(ctx, b)
    slv = fs.bicgstab.solver(fs.bicgstab.settings(maxiter=2000, rtol=1e-8))(dA, fs.op.jacobi)
    for step in range(3):
        M = P.CSR(A.nrows, A.ncols, A.rowptr, A.col, A.val.copy())
        if step == 1:
            M.val[A.rowptr[100] + 1] *= 1.5     # one lower entry no longer matches its partner
        dA.update_values(M.val)
        assert dA.index_coding() == (4 if step == 1 else 3)
        dA.apply(vx, vy, exact=True)
        assert np.array_equal(vy.numpy(), O.spmv(M, x))
        vsol = fs.Vector(ctx, A.nrows)
        info = slv(vb, vsol)
        assert info.status == "converged_rtol"
        r = b - M.to_scipy() @ vsol.numpy()
        assert np.linalg.norm(r) <= 1.5e-8 * np.linalg.norm(b)


@pytest.mark.parametrize("wl", ["diffusion3d-23", "diffusion3d-24"])
def test_spmv_on_unaligned_wrapped_vectors(ctx, wl):
    """A wrapped device vector that starts on an 8-byte boundary only (a
    torch view at an odd offset) is gathered element by element (the grid
    kernel's 16-byte loads are not used for it): same bits."""
    torch = pytest.importorskip("torch")
    A, _ = P.workload(wl)
    x = P.uniform(45, A.ncols)
    dA = fs.CSR(ctx, A)
    base = torch.zeros(A.ncols + 1, dtype=torch.float64, device="cuda")
    base[1:] = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    xv = fs.Vector.wrap(ctx, A.ncols, base.data_ptr() + 8)   # 8-byte aligned only
    y1, y2 = fs.Vector(ctx, A.nrows), fs.Vector(ctx, A.nrows)
    dA.apply(xv, y1, exact=True)
    dA.apply(fs.Vector(ctx, x), y2, exact=True)
    assert np.array_equal(y1.numpy(), y2.numpy())
    assert np.array_equal(y1.numpy(), O.spmv(A, x))


def test_row_patterns_fall_back_on_irregular_patterns(ctx):
    A = _ragged(3000, 7000, 5)
    dA = fs.CSR(ctx, A)
    assert dA.index_coding() == 0
    assert dA.index_coding(True) == 0
    assert dA.index_coding("symmetric") == 0


def _ragged(n, m, seed, long_rows=()):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, n)
    lens[rng.integers(0, n, 5)] = 0          # empty rows
    for r in long_rows:
        lens[r] = 5000                       # longer than a row block
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(lens)
    col = np.concatenate([np.sort(rng.choice(m, min(l, m), replace=False)) if l else
                          np.zeros(0, dtype=np.int64) for l in lens]).astype(np.int32)
    rp[1:] = np.cumsum([min(l, m) for l in lens])
    val = rng.standard_normal(rp[-1])
    return P.CSR(n, m, rp, col, val, "ragged")


def test_spmv_ragged_empty_and_long_rows(ctx):
    A = _ragged(3000, 7000, 3, long_rows=(17, 2999))
    x = np.random.default_rng(4).standard_normal(A.ncols)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.apply(vx, vy, exact=True)
    assert np.array_equal(vy.numpy(), O.spmv(A, x))
    dA.apply(vx, vy)
    assert (np.abs(vy.numpy() - O.spmv(A, x)) <= 2 * 5000 * 1.2e-16 * (abs(A.to_scipy()) @ np.abs(x))).all()


def test_spmv_index_widths_and_rectangular(ctx):
    A = _ragged(500, 1300, 5)
    A64 = P.CSR(A.nrows, A.ncols, A.rowptr, A.col.astype(np.int64), A.val)
    x = np.random.default_rng(6).standard_normal(A.ncols)
    for M in (A, A64):
        dA = fs.CSR(ctx, M)
        vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, M.nrows)
        dA.apply(vx, vy, exact=True)
        assert np.array_equal(vy.numpy(), O.spmv(A, x))


def test_spmv_f32(ctx):
    A, _ = P.workload("diffusion3d-20")
    x = P.uniform(8, A.ncols).astype(np.float32)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x, "f32"), fs.Vector(ctx, A.nrows, "f32")
    dA.apply(vx, vy)
    A32 = A.to_scipy().astype(np.float32).astype(np.float64)
    ref = A32 @ x.astype(np.float64)
    assert np.abs(vy.numpy() - ref).max() <= 1e-6 * np.abs(ref).max()


def test_residual_and_dinv(ctx):
    A, b = P.workload("convdiff3d-12")
    x = P.uniform(9, A.nrows)
    dA = fs.CSR(ctx, A)
    vb, vx, vr = fs.Vector(ctx, b), fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.residual(vb, vx, vr)
    r = O.residual(A, b, x)
    assert np.abs(vr.numpy() - r).max() <= 1e-13 * np.abs(b).max() * 10
    assert np.array_equal(dA.Dinv().numpy(), O.dinv(A))


@pytest.mark.parametrize("parts", [1, 3, 7])
def test_parcsr_split_is_bit_exact(ctx, parts):
    A, _ = P.workload("convdiff3d-14")
    x = P.uniform(10, A.nrows)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.parcsr_apply(parts, vx, vy)
    assert np.array_equal(vy.numpy(), O.parcsr_spmv(A, parts, x))


def test_transpose_spmv(ctx):
    A = _ragged(800, 600, 11, long_rows=(5,))
    x = np.random.default_rng(12).standard_normal(A.nrows)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.ncols)
    dA.apply_transpose(vx, vy)
    ref = A.to_scipy().T @ x
    assert np.abs(vy.numpy() - ref).max() <= 1e-12 * (abs(A.to_scipy().T) @ np.abs(x)).max()
    # values updated -> the CSC view follows
    A.val *= 2.0
    dA.update_values(A.val)
    dA.apply_transpose(vx, vy)
    assert np.abs(vy.numpy() - 2 * ref).max() <= 2e-12 * (abs(A.to_scipy().T) @ np.abs(x)).max()


def test_bad_inputs_are_rejected(ctx):
    A, _ = P.workload("poisson2d-8")
    bad = P.CSR(A.nrows, A.ncols, A.rowptr, A.col.copy(), A.val)
    bad.col[3] = 10_000
    with pytest.raises(fs.api._lib.FsError) as ei:
        fs.CSR(ctx, bad)
    assert ei.value.status == fs.api._lib.ERR_INVALID_ARG
    dA = fs.CSR(ctx, A)
    with pytest.raises(fs.api._lib.FsError):
        dA.apply(fs.Vector(ctx, 5), fs.Vector(ctx, A.nrows))


def test_matrix_market_operator_on_device(ctx):
    """A file read like the reference reads it drives the device operator and
    solver: the SpMV matches the oracle's row loop bit for bit and CG the
    oracle's iteration count on the float-rounded values."""
    from pathlib import Path
    from flecsolve_gb300.io import matrix_market
    A = matrix_market.read(Path(__file__).resolve().parent / "golden" / "mm" / "diffusion3d-6.mtx")
    x = P.uniform(47, A.ncols)
    dA = fs.CSR(ctx, A)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.apply(vx, vy, exact=True)
    assert np.array_equal(vy.numpy(), O.spmv(A, x))
    b = P.uniform(48, A.nrows)
    ref = O.solve("cg", A, b, maxiter=500, rtol=1e-10)
    vb, vs = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    slv = fs.cg.solver(fs.cg.settings(maxiter=500, rtol=1e-10), fs.cg.make_work(vb))(dA, fs.op.jacobi)
    info = slv(vb, vs)
    assert info.status == ref.status and abs(info.iters - ref.iters) <= 2
    assert np.linalg.norm(vs.numpy() - ref.x) <= 1e-10 * np.linalg.norm(ref.x)


@pytest.mark.parametrize("lanes", [0, 1, 4, 8, 16, 32])
def test_vector_spmv_schedules_on_power_law_rows(ctx, lanes):
    """Irregular rows (16 to 2048 nonzeros, random columns): every column-id
    schedule in FMA mode within the FMA bound of the reference's row sums,
    the same bits on every run; EXACT mode stays the reference's serial
    order whatever the schedule."""
    A = P.powerlaw(20000)
    x = P.uniform(11, A.ncols)
    dA = fs.CSR(ctx, A)
    assert dA.index_coding() == 0
    dA.set_lanes(lanes)
    vx, vy = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    ref = O.spmv(A, x)
    dA.apply(vx, vy)
    y1 = vy.numpy()
    import scipy.sparse as sp

    def csr(vals):
        # duplicate column ids stay separate entries (no scipy cast, which
        # would sum them first)
        return sp.csr_matrix((vals, A.col, A.rowptr), shape=(A.nrows, A.ncols))

    nnz_row = np.diff(A.rowptr)
    bound = 2 * nnz_row * np.finfo(np.float64).eps * (csr(np.abs(A.val)) @ np.abs(x))
    assert (np.abs(y1 - ref) <= bound).all()
    dA.apply(vx, vy)
    assert np.array_equal(vy.numpy(), y1)
    dA.apply(vx, vy, exact=True)
    assert np.array_equal(vy.numpy(), ref)
    # FP32 values
    x32 = x.astype(np.float32)
    dA.set_lanes(lanes, np.float32)
    vx32, vy32 = fs.Vector(ctx, x32, "f32"), fs.Vector(ctx, A.nrows, "f32")
    dA.apply(vx32, vy32)
    v32 = A.val.astype(np.float32).astype(np.float64)
    ref32 = csr(v32) @ x32.astype(np.float64)
    b32 = 2 * nnz_row * np.finfo(np.float32).eps * (csr(np.abs(v32)) @ np.abs(x32.astype(np.float64)))
    assert (np.abs(vy32.numpy() - ref32) <= b32).all()


def test_spmv_autotuner_picks_a_schedule(ctx):
    A = P.powerlaw(50000)
    dA = fs.CSR(ctx, A)
    for dt in (np.float64, np.float32):
        lanes = dA.tune(dt)
        assert lanes in (0, 1, 4, 8, 16, 32)
    with pytest.raises(fs.api._lib.FsError):
        dA.set_lanes(3)
    # stencil operators keep their row formats
    B, _ = P.workload("poisson2d-64")
    assert fs.CSR(ctx, B).tune() == 0


@pytest.mark.parametrize("lanes", [0, 1, 8, 32])
@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_solvers_over_vector_spmv(ctx, lanes, method):
    """The fused solver epilogues on the vector kernel: BiCGSTAB and GMRES(30)
    on a diagonally dominant power-law matrix, iterations within 2 of the
    oracle's, true residual at the tolerance."""
    A, b = P.workload("powerlaw-20000")
    dA = fs.CSR(ctx, A)
    dA.set_lanes(lanes)
    ns = getattr(fs, method)
    kw = dict(max_krylov_dim=30, restart=True) if method == "gmres" else {}
    vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
    slv = ns.solver(ns.settings(maxiter=500, rtol=1e-10, use_zero_guess=True, **kw))(dA, fs.op.jacobi)
    info = slv(vb, vx)
    ref = O.solve(method, A, b, maxiter=500, rtol=1e-10)
    assert info.status == ref.status == "converged_rtol"
    assert abs(info.iters - ref.iters) <= 2
    x = vx.numpy()
    assert np.linalg.norm(b - A.to_scipy() @ x) <= 1.01e-10 * np.linalg.norm(b)
