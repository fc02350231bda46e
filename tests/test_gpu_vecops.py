"""Vector Data/Operations policy on the GPU against the closed forms of the
reference's vector unit test (flecsolve/vectors/test/flecsi_vector.cc:21-401):
32 dofs, x_i = gid, y_i = 2 gid, z_i = 3 gid, each op checked elementwise
with tolerance 1e-8 * n, plus min/max/dot/l1/l2."""
import numpy as np
import pytest

import flecsolve_gb300 as fs

pytestmark = pytest.mark.gpu

N = 32
GID = np.arange(N, dtype=np.float64)


def _vecs(ctx, dtype):
    mk = lambda a: fs.Vector(ctx, a.astype(np.float32 if dtype == "f32" else np.float64), dtype)
    return mk(GID), mk(2 * GID), mk(3 * GID), fs.Vector(ctx, N, dtype)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_reference_vector_closed_forms(ctx, dtype):
    x, y, z, tmp = _vecs(ctx, dtype)
    tol = N * (1e-8 if dtype == "f64" else 1e-4)

    def check(v, ans):
        assert np.abs(v.numpy() - ans).sum() < tol * max(1.0, np.abs(ans).max() if dtype == "f32" else 1.0)

    X, Y, Z = GID.copy(), 2 * GID, 3 * GID
    tmp.add(x, z); check(tmp, X + Z)
    tmp.subtract(x, z); check(tmp, X - Z)
    tmp.multiply(x, z); check(tmp, X * Z)
    x.add_scalar(x, 1); X = X + 1; check(x, X)
    tmp.divide(y, x); check(tmp, Y / X)
    x.add_scalar(x, -1); X = X - 1
    tmp.scale(2, x); check(tmp, 2 * X)
    y.add_scalar(y, 1); Y = Y + 1
    tmp.reciprocal(y); check(tmp, 1 / Y)
    y.add_scalar(y, -1); Y = Y - 1
    tmp.linear_sum(8, y, 9, z); check(tmp, 8 * Y + 9 * Z)
    tmp.axpy(7, x, y); check(tmp, 7 * X + Y)
    tmp.copy(y); tmp.axpby(4, 11, z); check(tmp, 4 * Z + 11 * Y)
    tmp.add_scalar(y, -4); tmp.abs(tmp); check(tmp, np.abs(Y - 4))
    tmp.add_scalar(y, -7)
    assert tmp.min().get() == -7          # flecsi_vector.cc:376-377
    assert z.max().get() == 93            # flecsi_vector.cc:379
    x.set_scalar(1.5); y.set_scalar(3.8)
    assert abs(x.dot(y).get() - 32 * 1.5 * 3.8) < 1e-8 * (1 if dtype == "f64" else 1e3)
    x.set_scalar(-3.141719)
    assert abs(x.l1norm().get() - 32 * 3.141719) < 1e-8 * (1 if dtype == "f64" else 1e3)
    assert abs(x.l2norm().get() - np.sqrt(32 * 3.141719 ** 2)) < 1e-8 * (1 if dtype == "f64" else 1e3)
    assert x.inf_norm().get() == pytest.approx(3.141719, rel=1e-7)


def test_reductions_large_and_deterministic(ctx):
    n = 3_000_001
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    va, vb = fs.Vector(ctx, a), fs.Vector(ctx, b)
    d1 = va.dot(vb).get()
    d2 = va.dot(vb).get()
    assert d1 == d2  # fixed-order tree: same bits every call
    exact = float(np.dot(a.astype(np.longdouble), b.astype(np.longdouble)))
    assert abs(d1 - exact) <= 1e-13 * np.abs(a * b).sum()
    assert va.l2norm().get() == pytest.approx(np.linalg.norm(a), rel=1e-14)
    assert va.min().get() == a.min() and va.max().get() == a.max()
    assert va.inf_norm().get() == np.abs(a).max()
    assert va.l1norm().get() == pytest.approx(np.abs(a).sum(), rel=1e-13)


def test_f32_compensated_dot_is_accurate(ctx):
    n = 4_000_000
    rng = np.random.default_rng(1)
    a = rng.standard_normal(n).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32)
    va, vb = fs.Vector(ctx, a, "f32"), fs.Vector(ctx, b, "f32")
    exact = float(np.dot(a.astype(np.float64), b.astype(np.float64)))
    # compensated accumulation: error far below plain float summation
    assert abs(va.dot(vb).get() - exact) <= 1e-9 * np.abs(a.astype(np.float64) * b).sum()


def test_empty_and_size_mismatch(ctx):
    e = fs.Vector(ctx, 0)
    e.set_scalar(3.0)
    assert e.dot(e).get() == 0.0
    a, b = fs.Vector(ctx, 5), fs.Vector(ctx, 6)
    with pytest.raises(fs.api._lib.FsError) as ei:
        a.add(a, b)
    assert ei.value.status == fs.api._lib.ERR_SIZE_MISMATCH


def test_set_random_is_seeded(ctx):
    a, b = fs.Vector(ctx, 1000), fs.Vector(ctx, 1000)
    a.set_random(7); b.set_random(7)
    assert np.array_equal(a.numpy(), b.numpy())
    v = a.numpy()
    assert v.min() >= 0 and v.max() < 1 and abs(v.mean() - 0.5) < 0.05
