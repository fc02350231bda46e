"""vec::multi on the device (flecsolve/vectors/multi.hh, operations/multi.hh)
and the multivector CG test of the reference (solvers/test/cgmulti.cc:35-76):
a solver bound to an operator on one variable solves that component of a
multivector with the single-vector iteration count."""
import numpy as np
import pytest

import flecsolve_gb300 as fs
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu


def test_multi_ops_and_reductions(ctx):
    rng = np.random.default_rng(3)
    a = [rng.standard_normal(n) for n in (1000, 37, 4096, 5)]
    b = [rng.standard_normal(n) for n in (1000, 37, 4096, 5)]
    A = fs.Multi(ctx, a, vars=["rho", "u", "v", "e"])
    B = fs.Multi(ctx, b, vars=["rho", "u", "v", "e"])
    T = fs.Multi(ctx, [x.size for x in a])
    T.axpy(2.5, A, B)
    for got, x, y in zip(T.numpy(), a, b):
        assert np.allclose(got, 2.5 * x + y, rtol=0, atol=1e-14)
    assert A.dot(B).get() == pytest.approx(sum(float(x @ y) for x, y in zip(a, b)), rel=1e-13)
    assert A.l2norm().get() == pytest.approx(np.sqrt(sum(float(x @ x) for x in a)), rel=1e-13)
    assert A.l1norm().get() == pytest.approx(sum(np.abs(x).sum() for x in a), rel=1e-13)
    assert A.inf_norm().get() == max(np.abs(x).max() for x in a)
    assert A.min().get() == min(x.min() for x in a)
    assert A.max().get() == max(x.max() for x in a)
    assert np.array_equal(A.subset("v").numpy(), a[2])
    # the components are views of one allocation: the whole vector sees them
    assert np.array_equal(A.whole.numpy(), np.concatenate(a))


def test_multivector_cg_matches_single(ctx):
    """cgmulti.cc: b = (0, rand), x = (rand, rand); CG with the operator on
    var1 (resp. var2) solves that component with the single-vector count."""
    Ah, _ = P.workload("diffusion3d-14")
    n = Ah.nrows
    b2 = P.uniform(3, n, 0.0, 1.0)
    x1, x2 = P.uniform(7, n, 0.0, 1.0), P.uniform(4, n, 0.0, 1.0)
    s = fs.cg.settings(maxiter=2000, rtol=1e-9, use_zero_guess=False)
    for var, xb, bb in (("var1", x1, np.zeros(n)), ("var2", x2, b2)):
        bm = fs.Multi(ctx, [np.zeros(n), b2], vars=["var1", "var2"])
        xm = fs.Multi(ctx, [x1, x2], vars=["var1", "var2"])
        op_v = fs.CSR(ctx, Ah, var=var)
        info_multi = fs.cg.solver(s, fs.cg.make_work(bm.subset(var)))(fs.op.ref(op_v))(bm, xm)
        A1 = fs.CSR(ctx, Ah)
        xs, bs = fs.Vector(ctx, xb), fs.Vector(ctx, bb)
        info_single = fs.cg.solver(s, fs.cg.make_work(bs))(fs.op.ref(A1))(bs, xs)
        assert info_multi.iters == info_single.iters
        assert np.array_equal(xm.subset(var).numpy(), xs.numpy())
        other = "var2" if var == "var1" else "var1"
        assert np.array_equal(xm.subset(other).numpy(), x2 if other == "var2" else x1)
