"""CPU tests of the adjoint's host logic: the face layout helpers agree with
the generator's assembly, the face-gradient formula agrees with central
finite differences of dense solves, and the checkpoint schedule covers every
time step exactly once."""
import numpy as np
import pytest

from flecsolve_gb300 import adjoint as ad
from flecsolve_gb300 import problems as P


@pytest.mark.parametrize("dim,n", [(2, 4), (3, 3)])
def test_face_delta_matches_assembled_unit_faces(dim, n):
    """K(e_f) x from the local stencil equals the generator's matrix for the
    single-face coefficient field e_f, for every face."""
    nf = P.grid_faces(dim, n)
    x = P.uniform(11, n ** dim)
    for f in range(nf):
        e = np.zeros(nf)
        e[f] = 1.0
        K = P.assemble_diffusion(dim, n, e).to_scipy()
        np.testing.assert_allclose(ad.face_delta_apply(dim, n, [f], 1.0, x), K @ x,
                                   rtol=0, atol=1e-15)


def test_face_cells_cover_each_interior_pair_once():
    dim, n = 3, 5
    a, b = ad.face_cells(dim, n, np.arange(P.grid_faces(dim, n)))
    inner = (a >= 0) & (b >= 0)
    A = P.laplace3d(n).to_scipy().tocoo()
    off = {(int(i), int(j)) for i, j in zip(A.row, A.col) if i < j}
    assert {(int(i), int(j)) for i, j in zip(a[inner], b[inner])} == off
    # 6 n^2 boundary faces, each touching exactly one cell
    assert (~inner).sum() == 6 * n * n
    assert ((a < 0) ^ (b < 0))[~inner].all()


def test_face_gradient_formula_matches_dense_fd():
    """dL/dc_f = -(lam_a - lam_b)(x_a - x_b) (interior), -lam_c x_c
    (boundary), dL/db = lam, for L = ||A(c)^-1 b - t||^2 with dense solves."""
    dim, n = 2, 5
    c = P.faces_lognormal(dim, n, seed=2)
    b = P.uniform(3, n * n)
    t = P.uniform(4, n * n)

    def loss(cc, bb):
        A = P.assemble_diffusion(dim, n, cc).to_scipy().toarray()
        x = np.linalg.solve(A, bb)
        return float((x - t) @ (x - t))

    A = P.assemble_diffusion(dim, n, c).to_scipy().toarray()
    x = np.linalg.solve(A, b)
    lam = np.linalg.solve(A.T, 2 * (x - t))
    fa, fb = ad.face_cells(dim, n, np.arange(c.size))
    inner = (fa >= 0) & (fb >= 0)
    g = np.where(inner, -(lam[fa] - lam[fb]) * (x[fa] - x[fb]), 0.0)
    cb = np.where(fa >= 0, fa, fb)
    g[~inner] = -lam[cb[~inner]] * x[cb[~inner]]
    for f in range(c.size):
        h = 1e-6 * abs(c[f])
        cp, cm = c.copy(), c.copy()
        cp[f] += h
        cm[f] -= h
        fd = (loss(cp, b) - loss(cm, b)) / (2 * h)
        assert fd == pytest.approx(g[f], rel=1e-5, abs=1e-9)
    for i in range(0, n * n, 3):
        h = 1e-6 * abs(b[i])
        bp, bm = b.copy(), b.copy()
        bp[i] += h
        bm[i] -= h
        assert (loss(c, bp) - loss(c, bm)) / (2 * h) == pytest.approx(lam[i], rel=1e-5, abs=1e-9)


@pytest.mark.parametrize("nsteps,every", [(200, 20), (7, 3), (5, 5), (1, 20), (21, 20)])
def test_checkpoint_segments_cover_all_steps_in_reverse(nsteps, every):
    segs = ad.checkpoint_segments(nsteps, every)
    assert segs[0][1] == nsteps and segs[-1][0] == 0
    steps = [k for s0, s1 in segs for k in range(s1 - 1, s0 - 1, -1)]
    assert steps == list(range(nsteps - 1, -1, -1))
    assert all(s0 % every == 0 and 0 < s1 - s0 <= every for s0, s1 in segs)
    assert ad.checkpoint_segments(0, every) == []
