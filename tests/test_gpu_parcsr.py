"""The distributed CSR operator's colors on the device (fs_parcsr): every
color of a matrix split as read_mat splits it (flecsolve/matrices/
parcsr.hh:133-173), its colmap as the reference's coloring builds it, its
column vector assembled from the owners' values, and y = diag x + offd x of
each color -- the bits of fs_parcsr_spmv on the whole matrix and of the
oracle's parcsr SpMV (parcsr.hh:60-91)."""
import numpy as np
import pytest

import flecsolve_gb300 as fs
import pyoracle as O
from flecsolve_gb300 import parcsr as PC
from flecsolve_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _random(n, seed):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    M = (sp.random(n, n, density=0.01, random_state=rng, format="csr") + sp.eye(n)).tocsr()
    M.sort_indices()
    return P.CSR(n, n, M.indptr.astype(np.int64), M.indices.astype(np.int32), M.data)


@pytest.mark.parametrize("name,colors", [("diffusion3d-12", 2), ("diffusion3d-12", 5),
                                         ("convdiff3d-10", 3), ("random", 4)])
def test_colors_reproduce_parcsr_spmv(ctx, name, colors):
    A = _random(2000, 9) if name == "random" else P.workload(name)[0]
    x = P.uniform(92, A.ncols)
    dA = fs.CSR(ctx, A)
    vx, y_all = fs.Vector(ctx, x), fs.Vector(ctx, A.nrows)
    dA.parcsr_apply(colors, vx, y_all)
    y = np.empty(A.nrows)
    for c in range(colors):
        cr = PC.color_rows(A, c, colors)
        pa = PC.ParCSR(ctx, cr)
        g = pa.ghosts()
        assert np.array_equal(g, cr.ghosts())
        nrows, nown, nghost, nd, no = pa.shape()
        assert (nrows, nown, nghost, nd + no) == (cr.nrows, cr.col_end - cr.col_begin, g.size,
                                                  cr.rowptr[-1])
        # the halo exchange of one process: the owners' values at the ghosts
        xc = fs.Vector(ctx, np.concatenate([x[cr.col_begin:cr.col_end], x[g]]))
        yc = fs.Vector(ctx, cr.nrows)
        pa.apply(xc, yc)
        y[cr.row_begin:cr.row_end] = yc.numpy()
    assert np.array_equal(y, y_all.numpy())
    assert np.array_equal(y, O.parcsr_spmv(A, colors, x))


def test_color_spmv_rejects_wrong_column_vector(ctx):
    A, _ = P.workload("diffusion3d-8")
    cr = PC.color_rows(A, 0, 2)
    pa = PC.ParCSR(ctx, cr)
    bad = fs.Vector(ctx, cr.col_end - cr.col_begin)   # the ghosts missing
    with pytest.raises(fs.api._lib.FsError) as ei:
        pa.apply(bad, fs.Vector(ctx, cr.nrows))
    assert ei.value.status == fs.api._lib.ERR_SIZE_MISMATCH
