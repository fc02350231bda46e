"""Seeded synthetic problems (thin ctypes layer over ``libfsproblems.so``).

The generators themselves are in ``csrc/problems.c``; this module only
allocates numpy arrays and names the workloads:

* ``poisson2d(n)``            5-point Laplacian, diagonal 4, off-diagonals -1
* ``diffusion(dim, n, ...)``  variable-coefficient finite-volume diffusion
                              with log-normal cells and harmonic faces
* ``convdiff3d(n, ...)``      7-point upwind convection-diffusion
* ``uniform(seed, n)``        right-hand sides U[-1, 1]

A problem is a :class:`CSR` with int64 row offsets, int32 column ids and
float64 values (the reference's ``mat::csr<double>`` holds ``std::size_t``
indices, flecsolve/matrices/seq.hh:257-261; the C ABI accepts either width).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

from . import build as _build

_i64 = C.c_int64
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


@lru_cache(maxsize=1)
def lib() -> C.CDLL:
    path = _build.build_problems()
    L = C.CDLL(str(path))
    L.fsp_grid_rows.restype = _i64
    L.fsp_grid_rows.argtypes = [C.c_int, _i64]
    L.fsp_grid_nnz.restype = _i64
    L.fsp_grid_nnz.argtypes = [C.c_int, _i64]
    L.fsp_grid_faces.restype = _i64
    L.fsp_grid_faces.argtypes = [C.c_int, _i64]
    L.fsp_uniform.argtypes = [C.c_uint64, _i64, C.c_double, C.c_double, _dp]
    L.fsp_normal.argtypes = [C.c_uint64, _i64, C.c_double, C.c_double, _dp]
    L.fsp_randint.argtypes = [C.c_uint64, _i64, _i64, _i64, _i64p]
    L.fsp_faces_const.argtypes = [C.c_int, _i64, C.c_double, _dp]
    L.fsp_faces_lognormal.argtypes = [C.c_int, _i64, C.c_double, C.c_double,
                                      C.c_uint64, _dp, _dp]
    L.fsp_assemble_diffusion.argtypes = [C.c_int, _i64, _dp, _i64p, _i32p, _dp]
    L.fsp_assemble_convdiff3d.argtypes = [_i64, C.c_double, C.c_uint64, _i64p,
                                          _i32p, _dp, _dp]
    L.fsp_exp_.restype = C.c_double
    L.fsp_exp_.argtypes = [C.c_double]
    L.fsp_log_.restype = C.c_double
    L.fsp_log_.argtypes = [C.c_double]
    return L


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class CSR:
    """Host CSR matrix: int64 ``rowptr``, int32 ``col``, float64 ``val``."""
    nrows: int
    ncols: int
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def diagonal(self) -> np.ndarray:
        d = np.zeros(self.nrows)
        rows = np.repeat(np.arange(self.nrows), np.diff(self.rowptr))
        m = self.col == rows
        d[rows[m]] = self.val[m]
        return d

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowptr),
                             shape=(self.nrows, self.ncols))


def uniform(seed: int, n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(n)
    lib().fsp_uniform(seed, n, lo, hi, _p(out, _dp))
    return out


def normal(seed: int, n: int, mu: float = 0.0, sigma: float = 1.0) -> np.ndarray:
    out = np.empty(n)
    lib().fsp_normal(seed, n, mu, sigma, _p(out, _dp))
    return out


def randint(seed: int, n: int, lo: int, hi: int) -> np.ndarray:
    out = np.empty(n, dtype=np.int64)
    lib().fsp_randint(seed, n, lo, hi, _p(out, _i64p))
    return out


def grid_faces(dim: int, n: int) -> int:
    return int(lib().fsp_grid_faces(dim, n))


def faces_const(dim: int, n: int, c: float = 1.0) -> np.ndarray:
    f = np.empty(grid_faces(dim, n))
    lib().fsp_faces_const(dim, n, c, _p(f, _dp))
    return f


def faces_lognormal(dim: int, n: int, seed: int, sigma: float = 1.0,
                    mu: float = 0.0, return_cells: bool = False):
    f = np.empty(grid_faces(dim, n))
    cells = np.empty(int(lib().fsp_grid_rows(dim, n)))
    lib().fsp_faces_lognormal(dim, n, mu, sigma, seed, _p(f, _dp), _p(cells, _dp))
    return (f, cells) if return_cells else f


def faces_to_fields(n: int, faces: np.ndarray):
    """The 3-D face coefficients of the generator's layout as the three face
    fields of a finite-volume mesh with boundary layers ((n+1)^3 each,
    [k][j][i]; x face f of a line between cells f and f+1 counting the
    boundary cell): with dA/dx = 1 and Dirichlet 0 on every face the
    diffusion operator on those fields is ``assemble_diffusion(3, n, faces)``."""
    m = n * n * (n + 1)
    cx, cy, cz = faces[:m], faces[m:2 * m], faces[2 * m:]
    out = [np.zeros((n + 1, n + 1, n + 1)) for _ in range(3)]
    out[0][1:, 1:, :] = cx.reshape(n, n, n + 1)
    out[1][1:, :, 1:] = cy.reshape(n, n + 1, n)
    out[2][:, 1:, 1:] = cz.reshape(n + 1, n, n)
    return out


def assemble_diffusion(dim: int, n: int, faces: np.ndarray, name: str = "") -> CSR:
    L = lib()
    N = int(L.fsp_grid_rows(dim, n))
    nnz = int(L.fsp_grid_nnz(dim, n))
    faces = np.ascontiguousarray(faces, dtype=np.float64)
    assert faces.size == grid_faces(dim, n)
    rp = np.empty(N + 1, dtype=np.int64)
    col = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz)
    L.fsp_assemble_diffusion(dim, n, _p(faces, _dp), _p(rp, _i64p),
                             _p(col, _i32p), _p(val, _dp))
    return CSR(N, N, rp, col, val, name)


def poisson2d(n: int) -> CSR:
    """5-point Laplacian on an n x n interior grid (diag 4, off -1)."""
    return assemble_diffusion(2, n, faces_const(2, n, 1.0), f"poisson2d-{n}")


def laplace3d(n: int) -> CSR:
    """7-point Laplacian on an n^3 grid (diag 6, off -1)."""
    return assemble_diffusion(3, n, faces_const(3, n, 1.0), f"laplace3d-{n}")


def diffusion(dim: int, n: int, seed: int, sigma: float = 1.0) -> CSR:
    """Log-normal variable-coefficient diffusion with harmonic face averages."""
    return assemble_diffusion(dim, n, faces_lognormal(dim, n, seed, sigma),
                              f"diffusion{dim}d-{n}-s{seed}")


def convdiff3d(n: int, seed: int = 4, pe_max: float = 5.0,
               return_velocity: bool = False):
    """Upwind convection-diffusion with a seeded solenoidal vortex."""
    L = lib()
    N = n ** 3
    nnz = int(L.fsp_grid_nnz(3, n))
    rp = np.empty(N + 1, dtype=np.int64)
    col = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz)
    vel = np.empty(grid_faces(3, n))
    L.fsp_assemble_convdiff3d(n, pe_max, seed, _p(rp, _i64p), _p(col, _i32p),
                              _p(val, _dp), _p(vel, _dp))
    A = CSR(N, N, rp, col, val, f"convdiff3d-{n}-s{seed}")
    return (A, vel) if return_velocity else A


# Workloads named by what they are (sizes and seeds of the benchmark suite).
def powerlaw(n: int, seed: int = 9, xmin: int = 16, alpha: float = 1.6, cap: int = 2048) -> CSR:
    """Irregular n x n matrix with power-law row lengths: a row holds
    min(cap, floor(xmin u^(-1/alpha))) entries (u ~ U[0, 1), seed), the
    first on the diagonal, the others at uniform random columns (seed + 1;
    an accidental diagonal moves one column right) with values U[-1, 1]
    (seed + 2); the diagonal is 1 + the sum of the row's other magnitudes,
    so the matrix is strictly diagonally dominant."""
    u = uniform(seed, n, 0.0, 1.0)
    lens = np.minimum(cap, np.floor(xmin * np.maximum(u, 1e-300) ** (-1.0 / alpha)))
    lens = np.minimum(lens, n).astype(np.int64)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=rowptr[1:])
    nnz = int(rowptr[-1])
    rows = np.repeat(np.arange(n, dtype=np.int64), lens)
    col = randint(seed + 1, nnz, 0, n - 1)
    col = np.where(col == rows, (col + 1) % n, col)
    val = uniform(seed + 2, nnz, -1.0, 1.0)
    starts = rowptr[:-1]
    col[starts] = np.arange(n)
    off = np.abs(val)
    off[starts] = 0.0
    val[starts] = 1.0 + np.add.reduceat(off, starts)
    return CSR(n, n, rowptr, col.astype(np.int32), val, f"powerlaw-{n}")


def workload(name: str):
    """Return (A, b) for a named workload.

    ``poisson2d-128``      2-D Poisson 128^2, RHS U[-1,1] seed 1
    ``diffusion3d-256``    3-D log-normal diffusion 256^3 (faces seed 2,
                           RHS U[-1,1] seed 3)
    ``convdiff3d-192``     3-D upwind convection-diffusion 192^3 (seed 4),
                           RHS U[-1,1] seed 3
    ``powerlaw-2097152``   irregular rows (:func:`powerlaw`, seed 9), n rows,
                           RHS U[-1,1] seed 3
    Any size suffix works (e.g. ``diffusion3d-48``).
    """
    kind, n = name.rsplit("-", 1)
    n = int(n)
    if kind == "poisson2d":
        A = poisson2d(n)
        b = uniform(1, A.nrows)
    elif kind == "diffusion3d":
        A = diffusion(3, n, seed=2)
        b = uniform(3, A.nrows)
    elif kind == "diffusion2d":
        A = diffusion(2, n, seed=2)
        b = uniform(3, A.nrows)
    elif kind == "laplace3d":
        A = laplace3d(n)
        b = uniform(6, A.nrows)
    elif kind == "convdiff3d":
        A = convdiff3d(n, seed=4)
        b = uniform(3, A.nrows)
    elif kind == "powerlaw":
        A = powerlaw(n)
        b = uniform(3, A.nrows)
    else:
        raise ValueError(f"unknown workload {name}")
    A.name = name
    return A, b


def block_diagonal(mats):
    """Concatenate square CSR matrices into one block-diagonal CSR; returns
    (CSR, row offsets)."""
    sizes = [m.nrows for m in mats]
    off = np.zeros(len(mats) + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    nnz = [m.nnz for m in mats]
    noff = np.zeros(len(mats) + 1, dtype=np.int64)
    noff[1:] = np.cumsum(nnz)
    rp = np.empty(off[-1] + 1, dtype=np.int64)
    col = np.empty(noff[-1], dtype=np.int32)
    val = np.empty(noff[-1])
    rp[-1] = noff[-1]
    for k, m in enumerate(mats):
        rp[off[k]:off[k + 1]] = m.rowptr[:-1] + noff[k]
        col[noff[k]:noff[k + 1]] = m.col + off[k]
        val[noff[k]:noff[k + 1]] = m.val
    return CSR(int(off[-1]), int(off[-1]), rp, col, val, "block-diagonal"), off


def batch_diffusion2d(nsys: int = 512, side_lo: int = 32, side_hi: int = 256, seed: int = 5):
    """Independent 2-D log-normal diffusion systems with sides drawn uniformly
    from [side_lo, side_hi] (seed), system s with face seed 1000 + s and RHS
    U[-1,1] seed 2000 + s.  Returns (block-diagonal CSR, offsets, rhs, sides)."""
    sides = randint(seed, nsys, side_lo, side_hi)
    mats = [diffusion(2, int(n), seed=1000 + k) for k, n in enumerate(sides)]
    A, off = block_diagonal(mats)
    b = np.concatenate([uniform(2000 + k, m.nrows) for k, m in enumerate(mats)])
    A.name = f"batch{nsys}-diffusion2d-{side_lo}-{side_hi}"
    return A, off, b, sides
