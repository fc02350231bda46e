"""Distributed CSR operator: flecsolve's ``mat::parcsr`` over ``topo::csr``
(flecsolve/matrices/parcsr.hh:29-177, flecsolve/topo/csr.hh:413-632), one
color per rank, with a host-staged halo exchange.

* Rows and columns are split into ``colors`` contiguous blocks as
  ``flecsi::util::equal_map`` splits them (FleCSI 2.4, a dependency absent
  from the reference; its published rule: blocks of n // colors, the first
  n % colors one longer), as ``read_mat`` distributes a matrix
  (parcsr.hh:133-173).
* A color's ghost columns are the column ids of its rows outside its own
  column block, sorted and unique (the colmap of topo/csr.hh:501-518); its
  column vector is [owned values, ghost values in colmap order].
* :class:`HaloPlan` is the copy plan (topo/csr.hh:240-304): for every peer
  the ghost ids it owns (received) and the owned rows it needs (sent).  The
  exchange stages the values through host memory over a
  ``torch.distributed`` process group (``gloo`` works without a GPU), one
  point-to-point message per neighbour.
* :class:`ParCSR` is one color on the device (``fs_parcsr``): y = diag x +
  offd x_cols with the reference's row arithmetic, the bits of
  ``fs_parcsr_spmv`` on the whole matrix.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np


def equal_map_start(n: int, colors: int, c: int) -> int:
    """First index of block c when n indices are split into `colors` blocks
    (blocks of n // colors, the first n % colors one longer)."""
    q, r = divmod(n, colors)
    return c * q + min(c, r)


def equal_map_bin(n: int, colors: int, i):
    """The block of index (or index array) i."""
    q, r = divmod(n, colors)
    i = np.asarray(i)
    brk = (q + 1) * r
    return np.where(i < brk, i // (q + 1), r + (i - brk) // max(q, 1))


@dataclass
class ColorRows:
    """The rows of one color of a global CSR matrix, with global column ids
    (what read_mat hands a color, parcsr.hh:146-156)."""
    color: int
    colors: int
    nrows_global: int
    ncols_global: int
    row_begin: int
    row_end: int
    col_begin: int
    col_end: int
    rowptr: np.ndarray   # int64, local
    gcol: np.ndarray     # int64, global column ids
    val: np.ndarray      # float64

    @property
    def nrows(self) -> int:
        return self.row_end - self.row_begin

    def ghosts(self) -> np.ndarray:
        """The colmap: global ids of the columns outside the owned block,
        sorted and unique."""
        c = self.gcol
        return np.unique(c[(c < self.col_begin) | (c >= self.col_end)]).astype(np.int64)

    def split(self):
        """init_mats (topo/csr.hh:553-618) on the host: the diag and offd
        parts, each row in input order; offd columns are nown + the ghost's
        position in the colmap."""
        g = self.ghosts()
        nown = self.col_end - self.col_begin
        own = (self.gcol >= self.col_begin) & (self.gcol < self.col_end)
        rows = np.repeat(np.arange(self.nrows), np.diff(self.rowptr))
        dcol = (self.gcol[own] - self.col_begin).astype(np.int64)
        ocol = (nown + np.searchsorted(g, self.gcol[~own])).astype(np.int64)
        drp = np.zeros(self.nrows + 1, np.int64)
        orp = np.zeros(self.nrows + 1, np.int64)
        np.add.at(drp, rows[own] + 1, 1)
        np.add.at(orp, rows[~own] + 1, 1)
        return (np.cumsum(drp), dcol, self.val[own]), (np.cumsum(orp), ocol, self.val[~own]), g


def color_rows(A, color: int, colors: int) -> ColorRows:
    """The rows of `color` of the global CSR `A` (rowptr / col / val)."""
    n, m = int(A.nrows), int(A.ncols)
    r0, r1 = equal_map_start(n, colors, color), equal_map_start(n, colors, color + 1)
    c0, c1 = equal_map_start(m, colors, color), equal_map_start(m, colors, color + 1)
    rp = np.asarray(A.rowptr, np.int64)
    k0, k1 = int(rp[r0]), int(rp[r1])
    return ColorRows(color, colors, n, m, r0, r1, c0, c1, rp[r0:r1 + 1] - k0,
                     np.asarray(A.col[k0:k1], np.int64), np.asarray(A.val[k0:k1], np.float64))


def host_color_spmv(cr: ColorRows, x_cols: np.ndarray) -> np.ndarray:
    """y = diag x + offd x_cols on the host with the reference's arithmetic
    (each part's row sum left to right, products rounded, then added) -- the
    checker of the host-side plan and exchange (small sizes: a Python loop)."""
    (drp, dcol, dval), (orp, ocol, oval), _ = cr.split()
    y = np.empty(cr.nrows)
    for i in range(cr.nrows):
        yd = 0.0
        for k in range(drp[i], drp[i + 1]):
            yd += float(dval[k]) * float(x_cols[dcol[k]])
        yo = 0.0
        for k in range(orp[i], orp[i + 1]):
            yo += float(oval[k]) * float(x_cols[ocol[k]])
        y[i] = yd + yo
    return y


class HaloPlan:
    """The copy plan of one color: which ghost values come from which owner,
    and which owned values each peer needs.  Built collectively (every rank
    of `group` calls it with its own color, one color per rank)."""

    def __init__(self, cr: ColorRows, group=None):
        import torch.distributed as dist
        self.cr = cr
        self.ghosts = cr.ghosts()
        owners = equal_map_bin(cr.ncols_global, cr.colors, self.ghosts) if self.ghosts.size else \
            np.zeros(0, np.int64)
        self.recv = {int(q): np.nonzero(owners == q)[0] for q in np.unique(owners)}
        # every rank learns what every other needs from it
        world = dist.get_world_size(group)
        assert world == cr.colors, "one color per rank"
        req = {int(q): self.ghosts[idx] for q, idx in self.recv.items()}
        allreq = [None] * world
        dist.all_gather_object(allreq, req, group=group)
        self.send = {}
        for p in range(world):
            if p == cr.color:
                continue
            want = allreq[p].get(cr.color)
            if want is not None and len(want):
                self.send[p] = (np.asarray(want, np.int64) - cr.col_begin)
        self.group = group

    def exchange(self, x_own: np.ndarray) -> np.ndarray:
        """The color's column vector [x_own, ghost values]: the owned values
        every peer needs are sent, the ghost values received (host-staged
        point-to-point messages, a fixed order per pair)."""
        import torch
        import torch.distributed as dist
        nown = self.cr.col_end - self.cr.col_begin
        out = np.empty(nown + self.ghosts.size)
        out[:nown] = x_own
        reqs = []
        bufs = {}
        for q, idx in sorted(self.recv.items()):
            bufs[q] = torch.empty(idx.size, dtype=torch.float64)
            reqs.append(dist.irecv(bufs[q], src=q, group=self.group))
        for p, idx in sorted(self.send.items()):
            reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(x_own[idx])), dst=p,
                                   group=self.group))
        for r in reqs:
            r.wait()
        for q, idx in self.recv.items():
            out[nown + idx] = bufs[q].numpy()
        return out


class ParCSR:
    """One color on the device (``fs_parcsr``)."""

    def __init__(self, ctx, cr: ColorRows):
        from ._lib import check, lib
        self.ctx, self.cr = ctx, cr
        rp = np.ascontiguousarray(cr.rowptr, np.int64)
        gc = np.ascontiguousarray(cr.gcol, np.int64)
        va = np.ascontiguousarray(cr.val, np.float64)
        h = C.c_void_p()
        check(lib().fs_parcsr_create(ctx.h, cr.col_begin, cr.col_end, cr.nrows,
                                     rp.ctypes.data_as(C.c_void_p), gc.ctypes.data_as(C.c_void_p),
                                     va.ctypes.data_as(C.c_void_p), C.byref(h)),
              ctx.h, "fs_parcsr_create")
        self.h = h

    def ghosts(self) -> np.ndarray:
        from ._lib import check, lib
        n = C.c_int64(0)
        check(lib().fs_parcsr_ghosts(self.h, None, C.byref(n)), self.ctx.h)
        out = np.empty(n.value, np.int64)
        m = C.c_int64(out.size)
        check(lib().fs_parcsr_ghosts(self.h, out.ctypes.data_as(C.c_void_p), C.byref(m)), self.ctx.h)
        return out[: m.value]

    def shape(self):
        from ._lib import check, lib
        v = [C.c_int64() for _ in range(5)]
        check(lib().fs_parcsr_shape(self.h, *[C.byref(x) for x in v]), self.ctx.h)
        return tuple(x.value for x in v)

    def apply(self, x_cols, y):
        """y = diag x + offd x_cols (device vectors: x_cols holds the owned
        then the ghost values)."""
        from ._lib import check, lib
        check(lib().fs_parcsr_color_spmv(self.h, x_cols.h, y.h), self.ctx.h, "fs_parcsr_color_spmv")

    def __del__(self):
        try:
            if getattr(self, "h", None):
                from ._lib import lib
                lib().fs_parcsr_destroy(self.h)
                self.h = None
        except Exception:
            pass
