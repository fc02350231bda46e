"""MatrixMarket input, as the reference reads it.

Mirrors ``flecsolve::mat::io::matrix_market`` (flecsolve/matrices/io/
matrix_market.hh:31-183): ``matrix_market.read(path)`` is
``matrix_market<double>::read(path).tocsr()`` and
``matrix_market.definition(path).matrix(rows)`` cuts a row range the way the
reference's ``definition::matrix`` does for a partitioned operator.  Parsing
and the COO-to-CSR conversion run in the host code of ``libfsgpu.so``
(``fs_mm_*`` in ``include/fsgpu.h``), so no device is needed; the result is a
host :class:`flecsolve_gb300.problems.CSR` that ``CSR(ctx, A)`` uploads.

The reader reproduces the reference's rules, quirks included: values are
read with ``std::stof`` (rounded to float, then widened), a "symmetric"
anywhere in the header (also "skew-symmetric") mirrors the off-diagonal
entries with the same value, fields are separated by single spaces, rows keep
the file order of their entries and duplicates are kept.  Files the
reference's reader throws on raise :class:`FsError` with status ``ERR_IO``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check, lib
from .problems import CSR


class _File:
    def __init__(self, path):
        self.h = C.c_void_p()
        check(lib().fs_mm_read(os.fsencode(os.fspath(path)), C.byref(self.h)), None,
              f"fs_mm_read({path})")
        r, c, z, sym = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
        check(lib().fs_mm_shape(self.h, C.byref(r), C.byref(c), C.byref(z), C.byref(sym)))
        self.nrows, self.ncols, self.nnz, self.symmetric = r.value, c.value, z.value, bool(sym.value)

    def rows(self, begin: int, end: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        nz = C.c_int64()
        check(lib().fs_mm_rows(self.h, begin, end, None, None, None, C.byref(nz)))
        rp = np.empty(end - begin + 1, dtype=np.int64)
        col = np.empty(nz.value, dtype=np.int64)
        val = np.empty(nz.value, dtype=np.float64)
        check(lib().fs_mm_rows(self.h, begin, end, rp.ctypes.data_as(C.c_void_p),
                               col.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p),
                               None))
        return rp, col, val

    def close(self):
        if self.h:
            lib().fs_mm_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _int32_if_fits(col: np.ndarray, ncols: int) -> np.ndarray:
    return col.astype(np.int32) if ncols < 2 ** 31 else col


class matrix_market:
    """``mat::io::matrix_market<double>`` (matrix_market.hh:31)."""

    @staticmethod
    def read(path) -> CSR:
        """The whole matrix: ``read(path).tocsr()`` (matrix_market.hh:64-101,
        seq.hh:324-352)."""
        f = _File(path)
        rp, col, val = f.rows(0, f.nrows)
        return CSR(f.nrows, f.ncols, rp, _int32_if_fits(col, f.ncols), val,
                   os.path.basename(os.fspath(path)))

    class definition:
        """``matrix_market::definition`` (matrix_market.hh:103-165): the
        header is read on construction, the matrix on first use."""

        def __init__(self, path):
            self._f = _File(path)

        def num_rows(self) -> int:
            return self._f.nrows

        def num_cols(self) -> int:
            return self._f.ncols

        def matrix(self, rows) -> CSR:
            """Rows ``rows`` (a contiguous range) with global column ids and
            offsets relative to the range's first entry."""
            rows = range(rows.start, rows.stop) if isinstance(rows, range) else rows
            lo, hi = int(rows[0]), int(rows[-1]) + 1
            if list(rows) != list(range(lo, hi)):
                raise ValueError("definition.matrix takes a contiguous row range")
            rp, col, val = self._f.rows(lo, hi)
            return CSR(hi - lo, self._f.ncols, rp, _int32_if_fits(col, self._f.ncols), val)


__all__ = ["matrix_market"]
