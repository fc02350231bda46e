"""MatrixMarket input against the reference's own reader
(flecsolve/matrices/io/matrix_market.hh + coo::tocsr, matrices/seq.hh:324-352).

The fixtures in tests/golden/mm/ were written by tests/golden/make_mm_golden.py,
which also ran each file through the reference's reader (oracle/_ref/ref_mm)
and stored the CSR it produced.  The reader here must give the same CSR bit
for bit -- values rounded through float, mirrored symmetric entries in file
order, duplicates kept, row ranges cut as definition::matrix cuts them -- and
must reject exactly the files the reference's reader throws on.  Host code
only: no device is needed."""
import json
from pathlib import Path

import numpy as np
import pytest

from flecsolve_gb300 import _lib
from flecsolve_gb300.io import matrix_market

MM = Path(__file__).resolve().parent / "golden" / "mm"
META = json.loads((MM / "golden_mm.json").read_text())["cases"]
GOLD = np.load(MM / "golden_mm.npz")


@pytest.mark.parametrize("case", META, ids=[c["key"] for c in META])
def test_matches_reference_reader(case):
    path = MM / case["file"]
    if case["throws"]:
        with pytest.raises(_lib.FsError) as ei:
            matrix_market.read(path)
        assert ei.value.status == _lib.ERR_IO
        return
    k = case["key"]
    if case["rows"] is None:
        A = matrix_market.read(path)
    else:
        d = matrix_market.definition(path)
        A = d.matrix(range(*case["rows"]))
    nr, nc = GOLD[k + ":shape"]
    assert A.nrows == nr and A.ncols == nc
    assert np.array_equal(A.rowptr, GOLD[k + ":rowptr"])
    assert np.array_equal(A.col.astype(np.int64), GOLD[k + ":col"])
    # bit for bit (also -0.0 and the float rounding of every value)
    assert np.array_equal(A.val.view(np.uint64), GOLD[k + ":val"].view(np.uint64))


def test_values_are_rounded_through_float():
    A = matrix_market.read(MM / "general.mtx")
    assert np.array_equal(A.val, A.val.astype(np.float32).astype(np.float64))
    assert (A.val == np.float64(np.float32(0.1))).any()


def test_symmetric_mirror_follows_each_entry():
    # the mirrored entry lands in the other row right after the entries that
    # precede it in the file: rows keep file order
    A = matrix_market.read(MM / "symmetric.mtx")
    S = A.to_scipy()
    assert (S != S.T).nnz == 0
    lo = matrix_market.read(MM / "skew.mtx").to_scipy()
    assert (lo != lo.T).nnz == 0  # "skew-symmetric" mirrors with the same sign


def test_out_of_range_ids_and_missing_file(tmp_path):
    for body in ("2 2 1\n3 1 1.0\n", "2 2 1\n0 1 1.0\n", "2 2 1\n1 5 1.0\n"):
        p = tmp_path / "bad.mtx"
        p.write_text("%%MatrixMarket matrix coordinate real general\n" + body)
        with pytest.raises(_lib.FsError) as ei:
            matrix_market.read(p)
        assert ei.value.status == _lib.ERR_IO
    with pytest.raises(_lib.FsError) as ei:
        matrix_market.read(tmp_path / "missing.mtx")
    assert ei.value.status == _lib.ERR_IO


def test_definition_sizes_and_ranges():
    d = matrix_market.definition(MM / "diffusion3d-6.mtx")
    assert (d.num_rows(), d.num_cols()) == (216, 216)
    whole = matrix_market.read(MM / "diffusion3d-6.mtx")
    parts = [d.matrix(range(a, b)) for a, b in ((0, 70), (70, 150), (150, 216))]
    assert np.array_equal(np.concatenate([p.val for p in parts]), whole.val)
    assert np.array_equal(np.concatenate([p.col for p in parts]), whole.col)
    with pytest.raises(ValueError):
        d.matrix([0, 2, 3])
