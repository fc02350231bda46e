"""Generate the MatrixMarket fixtures in tests/golden/mm/ and their CSR as the
reference's own reader produces it.

Writes small MatrixMarket files that cover the reference reader's rules
(flecsolve/matrices/io/matrix_market.hh): general / symmetric / integer
fields, "symmetric" in a comment or in "skew-symmetric", unsorted entries and
duplicates, CRLF line ends, values that round when read as float, a row
range cut by definition::matrix, and files the reader throws on (no value
field, values outside the float range, a doubled separator, too few entry
lines, an index outside int) -- and a pattern file, whose missing value
field the reader fills with the column field.  Each file is run through ``oracle/_ref/ref_mm``
(``make -C oracle ref``: the reference header compiled with the stand-ins of
oracle/ref_shim) and the CSR it wrote is stored in ``golden_mm.npz``; the
list of cases and whether the reference threw is ``golden_mm.json``.

Usage (needs the reference headers, i.e. only where they are mounted):
    python tests/golden/make_mm_golden.py
"""
from __future__ import annotations

import json
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
MM = HERE / "mm"
sys.path.insert(0, str(ROOT))

from flecsolve_gb300 import problems as P  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "ref_mm"


def write(name: str, text: str, newline: str = "\n") -> Path:
    p = MM / name
    p.write_bytes(text.replace("\n", newline).encode())
    return p


def entries(rows, cols, vals, fmt="{:.17g}"):
    return "".join(f"{r} {c} {fmt.format(v)}\n" for r, c, v in zip(rows, cols, vals))


def make_files() -> list[tuple[str, list]]:
    """(file, [row ranges]) -- an empty range list reads the whole matrix."""
    MM.mkdir(exist_ok=True)
    rng = np.random.default_rng(20251204)
    cases = []
    # general real: unsorted, duplicates, values of many magnitudes, -0
    n, m, k = 23, 19, 70
    r = rng.integers(1, n + 1, k)
    c = rng.integers(1, m + 1, k)
    r[10], c[10] = r[3], c[3]  # duplicate entries
    v = rng.standard_normal(k) * 10.0 ** rng.integers(-30, 30, k)
    v[5] = -0.0
    v[6] = 0.1
    write("general.mtx", "%%MatrixMarket matrix coordinate real general\n% a comment\n"
          f"{n} {m} {k}\n" + entries(r, c, v))
    cases.append(("general.mtx", []))
    # symmetric: lower triangle with diagonal, mirrored by the reader
    n = 30
    lo = [(i, j) for i in range(1, n + 1) for j in range(1, i + 1) if (i * 7 + j * 3) % 5 == 0 or i == j]
    rng.shuffle(lo)
    v = rng.uniform(-1, 1, len(lo))
    write("symmetric.mtx", "%%MatrixMarket matrix coordinate real symmetric\n"
          f"{n} {n} {len(lo)}\n" + entries([a for a, _ in lo], [b for _, b in lo], v))
    cases.append(("symmetric.mtx", []))
    cases.append(("symmetric.mtx", [[5, 17], [0, 30], [29, 30]]))
    # skew-symmetric header: the reader mirrors with the same sign
    sl = [(i, j) for i in range(2, 12) for j in range(1, i) if (i + j) % 3 == 0]
    write("skew.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric\n"
          f"11 11 {len(sl)}\n" + entries([a for a, _ in sl], [b for _, b in sl], rng.uniform(-2, 2, len(sl))))
    cases.append(("skew.mtx", []))
    # "symmetric" in a comment of a general file
    write("comment_symmetric.mtx", "%%MatrixMarket matrix coordinate real general\n"
          "% not symmetric at all\n5 5 4\n2 1 1.5\n3 3 2\n5 1 -1e-3\n4 5 7\n")
    cases.append(("comment_symmetric.mtx", []))
    # integer field
    write("integer.mtx", "%%MatrixMarket matrix coordinate integer general\n"
          "4 6 5\n1 6 3\n4 1 -12\n2 2 123456789\n1 1 7\n4 6 0\n")
    cases.append(("integer.mtx", []))
    # CRLF line ends
    write("crlf.mtx", "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1 1.25\n2 3 0.3\n3 2 -4\n",
          newline="\r\n")
    cases.append(("crlf.mtx", []))
    # a generated diffusion operator, every value rounding when read as float
    A, _ = P.workload("diffusion3d-6")
    rows = np.repeat(np.arange(A.nrows), np.diff(A.rowptr)) + 1
    write("diffusion3d-6.mtx", "%%MatrixMarket matrix coordinate real general\n"
          f"{A.nrows} {A.ncols} {A.nnz}\n" + entries(rows, A.col + 1, A.val))
    cases.append(("diffusion3d-6.mtx", []))
    cases.append(("diffusion3d-6.mtx", [[50, 130], [200, 216], [0, 1]]))
    # files the reference's reader throws on
    write("pattern.mtx", "%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 1\n2 3\n")
    write("overflow.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n2 2 1e39\n")
    write("underflow.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n2 2 1e-50\n")
    write("double_space.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n2  2 1\n")
    write("short.mtx", "%%MatrixMarket matrix coordinate real general\n4 4 5\n1 1 1\n2 2 1\n3 3 1\n4 4 1\n")
    write("int_range.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 1\n99999999999 1 1\n")
    for f in ("pattern.mtx", "overflow.mtx", "underflow.mtx", "double_space.mtx", "short.mtx",
              "int_range.mtx"):
        cases.append((f, []))
    return cases


def run_ref(path: Path, rng=None):
    out = MM / "_ref.bin"
    cmd = [str(REF), str(path), str(out)] + ([str(rng[0]), str(rng[1])] if rng else [])
    subprocess.run(cmd, check=True)
    b = out.read_bytes()
    out.unlink()
    ok = struct.unpack_from("<i", b, 0)[0]
    if not ok:
        return None
    nr, nc, nz = struct.unpack_from("<qqq", b, 4)
    o = 28
    rp = np.frombuffer(b, "<i8", nr + 1, o)
    o += 8 * (nr + 1)
    col = np.frombuffer(b, "<i8", nz, o)
    o += 8 * nz
    val = np.frombuffer(b, "<f8", nz, o)
    return nr, nc, rp.copy(), col.copy(), val.copy()


def main():
    if not REF.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    arrays, meta = {}, []
    for fname, ranges in make_files():
        for rg in (ranges or [None]):
            key = fname.replace(".mtx", "") + (f"@{rg[0]}-{rg[1]}" if rg else "")
            res = run_ref(MM / fname, rg)
            meta.append({"key": key, "file": fname, "rows": rg, "throws": res is None})
            if res is not None:
                nr, nc, rp, col, val = res
                arrays[key + ":shape"] = np.array([nr, nc], dtype=np.int64)
                arrays[key + ":rowptr"] = rp
                arrays[key + ":col"] = col
                arrays[key + ":val"] = val
    np.savez_compressed(MM / "golden_mm.npz", **arrays)
    (MM / "golden_mm.json").write_text(json.dumps({"cases": meta}, indent=1) + "\n")
    print(f"{len(meta)} cases, {sum(c['throws'] for c in meta)} rejected by the reference")


if __name__ == "__main__":
    main()
