"""The algorithmic-byte models behind bench.py's roofline fractions, pinned
on small hand-computed cases (s_v = value bytes, N rows, K = 3 upper
offsets): every format's SpMV, and the per-step basis traffic of GMRES with
each orthogonalisation."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import bench  # noqa: E402

N, NNZ = 1000, 7000


def test_spmv_bytes_per_format():
    # x read once and y written once: 2 N s_v on top of the matrix data
    assert bench.spmv_bytes(N, NNZ, 4, 0) == NNZ * 4 + 4 * NNZ + 4 * (N + 1) + 8 * N
    assert bench.spmv_bytes(N, NNZ, 8, 1, nblk=4) == NNZ * 8 + N + 16 * 4 + 16 * N
    assert bench.spmv_bytes(N, NNZ, 4, 2) == 4 * N * 4 + N + 8 * N        # diagonal + 3 upper, pattern ids
    assert bench.spmv_bytes(N, NNZ, 4, 3) == 4 * N * 4 + 8 * N            # grid: no index byte
    assert bench.spmv_bytes(N, NNZ, 4, 4) == 7 * N * 4 + 8 * N            # general grid: + 3 lower


def test_gmres_basis_traffic_per_orthogonalisation():
    """Three steps of one cycle (kp1 = 1, 2, 3), no restart: the cycle-end
    terms and the SpMVs are the same for every method, so the differences are
    the basis passes: CGS2 3 (kp1 + 1) + 1 vectors a step; delayed CGS2
    2 (kp1 + 1) + 2 (one write fewer at kp1 = 1); MGS 4 kp1 + 3."""
    sb = 4
    args = (N, NNZ, 3, 0, 3, 0)
    cgs2 = bench.gmres_solve_bytes(*args, m=30, ortho="cgs2", basis_bytes=sb)
    dcgs2 = bench.gmres_solve_bytes(*args, m=30, ortho="dcgs2", basis_bytes=sb)
    mgs = bench.gmres_solve_bytes(*args, m=30, ortho="mgs", basis_bytes=sb)
    vec = N * sb
    assert cgs2 - dcgs2 == ((7 + 10 + 13) - (5 + 8 + 10)) * vec
    assert mgs - dcgs2 == ((7 + 11 + 15) - (5 + 8 + 10)) * vec
    # a restart adds the delayed CGS2's last pass of dots (m + 2 vectors)
    r1 = bench.gmres_solve_bytes(N, NNZ, 3, 0, 3, 1, m=30, ortho="dcgs2", basis_bytes=sb)
    r1_cgs2 = bench.gmres_solve_bytes(N, NNZ, 3, 0, 3, 1, m=30, ortho="cgs2", basis_bytes=sb)
    assert (r1 - dcgs2) - (r1_cgs2 - cgs2) == 32 * vec
