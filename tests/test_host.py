"""CPU tests of the host side: the C ABI library loads and exports every
symbol declared in include/*.h, argument checking needs no GPU, and the
generators produce the operators they claim (symmetry, divergence-free
convection, M-matrix signs)."""
import ctypes as C
import os

import numpy as np
import pytest

from flecsolve_gb300 import _lib, build, problems as P


@pytest.fixture(scope="module")
def L():
    build.build_gpu()
    return _lib.lib()


def test_library_exports_every_header_symbol(L):
    names = _lib.header_symbols()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(L, n)]
    assert missing == []


def test_status_strings_and_bad_handles(L):
    assert L.fs_status_string(0) == b"ok"
    assert L.fs_status_string(_lib.ERR_BREAKDOWN) == b"solver breakdown"
    n = C.c_int64()
    assert L.fs_vec_size(None, C.byref(n)) == _lib.ERR_BAD_HANDLE
    assert L.fs_csr_destroy(None) == _lib.ERR_BAD_HANDLE
    assert L.fs_krylov_destroy(None) == _lib.ERR_BAD_HANDLE
    assert L.fs_ctx_create(0, None) == _lib.ERR_INVALID_ARG
    s = _lib.KrylovSettings()
    assert L.fs_krylov_settings_default(C.byref(s)) == 0
    # gmres.hh:414-418 defaults
    assert (s.max_krylov_dim, s.pre_side, s.restart) == (-1, _lib.RIGHT, 0)


def test_no_device_is_reported_not_faked(L):
    """Without a usable device the context call fails with FS_ERR_NO_DEVICE:
    nothing falls back to the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert L.fs_ctx_create(0, C.byref(h)) == _lib.ERR_NO_DEVICE


def test_diffusion_is_symmetric_positive_diagonal():
    A = P.diffusion(3, 9, seed=3).to_scipy()
    assert abs(A - A.T).max() == 0.0
    d = A.diagonal()
    assert (d > 0).all()
    off = A - __import__("scipy.sparse", fromlist=["diags"]).diags(d)
    assert off.max() <= 0.0
    # diagonally dominant rows (boundary rows strictly)
    rs = np.asarray(abs(off).sum(axis=1)).ravel()
    assert (d >= rs - 1e-12 * d).all()


def test_poisson_is_classic_five_point():
    A = P.poisson2d(6)
    S = A.to_scipy().toarray()
    assert set(np.diag(S)) == {4.0}
    assert set(np.unique(S[S != 0])) == {-1.0, 4.0}
    assert A.nnz == 5 * 36 - 4 * 6


def test_convdiff_vortex_is_divergence_free_and_m_matrix():
    n = 10
    A, vel = P.convdiff3d(n, seed=4, return_velocity=True)
    assert abs(vel).max() == pytest.approx(5.0)
    ux = vel[: n * n * (n + 1)].reshape(n, n, n + 1)
    uy = vel[n * n * (n + 1): 2 * n * n * (n + 1)].reshape(n, n + 1, n)
    uz = vel[2 * n * n * (n + 1):].reshape(n + 1, n, n)
    div = (ux[:, :, 1:] - ux[:, :, :-1]) + (uy[:, 1:, :] - uy[:, :-1, :]) + (uz[1:] - uz[:-1])
    assert abs(div).max() < 1e-12
    # no normal flow through the walls
    assert abs(ux[:, :, 0]).max() == 0 and abs(ux[:, :, -1]).max() == 0
    S = A.to_scipy()
    d = S.diagonal()
    off = S - __import__("scipy.sparse", fromlist=["diags"]).diags(d)
    assert off.max() <= 0.0 and (d > 0).all()
    assert abs(S - S.T).max() > 0.1  # genuinely nonsymmetric


def test_own_exp_log_match_libm_closely():
    L = P.lib()
    for x in (-3.7, -0.5, 0.0, 1e-3, 0.69, 2.5, 10.0):
        assert L.fsp_exp_(x) == pytest.approx(np.exp(x), rel=4e-16)
    for x in (1e-9, 0.3, 0.999, 1.0, 1.7, 123.0):
        assert L.fsp_log_(x) == pytest.approx(np.log(x), rel=4e-16, abs=4e-16)


def test_lognormal_statistics():
    f, cells = P.faces_lognormal(3, 20, seed=2, return_cells=True)
    lg = np.log(cells)
    assert abs(lg.mean()) < 0.05 and abs(lg.std() - 1.0) < 0.05


def test_cpp_api_header_compiles_and_links():
    """The C++ mirror of the reference's API builds against the C ABI
    (running it needs a GPU: tests/test_gpu_cpp_api.py)."""
    exe = build.build_cpp_tests()
    assert exe.exists()


def test_flecsolve_device_binding_compiles():
    """include/flecsolve_gb300/flecsolve_device.hh under flecsolve's own
    solver templates (where a flecsolve checkout is staged): the program that
    runs them on the GPU builds and links against the library."""
    from flecsolve_gb300 import build
    build.build_gpu()
    exe = build.build_template_test()
    if exe is None:
        pytest.skip("no flecsolve checkout staged in baseline/_ref")
    assert exe.exists()
