"""The allocation-free dot product (fs_dot_f64_noalloc) against the library's
context-based dot (fs_vec_dot), through the C ABI.

The entry point is for callers that cannot allocate device memory (their
device memory belongs to another allocator, they cannot take cudaMalloc's
implicit synchronisation, or they hold only raw pointers and a stream); its
scratch is a static device array.  This file is collected last so that a run
stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import flecsolve_gb300 as fs
from flecsolve_gb300 import _lib

pytestmark = pytest.mark.gpu

MAX_N = 67108864  # FS_DOT_NOALLOC_MAX_N


def _fn():
    L = _lib.lib()
    f = L.fs_dot_f64_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _call(ctx, a, b, n, out):
    return _fn()(C.c_void_p(a.device_ptr), C.c_void_p(b.device_ptr), n,
                 C.c_void_p(out.device_ptr), C.c_void_p(ctx.stream))


@pytest.mark.parametrize("n", [3_000_001, 4096 * 5 + 17])
def test_noalloc_dot_matches_context_dot_twice(ctx, n):
    rng = np.random.default_rng(n)
    out = fs.Vector(ctx, 1)
    for call in range(2):  # two calls in a row: the shared scratch is reused
        a = rng.standard_normal(n)
        b = rng.standard_normal(n)
        va, vb = fs.Vector(ctx, a), fs.Vector(ctx, b)
        assert _call(ctx, va, vb, n, out) == _lib.OK
        got = out.numpy()[0]
        want = va.dot(vb).get()
        # the same tolerance as the reduction tests of the vector policy
        assert abs(got - want) <= 1e-13 * np.abs(a * b).sum(), (call, got, want)


def test_noalloc_dot_limits(ctx):
    out = fs.Vector(ctx, 1)
    out.set_scalar(7.0)
    a = fs.Vector(ctx, 8)
    assert _call(ctx, a, a, 0, out) == _lib.OK
    assert out.numpy()[0] == 0.0
    # beyond the static scratch capacity: rejected before any launch
    assert _call(ctx, a, a, MAX_N + 1, out) == _lib.ERR_INVALID_ARG
    assert _fn()(None, None, 5, C.c_void_p(out.device_ptr), None) == _lib.ERR_INVALID_ARG
