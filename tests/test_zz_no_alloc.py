"""The allocation-free dot product (gbfem_dot_noalloc) through the C-ABI.

Callers that cannot let the library allocate device memory -- a host whose
memory pool already owns all of HBM, or a latency-critical loop that cannot
take cudaMalloc's implicit synchronisation -- use gbfem_dot_noalloc, which
keeps its partial sums in a fixed device array instead of allocated scratch.
Up to 1024 chunks of 8192 it partitions the vector as gbfem_dot does and must
return bitwise the same value; past that (up to its 65536-partial limit) it is
checked against a float64 numpy dot and against an exactly known sum.  This
file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 65536 * 8192


def _fn(gb):
    L = gb.lib()
    L.gbfem_dot_noalloc.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    return L.gbfem_dot_noalloc


def _noalloc(gb, x, y):
    r = C.c_double()
    gb.check(_fn(gb)(x.precision, x.n, x.ptr, y.ptr, C.byref(r), None))
    return r.value


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_dot_matches_allocating_dot_twice(gb, precision):
    dt = np.float64 if precision == 0 else np.float32
    rng = np.random.default_rng(42 + precision)
    for n in (3_000_001, 1_000):  # second size leaves stale partials behind the first
        x = rng.uniform(-1, 1, n).astype(dt)
        y = rng.uniform(-1, 1, n).astype(dt)
        dx, dy = gb.DeviceArray.from_numpy(x), gb.DeviceArray.from_numpy(y)
        ref = gb.dot(dx, dy)
        first = _noalloc(gb, dx, dy)
        second = _noalloc(gb, dx, dy)
        assert first == second
        assert first == ref  # same partition as gbfem_dot below 1024 chunks: bitwise equal


def test_noalloc_dot_beyond_1024_partials(gb):
    """n = 1024 * 8192 + 1: 1025 partials, which pass 2 loops over in its
    single CTA (gbfem_dot would use 1024 longer chunks here)."""
    n = 1024 * 8192 + 1
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    dx, dy = gb.DeviceArray.from_numpy(x), gb.DeviceArray.from_numpy(y)
    got = _noalloc(gb, dx, dy)
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    ref = float(np.dot(x64, y64))
    scale = float(np.dot(np.abs(x64), np.abs(y64)))
    assert abs(got - ref) <= 1e-13 * scale
    assert abs(got - gb.dot(dx, dy)) <= 1e-13 * scale
    assert _noalloc(gb, dx, dy) == got


def test_noalloc_dot_at_its_maximum_size(gb):
    """n = 65536 * 8192 exactly, the largest accepted size: x_i = (i mod 7) - 3
    in FP32, so x.x is an integer the FP64 sums hold exactly, whatever the
    order -- a missed or doubly counted chunk changes it."""
    n = MAX_N
    x = np.tile(np.arange(7, dtype=np.float32) - 3.0, n // 7 + 1)[:n]
    full, rest = divmod(n, 7)
    exact = float(full * 28 + sum((k - 3) ** 2 for k in range(rest)))
    dx = gb.DeviceArray.from_numpy(x)
    del x
    assert _noalloc(gb, dx, dx) == exact
    assert _noalloc(gb, dx, dx) == exact


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(gb):
    x = gb.DeviceArray.from_numpy(np.ones(4))
    r = C.c_double()
    rc = _fn(gb)(0, MAX_N + 1, x.ptr, x.ptr, C.byref(r), None)
    assert rc != 0
    assert b"exceeds the maximum" in gb.lib().gbfem_last_error()


def test_noalloc_dot_host_side_argument_checks(gb):
    """The early returns before any device work: n = 0 gives 0.0, a null
    result pointer and an unknown precision are rejected."""
    f = _fn(gb)
    x = gb.DeviceArray.from_numpy(np.ones(4))
    r = C.c_double(123.0)
    assert f(0, 0, x.ptr, x.ptr, C.byref(r), None) == 0
    assert r.value == 0.0
    assert f(7, 4, x.ptr, x.ptr, C.byref(r), None) != 0
    assert b"precision" in gb.lib().gbfem_last_error()
    assert f(0, 4, x.ptr, x.ptr, None, None) != 0
    assert b"null" in gb.lib().gbfem_last_error()
