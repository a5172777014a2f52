"""The allocation-free dot product (gbfem_dot_noalloc) through the C-ABI.

Callers that cannot let the library allocate device memory -- a host whose
memory pool already owns all of HBM, or a latency-critical loop that cannot
take cudaMalloc's implicit synchronisation -- use gbfem_dot_noalloc, which
keeps its partial sums in a fixed device array instead of allocated scratch.
Its results must agree with gbfem_dot (the allocating entry point).  This
file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 65536 * 8192


def _noalloc(gb, x, y):
    L = gb.lib()
    L.gbfem_dot_noalloc.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    r = C.c_double()
    gb.check(L.gbfem_dot_noalloc(x.precision, x.n, x.ptr, y.ptr, C.byref(r), None))
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
        assert abs(first - ref) <= 1e-12 * max(1.0, abs(ref))


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(gb):
    x = gb.DeviceArray.from_numpy(np.ones(4))
    L = gb.lib()
    L.gbfem_dot_noalloc.argtypes = [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    r = C.c_double()
    rc = L.gbfem_dot_noalloc(0, MAX_N + 1, x.ptr, x.ptr, C.byref(r), None)
    assert rc != 0
    assert b"exceeds the maximum" in L.gbfem_last_error()
