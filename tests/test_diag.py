"""Diagnostics: the non-finite scan (GPU form of LSMLIB's EXAMINE_ARRAY)
against numpy, and the bounded-wait self-test — a kernel waits on a barrier
nothing releases, gives up, reports LSMGPU_ERR_TIMEOUT, and the context stays
usable for the next call.  No GPU fault is raised."""
import ctypes

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

GB = (-3, 20, -2, 14, -1, 9)
BOX = (0, 17, 0, 12, 0, 8)


def _box(b):
    return (ctypes.c_int * 6)(*b)


def _scan(lib, arr, precision):
    fn = getattr(lib, "lsmgpu_count_nonfinite_" + precision)
    fn.restype = ctypes.c_int
    cnt = ctypes.c_longlong(-1)
    first = (ctypes.c_int * 3)()
    rc = fn(ctypes.c_void_p(arr.ctypes.data), _box(GB), _box(BOX), ctypes.byref(cnt), first)
    return rc, cnt.value, tuple(first)


def _expected(arr):
    sub = arr[BOX[0] - GB[0]:BOX[1] - GB[0] + 1, BOX[2] - GB[2]:BOX[3] - GB[2] + 1,
              BOX[4] - GB[4]:BOX[5] - GB[4] + 1]
    bad = ~np.isfinite(sub)
    n = int(bad.sum())
    if n == 0:
        return 0, (BOX[0] - 1, BOX[2] - 1, BOX[4] - 1)
    flat = np.flatnonzero(bad.ravel(order="F"))[0]
    i, j, k = np.unravel_index(flat, sub.shape, order="F")
    return n, (BOX[0] + int(i), BOX[2] + int(j), BOX[4] + int(k))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_nonfinite_scan_matches_numpy(precision, gpu_lib):
    dt = np.float64 if precision == "f64" else np.float32
    rng = np.random.default_rng(4)
    arr = np.asfortranarray(rng.standard_normal(H.shape_of(GB)).astype(dt))
    rc, n, first = _scan(gpu_lib, arr, precision)
    assert rc == 0 and (n, first) == _expected(arr)
    # plant NaN and inf (array indices; cells (2, 5, 2) and (8, 1, 5) lie in
    # the box, the other two in the ghost cells outside it)
    for idx, v in (((5, 7, 3), np.nan), ((2, 9, 8), np.inf), ((11, 3, 6), -np.inf), ((0, 0, 0), np.nan)):
        arr[idx] = v
    rc, n, first = _scan(gpu_lib, arr, precision)
    assert rc == 0 and (n, first) == _expected(arr) == (2, (2, 5, 2))


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_the_context_survives(gpu_lib):
    fn = gpu_lib.lsmgpu_selftest_bounded_wait
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_uint]
    assert fn(1000) == L_TIMEOUT
    code, msg = L.last_error(gpu_lib)
    assert code == L_TIMEOUT and "gave up" in msg
    assert fn(2 ** 21) == 4  # budget above the maximum: refused, nothing launched
    # the next call works
    vals = H.dense_case("lsm3dhjweno5_", seed=2)
    a, _ = H.run(H.oracle(), "lsm3dhjweno5_", vals)
    b, _ = H.run(gpu_lib, "lsm3dhjweno5_", vals)
    L.check(gpu_lib)
    assert H.same(a["phi_x_plus"], b["phi_x_plus"])


L_TIMEOUT = 5
