"""The bounds-check build (liblsmgpu_bc.so, LSMGPU_BOUNDS_CHECK): every
dense drop-in entry point, and the list (_LOCAL) routines of the narrow-band
tests, run through it on the same seeded inputs give results identical to
the regular library's, with no array access outside an array's box recorded.
This is the out-of-bounds check that stands in for a memory checker."""
import ctypes

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests.test_oracle_pin import DENSE


@pytest.fixture(scope="module")
def bc_lib(gpu_lib):
    from lsmlib_gb300 import build as B
    path = B.build(bounds_check=True)
    h = L.lib(path)
    h.lsmgpu_bounds_check_read.restype = ctypes.c_int
    return h


def _oob(h):
    n = ctypes.c_longlong(-1)
    first = (ctypes.c_int * 3)()
    assert h.lsmgpu_bounds_check_read(ctypes.byref(n), first) == 0, L.last_error(h)
    return n.value, tuple(first)


def test_regular_library_reports_no_bounds_check():
    h = L.lib()
    h.lsmgpu_bounds_check_read.restype = ctypes.c_int
    n = ctypes.c_longlong(0)
    assert h.lsmgpu_bounds_check_read(ctypes.byref(n), None) == 3  # LSMGPU_ERR_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("sym", DENSE)
def test_dense_entry_points_stay_in_bounds(sym, bc_lib, gpu_lib):
    extra = {"use_phi0_for_sgn": 1} if "reinit" in sym else {}
    vals = H.dense_case(sym, seed=7, scalars=extra)
    a, sa = H.run(gpu_lib, sym, vals)
    _oob(bc_lib)
    b, sb = H.run(bc_lib, sym, vals)
    L.check(bc_lib)
    assert _oob(bc_lib) == (0, (0, 0, 0)), sym
    for k in a:
        assert H.same(a[k], b[k]), (sym, k)
    for k in sa:
        assert sa[k] == sb[k] or (sa[k] != sa[k] and sb[k] != sb[k]), (sym, k)
