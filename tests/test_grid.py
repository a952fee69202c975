"""Grid construction (createGridSetDx / DxDyDz / GridDims, copyGrid,
setIndexSpaceLimits*) against LSMLIB's own src/utils/lsm_grid.c compiled by
oracle/build.py: every member of the structure equal, for each accuracy
level, 2D and 3D, and a dimension count LSMLIB replaces by 2."""
import ctypes
import os

import pytest

import lsmlib_gb300 as L
from tests import harness as H

REFIO = os.path.join(H.ROOT, "oracle", "_ref", "liblsmrefio.so")


class Grid(ctypes.Structure):
    _fields_ = [("num_dims", ctypes.c_int), ("x_lo", ctypes.c_double * 3), ("x_hi", ctypes.c_double * 3),
                ("x_lo_ghostbox", ctypes.c_double * 3), ("x_hi_ghostbox", ctypes.c_double * 3),
                ("grid_dims", ctypes.c_int * 3), ("grid_dims_ghostbox", ctypes.c_int * 3),
                ("dx", ctypes.c_double * 3), ("num_gridpts", ctypes.c_int)] + \
               [(n, ctypes.c_int) for n in (
                   "ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb",
                   "ilo_fb", "ihi_fb", "jlo_fb", "jhi_fb", "klo_fb", "khi_fb",
                   "ilo_D1_fb", "ihi_D1_fb", "jlo_D1_fb", "jhi_D1_fb", "klo_D1_fb", "khi_D1_fb",
                   "ilo_D2_fb", "ihi_D2_fb", "jlo_D2_fb", "jhi_D2_fb", "klo_D2_fb", "khi_D2_fb",
                   "ilo_D3_fb", "ihi_D3_fb", "jlo_D3_fb", "jhi_D3_fb", "klo_D3_fb", "khi_D3_fb",
                   "num_nb_levels")] + \
               [(n, ctypes.c_ubyte) for n in ("mark_gb", "mark_D1", "mark_D2", "mark_D3", "mark_fb")] + \
               [("beta", ctypes.c_double), ("gamma", ctypes.c_double)]


def _fns(lib):
    P = ctypes.POINTER(Grid)
    D3 = ctypes.c_double * 3
    lib.createGridSetDx.restype = P
    lib.createGridSetDx.argtypes = [ctypes.c_int, ctypes.c_double, D3, D3, ctypes.c_int]
    lib.createGridSetDxDyDz.restype = P
    lib.createGridSetDxDyDz.argtypes = [ctypes.c_int] + [ctypes.c_double] * 3 + [D3, D3, ctypes.c_int]
    lib.createGridSetGridDims.restype = P
    lib.createGridSetGridDims.argtypes = [ctypes.c_int, ctypes.c_int * 3, D3, D3, ctypes.c_int]
    lib.copyGrid.restype = P
    lib.copyGrid.argtypes = [P]
    lib.destroyGrid.argtypes = [P]
    return lib


def _fields(g):
    out = {}
    for name, _ in Grid._fields_:
        v = getattr(g, name)
        out[name] = tuple(v) if hasattr(v, "__len__") else v
    return out


def _reference():
    if not os.path.exists(REFIO):
        pytest.skip("LSMLIB's lsm_grid.c not built here (reference tree absent)")
    return _fns(ctypes.CDLL(REFIO, mode=ctypes.RTLD_LOCAL))


CASES = [(3, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)), (3, (0.0, -0.5, 0.25), (1.3, 0.7, 2.0)),
         (2, (-1.0, 0.0, 0.0), (1.0, 2.5, 0.0)), (4, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))]


@pytest.mark.parametrize("accuracy", [0, 1, 2, 3])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_grid_construction_matches_lsmlib(accuracy, case):
    ref, ours = _reference(), _fns(L.lib())
    nd, lo, hi = CASES[case]
    D3 = ctypes.c_double * 3
    calls = [("createGridSetDx", (nd, 0.037, D3(*lo), D3(*hi), accuracy)),
             ("createGridSetDxDyDz", (nd, 0.05, 0.031, 0.07, D3(*lo), D3(*hi), accuracy)),
             ("createGridSetGridDims", (nd, (ctypes.c_int * 3)(40, 33, 17), D3(*lo), D3(*hi), accuracy))]
    for name, args in calls:
        a = getattr(ref, name)(*args)
        b = getattr(ours, name)(*args)
        assert _fields(a.contents) == _fields(b.contents), name
        c = ours.copyGrid(b)
        assert _fields(c.contents) == _fields(b.contents)
        ours.destroyGrid(c)
        ours.destroyGrid(b)
        ref.destroyGrid(a)
