"""LSMLIB's 2D routines without a 3D counterpart (csrc/plane2d.cu): the
9-point and signed-distance mean curvatures, the central divergence (dense
and list forms) and the second-order delta function, against the
reference's own routines (translated Fortran, oracle/_ref) on seeded inputs,
bit for bit, on host arrays.  The list cases take every fill-box
cell, split into four levels, with a few boundary marks (tests/test_lifted.py)."""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import test_lifted as TL

PLANE = sorted(s for s, v in L.ABI.items() if v.get("plane2d"))
TL.DIMS.update({s: 2 for s in PLANE})


def test_plane_routines_are_declared():
    assert len(PLANE) == 7
    h = L.lib()
    for s in PLANE:
        assert hasattr(h, s), s


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available")
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("sym", PLANE)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_plane2d_gpu_matches_reference(sym, seed, ref, gpu_lib):
    vals = TL.case(sym, seed)
    if "phi" in vals and "sgndist" in sym:
        # near-signed-distance input: |1 - phi Laplacian| stays away from 0
        vals["phi"] = np.asfortranarray(0.05 * vals["phi"])
    a1, s1 = H.run(ref, sym, vals)
    a2, s2 = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    TL.compare(sym, a1, s1, a2, s2)


@pytest.mark.gpu
def test_delta_order2_has_interface_cells(ref):
    """The delta-function case crosses phi = 0 (both branches of each side run)."""
    vals = TL.case("lsm2ddeltafunctionorder2_", 0)
    a, _ = H.run(ref, "lsm2ddeltafunctionorder2_", vals)
    fb = (slice(3, 13), slice(3, 11))
    assert np.count_nonzero(a["delta"][fb]) > 10
