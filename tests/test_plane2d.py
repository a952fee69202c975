"""LSMLIB's 2D routines without a 3D counterpart (csrc/plane2d.cu): the
9-point and signed-distance mean curvatures, the central divergence (dense
and list forms), the second-order delta function, the precomputed-delta
surface integrals and the list mean absolute difference, against the
reference's own routines (translated Fortran, oracle/_ref) on seeded inputs,
on host arrays: bit for bit, and sums within (n + 16) 2^-53 sum|term| of the
reference's serial sum.  The list cases take every fill-box cell, split into
four levels, with a few boundary marks (tests/test_lifted.py).

lsm2dSurfaceIntegralPrecomputedDelta cannot be called as declared (its
Fortran argument list leaves out the index box it loops over); it is checked
against the reference's control-volume form with every control volume
positive, which adds the same terms in the same order."""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import test_lifted as TL

PLANE = sorted(s for s, v in L.ABI.items() if v.get("plane2d"))
TL.DIMS.update({s: 2 for s in PLANE})


SUMS2 = {"lsm2dsurfaceintegralprecomputeddelta_", "lsm2dsurfaceintegralprecomputeddeltacontrolvolume_",
         "lsm2daveabsdifflocal_"}
U = 2.0 ** -53


def test_plane_routines_are_declared():
    assert len(PLANE) == 10
    h = L.lib()
    for s in PLANE:
        assert hasattr(h, s), s


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available")
    return r


def sum_scale(ref, sym, vals):
    """sum |term| of the reference's serial sum"""
    v = dict(vals)
    for k in ("f", "delta_phi", "grad_phi_mag"):
        if k in v:
            v[k] = np.abs(v[k]).copy(order="F")
    out = [a[0] for a in L.ABI[sym]["args"] if not a[2] and a[3]][0]
    return abs(H.run(ref, sym, v)[1][out])


@pytest.mark.gpu
@pytest.mark.parametrize("sym", sorted(SUMS2 - {"lsm2dsurfaceintegralprecomputeddelta_"}))
@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("sgn", [1, -1])
def test_plane2d_sums_match_reference(sym, seed, sgn, ref, gpu_lib):
    vals = TL.case(sym, seed)
    if "control_vol_sgn" in vals:
        vals["control_vol_sgn"] = sgn
    s1 = H.run(ref, sym, vals)[1]
    s2 = H.run(gpu_lib, sym, vals)[1]
    L.check(gpu_lib)
    out = [a[0] for a in L.ABI[sym]["args"] if not a[2] and a[3]][0]
    n = int(np.prod(TL.shape(2)))
    assert abs(s1[out] - s2[out]) <= (n + 16) * U * sum_scale(ref, sym, vals), (s1[out], s2[out])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_delta_integral_equals_control_volume_form_with_positive_volumes(seed, ref, gpu_lib):
    sym, cv_sym = "lsm2dsurfaceintegralprecomputeddelta_", "lsm2dsurfaceintegralprecomputeddeltacontrolvolume_"
    vals = TL.case(sym, seed)
    cv_vals = TL.case(cv_sym, seed)
    for k in ("f", "delta_phi", "grad_phi_mag", "dx", "dy"):
        cv_vals[k] = vals[k]
    cv_vals["control_vol"] = np.ones_like(vals["f"], order="F")
    cv_vals["control_vol_sgn"] = 1
    want = H.run(ref, cv_sym, cv_vals)[1]["int_f"]
    got = H.run(gpu_lib, sym, vals)[1]["int_f"]
    L.check(gpu_lib)
    n = int(np.prod(TL.shape(2)))
    assert abs(want - got) <= (n + 16) * U * sum_scale(ref, cv_sym, cv_vals), (want, got)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", sorted(set(PLANE) - SUMS2))
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
