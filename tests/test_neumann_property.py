"""LSMLIB's boundary-condition property test, ported
(tests/boundary_conditions/test_neumann_bc_3d.cc: ENO1 :134, ENO2 :367,
ENO3 :609, WENO5 :860).

Fixture (test_neumann_bc_3d.cc:47-97): a 25 x 20 x 30 box with 3 ghost
cells, dx = 1/25, dy = 1/20, dz = 1/30, and
  phi = (x-0.25)^2 + 4 (y-0.35)^2 + 0.25 (z-0.45)^2 - 0.25
at cell centres, where the fixture takes z from the j index
(z = (j+0.5) dz), as the reference does.  After the homogeneous Neumann
ghost fill on all six faces, the HJ derivative normal to each face, on the
one-sided stencil pointing out of the box (x-lower: phi_x_minus, x-upper:
phi_x_plus, ...), is zero within 1e-6 at every face cell.

Runs on the oracle (CPU), the translated reference (CPU, when available)
and the GPU drop-in kernels (gpu).
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

DIMS = (25, 20, 30)
FB = (0, 24, 0, 19, 0, 29)
GB = (-3, 27, -3, 22, -3, 32)
DX = (1.0 / 25, 1.0 / 20, 1.0 / 30)

SCHEMES = {
    "eno1": ("lsm3dhomogeneousneumanneno1_", "lsm3dhjeno1_"),
    "eno2": ("lsm3dhomogeneousneumanneno2_", "lsm3dhjeno2_"),
    "eno3": ("lsm3dhomogeneousneumanneno3_", "lsm3dhjeno3_"),
    "weno5": ("lsm3dhomogeneousneumannweno5_", "lsm3dhjweno5_"),
}


def fixture_phi():
    phi = np.zeros(H.shape_of(GB), order="F")
    i = np.arange(DIMS[0])[:, None, None]
    j = np.arange(DIMS[1])[None, :, None]
    x = (i + 0.5) * DX[0]
    y = (j + 0.5) * DX[1]
    z = (j + 0.5) * DX[2]   # test_neumann_bc_3d.cc:88 takes z from j
    val = (x - 0.25) ** 2 + 4 * (y - 0.35) ** 2 + 0.25 * (z - 0.45) ** 2 - 0.25
    phi[3:3 + DIMS[0], 3:3 + DIMS[1], 3:3 + DIMS[2]] = np.broadcast_to(val, DIMS)
    return phi


def boundary_derivatives(handle, scheme):
    bc, hj = SCHEMES[scheme]
    phi = fixture_phi()
    for face in range(6):   # the fill writes phi in place, faces 0..5 in turn
        vals, _ = H.make_call(bc, GB, FB, arrays={"phi": phi}, scalars={"bdry_location_idx": face})
        L.invoke(handle, bc, vals)
    vals, arrs = H.make_call(hj, GB, FB, arrays={"phi": phi},
                             scalars={"dx": DX[0], "dy": DX[1], "dz": DX[2]}, fill=0.0)
    L.invoke(handle, hj, vals)
    inner = lambda a: a[3:3 + DIMS[0], 3:3 + DIMS[1], 3:3 + DIMS[2]]
    px, py, pz = (inner(arrs["phi_%s_plus" % a]) for a in "xyz")
    mx, my, mz = (inner(arrs["phi_%s_minus" % a]) for a in "xyz")
    return [mx[0], px[-1], my[:, 0], py[:, -1], mz[:, :, 0], pz[:, :, -1]]


def _check(handle, scheme):
    for face, vals in enumerate(boundary_derivatives(handle, scheme)):
        assert np.max(np.abs(vals)) <= 1e-6, (scheme, face, np.max(np.abs(vals)))


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_neumann_property_oracle(scheme):
    _check(H.oracle(), scheme)


@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_neumann_property_reference(scheme):
    ref = H.reference()
    if ref is None:
        pytest.skip("reference translation not available")
    _check(ref, scheme)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_neumann_property_gpu(scheme, gpu_lib):
    _check(gpu_lib, scheme)
    # and the GPU values equal the oracle's bit for bit
    for a, b in zip(boundary_derivatives(gpu_lib, scheme), boundary_derivatives(H.oracle(), scheme)):
        assert H.same(a, b)
