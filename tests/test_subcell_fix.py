"""Subcell-fix reinitialization chain on a level set with an interface:
lsm3dComputeDistanceForSubcellFix -> lsm3dHJENO1 ->
lsm3dComputeReinitializationEqnRHSSubcellFixOrder1, so both branches of the
RHS (Godunov away from the interface, the distance form next to it) run.
The C oracle against the reference's own (translated) kernels on the CPU,
the GPU library against the oracle, bit for bit.  Host and device arrays.
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

GB = (-3, 17, -2, 15, -3, 12)
FB = (0, 14, 0, 13, 0, 9)
SC = {"dx": 0.1, "dy": 0.12, "dz": 0.09}


def _phi0(seed):
    rng = np.random.default_rng(seed)
    phi0 = H.sphere_phi(GB, 0.1, center=(0.7, 0.8, 0.45), r=0.5, lo=0.0)
    phi0 = phi0 * (1.0 + 0.3 * rng.random(phi0.shape))
    phi0[rng.random(phi0.shape) < 0.02] = 0.0     # exact zeros: sgn(phi0) = 0 cells
    return np.asfortranarray(phi0)


def chain(lib, seed):
    phi0 = _phi0(seed)
    rng = np.random.default_rng(seed + 50)
    phi = np.asfortranarray(phi0 + 0.05 * rng.standard_normal(phi0.shape))
    v, _ = H.make_call("lsm3dcomputedistanceforsubcellfix_", GB, FB, arrays={"phi0": phi0}, scalars=SC,
                       fill=7.0)
    d, _ = H.run(lib, "lsm3dcomputedistanceforsubcellfix_", v)
    v, _ = H.make_call("lsm3dhjeno1_", GB, FB, arrays={"phi": phi}, scalars=SC, fill=0.0)
    g, _ = H.run(lib, "lsm3dhjeno1_", v)
    arrays = {"phi": phi, "phi0": phi0, "distance0": d["distance0"]}
    for n in ("phi_x_plus", "phi_y_plus", "phi_z_plus", "phi_x_minus", "phi_y_minus", "phi_z_minus"):
        arrays[n] = g[n]
    v, _ = H.make_call("lsm3dcomputereinitializationeqnrhssubcellfixorder1_", GB, FB, arrays=arrays,
                       scalars=SC, fill=-3.0)
    r, _ = H.run(lib, "lsm3dcomputereinitializationeqnrhssubcellfixorder1_", v)
    return d["distance0"], r["reinit_rhs"]


def test_chain_has_both_branches():
    d, _ = chain(H.oracle(), 0)
    fb = tuple(slice(FB[2 * a] - GB[2 * a], FB[2 * a + 1] - GB[2 * a] + 1) for a in range(3))
    flag = -1000.0 * 0.12
    far = np.sum(d[fb] == flag)
    assert 0 < far < d[fb].size


@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_chain_matches_reference(seed):
    ref = H.reference()
    if ref is None:
        pytest.skip("reference translation not available")
    d1, r1 = chain(H.oracle(), seed)
    d2, r2 = chain(ref, seed)
    assert H.same(d1, d2)
    assert H.same(r1, r2)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_chain_bit_exact(seed, gpu_lib):
    d1, r1 = chain(H.oracle(), seed)
    d2, r2 = chain(gpu_lib, seed)
    L.check(gpu_lib)
    assert H.same(d1, d2)
    assert H.same(r1, r2)
