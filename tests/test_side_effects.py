"""Exact side-effect mode (lsmgpu_set_exact_side_effects): the dense HJ
derivative routines leave their scratch arrays D1 / D2 / D3 as LSMLIB's do
(the last direction's undivided differences, 1e10 outside their fill range),
checked against the reference's own routines entry for entry together with
the outputs; by default the scratch arrays keep the caller's values."""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

ROUTINES = ["lsm3dhjeno1_", "lsm3dhjeno2_", "lsm3dhjeno3_", "lsm3dhjweno5_", "lsm3dupwindhjeno1_",
            "lsm3dupwindhjeno2_", "lsm3dupwindhjeno3_", "lsm3dupwindhjweno5_",
            "lsm2dhjweno5_", "lsm2dupwindhjeno3_", "lsm1dhjeno2_"]


def _scratch(sym):
    return [a[0] for a in L.ABI[sym]["args"] if a[2] and a[0] in ("d1", "d2", "d3")]


def test_side_effect_switch_without_gpu():
    h = L.lib()
    h.lsmgpu_get_exact_side_effects.restype = int
    old = h.lsmgpu_get_exact_side_effects()
    h.lsmgpu_set_exact_side_effects(1)
    assert h.lsmgpu_get_exact_side_effects() == 1
    h.lsmgpu_set_exact_side_effects(0)
    assert h.lsmgpu_get_exact_side_effects() == 0
    h.lsmgpu_set_exact_side_effects(old)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", ROUTINES)
def test_scratch_arrays_equal_reference_in_exact_mode(sym, gpu_lib):
    ref = H.reference()
    if ref is None:
        pytest.skip("reference translation not available")
    assert _scratch(sym)
    vals = H.dense_case(sym, seed=3)
    want, _ = H.run(ref, sym, vals)
    gpu_lib.lsmgpu_set_exact_side_effects(1)
    try:
        got, _ = H.run(gpu_lib, sym, vals)
        L.check()
    finally:
        gpu_lib.lsmgpu_set_exact_side_effects(0)
    for k in want:
        assert H.same(want[k], got[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("sym", ["lsm3dhjweno5_", "lsm3dupwindhjeno3_"])
def test_scratch_arrays_untouched_by_default(sym, gpu_lib):
    vals = H.dense_case(sym, seed=4)
    gpu_lib.lsmgpu_set_exact_side_effects(0)
    got, _ = H.run(gpu_lib, sym, vals)
    L.check()
    for k in _scratch(sym):
        assert H.same(vals[k], got[k]), k
