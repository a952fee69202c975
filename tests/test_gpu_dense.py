"""GPU parity: every dense drop-in entry point against the C oracle.

The FP64 kernels keep LSMLIB's operation order and are compiled without FMA
contraction, so the bar is bit-for-bit equality (+0 == -0), on host arrays
(staged through the device) and on device arrays (used in place).
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

from tests.test_oracle_pin import DENSE
from tests.test_geometry import NOT_BIT_EXACT

# sums and the ** 1.5 curvature have their own bars in test_geometry.py
BIT_EXACT = [s for s in DENSE if s not in NOT_BIT_EXACT]


@pytest.mark.gpu
@pytest.mark.parametrize("sym", BIT_EXACT)
@pytest.mark.parametrize("seed", [0, 1])
def test_dense_host_arrays_bit_exact(sym, seed, gpu_lib):
    extra = {"use_phi0_for_sgn": seed} if "reinit" in sym else {}
    vals = H.dense_case(sym, seed=seed, scalars=extra)
    a_or, s_or = H.run(H.oracle(), sym, vals)
    a_gpu, s_gpu = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    for name in H.written_names(sym):
        if name in ("d1", "d2", "d3"):
            continue
        if name in a_or:
            assert H.same(a_or[name], a_gpu[name]), "%s: %s differs, max |diff| %g" % (
                sym, name, np.nanmax(np.abs(a_or[name] - a_gpu[name])))
        else:
            assert H.same(s_or[name], s_gpu[name]), "%s: %s %r vs %r" % (sym, name, s_or[name], s_gpu[name])


@pytest.mark.gpu
@pytest.mark.parametrize("sym", ["lsm3dhjweno5_", "lsm3dupwindhjweno5_", "lsm3dtvdrk3stage3_",
                                 "lsm3dcomputestableadvectiondt_", "lsm3dcomputemeancurvatureorder2_"])
def test_dense_device_arrays_bit_exact(sym, gpu_lib):
    import torch
    vals = H.dense_case(sym, seed=3)
    a_or, s_or = H.run(H.oracle(), sym, vals)
    dev = {}
    for k, v in vals.items():
        if isinstance(v, np.ndarray):
            # a Fortran-ordered array's memory is the C-ordered transpose
            dev[k] = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
        else:
            dev[k] = v
    sc = L.invoke(gpu_lib, sym, dev)
    torch.cuda.synchronize()
    L.check(gpu_lib)
    for name in H.written_names(sym):
        if name in ("d1", "d2", "d3"):
            continue
        if name in a_or:
            got = dev[name].cpu().numpy().T
            assert H.same(a_or[name], got), "%s: %s differs" % (sym, name)
        else:
            assert H.same(s_or[name], sc[name])


@pytest.mark.gpu
def test_bounds_error_is_reported_and_nothing_written(gpu_lib):
    sym = "lsm3dhjweno5_"
    # fill box reaches the ghost box edge: WENO5 needs 3 more cells
    vals = H.dense_case(sym, seed=0, fb=(-2, 9, 0, 7, 0, 5))
    before = {k: v.copy() for k, v in vals.items() if isinstance(v, np.ndarray)}
    L.invoke(gpu_lib, sym, vals)
    code, msg = L.last_error(gpu_lib)
    assert code == 1 and "ghost box" in msg
    for k, v in before.items():
        assert H.same(v, vals[k])
    # a valid call clears the status
    vals = H.dense_case(sym, seed=0)
    L.invoke(gpu_lib, sym, vals)
    assert L.last_error(gpu_lib)[0] == 0
