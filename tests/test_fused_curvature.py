"""lsmgpu_mean_curvature_o2_{f64,f32}: the fused central gradient, |grad phi|
and second-order mean curvature against the oracle's LSMLIB call sequence
(lsm3dCentralGradOrder2 -> lsm3dGradientMagnitude ->
lsm3dComputeMeanCurvatureOrder2).

FP64: bit-for-bit on the fill box, host (staged) and device arrays.  Host
outputs are written back over the fill box only, so every other cell of
kappa and |grad phi| keeps the caller's value; the test fills them with a
pattern and checks it survives.  FP32: within 1e-4 relative to the largest
|kappa| (curvature divides by |grad phi|^3).
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

GB = (-3, 21, -2, 17, -4, 14)
FB = (0, 18, 0, 15, -2, 12)
DX, DY, DZ = 0.1, 0.11, 0.09


def _phi(seed):
    rng = np.random.default_rng(seed)
    phi = H.sphere_phi(GB, DX, center=(0.9, 0.8, 0.5), r=0.45, lo=0.0)
    return np.asfortranarray(phi * (1.0 + 0.2 * rng.random(phi.shape)))


def oracle_chain(phi):
    o = H.oracle()
    sc = {"dx": DX, "dy": DY, "dz": DZ}
    v, _ = H.make_call("lsm3dcentralgradorder2_", GB, FB, arrays={"phi": phi}, scalars=sc, fill=0.0)
    g, _ = H.run(o, "lsm3dcentralgradorder2_", v)
    v, _ = H.make_call("lsm3dgradientmagnitude_", GB, FB,
                       arrays={"phi_x": g["phi_x"], "phi_y": g["phi_y"], "phi_z": g["phi_z"]}, scalars=sc,
                       fill=0.0)
    m, _ = H.run(o, "lsm3dgradientmagnitude_", v)
    v, _ = H.make_call("lsm3dcomputemeancurvatureorder2_", GB, FB,
                       arrays={"phi": phi, "phi_x": g["phi_x"], "phi_y": g["phi_y"], "phi_z": g["phi_z"],
                               "grad_phi_mag": m["grad_phi_mag"]}, scalars=sc, fill=0.0)
    k, _ = H.run(o, "lsm3dcomputemeancurvatureorder2_", v)
    return k["kappa"], m["grad_phi_mag"]


FBS = tuple(slice(FB[2 * d] - GB[2 * d], FB[2 * d + 1] - GB[2 * d] + 1) for d in range(3))


def test_gradient_magnitude_output_name():
    # the chain above reads the |grad phi| output by this name
    assert "grad_phi_mag" in H.written_names("lsm3dgradientmagnitude_")


@pytest.mark.gpu
@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("seed", [0, 1])
def test_fused_curvature_f64_bit_exact(device, seed, gpu_lib):
    import torch
    phi = _phi(seed)
    want_k, want_m = oracle_chain(phi)
    pattern = np.asfortranarray(np.random.default_rng(seed + 9).standard_normal(H.shape_of(GB)))
    kap, mag = pattern.copy(order="F"), (pattern * 2.0).copy(order="F")
    if device:
        t = [torch.from_numpy(np.ascontiguousarray(a.T)).cuda() for a in (kap, phi, mag)]
        L.mean_curvature_o2(t[0], GB, t[1], GB, FB, DX, grad_phi_mag=t[2], precision="f64", dy=DY, dz=DZ)
        torch.cuda.synchronize()
        kap, mag = t[0].cpu().numpy().T, t[2].cpu().numpy().T
    else:
        L.mean_curvature_o2(kap, GB, phi, GB, FB, DX, grad_phi_mag=mag, precision="f64", dy=DY, dz=DZ)
    assert H.same(kap[FBS], want_k[FBS])
    assert H.same(mag[FBS], want_m[FBS])
    outside = np.ones(kap.shape, bool)
    outside[FBS] = False
    assert H.same(kap[outside], pattern[outside])
    assert H.same(mag[outside], 2.0 * pattern[outside])


@pytest.mark.gpu
def test_fused_curvature_f32_within_tolerance(gpu_lib):
    phi = _phi(3)
    want_k, _ = oracle_chain(phi)
    kap = np.zeros(H.shape_of(GB), np.float32, order="F")
    L.mean_curvature_o2(kap, GB, np.asfortranarray(phi.astype(np.float32)), GB, FB, DX, precision="f32",
                        dy=DY, dz=DZ)
    err = np.max(np.abs(kap[FBS].astype(np.float64) - want_k[FBS]))
    assert err <= 1e-4 * np.max(np.abs(want_k[FBS])), err


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_fused_curvature_pinned_host_pipelined(precision, gpu_lib):
    """Pinned host phi and kappa without |grad phi|: the slab-pipelined
    transfers (37 fill-box planes cut into 8 uneven slabs).  Equal bit for bit
    to the call on device arrays; kappa outside the fill box keeps the
    caller's values."""
    import torch
    gb = (-3, 21, -2, 17, -4, 40)
    fb = (0, 18, 0, 15, -2, 34)
    real = np.float64 if precision == "f64" else np.float32
    phi = H.sphere_phi(gb, DX, center=(0.9, 0.8, 1.5), r=0.8, lo=0.0)
    phi = np.asfortranarray((phi * (1.0 + 0.2 * np.random.default_rng(5).random(phi.shape))).astype(real))
    pattern = np.asfortranarray(np.random.default_rng(6).standard_normal(phi.shape).astype(real))
    host = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).pin_memory()
    hp, hk = host(phi), host(pattern)
    L.mean_curvature_o2(hk, gb, hp, gb, fb, DX, precision=precision, dy=DY, dz=DZ)
    dp, dk = hp.cuda(), host(pattern).cuda()
    L.mean_curvature_o2(dk, gb, dp, gb, fb, DX, precision=precision, dy=DY, dz=DZ)
    torch.cuda.synchronize()
    got, want = hk.numpy().T, dk.cpu().numpy().T
    assert H.same(got, want)
    fbs = tuple(slice(fb[2 * d] - gb[2 * d], fb[2 * d + 1] - gb[2 * d] + 1) for d in range(3))
    outside = np.ones(got.shape, bool)
    outside[fbs] = False
    assert H.same(got[outside], pattern[outside])
