"""Fused WENO5 / TVD-RK3 steppers against the oracle's LSMLIB call sequence.

FP64: bit-for-bit equality with the per-stage composition of the oracle's
routines (derivatives -> RHS -> TVD-RK3 stage -> ghost fill), for both
modes, all boundary conditions, both sign forms of the reinitialization,
on host arrays (staged) and device arrays.
FP32: within the stated tolerance of the FP64 oracle (L-inf <= 1e-5 on
these O(1) fields).
The CPU part checks the oracle composition against the same composition of
the reference's own (translated) kernels.
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O

FB = (0, 23, 0, 19, 0, 15)
GB = (-3, 26, -3, 22, -3, 18)
DX = 2.0 / 24


def _phi(seed):
    rng = np.random.default_rng(seed)
    phi = H.sphere_phi(GB, DX, center=(-0.55, -0.6, -0.7), r=0.3)
    phi = phi * (1.0 + 0.3 * rng.random(phi.shape))   # not a distance function
    return np.asfortranarray(phi)


def _vel(seed, const=False):
    rng = np.random.default_rng(seed + 100)
    shape = H.shape_of(GB)
    if const:
        return [np.full(shape, v, order="F") for v in (1.0, -0.5, 0.25)]
    v = [np.asfortranarray(rng.uniform(-1, 1, shape)) for _ in range(3)]
    v[0][rng.random(shape) < 0.05] = 0.0
    return v


CASES = [("reinit", L.BC_PERIODIC, 0), ("reinit", L.BC_SIGNED_LINEAR, 1), ("reinit", L.BC_LINEAR, 0),
         ("advect", L.BC_PERIODIC, 0), ("advect", L.BC_COPY, 0), ("advect_const", L.BC_PERIODIC, 0)]


def _oracle_run(lib, mode, bc, use0, steps=2, seed=0):
    phi = _phi(seed)
    vel = _vel(seed, const=(mode == "advect_const")) if mode != "reinit" else None
    dt = 0.5 * DX if mode == "reinit" else DX / 3.5
    m = "reinit" if mode == "reinit" else "advect"
    return phi, vel, dt, O.tvdrk3_run(lib, m, phi, GB, FB, DX, dt, steps, bc, vel=vel, use0=use0)


@pytest.mark.parametrize("mode,bc,use0", CASES)
def test_oracle_composition_matches_reference(mode, bc, use0):
    ref = H.reference()
    if ref is None:
        pytest.skip("reference translation not available")
    _, _, _, a = _oracle_run(H.oracle(), mode, bc, use0)
    _, _, _, b = _oracle_run(ref, mode, bc, use0)
    assert H.same(a, b)


def _gpu_run(mode, bc, use0, phi, vel, dt, steps, precision="f64", device=False):
    import torch
    real = np.float64 if precision == "f64" else np.float32
    p = np.asfortranarray(phi.astype(real))
    arg = p
    if device:
        t = torch.from_numpy(np.ascontiguousarray(p.T)).cuda()
        arg = t
    if mode == "reinit":
        L.reinit_weno5_tvdrk3(arg, GB, FB, DX, dt, steps, use_phi0_for_sgn=use0, bc=bc, precision=precision)
    elif mode == "advect_const":
        L.advect_weno5_tvdrk3(arg, GB, FB, DX, dt, steps, vel_const=(1.0, -0.5, 0.25), bc=bc,
                              precision=precision)
    else:
        v = [np.asfortranarray(x.astype(real)) for x in vel]
        if device:
            v = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in v]
        L.advect_weno5_tvdrk3(arg, GB, FB, DX, dt, steps, vel=v, vel_gb=GB, bc=bc, precision=precision)
    if device:
        torch.cuda.synchronize()
        return t.cpu().numpy().T
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("mode,bc,use0", CASES)
@pytest.mark.parametrize("device", [False, True])
def test_fused_f64_bit_exact(mode, bc, use0, device, gpu_lib):
    phi, vel, dt, want = _oracle_run(H.oracle(), mode, bc, use0)
    got = _gpu_run(mode, bc, use0, phi, vel, dt, 2, "f64", device)
    assert H.same(want, got), "max |diff| %g" % np.max(np.abs(want - got))


@pytest.mark.gpu
@pytest.mark.parametrize("mode,bc,use0", CASES)
def test_fused_f32_within_tolerance(mode, bc, use0, gpu_lib):
    phi, vel, dt, want = _oracle_run(H.oracle(), mode, bc, use0)
    got = _gpu_run(mode, bc, use0, phi, vel, dt, 2, "f32")
    inner = (slice(3, -3),) * 3
    err = np.max(np.abs(want[inner] - got[inner].astype(np.float64)))
    assert err <= 1e-5, err


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_fused_advect_anisotropic_grid(precision, gpu_lib):
    """Uneven extents and spacings per axis (as the batched grids have)."""
    fb = (0, 15, 0, 17, 0, 7)
    gb = (-3, 18, -3, 20, -3, 10)
    sp = (2.0 / 16, 2.0 / 18, 2.0 / 8)
    rng = np.random.default_rng(4)
    c = [-1.0 + (np.arange(-3, m + 3) + 0.5) * 2.0 / m for m in (16, 18, 8)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    phi = np.asfortranarray(np.sqrt((X / 0.5) ** 2 + (Y / 0.3) ** 2 + (Z / 0.4) ** 2) - 1.0)
    vel = (0.7, -0.4, 0.9)
    dt = 0.5 / sum(abs(v) / s for v, s in zip(vel, sp))
    v = [np.full(phi.shape, x, order="F") for x in vel]
    want = O.tvdrk3_run(H.oracle(), "advect", phi, gb, fb, sp, dt, 2, L.BC_PERIODIC, vel=v)
    real = np.float64 if precision == "f64" else np.float32
    got = np.asfortranarray(phi.astype(real))
    L.advect_weno5_tvdrk3(got, gb, fb, sp[0], dt, 2, vel_const=vel, bc=L.BC_PERIODIC, precision=precision,
                          dy=sp[1], dz=sp[2])
    err = np.abs(got.astype(np.float64) - want)
    where = np.unravel_index(np.argmax(err), err.shape)
    if precision == "f64":
        assert H.same(want, got), (np.max(err), where)
    else:
        assert np.max(err[3:-3, 3:-3, 3:-3]) <= 1e-5, (np.max(err), where)


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [L.BC_PERIODIC, L.BC_SIGNED_LINEAR])
@pytest.mark.parametrize("vel", [(1.0, 0.5, 0.25), (-0.6, 0.8, -0.3)])
def test_fused_advect_f32_four_plane_tiles(bc, vel, gpu_lib):
    """64^3 with 13 planes: the FP32 advection stage runs 4-plane tiles there
    (they fill the waves of resident CTAs better than 8-plane ones), the last
    one ragged; constant velocities of either sign (the per-grid stencil
    side), periodic and extrapolated ghosts (the in-tile face ghosts)."""
    n, nz = 64, 13
    fb = (0, n - 1, 0, n - 1, 0, nz - 1)
    gb = (-3, n + 2, -3, n + 2, -3, nz + 2)
    sp = (2.0 / n, 2.0 / n, 2.0 / nz)
    c = [-1.0 + (np.arange(-3, m + 3) + 0.5) * 2.0 / m for m in (n, n, nz)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    phi = np.asfortranarray(np.sqrt((X - 0.1) ** 2 + (Y + 0.05) ** 2 + Z ** 2) - 0.45)
    dt = 0.5 / sum(abs(v) / s for v, s in zip(vel, sp))
    v = [np.full(phi.shape, x, order="F") for x in vel]
    steps = 3
    want = O.tvdrk3_run(H.oracle(), "advect", phi, gb, fb, sp, dt, steps, bc, vel=v)
    got = np.asfortranarray(phi.astype(np.float32))
    L.advect_weno5_tvdrk3(got, gb, fb, sp[0], dt, steps, vel_const=vel, bc=bc, precision="f32",
                          dy=sp[1], dz=sp[2])
    L.check()
    err = np.abs(got.astype(np.float64) - want)[3:-3, 3:-3, 3:-3]
    assert np.max(err) <= 1e-5, np.max(err)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_identical_calls_replay_the_cached_graph(precision, gpu_lib):
    """A second call with the same buffers, sizes and parameters replays the
    graph captured by the first (no new capture) and gives the same result."""
    import torch
    phi = _phi(7)
    dtype = torch.float64 if precision == "f64" else torch.float32
    t0 = torch.from_numpy(np.ascontiguousarray(phi.T)).cuda().to(dtype)
    a, b = t0.clone(), t0.clone()
    L.reinit_weno5_tvdrk3(a, GB, FB, DX, 0.5 * DX, 3, use_phi0_for_sgn=1, bc=L.BC_SIGNED_LINEAR,
                          precision=precision)
    torch.cuda.synchronize()
    before = L.graph_capture_count()
    L.reinit_weno5_tvdrk3(b, GB, FB, DX, 0.5 * DX, 3, use_phi0_for_sgn=1, bc=L.BC_SIGNED_LINEAR,
                          precision=precision)
    torch.cuda.synchronize()
    L.check()
    assert L.graph_capture_count() == before
    assert torch.equal(a, b)
