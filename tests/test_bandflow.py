"""Narrow-band curvature flow (Vn = 1 - 0.1 kappa, HJ WENO5 on the band,
TVD-RK3, band rebuilt every few steps) against the oracle's LSMLIB *_LOCAL
call sequence (tests/oracle_runs.band_run).

FP64: bit-for-bit phi, per-step dt and level-0 band sizes.  FP32: phi within
1e-5 of the FP64 oracle on band cells, same band sizes."""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O

N = 24
FB = (0, N - 1) * 3
GB = (-3, N + 2) * 3
FB = (FB[0], FB[1], FB[0], FB[1], FB[0], FB[1])
GB = (GB[0], GB[1], GB[0], GB[1], GB[0], GB[1])
DX = 2.0 / N


def spheres_phi(seed=7, count=3):
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-0.35, 0.35, size=(count, 3))
    rad = rng.uniform(0.2, 0.3, size=count)
    c = -1.0 + (np.arange(-3, N + 3) + 0.5) * DX
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    d = np.min([np.sqrt((X - p[0]) ** 2 + (Y - p[1]) ** 2 + (Z - p[2]) ** 2) - r for p, r in zip(cen, rad)], axis=0)
    return np.asfortranarray(d)


ARGS = dict(n_steps=6, rebuild_every=3, gamma=3 * DX, beta=1.5 * DX, a_n=1.0, b_n=0.1, cfl=0.5)


def oracle_result(phi):
    return O.band_run(H.oracle(), phi, GB, FB, DX, ARGS["n_steps"], ARGS["rebuild_every"], ARGS["gamma"],
                      ARGS["beta"], ARGS["a_n"], ARGS["b_n"], ARGS["cfl"])


def test_oracle_band_flow_runs():
    phi = spheres_phi()
    out, dts, bands = oracle_result(phi)
    assert len(dts) == ARGS["n_steps"] and all(d > 0 for d in dts)
    assert np.max(np.abs(out - phi)) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("device", [False, True])
def test_band_flow_f64_bit_exact(device, gpu_lib):
    import torch
    phi = spheres_phi()
    want, want_dt, bands = oracle_result(phi)
    if device:
        t = torch.from_numpy(np.ascontiguousarray(phi.T)).cuda()
        dts, counts = L.band_flow_weno5_tvdrk3(t, GB, FB, DX, ARGS["n_steps"], ARGS["rebuild_every"], ARGS["gamma"],
                                               ARGS["beta"], ARGS["a_n"], ARGS["b_n"], ARGS["cfl"], "f64")
        got = t.cpu().numpy().T
    else:
        got = phi.copy(order="F")
        dts, counts = L.band_flow_weno5_tvdrk3(got, GB, FB, DX, ARGS["n_steps"], ARGS["rebuild_every"], ARGS["gamma"],
                                               ARGS["beta"], ARGS["a_n"], ARGS["b_n"], ARGS["cfl"], "f64")
    assert [int(b[5][0] + 1) for b in bands] == list(counts)
    assert np.array_equal(np.asarray(want_dt), dts)
    assert H.same(want, got), np.max(np.abs(want - got))


@pytest.mark.gpu
@pytest.mark.parametrize("n_steps,rebuild_every,gamma", [(12, 2, 2.5 * DX), (13, 1, 3 * DX)])
def test_band_flow_f64_many_rebuilds_bit_exact(n_steps, rebuild_every, gamma, gpu_lib):
    """Rebuilds after the first draw the new level 0 from the previous one
    (the flow changes phi only there); many rebuilds on a moving front, every
    level-0 count, dt and the final phi equal to the oracle's (which rebuilds
    over the whole grid each time)."""
    phi = spheres_phi(seed=9, count=4)
    args = dict(ARGS, n_steps=n_steps, rebuild_every=rebuild_every, gamma=gamma, beta=gamma / 2)
    want, want_dt, bands = O.band_run(H.oracle(), phi, GB, FB, DX, n_steps, rebuild_every, args["gamma"],
                                      args["beta"], args["a_n"], args["b_n"], args["cfl"])
    got = phi.copy(order="F")
    dts, counts = L.band_flow_weno5_tvdrk3(got, GB, FB, DX, n_steps, rebuild_every, args["gamma"], args["beta"],
                                           args["a_n"], args["b_n"], args["cfl"], "f64")
    assert [int(b[5][0] + 1) for b in bands] == list(counts)
    assert np.array_equal(np.asarray(want_dt), dts)
    assert H.same(want, got), np.max(np.abs(want - got))


@pytest.mark.gpu
def test_band_flow_f32_within_tolerance(gpu_lib):
    phi = spheres_phi()
    want, want_dt, bands = oracle_result(phi)
    got = np.asfortranarray(phi.astype(np.float32))
    dts, counts = L.band_flow_weno5_tvdrk3(got, GB, FB, DX, ARGS["n_steps"], ARGS["rebuild_every"], ARGS["gamma"],
                                           ARGS["beta"], ARGS["a_n"], ARGS["b_n"], ARGS["cfl"], "f32")
    assert [int(b[5][0] + 1) for b in bands] == list(counts)
    assert np.max(np.abs(np.asarray(want_dt) - dts)) <= 1e-5 * max(want_dt)
    band = np.abs(phi) < ARGS["gamma"]
    assert np.max(np.abs(want - got.astype(np.float64))[band]) <= 1e-5
