"""The k-slab threaded oracle runs (tests/oracle_threads.py) reproduce the
serial LSMLIB call compositions of tests/oracle_runs.py bit for bit."""
import numpy as np

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O
from tests.oracle_threads import SlabRun, periodic_fill

FB = (0, 15, 0, 13, 0, 17)
GB = (-3, 18, -3, 16, -3, 20)
DX = 2.0 / 16


def _phi():
    rng = np.random.default_rng(2)
    phi = H.sphere_phi(GB, DX, center=(-0.5, -0.4, -0.6), r=0.35)
    return np.asfortranarray(phi * (1.0 + 0.3 * rng.random(phi.shape)))


def test_slab_periodic_fill_matches_oracle_runs():
    for gb, fb in ((GB, FB), ((-4, 12, -3, 9, -5, 14), (0, 8, 0, 6, 0, 9)), ((-3, 5, -3, 5, -3, 5), (0, 2, 0, 2, 0, 2))):
        a = np.asfortranarray(np.random.default_rng(1).standard_normal(H.shape_of(gb)))
        b = a.copy(order="F")
        O.periodic_fill(a, gb, fb)
        periodic_fill(b, gb, fb)
        assert np.array_equal(a, b)


def test_threaded_reinit_matches_serial():
    phi = _phi()
    want = O.tvdrk3_run(H.oracle(), "reinit", phi, GB, FB, DX, 0.5 * DX, 2, L.BC_SIGNED_LINEAR, use0=1)
    got = SlabRun(H.oracle(), GB, FB, threads=4).run("reinit", phi, DX, 0.5 * DX, 2, L.BC_SIGNED_LINEAR, use0=1)
    assert H.same(want, got)


def test_threaded_advection_matches_serial():
    phi = _phi()
    vel = [np.full(H.shape_of(GB), v, order="F") for v in (1.0, 0.5, 0.25)]
    want = O.tvdrk3_run(H.oracle(), "advect", phi, GB, FB, DX, DX / 3.5, 2, L.BC_PERIODIC, vel=vel)
    got = SlabRun(H.oracle(), GB, FB, threads=5).run("advect", phi, DX, DX / 3.5, 2, L.BC_PERIODIC, vel=vel)
    assert H.same(want, got)


def test_threaded_advection_matches_serial_at_64_on_many_threads():
    # slabs racing for shared arrays show at this size (the zero-out of the
    # right-hand side clears its whole ghost box)
    import bench
    gb, fb = bench.boxes(64)
    phi, vel, dt, dx = bench.advection_case(64)
    vf = [np.full(phi.shape, v, order="F") for v in vel]
    want = O.tvdrk3_run(H.oracle(), "advect", phi, gb, fb, dx, dt, 1, L.BC_PERIODIC, vel=vf)
    got = SlabRun(H.oracle(), gb, fb, threads=16).run("advect", phi, dx, dt, 1, L.BC_PERIODIC, vel=vf)
    assert H.same(want, got)


def test_threaded_curvature_matches_serial():
    from tests.test_fused_curvature import oracle_chain, GB as CGB, FB as CFB, DX as CDX, DY, DZ, _phi as cphi
    phi = cphi(1)
    want_k, want_m = oracle_chain(phi)
    k, m = SlabRun(H.oracle(), CGB, CFB, threads=3).mean_curvature(phi, (CDX, DY, DZ))
    sl = tuple(slice(CFB[2 * d] - CGB[2 * d], CFB[2 * d + 1] - CGB[2 * d] + 1) for d in range(3))
    assert H.same(k[sl], want_k[sl]) and H.same(m[sl], want_m[sl])
