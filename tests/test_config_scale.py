"""Parity at the workloads' own sizes (GPU against the oracle).

1. Advection, 128^3 x 50 steps, periodic, FP64: the fused stepper equals
   the oracle's LSMLIB call sequence bit for bit.
2. Reinitialization, 256^3 x 20 iterations (phi0 sign form, signed linear
   extrapolation) + mean curvature: FP64 equals the oracle bit for bit; FP32
   within 1e-5 L-inf of that oracle result, its curvature within 2e-4 of the
   largest |kappa| near the interface.
3. Narrow band, 512^3, 64 spheres (seed 7), half-width 6 dx, inner 3 dx,
   3 neighbour levels: the band build's lists, levels, outer lists and marks
   equal the reference's lsm3dDetermineNarrowBand (translated Fortran, or
   the oracle when the translation is absent) entry for entry.
4. Batched: the first 64 grids of the seed-11 batch, 30 steps, FP32 batched
   launch within 1e-5 L-inf of the FP64 oracle within 3 dx of the
   interface, 5e-5 elsewhere (where the periodic extension of the
   ellipsoid distance has kinks at the domain faces).
5. Adjoint at 64^3 x 40 steps: the FP64 GPU gradient against the FP64
   oracle reverse mode (1e-10 of the gradient's largest entry), and the
   FP64 / FP32 gradients against central differences (h = 1e-3) along 32
   random directions.
6. Near-flat data in FP32: a constant field and a field of size 1e-20 (the
   (S + eps)^2 underflow of a single-precision WENO5,
   spatial_derivatives3d.f.in:1314-1320): no NaN or infinity, and the FP64
   oracle's result within the stated tolerance.
The oracle runs split each call into k-slabs over the host's cores
(tests/oracle_threads.py)."""
import os
import threading

import numpy as np
import pytest

import bench
import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O
from tests.oracle_threads import SlabRun, parallel


def _dev(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    return t if dtype is None else t.to(dtype)


def _host(t):
    return t.cpu().numpy().T


# ---------------------------------------------------------------------------
# 1. advection 128^3, 50 steps, FP64
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_config1_advection_128_fp64_bit_exact(gpu_lib):
    import torch
    n, steps = 128, 50
    gb, fb = bench.boxes(n)
    phi, vel, dt, dx = bench.advection_case(n)
    vf = [np.full(phi.shape, v, order="F") for v in vel]
    want = SlabRun(H.oracle(), gb, fb).run("advect", phi, dx, dt, steps, L.BC_PERIODIC, vel=vf)
    t = _dev(phi, torch.float64)
    L.advect_weno5_tvdrk3(t, gb, fb, dx, dt, steps, vel_const=vel, precision="f64")
    got = _host(t)
    L.check()
    assert H.same(want, got), np.max(np.abs(want - got))
    # the FP32 form (4-plane tiles at this size) against the same oracle run:
    # within 1e-5 within 3 dx of the interface, 5e-5 elsewhere
    t32 = _dev(phi, torch.float32)
    L.advect_weno5_tvdrk3(t32, gb, fb, dx, dt, steps, vel_const=vel, precision="f32")
    got32 = _host(t32).astype(np.float64)
    L.check()
    inner = (slice(3, -3),) * 3
    err = np.abs(got32 - want)[inner]
    near = np.abs(want[inner]) <= 3 * dx
    assert np.max(err[near]) <= 1e-5, np.max(err[near])
    assert np.max(err) <= 5e-5, np.max(err)


@pytest.mark.gpu
def test_advection_f32_192_eight_plane_tiles(gpu_lib):
    """192^3 (the adjoint workload's size, where the FP32 advection stage runs
    8-plane tiles), velocity field of the adjoint workload, 4 steps, periodic:
    within 1e-5 of the FP64 oracle within 3 dx of the interface, 5e-5 elsewhere."""
    import torch
    n, steps = 192, 4
    gb, fb = bench.boxes(n)
    phi, vel, tgt, dx, dt = bench.adjoint_case(n)
    pad = lambda a: np.asfortranarray(np.pad(a, 3, mode="wrap"))
    P, V = pad(phi), [pad(v) for v in vel]
    want = SlabRun(H.oracle(), gb, fb).run("advect", P, dx, dt, steps, L.BC_PERIODIC, vel=V)
    t = _dev(P, torch.float32)
    vt = [_dev(v, torch.float32) for v in V]
    L.advect_weno5_tvdrk3(t, gb, fb, dx, dt, steps, vel=vt, vel_gb=gb, precision="f32")
    got = _host(t).astype(np.float64)
    L.check()
    inner = (slice(3, -3),) * 3
    err = np.abs(got - want)[inner]
    near = np.abs(want[inner]) <= 3 * dx
    assert np.max(err[near]) <= 1e-5, np.max(err[near])
    assert np.max(err) <= 5e-5, np.max(err)


# ---------------------------------------------------------------------------
# 2. reinitialization 256^3, 20 iterations, + mean curvature
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_config2_reinit_256_fp64_bit_exact_fp32_within_1e5(gpu_lib):
    import torch
    n, iters = 256, 20
    gb, fb = bench.boxes(n)
    phi, dx = bench.initial_phi(n)
    run = SlabRun(H.oracle(), gb, fb)
    want = run.run("reinit", phi, dx, 0.5 * dx, iters, L.BC_SIGNED_LINEAR, use0=1)
    want_k, _ = run.mean_curvature(want, dx)
    inner = (slice(3, -3),) * 3

    t64 = _dev(phi, torch.float64)
    L.reinit_weno5_tvdrk3(t64, gb, fb, dx, 0.5 * dx, iters, use_phi0_for_sgn=1, bc=L.BC_SIGNED_LINEAR,
                          precision="f64")
    k64 = torch.zeros_like(t64)
    L.mean_curvature_o2(k64, gb, t64, gb, fb, dx, precision="f64")
    got = _host(t64)
    assert H.same(want, got), np.max(np.abs(want - got))
    assert H.same(want_k[inner], _host(k64)[inner])

    t32 = _dev(phi, torch.float32)
    L.reinit_weno5_tvdrk3(t32, gb, fb, dx, 0.5 * dx, iters, use_phi0_for_sgn=1, bc=L.BC_SIGNED_LINEAR,
                          precision="f32")
    k32 = torch.zeros_like(t32)
    L.mean_curvature_o2(k32, gb, t32, gb, fb, dx, precision="f32")
    L.check()
    err = np.abs(_host(t32).astype(np.float64) - want)[inner]
    assert np.max(err) <= 1e-5, np.max(err)
    band = np.abs(want[inner]) < 3 * dx
    kerr = np.abs(_host(k32).astype(np.float64)[inner] - want_k[inner])[band]
    assert np.max(kerr) <= 2e-4 * np.max(np.abs(want_k[inner][band])), np.max(kerr)


# ---------------------------------------------------------------------------
# 3. narrow-band lists at 512^3
# ---------------------------------------------------------------------------
def _band_values(phi, nb, ix, iy, iz, n_lo, n_hi, outer, gb, dx, level):
    cap = ix.shape[0]
    vals = {"phi": phi, "narrow_band": nb, "index_x": ix, "index_y": iy, "index_z": iz,
            "nlo_index": 0, "nhi_index": cap - 1, "n_lo": n_lo, "n_hi": n_hi,
            "index_outer": outer, "nlo_index_outer": 0, "nhi_index_outer": cap - 1,
            "nlo_outer_plus": 0, "nhi_outer_plus": 0, "nlo_outer_minus": 0, "nhi_outer_minus": 0,
            "width": 6 * dx, "width_inner": 3 * dx, "level": level}
    for w, v in zip(("ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb"), gb):
        vals[w] = v
        vals[w.replace("_gb", "_nb_gb")] = v
    return vals


@pytest.mark.gpu
def test_config3_band_lists_512_equal_reference(gpu_lib):
    import torch
    n, level = 512, 3
    gb, fb = bench.boxes(n)
    tphi, dx = bench.band_case("cuda", n, dtype=torch.float64)
    phi = np.asfortranarray(tphi.cpu().numpy().T)
    cap = 1 << 24  # entries per list; the band holds about 6e6 cells
    shape = phi.shape
    ref = H.reference() or H.oracle()

    def arrays(dev):
        if dev:
            z = lambda dt, m: torch.zeros(m, dtype=dt, device="cuda")
            nb = torch.zeros(tuple(reversed(shape)), dtype=torch.uint8, device="cuda")
            return (nb, z(torch.int32, cap), z(torch.int32, cap), z(torch.int32, cap),
                    np.zeros(level + 1, np.int32), np.zeros(level + 1, np.int32), z(torch.int32, cap))
        return (np.zeros(shape, np.uint8, order="F"), np.zeros(cap, np.int32), np.zeros(cap, np.int32),
                np.zeros(cap, np.int32), np.zeros(level + 1, np.int32), np.zeros(level + 1, np.int32),
                np.zeros(cap, np.int32))

    ha = arrays(False)
    want = L.invoke(ref, "lsm3ddeterminenarrowband_", _band_values(phi, *ha, gb, dx, level))
    da = arrays(True)
    got = L.invoke(gpu_lib, "lsm3ddeterminenarrowband_", _band_values(tphi, *da, gb, dx, level))
    torch.cuda.synchronize()
    L.check()
    nb_w, ix_w, iy_w, iz_w, lo_w, hi_w, out_w = ha
    nb_g, ix_g, iy_g, iz_g, lo_g, hi_g, out_g = da
    assert np.array_equal(lo_w, lo_g) and np.array_equal(hi_w, hi_g), (lo_w, hi_w, lo_g, hi_g)
    m = int(hi_w[level]) + 1
    assert m > 2_000_000  # the 64-sphere band at 512^3
    for a, b in ((ix_w, ix_g), (iy_w, iy_g), (iz_w, iz_g)):
        assert np.array_equal(a[:m], b[:m].cpu().numpy())
    for key in ("nlo_outer_plus", "nhi_outer_plus", "nlo_outer_minus", "nhi_outer_minus",
                "nlo_index_outer", "nhi_index_outer"):
        assert want[key] == got[key], key
    og = out_g.cpu().numpy()
    n_outer = 0
    for side in ("plus", "minus"):
        lo, hi = want["nlo_outer_" + side], want["nhi_outer_" + side]
        if hi >= lo:
            n_outer += hi - lo + 1
            assert np.array_equal(out_w[lo:hi + 1], og[lo:hi + 1]), side
    assert n_outer > 0
    assert np.array_equal(nb_w, _host(nb_g))


# ---------------------------------------------------------------------------
# 4. batched: 64 grids of the seed-11 batch, 30 steps, FP32
# ---------------------------------------------------------------------------
def _ellipsoid(dims, axes):
    c = [-1.0 + (np.arange(-3, m + 3) + 0.5) * 2.0 / m for m in dims]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    f = (np.sqrt((X / axes[0]) ** 2 + (Y / axes[1]) ** 2 + (Z / axes[2]) ** 2) - 1.0) * axes.min()
    return np.asfortranarray(f)


@pytest.mark.gpu
def test_config4_batched_slice_fp32_against_oracle(gpu_lib):
    steps, n_grids = 30, 64
    dims, axes, vel, spacing, dt = (a[:n_grids] for a in bench.batched_params(4096))
    fields = [_ellipsoid([int(v) for v in dims[g]], axes[g]) for g in range(n_grids)]
    sizes = [f.size for f in fields]
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    buf = np.zeros(int(sum(sizes)), np.float32)
    for f, o in zip(fields, offsets):
        buf[o:o + f.size] = f.ravel(order="F")
    L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, dt, steps)
    want = [None] * n_grids
    queue = list(range(n_grids))
    lock = threading.Lock()

    def worker(_):
        while True:
            with lock:
                if not queue:
                    return
                g = queue.pop()
            nx, ny, nz = (int(v) for v in dims[g])
            gb = (-3, nx + 2, -3, ny + 2, -3, nz + 2)
            fb = (0, nx - 1, 0, ny - 1, 0, nz - 1)
            v = [np.full(fields[g].shape, float(c), order="F") for c in vel[g]]
            # the spacing and dt the FP32 entry point receives, as doubles
            sp = tuple(float(np.float32(x)) for x in spacing[g])
            want[g] = O.tvdrk3_run(H.oracle(), "advect", fields[g], gb, fb, sp, float(np.float32(dt[g])), steps,
                                   L.BC_PERIODIC, vel=v)

    parallel(worker, min(16, os.cpu_count() or 1))
    worst_near, worst_far = 0.0, 0.0
    inner = (slice(3, -3),) * 3
    for g in range(n_grids):
        got = buf[offsets[g]:offsets[g] + sizes[g]].reshape(fields[g].shape, order="F")
        err = np.abs(got[inner].astype(np.float64) - want[g][inner])
        near = np.abs(want[g][inner]) < 3 * float(spacing[g].max())
        worst_near = max(worst_near, float(err[near].max()) if near.any() else 0.0)
        worst_far = max(worst_far, float(err.max()))
    assert worst_near <= 1e-5, worst_near
    assert worst_far <= 5e-5, worst_far


# ---------------------------------------------------------------------------
# 5. adjoint at 64^3: oracle gradient and 32 finite-difference directions
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_config5_adjoint_64_oracle_gradient_and_32_directions(gpu_lib):
    from tests.test_adjoint import adjoint_case, gpu_adjoint, oracle_adjoint, smooth_unit, unit
    n, steps = 64, 40
    phi, vel, tgt, sp, dt = adjoint_case((n, n, n))
    eps = 1.5 * sp[0]
    box = {}
    th = threading.Thread(target=lambda: box.update(r=oracle_adjoint(phi, vel, tgt, sp, dt, steps, eps)))
    th.start()  # the CPU reverse mode runs while the GPU computes the differences below
    J64, g64, gv64 = gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, "f64", 8)
    _, g32, gv32 = gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, "f32", 8)
    Jof = lambda p, v: gpu_adjoint(p, v, tgt, sp, dt, steps, eps, "f64", grads=False)[0]

    def cd(d, dv, h):
        return (Jof(phi + h * d, [v + h * e for v, e in zip(vel, dv)]) -
                Jof(phi - h * d, [v - h * e for v, e in zip(vel, dv)])) / (2 * h)

    rng = np.random.default_rng(32)
    h = 1e-3
    worst = {"f64": 0.0, "f32": 0.0}
    for q in range(32):
        # joint unit directions in (phi0, u, v, w): 16 smooth, 16 white noise
        if q < 16:
            d, *dv = smooth_unit(rng, phi.shape, 4)
            fd = cd(d, dv, h)
        else:
            d, *dv = unit(rng, phi.shape, 4)
            # white noise: Richardson extrapolation from h and h/2 (the plain
            # difference carries an O(h^2) truncation error near 1e-3 there)
            fd = (4 * cd(d, dv, h / 2) - cd(d, dv, h)) / 3
        for key, g, gv in (("f64", g64, gv64), ("f32", g32, gv32)):
            an = np.sum(g * d) + sum(np.sum(a * e) for a, e in zip(gv, dv))
            worst[key] = max(worst[key], abs(an - fd) / abs(fd))
    th.join()
    Jw, _, gw, gvw = box["r"]
    assert abs(J64 - Jw) <= 1e-12 * abs(Jw)
    scale = max(np.max(np.abs(gw)), max(np.max(np.abs(v)) for v in gvw))
    assert np.max(np.abs(g64 - gw)) <= 1e-10 * scale
    for a, b in zip(gv64, gvw):
        assert np.max(np.abs(a - b)) <= 1e-10 * scale
    assert worst["f64"] <= 1e-4, worst
    assert worst["f32"] <= 3e-4, worst


# ---------------------------------------------------------------------------
# 6. near-flat data, FP32
# ---------------------------------------------------------------------------
NF_FB = (0, 23, 0, 19, 0, 17)
NF_GB = (-3, 26, -3, 22, -3, 20)
NF_DX = 2.0 / 24


def _smooth_field(scale):
    c = [-1.0 + (np.arange(NF_GB[2 * a], NF_GB[2 * a + 1] + 1) + 0.5) * NF_DX for a in range(3)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    return np.asfortranarray(scale * (0.3 + np.sin(2 * X) * np.cos(3 * Y) + 0.5 * Z))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["constant", "tiny"])
@pytest.mark.parametrize("mode", ["reinit", "advect"])
def test_near_flat_fp32(case, mode, gpu_lib):
    phi = np.asfortranarray(np.full(H.shape_of(NF_GB), 0.3)) if case == "constant" else _smooth_field(1e-20)
    steps = 3
    if mode == "reinit":
        want = O.tvdrk3_run(H.oracle(), "reinit", phi, NF_GB, NF_FB, NF_DX, 0.5 * NF_DX, steps,
                            L.BC_SIGNED_LINEAR, use0=1)
        got = np.asfortranarray(phi.astype(np.float32))
        L.reinit_weno5_tvdrk3(got, NF_GB, NF_FB, NF_DX, 0.5 * NF_DX, steps, use_phi0_for_sgn=1,
                              bc=L.BC_SIGNED_LINEAR, precision="f32")
    else:
        vel = (1.0, -0.5, 0.25)
        vf = [np.full(phi.shape, v, order="F") for v in vel]
        want = O.tvdrk3_run(H.oracle(), "advect", phi, NF_GB, NF_FB, NF_DX, NF_DX / 3.5, steps, L.BC_PERIODIC,
                            vel=vf)
        got = np.asfortranarray(phi.astype(np.float32))
        L.advect_weno5_tvdrk3(got, NF_GB, NF_FB, NF_DX, NF_DX / 3.5, steps, vel_const=vel, bc=L.BC_PERIODIC,
                              precision="f32")
    L.check()
    inner = (slice(3, -3),) * 3
    g = got[inner].astype(np.float64)
    assert np.all(np.isfinite(g))
    err = np.max(np.abs(g - want[inner]))
    if case == "constant":
        assert err <= 1e-6, err
    else:
        # values of size 1e-20: FP32 keeps 24 bits of them; the bound is relative
        assert err <= 1e-5 * np.max(np.abs(want[inner])), err
