"""Batched advection of uneven grids (one persistent launch per stage, CUDA
graph, autotuned tiles) against per-grid single-grid runs and the FP64
oracle.  The per-cell FP32 arithmetic is the same kernel code in every mode,
so batched, launch-loop and single-grid results must be identical; against
the FP64 oracle the FP32 error bound is 1e-5 on these O(1) fields."""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O


def make_batch(n, seed=11, lo=8, hi=20):
    """Small uneven grids: sides U{lo..hi} per axis, an ellipsoid-like level
    set on [-1,1]^3 (cell centres), constant velocity U[-1,1]^3, dt at CFL 0.5."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(lo, hi + 1, size=(n, 3))
    vel = rng.uniform(-1, 1, size=(n, 3))
    spacing = 2.0 / dims
    dt = 0.5 / (np.abs(vel) / spacing).sum(axis=1)
    fields, offsets, off = [], [], 0
    for g in range(n):
        nx, ny, nz = (int(v) for v in dims[g])
        axes = rng.uniform(0.2, 0.6, size=3)
        c = [-1.0 + (np.arange(-3, m + 3) + 0.5) * 2.0 / m for m in (nx, ny, nz)]
        X, Y, Z = np.meshgrid(*c, indexing="ij")
        phi = np.sqrt((X / axes[0]) ** 2 + (Y / axes[1]) ** 2 + (Z / axes[2]) ** 2) - 1.0
        phi = np.asfortranarray(phi * axes.min())
        fields.append(phi)
        offsets.append(off)
        off += phi.size
    return dims, vel, spacing, dt, fields, np.array(offsets)


def pack(fields, offsets, dtype=np.float32):
    buf = np.zeros(int(offsets[-1] + fields[-1].size), dtype=dtype)
    for f, o in zip(fields, offsets):
        buf[o:o + f.size] = f.ravel(order="F")
    return buf


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0, L.BATCH_NO_GRAPH, L.BATCH_LOOP, L.batch_tz(4), L.batch_tz(16)])
def test_batch_equals_single_grid_runs(flags, gpu_lib):
    dims, vel, spacing, dt, fields, offsets = make_batch(24)
    buf = pack(fields, offsets)
    L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, dt, 3, flags=flags)
    for g, f in enumerate(fields):
        nx, ny, nz = (int(v) for v in dims[g])
        single = np.asfortranarray(f.astype(np.float32))
        gb = (-3, nx + 2, -3, ny + 2, -3, nz + 2)
        fb = (0, nx - 1, 0, ny - 1, 0, nz - 1)
        L.advect_weno5_tvdrk3(single, gb, fb, float(spacing[g, 0]), float(dt[g]), 3,
                              vel_const=tuple(float(v) for v in vel[g]), precision="f32",
                              dy=float(spacing[g, 1]), dz=float(spacing[g, 2]))
        got = buf[offsets[g]:offsets[g] + f.size].reshape(f.shape, order="F")
        assert np.array_equal(got, single), g


@pytest.mark.gpu
def test_batch_fp32_against_fp64_oracle(gpu_lib):
    dims, vel, spacing, dt, fields, offsets = make_batch(4, seed=5)
    buf = pack(fields, offsets)
    L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, dt, 2)
    for g, f in enumerate(fields):
        nx, ny, nz = (int(v) for v in dims[g])
        gb = (-3, nx + 2, -3, ny + 2, -3, nz + 2)
        fb = (0, nx - 1, 0, ny - 1, 0, nz - 1)
        v = [np.full(f.shape, float(c), order="F") for c in vel[g]]
        want = O.tvdrk3_run(H.oracle(), "advect", f, gb, fb, tuple(float(x) for x in spacing[g]),
                            float(dt[g]), 2, L.BC_PERIODIC, vel=v)
        got = buf[offsets[g]:offsets[g] + f.size].reshape(f.shape, order="F")
        assert np.max(np.abs(got[3:-3, 3:-3, 3:-3] - want[3:-3, 3:-3, 3:-3])) <= 1e-5
