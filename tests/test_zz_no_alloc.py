"""The allocation-free dt entry point against the regular one.

lsmgpu_compute_stable_advection_dt_noalloc serves callers that cannot let a
library allocate device memory (a solver living inside another framework's
memory pool, or a time-step loop that must not stall on the device
synchronisation cudaMalloc/cudaFree can cause).  Its scratch is a fixed
file-scope device array that every call reuses, so these tests call it twice
in a row with data whose maximum shrinks, which would expose a result left
over from the previous call, and check both results against
lsm3dcomputestableadvectiondt_ (the same maximum and formula, so the values
must be equal), and that the calls leave the library's device arena and the
device's free memory unchanged.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import lsmlib_gb300 as L

GB = (-3, 70, -2, 40, -1, 33)
IB = (0, 66, 0, 37, 0, 31)


def _noalloc(h):
    fn = h.lsmgpu_compute_stable_advection_dt_noalloc
    fn.restype = ctypes.c_int
    return fn


def _args(dt_ptr, vel, gb, ib, dx=(0.1, 0.12, 0.09), cfl=0.5):
    ints = [ctypes.byref(ctypes.c_int(v)) for v in gb] + [ctypes.byref(ctypes.c_int(v)) for v in ib]
    return ([dt_ptr] + [ctypes.c_void_p(v.data_ptr()) for v in vel] + ints +
            [ctypes.byref(ctypes.c_double(d)) for d in dx] + [ctypes.byref(ctypes.c_double(cfl))])


def _existing(h, vel, gb, ib, dx=(0.1, 0.12, 0.09), cfl=0.5):
    vals = {"vel_x": vel[0], "vel_y": vel[1], "vel_z": vel[2], "dt": -5.0,
            "dx": dx[0], "dy": dx[1], "dz": dx[2], "cfl_number": cfl}
    for n, v in zip(("ilo_vel_gb", "ihi_vel_gb", "jlo_vel_gb", "jhi_vel_gb", "klo_vel_gb", "khi_vel_gb"), gb):
        vals[n] = v
    for n, v in zip(("ilo_ib", "ihi_ib", "jlo_ib", "jhi_ib", "klo_ib", "khi_ib"), ib):
        vals[n] = v
    out = L.invoke(h, "lsm3dcomputestableadvectiondt_", vals)
    L.check(h)
    return out["dt"]


def _velocity(scale, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    shape = (GB[5] - GB[4] + 1, GB[3] - GB[2] + 1, GB[1] - GB[0] + 1)  # Fortran order, reversed
    return [(scale * (2 * torch.rand(shape, generator=g, dtype=torch.float64) - 1)).cuda() for _ in range(3)]


@pytest.mark.gpu
def test_noalloc_dt_matches_existing_entry_point_on_two_calls(gpu_lib):
    import torch
    fn = _noalloc(gpu_lib)
    dt_dev = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    results = []
    for call, (scale, seed) in enumerate([(3.0, 1), (0.5, 2)]):
        vel = _velocity(scale, seed)
        want = _existing(gpu_lib, vel, GB, IB)
        # device result
        rc = fn(*_args(ctypes.c_void_p(dt_dev.data_ptr()), vel, GB, IB))
        assert rc == 0, L.last_error(gpu_lib)
        torch.cuda.synchronize()
        got_dev = float(dt_dev.item())
        # host result
        host = ctypes.c_double(-1.0)
        rc = fn(*_args(ctypes.cast(ctypes.pointer(host), ctypes.c_void_p), vel, GB, IB))
        assert rc == 0, L.last_error(gpu_lib)
        assert got_dev == want and host.value == want, (call, got_dev, host.value, want)
        results.append(want)
    assert results[1] > results[0]  # the second call's smaller maximum was not masked


def _arena_bytes(h):
    fn = h.lsmgpu_arena_bytes
    fn.restype = ctypes.c_longlong
    return int(fn())


@pytest.mark.gpu
def test_noalloc_dt_allocates_nothing(gpu_lib):
    """No arena growth and no change of the device's free memory across calls
    (the first call of the process may load the library's module, which
    places the fixed scratch array; free memory is compared after it)."""
    import torch
    fn = _noalloc(gpu_lib)
    vel = _velocity(2.0, 5)
    want = _existing(gpu_lib, vel, GB, IB)
    torch.cuda.synchronize()
    arena0 = _arena_bytes(gpu_lib)
    host = ctypes.c_double(-1.0)
    assert fn(*_args(ctypes.cast(ctypes.pointer(host), ctypes.c_void_p), vel, GB, IB)) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    torch0 = torch.cuda.memory_allocated()
    for _ in range(3):
        host.value = -1.0
        assert fn(*_args(ctypes.cast(ctypes.pointer(host), ctypes.c_void_p), vel, GB, IB)) == 0
        assert host.value == want
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert _arena_bytes(gpu_lib) == arena0
    assert free1 == free0 and torch.cuda.memory_allocated() == torch0


@pytest.mark.gpu
def test_noalloc_rejects_boxes_beyond_its_scratch(gpu_lib):
    fn = _noalloc(gpu_lib)
    vel = _velocity(1.0, 3)
    huge = (0, 1023, 0, 1023, 0, 1023)   # 2^30 cells > the 536,870,912-cell limit
    host = ctypes.c_double(-1.0)
    rc = fn(*_args(ctypes.cast(ctypes.pointer(host), ctypes.c_void_p), vel, huge, huge))
    code, msg = L.last_error(gpu_lib)
    assert rc == 4 and code == 4 and "at most" in msg
    assert host.value == -1.0
