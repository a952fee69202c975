"""lsmlib_gb300 — GB300-native level-set kernels with LSMLIB's C interface.

The product is the shared library ``liblsmgpu.so`` (CUDA, sm_103a) in this
directory.  It exports LSMLIB's 3D toolbox routines under LSMLIB's own symbol
names and argument lists (include/lsmgpu_toolbox3d.h) plus fused
time-stepping entry points (include/lsmgpu.h).  This module is a thin ctypes
binding used by the tests and the benchmark:

* :func:`lib` loads the library (and fails loudly when it is missing — there
  is no CPU fallback);
* :data:`ABI` lists every drop-in entry point with its argument list
  (name, kind, is-array, written), mirroring the reference's Fortran
  signature;
* :func:`invoke` calls an entry point by symbol name with arguments given by
  their LSMLIB names.
"""
import ctypes
import json
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblsmgpu.so")

with open(os.path.join(_HERE, "abi.json")) as _f:
    ABI = json.load(_f)

_lib = None


def lib(path=None):
    """Load liblsmgpu.so once and return the ctypes handle."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "liblsmgpu.so is not built (%s); run `python -m lsmlib_gb300.build` "
            "— the level-set kernels have no CPU fallback" % p)
    handle = ctypes.CDLL(p, mode=ctypes.RTLD_LOCAL)
    handle.lsmgpu_get_last_error.restype = ctypes.c_int
    handle.lsmgpu_get_last_error.argtypes = [ctypes.c_char_p, ctypes.c_int]
    handle.lsmgpu_set_stream.argtypes = [ctypes.c_void_p]
    handle.lsmgpu_get_stream.restype = ctypes.c_void_p
    handle.lsmgpu_launch_count.restype = ctypes.c_longlong
    handle.lsmgpu_graph_capture_count.restype = ctypes.c_longlong
    handle.lsmgpu_arena_bytes.restype = ctypes.c_longlong
    handle.lsmgpu_version.restype = ctypes.c_char_p
    if path is None:
        _lib = handle
    return handle


def last_error(handle=None):
    """(code, message) of the last call on this thread."""
    h = handle or lib()
    buf = ctypes.create_string_buffer(512)
    code = h.lsmgpu_get_last_error(buf, 512)
    return code, buf.value.decode()


def check(handle=None):
    code, msg = last_error(handle)
    if code != 0:
        raise RuntimeError("lsmgpu error %d: %s" % (code, msg))


def set_stream(stream_ptr, handle=None):
    (handle or lib()).lsmgpu_set_stream(ctypes.c_void_p(stream_ptr or 0))


def launch_count(handle=None):
    return int((handle or lib()).lsmgpu_launch_count())


def graph_capture_count(handle=None):
    """Graphs the fused steppers captured so far (a cache miss captures)."""
    return int((handle or lib()).lsmgpu_graph_capture_count())


def measure_fma_rates(handle=None):
    """(FP32 lane operations/s through packed FFMA2, FP64 FMAs/s) measured by
    the library's fixed-length probe kernels on the current device."""
    h = handle or lib()
    a, b = ctypes.c_double(0.0), ctypes.c_double(0.0)
    h.lsmgpu_measure_fma_rates.restype = ctypes.c_int
    rc = h.lsmgpu_measure_fma_rates(ctypes.byref(a), ctypes.byref(b))
    if rc != 0:
        raise RuntimeError("lsmgpu_measure_fma_rates failed: %s" % (last_error(h)[1],))
    return a.value, b.value


def arena_bytes(handle=None):
    """Device bytes held by the library's staging / temporary arena."""
    return int((handle or lib()).lsmgpu_arena_bytes())


_SCALAR_CT = {"real": ctypes.c_double, "double": ctypes.c_double, "int": ctypes.c_int,
              "logical": ctypes.c_int, "int1": ctypes.c_ubyte}


def _ptr(v):
    """Address of an array argument: numpy array, torch tensor or int."""
    if v is None:
        return None
    if isinstance(v, int):
        return ctypes.c_void_p(v)
    if hasattr(v, "data_ptr"):
        return ctypes.c_void_p(v.data_ptr())
    if hasattr(v, "ctypes"):
        return ctypes.c_void_p(v.ctypes.data)
    raise TypeError("unsupported array argument %r" % type(v))


def invoke(handle, sym, values, abi=None):
    """Call `sym` on `handle` (any library exporting LSMLIB's signatures).

    `values` maps each LSMLIB argument name to an array (numpy / torch /
    device address) or a scalar.  Scalars are passed by reference, as
    Fortran does; the returned dict holds every scalar argument's value
    after the call (so outputs such as dt can be read back).
    """
    spec = (abi or ABI)[sym]
    args, refs = [], {}
    for name, kind, is_arr, _written in spec["args"]:
        if name not in values:
            raise KeyError("%s: missing argument %s" % (sym, name))
        v = values[name]
        if is_arr:
            args.append(_ptr(v))
        else:
            r = _SCALAR_CT[kind](v)
            refs[name] = r
            args.append(ctypes.byref(r))
    fn = getattr(handle, sym)
    fn.restype = None
    fn(*args)
    return {k: r.value for k, r in refs.items()}


# ---------------------------------------------------------------------------
# fused time steppers (include/lsmgpu.h)
# ---------------------------------------------------------------------------
BC_PERIODIC, BC_LINEAR, BC_SIGNED_LINEAR, BC_COPY = 0, 1, 2, 3


def _box(b):
    return (ctypes.c_int * 6)(*[int(v) for v in b])


def _fused(name, real):
    h = lib()
    fn = getattr(h, name)
    fn.restype = ctypes.c_int
    return fn, real


def reinit_weno5_tvdrk3(phi, gb, fb, dx, dtau, n_iter, use_phi0_for_sgn=0, bc=BC_PERIODIC,
                        precision="f64", dy=None, dz=None):
    """Reinitialise `phi` in place (numpy array in Fortran order over `gb`, or
    a torch/device address) with n_iter WENO5 / TVD-RK3 pseudo-time steps."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn, _ = _fused("lsmgpu_reinit_weno5_tvdrk3_" + precision, real)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, real, real, real, real,
                   ctypes.c_int, ctypes.c_int, ctypes.c_int]
    rc = fn(_ptr(phi), _box(gb), _box(fb), dx, dy or dx, dz or dx, dtau, int(n_iter),
            int(use_phi0_for_sgn), int(bc))
    if rc != 0:
        raise RuntimeError("lsmgpu reinit failed: %s" % (last_error()[1],))


def advect_weno5_tvdrk3(phi, gb, fb, dx, dt, n_steps, vel=None, vel_gb=None, vel_const=None,
                        bc=BC_PERIODIC, precision="f64", dy=None, dz=None):
    """Advect `phi` in place by n_steps WENO5 / TVD-RK3 steps with velocity
    fields `vel` (3 arrays over vel_gb) or the constant `vel_const`."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn, _ = _fused("lsmgpu_advect_weno5_tvdrk3_" + precision, real)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   real, real, real, real, ctypes.c_int, ctypes.c_int]
    if vel is not None:
        vx, vy, vz = (_ptr(v) for v in vel)
        vgb = _box(vel_gb)
        vc = None
    else:
        vx = vy = vz = None
        vgb = None
        vc = (real * 3)(*vel_const)
    rc = fn(_ptr(phi), _box(gb), _box(fb), vx, vy, vz, vgb, vc, dx, dy or dx, dz or dx, dt,
            int(n_steps), int(bc))
    if rc != 0:
        raise RuntimeError("lsmgpu advect failed: %s" % (last_error()[1],))


def mean_curvature_o2(kappa, kappa_gb, phi, phi_gb, fb, dx, grad_phi_mag=None, precision="f64",
                      dy=None, dz=None):
    """Second-order mean curvature of phi into kappa (and |grad phi|)."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn, _ = _fused("lsmgpu_mean_curvature_o2_" + precision, real)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, real, real, real]
    rc = fn(_ptr(kappa), _box(kappa_gb), _ptr(phi), _box(phi_gb), _ptr(grad_phi_mag), _box(fb),
            dx, dy or dx, dz or dx)
    if rc != 0:
        raise RuntimeError("lsmgpu mean curvature failed: %s" % (last_error()[1],))


BATCH_LOOP, BATCH_NO_GRAPH = 1, 2


def batch_tz(n):
    return n << 8


def advect_batch_weno5_tvdrk3(phi, offsets, dims, vel, spacing, dt, n_steps, flags=0):
    """Advect a packed batch of grids in place (FP32).  `phi` is one float32
    buffer (numpy, torch or device address); grid g holds (nx+6)(ny+6)(nz+6)
    values from offsets[g]; dims/vel/spacing are (n, 3) arrays, dt has n
    entries."""
    import numpy as np
    h = lib()
    fn = h.lsmgpu_advect_batch_weno5_tvdrk3_f32
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    dm = np.ascontiguousarray(dims, dtype=np.int32)
    v = np.ascontiguousarray(vel, dtype=np.float32)
    sp = np.ascontiguousarray(spacing, dtype=np.float32)
    d = np.ascontiguousarray(dt, dtype=np.float32)
    rc = fn(_ptr(phi), off.ctypes.data, dm.ctypes.data, len(off), v.ctypes.data, sp.ctypes.data,
            d.ctypes.data, int(n_steps), BC_PERIODIC, int(flags))
    if rc != 0:
        raise RuntimeError("lsmgpu batch advect failed: %s" % (last_error()[1],))


def band_flow_weno5_tvdrk3(phi, gb, fb, dx, n_steps, rebuild_every, gamma, beta, a_n=1.0, b_n=0.1,
                           cfl=0.5, precision="f64"):
    """Narrow-band curvature flow in place; returns (dt per step, level-0
    cells per rebuild)."""
    import numpy as np
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    h = lib()
    fn = getattr(h, "lsmgpu_band_flow_weno5_tvdrk3_" + precision)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, real, real, real, real, real, real,
                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    dts = np.zeros(max(n_steps, 1), np.float64)
    bands = np.zeros(max((n_steps + rebuild_every - 1) // rebuild_every, 1), np.int64)
    rc = fn(_ptr(phi), _box(gb), _box(fb), dx, a_n, b_n, cfl, gamma, beta, int(n_steps), int(rebuild_every),
            dts.ctypes.data, bands.ctypes.data)
    if rc != 0:
        raise RuntimeError("lsmgpu band flow failed: %s" % (last_error()[1],))
    return dts[:n_steps], bands


def _zeros_like(a):
    """A zero array of the same kind, dtype, shape and device as `a`."""
    if hasattr(a, "data_ptr"):
        import torch
        return torch.zeros_like(a)
    import numpy as np
    return np.zeros_like(a, order="F")


def advect_adjoint_weno5_tvdrk3(phi, gb, fb, vel, vel_gb, phi_target, dx, dt, n_steps, heaviside_eps,
                                checkpoint_every=8, precision="f64", dy=None, dz=None, grads=True,
                                grad_vel=True):
    """Objective J of n_steps periodic advection steps and (when `grads`) its
    gradients.  Returns (J, grad_phi, [grad_vel_x, grad_vel_y, grad_vel_z]);
    the gradients are new arrays of the kind of `phi` / `vel` (None when not
    requested)."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    h = lib()
    fn = getattr(h, "lsmgpu_advect_adjoint_weno5_tvdrk3_" + precision)
    fn.restype = ctypes.c_int
    fn.argtypes = ([ctypes.c_void_p] * 8 + [real] * 4 + [ctypes.c_int, ctypes.c_int, ctypes.c_double] +
                   [ctypes.c_void_p] * 5)
    J = ctypes.c_double(0.0)
    gphi = _zeros_like(phi) if grads else None
    gv = [_zeros_like(v) for v in vel] if (grads and grad_vel) else [None, None, None]
    rc = fn(_ptr(phi), _box(gb), _box(fb), _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), _box(vel_gb),
            _ptr(phi_target), dx, dy or dx, dz or dx, dt, int(n_steps), int(checkpoint_every),
            float(heaviside_eps), ctypes.byref(J), _ptr(gphi), _ptr(gv[0]), _ptr(gv[1]), _ptr(gv[2]))
    if rc != 0:
        raise RuntimeError("lsmgpu advect adjoint failed: %s" % (last_error()[1],))
    return J.value, gphi, gv


def advect_vjp_weno5_tvdrk3(phi, gb, fb, vel, vel_gb, grad_out, dx, dt, n_steps, checkpoint_every=8,
                            precision="f64", dy=None, dz=None, grad_vel=True):
    """Vector-Jacobian product of n_steps periodic advection steps: returns
    (phi_T, grad_phi, [grad_vel_x, grad_vel_y, grad_vel_z]) for the upstream
    gradient grad_out = dJ/dphi_T (new arrays of the kind of `phi`)."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn = getattr(lib(), "lsmgpu_advect_vjp_weno5_tvdrk3_" + precision)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 7 + [real] * 4 + [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6
    out = _zeros_like(phi)
    gphi = _zeros_like(phi)
    gv = [_zeros_like(v) for v in vel] if grad_vel else [None, None, None]
    rc = fn(_ptr(phi), _box(gb), _box(fb), _ptr(vel[0]), _ptr(vel[1]), _ptr(vel[2]), _box(vel_gb), dx, dy or dx,
            dz or dx, dt, int(n_steps), int(checkpoint_every), _ptr(grad_out), _ptr(out), _ptr(gphi),
            _ptr(gv[0]), _ptr(gv[1]), _ptr(gv[2]))
    if rc != 0:
        raise RuntimeError("lsmgpu advect vjp failed: %s" % (last_error()[1],))
    return out, gphi, gv


def reinit_vjp_weno5_tvdrk3(phi, gb, fb, grad_out, dx, dtau, n_iter, checkpoint_every=8, precision="f64",
                            dy=None, dz=None):
    """Vector-Jacobian product of n_iter periodic reinitialization iterations
    (phi0 sign form): returns (phi_T, grad_phi) for grad_out = dJ/dphi_T."""
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    fn = getattr(lib(), "lsmgpu_reinit_vjp_weno5_tvdrk3_" + precision)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 3 + [real] * 4 + [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3
    out = _zeros_like(phi)
    gphi = _zeros_like(phi) if grad_out is not None else None
    rc = fn(_ptr(phi), _box(gb), _box(fb), dx, dy or dx, dz or dx, dtau, int(n_iter), int(checkpoint_every),
            _ptr(grad_out), _ptr(out), _ptr(gphi))
    if rc != 0:
        raise RuntimeError("lsmgpu reinit vjp failed: %s" % (last_error()[1],))
    return out, gphi
