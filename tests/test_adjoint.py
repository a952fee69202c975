"""Adjoint of periodic WENO5 / TVD-RK3 advection (no LSMLIB counterpart).

CPU: the smoothed Heaviside / delta of the objective against LSMLIB's own
known-answer vectors (tests/toolbox/test_calculus_toolbox.cc, fixture in
tests/golden/); the FP64 CPU reverse-mode oracle's forward map against the
oracle's LSMLIB call sequence (bit-exact) and its gradient against central
finite differences.
GPU: the FP64 adjoint against the oracle's gradient; checkpoint spacing
changes nothing; FP32 against FP64; central finite differences (h = 1e-3,
FP64 forward) along random unit directions, the objective of the 192^3
workload built at 64^3; device-pointer calls; the torch.autograd.Function
wrapper; argument errors.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "calculus_toolbox_kat.json")


def _oracle_fn():
    lib = H.oracle()
    f = lib.oracle_advect_objective_adjoint
    f.restype = ctypes.c_double
    P = ctypes.c_void_p
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int, ctypes.c_double] + [P] * 10
    return f


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def oracle_adjoint(phi, vel, tgt, spacing, dt, steps, eps, grads=True):
    """(J, phi_T, grad_phi, grad_vel) of the CPU oracle on compact periodic
    arrays (Fortran order)."""
    f = _oracle_fn()
    phi = np.asfortranarray(phi, dtype=np.float64)
    vel = [np.asfortranarray(v, dtype=np.float64) for v in vel]
    tgt = np.asfortranarray(tgt, dtype=np.float64)
    nx, ny, nz = phi.shape
    fin = np.zeros_like(phi, order="F")
    gp = np.zeros_like(phi, order="F") if grads else None
    gv = [np.zeros_like(phi, order="F") for _ in range(3)] if grads else [None] * 3
    J = f(nx, ny, nz, *[float(s) for s in spacing], float(dt), int(steps), float(eps), _p(phi),
          *[_p(v) for v in vel], _p(tgt), _p(fin), _p(gp), *[_p(g) for g in gv])
    return J, fin, gp, gv


def adjoint_case(dims, seed=3, noise=0.05, shift=0.1, r=0.4):
    """The config-5 problem on (nx, ny, nz) cells of [-1, 1]^3 (periodic):
    sphere of radius r, target shifted by `shift` in x, velocity
    (sin(pi y) cos(pi z), sin(pi z) cos(pi x), sin(pi x) cos(pi y)) plus
    N(0, noise) per cell, dt at CFL 0.5.  Returns compact interior arrays."""
    sp = tuple(2.0 / n for n in dims)
    c = [-1.0 + (np.arange(n) + 0.5) * h for n, h in zip(dims, sp)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    phi = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - r
    tgt = np.sqrt((X - shift) ** 2 + Y ** 2 + Z ** 2) - r
    rng = np.random.default_rng(seed)
    base = (np.sin(np.pi * Y) * np.cos(np.pi * Z), np.sin(np.pi * Z) * np.cos(np.pi * X),
            np.sin(np.pi * X) * np.cos(np.pi * Y))
    vel = [b + rng.normal(0.0, noise, X.shape) for b in base]
    dt = 0.5 / max(np.max(np.abs(vel[0]) / sp[0] + np.abs(vel[1]) / sp[1] + np.abs(vel[2]) / sp[2]), 1e-30)
    f = lambda a: np.asfortranarray(a)
    return f(phi), [f(v) for v in vel], f(tgt), sp, dt


def ghosted(a, real=np.float64):
    """Compact interior -> array over the ghost box (3 ghost cells, zeros)."""
    out = np.zeros(tuple(n + 6 for n in a.shape), dtype=real, order="F")
    out[3:-3, 3:-3, 3:-3] = a
    return out


def boxes(dims):
    nx, ny, nz = dims
    return (-3, nx + 2, -3, ny + 2, -3, nz + 2), (0, nx - 1, 0, ny - 1, 0, nz - 1)


def gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, precision="f64", ckpt=8, grads=True):
    real = np.float64 if precision == "f64" else np.float32
    gb, fb = boxes(phi.shape)
    P, V, T = ghosted(phi, real), [ghosted(v, real) for v in vel], ghosted(tgt, real)
    J, gp, gv = L.advect_adjoint_weno5_tvdrk3(P, gb, fb, V, gb, T, sp[0], dt, steps, eps, checkpoint_every=ckpt,
                                              precision=precision, dy=sp[1], dz=sp[2], grads=grads)
    if not grads:
        return J, None, None
    inner = (slice(3, -3),) * 3
    return J, gp[inner].astype(np.float64), [g[inner].astype(np.float64) for g in gv]


def unit(rng, shape, k=1):
    d = [rng.standard_normal(shape) for _ in range(k)]
    n = np.sqrt(sum(np.sum(x * x) for x in d))
    return [np.asfortranarray(x / n) for x in d]


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------
def test_heaviside_and_delta_known_answers():
    kat = json.load(open(GOLDEN))
    lib = H.oracle()
    for name in ("oracle_heaviside", "oracle_delta"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = [ctypes.c_double, ctypes.c_double]
    d_phi = kat["d_phi"]
    eps = kat["eps_over_d_phi"] * d_phi
    for i in range(20):
        x = -1.0 + i * d_phi
        h = lib.oracle_heaviside(x, eps)
        d = lib.oracle_delta(x, eps)
        assert abs(h - kat["heaviside"][i]) <= kat["tolerance"]
        assert abs(d - kat["delta"][i]) <= kat["tolerance"]
        # the fixture is printed to 15 digits; the formulas agree to that
        assert abs(h - kat["heaviside"][i]) <= 2e-15
        assert abs(d - kat["delta"][i]) <= 5e-15 * max(1.0, abs(d))


def test_oracle_adjoint_forward_is_the_lsmlib_sequence():
    dims = (12, 10, 14)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    J, fin, _, _ = oracle_adjoint(phi, vel, tgt, sp, dt, 3, 1.5 * sp[0], grads=False)
    gb, fb = boxes(dims)
    g = ghosted(phi)
    O.periodic_fill(g, gb, fb)
    want = O.tvdrk3_run(H.oracle(), "advect", g, gb, fb, sp, dt, 3, L.BC_PERIODIC,
                        vel=[O_periodic(v, gb, fb) for v in vel])
    assert H.same(fin, want[3:-3, 3:-3, 3:-3])


def O_periodic(v, gb, fb):
    g = ghosted(v)
    O.periodic_fill(g, gb, fb)
    return g


def test_oracle_adjoint_matches_finite_differences():
    dims = (12, 10, 14)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    steps = 4
    J, _, gp, gv = oracle_adjoint(phi, vel, tgt, sp, dt, steps, eps)
    Jof = lambda p, v: oracle_adjoint(p, v, tgt, sp, dt, steps, eps, grads=False)[0]
    rng = np.random.default_rng(7)
    h = 1e-5
    for _ in range(4):
        (d,) = unit(rng, dims)
        fd = (Jof(phi + h * d, vel) - Jof(phi - h * d, vel)) / (2 * h)
        an = np.sum(gp * d)
        assert abs(fd - an) <= 1e-5 * abs(fd), (fd, an)
        dv = unit(rng, dims, 3)
        fd = (Jof(phi, [v + h * e for v, e in zip(vel, dv)]) - Jof(phi, [v - h * e for v, e in zip(vel, dv)])) / (2 * h)
        an = sum(np.sum(g * e) for g, e in zip(gv, dv))
        assert abs(fd - an) <= 1e-5 * abs(fd), (fd, an)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("dims,steps,ckpt", [((20, 18, 16), 7, 3), ((16, 16, 16), 4, 8), ((40, 9, 33), 2, 1),
                                             ((264, 7, 6), 2, 1)])
def test_adjoint_f64_matches_oracle(dims, steps, ckpt, gpu_lib):
    """(264, 7, 6): rows longer than one CTA takes, the segmented x kernel."""
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    Jw, _, gw, gvw = oracle_adjoint(phi, vel, tgt, sp, dt, steps, eps)
    J, gp, gv = gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, "f64", ckpt)
    assert abs(J - Jw) <= 1e-13 * abs(Jw)
    assert rel(gp, gw) <= 1e-11
    for a, b in zip(gv, gvw):
        assert rel(a, b) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_adjoint_checkpoint_spacing_changes_nothing(precision, gpu_lib):
    phi, vel, tgt, sp, dt = adjoint_case((24, 20, 18))
    eps = 1.5 * sp[0]
    base = gpu_adjoint(phi, vel, tgt, sp, dt, 9, eps, precision, ckpt=9)
    for ckpt in (1, 2, 4, 100, 0):   # 0: the library picks the spacing
        J, gp, gv = gpu_adjoint(phi, vel, tgt, sp, dt, 9, eps, precision, ckpt=ckpt)
        assert J == base[0]
        assert np.array_equal(gp, base[1])
        for a, b in zip(gv, base[2]):
            assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(24, 20, 18), (37, 19, 21), (33, 7, 13), (264, 7, 9)])
def test_adjoint_f32_against_fp64_oracle(dims, gpu_lib):
    """Odd ny / nz: the last line pair of the two-line FP32 kernels has one
    line; nx not a multiple of 32: idle lanes; nz not a multiple of the x
    kernel's 8-plane chunks; nx = 264: rows longer than one CTA takes (the
    scalar kernels)."""
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    Jw, _, gw, gvw = oracle_adjoint(phi, vel, tgt, sp, dt, 6, eps)
    J, gp, gv = gpu_adjoint(phi, vel, tgt, sp, dt, 6, eps, "f32", 4)
    assert abs(J - Jw) <= 1e-5 * abs(Jw)
    assert np.linalg.norm(gp - gw) <= 1e-4 * np.linalg.norm(gw)
    for a, b in zip(gv, gvw):
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b)


def smooth_unit(rng, dims, k=1):
    """Random smooth unit directions: each component a product of random
    low-wavenumber sinusoids on [-1, 1]^3, normalised jointly."""
    c = [-1.0 + (np.arange(n) + 0.5) * 2.0 / n for n in dims]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    d = []
    for _ in range(k):
        a = rng.uniform(-2, 2, 3)
        b = rng.uniform(-2, 2, 3)
        ph = rng.uniform(0, 2 * np.pi, 2)
        d.append(np.sin(np.pi * (a[0] * X + a[1] * Y + a[2] * Z) + ph[0]) *
                 np.cos(np.pi * (b[0] * X + b[1] * Y + b[2] * Z) + ph[1]))
    n = np.sqrt(sum(np.sum(x * x) for x in d))
    return [np.asfortranarray(x / n) for x in d]


@pytest.mark.gpu
def test_adjoint_matches_central_differences_64(gpu_lib):
    """The config-5 objective at 64^3 (40 steps, checkpoint every 8): FP32
    and FP64 gradients against FP64 central differences along random unit
    directions in phi and in the velocity fields, within 1e-4 relative (FP32
    on white-noise directions: 3e-4).
    Smooth directions: h = 1e-3.  White-noise directions perturb every cell
    independently, where the WENO weights are strongly nonlinear and the
    h = 1e-3 difference itself carries an O(h^2) truncation error near 1e-3;
    for those the difference is Richardson-extrapolated from h = 1e-3 and
    5e-4 (error O(h^4))."""
    n = 64
    phi, vel, tgt, sp, dt = adjoint_case((n, n, n))
    eps = 1.5 * sp[0]
    steps = 40
    _, g64, gv64 = gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, "f64", 8)
    _, g32, gv32 = gpu_adjoint(phi, vel, tgt, sp, dt, steps, eps, "f32", 8)
    Jof = lambda p, v: gpu_adjoint(p, v, tgt, sp, dt, steps, eps, "f64", grads=False)[0]
    cd_phi = lambda d, h: (Jof(phi + h * d, vel) - Jof(phi - h * d, vel)) / (2 * h)
    cd_vel = lambda dv, h: (Jof(phi, [v + h * e for v, e in zip(vel, dv)]) -
                            Jof(phi, [v - h * e for v, e in zip(vel, dv)])) / (2 * h)
    rng = np.random.default_rng(11)
    h = 1e-3
    for kind in ("smooth", "white"):
        for _ in range(2):
            if kind == "smooth":
                (d,) = smooth_unit(rng, phi.shape)
                dv = smooth_unit(rng, phi.shape, 3)
                fd, fdv = cd_phi(d, h), cd_vel(dv, h)
            else:
                (d,) = unit(rng, phi.shape)
                dv = unit(rng, phi.shape, 3)
                fd = (4 * cd_phi(d, h / 2) - cd_phi(d, h)) / 3
                fdv = (4 * cd_vel(dv, h / 2) - cd_vel(dv, h)) / 3
            # FP32 state: within 1e-4 on smooth directions; white-noise
            # directions weigh the gradient's cell-scale content, where FP32
            # rounding of the recomputed states shows (measured up to 1.1e-4)
            tol32 = 1e-4 if kind == "smooth" else 3e-4
            for g, tol in ((g64, 1e-4), (g32, tol32)):
                assert abs(np.sum(g * d) - fd) <= tol * abs(fd), (kind, np.sum(g * d), fd)
            for gv, tol in ((gv64, 1e-4), (gv32, tol32)):
                an = sum(np.sum(a * e) for a, e in zip(gv, dv))
                assert abs(an - fdv) <= tol * abs(fdv), (kind, an, fdv)


@pytest.mark.gpu
def test_adjoint_device_pointers_match_host(gpu_lib):
    import torch
    dims = (20, 18, 16)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    J, gp, gv = gpu_adjoint(phi, vel, tgt, sp, dt, 5, eps, "f32", 2)
    gb, fb = boxes(dims)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(ghosted(a, np.float32).T)).cuda()
    Jd, gpd, gvd = L.advect_adjoint_weno5_tvdrk3(dev(phi), gb, fb, [dev(v) for v in vel], gb, dev(tgt), sp[0], dt,
                                                 5, eps, checkpoint_every=2, precision="f32", dy=sp[1], dz=sp[2])
    torch.cuda.synchronize()
    inner = (slice(3, -3),) * 3
    assert Jd == J
    assert np.array_equal(gpd.cpu().numpy().T[inner].astype(np.float64), gp)
    for a, b in zip(gvd, gv):
        assert np.array_equal(a.cpu().numpy().T[inner].astype(np.float64), b)


@pytest.mark.gpu
def test_adjoint_autograd_function(gpu_lib):
    import torch
    from tests.adjoint_autograd import AdvectObjective
    dims = (16, 16, 16)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    J, gp, gv = gpu_adjoint(phi, vel, tgt, sp, dt, 3, eps, "f64", 2)
    p = torch.tensor(phi, dtype=torch.float64, device="cuda", requires_grad=True)
    v = [torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True) for x in vel]
    t = torch.tensor(tgt, dtype=torch.float64, device="cuda")
    Jt = AdvectObjective.apply(p, v[0], v[1], v[2], t, sp, dt, 3, eps, 2)
    Jt.backward()
    assert float(Jt.detach()) == J
    assert np.array_equal(p.grad.cpu().numpy(), gp)
    for a, b in zip(v, gv):
        assert np.array_equal(a.grad.cpu().numpy(), b)


@pytest.mark.gpu
def test_adjoint_argument_errors(gpu_lib):
    phi, vel, tgt, sp, dt = adjoint_case((12, 12, 12))
    gb, fb = boxes(phi.shape)
    P, V, T = ghosted(phi), [ghosted(v) for v in vel], ghosted(tgt)
    with pytest.raises(RuntimeError, match="checkpoint_every"):
        L.advect_adjoint_weno5_tvdrk3(P, gb, fb, V, gb, T, sp[0], dt, 3, 0.1, checkpoint_every=-1)
    with pytest.raises(RuntimeError, match="6 cells"):
        L.advect_adjoint_weno5_tvdrk3(P, gb, (0, 4, 0, 11, 0, 11), V, gb, T, sp[0], dt, 3, 0.1)
    with pytest.raises(RuntimeError, match="3 ghost cells"):
        L.advect_adjoint_weno5_tvdrk3(P, (0, 17, -3, 14, -3, 14), fb, V, gb, T, sp[0], dt, 3, 0.1)


# ---------------------------------------------------------------------------
# vector-Jacobian products (advection and reinitialization), CPU oracle
# ---------------------------------------------------------------------------
def _vjp_fns():
    lib = H.oracle()
    P = ctypes.c_void_p
    fa = lib.oracle_advect_vjp
    fa.restype = None
    fa.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int] + [P] * 9
    fr = lib.oracle_reinit_vjp
    fr.restype = None
    fr.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 4 + [ctypes.c_int] + [P] * 4
    return fa, fr


def oracle_advect_vjp(phi, vel, gout, sp, dt, steps, grads=True):
    fa, _ = _vjp_fns()
    phi = np.asfortranarray(phi, dtype=np.float64)
    vel = [np.asfortranarray(v, dtype=np.float64) for v in vel]
    gout = np.asfortranarray(gout, dtype=np.float64)
    fin = np.zeros_like(phi, order="F")
    gp = np.zeros_like(phi, order="F")
    gv = [np.zeros_like(phi, order="F") for _ in range(3)]
    fa(*phi.shape, *[float(x) for x in sp], float(dt), int(steps), _p(phi), *[_p(v) for v in vel], _p(gout),
       _p(fin), _p(gp), *[_p(g) for g in gv])
    return fin, gp, gv


def oracle_reinit_vjp(phi, gout, sp, dtau, steps):
    _, fr = _vjp_fns()
    phi = np.asfortranarray(phi, dtype=np.float64)
    gout = np.asfortranarray(gout, dtype=np.float64)
    fin = np.zeros_like(phi, order="F")
    gp = np.zeros_like(phi, order="F")
    fr(*phi.shape, *[float(x) for x in sp], float(dtau), int(steps), _p(phi), _p(gout), _p(fin), _p(gp))
    return fin, gp


def reinit_case(dims, seed=5):
    """A non-distance level set (the reinitialization workload's form) on
    (nx, ny, nz) cells of [-1, 1]^3 with a smooth random perturbation."""
    sp = tuple(2.0 / n for n in dims)
    c = [-1.0 + (np.arange(n) + 0.5) * h for n, h in zip(dims, sp)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    phi = (r - 0.5) * (0.1 + (X - 0.3) ** 2 + (Y - 0.3) ** 2 + (Z + 0.2) ** 2)
    return np.asfortranarray(phi), sp, 0.5 * min(sp)


def test_oracle_reinit_forward_is_the_lsmlib_sequence():
    dims = (12, 10, 14)
    phi, sp, dtau = reinit_case(dims)
    fin, _ = oracle_reinit_vjp(phi, np.zeros(dims), sp, dtau, 3)
    gb, fb = boxes(dims)
    g = ghosted(phi)
    O.periodic_fill(g, gb, fb)
    want = O.tvdrk3_run(H.oracle(), "reinit", g, gb, fb, sp, dtau, 3, L.BC_PERIODIC, use0=1)
    assert H.same(fin, want[3:-3, 3:-3, 3:-3])


def test_oracle_advect_vjp_matches_objective_gradient():
    """The VJP with grad_out = dJ/dphi_T reproduces the objective gradient."""
    dims = (12, 10, 14)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    J, fin, gp, gv = oracle_adjoint(phi, vel, tgt, sp, dt, 3, eps)
    lib = H.oracle()
    for name in ("oracle_heaviside", "oracle_delta"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = [ctypes.c_double, ctypes.c_double]
    vol = sp[0] * sp[1] * sp[2]
    hv = np.vectorize(lambda x: lib.oracle_heaviside(x, eps))
    dl = np.vectorize(lambda x: lib.oracle_delta(x, eps))
    lam = np.asfortranarray(2.0 * (hv(fin) - hv(tgt)) * dl(fin) * vol)
    _, gp2, gv2 = oracle_advect_vjp(phi, vel, lam, sp, dt, 3)
    assert rel(gp2, gp) <= 1e-14
    for a, b in zip(gv2, gv):
        assert rel(a, b) <= 1e-14


def test_oracle_reinit_vjp_matches_finite_differences():
    dims = (12, 10, 14)
    phi, sp, dtau = reinit_case(dims)
    steps = 3
    rng = np.random.default_rng(9)
    gout = np.asfortranarray(rng.standard_normal(dims))
    _, gp = oracle_reinit_vjp(phi, gout, sp, dtau, steps)
    F = lambda p: float(np.sum(gout * oracle_reinit_vjp(p, np.zeros(dims), sp, dtau, steps)[0]))
    h = 1e-6
    for _ in range(4):
        (d,) = smooth_unit(rng, dims)
        fd = (F(phi + h * d) - F(phi - h * d)) / (2 * h)
        an = float(np.sum(gp * d))
        assert abs(fd - an) <= 1e-6 * max(abs(fd), 1e-3 * np.linalg.norm(gp)), (fd, an)


def gpu_reinit_vjp(phi, gout, sp, dtau, steps, precision="f64", ckpt=8):
    real = np.float64 if precision == "f64" else np.float32
    gb, fb = boxes(phi.shape)
    out, gp = L.reinit_vjp_weno5_tvdrk3(ghosted(phi, real), gb, fb, None if gout is None else ghosted(gout, real),
                                        sp[0], dtau, steps, checkpoint_every=ckpt, precision=precision,
                                        dy=sp[1], dz=sp[2])
    inner = (slice(3, -3),) * 3
    return out[inner].astype(np.float64), None if gp is None else gp[inner].astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,steps,ckpt", [((20, 18, 16), 5, 2), ((16, 16, 16), 3, 8)])
def test_reinit_vjp_f64_matches_oracle(dims, steps, ckpt, gpu_lib):
    phi, sp, dtau = reinit_case(dims)
    rng = np.random.default_rng(21)
    gout = np.asfortranarray(rng.standard_normal(dims))
    fin_w, gw = oracle_reinit_vjp(phi, gout, sp, dtau, steps)
    fin, gp = gpu_reinit_vjp(phi, gout, sp, dtau, steps, "f64", ckpt)
    assert H.same(fin, fin_w)
    assert rel(gp, gw) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(24, 20, 18), (35, 17, 11)])
def test_reinit_vjp_f32_against_fp64_oracle(dims, gpu_lib):
    phi, sp, dtau = reinit_case(dims)
    rng = np.random.default_rng(22)
    gout = np.asfortranarray(rng.standard_normal(dims))
    fin_w, gw = oracle_reinit_vjp(phi, gout, sp, dtau, 4)
    fin, gp = gpu_reinit_vjp(phi, gout, sp, dtau, 4, "f32", 2)
    assert np.max(np.abs(fin - fin_w)) <= 1e-5
    assert np.linalg.norm(gp - gw) <= 1e-3 * np.linalg.norm(gw), np.linalg.norm(gp - gw) / np.linalg.norm(gw)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_reinit_vjp_checkpoint_spacing_changes_nothing(precision, gpu_lib):
    dims = (20, 18, 16)
    phi, sp, dtau = reinit_case(dims)
    gout = np.asfortranarray(np.random.default_rng(23).standard_normal(dims))
    base = gpu_reinit_vjp(phi, gout, sp, dtau, 7, precision, 7)
    for ckpt in (1, 3, 50, 0):
        fin, gp = gpu_reinit_vjp(phi, gout, sp, dtau, 7, precision, ckpt)
        assert np.array_equal(fin, base[0]) and np.array_equal(gp, base[1])


@pytest.mark.gpu
def test_reinit_vjp_matches_central_differences(gpu_lib):
    """20 reinitialization iterations at 48^3 (the headline workload's field
    and dtau = 0.5 dx): FP64 and FP32 VJPs against FP64 central differences
    of <grad_out, phi_T> along smooth random unit directions.  The Godunov
    and sign maxima make the map piecewise smooth, so the step is h = 1e-5:
    measured, the differences converge to the FP64 VJP (relative error 7e-5 to
    8e-4 at h = 1e-3, 6e-6 to 3e-5 at 1e-4, 3e-8 to 2e-7 at 1e-5) as steps
    stop crossing switching points.  FP32 carries its own rounding (up to 2e-4
    relative on these directions)."""
    n = 48
    phi, sp, dtau = reinit_case((n, n, n))
    rng = np.random.default_rng(24)
    gout = np.asfortranarray(rng.standard_normal(phi.shape))
    _, g64 = gpu_reinit_vjp(phi, gout, sp, dtau, 20, "f64", 8)
    _, g32 = gpu_reinit_vjp(phi, gout, sp, dtau, 20, "f32", 8)
    F = lambda p: float(np.sum(gout * gpu_reinit_vjp(p, None, sp, dtau, 20, "f64")[0]))
    h = 1e-5
    for _ in range(3):
        (d,) = smooth_unit(rng, phi.shape)
        fd = (F(phi + h * d) - F(phi - h * d)) / (2 * h)
        assert abs(np.sum(g64 * d) - fd) <= 1e-6 * abs(fd), (np.sum(g64 * d), fd)
        assert abs(np.sum(g32 * d) - fd) <= 1e-3 * abs(fd), (np.sum(g32 * d), fd)


@pytest.mark.gpu
def test_advect_vjp_matches_objective_gradient(gpu_lib):
    dims = (20, 18, 16)
    phi, vel, tgt, sp, dt = adjoint_case(dims)
    eps = 1.5 * sp[0]
    J, fin, gw, gvw = oracle_adjoint(phi, vel, tgt, sp, dt, 5, eps)
    lib = H.oracle()
    for name in ("oracle_heaviside", "oracle_delta"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = [ctypes.c_double, ctypes.c_double]
    vol = sp[0] * sp[1] * sp[2]
    hv = np.vectorize(lambda x: lib.oracle_heaviside(x, eps))
    dl = np.vectorize(lambda x: lib.oracle_delta(x, eps))
    lam = np.asfortranarray(2.0 * (hv(fin) - hv(tgt)) * dl(fin) * vol)
    gb, fb = boxes(dims)
    out, gp, gv = L.advect_vjp_weno5_tvdrk3(ghosted(phi), gb, fb, [ghosted(v) for v in vel], gb, ghosted(lam),
                                            sp[0], dt, 5, checkpoint_every=2, dy=sp[1], dz=sp[2])
    inner = (slice(3, -3),) * 3
    assert H.same(out[inner], fin)
    assert rel(gp[inner], gw) <= 1e-11
    for a, b in zip(gv, gvw):
        assert rel(a[inner], b) <= 1e-11


@pytest.mark.gpu
def test_reinit_autograd_function(gpu_lib):
    import torch
    from tests.adjoint_autograd import Reinit
    dims = (16, 16, 16)
    phi, sp, dtau = reinit_case(dims)
    w = np.asfortranarray(np.random.default_rng(25).standard_normal(dims))
    fin, gp = gpu_reinit_vjp(phi, w, sp, dtau, 4, "f64", 2)
    p = torch.tensor(phi, dtype=torch.float64, device="cuda", requires_grad=True)
    out = Reinit.apply(p, sp, dtau, 4, 2)
    loss = (out * torch.tensor(w, dtype=torch.float64, device="cuda")).sum()
    loss.backward()
    assert np.array_equal(out.detach().cpu().numpy(), fin)
    assert np.array_equal(p.grad.cpu().numpy(), gp)
