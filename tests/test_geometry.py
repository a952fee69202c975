"""Geometry and integral reductions: volumes, areas, volume and surface
integrals, voxel counts, mean absolute difference, unit normals, mean
curvature (lsm_geometry3d_fort.f.in, lsm_math_utils3d.f.in) and the
control-volume variants of the max-norm and stable-dt reductions.

Oracle: the C restatement, pinned bit for bit against the reference's own
(translated) routines on seeded inputs for each control-volume sign and an
empty box.

GPU bars:
* bit-for-bit: voxel counts, unit and signed unit normals, the control-volume
  max-norm / dt reductions (maxima do not depend on order);
* sums: |gpu - oracle| <= (n + 16) * 2**-53 * S, with n the cells summed and
  S the sum of |term| — the serial sum's own rounding bound plus a few ulp per
  term for CUDA's sin / cos in the smoothing band;
* mean curvature: within 8 ulp of the oracle (the reference's
  norm_grad_phi_sq ** 1.5 is evaluated as s * sqrt(s));
and, at 128^3, size-independent properties: the volume inside plus outside is
the box volume, counts add up, the sphere's volume and area are close to
4/3 pi r^3 and 4 pi r^2, and repeated calls give identical bits.
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

U = 2.0 ** -53

# reductions that add floating-point terms (order dependent)
SUMS = ["lsm3daveabsdiff_", "lsm3dvolumeintegralphilessthanzero_", "lsm3dvolumeintegralphigreaterthanzero_",
        "lsm3dsurfaceintegral_", "lsm3dvolumeintegralphilessthanzerocontrolvolume_",
        "lsm3dvolumeintegralphigreaterthanzerocontrolvolume_", "lsm3dsurfaceintegralcontrolvolume_",
        "lsm3dvolumeregionphilessthanzero_", "lsm3dvolumeregionphigreaterthanzero_",
        "lsm3dsurfaceareazerolevelset_", "lsm3dsurfaceareazerolevelsetdelta_",
        "lsm3dvolumeregionphilessthanzerocontrolvolume_", "lsm3dvolumeregionphigreaterthanzerocontrolvolume_",
        "lsm3dsurfaceareazerolevelsetcontrolvolume_", "lsm3dsurfaceareazerolevelsetdeltacontrolvolume_"]
COUNTS = ["lsm3dvoxelcountgreaterthanzero_", "lsm3dvoxelcountlessthanzero_",
          "lsm3dvoxelcountgreaterthanzerocontrolvolume_", "lsm3dvoxelcountlessthanzerocontrolvolume_"]
CV_MAX = ["lsm3dmaxnormdiffcontrolvolume_", "lsm3dcomputestableadvectiondtcontrolvolume_",
          "lsm3dcomputestablenormalveldtcontrolvolume_", "lsm3dcomputestableconstnormalveldtcontrolvolume_"]
NORMALS = ["lsm3dcomputeunitnormal_", "lsm3dcomputesignedunitnormal_"]
KAPPA = "lsm3dcomputemeancurvature_"
# the dense parity test leaves these to this file (not bit-exact by design)
NOT_BIT_EXACT = set(SUMS) | {KAPPA}

IB = (1, 8, 0, 6, 2, 5)   # an index box strictly inside the fill box


def out_scalar(sym):
    return [a[0] for a in L.ABI[sym]["args"] if not a[2] and a[0] in
            ("ave_abs_diff", "count", "int_f", "volume", "area", "max_norm_diff", "dt")][0]


def has_cv(sym):
    return any(a[0] == "control_vol" for a in L.ABI[sym]["args"])


def case(sym, seed, sgn=1, ib=None, eps=0.45):
    sc = {"epsilon": eps}
    if has_cv(sym):
        sc["control_vol_sgn"] = sgn
    vals = H.dense_case(sym, seed=seed, scalars=sc)
    if ib is not None:
        for nm, v in zip(("ilo_ib", "ihi_ib", "jlo_ib", "jhi_ib", "klo_ib", "khi_ib"), ib):
            if nm in vals:
                vals[nm] = v
    return vals


def ib_of(vals):
    names = ("ilo_ib", "ihi_ib", "jlo_ib", "jhi_ib", "klo_ib", "khi_ib")
    if names[0] not in vals:
        names = ("ilo_fb", "ihi_fb", "jlo_fb", "jhi_fb", "klo_fb", "khi_fb")
    return tuple(vals[n] for n in names)


def abs_scale(lib, sym, vals):
    """Sum of |term| (for the mean absolute difference, the mean of them):
    the same routine with |F|, every other term being >= 0."""
    v = dict(vals)
    if "f" in v:
        v["f"] = np.abs(v["f"]).copy(order="F")
    return abs(H.run(lib, sym, v)[1][out_scalar(sym)])


def n_cells(vals):
    b = ib_of(vals)
    return int(np.prod([max(0, b[2 * d + 1] - b[2 * d] + 1) for d in range(3)]))


def assert_sum_close(sym, got, want, scale, n):
    tol = (n + 16) * U * scale
    assert abs(got - want) <= tol, "%s: %r vs %r (|diff| %g > %g)" % (sym, got, want, abs(got - want), tol)


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available (no reference tree or lsmref.c)")
    return r


# ---- the oracle against the reference (CPU) --------------------------------------------

@pytest.mark.parametrize("sym", SUMS + COUNTS + CV_MAX)
@pytest.mark.parametrize("sgn", [1, 0, -1])
def test_oracle_matches_reference_each_sign(sym, sgn, ref):
    if not has_cv(sym) and sgn != 1:
        pytest.skip("no control volume")
    for seed, ib in ((2, None), (3, IB)):
        vals = case(sym, seed, sgn=sgn, ib=ib)
        s_ref = H.run(ref, sym, vals)[1]
        s_or = H.run(H.oracle(), sym, vals)[1]
        k = out_scalar(sym)
        assert H.same(s_ref[k], s_or[k]), "%s sgn %d: %r vs %r" % (sym, sgn, s_ref[k], s_or[k])


@pytest.mark.parametrize("sym", SUMS + COUNTS)
def test_oracle_matches_reference_empty_box(sym, ref):
    vals = case(sym, 4, ib=(3, 2, 0, 6, 2, 5))
    k = out_scalar(sym)
    a = H.run(ref, sym, vals)[1][k]
    b = H.run(H.oracle(), sym, vals)[1][k]
    assert H.same(a, b) and a == 0


@pytest.mark.parametrize("eps", [0.05, 0.45, 3.0])
def test_oracle_matches_reference_epsilon(eps, ref):
    for sym in ("lsm3dvolumeregionphilessthanzero_", "lsm3dsurfaceareazerolevelset_", "lsm3dsurfaceintegral_"):
        vals = case(sym, 5, eps=eps)
        k = out_scalar(sym)
        assert H.same(H.run(ref, sym, vals)[1][k], H.run(H.oracle(), sym, vals)[1][k])


def test_oracle_volume_inside_plus_outside_is_box_volume():
    vals = case("lsm3dvolumeregionphilessthanzero_", 6)
    lt = H.run(H.oracle(), "lsm3dvolumeregionphilessthanzero_", vals)[1]["volume"]
    gt = H.run(H.oracle(), "lsm3dvolumeregionphigreaterthanzero_", vals)[1]["volume"]
    total = n_cells(vals) * vals["dx"] * vals["dy"] * vals["dz"]
    assert abs(lt + gt - total) <= 1e-12 * total


# ---- the GPU against the oracle ----------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("sym", SUMS)
@pytest.mark.parametrize("sgn", [1, -1])
@pytest.mark.parametrize("ib", [None, IB])
def test_gpu_sums_match_oracle(sym, sgn, ib, gpu_lib):
    if not has_cv(sym) and sgn != 1:
        pytest.skip("no control volume")
    vals = case(sym, 7, sgn=sgn, ib=ib)
    k = out_scalar(sym)
    want = H.run(H.oracle(), sym, vals)[1][k]
    got = H.run(gpu_lib, sym, vals)[1][k]
    L.check(gpu_lib)
    assert_sum_close(sym, got, want, abs_scale(H.oracle(), sym, vals), n_cells(vals))


@pytest.mark.gpu
@pytest.mark.parametrize("sym", COUNTS + CV_MAX)
@pytest.mark.parametrize("sgn", [1, 0, -1])
def test_gpu_counts_and_maxima_bit_exact(sym, sgn, gpu_lib):
    if not has_cv(sym) and sgn != 1:
        pytest.skip("no control volume")
    for seed, ib in ((8, None), (9, IB), (10, (3, 2, 0, 6, 2, 5))):
        vals = case(sym, seed, sgn=sgn, ib=ib)
        k = out_scalar(sym)
        want = H.run(H.oracle(), sym, vals)[1][k]
        got = H.run(gpu_lib, sym, vals)[1][k]
        L.check(gpu_lib)
        assert H.same(want, got), "%s sgn %d ib %s: %r vs %r" % (sym, sgn, ib, want, got)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", NORMALS)
@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_normals_bit_exact(sym, seed, gpu_lib):
    vals = H.dense_case(sym, seed=seed)
    # cells with a vanishing gradient or phi take the reference's fallbacks
    for nm in ("phi_x", "phi_y", "phi_z"):
        vals[nm][2:4, 1:3, 1] = 0.0
    if "phi" in vals:
        vals["phi"][5, 4, 2] = 0.0
    a = H.run(H.oracle(), sym, vals)[0]
    b = H.run(gpu_lib, sym, vals)[0]
    L.check(gpu_lib)
    for nm in ("normal_x", "normal_y", "normal_z"):
        assert H.same(a[nm], b[nm]), nm


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_mean_curvature_within_8_ulp(seed, gpu_lib):
    vals = H.dense_case(KAPPA, seed=seed)
    for nm in ("phi_x", "phi_y", "phi_z"):
        vals[nm][2:4, 1:3, 1] = 0.0
    a = H.run(H.oracle(), KAPPA, vals)[0]["kappa"]
    b = H.run(gpu_lib, KAPPA, vals)[0]["kappa"]
    L.check(gpu_lib)
    fin = np.isfinite(a)
    assert np.array_equal(fin, np.isfinite(b))
    assert np.all(np.abs(a[fin] - b[fin]) <= 8 * U * np.abs(a[fin])), np.max(np.abs(a[fin] - b[fin]))


def sphere_case(n, r=0.35, eps_cells=1.5):
    """Sphere signed distance on [-1, 1)^3 with n cells per axis and 3 ghost
    cells, its exact gradient, and a control volume split at x = 0."""
    dx = 2.0 / n
    gb = (-3, n + 2) * 3
    phi = H.sphere_phi(gb, dx, center=(0.05, -0.03, 0.02), r=r)
    i = np.arange(gb[0], gb[1] + 1)
    x = -1.0 + (i + 0.5) * dx
    X, Y, Z = np.meshgrid(x - 0.05, x + 0.03, x - 0.02, indexing="ij")
    d = np.sqrt(X * X + Y * Y + Z * Z)
    d[d == 0] = 1.0
    grads = [np.asfortranarray(c / d) for c in (X, Y, Z)]
    cv = np.asfortranarray(np.where(X + 0.05 < 0, 1.0, -1.0))
    return dict(gb=gb, ib=(0, n - 1) * 3, dx=dx, phi=phi, grads=grads, cv=cv, eps=eps_cells * dx, r=r)


def geo_vals(sym, c, sgn=1):
    arrays = {"phi": c["phi"], "delta_phi": c["phi"], "phi_x": c["grads"][0], "phi_y": c["grads"][1],
              "phi_z": c["grads"][2], "control_vol": c["cv"], "f": c["phi"] * 0.0 + 1.0,
              "field1": c["phi"], "field2": c["grads"][0]}
    names = {a[0] for a in L.ABI[sym]["args"] if a[2]}
    sc = {"dx": c["dx"], "dy": c["dx"], "dz": c["dx"], "epsilon": c["eps"], "control_vol_sgn": sgn,
          "volume": -7.0, "area": -7.0, "int_f": -7.0, "count": -7, "ave_abs_diff": -7.0}
    vals, _ = H.make_call(sym, c["gb"], c["ib"], arrays={k: v for k, v in arrays.items() if k in names},
                          scalars=sc, boxes={"ib": c["ib"]})
    return vals


@pytest.mark.gpu
def test_gpu_sphere_properties_128(gpu_lib):
    import torch
    c = sphere_case(128)
    dv = c["dx"] ** 3
    run = lambda sym, sgn=1: L.invoke(gpu_lib, sym, geo_vals(sym, c, sgn))[out_scalar(sym)]
    lt = run("lsm3dvolumeregionphilessthanzero_")
    gt = run("lsm3dvolumeregionphigreaterthanzero_")
    L.check(gpu_lib)
    total = 128 ** 3 * dv
    assert abs(lt + gt - total) <= 1e-12 * total
    r = c["r"]
    # the smoothed Heaviside biases the volume by O((eps / r)^2), 1.8e-3 here
    assert abs(lt - 4.0 / 3.0 * np.pi * r ** 3) <= 5e-3 * lt
    area = run("lsm3dsurfaceareazerolevelset_")
    assert abs(area - 4.0 * np.pi * r ** 2) <= 3e-3 * area
    # the integral of 1 over {phi < 0} is the volume
    assert abs(run("lsm3dvolumeintegralphilessthanzero_") - lt) <= 1e-12 * lt
    # control volume split in two halves: the halves add to the whole
    halves = run("lsm3dvolumeregionphilessthanzerocontrolvolume_", 1) + \
        run("lsm3dvolumeregionphilessthanzerocontrolvolume_", -1)
    assert abs(halves - lt) <= 1e-12 * lt
    cg = run("lsm3dvoxelcountgreaterthanzero_")
    cl = run("lsm3dvoxelcountlessthanzero_")
    assert cg + cl == 128 ** 3 - int(np.count_nonzero(c["phi"][3:-3, 3:-3, 3:-3] == 0.0))
    assert cl == int(np.count_nonzero(c["phi"][3:-3, 3:-3, 3:-3] < 0.0))
    # identical bits on repeat, and through device arrays
    assert H.same(run("lsm3dsurfaceareazerolevelset_"), area)
    v = geo_vals("lsm3dsurfaceareazerolevelset_", c)
    dev = {k: (torch.from_numpy(np.ascontiguousarray(a.T)).cuda() if isinstance(a, np.ndarray) else a)
           for k, a in v.items()}
    assert H.same(L.invoke(gpu_lib, "lsm3dsurfaceareazerolevelset_", dev)["area"], area)
    # against the oracle at full size
    for sym in ("lsm3dvolumeregionphilessthanzero_", "lsm3dsurfaceareazerolevelset_"):
        vals = geo_vals(sym, c)
        want = H.run(H.oracle(), sym, vals)[1][out_scalar(sym)]
        assert_sum_close(sym, run(sym), want, abs(want), 128 ** 3)


@pytest.mark.gpu
@pytest.mark.parametrize("eps", [0.0, -0.3, 0.05, 3.0])
def test_gpu_sums_any_epsilon(eps, gpu_lib):
    """Positive finite epsilons classify cells on bit patterns; zero and
    negative ones take the reference's comparisons as written."""
    for sym in ("lsm3dvolumeregionphilessthanzero_", "lsm3dvolumeregionphigreaterthanzero_",
                "lsm3dvolumeintegralphilessthanzero_", "lsm3dsurfaceareazerolevelset_"):
        vals = case(sym, 11, eps=eps)
        k = out_scalar(sym)
        want = H.run(H.oracle(), sym, vals)[1][k]
        got = H.run(gpu_lib, sym, vals)[1][k]
        L.check(gpu_lib)
        if not np.isfinite(want):
            assert H.same(want, got), "%s eps %g: %r vs %r" % (sym, eps, want, got)
            continue
        assert_sum_close(sym, got, want, abs_scale(H.oracle(), sym, vals), n_cells(vals))
