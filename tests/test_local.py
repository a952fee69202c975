"""Narrow-band (index-list) entry points, band construction and boundary
conditions: the C oracle against the reference's own (translated) kernels on
the CPU, and the GPU library against the oracle.

Bars: bit-for-bit for every array and integer output (index lists, level
bounds, marks, outer lists); the order-dependent average of
lsm3dcomputeavegradphilocal_ within 1e-12 relative.  Cases cover negative
lower bounds, four band levels, stale scratch contents, boundary-layer marks
and an empty band.
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

# the band (width 2 dx, 3 levels) and its stencils stay inside the ghost box,
# where LSMLIB's routines are well defined
GB = (-3, 22, -3, 20, -3, 20)
FB = (0, 19, 0, 17, 0, 17)
DX = 0.1
LEVEL = 3

LOCAL = [s for s in L.ABI if s.startswith("lsm3d") and any(a[0] == "index_x" for a in L.ABI[s]["args"])
         and s not in ("lsm3ddeterminenarrowband_", "lsm3dmarknarrowbandneighbors_",
                       "lsm3ddeterminenarrowbandfrommask_", "lsm3dcheckouternarrowbandlayer_",
                       # no 3D original: checked through their 2D forms (test_lifted.py)
                       "lsm3ddeterminenarrowbandfromtwolevelsets_", "lsm3ddeterminenarrowbandawayfrommask_")]
# LSMLIB's lsm3dComputeStableConstNormalVelDtLOCAL reads unassigned locals;
# the oracle implements the dense formula and is pinned against it below
REF_UNDEFINED = {"lsm3dcomputestableconstnormalveldtlocal_"}
BC = [s for s in L.ABI if s.startswith("lsm3d") and ("extrapolation" in s or "neumann" in s)]
NEW_3D = {"lsm3dhjeno3local_", "lsm3dhjweno5local_", "lsm3dupwindhjeno2local_"}


def band_phi(seed, gb=GB):
    phi = H.sphere_phi(gb, DX, center=(0.95, 0.85, 0.85), r=0.33, lo=0.0)
    rng = np.random.default_rng(seed)
    return np.asfortranarray(phi + 0.01 * rng.standard_normal(phi.shape))


def build_band(lib, phi, gb=GB, width=2.0 * DX, width_inner=1.0 * DX, level=LEVEL):
    """Run lsm3ddeterminenarrowband_ on `lib`; returns every output."""
    n = H.shape_of(gb)
    cap = int(np.prod(n))
    out = {
        "phi": phi, "narrow_band": np.zeros(n, dtype=np.uint8, order="F"),
        "index_x": np.full(cap, -99, np.int32), "index_y": np.full(cap, -99, np.int32),
        "index_z": np.full(cap, -99, np.int32), "nlo_index": 0, "nhi_index": cap - 1,
        "n_lo": np.full(level + 1, -7, np.int32), "n_hi": np.full(level + 1, -7, np.int32),
        "index_outer": np.full(cap, -99, np.int32), "nlo_index_outer": 0, "nhi_index_outer": cap - 1,
        "nlo_outer_plus": 0, "nhi_outer_plus": 0, "nlo_outer_minus": 0, "nhi_outer_minus": 0,
        "width": width, "width_inner": width_inner, "level": level,
    }
    for nm, v in zip(("ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb"), gb):
        out[nm] = v
    for nm, v in zip(("ilo_nb_gb", "ihi_nb_gb", "jlo_nb_gb", "jhi_nb_gb", "klo_nb_gb", "khi_nb_gb"), gb):
        out[nm] = v
    sc = L.invoke(lib, "lsm3ddeterminenarrowband_", out)
    out.update(sc)
    return out


def local_case(sym, seed=0):
    """Arguments for a *_local routine: a band built by the oracle, random
    fields, random (stale) scratch, level-0 gate for derivatives and a wider
    gate for pointwise routines."""
    rng = np.random.default_rng(seed)
    band = build_band(H.oracle(), band_phi(seed))
    n_lo, n_hi = band["n_lo"], band["n_hi"]
    # boundary-layer marks over part of the band, as the drivers add them
    nb = band["narrow_band"].copy(order="F")
    nb[rng.random(nb.shape) < 0.03] = 120
    arrays = {"index_x": band["index_x"], "index_y": band["index_y"], "index_z": band["index_z"],
              "narrow_band": nb}
    scalars = dict(H.DEFAULT_SCALARS)
    scalars.update({"nlo_index": int(n_lo[0]), "nhi_index": int(n_hi[LEVEL]),
                    "mark_fb": 2, "mark_d1": 4, "mark_d2": 4, "mark_d3": 4,
                    "beta": 1.5 * DX, "gamma": 3.0 * DX, "n": 2, "dir": 2,
                    "grad_phi_ave": -1.0, "max_norm_diff": -1.0, "dt": 0.01})
    for l in range(4):
        scalars["nlo_index%d" % l] = int(n_lo[l])
        scalars["nhi_index%d" % l] = int(n_hi[l])
    if any(a[0] == "nlo_index0" for a in L.ABI[sym]["args"]):
        scalars["mark_fb"] = 1      # derivatives on level-0 cells
        scalars["mark_d1"] = 4      # differences over levels 0..3
        scalars["mark_d2"] = 3
        scalars["mark_d3"] = 2
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        if not is_arr or name in arrays:
            continue
        if kind == "real":
            a = H.rough_field(rng, GB)
            if name.startswith("vel"):
                a[rng.random(a.shape) < 0.1] = 0.0
            if name == "grad_phi_mag":
                a = np.abs(a)
            arrays[name] = np.asfortranarray(a)
    vals, _ = H.make_call(sym, GB, FB, arrays=arrays, scalars=scalars)
    return vals


def compare(sym, a1, s1, a2, s2, rel=0.0):
    for name in H.written_names(sym):
        if name in a1:
            assert H.same(a1[name], a2[name]), "%s: %s differs" % (sym, name)
        elif rel:
            assert abs(s1[name] - s2[name]) <= rel * abs(s1[name]), (sym, name, s1[name], s2[name])
        else:
            assert H.same(s1[name], s2[name]), "%s: %s %r vs %r" % (sym, name, s1[name], s2[name])


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available")
    return r


# ---------------------------------------------------------------- CPU pins
@pytest.mark.parametrize("sym", [s for s in LOCAL if s not in REF_UNDEFINED and s not in NEW_3D])
@pytest.mark.parametrize("seed", [0, 1])
def test_local_oracle_matches_reference(sym, seed, ref):
    vals = local_case(sym, seed)
    a1, s1 = H.run(ref, sym, vals)
    a2, s2 = H.run(H.oracle(), sym, vals)
    compare(sym, a1, s1, a2, s2)


def test_const_normal_vel_dt_local_is_dense_formula_on_band():
    """The oracle's lsm3dcomputestableconstnormalveldtlocal_ (whose LSMLIB
    original reads unassigned variables) equals the dense routine restricted
    to the gated cells."""
    sym = "lsm3dcomputestableconstnormalveldtlocal_"
    vals = local_case(sym, 0)
    _, s = H.run(H.oracle(), sym, vals)
    ix, iy, iz = vals["index_x"], vals["index_y"], vals["index_z"]
    nb = vals["narrow_band"]
    best = -1.0
    mx = max(vals["dx"], vals["dy"], vals["dz"]) ** 2
    for l in range(vals["nlo_index"], vals["nhi_index"] + 1):
        c = (ix[l] - GB[0], iy[l] - GB[2], iz[l] - GB[4])
        if nb[c] > vals["mark_fb"]:
            continue
        cur = [max(abs(vals["phi_%s_plus" % d][c]), abs(vals["phi_%s_minus" % d][c])) for d in "xyz"]
        ng = np.sqrt(cur[0] * cur[0] + cur[1] * cur[1] + cur[2] * cur[2] + mx)
        h = abs(vals["vel_n"]) / ng * (cur[0] / vals["dx"] + cur[1] / vals["dy"] + cur[2] / vals["dz"])
        best = max(best, h)
    assert abs(s["dt"] - vals["cfl_number"] / (best + 1e-36)) <= 1e-12 * s["dt"]


def test_new_3d_local_weno5_matches_dense_on_band():
    """lsm3dhjweno5local_ (no 3D original) equals the dense lsm3dHJWENO5 on
    level-0 cells whose stencil lies in levels 0..3 (up to the local epsilon
    floor 1e-35 vs 1e-36, which only matters for |v| < 1e-15)."""
    sym = "lsm3dhjweno5local_"
    vals = local_case(sym, 0)
    a, _ = H.run(H.oracle(), sym, vals)
    dense = H.dense_case("lsm3dhjweno5_", seed=0, gb=GB, fb=FB)
    dense["phi"] = vals["phi"]
    for k in ("dx", "dy", "dz"):
        dense[k] = vals[k]
    b, _ = H.run(H.oracle(), "lsm3dhjweno5_", dense)
    ix, iy, iz, nb = vals["index_x"], vals["index_y"], vals["index_z"], vals["narrow_band"]
    checked = 0
    for l in range(vals["nlo_index0"], vals["nhi_index0"] + 1):
        i, j, k = ix[l], iy[l], iz[l]
        if not (FB[0] <= i <= FB[1] and FB[2] <= j <= FB[3] and FB[4] <= k <= FB[5]):
            continue
        c = (i - GB[0], j - GB[2], k - GB[4])
        if nb[c] > 1:
            continue
        ok = all(1 <= nb[c[0] + o * (d == 0), c[1] + o * (d == 1), c[2] + o * (d == 2)] <= 4
                 for d in range(3) for o in range(-3, 4)
                 if 0 <= c[0] + o * (d == 0) < nb.shape[0] and 0 <= c[1] + o * (d == 1) < nb.shape[1]
                 and 0 <= c[2] + o * (d == 2) < nb.shape[2])
        if not ok:
            continue
        for nm in ("phi_x_plus", "phi_y_minus", "phi_z_plus", "phi_x_minus"):
            assert abs(a[nm][c] - b[nm][c]) <= 1e-12 * max(1.0, abs(b[nm][c]))
        checked += 1
    assert checked > 50


# (list routine, dense routine, outputs, [(offsets along each axis, largest
# narrow_band value they may hold)]): where every such neighbour holds a
# computed difference, the list routine's result is the dense one's, bit for
# bit.  ENO3 reads D3 (levels 0-1) at c-1..c+2, which reads D2 (levels 0-2)
# at c-2..c+2, which reads D1 (levels 0-3) at c-2..c+3; upwind ENO2 reads D2
# (levels 0-1) at c-1..c+1 and D1 (levels 0-2) at c-1..c+2.
NEW_VS_DENSE = [
    ("lsm3dhjeno3local_", "lsm3dhjeno3_",
     ("phi_x_plus", "phi_y_minus", "phi_z_plus", "phi_x_minus", "phi_y_plus", "phi_z_minus"),
     [(range(-2, 4), 4), (range(-2, 3), 3), (range(-1, 3), 2)]),
    ("lsm3dupwindhjeno2local_", "lsm3dupwindhjeno2_", ("phi_x", "phi_y", "phi_z"),
     [(range(-1, 3), 3), (range(-1, 2), 2)]),
]


@pytest.mark.parametrize("sym,dense_sym,outs,reach", NEW_VS_DENSE)
def test_new_3d_local_matches_dense_on_band(sym, dense_sym, outs, reach):
    """3D list routines LSMLIB lacks (they follow its 2D list routines) equal
    LSMLIB's dense 3D routine on level-0 cells whose differences are all
    computed from phi."""
    vals = local_case(sym, 0)
    a, _ = H.run(H.oracle(), sym, vals)
    dense = H.dense_case(dense_sym, seed=0, gb=GB, fb=FB)
    for k in ("phi", "vel_x", "vel_y", "vel_z", "dx", "dy", "dz"):
        if k in dense and k in vals:
            dense[k] = vals[k]
    b, _ = H.run(H.oracle(), dense_sym, dense)
    ix, iy, iz, nb = vals["index_x"], vals["index_y"], vals["index_z"], vals["narrow_band"]
    checked = 0
    for l in range(vals["nlo_index0"], vals["nhi_index0"] + 1):
        i, j, k = ix[l], iy[l], iz[l]
        if not (FB[0] <= i <= FB[1] and FB[2] <= j <= FB[3] and FB[4] <= k <= FB[5]):
            continue
        c = (i - GB[0], j - GB[2], k - GB[4])
        if nb[c] > 1:
            continue
        ok = True
        for offs, top in reach:
            for d in range(3):
                for o in offs:
                    q = list(c)
                    q[d] += o
                    if not (0 <= q[d] < nb.shape[d]) or not (1 <= nb[tuple(q)] <= top):
                        ok = False
        if not ok:
            continue
        for nm in outs:
            assert H.same(a[nm][c], b[nm][c]), (sym, nm, c, a[nm][c], b[nm][c])
        checked += 1
    assert checked > 30, checked


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_band_construction_oracle_matches_reference(seed, ref):
    phi = band_phi(seed)
    a = build_band(ref, phi)
    b = build_band(H.oracle(), phi)
    for k in a:
        assert H.same(np.asarray(a[k]), np.asarray(b[k])), k


def test_empty_band_oracle_matches_reference(ref):
    phi = np.asfortranarray(np.full(H.shape_of(GB), 5.0))
    a = build_band(ref, phi)
    b = build_band(H.oracle(), phi)
    for k in ("n_lo", "n_hi", "nlo_outer_plus", "nhi_outer_plus", "nlo_outer_minus", "nhi_outer_minus"):
        if k in ("n_lo", "n_hi"):
            assert H.same(a[k][0], b[k][0]), k  # deeper levels are left unwritten
        else:
            assert a[k] == b[k], k
    assert H.same(a["narrow_band"], b["narrow_band"])


@pytest.mark.parametrize("sym", BC)
@pytest.mark.parametrize("face", range(6))
def test_bc_oracle_matches_reference(sym, face, ref):
    rng = np.random.default_rng(face)
    phi = np.asfortranarray(rng.standard_normal(H.shape_of(GB)))
    vals, _ = H.make_call(sym, GB, FB, arrays={"phi": phi}, scalars={"bdry_location_idx": face})
    a1, _ = H.run(ref, sym, vals)
    a2, _ = H.run(H.oracle(), sym, vals)
    assert H.same(a1["phi"], a2["phi"])


# ---------------------------------------------------------------- GPU parity
@pytest.mark.gpu
@pytest.mark.parametrize("sym", LOCAL)
@pytest.mark.parametrize("seed", [0, 1])
def test_local_gpu_matches_oracle(sym, seed, gpu_lib):
    vals = local_case(sym, seed)
    a1, s1 = H.run(H.oracle(), sym, vals)
    a2, s2 = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    compare(sym, a1, s1, a2, s2, rel=1e-12 if sym == "lsm3dcomputeavegradphilocal_" else 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("level", [0, 1, 3])
def test_band_construction_gpu_bit_exact(seed, level, gpu_lib):
    phi = band_phi(seed)
    a = build_band(H.oracle(), phi, level=level)
    b = build_band(gpu_lib, phi, level=level)
    L.check(gpu_lib)
    for k in a:
        assert H.same(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.gpu
def test_band_construction_gpu_empty_and_capacity(gpu_lib):
    phi = np.asfortranarray(np.full(H.shape_of(GB), 5.0))
    a = build_band(H.oracle(), phi)
    b = build_band(gpu_lib, phi)
    L.check(gpu_lib)
    assert a["n_hi"][0] == b["n_hi"][0] and a["nlo_outer_plus"] == b["nlo_outer_plus"]
    assert H.same(a["narrow_band"], b["narrow_band"])
    # index arrays too small: the GPU reports a capacity error and writes no list
    vals = build_band(H.oracle(), band_phi(0))
    small = dict(vals)
    small["nhi_index"] = 10
    small["narrow_band"] = np.zeros_like(vals["narrow_band"])
    L.invoke(gpu_lib, "lsm3ddeterminenarrowband_", small)
    assert L.last_error(gpu_lib)[0] == 4


@pytest.mark.gpu
@pytest.mark.parametrize("sym", BC)
@pytest.mark.parametrize("face", range(6))
def test_bc_gpu_matches_oracle(sym, face, gpu_lib):
    rng = np.random.default_rng(face)
    phi = np.asfortranarray(rng.standard_normal(H.shape_of(GB)))
    vals, _ = H.make_call(sym, GB, FB, arrays={"phi": phi}, scalars={"bdry_location_idx": face})
    a1, _ = H.run(H.oracle(), sym, vals)
    a2, _ = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    assert H.same(a1["phi"], a2["phi"])


@pytest.mark.gpu
def test_check_outer_layer_and_mask_band_gpu(gpu_lib):
    phi = band_phi(3)
    band = build_band(H.oracle(), phi)
    for flip in (False, True):
        p2 = phi.copy(order="F")
        if flip:
            p2 = -p2 + 0.05   # moves the zero level across the outer layer
        vals = dict(band)
        vals["phi"] = p2
        vals["change_sign"] = -1
        a = L.invoke(H.oracle(), "lsm3dcheckouternarrowbandlayer_", dict(vals))
        b = L.invoke(gpu_lib, "lsm3dcheckouternarrowbandlayer_", dict(vals))
        assert a["change_sign"] == b["change_sign"]
    n = H.shape_of(GB)
    cap = int(np.prod(n))
    for use_sign in (1, 0):
        outs = []
        for lib in (H.oracle(), gpu_lib):
            v = {"mask": phi, "narrow_band": np.zeros(n, np.uint8, order="F"),
                 "index_x": np.zeros(cap, np.int32), "index_y": np.zeros(cap, np.int32),
                 "index_z": np.zeros(cap, np.int32), "nlo_index": 0, "nhi_index": cap - 1,
                 "n_lo": np.zeros(LEVEL + 1, np.int32), "n_hi": np.zeros(LEVEL + 1, np.int32),
                 "level": LEVEL, "use_mask_sign": use_sign}
            for nm, val in zip(("ilo_mask_gb", "ihi_mask_gb", "jlo_mask_gb", "jhi_mask_gb", "klo_mask_gb",
                                "khi_mask_gb"), GB):
                v[nm] = val
            for nm, val in zip(("ilo_nb_gb", "ihi_nb_gb", "jlo_nb_gb", "jhi_nb_gb", "klo_nb_gb", "khi_nb_gb"), GB):
                v[nm] = val
            L.invoke(lib, "lsm3ddeterminenarrowbandfrommask_", v)
            outs.append(v)
        for k in ("narrow_band", "index_x", "index_y", "index_z", "n_lo", "n_hi"):
            assert H.same(outs[0][k], outs[1][k]), k
