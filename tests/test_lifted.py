"""LSMLIB's 2D and 1D routines (include/lsmgpu_toolbox2d.h, _1d.h), which run
the 3D kernels with the missing axes lifted (stride 0, see csrc/lift.cuh).

CPU: the principle, on the oracle — the 3D routine applied to data copied
along the missing axes returns, on the middle plane, exactly what the
reference's own 2D / 1D routine returns (its mechanical translation,
oracle/_ref).  GPU: every lifted entry point against the reference's 2D / 1D
routine on seeded inputs — bit for bit; sums (volumes, integrals, the band
average) within (n + 16) 2^-53 S, S the sum of |term|, as in test_geometry.
"""
import re

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H
from tests.test_geometry import SUMS

LIFTED = sorted(s for s, v in L.ABI.items() if "lifted_from" in v)
# reference routines that cannot be called through their C declaration
# (lsm2dHJENO3LOCAL leaves index_x / index_y out of its Fortran argument list):
# checked against the oracle's 3D routine on one-cell-thick arrays instead
REF_UNUSABLE = [s for s in LIFTED if L.ABI[s].get("ref_unusable")]
DIMS = {s: int(s[3]) for s in LIFTED}
GB = {2: (-3, 12, -3, 10), 1: (-3, 14)}
FB = {2: (0, 9, 0, 7), 1: (0, 11)}
BOUND = re.compile(r"^(ilo|ihi|jlo|jhi)_(.*)$")
SCRATCH = ("d1", "d2", "d3")   # dense routines accept their scratch and leave it alone
VOLUME = re.compile(r"volumeintegral|volumeregion|surfaceintegral|surfacearea")
U = 2.0 ** -53
# 2D narrow-band construction: its own cases below
BAND2 = ("lsm2ddeterminenarrowband_", "lsm2dmarknarrowbandneighbors_", "lsm2ddeterminenarrowbandfrommask_",
         "lsm2ddeterminenarrowbandfromtwolevelsets_", "lsm2ddeterminenarrowbandawayfrommask_")
# builders whose level 0 is selected by |phi| < width
WIDTH_BAND2 = ("lsm2ddeterminenarrowband_", "lsm2ddeterminenarrowbandfromtwolevelsets_",
               "lsm2ddeterminenarrowbandawayfrommask_")


def is_local(sym):
    return any(a[0] == "index_x" or a[0] == "narrow_band" for a in L.ABI[sym]["args"])


def is_bc(sym):
    return "extrapolation" in sym or "neumann" in sym


def tolerant(sym):
    base = L.ABI[sym]["lifted_from"]
    return base in SUMS or base == "lsm3dcomputeavegradphilocal_"


def shape(d):
    return tuple(GB[d][2 * q + 1] - GB[d][2 * q] + 1 for q in range(d))


def field(rng, d):
    n = shape(d)
    t = sum(np.linspace(0, 3 - q, n[q]).reshape([-1 if p == q else 1 for p in range(d)]) for q in range(d))
    return np.asfortranarray(np.sin(t) + 0.3 * rng.standard_normal(n))


def lists(rng, d, phi):
    """Every fill-box cell, in memory order, split into four levels by |phi|
    rank; narrow_band holds level + 1 there (a few boundary marks of 120)."""
    fb, gb = FB[d], GB[d]
    cells = [c for c in np.ndindex(*[fb[2 * q + 1] - fb[2 * q] + 1 for q in range(d)][::-1])]
    cells = [tuple(fb[2 * q] + c[d - 1 - q] for q in range(d)) for c in cells]   # x fastest
    mag = np.array([abs(phi[tuple(c[q] - gb[2 * q] for q in range(d))]) for c in cells])
    level = np.minimum((np.argsort(np.argsort(mag, kind="stable"), kind="stable") * 4) // len(cells), 3)
    order = sorted(range(len(cells)), key=lambda m: (level[m], m))
    nb = np.zeros(shape(d), dtype=np.uint8, order="F")
    ix, iy, bounds = [], [], []
    for lev in range(4):
        members = [m for m in order if level[m] == lev]
        bounds.append((len(ix), len(ix) + len(members) - 1))
        for m in members:
            c = cells[m]
            ix.append(c[0])
            if d == 2:
                iy.append(c[1])
            nb[tuple(c[q] - gb[2 * q] for q in range(d))] = lev + 1
    nb[rng.random(nb.shape) < 0.03] = 120
    return np.array(ix, np.int32), np.array(iy, np.int32), bounds, nb


def case(sym, seed, face=0):
    d = DIMS[sym]
    rng = np.random.default_rng(seed)
    args = L.ABI[sym]["args"]
    sc = dict(H.DEFAULT_SCALARS)
    sc.update({"bdry_location_idx": face, "n": 2, "dir": 1 + seed % d, "beta": 0.15, "gamma": 0.3,
               "grad_phi_ave": -1.0, "dt": 0.01, "mark_fb": 2, "mark_d1": 4, "mark_d2": 4, "mark_d3": 4,
               "change_sign": -1, "mark_boundary_layer": 7})
    vals = {}
    phi = field(rng, d)
    if is_local(sym):
        ix, iy, bounds, nb = lists(rng, d, phi)
        vals.update({"index_x": ix, "index_y": iy, "narrow_band": nb})
        sc.update({"nlo_index": bounds[0][0], "nhi_index": bounds[3][1]})
        for lev in range(4):
            sc["nlo_index%d" % lev], sc["nhi_index%d" % lev] = bounds[lev]
        if any(a[0] == "nlo_index0" for a in args):
            sc.update({"mark_fb": 1, "mark_d1": 4, "mark_d2": 3, "mark_d3": 2})
        # outer layer: the deepest level's entries, first half "plus", second half "minus"
        outer = np.arange(bounds[3][0], bounds[3][1] + 1, dtype=np.int32)
        half = len(outer) // 2
        vals["index_outer"] = outer
        sc.update({"nlo_index_outer": 0, "nhi_index_outer": len(outer) - 1, "nlo_outer_plus": 0,
                   "nhi_outer_plus": half - 1, "nlo_outer_minus": half, "nhi_outer_minus": len(outer) - 1})
    for name, kind, is_arr, written in args:
        m = BOUND.match(name)
        if m:
            grp = m.group(2)
            b = FB[d] if (grp in ("fb", "ib") or grp.endswith("_fb")) else GB[d]
            vals[name] = b[["ilo", "ihi", "jlo", "jhi"].index(m.group(1))]
        elif is_arr and name not in vals:
            if kind == "real" and not written:
                a = phi.copy(order="F") if name == "phi" else field(rng, d)
                if name.startswith("vel"):
                    a[rng.random(a.shape) < 0.1] = 0.0
                if name == "grad_phi_mag":
                    a = np.abs(a)
                vals[name] = a
            elif kind == "real":
                vals[name] = np.asfortranarray(rng.standard_normal(shape(d)))
            else:
                raise KeyError("%s: no case for array %s" % (sym, name))
        elif not is_arr:
            vals[name] = sc[name]
    return vals


def compare(sym, a1, s1, a2, s2, scale=None, n=0):
    for name in H.written_names(sym):
        if name in SCRATCH and not is_local(sym):
            continue
        if name in a1:
            assert H.same(a1[name], a2[name]), "%s: %s differs, max |diff| %g" % (
                sym, name, np.nanmax(np.abs(a1[name] - a2[name])))
        elif scale is not None:
            tol = (n + 16) * U * scale
            assert abs(s1[name] - s2[name]) <= tol, (sym, name, s1[name], s2[name])
        else:
            assert H.same(s1[name], s2[name]), "%s: %s %r vs %r" % (sym, name, s1[name], s2[name])


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available")
    return r


def test_every_lifted_routine_has_a_reference_routine(ref):
    assert len(LIFTED) >= 100
    for s in LIFTED:
        assert hasattr(ref, s), s


# ---- CPU: the 3D oracle on data copied along the missing axes ---------------------------

DENSE = [s for s in LIFTED if not is_local(s) and not is_bc(s) and not L.ABI[s].get("by_hand")]
BY_HAND = [s for s in LIFTED if L.ABI[s].get("by_hand")]


@pytest.mark.parametrize("sym", BY_HAND)
@pytest.mark.parametrize("sgn", [1, -1])
def test_by_hand_1d_dt_is_the_advection_dt_of_vel_n(sym, sgn, ref):
    """lsm1dComputeStableNormalVelDt (and its control-volume form) reads only
    |vel_n| / dx: the reference's own routine equals the oracle's 3D advection
    dt with vel_x = vel_n and zero y, z velocities, bit for bit."""
    vals = case(sym, 5)
    vals["control_vol_sgn"] = sgn
    _, s_ref = H.run(ref, sym, vals)
    sym3 = L.ABI[sym]["lifted_from"]
    v3 = {}
    for name, kind, is_arr, written in L.ABI[sym3]["args"]:
        m = re.match(r"^(ilo|ihi|jlo|jhi|klo|khi)_(.*)$", name)
        if m:
            v3[name] = vals[name] if m.group(1)[0] == "i" else 0
        elif name == "vel_x":
            v3[name] = np.asfortranarray(vals["vel_n"].reshape(-1, 1, 1))
        elif is_arr and name in vals:
            v3[name] = np.asfortranarray(np.asarray(vals[name]).reshape(-1, 1, 1))
        elif is_arr:
            v3[name] = np.zeros((len(vals["vel_n"]), 1, 1), order="F")
        elif name in vals:
            v3[name] = vals[name]
        else:
            v3[name] = vals["dx"]
    _, s3 = H.run(H.oracle(), sym3, v3)
    assert H.same(s_ref["dt"], s3["dt"]), (s_ref["dt"], s3["dt"])


def lifted_3d_call(sym, vals, copies=7):
    """Arguments of the 3D routine for a 2D / 1D call: arrays copied `copies`
    times along each missing axis, boxes 0:copies-1 there (fill boxes the
    middle cell), zero arrays for the missing components, dz (dy) = dx, or 1
    where the routine multiplies a cell volume."""
    d = DIMS[sym]
    sym3 = L.ABI[sym]["lifted_from"]
    mid = copies // 2
    out = {}
    for name, kind, is_arr, written in L.ABI[sym3]["args"]:
        m = re.match(r"^(ilo|ihi|jlo|jhi|klo|khi)_(.*)$", name)
        if m:
            axis = "ijk".index(m.group(1)[0])
            if axis < d:
                key = [a[0] for a in L.ABI[sym]["args"] if a[0].startswith(m.group(1)[:3])
                       and BOUND.match(a[0]).group(2) in (m.group(2), "fb" if m.group(2).endswith("fb") else None)]
                out[name] = vals[key[0]] if key else vals[name]
            else:
                grp = m.group(2)
                fill = grp in ("fb", "ib") or grp.endswith("_fb")
                out[name] = mid if fill else (0 if m.group(1)[1:] == "lo" else copies - 1)
        elif is_arr:
            a = vals.get(name)
            if a is None:
                a = np.zeros(shape(d))
            a = np.asarray(a)
            for _ in range(3 - d):
                a = np.repeat(a[..., None], copies, axis=-1)
            out[name] = np.asfortranarray(a)
        elif name in vals:
            out[name] = vals[name]
        elif name == "dir":
            out[name] = 1   # a 1D routine differences along x
        else:
            out[name] = 1.0 if VOLUME.search(sym3) else vals["dx"]
    return sym3, out


@pytest.mark.parametrize("sym", DENSE)
def test_lift_principle_on_the_oracle(sym, ref):
    vals = case(sym, 3)
    a_ref, s_ref = H.run(ref, sym, vals)
    sym3, v3 = lifted_3d_call(sym, vals)
    a3, s3 = H.run(H.oracle(), sym3, v3)
    d = DIMS[sym]
    mid = (slice(None),) * d + (3,) * (3 - d)
    for name in H.written_names(sym):
        if name in SCRATCH:
            continue
        if name in a_ref:
            got = a3[name][mid]
            fb, gb = FB[d], GB[d]
            sel = tuple(slice(fb[2 * q] - gb[2 * q], fb[2 * q + 1] - gb[2 * q] + 1) for q in range(d))
            assert H.same(a_ref[name][sel], got[sel]), "%s: %s" % (sym, name)
        elif tolerant(sym):
            assert abs(s_ref[name] - s3[name]) <= 1e-12 * max(1.0, abs(s_ref[name])), (sym, name)
        else:
            assert H.same(s_ref[name], s3[name]), (sym, name, s_ref[name], s3[name])


# ---- GPU: every lifted routine against the reference's -----------------------------------

def thin_3d_call(sym, vals):
    """The 3D routine's arguments for a 2D / 1D call on arrays one cell thick
    along each missing axis (k bounds 0:0, index_z all 0, zero arrays for the
    missing components, dz = dx): the oracle skips every difference along
    those axes there, as the lifted library routine does."""
    d = DIMS[sym]
    sym3 = L.ABI[sym]["lifted_from"]
    out = {}
    for name, kind, is_arr, written in L.ABI[sym3]["args"]:
        m = re.match(r"^(ilo|ihi|jlo|jhi|klo|khi)_(.*)$", name)
        if m:
            axis = "ijk".index(m.group(1)[0])
            out[name] = vals[name] if axis < d else 0
        elif is_arr and name in vals:
            a = np.asarray(vals[name])
            out[name] = a if a.ndim == 1 else np.asfortranarray(a.reshape(a.shape + (1,) * (3 - d), order="F"))
        elif is_arr and kind == "int":
            out[name] = np.zeros_like(np.asarray(vals["index_x"]))
        elif is_arr:
            out[name] = np.zeros(shape(d) + (1,) * (3 - d), order="F")
        elif name in vals:
            out[name] = vals[name]
        else:
            out[name] = vals["dx"]
    return sym3, out


def test_unusable_reference_routines_are_known():
    assert REF_UNUSABLE == ["lsm2dhjeno3local_"]


@pytest.mark.gpu
@pytest.mark.parametrize("sym", REF_UNUSABLE)
@pytest.mark.parametrize("seed", [0, 1])
def test_lifted_gpu_matches_thin_oracle(sym, seed, gpu_lib):
    vals = case(sym, seed)
    sym3, v3 = thin_3d_call(sym, vals)
    a3, _ = H.run(H.oracle(), sym3, v3)
    a2, _ = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    for name in H.written_names(sym):
        assert H.same(a3[name].reshape(a2[name].shape, order="F"), a2[name]), "%s: %s" % (sym, name)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", [s for s in LIFTED if s not in BAND2 and s not in REF_UNUSABLE])
def test_lifted_gpu_matches_reference(sym, ref, gpu_lib):
    faces = range(2 * DIMS[sym]) if is_bc(sym) else [0]
    for face in faces:
        for seed in (0, 1):
            vals = case(sym, seed, face)
            a1, s1 = H.run(ref, sym, vals)
            a2, s2 = H.run(gpu_lib, sym, vals)
            L.check(gpu_lib)
            scale, n = None, 0
            if tolerant(sym):
                v = dict(vals)
                if "f" in v:
                    v["f"] = np.abs(v["f"]).copy(order="F")
                out = [a[0] for a in L.ABI[sym]["args"] if not a[2] and a[3]][0]
                scale = abs(H.run(ref, sym, v)[1][out])
                n = int(np.prod(shape(DIMS[sym])))
            compare(sym, a1, s1, a2, s2, scale, n)


# ---- 2D narrow-band construction -----------------------------------------------------------

GB_BAND = (-3, 40, -3, 36)
DXB = 0.05


def band_phi2(seed):
    i = np.arange(GB_BAND[0], GB_BAND[1] + 1)
    j = np.arange(GB_BAND[2], GB_BAND[3] + 1)
    X, Y = np.meshgrid((i + 0.5) * DXB, (j + 0.5) * DXB, indexing="ij")
    phi = np.sqrt((X - 0.95) ** 2 + (Y - 0.85) ** 2) - 0.5
    rng = np.random.default_rng(seed)
    return np.asfortranarray(phi + 0.01 * rng.standard_normal(phi.shape))


def band2_call(sym, seed, level=3, phi=None):
    """Every argument of a 2D band-construction call over GB_BAND, with list
    capacity for every cell and stale contents in the outputs.  psi is a
    second circle crossing phi's; the away-from-mask mask differs from phi by
    more than max(dx, dy) on part of the band."""
    n = (GB_BAND[1] - GB_BAND[0] + 1, GB_BAND[3] - GB_BAND[2] + 1)
    cap = n[0] * n[1]
    phi = band_phi2(seed) if phi is None else phi
    mask = phi
    if sym == "lsm2ddeterminenarrowbandawayfrommask_":
        i = np.arange(n[0]).reshape(-1, 1)
        mask = np.asfortranarray(phi + 2.0 * DXB * (i % 3 == 0))
    psi = np.asfortranarray(np.roll(band_phi2(seed + 7), 9, axis=0))
    v = {"phi": phi, "mask": mask, "psi": psi, "dx": DXB, "dy": 1.1 * DXB, "narrow_band": np.zeros(n, dtype=np.uint8, order="F"),
         "index_x": np.full(cap, -99, np.int32), "index_y": np.full(cap, -99, np.int32),
         "nlo_index": 0, "nhi_index": cap - 1, "n_lo": np.full(level + 1, -7, np.int32),
         "n_hi": np.full(level + 1, -7, np.int32), "index_outer": np.full(cap, -99, np.int32),
         "nlo_index_outer": 0, "nhi_index_outer": cap - 1, "nlo_outer_plus": 0, "nhi_outer_plus": 0,
         "nlo_outer_minus": 0, "nhi_outer_minus": 0, "width": 2.0 * DXB, "width_inner": DXB, "level": level,
         "use_mask_sign": 1 + seed % 2}
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        m = BOUND.match(name)
        if m:
            v[name] = GB_BAND[["ilo", "ihi", "jlo", "jhi"].index(m.group(1))]
    return {a[0]: v[a[0]] for a in L.ABI[sym]["args"]}


def band2_inputs(lib, sym, seed):
    """For the neighbour routine: level-0 lists from the same library's
    lsm2ddeterminenarrowband_ (level 0 only)."""
    vals = band2_call(sym, seed)
    if sym == "lsm2dmarknarrowbandneighbors_":
        base = band2_call("lsm2ddeterminenarrowband_", seed, level=0)
        a, s = H.run(lib, "lsm2ddeterminenarrowband_", base)
        for k in ("narrow_band", "index_x", "index_y"):
            vals[k] = a[k]
        vals["n_lo"][0], vals["n_hi"][0] = a["n_lo"][0], a["n_hi"][0]
    return vals


def band2_compare(sym, r1, r2):
    a1, s1 = r1
    a2, s2 = r2
    for name in H.written_names(sym):
        if name in a1:
            assert H.same(a1[name], a2[name]), "%s: %s differs" % (sym, name)
        else:
            assert s1[name] == s2[name], "%s: %s %r vs %r" % (sym, name, s1[name], s2[name])


@pytest.mark.parametrize("sym", BAND2)
@pytest.mark.parametrize("seed", [0, 1])
def test_band2_principle_on_the_oracle(sym, seed, ref):
    """The 3D oracle on the 2D grid as a grid one cell deep (k = 0:0) builds
    the reference 2D routine's lists, levels and marks."""
    vals = band2_inputs(ref, sym, seed)
    r_ref = H.run(ref, sym, vals)
    sym3 = L.ABI[sym]["lifted_from"]
    v3 = {}
    cap = len(vals["index_x"])
    for name, kind, is_arr, written in L.ABI[sym3]["args"]:
        if name in vals:
            v3[name] = vals[name]
        elif name == "index_z":
            v3[name] = np.zeros(cap, np.int32)
        elif name.startswith(("klo", "khi")):
            v3[name] = 0
        elif name == "dz":
            v3[name] = vals["dx"]
        else:
            raise KeyError(name)
    a3, s3 = H.run(H.oracle(), sym3, v3)
    band2_compare(sym, r_ref, (a3, s3))


def degenerate_phi(kind):
    """5 everywhere (no cell within the width), or one cell at 0"""
    n = (GB_BAND[1] - GB_BAND[0] + 1, GB_BAND[3] - GB_BAND[2] + 1)
    phi = np.full(n, 5.0, order="F")
    if kind == "single":
        phi[17, 11] = 0.0
    return phi


def degenerate_call(sym, kind):
    # an empty level 0 with two or more neighbour levels makes the reference
    # read list entry -1 (localization2d.f:120); one level keeps it defined
    vals = band2_call(sym, 0, level=1 if kind == "empty" else 3, phi=degenerate_phi(kind))
    if "psi" in vals:
        vals["psi"] = np.zeros_like(vals["phi"], order="F")
    if "mask" in vals:
        vals["mask"] = np.asfortranarray(vals["phi"] + 1.0)
    return vals


@pytest.mark.parametrize("sym", WIDTH_BAND2)
@pytest.mark.parametrize("kind", ["empty", "single"])
def test_band2_degenerate_principle_on_the_oracle(sym, kind, ref):
    """Empty and one-cell bands: the list bookkeeping of the 2D routines
    (n_hi(0) = count - 1; neighbour levels only from two cells up in
    lsm2dDetermineNarrowBand) through the 3D-array forms the 2D entry
    points run on."""
    vals = degenerate_call(sym, kind)
    r_ref = H.run(ref, sym, vals)
    sym3 = L.ABI[sym]["lifted_from"]
    v3 = {}
    for name, kind_, is_arr, written in L.ABI[sym3]["args"]:
        if name in vals:
            v3[name] = vals[name]
        elif name == "index_z":
            v3[name] = np.zeros(len(vals["index_x"]), np.int32)
        elif name.startswith(("klo", "khi")):
            v3[name] = 0
        elif name == "dz":
            v3[name] = vals["dx"]
    r3 = H.run(H.oracle(), sym3, v3)
    band2_compare(sym, r_ref, r3)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", WIDTH_BAND2)
@pytest.mark.parametrize("kind", ["empty", "single"])
def test_band2_degenerate_gpu_matches_reference(sym, kind, ref, gpu_lib):
    vals = degenerate_call(sym, kind)
    r_ref = H.run(ref, sym, vals)
    r_gpu = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    band2_compare(sym, r_ref, r_gpu)


@pytest.mark.gpu
@pytest.mark.parametrize("sym", BAND2)
@pytest.mark.parametrize("seed", [0, 1])
def test_band2_gpu_matches_reference(sym, seed, ref, gpu_lib):
    vals = band2_inputs(ref, sym, seed)
    r_ref = H.run(ref, sym, vals)
    r_gpu = H.run(gpu_lib, sym, vals)
    L.check(gpu_lib)
    band2_compare(sym, r_ref, r_gpu)
