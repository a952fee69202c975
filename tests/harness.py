"""Test harness: drive any library that exports LSMLIB's signatures (the GPU
library, the C oracle, the translated reference) with the same arguments.

Arrays are numpy arrays in Fortran (column-major) order over their ghost box,
as LSMLIB stores them.
"""
import ctypes
import os
import re

import numpy as np

import lsmlib_gb300 as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "liblsmoracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "liblsmref.so")

_libs = {}


def _load(path):
    if path not in _libs:
        _libs[path] = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    return _libs[path]


def oracle():
    if not os.path.exists(ORACLE_SO):
        from oracle import build as ob
        ob.build_oracle()
    return _load(ORACLE_SO)


def reference():
    """The reference's own kernels (translated Fortran), or None."""
    if not os.path.exists(REF_SO):
        try:
            from oracle import build as ob
            ob.build_ref()
        except Exception:
            return None
    return _load(REF_SO) if os.path.exists(REF_SO) else None


_BOX_RE = re.compile(r"^(ilo|ihi|jlo|jhi|klo|khi)_(.*)$")


def arg_layout(sym):
    """Map each array argument of `sym` to the name of its 6-int bound group
    (e.g. 'grad_phi_plus_gb', 'fb', 'ib'), or to 'index:<lo>,<hi>' for 1-D
    arrays bounded by two scalar arguments."""
    args = L.ABI[sym]["args"]
    pending, layout = [], {}
    names = [a[0] for a in args]
    for idx, (name, kind, is_arr, _w) in enumerate(args):
        if is_arr:
            pending.append(name)
            continue
        m = _BOX_RE.match(name)
        if m and m.group(1) == "ilo" and pending:
            for p in pending:
                layout[p] = m.group(2)
            pending = []
    for p in pending:
        layout[p] = None
    return layout


def box_args(sym, boxes, default_gb, fb):
    """Scalar values for every *lo/*hi bound argument.

    boxes: dict group-name -> (ilo, ihi, jlo, jhi, klo, khi); groups named
    'fb', '*_fb' and 'ib' default to `fb`, every other group to default_gb."""
    vals = {}
    for name, kind, is_arr, _w in L.ABI[sym]["args"]:
        m = _BOX_RE.match(name)
        if not m or is_arr:
            continue
        which, grp = m.group(1), m.group(2)
        if grp in boxes:
            b = boxes[grp]
        elif grp == "fb" or grp.endswith("_fb") or grp == "ib":
            b = fb
        else:
            b = default_gb
        vals[name] = b[["ilo", "ihi", "jlo", "jhi", "klo", "khi"].index(which)]
    return vals


def shape_of(b):
    return (b[1] - b[0] + 1, b[3] - b[2] + 1, b[5] - b[4] + 1)


def make_call(sym, gb, fb, arrays=None, scalars=None, boxes=None, fill=np.nan):
    """Full argument dict for `sym`.  Arrays not supplied are allocated over
    their ghost box: written arrays filled with `fill`, read arrays must be
    given (KeyError otherwise)."""
    arrays = dict(arrays or {})
    boxes = dict(boxes or {})
    vals = box_args(sym, boxes, gb, fb)
    layout = arg_layout(sym)
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        if is_arr:
            if name not in arrays:
                grp = layout.get(name)
                b = boxes.get(grp, gb) if grp else gb
                if not written:
                    raise KeyError("%s: input array %s not supplied" % (sym, name))
                dt = np.float64 if kind in ("real", "double") else (np.int32 if kind == "int" else np.uint8)
                a = np.empty(shape_of(b), dtype=dt, order="F")
                a[...] = fill if dt == np.float64 else 0
                arrays[name] = a
            vals[name] = arrays[name]
        elif name not in vals:
            if scalars is None or name not in scalars:
                raise KeyError("%s: scalar %s not supplied" % (sym, name))
            vals[name] = scalars[name]
    scalar_names = {a[0] for a in L.ABI[sym]["args"] if not a[2]}
    for k, v in (scalars or {}).items():
        if k in scalar_names:
            vals[k] = v
    return vals, arrays


def run(handle, sym, vals):
    """Invoke and return (arrays-after, scalars-after) — arrays are copied so
    the same inputs can be reused for another library."""
    v = {}
    for k, a in vals.items():
        v[k] = a.copy(order="F") if isinstance(a, np.ndarray) else a
    sc = L.invoke(handle, sym, v)
    arrs = {k: a for k, a in v.items() if isinstance(a, np.ndarray)}
    return arrs, sc


def written_names(sym):
    return [a[0] for a in L.ABI[sym]["args"] if a[3]]


def same(a, b):
    """Bitwise-equal values, treating +0 == -0 and NaN == NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return False
    eq = (a == b) | (np.isnan(a) & np.isnan(b)) if a.dtype.kind == "f" else (a == b)
    return bool(np.all(eq))


def sphere_phi(gb, dx, center=(0.1, -0.05, 0.0), r=0.35, lo=-1.0):
    """Signed distance to a sphere on cell centres x_i = lo + (i + 1/2) dx."""
    i = np.arange(gb[0], gb[1] + 1)
    j = np.arange(gb[2], gb[3] + 1)
    k = np.arange(gb[4], gb[5] + 1)
    x = lo + (i + 0.5) * dx
    y = lo + (j + 0.5) * dx
    z = lo + (k + 0.5) * dx
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    d = np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2 + (Z - center[2]) ** 2) - r
    return np.asfortranarray(d)


def rough_field(rng, gb, scale=1.0):
    """Smooth field plus noise, so every ENO/WENO branch is taken."""
    n = shape_of(gb)
    base = rng.standard_normal(n) * 0.3
    t = np.linspace(0, 3, n[0])[:, None, None] + np.linspace(0, 2, n[1])[None, :, None] + \
        np.linspace(0, 1, n[2])[None, None, :]
    return np.asfortranarray(scale * (np.sin(t) + base))


# ---------------------------------------------------------------------------
# generic seeded cases for the dense entry points
# ---------------------------------------------------------------------------
DEFAULT_SCALARS = {"dx": 0.1, "dy": 0.12, "dz": 0.09, "dt": 0.013, "cfl_number": 0.5,
                   "b": 0.3, "vel_n": 0.7, "use_phi0_for_sgn": 0,
                   "max_norm_diff": -7.0, "epsilon": 0.45, "control_vol_sgn": 1,
                   "ave_abs_diff": -7.0, "count": -7, "int_f": -7.0, "volume": -7.0, "area": -7.0,
                   "n": 3, "dir": 2}

GB = (-3, 12, -3, 10, -3, 8)     # ghost box with negative lower bounds
FB = (0, 9, 0, 7, 0, 5)          # fill box three cells inside it


def dense_case(sym, seed=0, gb=GB, fb=FB, scalars=None):
    rng = np.random.default_rng(seed)
    sc = dict(DEFAULT_SCALARS)
    sc.update(scalars or {})
    layout = arg_layout(sym)
    arrays = {}
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        if not is_arr or written:
            continue
        a = rough_field(rng, gb)
        if name.startswith("vel"):
            mask = rng.random(shape_of(gb)) < 0.1
            a[mask] = 0.0
        if name == "grad_phi_mag":
            a = np.abs(a)
            a[rng.random(shape_of(gb)) < 0.05] = 0.0
        arrays[name] = np.asfortranarray(a)
    # outputs start from a recognisable pattern so untouched cells compare too
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        if is_arr and written and name not in arrays:
            arrays[name] = np.asfortranarray(rng.standard_normal(shape_of(gb)))
    vals, arrays = make_call(sym, gb, fb, arrays=arrays, scalars=sc)
    return vals
