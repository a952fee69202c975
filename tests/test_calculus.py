"""lsmheaviside_ / lsmdeltafunction_: the library's scalar smoothed Heaviside
and delta functions against the known answers of LSMLIB's own test
(tests/toolbox/test_calculus_toolbox.cc, tolerance 1e-6, committed as
tests/golden/calculus_toolbox_kat.json) and bit for bit against the
reference's (translated) routines over a sweep that crosses both clip points.
Host functions: no GPU needed."""
import ctypes
import json
import os

import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "calculus_toolbox_kat.json")


def _eval(lib, sym, x, eps):
    fn = getattr(lib, sym)
    fn.restype = None
    fn.argtypes = [ctypes.POINTER(ctypes.c_double)] * 3
    out = ctypes.c_double(-7.0)
    fn(ctypes.byref(out), ctypes.byref(ctypes.c_double(x)), ctypes.byref(ctypes.c_double(eps)))
    return out.value


@pytest.mark.parametrize("sym,key", [("lsmheaviside_", "heaviside"), ("lsmdeltafunction_", "delta")])
def test_known_answers(sym, key):
    kat = json.load(open(GOLDEN))
    d = kat["d_phi"]
    eps = kat["eps_over_d_phi"] * d
    for i, want in enumerate(kat[key]):
        got = _eval(L.lib(), sym, -1.0 + i * d, eps)
        assert abs(got - want) <= kat["tolerance"], (sym, i, got, want)


@pytest.mark.parametrize("sym", ["lsmheaviside_", "lsmdeltafunction_"])
def test_bit_exact_against_reference(sym):
    ref = H.reference()
    if ref is None:
        pytest.skip("reference translation not available")
    eps = 0.3
    xs = np.concatenate([np.linspace(-0.5, 0.5, 1001), [-eps, eps, np.nextafter(eps, 1), -0.0, 0.0]])
    for x in xs:
        a, b = _eval(L.lib(), sym, float(x), eps), _eval(ref, sym, float(x), eps)
        assert H.same(a, b), (sym, x, a, b)
