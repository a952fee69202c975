"""Pin the C oracle against the reference's own kernels.

The reference (LSMLIB) is Fortran 77; oracle/f77ref.py translates its source
files mechanically into C (oracle/_ref/liblsmref.so).  The hand-written
oracle (oracle/liblsmoracle.so) must agree with it bit for bit on every
dense entry point, on seeded inputs with negative lower bounds, so both the
restatement and the translation are checked against each other.
"""
import numpy as np
import pytest

import lsmlib_gb300 as L
from tests import harness as H

DENSE = [s for s in L.ABI if s.startswith("lsm3d")
         and not any(a[0] in ("index_x", "narrow_band") for a in L.ABI[s]["args"])
         and "extrapolation" not in s and "neumann" not in s]


@pytest.fixture(scope="module")
def ref():
    r = H.reference()
    if r is None:
        pytest.skip("reference translation not available (no reference tree or lsmref.c)")
    return r


@pytest.mark.parametrize("sym", DENSE)
@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_matches_reference(sym, seed, ref):
    extra = {"use_phi0_for_sgn": seed} if "reinit" in sym else {}
    vals = H.dense_case(sym, seed=seed, scalars=extra)
    a_ref, s_ref = H.run(ref, sym, vals)
    a_or, s_or = H.run(H.oracle(), sym, vals)
    for name in H.written_names(sym):
        if name in ("d1", "d2", "d3"):
            continue  # scratch: the oracle does not write it
        if name in a_ref:
            assert H.same(a_ref[name], a_or[name]), "%s: array %s differs" % (sym, name)
        else:
            assert H.same(s_ref[name], s_or[name]), "%s: scalar %s differs %r %r" % (
                sym, name, s_ref[name], s_or[name])
