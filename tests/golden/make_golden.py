"""Extract the known-answer vectors of LSMLIB's own test suite that pin this
path, into small JSON fixtures next to this script.

Source: tests/toolbox/test_calculus_toolbox.cc of LSMLIB (fixture x_i =
-1 + i*d_phi, d_phi = 0.1, eps = 3*d_phi; expected LSM_HEAVISIDE and
LSM_DELTA_FUNCTION values at 20 points, tolerance 1e-6).

Usage: python tests/golden/make_golden.py [path to the LSMLIB source tree]
(run where the LSMLIB sources are available; the fixtures are committed).
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _array(src, name):
    m = re.search(r"LSMLIB_REAL\s+%s\[20\]\s*=\s*\{([^}]*)\}" % name, src)
    if not m:
        raise SystemExit("array %s not found" % name)
    vals = [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
    assert len(vals) == 20, name
    return vals


def main(root):
    path = os.path.join(root, "tests", "toolbox", "test_calculus_toolbox.cc")
    src = open(path).read()
    assert re.search(r"d_phi\s*=\s*0\.1;", src) and re.search(r"eps\s*=\s*3\.0\s*\*\s*d_phi;", src)
    out = {
        "source": "tests/toolbox/test_calculus_toolbox.cc (LSMLIB)",
        "d_phi": 0.1,
        "eps_over_d_phi": 3.0,
        "x": "x_i = -1.0 + i * d_phi, i = 0..19",
        "tolerance": 1e-6,
        "heaviside": _array(src, "h_expected"),
        "delta": _array(src, "d_expected"),
    }
    with open(os.path.join(HERE, "calculus_toolbox_kat.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print("wrote calculus_toolbox_kat.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LSMLIB_REFERENCE_TREE", "/root/reference"))
