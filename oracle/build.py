"""Build the CPU oracle libraries (test infrastructure only).

* oracle/liblsmoracle.so — the C restatement of LSMLIB's kernels in this
  directory (oracle_*.c), compiled -O2 -ffp-contract=off so no fused
  multiply-add alters a rounding.
* oracle/_ref/liblsmref.so — LSMLIB's own Fortran kernels, translated to C by
  f77ref.py from the reference source tree (when it is present) and compiled
  the same way.  The translated C (oracle/_ref/lsmref.c) is kept out of
  version control; where the reference tree is absent, an existing
  lsmref.c is compiled as is.

Nothing in the product links or loads either library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_TREE = "/root/reference"

# Hot-path Fortran sources of the reference, relative to its src/ directory.
REF_SOURCES = [
    "toolbox/lsm_spatial_derivatives3d.f.in",
    "toolbox/lsm_spatial_derivatives3d_local.f.in",
    "toolbox/lsm_tvd_runge_kutta3d.f",
    "toolbox/lsm_tvd_runge_kutta3d_local.f",
    "toolbox/lsm_level_set_evolution3d.f.in",
    "toolbox/lsm_level_set_evolution3d_local.f.in",
    "toolbox/lsm_math_utils3d.f.in",
    "toolbox/lsm_math_utils3d_local.f.in",
    "toolbox/lsm_localization3d.f",
    "reinitialization/lsm_reinitialization3d.f.in",
    "reinitialization/lsm_reinitialization3d_local.f.in",
    "geometry/lsm_curvature3d.f.in",
    "geometry/lsm_curvature3d_local.f.in",
    "boundary_conditions/lsm_boundary_conditions3d.f",
    "toolbox/lsm_calculus_toolbox.f",
    "toolbox/lsm_calculus_toolbox3d.f.in",
    "geometry/lsm_geometry3d_fort.f.in",
    "toolbox/lsm_spatial_derivatives2d_local.f.in",
]

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=gnu99",
          "-Wl,-Bsymbolic"]


def _cc():
    return os.environ.get("CC", "gcc")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("%s\n%s" % (" ".join(cmd), p.stdout + p.stderr))


def build_oracle():
    srcs = sorted(os.path.join(HERE, f) for f in os.listdir(HERE)
                  if f.startswith("oracle_") and f.endswith(".c"))
    out = os.path.join(HERE, "liblsmoracle.so")
    _run([_cc()] + CFLAGS + ["-o", out] + srcs + ["-lm"])
    return out


def build_ref():
    """Translate (if the reference tree exists) and compile the reference."""
    os.makedirs(REF_DIR, exist_ok=True)
    csrc = os.path.join(REF_DIR, "lsmref.c")
    sigs = os.path.join(REF_DIR, "sigs.json")
    if os.path.isdir(REFERENCE_TREE):
        srcs = [os.path.join(REFERENCE_TREE, "src", s) for s in REF_SOURCES]
        _run([sys.executable, os.path.join(HERE, "f77ref.py"), "--precision", "double",
              "--sig-json", sigs, csrc] + srcs)
    if not os.path.exists(csrc):
        return None
    out = os.path.join(REF_DIR, "liblsmref.so")
    _run([_cc()] + CFLAGS + ["-w", "-o", out, csrc, "-lm"])
    return out


def build():
    o = build_oracle()
    r = build_ref()
    return o, r


if __name__ == "__main__":
    print(build())
