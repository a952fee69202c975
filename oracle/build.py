"""Build the CPU oracle libraries (test infrastructure only).

* oracle/liblsmoracle.so — the C restatement of LSMLIB's kernels in this
  directory (oracle_*.c), compiled -O2 -ffp-contract=off so no fused
  multiply-add alters a rounding.
* oracle/_ref/liblsmref.so — LSMLIB's own Fortran kernels, translated to C by
  f77ref.py from the reference source tree (when it is present) and compiled
  the same way.
* oracle/_ref/liblsmrefio.so — LSMLIB's own Grid / data-array file code
  (src/utils, C), compiled from the reference tree when it is present.  The translated C (oracle/_ref/lsmref.c) is kept out of
  version control; where the reference tree is absent, an existing
  lsmref.c is compiled as is.

Nothing in the product links or loads either library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# LSMLIB source tree (read only); LSMLIB_REFERENCE_TREE overrides the default
REFERENCE_TREE = os.environ.get("LSMLIB_REFERENCE_TREE", "/root/reference")

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
    # 2D and 1D forms of the dense hot-path routines
    "toolbox/lsm_spatial_derivatives2d.f.in",
    "toolbox/lsm_tvd_runge_kutta2d.f",
    "toolbox/lsm_level_set_evolution2d.f.in",
    "reinitialization/lsm_reinitialization2d.f.in",
    "geometry/lsm_curvature2d.f.in",
    "toolbox/lsm_math_utils2d.f.in",
    "boundary_conditions/lsm_boundary_conditions2d.f",
    "toolbox/lsm_spatial_derivatives1d.f.in",
    "toolbox/lsm_tvd_runge_kutta1d.f",
    "toolbox/lsm_level_set_evolution1d.f.in",
    "reinitialization/lsm_reinitialization1d.f.in",
    "toolbox/lsm_math_utils1d.f.in",
    "boundary_conditions/lsm_boundary_conditions1d.f",
    "toolbox/lsm_tvd_runge_kutta2d_local.f",
    "toolbox/lsm_level_set_evolution2d_local.f.in",
    "reinitialization/lsm_reinitialization2d_local.f.in",
    "geometry/lsm_curvature2d_local.f.in",
    "toolbox/lsm_math_utils2d_local.f.in",
    "toolbox/lsm_localization2d.f",
    "toolbox/lsm_calculus_toolbox2d.f.in",
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


# The reference's on-disk format code (C), compiled from its own files.
REF_IO_SOURCES = ["utils/lsm_grid.c", "utils/lsm_data_arrays.c", "utils/lsm_file.c"]

# The values the reference's build writes into lsmlib_config.h for its
# double-precision configuration (include/lsmlib_config.h.in).
REF_IO_CONFIG = """#define LSMLIB_DOUBLE_PRECISION
#define LSMLIB_REAL double
#define LSMLIB_ZERO_TOL 1.e-11
#define LSMLIB_REAL_MAX 1.7976931348623157e308
#define LSMLIB_REAL_MIN 2.2250738585072014e-308
#define LSMLIB_REAL_EPSILON 2.2204460492503131e-16
"""


def build_ref_io():
    """Compile the reference's Grid / data-array file code
    (oracle/_ref/liblsmrefio.so) when the reference tree is present."""
    if not os.path.isdir(REFERENCE_TREE):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    with open(os.path.join(REF_DIR, "lsmlib_config.h"), "w") as f:
        f.write(REF_IO_CONFIG)
    srcs = [os.path.join(REFERENCE_TREE, "src", s) for s in REF_IO_SOURCES]
    out = os.path.join(REF_DIR, "liblsmrefio.so")
    _run([_cc(), "-O2", "-fPIC", "-shared", "-w", "-I", REF_DIR,
          "-I", os.path.join(REFERENCE_TREE, "src", "utils"), "-o", out] + srcs + ["-lm"])
    return out


def build():
    o = build_oracle()
    r = build_ref()
    build_ref_io()
    return o, r


if __name__ == "__main__":
    print(build())
