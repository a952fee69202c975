"""The drop-in boundary from C: tests/c_driver/reinit_weno5.c, a program
written against LSMLIB's own headers, compiled and linked unchanged.

CPU: built against LSMLIB's headers (src/toolbox, src/reinitialization,
src/boundary_conditions, src/utils, with the double-precision
lsmlib_config.h oracle/build.py writes), it links against liblsmgpu.so, and
linked against the reference's own objects (its kernels translated to C and
its lsm_grid.c) it writes the same bytes as linked against the C oracle; the
same source also builds against this library's headers (-DLSMGPU_HEADERS).
GPU: linked against liblsmgpu.so (host arrays, so every call stages its
arrays) it writes the same bytes as linked against the reference's kernels.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import harness as H

ROOT = H.ROOT
SRC = os.path.join(ROOT, "tests", "c_driver", "reinit_weno5.c")
LIBDIR = os.path.join(ROOT, "lsmlib_gb300")
REF = os.path.join(ROOT, "oracle", "_ref")
TREE = os.environ.get("LSMLIB_REFERENCE_TREE", "/root/reference")
LSMLIB_INCLUDES = ["src/utils", "src/toolbox", "src/reinitialization", "src/boundary_conditions"]


def _cc():
    return os.environ.get("CC", "gcc")


def _build(out, includes, defines=(), libs=(), rpaths=()):
    cmd = [_cc(), "-O2", "-std=gnu99", "-ffp-contract=off", SRC, "-o", out] + ["-I" + d for d in includes] + \
          ["-D" + d for d in defines] + list(libs) + ["-Wl,-rpath," + r for r in rpaths] + ["-lm"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, " ".join(cmd) + "\n" + p.stdout + p.stderr


def _run(exe, n, iters, out):
    p = subprocess.run([exe, str(n), str(iters), out], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    return np.fromfile(out, dtype=np.float64)


def _lsmlib_includes():
    if not os.path.isdir(os.path.join(TREE, "src")) or not os.path.exists(os.path.join(REF, "lsmlib_config.h")):
        pytest.skip("LSMLIB's headers are not present here")
    return [REF] + [os.path.join(TREE, d) for d in LSMLIB_INCLUDES]


def _gpu_lib():
    from lsmlib_gb300 import build as B
    B.build()
    return ["-L" + LIBDIR, "-llsmgpu"], [LIBDIR]


def test_builds_against_lsmlib_headers_and_links_to_liblsmgpu(tmp_path):
    inc = _lsmlib_includes()
    libs, rp = _gpu_lib()
    _build(str(tmp_path / "drv_gpu"), inc, libs=libs, rpaths=rp)
    _build(str(tmp_path / "drv_gpu_own_headers"), [os.path.join(ROOT, "include")], ["LSMGPU_HEADERS"], libs, rp)


def test_reference_objects_and_oracle_write_the_same_bytes(tmp_path):
    inc = _lsmlib_includes()
    ref_k, ref_io = os.path.join(REF, "liblsmref.so"), os.path.join(REF, "liblsmrefio.so")
    if not (os.path.exists(ref_k) and os.path.exists(ref_io)):
        pytest.skip("the reference's objects are not built here")
    H.oracle()
    exe_ref, exe_orc = str(tmp_path / "drv_ref"), str(tmp_path / "drv_oracle")
    # the reference: its kernels and its own lsm_grid.c
    _build(exe_ref, inc, libs=[ref_k, ref_io], rpaths=[REF])
    # the oracle's kernels; the Grid functions from liblsmgpu.so
    libs, rp = _gpu_lib()
    _build(exe_orc, inc, libs=[H.ORACLE_SO] + libs, rpaths=[os.path.dirname(H.ORACLE_SO)] + rp)
    a = _run(exe_ref, 24, 3, str(tmp_path / "ref.bin"))
    b = _run(exe_orc, 24, 3, str(tmp_path / "oracle.bin"))
    assert a.size == 32 ** 3 and np.array_equal(a, b)


@pytest.mark.gpu
def test_c_driver_on_liblsmgpu_equals_reference(tmp_path, gpu_lib):
    """liblsmgpu.so against the reference's kernels (translated Fortran, or
    the C oracle where the translation is absent), the same program built
    against this library's headers; the Grid functions come from
    liblsmgpu.so in both (the reference's kernels are linked first, so their
    symbols win)."""
    libs, rp = _gpu_lib()
    inc = [os.path.join(ROOT, "include")]
    ref_k = os.path.join(REF, "liblsmref.so")
    if not os.path.exists(ref_k):
        H.reference()
    kern = ref_k if os.path.exists(ref_k) else H.oracle() and H.ORACLE_SO
    exe_gpu, exe_ref = str(tmp_path / "drv_gpu"), str(tmp_path / "drv_ref")
    _build(exe_gpu, inc, ["LSMGPU_HEADERS"], libs, rp)
    _build(exe_ref, inc, ["LSMGPU_HEADERS"], [kern] + libs, [os.path.dirname(kern)] + rp)
    a = _run(exe_ref, 40, 4, str(tmp_path / "ref.bin"))
    b = _run(exe_gpu, 40, 4, str(tmp_path / "gpu.bin"))
    assert a.size == 48 ** 3
    assert np.array_equal(a, b), np.max(np.abs(a - b))
