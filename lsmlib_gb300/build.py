"""Build liblsmgpu.so (the GB300 kernels behind the C interface) in-tree.

Each .cu file under csrc/ compiles to its own object with nvcc for sm_103a,
in parallel; the objects link into lsmlib_gb300/liblsmgpu.so.  Translation
units that hold FP64 parity kernels are compiled with -fmad=false so their
products and sums round exactly like LSMLIB's Fortran (no fused multiply-add);
the FP32 fast-path units keep FMA contraction.

Usage:  python -m lsmlib_gb300.build   (or lsmlib_gb300.build.build())
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblsmgpu.so")
# the bounds-check build (LSMGPU_BOUNDS_CHECK): its own objects and library
BUILD_BC = os.path.join(HERE, "_build_bc")
libBC = os.path.join(HERE, "liblsmgpu_bc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code computes some per-call constants (e.g. the cut-off's (gamma -
# 3 beta)); -ffp-contract=off keeps the host compiler from fusing them into
# FMAs on hosts that have them (Arm), so they round as LSMLIB's do.
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "--extended-lambda", "-I", os.path.join(HERE, "..", "include")]

# FP64 parity units: no contraction of a*b+c into FMA
NO_FMA = {"dense.cu", "dense2.cu", "local.cu", "band.cu", "fused_f64.cu", "batched_f64.cu", "adjoint_f64.cu", "diag.cu",
          "noalloc.cu", "bandflow_f64.cu", "geometry.cu", "plane2d.cu", "lifted_by_hand.cu"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the lsmgpu CUDA library cannot be built")


def _compile(src, extra, build_dir=BUILD):
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest_input(src):
        return obj, ""
    flags = list(COMMON)
    if os.path.basename(src) in NO_FMA:
        flags += ["-fmad=false"]
    cmd = [nvcc()] + ARCH + flags + extra + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), p.stdout + p.stderr))
    return obj, p.stdout + p.stderr


def _newest_input(src):
    t = os.path.getmtime(src)
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def build(verbose=False, extra=None, bounds_check=False):
    """Compile and link liblsmgpu.so (or, with bounds_check, the
    bounds-checked liblsmgpu_bc.so); returns the library's path."""
    build_dir, lib = (BUILD_BC, libBC) if bounds_check else (BUILD, LIB)
    os.makedirs(build_dir, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    extra = list(extra or []) + (["-DLSMGPU_BOUNDS_CHECK"] if bounds_check else [])
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        tmp = lib + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-ldl"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), p.stdout + p.stderr))
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, bounds_check="--bounds-check" in sys.argv))
