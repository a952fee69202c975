"""Run one fused call of the level-set hot path on cuda:0, for profilers.

  python -m lsmlib_gb300.profile_case --mode reinit --n 256 --iters 1 --precision f32
  python -m lsmlib_gb300.profile_case --mode adjoint --n 128 --iters 8 --precision f32
  python -m lsmlib_gb300.profile_case --mode band --n 256 --iters 10
  python -m lsmlib_gb300.profile_case --mode batched --n 512 --iters 2
  python -m lsmlib_gb300.profile_case --mode geometry --n 256 --iters 1

Builds the same analytic field as bench.py, moves it to the device, and runs
`iters` WENO5 / TVD-RK3 iterations (3 stage kernels each) of reinitialization
or constant-velocity advection, then the mean curvature.  The stage kernels
are k_stage<float|double, mode>; ncu can select them with -k regex:k_stage.
Mode adjoint runs the advection objective gradient of bench.adjoint_case
(`iters` steps, checkpoint every 4): forward stages k_stage_f32 / k_stage,
adjoint stages k_adj_xz and k_adj_y.
Mode band runs `iters` narrow-band curvature-flow steps of bench.band_case
at n^3 (rebuild every 5 steps, FP32).  Mode batched advects `n` grids of
bench.batched_case `iters` steps (persistent kernel in a CUDA graph).
Mode geometry runs bench.sub_geometry at n^3 with `iters` calls per entry
(volume, area, count; kernels k_row_sums and k_sum_parts).
"""
import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", choices=["reinit", "advect", "adjoint", "band", "batched", "geometry"], default="reinit")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--iters", type=int, default=1)
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32")
    ap.add_argument("--bc", type=int, default=2)
    a = ap.parse_args()
    import torch
    import lsmlib_gb300 as L
    from lsmlib_gb300 import build as B
    import bench
    B.build()
    L.set_stream(torch.cuda.current_stream().cuda_stream)
    gb, fb = bench.boxes(a.n)
    dt = torch.float32 if a.precision == "f32" else torch.float64
    if a.mode == "adjoint":
        phi0, vel, tgt, h, tstep = bench.adjoint_case(a.n)
        ghost = lambda v: torch.from_numpy(np.ascontiguousarray(np.pad(v, 3).T)).cuda().to(dt)
        J, gp, gv = L.advect_adjoint_weno5_tvdrk3(ghost(phi0), gb, fb, [ghost(v) for v in vel], gb, ghost(tgt), h,
                                                  tstep, a.iters, 1.5 * h, checkpoint_every=4,
                                                  precision=a.precision)
        torch.cuda.synchronize()
        L.check()
        print("ok", a.mode, a.n, a.iters, a.precision, "J", J, "launches", L.launch_count())
        return
    if a.mode == "geometry":
        r = bench.sub_geometry(torch.cuda.current_stream(), "cuda", n=a.n, reps=a.iters)
        L.check()
        print("ok", a.mode, a.n, {k: v["ms_per_call"] for k, v in r.items() if isinstance(v, dict)})
        return
    if a.mode == "band":
        phi, dx = bench.band_case("cuda", a.n)
        dts, bands = L.band_flow_weno5_tvdrk3(phi, gb, fb, dx, a.iters, 5, 6 * dx, 3 * dx, a_n=1.0, b_n=0.1,
                                              cfl=0.5, precision="f32")
        torch.cuda.synchronize()
        L.check()
        print("ok", a.mode, a.n, a.iters, "band cells", int(bands[0]), "launches", L.launch_count())
        return
    if a.mode == "batched":
        buf, offsets, dims, vel, spacing, tstep = bench.batched_case("cuda", a.n)
        L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, tstep, a.iters)
        torch.cuda.synchronize()
        L.check()
        print("ok", a.mode, a.n, "grids", a.iters, "steps", "launches", L.launch_count())
        return
    phi64, dx = bench.initial_phi(a.n)
    phi = torch.from_numpy(np.ascontiguousarray(phi64.T)).cuda().to(dt)
    kappa = torch.zeros_like(phi)
    if a.mode == "reinit":
        L.reinit_weno5_tvdrk3(phi, gb, fb, dx, 0.5 * dx, a.iters, use_phi0_for_sgn=1, bc=a.bc,
                              precision=a.precision)
    else:
        L.advect_weno5_tvdrk3(phi, gb, fb, dx, dx / 3.5, a.iters, vel_const=(1.0, 0.5, 0.25),
                              bc=a.bc, precision=a.precision)
    L.mean_curvature_o2(kappa, gb, phi, gb, fb, dx, precision=a.precision)
    torch.cuda.synchronize()
    L.check()
    print("ok", a.mode, a.n, a.iters, a.precision, "launches", L.launch_count())


if __name__ == "__main__":
    main()
