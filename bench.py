#!/usr/bin/env python3
"""Benchmark of the level-set hot path: reinitialization + mean curvature on a
256^3 grid (WENO5 / TVD-RK3), the workload LSMLIB's reinitialization drivers
run, in the GB300 FP32 form, with the FP64 form beside it.

Workload (one "step"): phi = (|x| - 0.5) * (0.1 + (x-0.3)^2 + (y-0.3)^2 +
(z+0.2)^2) on cell centres of [-1,1]^3, N = 256, dx = 2/N, 3 ghost cells;
20 pseudo-time TVD-RK3 iterations of the reinitialization equation with HJ
WENO5 plus/minus derivatives, dtau = 0.5 dx, smoothed sign from phi0
(epsilon = dx), signed linear extrapolation in the ghost cells after every
stage (the reference drivers' boundary condition); then second-order mean
curvature.  Unit of work: one interior cell advanced one full TVD-RK3
iteration (a cell-update).  Inputs are synthetic (seedless analytic field).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  --impl reference times the reference's own
CPU kernels (LSMLIB's Fortran translated to C under oracle/_ref, else the C
oracle) on the host cores for a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "WENO5+TVD-RK3 reinitialization cell-updates/s (256^3, 20 iterations + mean curvature)"
UNIT = "Gcell-updates/s"
N_DEFAULT = 256
ITERS = 20
GHOST = 3
# algorithmic bytes of the fused FP32 stage kernel per cell (phi0 sign form):
# stage 1 reads phi^n and phi0 and writes phi1 (12 B), stages 2 and 3 also
# read phi^n (16 B): 44 B per cell-update = 11 * 4 B
ALG_BYTES_PER_CELL_UPDATE = {"f32": 44.0, "f64": 88.0}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def boxes(n):
    fb = (0, n - 1, 0, n - 1, 0, n - 1)
    gb = (-GHOST, n - 1 + GHOST) * 3
    gb = (gb[0], gb[1], gb[0], gb[1], gb[0], gb[1])
    return gb, fb


def initial_phi(n):
    """Config-2 level set on cell centres x_i = -1 + (i + 1/2) dx, ghosts included."""
    dx = 2.0 / n
    c = -1.0 + (np.arange(-GHOST, n + GHOST) + 0.5) * dx
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    phi = (r - 0.5) * (0.1 + (X - 0.3) ** 2 + (Y - 0.3) ** 2 + (Z + 0.2) ** 2)
    return np.asfortranarray(phi), dx


def adjoint_case(n, seed=3, noise=0.05, shift=0.1, r=0.4):
    """The gradient workload (192^3 in its published form): periodic
    [-1, 1]^3 with n cells per axis, phi0 = sphere of radius r, target = the
    sphere shifted by `shift` in x, velocity (sin(pi y) cos(pi z),
    sin(pi z) cos(pi x), sin(pi x) cos(pi y)) plus N(0, noise) per cell
    (numpy seed `seed`), dt at CFL 0.5.  Returns interior arrays (Fortran
    order), the spacing and dt; the objective width is 1.5 dx."""
    h = 2.0 / n
    c = -1.0 + (np.arange(n) + 0.5) * h
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    phi = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - r
    tgt = np.sqrt((X - shift) ** 2 + Y ** 2 + Z ** 2) - r
    rng = np.random.default_rng(seed)
    base = (np.sin(np.pi * Y) * np.cos(np.pi * Z), np.sin(np.pi * Z) * np.cos(np.pi * X),
            np.sin(np.pi * X) * np.cos(np.pi * Y))
    vel = [b + rng.normal(0.0, noise, X.shape) for b in base]
    dt = 0.5 / float(np.max((np.abs(vel[0]) + np.abs(vel[1]) + np.abs(vel[2])) / h))
    f = np.asfortranarray
    return f(phi), [f(v) for v in vel], f(tgt), h, dt


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU reference sample (reference arm and cpu_baseline)
# ---------------------------------------------------------------------------
def cpu_library():
    """(ctypes handle, kind): the reference's own kernels translated to C when
    built (oracle/_ref), else the C oracle restatement."""
    ref = os.path.join(ROOT, "oracle", "_ref", "liblsmref.so")
    if not os.path.exists(ref):
        try:
            from oracle import build as ob
            ob.build()
        except Exception:
            pass
    if os.path.exists(ref):
        return ctypes.CDLL(ref, mode=ctypes.RTLD_LOCAL), "reference"
    orc = os.path.join(ROOT, "oracle", "liblsmoracle.so")
    if not os.path.exists(orc):
        from oracle import build as ob
        ob.build_oracle()
    return ctypes.CDLL(orc, mode=ctypes.RTLD_LOCAL), "port"


def _ip(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _dp(v):
    return ctypes.byref(ctypes.c_double(float(v)))


def _arr(a):
    return ctypes.c_void_p(a.ctypes.data)


class CpuReinit:
    """LSMLIB's reinitialization call sequence on the host, split into k-slabs
    over threads (ctypes releases the GIL): per stage each thread runs
    lsm3dhjweno5 -> lsm3dcomputereinitializationeqnrhs -> lsm3dtvdrk3stageN on
    its slab, then the six signed-linear-extrapolation face calls fill the
    ghost cells."""

    def __init__(self, lib, phi, gb, fb, dx, threads):
        self.lib, self.gb, self.fb, self.dx = lib, gb, fb, dx
        self.phi = phi.copy(order="F")
        self.phi0 = phi.copy(order="F")
        shape = phi.shape
        z = lambda: np.zeros(shape, order="F")
        self.u1, self.u2, self.un = z(), z(), z()
        self.pp = [z(), z(), z()]
        self.pm = [z(), z(), z()]
        self.rhs = z()
        nk = fb[5] - fb[4] + 1
        t = max(1, min(threads, nk))
        edges = np.linspace(fb[4], fb[5] + 1, t + 1).astype(int)
        self.slabs = [(edges[s], edges[s + 1] - 1) for s in range(t) if edges[s + 1] > edges[s]]
        nx, ny = fb[1] - fb[0] + 7, fb[3] - fb[2] + 7
        self.d1 = [np.zeros((nx, ny, (k1 - k0 + 7)), order="F") for k0, k1 in self.slabs]

    def _slab_stage(self, s, src, out, stage, dt):
        lib, gb, fb = self.lib, self.gb, self.fb
        k0, k1 = self.slabs[s]
        sfb = (fb[0], fb[1], fb[2], fb[3], k0, k1)
        dgb = (fb[0] - 3, fb[1] + 3, fb[2] - 3, fb[3] + 3, k0 - 3, k1 + 3)
        G = [_ip(v) for v in gb]
        F = [_ip(v) for v in sfb]
        D = [_ip(v) for v in dgb]
        dx = _dp(self.dx)
        lib.lsm3dhjweno5_(_arr(self.pp[0]), _arr(self.pp[1]), _arr(self.pp[2]), *G,
                          _arr(self.pm[0]), _arr(self.pm[1]), _arr(self.pm[2]), *G,
                          _arr(src), *G, _arr(self.d1[s]), *D, *F, dx, dx, dx)
        lib.lsm3dcomputereinitializationeqnrhs_(
            _arr(self.rhs), *G, _arr(src), *G, _arr(self.phi0), *G,
            _arr(self.pp[0]), _arr(self.pp[1]), _arr(self.pp[2]), *G,
            _arr(self.pm[0]), _arr(self.pm[1]), _arr(self.pm[2]), *G, *F, dx, dx, dx, _ip(1))
        if stage == 1:
            lib.lsm3dtvdrk3stage1_(_arr(out), *G, _arr(self.phi), *G, _arr(self.rhs), *G, *F, _dp(dt))
        elif stage == 2:
            lib.lsm3dtvdrk3stage2_(_arr(out), *G, _arr(src), *G, _arr(self.phi), *G, _arr(self.rhs), *G,
                                   *F, _dp(dt))
        else:
            lib.lsm3dtvdrk3stage3_(_arr(out), *G, _arr(src), *G, _arr(self.phi), *G, _arr(self.rhs), *G,
                                   *F, _dp(dt))

    def _bc(self, a):
        G = [_ip(v) for v in self.gb]
        F = [_ip(v) for v in self.fb]
        for face in range(6):
            self.lib.lsm3dsignedlinearextrapolation_(_arr(a), *G, *F, _ip(face))

    def _stage(self, src, out, stage, dt):
        ths = [threading.Thread(target=self._slab_stage, args=(s, src, out, stage, dt))
               for s in range(len(self.slabs))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        self._bc(out)

    def iterate(self, n, dt):
        for _ in range(n):
            self._stage(self.phi, self.u1, 1, dt)
            self._stage(self.u1, self.u2, 2, dt)
            self._stage(self.u2, self.un, 3, dt)
            self.phi, self.un = self.un, self.phi

    def reset(self, phi):
        self.phi[...] = phi
        self.phi0[...] = phi

    def _slab_curvature(self, s, kappa, mag):
        lib, gb, fb = self.lib, self.gb, self.fb
        k0, k1 = self.slabs[s]
        F = [_ip(v) for v in (fb[0], fb[1], fb[2], fb[3], k0, k1)]
        G = [_ip(v) for v in gb]
        dx = _dp(self.dx)
        g = self.pp
        lib.lsm3dcentralgradorder2_(_arr(g[0]), _arr(g[1]), _arr(g[2]), *G, _arr(self.phi), *G, *F, dx, dx, dx)
        lib.lsm3dgradientmagnitude_(_arr(g[0]), _arr(g[1]), _arr(g[2]), _arr(mag), *G, *F)
        lib.lsm3dcomputemeancurvatureorder2_(_arr(kappa), *G, _arr(self.phi), *G, _arr(g[0]), _arr(g[1]),
                                             _arr(g[2]), _arr(mag), *G, *F, dx, dx, dx)

    def curvature(self, kappa, mag):
        """LSMLIB's curvature pass on the current phi: second-order central
        gradient, |grad phi|, mean curvature (per k-slab)."""
        ths = [threading.Thread(target=self._slab_curvature, args=(s, kappa, mag))
               for s in range(len(self.slabs))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()


def cpu_sample(n, iters, threads, warmup=0):
    """Time `iters` reinitialization iterations of the full n^3 workload on the
    host; returns (cell-updates/s, seconds, kind)."""
    lib, kind = cpu_library()
    phi, dx = initial_phi(n)
    gb, fb = boxes(n)
    r = CpuReinit(lib, phi, gb, fb, dx, threads)
    if warmup:
        r.iterate(warmup, 0.5 * dx)
    t0 = time.perf_counter()
    r.iterate(iters, 0.5 * dx)
    sec = time.perf_counter() - t0
    return n ** 3 * iters / sec, sec, kind


# ---------------------------------------------------------------------------
# distributed helpers
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world, device):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def headline_config(n, world):
    return {"workload": "reinit-weno5-tvdrk3-256 + mean curvature", "n": n,
            "iterations": ITERS, "dtau": "0.5 dx", "sign": "phi0 form, eps = dx",
            "bc": "signed linear extrapolation", "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "inputs larger than L2 (4 x 79 MB padded FP32 fields per stage)"}


def reference_arm(args, world, rank):
    """The reference's own kernels (LSMLIB's Fortran translated to C, or the C
    oracle when the translation is absent) on the host: each step is the
    whole workload of the GPU arm's step (the 20 reinitialization iterations
    from the initial field, then the curvature pass), with every LSMLIB call
    split into k-slabs over all host threads by this script."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.n
    lib, kind = cpu_library()
    phi, dx = initial_phi(n)
    gb, fb = boxes(n)
    r = CpuReinit(lib, phi, gb, fb, dx, threads)
    kappa = np.zeros_like(phi, order="F")
    mag = np.zeros_like(phi, order="F")

    def step():
        r.reset(phi)
        r.iterate(ITERS, 0.5 * dx)
        r.curvature(kappa, mag)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    sec = time.perf_counter() - t0
    value = n ** 3 * ITERS * args.steps / sec / 1e9
    sample = ("the whole workload per step (%d reinitialization iterations of the %d^3 field + the curvature "
              "pass), LSMLIB's kernels called per k-slab over %d host threads by bench.py" % (ITERS, n, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic level set)",
        "config": dict(headline_config(n, 1), sample=sample),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def gpu_arm(args, world, rank, local):
    import torch
    import lsmlib_gb300 as L
    from lsmlib_gb300 import build as B
    B.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    h = L.lib()
    stream = torch.cuda.current_stream(dev)
    L.set_stream(stream.cuda_stream)

    n = args.n
    gb, fb = boxes(n)
    phi64, dx = initial_phi(n)
    dtau = 0.5 * dx
    bc = L.BC_SIGNED_LINEAR

    def dev_tensor(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev, dtype)

    pristine = dev_tensor(phi64, torch.float32)
    phi = torch.empty_like(pristine)
    kappa = torch.zeros_like(pristine)
    cells = n ** 3

    def step():
        phi.copy_(pristine)
        L.reinit_weno5_tvdrk3(phi, gb, fb, dx, dtau, ITERS, use_phi0_for_sgn=1, bc=bc, precision="f32")
        L.mean_curvature_o2(kappa, gb, phi, gb, fb, dx, precision="f32")

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    launches0 = L.launch_count()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    launches = L.launch_count() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, dev)
    value = world * cells * ITERS / (ms / 1e3) / 1e9

    # roofline of the dominant kernel (the fused reinitialization stage):
    # stage-only time from the difference of two runs with the workload's
    # boundary condition (each stage computes its face ghosts; one ghost fill
    # follows the last stage of a call), so the difference is 3*(n_b - n_a)
    # stage launches exactly
    def stage_time(iters, reps=3):
        best = None
        for _ in range(reps):
            phi.copy_(pristine)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            L.reinit_weno5_tvdrk3(phi, gb, fb, dx, dtau, iters, use_phi0_for_sgn=1, bc=bc, precision="f32")
            b.record(stream)
            torch.cuda.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        return best

    t1, t11 = stage_time(1), stage_time(11)
    stage_ms = (t11 - t1) / 30.0
    bytes_per_launch = ALG_BYTES_PER_CELL_UPDATE["f32"] / 3.0 * cells
    achieved = bytes_per_launch / (stage_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": MEASURED_STAGE_TRAFFIC,
                "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one stage-2 launch "
                                "(algorithmic 268.4 MB for that stage; achieved uses the 3-stage mean, 14.67 B/cell)",
                "kernel": "k_reinit_x2 (fused WENO5 + reinit RHS + TVD-RK3 stage, windows shared between "
                          "neighbouring cells, packed FP32x2)",
                "note": "the kernel is bound by arithmetic issue, not by DRAM (fp32_pipe below); see "
                        "profiles/k_reinit_x2_reinit_f32_256.md",
                "stage_ms": stage_ms, "peak_source": peak_kind}

    # end to end through the C ABI with host (pinned) buffers
    host_phi = torch.from_numpy(np.ascontiguousarray(phi64.T).astype(np.float32)).pin_memory()
    host_kappa = torch.zeros_like(host_phi).pin_memory()
    e2e_steps = max(1, min(args.steps, 10))
    # reinitialization works in place: the pinned input is restored from the
    # pristine host copy before each step, outside the step's timed interval
    host_work = host_phi.clone().pin_memory()

    def e2e_step():
        wk = host_work.numpy()
        L.reinit_weno5_tvdrk3(wk.ctypes.data, gb, fb, dx, dtau, ITERS, use_phi0_for_sgn=1, bc=bc,
                              precision="f32")
        L.mean_curvature_o2(host_kappa.numpy().ctypes.data, gb, wk.ctypes.data, gb, fb, dx,
                            precision="f32")

    host_work.copy_(host_phi)
    e2e_step()
    barrier(world)
    e2e_total = 0.0
    for q in range(e2e_steps):
        host_work.copy_(host_phi)
        t0 = time.perf_counter()
        e2e_step()
        e2e_total += time.perf_counter() - t0
    e2e_sec = e2e_total / e2e_steps
    e2e_sec = max_over_ranks(e2e_sec, world, dev)
    arr_bytes = host_phi.numel() * 4
    e2e = {"value": world * cells * ITERS / e2e_sec / 1e9, "unit": UNIT,
           # reinit: phi in and out; curvature: phi in, kappa out over the
           # fill box (the library copies back only the cells it writes)
           "h2d_bytes_per_step": 2 * arr_bytes, "d2h_bytes_per_step": arr_bytes + cells * 4}

    # FP64 parity form on the same workload, and the FP32 error against it
    phi_d64 = dev_tensor(phi64, torch.float64)
    kap64 = torch.zeros_like(phi_d64)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    L.reinit_weno5_tvdrk3(phi_d64, gb, fb, dx, dtau, ITERS, use_phi0_for_sgn=1, bc=bc, precision="f64")
    L.mean_curvature_o2(kap64, gb, phi_d64, gb, fb, dx, precision="f64")
    b.record(stream)
    torch.cuda.synchronize()
    ms64 = a.elapsed_time(b)
    step()
    torch.cuda.synchronize()
    inner = (slice(GHOST, -GHOST),) * 3
    p32 = phi.double().cpu().numpy()[inner]
    p64 = phi_d64.cpu().numpy()[inner]
    k32 = kappa.double().cpu().numpy()[inner]
    k64 = kap64.cpu().numpy()[inner]
    band = np.abs(p64) < 3 * dx
    err = {"phi_linf": float(np.max(np.abs(p32 - p64))), "phi_l1": float(np.mean(np.abs(p32 - p64))),
           "kappa_band_linf": float(np.max(np.abs(k32 - k64)[band])),
           "kappa_band_l1": float(np.mean(np.abs(k32 - k64)[band]))}
    fp64 = {"value": cells * ITERS / (ms64 / 1e3) / 1e9, "unit": UNIT, "ms_per_step": ms64,
            "fp32_speedup": ms64 / ms}

    # arithmetic roofs, against the device's FMA rates measured by the
    # library's probe kernels: the FP32 FMA pipe of the headline stage kernel
    # (its FMA-pipe instructions per cell-stage from one ncu capture, times
    # the live cell-stage rate, against the probe's FFMA2 instruction rate)
    # and the FP64 pipe of the parity form (FP64 operations per cell-update
    # from one ncu capture of a stage launch, times the live rate)
    fp32_lane_ops, fp64_fmas = L.measure_fma_rates()
    fp32_pipe = {"bound": "fp32 fma pipe", "unit": "FMA-pipe thread-instructions/s",
                 "peak": fp32_lane_ops / 2.0, "peak_source": "measured (FFMA2 probe, lsmgpu_measure_fma_rates)",
                 "instructions_per_cell_stage": MEASURED_FMA_PIPE_INSTR_PER_CELL_STAGE}
    fp32_pipe["achieved"] = MEASURED_FMA_PIPE_INSTR_PER_CELL_STAGE * cells / (stage_ms / 1e3)
    fp32_pipe["frac"] = fp32_pipe["achieved"] / fp32_pipe["peak"]
    roofline["fp32_pipe"] = fp32_pipe
    fp64["roofline"] = {"bound": "fp64 pipe", "unit": "FP64 operations/s", "peak": fp64_fmas,
                        "peak_source": "measured (DFMA probe, lsmgpu_measure_fma_rates)",
                        "fp64_ops_per_cell_update": MEASURED_FP64_OPS_PER_CELL_UPDATE}
    fp64["roofline"]["achieved"] = MEASURED_FP64_OPS_PER_CELL_UPDATE * cells * ITERS / (ms64 / 1e3)
    fp64["roofline"]["frac"] = fp64["roofline"]["achieved"] / fp64_fmas

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic level set of the reinitialization workload)",
        "config": headline_config(n, world),
        "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        "fp64": fp64, "fp32_error_vs_fp64": err,
    }
    if rank == 0 and not args.no_extra:
        line["other_workloads"] = {
            "advection_128": sub_advection(stream, dev),
            "narrow_band_512": sub_narrow_band(stream, dev),
            "batched_4096": sub_batched(stream, dev),
            "adjoint_192": sub_adjoint(stream, dev),
            "geometry_512": sub_geometry(stream, dev),
            "dropin_192": sub_dropin(stream, dev),
        }
    if rank == 0 and world == 1 and not args.no_cpu:
        # the reference's serial path (1 core), and the same kernels over
        # k-slabs on every host core beside it
        v, sec, kind = cpu_sample(n, 1, 1)
        line["cpu_baseline"] = {"value": v / 1e9, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": "1 reinitialization iteration of the %d^3 workload (%.1f s), serial, "
                                          "as the reference runs" % (n, sec)}
        threads = os.cpu_count() or 1
        v, sec, kind = cpu_sample(n, 1, threads)
        line["cpu_all_cores"] = {"value": v / 1e9, "unit": UNIT, "cores": threads, "kind": kind,
                                 "sample": "1 reinitialization iteration of the %d^3 workload (%.1f s), the "
                                           "reference's kernels called per k-slab over %d host threads by bench.py"
                                           % (n, sec, threads)}
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the other workloads of the hot path, each measured once per run
# ---------------------------------------------------------------------------
def _ev(stream):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _timed(fn, stream):
    import torch
    a, b = _ev(stream)
    torch.cuda.synchronize()
    a.record(stream)
    fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def advection_case(n=128):
    """Plain-method advection input on [-1, 1]^3: signed distance to a sphere
    of radius 0.35 at (0.1, -0.05, 0) on the cell centres (ghosts included),
    velocity (1, 0.5, 0.25), dt at CFL 0.5.  Returns (phi, vel, dt, dx)."""
    dx = 2.0 / n
    c = -1.0 + (np.arange(-GHOST, n + GHOST) + 0.5) * dx
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    phi = np.asfortranarray(np.sqrt((X - 0.1) ** 2 + (Y + 0.05) ** 2 + Z ** 2) - 0.35)
    vel = (1.0, 0.5, 0.25)
    dt = 0.5 * dx / sum(abs(v) for v in vel)
    return phi, vel, dt, dx


def sub_advection(stream, dev, n=128, steps=50):
    """Plain-method advection: 128^3 on [-1, 1]^3, periodic, signed distance
    to a sphere of radius 0.35 at (0.1, -0.05, 0), constant velocity
    (1, 0.5, 0.25), WENO5 / TVD-RK3 at CFL 0.5, 50 steps; FP64 parity form
    and FP32 form, and the FP32 error against FP64."""
    import torch
    import lsmlib_gb300 as L
    gb, fb = boxes(n)
    phi, vel, dt, dx = advection_case(n)
    out = {"workload": "advection-weno5-tvdrk3-128, sphere r=0.35, u=(1,0.5,0.25), CFL 0.5, 50 steps, periodic"}
    res = {}
    for prec, dtype in (("f64", torch.float64), ("f32", torch.float32)):
        t = torch.from_numpy(np.ascontiguousarray(phi.T)).to(dev, dtype)
        L.advect_weno5_tvdrk3(t, gb, fb, dx, dt, 1, vel_const=vel, precision=prec)  # warm-up
        t.copy_(torch.from_numpy(np.ascontiguousarray(phi.T)).to(dev, dtype))
        ms = _timed(lambda: L.advect_weno5_tvdrk3(t, gb, fb, dx, dt, steps, vel_const=vel, precision=prec), stream)
        res[prec] = t.double().cpu().numpy().T[GHOST:-GHOST, GHOST:-GHOST, GHOST:-GHOST]
        out[prec] = {"ms": ms, "Gcell_updates_per_s": n ** 3 * steps / (ms / 1e3) / 1e9}
    out["fp32_speedup"] = out["f64"]["ms"] / out["f32"]["ms"]
    d = np.abs(res["f32"] - res["f64"])
    near = np.abs(res["f64"]) < 3 * dx
    at = np.unravel_index(np.argmax(d), d.shape)
    out["fp32_error_vs_fp64"] = {"linf": float(d.max()), "l1": float(d.mean()),
                                 "linf_within_3dx_of_interface": float(d[near].max()),
                                 "linf_at_cell": [int(v) for v in at]}
    return out


def band_case(dev, n=512, n_spheres=64, seed=7, dtype=None):
    """Signed distance to the union of 64 spheres (centres U[-0.8, 0.8]^3,
    radii U[0.03, 0.10], numpy seed 7: centres drawn first, then radii) on
    the n^3 cell centres of [-1, 1]^3 with 3 ghost cells: a C-ordered CUDA
    tensor (FP32 unless `dtype` says otherwise) of the Fortran ghost-box
    array."""
    import torch
    dtype = dtype or torch.float32
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-0.8, 0.8, size=(n_spheres, 3))
    radii = rng.uniform(0.03, 0.10, size=n_spheres)
    dx = 2.0 / n
    c = -1.0 + (torch.arange(-GHOST, n + GHOST, device=dev, dtype=dtype) + 0.5) * dx
    z, y, x = c.view(-1, 1, 1), c.view(1, -1, 1), c.view(1, 1, -1)
    phi = torch.full((n + 2 * GHOST,) * 3, 1e30, device=dev, dtype=dtype)
    for (cx, cy, cz), r in zip(centres, radii):
        phi = torch.minimum(phi, torch.sqrt((x - float(cx)) ** 2 + (y - float(cy)) ** 2 + (z - float(cz)) ** 2)
                            - float(r))
    return phi, dx


def sub_narrow_band(stream, dev, n=512, steps=100, rebuild=5):
    """Narrow band: 512^3 on [-1, 1]^3 (band_case), band half-width 6 cells
    (inner width 3 cells), rebuilt every 5 steps, V_n = 1 - 0.1 kappa,
    WENO5 + TVD-RK3 on the band, 100 steps, FP32."""
    import lsmlib_gb300 as L
    gb, fb = boxes(n)
    phi, dx = band_case(dev, n)
    pristine = phi.clone()
    holder = {}

    def run(k=steps):
        holder["r"] = L.band_flow_weno5_tvdrk3(phi, gb, fb, dx, k, rebuild, 6 * dx, 3 * dx, a_n=1.0, b_n=0.1,
                                               cfl=0.5, precision="f32")
    run(1)  # warm-up: the library's device arena grows to this grid's buffers once
    phi.copy_(pristine)
    ms = _timed(run, stream)
    dts, bands = holder["r"]
    band_updates = int(sum(int(b) * min(rebuild, steps - i * rebuild) for i, b in enumerate(bands)))
    return {"workload": "narrow-band-512, 64 spheres (seed 7), half-width 6dx, rebuild every 5, "
                        "Vn = 1 - 0.1 kappa, 100 steps, FP32",
            "ms": ms, "band_cells_first_rebuild": int(bands[0]), "band_cell_updates": band_updates,
            "Gband_cell_updates_per_s": band_updates / (ms / 1e3) / 1e9,
            "grid_cell_updates_per_s_equivalent": n ** 3 * steps / (ms / 1e3) / 1e9}


def batched_params(n_grids=4096, seed=11, lo=16, hi=96):
    """Per-grid parameters of the batched workload: sides U{16..96} per axis,
    ellipsoid semi-axes U[0.2, 0.6], constant velocity U[-1, 1]^3 (numpy
    seed 11, drawn in that order), spacing 2 / side, dt at CFL 0.5."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(lo, hi + 1, size=(n_grids, 3))
    axes = rng.uniform(0.2, 0.6, size=(n_grids, 3))
    vel = rng.uniform(-1.0, 1.0, size=(n_grids, 3))
    spacing = 2.0 / dims
    dt = 0.5 / (np.abs(vel) / spacing).sum(axis=1)
    return dims, axes, vel, spacing, dt


def batched_case(dev, n_grids=4096, seed=11, lo=16, hi=96):
    """4096 grids (batched_params), each on [-1, 1]^3 with an ellipsoid level
    set (phi = (|x / a| - 1) min(a)) and a constant velocity.  Returns the
    packed FP32 CUDA buffer (3 ghost cells per grid), offsets, dims,
    velocities, spacings and dts."""
    import torch
    dims, axes, vel, spacing, dt = batched_params(n_grids, seed, lo, hi)
    sizes = np.prod(dims + 2 * GHOST, axis=1)
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    buf = torch.empty(int(sizes.sum()), device=dev, dtype=torch.float32)
    for g in range(n_grids):
        nx, ny, nz = (int(v) for v in dims[g])
        cs = [-1.0 + (torch.arange(-GHOST, m + GHOST, device=dev, dtype=torch.float32) + 0.5) * (2.0 / m)
              for m in (nx, ny, nz)]
        z, y, x = cs[2].view(-1, 1, 1), cs[1].view(1, -1, 1), cs[0].view(1, 1, -1)
        a = axes[g]
        f = (torch.sqrt((x / a[0]) ** 2 + (y / a[1]) ** 2 + (z / a[2]) ** 2) - 1.0) * float(a.min())
        buf[offsets[g]:offsets[g] + sizes[g]] = f.reshape(-1)
    return buf, offsets, dims, vel, spacing, dt


def sub_batched(stream, dev, n_grids=4096, steps=30):
    """Batched uneven grids (batched_case), periodic, WENO5 / TVD-RK3 at CFL
    0.5, 30 steps, FP32: one persistent launch per stage in a CUDA graph
    against one single-grid launch per grid per stage."""
    import lsmlib_gb300 as L
    buf, offsets, dims, vel, spacing, dt = batched_case(dev, n_grids)
    pristine = buf.clone()
    cells = int(np.prod(dims, axis=1).sum())
    out = {"workload": "batched-4096 uneven grids (sides U{16..96}, seed 11), ellipsoids, constant velocity, "
                       "30 steps, FP32", "grids": n_grids, "cells": cells}
    for name, flags in (("persistent_graph", 0), ("launch_loop", L.BATCH_LOOP)):
        buf.copy_(pristine)
        L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, dt, 1, flags=flags)  # tune / warm up
        buf.copy_(pristine)
        ms = _timed(lambda: L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, dt, steps, flags=flags),
                    stream)
        out[name] = {"ms": ms, "Gcell_updates_per_s": cells * steps / (ms / 1e3) / 1e9}
    out["speedup_vs_loop"] = out["launch_loop"]["ms"] / out["persistent_graph"]["ms"]
    return out


def sub_adjoint(stream, dev, n=192, steps=40, ckpt=8):
    """Gradient of J = sum (H(phi_T) - H(phi_target))^2 dx^3 after 40 periodic
    advection steps at 192^3 (adjoint_case), FP32 state, FP64 objective sum:
    objective-only time, full gradient time, and the cost of one reverse step
    (recomputation included) against one forward step — with the checkpoint
    spacing the library picks (the whole trajectory fits in HBM) and with a
    checkpoint every 8 steps."""
    import torch
    import lsmlib_gb300 as L
    phi, vel, tgt, h, dt = adjoint_case(n)
    gb, fb = boxes(n)
    dvc = lambda a: torch.from_numpy(np.ascontiguousarray(np.pad(a, GHOST).T)).to(dev, torch.float32)
    P, V, T = dvc(phi), [dvc(v) for v in vel], dvc(tgt)
    eps = 1.5 * h

    def measure(k):
        run = lambda grads: L.advect_adjoint_weno5_tvdrk3(P, gb, fb, V, gb, T, h, dt, steps, eps, checkpoint_every=k,
                                                          precision="f32", grads=grads)
        run(False)
        run(True)
        t_f = min(_timed(lambda: run(False), stream) for _ in range(3))
        t_g = min(_timed(lambda: run(True), stream) for _ in range(3))
        return {"objective_ms": t_f, "gradient_ms": t_g, "forward_step_ms": t_f / steps,
                "reverse_step_ms": (t_g - t_f) / steps, "reverse_to_forward_step": (t_g - t_f) / t_f}

    out = {"workload": "adjoint-192: 40 advection steps, sphere r=0.4, velocity field + N(0,0.05) (seed 3), "
                       "J with H_eps (eps=1.5dx), FP32 state / FP64 objective accumulation"}
    # checkpoint spacing chosen by the library: the 120 stage states of this
    # run (4.2 GB) fit in HBM, so the forward sweep keeps them all
    out.update(measure(0))
    out["checkpoint"] = "library-chosen (whole trajectory kept, nothing recomputed)"
    # checkpoint every 8 steps: the first four segments are recomputed
    out["checkpoint_every_%d" % ckpt] = measure(ckpt)
    return out



DROPIN_ROUTINES = ("lsm3dhjweno5_", "lsm3dupwindhjweno5_", "lsm3dtvdrk3stage2_",
                   "lsm3dcomputereinitializationeqnrhs_")


def dropin_values(sym, n, make):
    """Arguments of a drop-in routine over the n^3 fill box with 3 ghost cells:
    every array over the ghost box from `make(shape)`, LSMLIB's default
    spacings and scalars."""
    import lsmlib_gb300 as L
    gb = (-GHOST, n - 1 + GHOST)
    shape = (n + 2 * GHOST,) * 3
    names = ("ilo", "ihi", "jlo", "jhi", "klo", "khi")
    sc = {"dx": 2.0 / n, "dy": 2.0 / n, "dz": 2.0 / n, "dt": 0.4 / n, "use_phi0_for_sgn": 1}
    vals = {}
    for name, kind, is_arr, written in L.ABI[sym]["args"]:
        pre = name[:3]
        if is_arr:
            vals[name] = make(shape)
        elif pre in names and not is_arr:
            fill = name.endswith("_fb") or name[4:] == "fb"
            lo_hi = (0, n - 1) if fill else gb
            vals[name] = lo_hi[pre[1:] == "hi"]
        else:
            vals[name] = sc[name]
    return vals


def sub_dropin(stream, dev, n=192, reps=5):
    """LSMLIB's dense drop-in routines through the C ABI (FP64) on host
    arrays (staged: inputs copied in, outputs' fill box copied back, the call
    returns when done) and on device arrays (used in place), n^3 fill box."""
    import torch
    import lsmlib_gb300 as L
    lib = L.lib()
    rng = np.random.default_rng(5)
    out = {"workload": "dropin-%d: %s, FP64, random fields over the ghost box" % (n, ", ".join(DROPIN_ROUTINES))}
    for sym in DROPIN_ROUTINES:
        host = dropin_values(sym, n, lambda sh: np.asfortranarray(rng.standard_normal(sh)))
        L.invoke(lib, sym, host)
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            L.invoke(lib, sym, host)
            ts.append(time.perf_counter() - t0)
        devv = {k: (torch.from_numpy(np.ascontiguousarray(v.T)).to(dev) if isinstance(v, np.ndarray) else v)
                for k, v in host.items()}
        L.invoke(lib, sym, devv)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            L.invoke(lib, sym, devv)
        e1.record(stream)
        torch.cuda.synchronize()
        out[sym] = {"host_arrays_ms": 1e3 * sorted(ts)[reps // 2], "device_arrays_ms": e0.elapsed_time(e1) / reps}
    return out


def sub_geometry(stream, dev, n=512, reps=10):
    """Geometry reductions through the drop-in C entry points on device
    arrays (FP64): volume of {phi < 0}, area of {phi = 0} and the count of
    phi < 0 cells over the 512^3 box of a sphere's signed distance (radius
    0.5, 3 ghost cells, smoothing width 1.5 dx) with its exact gradient.
    Each call returns its scalar to the host, so a call's time includes that
    copy.  Algorithmic bytes: phi once (8 B/cell), plus the gradient (24 B)
    at the cells inside the smoothing band for the area."""
    import torch
    import lsmlib_gb300 as L
    lib = L.lib()
    dx = 2.0 / n
    c = -1.0 + (torch.arange(-GHOST, n + GHOST, device=dev, dtype=torch.float64) + 0.5) * dx
    z, y, x = c.view(-1, 1, 1), c.view(1, -1, 1), c.view(1, 1, -1)
    d = torch.sqrt(x * x + y * y + z * z).clamp_min(1e-12)
    phi = d - 0.5
    grads = [(x / d).contiguous(), (y / d).contiguous(), (z / d).contiguous()]
    del d
    eps = 1.5 * dx
    gb = (-GHOST, n - 1 + GHOST) * 3
    ib = (0, n - 1) * 3
    band = int((phi[GHOST:-GHOST, GHOST:-GHOST, GHOST:-GHOST].abs() < eps).sum())
    cells = n ** 3
    peak, src = measured_peaks()
    out = {"workload": "geometry-512: sphere r=0.5 signed distance on [-1, 1]^3, FP64, eps = 1.5 dx, "
                       "device arrays, scalar result copied to the host per call",
           "band_cells": band}

    def vals(sym):
        arrays = {"phi": phi, "phi_x": grads[0], "phi_y": grads[1], "phi_z": grads[2]}
        scalars = {"dx": dx, "dy": dx, "dz": dx, "epsilon": eps, "volume": 0.0, "area": 0.0, "count": 0}
        v = {}
        for name, kind, is_arr, _w in L.ABI[sym]["args"]:
            if is_arr:
                v[name] = arrays[name]
            elif name in scalars:
                v[name] = scalars[name]
            else:
                b = ib if name.endswith("_ib") else gb
                v[name] = b[["ilo", "ihi", "jlo", "jhi", "klo", "khi"].index(name[:3])]
        return v

    cases = (("volume", "lsm3dvolumeregionphilessthanzero_", 8.0 * cells),
             ("area", "lsm3dsurfaceareazerolevelset_", 8.0 * cells + 24.0 * band),
             ("count", "lsm3dvoxelcountlessthanzero_", 8.0 * cells))
    for key, sym, nbytes in cases:
        v = vals(sym)
        res = L.invoke(lib, sym, v)   # warm-up
        L.check(lib)
        ms = min(_timed(lambda: [L.invoke(lib, sym, v) for _ in range(reps)], stream) for _ in range(3)) / reps
        gbs = nbytes / (ms / 1e3) / 1e9
        out[key] = {"entry": sym, "ms_per_call": ms, "result": res[L.ABI[sym]["args"][0][0]],
                    "Gcells_per_s": cells / (ms / 1e3) / 1e9, "algorithmic_GBps": gbs,
                    "hbm_frac": gbs / peak, "peak_source": src}
    out["volume"]["exact"] = 4.0 / 3.0 * np.pi * 0.5 ** 3
    out["area"]["exact"] = 4.0 * np.pi * 0.5 ** 2
    return out


# DRAM bytes (read + write) of one fused FP32 reinitialization stage launch
# at 256^3, from one ncu capture of a stage-2 launch of k_reinit_x2
# (profiles/k_reinit_x2_reinit_f32_256.md: 233.1 + 51.5 MB; the stage's
# algorithmic bytes are 16 B/cell = 268.4 MB)
MEASURED_STAGE_TRAFFIC = 284.6e6

# FMA-pipe thread-instructions (a packed FFMA2 / FMUL2 / FADD2 counts once)
# per cell of one headline stage launch (k_reinit_x2, ncu
# sm__inst_executed_pipe_fma.sum x 32 / 256^3 cells), and FP64 pipe
# operations (DFMA + DMUL + DADD thread-instructions, the IEEE division and
# square-root sequences included) per cell-update of the FP64 parity form
# (3 x one stage launch of k_stage<double, REINIT> at 128^3); both from the
# captures summarised in profiles/k_reinit_x2_reinit_f32_256.md
MEASURED_FMA_PIPE_INSTR_PER_CELL_STAGE = 119.9
MEASURED_FP64_OPS_PER_CELL_UPDATE = 3 * 633.5


# ---------------------------------------------------------------------------
# one call of a hot-path workload on cuda:0, for profilers (--case)
# ---------------------------------------------------------------------------
def profile_case(a):
    """One fused call on cuda:0 (no timing): `--case reinit|advect` runs
    `--iters` WENO5 / TVD-RK3 iterations of the headline field at n^3 then the
    mean curvature (kernels k_stage*); `adjoint` the objective gradient of
    adjoint_case (checkpoint every 4; k_adj_x_x2, k_adj_march_x2); `band`
    `--iters` narrow-band steps of band_case (rebuild every 5, FP32);
    `batched` `--iters` steps of n grids of batched_case; `geometry`
    sub_geometry at n^3 with `--iters` calls per entry point."""
    import torch
    import lsmlib_gb300 as L
    from lsmlib_gb300 import build as B
    B.build()
    L.set_stream(torch.cuda.current_stream().cuda_stream)
    gb, fb = boxes(a.n)
    dt = torch.float32 if a.precision == "f32" else torch.float64
    if a.case == "adjoint":
        phi0, vel, tgt, h, tstep = adjoint_case(a.n)
        ghost = lambda v: torch.from_numpy(np.ascontiguousarray(np.pad(v, 3).T)).cuda().to(dt)
        J, _, _ = L.advect_adjoint_weno5_tvdrk3(ghost(phi0), gb, fb, [ghost(v) for v in vel], gb, ghost(tgt), h,
                                                tstep, a.iters, 1.5 * h, checkpoint_every=4, precision=a.precision)
        info = "J %r" % J
    elif a.case == "geometry":
        r = sub_geometry(torch.cuda.current_stream(), "cuda", n=a.n, reps=a.iters)
        info = str({k: v["ms_per_call"] for k, v in r.items() if isinstance(v, dict)})
    elif a.case == "band":
        phi, dx = band_case("cuda", a.n)
        _, bands = L.band_flow_weno5_tvdrk3(phi, gb, fb, dx, a.iters, 5, 6 * dx, 3 * dx, a_n=1.0, b_n=0.1, cfl=0.5,
                                            precision="f32")
        info = "band cells %d" % int(bands[0])
    elif a.case == "batched":
        buf, offsets, dims, vel, spacing, tstep = batched_case("cuda", a.n)
        L.advect_batch_weno5_tvdrk3(buf, offsets, dims, vel, spacing, tstep, a.iters)
        info = "%d grids" % a.n
    else:
        phi64, dx = initial_phi(a.n)
        phi = torch.from_numpy(np.ascontiguousarray(phi64.T)).cuda().to(dt)
        kappa = torch.zeros_like(phi)
        if a.case == "reinit":
            L.reinit_weno5_tvdrk3(phi, gb, fb, dx, 0.5 * dx, a.iters, use_phi0_for_sgn=1, bc=a.bc,
                                  precision=a.precision)
        else:
            L.advect_weno5_tvdrk3(phi, gb, fb, dx, dx / 3.5, a.iters, vel_const=(1.0, 0.5, 0.25), bc=a.bc,
                                  precision=a.precision)
        L.mean_curvature_o2(kappa, gb, phi, gb, fb, dx, precision=a.precision)
        info = ""
    torch.cuda.synchronize()
    L.check()
    print("ok", a.case, a.n, a.iters, a.precision, info, "launches", L.launch_count())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--no-extra", action="store_true", help="skip the other workloads")
    ap.add_argument("--case", choices=["reinit", "advect", "adjoint", "band", "batched", "geometry"],
                    help="run one call of that workload for a profiler instead of the benchmark")
    ap.add_argument("--iters", type=int, default=1, help="iterations / steps / calls of --case")
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32", help="precision of --case")
    ap.add_argument("--bc", type=int, default=2, help="boundary condition of --case reinit / advect")
    args = ap.parse_args()
    if args.case:
        profile_case(args)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        gpu_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
