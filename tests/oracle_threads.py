"""LSMLIB's per-stage call sequences over whole grids on the host, split into
k-slabs over threads, for the parity tests at the workloads' own sizes.

Each LSMLIB routine of the sequence evaluates a cell-wise formula over its
fill box, so calling it once per k-slab of the fill box (each slab with its
own D1 scratch array) gives every cell exactly the arithmetic of one call
over the whole box (lsm3dZeroOutLevelSetEqnRHS, which clears its whole
ghost box, runs once per stage before the slabs); ctypes releases the
interpreter lock during a call, so the slabs run in parallel on the host
cores.  The ghost fill after each
stage runs once over the whole array, as in oracle_runs.tvdrk3_run, whose
results these runs reproduce bit for bit (tests/test_oracle_threads.py).
"""
import os
import threading

import numpy as np

import lsmlib_gb300 as L
from tests import harness as H
from tests import oracle_runs as O


def slabs(fb, threads):
    nk = fb[5] - fb[4] + 1
    t = max(1, min(threads, nk))
    edges = np.linspace(fb[4], fb[5] + 1, t + 1).astype(int)
    return [(int(edges[s]), int(edges[s + 1] - 1)) for s in range(t) if edges[s + 1] > edges[s]]


def parallel(fn, n):
    """Run fn(0) .. fn(n-1) on n threads; re-raise the first exception."""
    errs = []

    def run(s):
        try:
            fn(s)
        except BaseException as exc:  # noqa: BLE001 - re-raised below
            errs.append(exc)

    ths = [threading.Thread(target=run, args=(s,)) for s in range(n)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    if errs:
        raise errs[0]


def periodic_fill(phi, gb, fb):
    """The periodic images of oracle_runs.periodic_fill (the 3-layer shell
    around fb), as three axis passes of slab copies: each pass copies over
    the full shell extent of the other two axes, so edges and corners get
    the image of their wrapped interior cell, the same values."""
    o = [fb[2 * a] - gb[2 * a] for a in range(3)]       # array index of fb's first cell
    n = [fb[2 * a + 1] - fb[2 * a] + 1 for a in range(3)]
    for a in range(3):
        sl = [slice(o[b] - 3, o[b] + n[b] + 3) for b in range(3)]

        def at(lo, hi):
            s = list(sl)
            s[a] = slice(lo, hi)
            return tuple(s)
        for g in range(1, 4):
            src_lo = o[a] + (n[a] - g) % n[a]
            phi[at(o[a] - g, o[a] - g + 1)] = phi[at(src_lo, src_lo + 1)]
            src_hi = o[a] + (g - 1) % n[a]
            phi[at(o[a] + n[a] - 1 + g, o[a] + n[a] + g)] = phi[at(src_hi, src_hi + 1)]


def apply_bc(lib, phi, gb, fb, bc):
    if bc == L.BC_PERIODIC:
        periodic_fill(phi, gb, fb)
    else:
        O.apply_bc(lib, phi, gb, fb, bc)


class SlabRun:
    """TVD-RK3 runs of advection or reinitialization over the fill box fb of
    arrays over the ghost box gb (Fortran order, FP64)."""

    def __init__(self, lib, gb, fb, threads=None):
        self.lib, self.gb, self.fb = lib, gb, fb
        self.slabs = slabs(fb, threads or os.cpu_count() or 1)
        shape = H.shape_of(gb)
        z = lambda: np.zeros(shape, order="F")
        self.g = [z(), z(), z()]
        self.gm = [z(), z(), z()]
        self.rhs = z()
        self.d1 = []
        for k0, k1 in self.slabs:
            box = (fb[0] - 3, fb[1] + 3, fb[2] - 3, fb[3] + 3, k0 - 3, k1 + 3)
            self.d1.append((np.zeros(H.shape_of(box), order="F"), box))

    def _slab_fb(self, s):
        k0, k1 = self.slabs[s]
        f = self.fb
        return (f[0], f[1], f[2], f[3], k0, k1)

    def _call(self, sym, s, arrays, scalars, d1=False):
        boxes = {}
        if d1:
            arrays = dict(arrays, d1=self.d1[s][0])
            boxes["d1_gb"] = self.d1[s][1]
        vals, _ = H.make_call(sym, self.gb, self._slab_fb(s), arrays=arrays, scalars=scalars, boxes=boxes)
        L.invoke(self.lib, sym, vals)

    def _rhs(self, s, mode, phi, sp, vel, phi0, use0):
        dx, dy, dz = sp
        if mode == "reinit":
            self._call("lsm3dhjweno5_", s, {
                "phi": phi, "phi_x_plus": self.g[0], "phi_y_plus": self.g[1], "phi_z_plus": self.g[2],
                "phi_x_minus": self.gm[0], "phi_y_minus": self.gm[1], "phi_z_minus": self.gm[2]},
                {"dx": dx, "dy": dy, "dz": dz}, d1=True)
            self._call("lsm3dcomputereinitializationeqnrhs_", s, {
                "reinit_rhs": self.rhs, "phi": phi, "phi0": phi0, "phi_x_plus": self.g[0],
                "phi_y_plus": self.g[1], "phi_z_plus": self.g[2], "phi_x_minus": self.gm[0],
                "phi_y_minus": self.gm[1], "phi_z_minus": self.gm[2]},
                {"dx": dx, "dy": dy, "dz": dz, "use_phi0_for_sgn": use0})
            return
        self._call("lsm3dupwindhjweno5_", s, {
            "phi": phi, "phi_x": self.g[0], "phi_y": self.g[1], "phi_z": self.g[2],
            "vel_x": vel[0], "vel_y": vel[1], "vel_z": vel[2]}, {"dx": dx, "dy": dy, "dz": dz}, d1=True)
        # (lsm3dZeroOutLevelSetEqnRHS clears the whole ghost box, so run()
        # calls it once per stage before the slabs start)
        self._call("lsm3daddadvectiontermtolserhs_", s, {
            "lse_rhs": self.rhs, "phi_x": self.g[0], "phi_y": self.g[1], "phi_z": self.g[2],
            "vel_x": vel[0], "vel_y": vel[1], "vel_z": vel[2]}, {})

    def run(self, mode, phi, sp, dt, n_steps, bc, vel=None, use0=0):
        """n_steps TVD-RK3 steps ('advect' with velocity fields `vel`, or
        'reinit'); returns the new phi (input untouched)."""
        sp = sp if isinstance(sp, (tuple, list)) else (sp, sp, sp)
        phi = phi.copy(order="F")
        phi0 = phi.copy(order="F")
        n = len(self.slabs)
        for _ in range(n_steps):
            u1 = np.zeros_like(phi, order="F")
            u2 = np.zeros_like(phi, order="F")
            un = np.zeros_like(phi, order="F")

            def st1(s):
                self._rhs(s, mode, phi, sp, vel, phi0, use0)
                self._call("lsm3dtvdrk3stage1_", s, {"u_stage1": u1, "u_cur": phi, "rhs": self.rhs}, {"dt": dt})

            def st2(s):
                self._rhs(s, mode, u1, sp, vel, phi0, use0)
                self._call("lsm3dtvdrk3stage2_", s, {"u_stage2": u2, "u_stage1": u1, "u_cur": phi,
                                                      "rhs": self.rhs}, {"dt": dt})

            def st3(s):
                self._rhs(s, mode, u2, sp, vel, phi0, use0)
                self._call("lsm3dtvdrk3stage3_", s, {"u_next": un, "u_stage2": u2, "u_cur": phi,
                                                      "rhs": self.rhs}, {"dt": dt})

            for st, out in ((st1, u1), (st2, u2), (st3, un)):
                if mode != "reinit":
                    vals, _ = H.make_call("lsm3dzerooutlevelseteqnrhs_", self.gb, self.fb,
                                          arrays={"lse_rhs": self.rhs})
                    L.invoke(self.lib, "lsm3dzerooutlevelseteqnrhs_", vals)
                parallel(st, n)
                apply_bc(self.lib, out, self.gb, self.fb, bc)
            phi = un
        return phi

    def mean_curvature(self, phi, sp):
        """LSMLIB's curvature pass: second-order central gradient, |grad phi|
        and mean curvature over the fill box; returns (kappa, |grad phi|)."""
        dx, dy, dz = sp if isinstance(sp, (tuple, list)) else (sp, sp, sp)
        shape = H.shape_of(self.gb)
        kappa = np.zeros(shape, order="F")
        mag = np.zeros(shape, order="F")

        def one(s):
            self._call("lsm3dcentralgradorder2_", s, {"phi": phi, "phi_x": self.g[0], "phi_y": self.g[1],
                                                        "phi_z": self.g[2]}, {"dx": dx, "dy": dy, "dz": dz})
            self._call("lsm3dgradientmagnitude_", s, {"phi_x": self.g[0], "phi_y": self.g[1], "phi_z": self.g[2],
                                                       "grad_phi_mag": mag}, {})
            self._call("lsm3dcomputemeancurvatureorder2_", s, {
                "kappa": kappa, "phi": phi, "phi_x": self.g[0], "phi_y": self.g[1], "phi_z": self.g[2],
                "grad_phi_mag": mag}, {"dx": dx, "dy": dy, "dz": dz})

        parallel(one, len(self.slabs))
        return kappa, mag
