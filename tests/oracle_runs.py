"""Multi-step runs composed from the oracle's LSMLIB-signature routines, the
way LSMLIB's drivers compose them (per stage: derivatives -> RHS -> TVD-RK3
stage -> ghost fill).  These are the references the fused GPU steppers are
checked against."""
import numpy as np

import lsmlib_gb300 as L
from tests import harness as H

BC_FNS = {L.BC_LINEAR: "lsm3dlinearextrapolation_",
          L.BC_SIGNED_LINEAR: "lsm3dsignedlinearextrapolation_",
          L.BC_COPY: "lsm3dcopyextrapolation_"}

_BC_ABI = {
    name: {"args": [["phi", "real", True, True]] +
           [[n, "int", False, False] for n in
            ("ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb",
             "ilo_fb", "ihi_fb", "jlo_fb", "jhi_fb", "klo_fb", "khi_fb", "bdry_location_idx")]}
    for name in BC_FNS.values()}


def periodic_fill(phi, gb, fb):
    """Periodic images in the 3 ghost layers around fb (all faces, edges and
    corners), in place."""
    n = [fb[1] - fb[0] + 1, fb[3] - fb[2] + 1, fb[5] - fb[4] + 1]
    idx = []
    for a in range(3):
        lo, hi = fb[2 * a] - 3, fb[2 * a + 1] + 3
        full = np.arange(lo, hi + 1)
        src = (full - fb[2 * a]) % n[a] + fb[2 * a]
        idx.append((full - gb[2 * a], src - gb[2 * a]))
    (dx_, sx_), (dy_, sy_), (dz_, sz_) = idx
    phi[np.ix_(dx_, dy_, dz_)] = phi[np.ix_(sx_, sy_, sz_)].copy()


def apply_bc(lib, phi, gb, fb, bc):
    if bc == L.BC_PERIODIC:
        periodic_fill(phi, gb, fb)
        return
    name = BC_FNS[bc]
    for face in range(6):
        vals = {"phi": phi, "bdry_location_idx": face}
        for n_, v in zip(("ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb"), gb):
            vals[n_] = v
        for n_, v in zip(("ilo_fb", "ihi_fb", "jlo_fb", "jhi_fb", "klo_fb", "khi_fb"), fb):
            vals[n_] = v
        L.invoke(lib, name, vals, abi=_BC_ABI)


def _rhs(lib, mode, phi, gb, fb, dx, vel, phi0, use0):
    dx, dy, dz = dx if isinstance(dx, (tuple, list)) else (dx, dx, dx)
    shape = H.shape_of(gb)
    z = lambda: np.zeros(shape, order="F")
    if mode == "reinit":
        pp = [z(), z(), z()]
        pm = [z(), z(), z()]
        vals, _ = H.make_call("lsm3dhjweno5_", gb, fb, arrays={
            "phi": phi, "phi_x_plus": pp[0], "phi_y_plus": pp[1], "phi_z_plus": pp[2],
            "phi_x_minus": pm[0], "phi_y_minus": pm[1], "phi_z_minus": pm[2]},
            scalars={"dx": dx, "dy": dy, "dz": dz})
        L.invoke(lib, "lsm3dhjweno5_", vals)
        rhs = z()
        vals, _ = H.make_call("lsm3dcomputereinitializationeqnrhs_", gb, fb, arrays={
            "reinit_rhs": rhs, "phi": phi, "phi0": phi0, "phi_x_plus": pp[0],
            "phi_y_plus": pp[1], "phi_z_plus": pp[2], "phi_x_minus": pm[0],
            "phi_y_minus": pm[1], "phi_z_minus": pm[2]},
            scalars={"dx": dx, "dy": dy, "dz": dz, "use_phi0_for_sgn": use0})
        L.invoke(lib, "lsm3dcomputereinitializationeqnrhs_", vals)
        return rhs
    g = [z(), z(), z()]
    vals, _ = H.make_call("lsm3dupwindhjweno5_", gb, fb, arrays={
        "phi": phi, "phi_x": g[0], "phi_y": g[1], "phi_z": g[2],
        "vel_x": vel[0], "vel_y": vel[1], "vel_z": vel[2]}, scalars={"dx": dx, "dy": dy, "dz": dz})
    L.invoke(lib, "lsm3dupwindhjweno5_", vals)
    rhs = np.asfortranarray(np.random.default_rng(0).standard_normal(shape))
    vals, _ = H.make_call("lsm3dzerooutlevelseteqnrhs_", gb, fb, arrays={"lse_rhs": rhs})
    L.invoke(lib, "lsm3dzerooutlevelseteqnrhs_", vals)
    vals, _ = H.make_call("lsm3daddadvectiontermtolserhs_", gb, fb, arrays={
        "lse_rhs": rhs, "phi_x": g[0], "phi_y": g[1], "phi_z": g[2],
        "vel_x": vel[0], "vel_y": vel[1], "vel_z": vel[2]})
    L.invoke(lib, "lsm3daddadvectiontermtolserhs_", vals)
    return rhs


def tvdrk3_run(lib, mode, phi, gb, fb, dx, dt, n_steps, bc, vel=None, use0=0):
    """n_steps TVD-RK3 steps of advection ('advect', velocity fields `vel`)
    or reinitialization ('reinit'); returns the new phi (input untouched)."""
    phi = phi.copy(order="F")
    phi0 = phi.copy(order="F")
    for _ in range(n_steps):
        u1 = np.zeros_like(phi, order="F")
        rhs = _rhs(lib, mode, phi, gb, fb, dx, vel, phi0, use0)
        vals, _ = H.make_call("lsm3dtvdrk3stage1_", gb, fb, arrays={
            "u_stage1": u1, "u_cur": phi, "rhs": rhs}, scalars={"dt": dt})
        L.invoke(lib, "lsm3dtvdrk3stage1_", vals)
        apply_bc(lib, u1, gb, fb, bc)
        u2 = np.zeros_like(phi, order="F")
        rhs = _rhs(lib, mode, u1, gb, fb, dx, vel, phi0, use0)
        vals, _ = H.make_call("lsm3dtvdrk3stage2_", gb, fb, arrays={
            "u_stage2": u2, "u_stage1": u1, "u_cur": phi, "rhs": rhs}, scalars={"dt": dt})
        L.invoke(lib, "lsm3dtvdrk3stage2_", vals)
        apply_bc(lib, u2, gb, fb, bc)
        un = np.zeros_like(phi, order="F")
        rhs = _rhs(lib, mode, u2, gb, fb, dx, vel, phi0, use0)
        vals, _ = H.make_call("lsm3dtvdrk3stage3_", gb, fb, arrays={
            "u_next": un, "u_stage2": u2, "u_cur": phi, "rhs": rhs}, scalars={"dt": dt})
        L.invoke(lib, "lsm3dtvdrk3stage3_", vals)
        apply_bc(lib, un, gb, fb, bc)
        phi = un
    return phi


# ---------------------------------------------------------------------------
# narrow-band curvature flow: the LSMLIB *_local call sequence
# ---------------------------------------------------------------------------
def band_run(lib, phi, gb, fb, dx, n_steps, rebuild_every, gamma, beta, a_n, b_n, cfl, level=3):
    """n_steps TVD-RK3 steps of phi_t + Vn |grad phi| = 0 with Vn = a_n - b_n*kappa
    on a narrow band rebuilt every `rebuild_every` steps (width gamma, inner
    width beta, `level` neighbour levels).  Per stage, on level-0 cells:
    central gradient -> |grad phi| -> mean curvature (kappa) -> Vn;
    HJ WENO5 plus/minus on the band; Godunov normal-velocity RHS; cubic
    cut-off between beta and gamma; TVD-RK3 stage.  dt = CFL-stable normal
    velocity dt from stage 1 of each step.  Band levels 1..level of the stage
    fields hold phi^n (refreshed at each rebuild).  Returns (phi, dts, bands)."""
    shape = H.shape_of(gb)
    cap = int(np.prod(shape))
    phi = phi.copy(order="F")
    z = lambda: np.zeros(shape, order="F")
    nb = np.zeros(shape, np.uint8, order="F")
    ix, iy, iz = (np.zeros(cap, np.int32) for _ in range(3))
    outer = np.zeros(cap, np.int32)
    n_lo = np.zeros(level + 1, np.int32)
    n_hi = np.zeros(level + 1, np.int32)
    box6 = lambda prefix: {"%s%s%s" % (w, "_" + prefix if prefix else "", "_gb"): v
                           for w, v in zip(("ilo", "ihi", "jlo", "jhi", "klo", "khi"), gb)}
    u1, u2 = z(), z()
    dts, bands = [], []
    pp, pm = [z(), z(), z()], [z(), z(), z()]
    g3, mag, kap, vn, rhs, d1 = [z(), z(), z()], z(), z(), z(), z(), z()

    def lists(level0_only=True):
        return {"index_x": ix, "index_y": iy, "index_z": iz, "narrow_band": nb,
                "nlo_index": int(n_lo[0]), "nhi_index": int(n_hi[0])}

    def call(sym, arrays, scalars):
        vals, _ = H.make_call(sym, gb, fb, arrays=arrays, scalars=scalars)
        return L.invoke(lib, sym, vals)

    def rhs_of(src, want_dt):
        common = dict(lists())
        sc = {"dx": dx, "dy": dx, "dz": dx, "mark_fb": 1,
              "nlo_index": int(n_lo[0]), "nhi_index": int(n_hi[0])}
        call("lsm3dcentralgradorder2local_", dict(common, phi=src, phi_x=g3[0], phi_y=g3[1], phi_z=g3[2]), sc)
        call("lsm3dgradientmagnitudelocal_", dict(common, phi_x=g3[0], phi_y=g3[1], phi_z=g3[2],
                                                 grad_phi_mag=mag), sc)
        call("lsm3dcomputemeancurvatureorder2local_", dict(common, kappa=kap, phi=src, phi_x=g3[0],
                                                           phi_y=g3[1], phi_z=g3[2], grad_phi_mag=mag), sc)
        vn[...] = a_n - b_n * kap
        sw = dict(sc)
        for l in range(4):
            sw["nlo_index%d" % l] = int(n_lo[min(l, level)])
            sw["nhi_index%d" % l] = int(n_hi[min(l, level)])
        sw.update({"mark_d1": level + 1})
        call("lsm3dhjweno5local_", dict(common, phi=src, d1=d1, phi_x_plus=pp[0], phi_y_plus=pp[1],
                                        phi_z_plus=pp[2], phi_x_minus=pm[0], phi_y_minus=pm[1],
                                        phi_z_minus=pm[2]), sw)
        call("lsm3dzerooutlevelseteqnrhslocal_", dict(common, lse_rhs=rhs), sc)
        call("lsm3daddnormalveltermtolserhslocal_", dict(common, lse_rhs=rhs, phi_x_plus=pp[0],
                                                         phi_y_plus=pp[1], phi_z_plus=pp[2],
                                                         phi_x_minus=pm[0], phi_y_minus=pm[1],
                                                         phi_z_minus=pm[2], vel_n=vn), sc)
        dt = None
        if want_dt:
            out = call("lsm3dcomputestablenormalveldtlocal_", dict(common, vel_n=vn, phi_x_plus=pp[0],
                                                                   phi_y_plus=pp[1], phi_z_plus=pp[2],
                                                                   phi_x_minus=pm[0], phi_y_minus=pm[1],
                                                                   phi_z_minus=pm[2]),
                       dict(sc, cfl_number=cfl, dt=0.0))
            dt = out["dt"]
        call("lsm3dmultiplycutofflserhslocal_", dict(common, phi=src, lse_rhs=rhs),
             dict(sc, beta=beta, gamma=gamma))
        return dt

    for step in range(n_steps):
        if step % rebuild_every == 0:
            vals = {"phi": phi, "narrow_band": nb, "index_x": ix, "index_y": iy, "index_z": iz,
                    "nlo_index": 0, "nhi_index": cap - 1, "n_lo": n_lo, "n_hi": n_hi,
                    "index_outer": outer, "nlo_index_outer": 0, "nhi_index_outer": cap - 1,
                    "nlo_outer_plus": 0, "nhi_outer_plus": 0, "nlo_outer_minus": 0,
                    "nhi_outer_minus": 0, "width": gamma, "width_inner": beta, "level": level}
            for w, v in zip(("ilo_gb", "ihi_gb", "jlo_gb", "jhi_gb", "klo_gb", "khi_gb"), gb):
                vals[w] = v
                vals[w.replace("_gb", "_nb_gb")] = v
            L.invoke(lib, "lsm3ddeterminenarrowband_", vals)
            bands.append((nb.copy(), ix[:n_hi[level] + 1].copy(), iy[:n_hi[level] + 1].copy(),
                          iz[:n_hi[level] + 1].copy(), n_lo.copy(), n_hi.copy()))
            u1[...] = phi
            u2[...] = phi
        dt = rhs_of(phi, True)
        dts.append(dt)
        common = dict(lists())
        sc = {"dt": dt, "mark_fb": 1, "nlo_index": int(n_lo[0]), "nhi_index": int(n_hi[0])}
        call("lsm3dtvdrk3stage1local_", dict(common, u_stage1=u1, u_cur=phi, rhs=rhs), sc)
        rhs_of(u1, False)
        call("lsm3dtvdrk3stage2local_", dict(common, u_stage2=u2, u_stage1=u1, u_cur=phi, rhs=rhs), sc)
        rhs_of(u2, False)
        call("lsm3dtvdrk3stage3local_", dict(common, u_next=phi, u_stage2=u2, u_cur=phi, rhs=rhs), sc)
    return phi, dts, bands
