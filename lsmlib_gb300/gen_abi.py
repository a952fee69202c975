#!/usr/bin/env python3
"""Maintainer tool: regenerate include/lsmgpu_toolbox{3d,2d,1d}.h,
lsmlib_gb300/abi.json and lsmlib_gb300/csrc/lifted.cu for the drop-in entry
points this library implements.

The 2D and 1D entry points run the 3D routines on their arrays (see
csrc/lift.cuh); lifted.cu holds one generated wrapper per routine that maps
its arguments onto the 3D routine's by position: missing array components
become stand-in buffers, missing k (and j) bounds 0, a missing dz (and dy)
the caller's dx (1 where the routine multiplies a cell volume).  A 2D / 1D
routine is lifted when its 3D counterpart is implemented, every one of its
arguments finds its place and its arithmetic is the 3D routine's with the
missing terms removed (NOT_LIFTED lists the exceptions).

The argument lists come from the signature dump that oracle/f77ref.py writes
when it translates the reference's Fortran (oracle/_ref/sigs.json, produced
by `python -m oracle.build`), so every declaration has the reference
routine's exact argument order; the C-header line cited beside each comes
from the reference tree's own headers (searched under $LSMLIB_REFERENCE_TREE/src).

    python -m lsmlib_gb300.gen_abi
"""
import json
import os
import re
import subprocess

REF = os.environ.get("LSMLIB_REFERENCE_TREE", "/root/reference")
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# symbol -> (header group, one-line description)
DESC = {
    # spatial derivatives
    "lsm3dhjeno1_": ("deriv", "first-order HJ ENO plus/minus gradients"),
    "lsm3dhjeno2_": ("deriv", "second-order HJ ENO plus/minus gradients"),
    "lsm3dhjeno3_": ("deriv", "third-order HJ ENO plus/minus gradients"),
    "lsm3dhjweno5_": ("deriv", "fifth-order HJ WENO plus/minus gradients"),
    "lsm3dupwindhjeno1_": ("deriv", "first-order upwind HJ ENO gradient for a velocity field"),
    "lsm3dupwindhjeno2_": ("deriv", "second-order upwind HJ ENO gradient"),
    "lsm3dupwindhjeno3_": ("deriv", "third-order upwind HJ ENO gradient"),
    "lsm3dupwindhjweno5_": ("deriv", "fifth-order upwind HJ WENO gradient"),
    "lsm3dcentralgradorder2_": ("deriv", "second-order central gradient"),
    "lsm3dcentralgradorder4_": ("deriv", "fourth-order central gradient"),
    "lsm3dlaplacianorder2_": ("deriv", "second-order Laplacian"),
    "lsm3dgradientmagnitude_": ("deriv", "|grad phi| with the reference's 1e-8 clamps"),
    "lsm3dcomputedn_": ("deriv", "n-th undivided difference along dir (1e10 outside the fill range)"),
    "lsm3ddeltafunctionorder1_": ("deriv", "first-order delta function from sign changes (z terms use norm_phi_x and 1/dx, as the reference does)"),
    # RK
    "lsm3drk1step_": ("rk", "forward Euler step u_next = u + dt*L"),
    "lsm3dtvdrk2stage1_": ("rk", "TVD RK2 stage 1 (an Euler step)"),
    "lsm3dtvdrk2stage2_": ("rk", "TVD RK2 stage 2: 0.5*(u + u1 + dt*L)"),
    "lsm3dtvdrk3stage1_": ("rk", "TVD RK3 stage 1 (an Euler step)"),
    "lsm3dtvdrk3stage2_": ("rk", "TVD RK3 stage 2: 0.75*u + 0.25*(u1 + dt*L)"),
    "lsm3dtvdrk3stage3_": ("rk", "TVD RK3 stage 3: u/3 + 2/3*(u2 + dt*L)"),
    # LSE
    "lsm3dzerooutlevelseteqnrhs_": ("lse", "zero the level set equation RHS over its ghost box"),
    "lsm3daddadvectiontermtolserhs_": ("lse", "rhs -= u . grad(phi)"),
    "lsm3daddnormalveltermtolserhs_": ("lse", "rhs -= Vn |grad phi| (Godunov), Vn a field"),
    "lsm3daddconstnormalveltermtolserhs_": ("lse", "rhs -= Vn |grad phi| (Godunov), Vn constant"),
    "lsm3daddconstcurvtermtolserhs_": ("lse", "rhs += b * kappa |grad phi| from first and second derivatives"),
    # reinit / curvature
    "lsm3dcomputereinitializationeqnrhs_": ("reinit", "reinitialization RHS sgn(phi)(1 - |grad phi|), Godunov"),
    "lsm3dcomputeorthogonalizationeqnrhs_": ("reinit", "orthogonalization RHS: grad(phi) upwinded along sgn(psi) grad(psi)"),
    "lsm3dcomputedistanceforsubcellfix_": ("reinit", "distance estimate next to sign changes of phi0 for the subcell fix (-1000 max(dx) elsewhere)"),
    "lsm3dcomputereinitializationeqnrhssubcellfixorder1_": ("reinit", "first-order reinitialization RHS with the Russo-Smereka subcell fix"),
    "lsm3dcomputemeancurvatureorder2_": ("geom", "second-order mean curvature"),
    "lsm3dcomputegaussiancurvatureorder2_": ("geom", "second-order Gaussian curvature"),
    "lsm3dcomputemeancurvatureorder4_": ("geom", "fourth-order mean curvature (cross derivatives from the first derivatives)"),
    "lsm3dcomputegaussiancurvatureorder4_": ("geom", "fourth-order Gaussian curvature (cross derivatives from the first derivatives)"),
    # reductions
    "lsm3dmaxnormdiff_": ("red", "max |field1 - field2| over an index box"),
    "lsm3dcomputestableadvectiondt_": ("red", "CFL-stable dt for advection"),
    "lsm3dcomputestablenormalveldt_": ("red", "CFL-stable dt for a normal velocity field"),
    "lsm3dcomputestableconstnormalveldt_": ("red", "CFL-stable dt for a constant normal velocity"),
    "lsm3daveabsdiff_": ("red", "mean |field1 - field2| over an index box"),
    "lsm3dvoxelcountgreaterthanzero_": ("red", "number of cells with phi > 0"),
    "lsm3dvoxelcountlessthanzero_": ("red", "number of cells with phi < 0"),
    "lsm3dvolumeintegralphilessthanzero_": ("red", "integral of F over {phi < 0} with a smoothed Heaviside"),
    "lsm3dvolumeintegralphigreaterthanzero_": ("red", "integral of F over {phi > 0} with a smoothed Heaviside"),
    "lsm3dsurfaceintegral_": ("red", "integral of F over {phi = 0} with a smoothed delta"),
    "lsm3dmaxnormdiffcontrolvolume_": ("red", "max |field1 - field2| over cells of one control-volume sign (seeded with the box corner)"),
    "lsm3dcomputestableadvectiondtcontrolvolume_": ("red", "CFL-stable advection dt over cells of one control-volume sign"),
    "lsm3dcomputestablenormalveldtcontrolvolume_": ("red", "CFL-stable normal-velocity dt over cells of one control-volume sign"),
    "lsm3dcomputestableconstnormalveldtcontrolvolume_": ("red", "CFL-stable constant normal-velocity dt over cells of one control-volume sign"),
    "lsm3dvolumeintegralphilessthanzerocontrolvolume_": ("red", "volume integral over {phi < 0} restricted to one control-volume sign"),
    "lsm3dvolumeintegralphigreaterthanzerocontrolvolume_": ("red", "volume integral over {phi > 0} restricted to one control-volume sign"),
    "lsm3dsurfaceintegralcontrolvolume_": ("red", "surface integral restricted to one control-volume sign"),
    "lsm3dvoxelcountgreaterthanzerocontrolvolume_": ("red", "number of cells with phi > 0 and the selected control-volume sign"),
    "lsm3dvoxelcountlessthanzerocontrolvolume_": ("red", "number of cells with phi < 0 and the selected control-volume sign"),
    # geometry
    "lsm3dcomputeunitnormal_": ("geo", "unit normal grad phi / |grad phi| ((1,0,0) where |grad phi| < zero_tol)"),
    "lsm3dcomputesignedunitnormal_": ("geo", "sgn(phi) grad phi / |grad phi| with the smoothed sign"),
    "lsm3dcomputemeancurvature_": ("geo", "mean curvature from first and second derivatives"),
    "lsm3dvolumeregionphilessthanzero_": ("geo", "volume of {phi < 0} with a smoothed Heaviside"),
    "lsm3dvolumeregionphigreaterthanzero_": ("geo", "volume of {phi > 0} with a smoothed Heaviside"),
    "lsm3dsurfaceareazerolevelset_": ("geo", "area of {phi = 0} with a smoothed delta"),
    "lsm3dsurfaceareazerolevelsetdelta_": ("geo", "area of {phi = 0} from a precomputed delta function"),
    "lsm3dvolumeregionphilessthanzerocontrolvolume_": ("geo", "volume of {phi < 0} over one control-volume sign"),
    "lsm3dvolumeregionphigreaterthanzerocontrolvolume_": ("geo", "volume of {phi > 0} over one control-volume sign"),
    "lsm3dsurfaceareazerolevelsetcontrolvolume_": ("geo", "area of {phi = 0} over one control-volume sign"),
    "lsm3dsurfaceareazerolevelsetdeltacontrolvolume_": ("geo", "area of {phi = 0} from a delta function over one control-volume sign"),
    # extra dense
    "lsm3dcentralhessian_": ("deriv", "second-order central Hessian"),
    "lsm3daveragegradphi_": ("deriv", "average of plus and minus gradients"),
    "lsm3dphiupwindgradf_": ("deriv", "gradient of F upwinded by the local extremum of phi"),
    "lsm3daddconstprecomputedcurvtermtolserhs_": ("lse", "rhs += b * kappa * |grad phi| (loops k,j from the fill box to the ghost box end and i over the ghost box, as the reference does)"),
    "lsm3daddexternalandnormalveltermtolserhs_": ("lse", "rhs -= u . grad(phi) + Vn |grad phi| with the combined Godunov upwinding (same loop bounds as the reference)"),
    # boundary conditions
    "lsm3dlinearextrapolation_": ("bc", "linear extrapolation into the ghost cells of one face"),
    "lsm3dsignedlinearextrapolation_": ("bc", "signed linear extrapolation into the ghost cells of one face"),
    "lsm3dcopyextrapolation_": ("bc", "copy extrapolation into the ghost cells of one face"),
    "lsm3dhomogeneousneumanneno1_": ("bc", "homogeneous Neumann fill for ENO1 (copy extrapolation)"),
    "lsm3dhomogeneousneumanneno2_": ("bc", "homogeneous Neumann fill for ENO2 (copy extrapolation)"),
    "lsm3dhomogeneousneumanneno3_": ("bc", "homogeneous Neumann fill for ENO3 (copy extrapolation)"),
    "lsm3dhomogeneousneumannweno5_": ("bc", "homogeneous Neumann fill for WENO5 (copy extrapolation)"),
    # local derivatives
    "lsm3dcomputednlocal_": ("local", "n-th undivided differences over an index list"),
    "lsm3dhjeno1local_": ("local", "HJ ENO1 plus/minus gradients on level-0 band cells"),
    "lsm3dhjeno2local_": ("local", "HJ ENO2 plus/minus gradients on level-0 band cells"),
    "lsm3dhjeno3local_": ("local", "HJ ENO3 plus/minus gradients on level-0 band cells"),
    "lsm3dhjweno5local_": ("local", "HJ WENO5 plus/minus gradients on level-0 band cells"),
    "lsm3dupwindhjeno2local_": ("local", "upwind HJ ENO2 gradient for a velocity field on level-0 band cells"),
    "lsm3dcentralgradorder2local_": ("local", "second-order central gradient on band cells"),
    "lsm3dcentralgradorder4local_": ("local", "fourth-order central gradient on band cells"),
    "lsm3dlaplacianorder2local_": ("local", "second-order Laplacian on band cells"),
    "lsm3dcomputeavegradphilocal_": ("local", "average |grad phi| over band cells"),
    "lsm3dgradientmagnitudelocal_": ("local", "|grad phi| on band cells (zero_tol clamps)"),
    # local RK
    "lsm3drk1steplocal_": ("local", "Euler step on band cells"),
    "lsm3dtvdrk2stage1local_": ("local", "TVD RK2 stage 1 on band cells"),
    "lsm3dtvdrk2stage2local_": ("local", "TVD RK2 stage 2 on band cells"),
    "lsm3dtvdrk3stage1local_": ("local", "TVD RK3 stage 1 on band cells"),
    "lsm3dtvdrk3stage2local_": ("local", "TVD RK3 stage 2 on band cells"),
    "lsm3dtvdrk3stage3local_": ("local", "TVD RK3 stage 3 on band cells"),
    # local LSE
    "lsm3dzerooutlevelseteqnrhslocal_": ("local", "zero the RHS on listed cells"),
    "lsm3daddadvectiontermtolserhslocal_": ("local", "advection term on band cells"),
    "lsm3daddnormalveltermtolserhslocal_": ("local", "normal velocity term (field) on band cells"),
    "lsm3daddconstnormalveltermtolserhslocal_": ("local", "normal velocity term (constant) on band cells"),
    "lsm3daddconstcurvtermtolserhslocal_": ("local", "curvature term on band cells"),
    "lsm3dcomputereinitializationeqnrhslocal_": ("local", "reinitialization RHS on band cells"),
    "lsm3dcomputeorthogonalizationeqnrhslocal_": ("local", "orthogonalization RHS on band cells"),
    "lsm3dcomputemeancurvatureorder2local_": ("local", "second-order mean curvature on band cells"),
    "lsm3dcomputegaussiancurvatureorder2local_": ("local", "second-order Gaussian curvature on band cells"),
    "lsm3dcomputemeancurvatureorder4local_": ("local", "fourth-order curvature on band cells: the Gaussian-curvature formula, as the reference routine evaluates it (lsmgpu_mean_curvature_order4_local gives the mean curvature)"),
    "lsm3dcomputegaussiancurvatureorder4local_": ("local", "fourth-order Gaussian curvature on band cells"),
    "lsm3daddconstprecomputedcurvtermtolserhslocal_": ("local", "rhs += b * kappa * |grad phi| on band cells"),
    "lsm3daddexternalandnormalveltermtolserhslocal_": ("local", "external plus normal velocity term with the combined Godunov upwinding on band cells"),
    "lsm3dmaxnormdifflocal_": ("local", "max |field1 - field2| over band cells (starts at 0)"),
    "lsm3dcomputestableadvectiondtlocal_": ("local", "CFL-stable advection dt over band cells"),
    "lsm3dcomputestablenormalveldtlocal_": ("local", "CFL-stable normal-velocity dt over band cells"),
    "lsm3dmaxnormdiffcontrolvolumelocal_": ("local", "max |field1 - field2| over band cells with a negative control volume (starts at 0)"),
    "lsm3dcomputestablenormalveldtcontrolvolumelocal_": ("local", "CFL-stable normal-velocity dt over band cells of one control-volume sign"),
    "lsm3dcomputestableconstnormalveldtlocal_": ("local", "CFL-stable constant normal-velocity dt over band cells (the reference routine reads two unassigned variables; this computes the dense routine's formula)"),
    # scalar functions
    "lsmheaviside_": ("calc", "smoothed Heaviside function of one value (evaluated on the calling thread)"),
    "lsmdeltafunction_": ("calc", "smoothed delta function of one value (evaluated on the calling thread)"),
    # band construction
    "lsm3ddeterminenarrowband_": ("band", "build the narrow band: level-0 list in sweep order, outer lists, BFS levels"),
    "lsm3dmarknarrowbandneighbors_": ("band", "breadth-first neighbour levels of a narrow band"),
    "lsm3dmarknarrowbandboundarylayer_": ("band", "mark the one-cell faces of a fill box"),
    "lsm3ddeterminenarrowbandfrommask_": ("band", "build a narrow band from the sign of a mask"),
    "lsm3ddeterminenarrowbandfromtwolevelsets_": ("band", "build a narrow band of cells near the zero sets of both phi and psi"),
    "lsm3ddeterminenarrowbandawayfrommask_": ("band", "build a narrow band of cells near phi = 0 and away from a mask (|phi - mask| > max dx)"),
    "lsm3dmultiplycutofflserhslocal_": ("band", "cubic cut-off of the RHS between beta and gamma"),
    "lsm3dcheckouternarrowbandlayer_": ("band", "1 when the outer band layer holds both signs of phi"),
    "lsm3dimposemasklocal_": ("band", "dest = max(mask, src) on listed cells"),
    "lsm3dcopydatalocal_": ("band", "dest = src on listed cells"),
}


# entry points LSMLIB lacks in 3D, with argument lists following the 2D
# *_local routines (spatial_derivatives2d_local.f.in:498, :816)
def _box(n):
    return [[f"{a}_{n}_gb", "int", False, False] for a in ("ilo", "ihi", "jlo", "jhi", "klo", "khi")]


_PM = ([["phi_x_plus", "real", True, True], ["phi_y_plus", "real", True, True], ["phi_z_plus", "real", True, True]]
       + _box("grad_phi_plus") +
       [["phi_x_minus", "real", True, True], ["phi_y_minus", "real", True, True], ["phi_z_minus", "real", True, True]]
       + _box("grad_phi_minus") + [["phi", "real", True, False]] + _box("phi"))
_TAIL_IDX = ([["dx", "real", False, False], ["dy", "real", False, False], ["dz", "real", False, False],
              ["index_x", "int", True, False], ["index_y", "int", True, False], ["index_z", "int", True, False]]
             + [[f"{a}_index{l}", "int", False, False] for l in range(4) for a in ("nlo", "nhi")]
             + [["narrow_band", "int1", True, False]] + _box("nb") + [["mark_fb", "int1", False, False]])
_UP2 = ([["phi_x", "real", True, True], ["phi_y", "real", True, True], ["phi_z", "real", True, True]]
        + _box("grad_phi") + [["phi", "real", True, False]] + _box("phi")
        + [["vel_x", "real", True, False], ["vel_y", "real", True, False], ["vel_z", "real", True, False]]
        + _box("vel") + [["d1", "real", True, True]] + _box("d1") + [["d2", "real", True, True]] + _box("d2")
        + [["dx", "real", False, False], ["dy", "real", False, False], ["dz", "real", False, False],
           ["index_x", "int", True, False], ["index_y", "int", True, False], ["index_z", "int", True, False]]
        + [[f"{a}_index{l}", "int", False, False] for l in range(3) for a in ("nlo", "nhi")]
        + [["narrow_band", "int1", True, False]] + _box("nb")
        + [["mark_fb", "int1", False, False], ["mark_d1", "int1", False, False], ["mark_d2", "int1", False, False]])
_BAND3 = ([[f"{a}_gb", "int", False, False] for a in ("ilo", "ihi", "jlo", "jhi", "klo", "khi")]
          + [["narrow_band", "int1", True, True]] + _box("nb")
          + [["index_x", "int", True, True], ["index_y", "int", True, True], ["index_z", "int", True, True],
             ["nlo_index", "int", False, False], ["nhi_index", "int", False, False],
             ["n_lo", "int", True, True], ["n_hi", "int", True, True], ["index_outer", "int", True, True],
             ["nlo_index_outer", "int", False, False], ["nhi_index_outer", "int", False, False],
             ["nlo_outer_plus", "int", False, True], ["nhi_outer_plus", "int", False, True],
             ["nlo_outer_minus", "int", False, True], ["nhi_outer_minus", "int", False, True],
             ["width", "real", False, False], ["width_inner", "real", False, False], ["level", "int", False, False]])
NEW_SIGS = {
    "lsm3ddeterminenarrowbandfromtwolevelsets_": {
        "src": "NEW (pattern: src/toolbox/lsm_localization2d.f:248)",
        "args": [["phi", "real", True, False], ["psi", "real", True, False]] + _BAND3},
    "lsm3ddeterminenarrowbandawayfrommask_": {
        "src": "NEW (pattern: src/toolbox/lsm_localization2d.f:365)",
        "args": [["phi", "real", True, False], ["mask", "real", True, False]] + _BAND3
                + [["dx", "real", False, False], ["dy", "real", False, False], ["dz", "real", False, False]]},
    "lsm3dupwindhjeno2local_": {"src": "NEW (pattern: src/toolbox/lsm_spatial_derivatives2d_local.f.in:1160)",
                                "args": _UP2},
    "lsm3dhjweno5local_": {"src": "NEW (pattern: src/toolbox/lsm_spatial_derivatives2d_local.f.in:816)",
                           "args": _PM + [["d1", "real", True, True]] + _box("d1") + _TAIL_IDX +
                                   [["mark_d1", "int1", False, False]]},
    "lsm3dhjeno3local_": {"src": "NEW (pattern: src/toolbox/lsm_spatial_derivatives2d_local.f.in:498)",
                          "args": _PM + [["d1", "real", True, True]] + _box("d1") + [["d2", "real", True, True]]
                                  + _box("d2") + [["d3", "real", True, True]] + _box("d3") + _TAIL_IDX +
                                  [["mark_d1", "int1", False, False], ["mark_d2", "int1", False, False],
                                   ["mark_d3", "int1", False, False]]},
}

GROUP_TITLE = {
    "deriv": "Spatial derivatives (src/toolbox/lsm_spatial_derivatives3d)",
    "rk": "TVD Runge-Kutta stages (src/toolbox/lsm_tvd_runge_kutta3d)",
    "lse": "Level set equation right-hand sides (src/toolbox/lsm_level_set_evolution3d)",
    "reinit": "Reinitialization (src/reinitialization/lsm_reinitialization3d)",
    "geom": "Curvature (src/geometry/lsm_curvature3d)",
    "red": "Reductions (src/toolbox/lsm_math_utils3d)",
    "geo": "Geometry: normals, curvature, volumes and areas (src/geometry/lsm_geometry3d_fort)",
    "local": "Narrow-band (index-list) variants (*_local)",
    "band": "Narrow-band construction and utilities (src/toolbox/lsm_localization3d)",
    "bc": "Boundary conditions (src/boundary_conditions/lsm_boundary_conditions3d)",
    "calc": "Smoothed Heaviside and delta functions (src/toolbox/lsm_calculus_toolbox)",
}


def header_line(sym):
    """(header path, line) of the C declaration whose LSM3D_* macro names sym."""
    out = subprocess.run(["grep", "-rn", "--include=*.h", sym, REF + "/src"],
                         capture_output=True, text=True).stdout
    for line in out.splitlines():
        path, ln, text = line.split(":", 2)
        m = re.match(r"\s*#define\s+(\w+)", text)
        macro = m.group(1) if m else None
        if not macro:
            # continuation style: '#define X \' on the previous line
            prev = open(path).read().splitlines()[int(ln) - 2]
            m = re.match(r"\s*#define\s+(\w+)", prev)
            macro = m.group(1) if m else None
        if not macro:
            continue
        txt = open(path).read().splitlines()
        for i, t in enumerate(txt, 1):
            if re.match(r"\s*void\s+" + macro + r"\s*\(", t):
                return os.path.relpath(path, REF), i
        return os.path.relpath(path, REF), int(ln)
    return None, None


def ctype(kind, is_arr, written):
    base = {"real": "double", "int": "int", "int1": "unsigned char", "logical": "int",
            "double": "double"}[kind]
    return ("" if written else "const ") + base + " *"


BOUND = re.compile(r"^(ilo|ihi|jlo|jhi|klo|khi)_")

# 2D / 1D routines whose arithmetic or loop bounds are not the 3D routine's
# with the missing terms removed and that no other routine covers (none at
# present; see LIFT_VIA and HAND_LIFTED).
NOT_LIFTED = set()

# 2D / 1D routines lifted onto a library entry point other than the 3D
# routine of the same name, which has the same argument list: the 3D
# MeanCurvatureOrder4 local routine evaluates the Gaussian-curvature formula
# (curvature3d_local.f.in:385-410), the 2D one the mean curvature
# the 2D orthogonalization RHS smooths sgn(psi) with max(dx)^2 alone, the 3D
# one with max(dx)^2 |grad psi|^2 (reinitialization2d.f.in:360,
# reinitialization3d.f.in:439); the 2D subcell-fix distance tests sign
# changes by negative products, takes the full central difference and returns
# 2 phi0 / delta (reinitialization2d.f.in:392)
LIFT_VIA = {"lsm2dcomputemeancurvatureorder4local_": ("lsmgpu_mean_curvature_order4_local",
                                                      "fourth-order mean curvature on band cells"),
            "lsm2dcomputeorthogonalizationeqnrhs_": ("lsmgpu_orthogonalization_rhs_unit_sgn_smoothing",
                                                     "orthogonalization RHS (sgn(psi) smoothed with max(dx)^2)"),
            "lsm2dcomputeorthogonalizationeqnrhslocal_": (
                "lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local",
                "orthogonalization RHS on band cells (sgn(psi) smoothed with max(dx)^2)"),
            "lsm2dcomputedistanceforsubcellfix_": ("lsmgpu_distance_for_subcell_fix_full_central",
                                                   "distance estimate for the subcell fix (2 phi0 / delta)"),
            # the 2D external + normal velocity term loops over the fill box
            # and adds nothing where |Vn| < zero_tol (level_set_evolution2d.f.in:399);
            # the 3D one loops from the fill box to the ghost box end
            # (level_set_evolution3d.f.in:620) and adds the advection part there
            "lsm2daddexternalandnormalveltermtolserhs_": (
                "lsmgpu_external_normal_vel_term_fill_box",
                "rhs -= u . grad(phi) + Vn |grad phi| over the fill box, combined Godunov upwinding"),
            # the 1D signed extrapolation takes the sign from the cell next to
            # the edge (boundary_conditions1d.f:103), the 3D one from the edge
            "lsm1dsignedlinearextrapolation_": ("lsmgpu_signed_linear_extrapolation_inner_sign",
                                                "signed linear extrapolation, sign from the cell next to the edge"),
            # the 2D band build sets n_hi(0) = count - 1 even for an empty band
            # and adds neighbour levels only when level 0 holds two or more
            # cells (localization2d.f:225-240); the 3D one (localization3d.f:274)
            # sets n_hi(0) = nlo for an empty band and adds them for any
            "lsm2ddeterminenarrowband_": ("lsmgpu_determine_narrow_band_2d_bookkeeping",
                                          "build the narrow band: level-0 list in sweep order, outer lists, BFS levels")}

# 1D routines written by hand in csrc/lifted_by_hand.cu: their arguments do
# not map by name onto the 3D routine they run on (the 1D normal-velocity dt
# reads only |vel_n| / dx, math_utils1d.f.in:157, :633: the 3D advection dt
# with vel_x = vel_n)
HAND_LIFTED = {"lsm1dcomputestablenormalveldt_": ("lsm3dcomputestableadvectiondt_",
                                                  "CFL-stable dt for a normal velocity: max |vel_n| / dx"),
               "lsm1dcomputestablenormalveldtcontrolvolume_": (
                   "lsm3dcomputestableadvectiondtcontrolvolume_",
                   "CFL-stable dt for a normal velocity over cells of one control-volume sign")}

# 3D routines whose dz (and dy) multiply a cell volume: lifted with 1 there
VOLUME_FACTOR = re.compile(r"volumeintegral|volumeregion|surfaceintegral|surfacearea")


def missing_component(name, dims):
    """True for an array argument that is a z (1D: y or z) component:
    phi_z_plus, vel_z, phi_xz, index_z, ..."""
    gone = "z" if dims == 2 else "yz"
    return any(re.fullmatch(r"[xyz]+", t) and any(c in t for c in gone) for t in name.split("_")[1:])


def lift_map(sym2, dims, abi3, sigs):
    """Argument expressions of the 3D call for the 2D / 1D routine sym2 and
    the Lift registrations, or None when the arguments do not map."""
    sym3 = "lsm3d" + sym2[5:]
    if sym3 not in abi3 or sym2 not in sigs or sym2 in NOT_LIFTED:
        return None
    spacing = "&L_.one" if VOLUME_FACTOR.search(sym3) else "dx"
    a3, a2 = abi3[sym3]["args"], sigs[sym2]["args"]
    names2 = [a[0] for a in a2]
    out, j = [], 0
    for name, kind, is_arr, written in a3:
        m = BOUND.match(name)
        if is_arr:
            if name in names2:
                if j >= len(a2) or a2[j][0] != name:
                    return None
                out.append(name)
                j += 1
            elif not missing_component(name, dims):
                return None
            elif written:
                if kind in ("real", "double"):
                    out.append("L_.junk()")
                elif kind == "int":
                    out.append("(int *)L_.junk()")   # e.g. the index_z list a 2D band build writes
                else:
                    return None
            else:
                out.append({"real": "L_.zero()", "double": "L_.zero()", "int": "L_.zero_int()"}.get(kind))
                if out[-1] is None:
                    return None
        elif m:
            axis = m.group(1)[0]
            if (dims == 2 and axis == "k") or (dims == 1 and axis in "jk"):
                out.append("&L_.k0")
            else:
                if j >= len(a2) or not BOUND.match(a2[j][0]) or a2[j][0][:3] != m.group(1):
                    return None
                out.append(a2[j][0])
                j += 1
        else:
            if j < len(a2) and a2[j][0] == name:
                out.append(name)
                j += 1
            elif (name == "dz" and dims <= 2) or (name == "dy" and dims == 1):
                out.append(spacing)
            elif name == "dir" and dims == 1:
                out.append("&L_.x_axis")   # a 1D routine differences along x
            else:
                return None
    if j != len(a2):
        return None
    regs = []
    for q, (name, kind, is_arr, written) in enumerate(a2):
        if name.startswith("ilo_"):
            if dims == 2:
                regs.append("L_.box(%s, %s, %s, %s);" % tuple(a2[q + t][0] for t in range(4)))
            else:
                regs.append("L_.box(%s, %s);" % (a2[q][0], a2[q + 1][0]))
        if name.startswith("nlo_index") and q + 1 < len(a2) and a2[q + 1][0].startswith("nhi_index"):
            regs.append("L_.list(%s, %s);" % (name, a2[q + 1][0]))
    return {"sym3": sym3, "call": LIFT_VIA.get(sym2, (sym3,))[0], "args": out, "regs": regs}


def write_lifted(abi, lifted):
    lines = [
        "// GENERATED by lsmlib_gb300/gen_abi.py -- do not edit.",
        "//",
        "// LSMLIB's 2D and 1D drop-in routines, each running the 3D routine on its",
        "// arrays with the missing axes lifted (lift.cuh).  Each wrapper cites the",
        "// reference routine it replaces; its declaration is in",
        "// include/lsmgpu_toolbox2d.h or include/lsmgpu_toolbox1d.h.",
        '#include "lift.cuh"',
        '#include "../../include/lsmgpu_toolbox3d.h"',
        '#include "../../include/lsmgpu_toolbox2d.h"',
        '#include "../../include/lsmgpu_toolbox1d.h"',
        "",
        "using lsmgpu::Lift;",
        "",
        'extern "C" {',
        "",
    ]
    for sym2, (dims, mp) in lifted.items():
        params = ", ".join(ctype(k, a, w) + n for n, k, a, w in abi[sym2]["args"])
        lines.append("// %s" % abi[sym2]["ref"])
        lines.append("void %s(%s) {" % (sym2, params))
        lines.append('  Lift L_(%d, "%s");' % (dims, sym2))
        for r in mp["regs"]:
            lines.append("  " + r)
        lines.append("  if (!L_.ready()) return;")
        lines.append("  %s(%s);" % (mp["call"], ", ".join(mp["args"])))
        lines.append("}")
        lines.append("")
    lines += ['}  // extern "C"', ""]
    with open(os.path.join(REPO, "lsmlib_gb300", "csrc", "lifted.cu"), "w") as f:
        f.write("\n".join(lines))


def write_header(path, guard, title, syms, abi, desc):
    lines = [
        "/*",
        " * lsmgpu drop-in entry points for LSMLIB's %s toolbox." % title,
        " *",
        " * Same conventions as lsmgpu_toolbox3d.h: LSMLIB's symbol names and",
        " * argument lists, column-major arrays over the ghost box given by the",
        " * bounds that follow them, double precision.  Each routine runs the 3D",
        " * kernels on its arrays (one cell along the missing axes, stride 0) and",
        " * matches the reference routine bit for bit.",
        " */",
        "#ifndef %s" % guard,
        "#define %s" % guard,
        "",
        "#ifdef __cplusplus",
        'extern "C" {',
        "#endif",
        "",
    ]
    for s in syms:
        a = abi[s]
        lines.append("/* %s." % desc[s])
        lines.append(f" * Replaces {a['ref']}" + (f"; C declaration {a['header']}." if a["header"] else "."))
        lines.append(" */")
        lines.append(f"void {s}(")
        args = a["args"]
        for i, (nm, kind, is_arr, written) in enumerate(args):
            sep = "," if i < len(args) - 1 else ");"
            lines.append(f"  {ctype(kind, is_arr, written)}{nm}{sep}")
        lines.append("")
    lines += ["#ifdef __cplusplus", "}", "#endif", "", "#endif /* %s */" % guard, ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


# LSMLIB's lsm2dHJENO3LOCAL (and lsm2dSurfaceIntegralPrecomputedDelta, below) reads index_x / index_y (spatial_derivatives2d_local.f.in:578,
# :642) but leaves them out of its Fortran argument list (:498-523); its C
# declaration (spatial_derivatives2d_local.h) passes them after dy, so callers
# pass them there and the drop-in takes them there.  The Fortran routine cannot
# be called correctly, so it is no parity target ("ref_unusable").
SIG_FROM_C_HEADER = {"lsm2dhjeno3local_": ("dy", [["index_x", "int", True, False], ["index_y", "int", True, False]]),
                     # loops over ilo_ib..jhi_ib (math_utils2d.f.in:760) that its
                     # Fortran argument list leaves out (:713-727); its C
                     # declaration (math_utils2d.h:462) passes them before dx
                     "lsm2dsurfaceintegralprecomputeddelta_": (
                         "jhi_grad_phi_gb", [["ilo_ib", "int", False, False], ["ihi_ib", "int", False, False],
                                             ["jlo_ib", "int", False, False], ["jhi_ib", "int", False, False]])}


# 2D routines with no 3D counterpart, written as 2D kernels (csrc/plane2d.cu)
PLANE2D = {
    "lsm2dcomputemeancurvature9stencil_": "mean curvature from a 9-point stencil (face gradients)",
    "lsm2dcomputemeancurvature9stencillocal_": "mean curvature from a 9-point stencil on band cells",
    "lsm2dcomputemeancurvaturesgndist_": "mean curvature of a signed distance function, Laplacian / (1 - phi Laplacian)",
    "lsm2dcomputemeancurvaturesgndistlocal_": "signed-distance mean curvature on band cells (dx where the denominator vanishes, as the reference)",
    "lsm2ddivergencecentral_": "second-order central divergence of (fx, fy)",
    "lsm2ddivergencecentrallocal_": "second-order central divergence on band cells",
    "lsm2ddeltafunctionorder2_": "second-order delta function (Smereka) from phi and the unit normal",
    "lsm2dsurfaceintegralprecomputeddelta_": "integral of F delta |grad phi| dV over an index box (index box from the C declaration)",
    "lsm2dsurfaceintegralprecomputeddeltacontrolvolume_": "integral of F delta |grad phi| dV over cells of one control-volume sign",
    "lsm2daveabsdifflocal_": "mean |field1 - field2| over band cells (0 when none)",
}


def fix_sigs(sigs):
    for sym, (after, extra) in SIG_FROM_C_HEADER.items():
        args = sigs[sym]["args"]
        if not any(a[0] == extra[0][0] for a in args):
            q = [a[0] for a in args].index(after) + 1
            sigs[sym]["args"] = args[:q] + extra + args[q:]
        sigs[sym]["ref_unusable"] = True
    return sigs


def main():
    sigs = fix_sigs(json.load(open(os.path.join(REPO, "oracle", "_ref", "sigs.json"))))
    abi, groups = {}, {}
    for s in DESC:
        if s in NEW_SIGS:
            abi[s] = {"ref": NEW_SIGS[s]["src"], "header": None, "args": NEW_SIGS[s]["args"]}
        else:
            sg = sigs[s]
            src, line = sg["src"].split(":")
            hpath, hline = header_line(s)
            abi[s] = {"ref": f"{os.path.relpath(src, REF)}:{line}",
                      "header": f"{hpath}:{hline}" if hpath else None, "args": sg["args"]}
        groups.setdefault(DESC[s][0], []).append(s)
    # library entry points with a 3D routine's argument list (declared in
    # include/lsmgpu.h, not in the toolbox header)
    for target, _ in LIFT_VIA.values():
        sym3 = next(s3 for s2, (t, _) in LIFT_VIA.items() if t == target for s3 in ["lsm3d" + s2[5:]])
        abi[target] = {"ref": abi[sym3]["ref"], "header": "include/lsmgpu.h", "args": abi[sym3]["args"],
                       "extension": "lsmgpu entry point with the argument list of the routine in ref"}
    # 2D and 1D routines lifted onto the 3D ones
    lifted, desc2 = {}, {}
    for s in sorted(sigs):
        dims = 2 if s.startswith("lsm2d") else (1 if s.startswith("lsm1d") else 0)
        if not dims:
            continue
        mp = lift_map(s, dims, abi, sigs)
        if mp is None:
            continue
        sg = sigs[s]
        src, line = sg["src"].split(":")
        hpath, hline = header_line(s)
        abi[s] = {"ref": f"{os.path.relpath(src, REF)}:{line}",
                  "header": f"{hpath}:{hline}" if hpath else None, "args": sg["args"], "lifted_from": mp["call"]}
        if sg.get("ref_unusable"):
            abi[s]["ref_unusable"] = True
        lifted[s] = (dims, mp)
        desc2[s] = "%dD form: %s" % (dims, LIFT_VIA[s][1] if s in LIFT_VIA else DESC[mp["sym3"]][1])
    for s, (sym3, text) in HAND_LIFTED.items():
        sg = sigs[s]
        src, line = sg["src"].split(":")
        hpath, hline = header_line(s)
        abi[s] = {"ref": f"{os.path.relpath(src, REF)}:{line}", "header": f"{hpath}:{hline}" if hpath else None,
                  "args": sg["args"], "lifted_from": sym3, "by_hand": True}
        lifted[s] = (1 if s.startswith("lsm1d") else 2, None)
        desc2[s] = "%dD form: %s" % (lifted[s][0], text)
    for s, text in PLANE2D.items():
        sg = sigs[s]
        src, line = sg["src"].split(":")
        hpath, hline = header_line(s)
        abi[s] = {"ref": f"{os.path.relpath(src, REF)}:{line}", "header": f"{hpath}:{hline}" if hpath else None,
                  "args": sg["args"], "plane2d": True}
        if sg.get("ref_unusable"):
            abi[s]["ref_unusable"] = True
        lifted[s] = (2, None)
        desc2[s] = "2D: " + text
    write_lifted(abi, {s: v for s, v in lifted.items() if v[1] is not None})
    for dims in (2, 1):
        syms = [s for s in lifted if lifted[s][0] == dims]
        write_header(os.path.join(REPO, "include", "lsmgpu_toolbox%dd.h" % dims), "LSMGPU_TOOLBOX%dD_H" % dims,
                     "%dD" % dims, syms, abi, desc2)
    with open(os.path.join(REPO, "lsmlib_gb300", "abi.json"), "w") as f:
        json.dump(abi, f, indent=1)
    lines = [
        "/*",
        " * lsmgpu drop-in entry points for LSMLIB's 3D toolbox.",
        " *",
        " * Every function below has the symbol name and argument list of the LSMLIB",
        " * Fortran routine it replaces (the name gfortran exports, which LSMLIB's C",
        " * headers #define their LSM3D_* macros to), so a program built against",
        " * LSMLIB's headers links against liblsmgpu.so unchanged.  All arguments are",
        " * pointers, arrays are column-major over the ghost box given by the six",
        " * bounds that follow them, and real numbers are double (LSMLIB's default",
        " * FP64 build).  Pointer, scratch and error rules: see lsmgpu.h.",
        " *",
        " * Each declaration cites the reference routine (Fortran file:line) and the",
        " * C declaration it mirrors (header file:line), relative to the LSMLIB tree.",
        " */",
        "#ifndef LSMGPU_TOOLBOX3D_H",
        "#define LSMGPU_TOOLBOX3D_H",
        "",
        "#ifdef __cplusplus",
        'extern "C" {',
        "#endif",
        "",
    ]
    for g, members in groups.items():
        lines += ["/* " + "-" * 70 + " */", "/* " + GROUP_TITLE[g] + " */", "/* " + "-" * 70 + " */", ""]
        for s in members:
            a = abi[s]
            lines.append(f"/* {DESC[s][1]}.")
            if a["ref"].startswith("NEW"):
                lines.append(" * No 3D counterpart in LSMLIB; arguments follow the 2D routine "
                             + a["ref"][len("NEW (pattern: "):-1] + ".")
            else:
                lines.append(f" * Replaces {a['ref']}" + (f"; C declaration {a['header']}." if a["header"] else "."))
            lines.append(" */")
            lines.append(f"void {s}(")
            args = a["args"]
            for i, (nm, kind, is_arr, written) in enumerate(args):
                sep = "," if i < len(args) - 1 else ");"
                lines.append(f"  {ctype(kind, is_arr, written)}{nm}{sep}")
            lines.append("")
    lines += ["#ifdef __cplusplus", "}", "#endif", "", "#endif /* LSMGPU_TOOLBOX3D_H */", ""]
    with open(os.path.join(REPO, "include", "lsmgpu_toolbox3d.h"), "w") as f:
        f.write("\n".join(lines))
    print(len(abi), "entry points,", len(lifted), "lifted 2D / 1D")


if __name__ == "__main__":
    main()
