// GENERATED by lsmlib_gb300/gen_abi.py -- do not edit.
//
// LSMLIB's 2D and 1D drop-in routines, each running the 3D routine on its
// arrays with the missing axes lifted (lift.cuh).  Each wrapper cites the
// reference routine it replaces; its declaration is in
// include/lsmgpu_toolbox2d.h or include/lsmgpu_toolbox1d.h.
#include "lift.cuh"
#include "../../include/lsmgpu_toolbox3d.h"
#include "../../include/lsmgpu_toolbox2d.h"
#include "../../include/lsmgpu_toolbox1d.h"

using lsmgpu::Lift;

extern "C" {

// src/toolbox/lsm_level_set_evolution1d.f.in:65
void lsm1daddadvectiontermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *ilo_fb, const int *ihi_fb) {
  Lift L_(1, "lsm1daddadvectiontermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3daddadvectiontermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x, L_.zero(), L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution1d.f.in:118
void lsm1daddnormalveltermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *ilo_fb, const int *ihi_fb) {
  Lift L_(1, "lsm1daddnormalveltermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3daddnormalveltermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_plus, L_.zero(), L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.zero(), L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_n, ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1471
void lsm1daveragegradphi_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *ilo_fb, const int *ihi_fb) {
  Lift L_(1, "lsm1daveragegradphi_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3daveragegradphi_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_plus, L_.zero(), L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.zero(), L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1198
void lsm1dcentralgradorder2_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dcentralgradorder2_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder2_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1250
void lsm1dcentralgradorder4_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dcentralgradorder4_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder4_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:49
void lsm1dcomputedn_(double *dn, const int *ilo_dn_gb, const int *ihi_dn_gb, const double *dn_minus_one, const int *ilo_dn_minus_one_gb, const int *ihi_dn_minus_one_gb, const int *ilo_fb, const int *ihi_fb, const int *n) {
  Lift L_(1, "lsm1dcomputedn_");
  L_.box(ilo_dn_gb, ihi_dn_gb);
  L_.box(ilo_dn_minus_one_gb, ihi_dn_minus_one_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dcomputedn_(dn, ilo_dn_gb, ihi_dn_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dn_minus_one, ilo_dn_minus_one_gb, ihi_dn_minus_one_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, n, &L_.x_axis);
}

// src/reinitialization/lsm_reinitialization1d.f.in:48
void lsm1dcomputereinitializationeqnrhs_(double *reinit_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *phi0, const int *ilo_phi0_gb, const int *ihi_phi0_gb, const double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *ilo_fb, const int *ihi_fb, const double *dx, const int *use_phi0_for_sgn) {
  Lift L_(1, "lsm1dcomputereinitializationeqnrhs_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_phi0_gb, ihi_phi0_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dcomputereinitializationeqnrhs_(reinit_rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi0, ilo_phi0_gb, ihi_phi0_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_plus, L_.zero(), L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.zero(), L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx, use_phi0_for_sgn);
}

// src/toolbox/lsm_math_utils1d.f.in:81
void lsm1dcomputestableadvectiondt_(double *dt, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *cfl_number) {
  Lift L_(1, "lsm1dcomputestableadvectiondt_");
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondt_(dt, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx, cfl_number);
}

// src/toolbox/lsm_math_utils1d.f.in:542
void lsm1dcomputestableadvectiondtcontrolvolume_(double *dt, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *cfl_number) {
  Lift L_(1, "lsm1dcomputestableadvectiondtcontrolvolume_");
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondtcontrolvolume_(dt, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx, cfl_number);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:169
void lsm1dcopyextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dcopyextrapolation_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dcopyextrapolation_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:135
void lsm1dhjeno1_(double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dhjeno1_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno1_(phi_x_plus, L_.junk(), L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.junk(), L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:228
void lsm1dhjeno2_(double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dhjeno2_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno2_(phi_x_plus, L_.junk(), L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.junk(), L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:344
void lsm1dhjeno3_(double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, double *d3, const int *ilo_d3_gb, const int *ihi_d3_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dhjeno3_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb);
  L_.box(ilo_d3_gb, ihi_d3_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno3_(phi_x_plus, L_.junk(), L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.junk(), L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d3, ilo_d3_gb, ihi_d3_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:499
void lsm1dhjweno5_(double *phi_x_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, double *phi_x_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dhjweno5_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhjweno5_(phi_x_plus, L_.junk(), L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x_minus, L_.junk(), L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:225
void lsm1dhomogeneousneumanneno1_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dhomogeneousneumanneno1_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno1_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:268
void lsm1dhomogeneousneumanneno2_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dhomogeneousneumanneno2_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno2_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:311
void lsm1dhomogeneousneumanneno3_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dhomogeneousneumanneno3_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno3_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:354
void lsm1dhomogeneousneumannweno5_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dhomogeneousneumannweno5_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumannweno5_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1305
void lsm1dlaplacianorder2_(double *laplacian_phi, const int *ilo_laplacian_phi_gb, const int *ihi_laplacian_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dlaplacianorder2_");
  L_.box(ilo_laplacian_phi_gb, ihi_laplacian_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dlaplacianorder2_(laplacian_phi, ilo_laplacian_phi_gb, ihi_laplacian_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:42
void lsm1dlinearextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dlinearextrapolation_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dlinearextrapolation_(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_math_utils1d.f.in:27
void lsm1dmaxnormdiff_(double *max_norm_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const int *ilo_ib, const int *ihi_ib) {
  Lift L_(1, "lsm1dmaxnormdiff_");
  L_.box(ilo_field1_gb, ihi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dmaxnormdiff_(max_norm_diff, field1, ilo_field1_gb, ihi_field1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils1d.f.in:470
void lsm1dmaxnormdiffcontrolvolume_(double *max_norm_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib) {
  Lift L_(1, "lsm1dmaxnormdiffcontrolvolume_");
  L_.box(ilo_field1_gb, ihi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dmaxnormdiffcontrolvolume_(max_norm_diff, field1, ilo_field1_gb, ihi_field1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1369
void lsm1dphiupwindgradf_(double *f_x, const int *ilo_grad_f_gb, const int *ihi_grad_f_gb, const double *f_x_plus, const int *ilo_grad_f_plus_gb, const int *ihi_grad_f_plus_gb, const double *f_x_minus, const int *ilo_grad_f_minus_gb, const int *ihi_grad_f_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_fb, const int *ihi_fb) {
  Lift L_(1, "lsm1dphiupwindgradf_");
  L_.box(ilo_grad_f_gb, ihi_grad_f_gb);
  L_.box(ilo_grad_f_plus_gb, ihi_grad_f_plus_gb);
  L_.box(ilo_grad_f_minus_gb, ihi_grad_f_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dphiupwindgradf_(f_x, L_.junk(), L_.junk(), ilo_grad_f_gb, ihi_grad_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, f_x_plus, L_.zero(), L_.zero(), ilo_grad_f_plus_gb, ihi_grad_f_plus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, f_x_minus, L_.zero(), L_.zero(), ilo_grad_f_minus_gb, ihi_grad_f_minus_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:32
void lsm1drk1step_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1drk1step_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3drk1step_(u_next, ilo_u_next_gb, ihi_u_next_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/boundary_conditions/lsm_boundary_conditions1d.f:103
void lsm1dsignedlinearextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *ilo_fb, const int *ihi_fb, const int *bdry_location_idx) {
  Lift L_(1, "lsm1dsignedlinearextrapolation_");
  L_.box(ilo_gb, ihi_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsmgpu_signed_linear_extrapolation_inner_sign(phi, ilo_gb, ihi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_math_utils1d.f.in:390
void lsm1dsurfaceintegral_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dsurfaceintegral_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dsurfaceintegral_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x, L_.zero(), L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils1d.f.in:924
void lsm1dsurfaceintegralcontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dsurfaceintegralcontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dsurfaceintegralcontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi_x, L_.zero(), L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:85
void lsm1dtvdrk2stage1_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1dtvdrk2stage1_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage1_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:137
void lsm1dtvdrk2stage2_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1dtvdrk2stage2_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage2_(u_next, ilo_u_next_gb, ihi_u_next_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:195
void lsm1dtvdrk3stage1_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1dtvdrk3stage1_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage1_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:247
void lsm1dtvdrk3stage2_(double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1dtvdrk3stage2_");
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage2_(u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta1d.f:303
void lsm1dtvdrk3stage3_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const double *dt) {
  Lift L_(1, "lsm1dtvdrk3stage3_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb);
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage3_(u_next, ilo_u_next_gb, ihi_u_next_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:680
void lsm1dupwindhjeno1_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dupwindhjeno1_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno1_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:771
void lsm1dupwindhjeno2_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dupwindhjeno2_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno2_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:888
void lsm1dupwindhjeno3_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, double *d3, const int *ilo_d3_gb, const int *ihi_d3_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dupwindhjeno3_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb);
  L_.box(ilo_d3_gb, ihi_d3_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno3_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d3, ilo_d3_gb, ihi_d3_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_spatial_derivatives1d.f.in:1042
void lsm1dupwindhjweno5_(double *phi_x, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *vel_x, const int *ilo_vel_gb, const int *ihi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *ilo_fb, const int *ihi_fb, const double *dx) {
  Lift L_(1, "lsm1dupwindhjweno5_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb);
  L_.box(ilo_fb, ihi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjweno5_(phi_x, L_.junk(), L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, vel_x, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_fb, ihi_fb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx);
}

// src/toolbox/lsm_math_utils1d.f.in:315
void lsm1dvolumeintegralphigreaterthanzero_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dvolumeintegralphigreaterthanzero_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphigreaterthanzero_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils1d.f.in:828
void lsm1dvolumeintegralphigreaterthanzerocontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dvolumeintegralphigreaterthanzerocontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphigreaterthanzerocontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils1d.f.in:238
void lsm1dvolumeintegralphilessthanzero_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dvolumeintegralphilessthanzero_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphilessthanzero_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils1d.f.in:732
void lsm1dvolumeintegralphilessthanzerocontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const double *dx, const double *epsilon) {
  Lift L_(1, "lsm1dvolumeintegralphilessthanzerocontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphilessthanzerocontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, &L_.one, &L_.one, epsilon);
}

// src/toolbox/lsm_level_set_evolution1d.f.in:25
void lsm1dzerooutlevelseteqnrhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb) {
  Lift L_(1, "lsm1dzerooutlevelseteqnrhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb);
  if (!L_.ready()) return;
  lsm3dzerooutlevelseteqnrhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:47
void lsm2daddadvectiontermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2daddadvectiontermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3daddadvectiontermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:55
void lsm2daddadvectiontermtolserhslocal_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddadvectiontermtolserhslocal_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddadvectiontermtolserhslocal_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:273
void lsm2daddconstcurvtermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi_xx, const double *phi_xy, const double *phi_yy, const int *ilo_grad2_phi_gb, const int *ihi_grad2_phi_gb, const int *jlo_grad2_phi_gb, const int *jhi_grad2_phi_gb, const double *b, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2daddconstcurvtermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_grad2_phi_gb, ihi_grad2_phi_gb, jlo_grad2_phi_gb, jhi_grad2_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3daddconstcurvtermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi_xx, phi_xy, L_.zero(), phi_yy, L_.zero(), L_.zero(), ilo_grad2_phi_gb, ihi_grad2_phi_gb, jlo_grad2_phi_gb, jhi_grad2_phi_gb, &L_.k0, &L_.k0, b, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:320
void lsm2daddconstcurvtermtolserhslocal_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi_xx, const double *phi_xy, const double *phi_yy, const int *ilo_grad2_phi_gb, const int *ihi_grad2_phi_gb, const int *jlo_grad2_phi_gb, const int *jhi_grad2_phi_gb, const double *b, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddconstcurvtermtolserhslocal_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_grad2_phi_gb, ihi_grad2_phi_gb, jlo_grad2_phi_gb, jhi_grad2_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddconstcurvtermtolserhslocal_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi_xx, phi_xy, L_.zero(), phi_yy, L_.zero(), L_.zero(), ilo_grad2_phi_gb, ihi_grad2_phi_gb, jlo_grad2_phi_gb, jhi_grad2_phi_gb, &L_.k0, &L_.k0, b, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:189
void lsm2daddconstnormalveltermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2daddconstnormalveltermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3daddconstnormalveltermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:227
void lsm2daddconstnormalveltermtolserhslocal_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddconstnormalveltermtolserhslocal_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddconstnormalveltermtolserhslocal_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:345
void lsm2daddconstprecomputedcurvtermtolserhs_(double *lse_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *b, const int *ilo_rhs_fb, const int *ihi_rhs_fb, const int *jlo_rhs_fb, const int *jhi_rhs_fb) {
  Lift L_(2, "lsm2daddconstprecomputedcurvtermtolserhs_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_rhs_fb, ihi_rhs_fb, jlo_rhs_fb, jhi_rhs_fb);
  if (!L_.ready()) return;
  lsm3daddconstprecomputedcurvtermtolserhs_(lse_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, b, ilo_rhs_fb, ihi_rhs_fb, jlo_rhs_fb, jhi_rhs_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:408
void lsm2daddconstprecomputedcurvtermtolserhslocal_(double *lse_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *grad_phi_mag, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *b, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddconstprecomputedcurvtermtolserhslocal_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddconstprecomputedcurvtermtolserhslocal_(lse_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, grad_phi_mag, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, b, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:399
void lsm2daddexternalandnormalveltermtolserhs_(double *lse_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *ilo_rhs_fb, const int *ihi_rhs_fb, const int *jlo_rhs_fb, const int *jhi_rhs_fb) {
  Lift L_(2, "lsm2daddexternalandnormalveltermtolserhs_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_rhs_fb, ihi_rhs_fb, jlo_rhs_fb, jhi_rhs_fb);
  if (!L_.ready()) return;
  lsmgpu_external_normal_vel_term_fill_box(lse_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, ilo_rhs_fb, ihi_rhs_fb, jlo_rhs_fb, jhi_rhs_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:474
void lsm2daddexternalandnormalveltermtolserhslocal_(double *lse_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddexternalandnormalveltermtolserhslocal_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddexternalandnormalveltermtolserhslocal_(lse_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:101
void lsm2daddnormalveltermtolserhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2daddnormalveltermtolserhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3daddnormalveltermtolserhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:126
void lsm2daddnormalveltermtolserhslocal_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2daddnormalveltermtolserhslocal_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3daddnormalveltermtolserhslocal_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, vel_n, ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_math_utils2d.f.in:69
void lsm2daveabsdiff_(double *ave_abs_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const int *jlo_field1_gb, const int *jhi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const int *jlo_field2_gb, const int *jhi_field2_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2daveabsdiff_");
  L_.box(ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3daveabsdiff_(ave_abs_diff, field1, ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2322
void lsm2daveragegradphi_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2daveragegradphi_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3daveragegradphi_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:1957
void lsm2dcentralgradorder2_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcentralgradorder2_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder2_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1392
void lsm2dcentralgradorder2local_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcentralgradorder2local_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder2local_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2021
void lsm2dcentralgradorder4_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcentralgradorder4_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder4_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1465
void lsm2dcentralgradorder4local_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcentralgradorder4local_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcentralgradorder4local_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2500
void lsm2dcentralhessian_(double *phi_xx, double *phi_xy, double *phi_yy, const int *ilo_hessian_gb, const int *ihi_hessian_gb, const int *jlo_hessian_gb, const int *jhi_hessian_gb, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcentralhessian_");
  L_.box(ilo_hessian_gb, ihi_hessian_gb, jlo_hessian_gb, jhi_hessian_gb);
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcentralhessian_(phi_xx, phi_xy, L_.junk(), phi_yy, L_.junk(), L_.junk(), ilo_hessian_gb, ihi_hessian_gb, jlo_hessian_gb, jhi_hessian_gb, &L_.k0, &L_.k0, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_localization2d.f:693
void lsm2dcheckouternarrowbandlayer_(int *change_sign, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const int *index_outer, const int *nlo_index_outer, const int *nhi_index_outer, const int *nlo_outer_plus, const int *nhi_outer_plus, const int *nlo_outer_minus, const int *nhi_outer_minus) {
  Lift L_(2, "lsm2dcheckouternarrowbandlayer_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.list(nlo_index, nhi_index);
  L_.list(nlo_index_outer, nhi_index_outer);
  if (!L_.ready()) return;
  lsm3dcheckouternarrowbandlayer_(change_sign, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, index_outer, nlo_index_outer, nhi_index_outer, nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1616
void lsm2dcomputeavegradphilocal_(double *grad_phi_ave, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputeavegradphilocal_");
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputeavegradphilocal_(grad_phi_ave, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/reinitialization/lsm_reinitialization2d.f.in:392
void lsm2dcomputedistanceforsubcellfix_(double *distance0, const double *phi0, const int *ilo_phi0_gb, const int *ihi_phi0_gb, const int *jlo_phi0_gb, const int *jhi_phi0_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcomputedistanceforsubcellfix_");
  L_.box(ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsmgpu_distance_for_subcell_fix_full_central(distance0, phi0, ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:49
void lsm2dcomputedn_(double *dn, const int *ilo_dn_gb, const int *ihi_dn_gb, const int *jlo_dn_gb, const int *jhi_dn_gb, const double *dn_minus_one, const int *ilo_dn_minus_one_gb, const int *ihi_dn_minus_one_gb, const int *jlo_dn_minus_one_gb, const int *jhi_dn_minus_one_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *n, const int *dir) {
  Lift L_(2, "lsm2dcomputedn_");
  L_.box(ilo_dn_gb, ihi_dn_gb, jlo_dn_gb, jhi_dn_gb);
  L_.box(ilo_dn_minus_one_gb, ihi_dn_minus_one_gb, jlo_dn_minus_one_gb, jhi_dn_minus_one_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcomputedn_(dn, ilo_dn_gb, ihi_dn_gb, jlo_dn_gb, jhi_dn_gb, &L_.k0, &L_.k0, dn_minus_one, ilo_dn_minus_one_gb, ihi_dn_minus_one_gb, jlo_dn_minus_one_gb, jhi_dn_minus_one_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, n, dir);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:43
void lsm2dcomputednlocal_(double *dn, const int *ilo_dn_gb, const int *ihi_dn_gb, const int *jlo_dn_gb, const int *jhi_dn_gb, const double *dn_minus_one, const int *ilo_dn_minus_one_gb, const int *ihi_dn_minus_one_gb, const int *jlo_dn_minus_one_gb, const int *jhi_dn_minus_one_gb, const int *n, const int *dir, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputednlocal_");
  L_.box(ilo_dn_gb, ihi_dn_gb, jlo_dn_gb, jhi_dn_gb);
  L_.box(ilo_dn_minus_one_gb, ihi_dn_minus_one_gb, jlo_dn_minus_one_gb, jhi_dn_minus_one_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputednlocal_(dn, ilo_dn_gb, ihi_dn_gb, jlo_dn_gb, jhi_dn_gb, &L_.k0, &L_.k0, dn_minus_one, ilo_dn_minus_one_gb, ihi_dn_minus_one_gb, jlo_dn_minus_one_gb, jhi_dn_minus_one_gb, &L_.k0, &L_.k0, n, dir, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/geometry/lsm_curvature2d.f.in:15
void lsm2dcomputemeancurvatureorder2_(double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcomputemeancurvatureorder2_");
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcomputemeancurvatureorder2_(kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/geometry/lsm_curvature2d_local.f.in:15
void lsm2dcomputemeancurvatureorder2local_(double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputemeancurvatureorder2local_");
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputemeancurvatureorder2local_(kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/geometry/lsm_curvature2d.f.in:252
void lsm2dcomputemeancurvatureorder4_(double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcomputemeancurvatureorder4_");
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcomputemeancurvatureorder4_(kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/geometry/lsm_curvature2d_local.f.in:299
void lsm2dcomputemeancurvatureorder4local_(double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb, const int *jhi_kappa_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputemeancurvatureorder4local_");
  L_.box(ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsmgpu_mean_curvature_order4_local(kappa, ilo_kappa_gb, ihi_kappa_gb, jlo_kappa_gb, jhi_kappa_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/reinitialization/lsm_reinitialization2d.f.in:255
void lsm2dcomputeorthogonalizationeqnrhs_(double *ortho_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *psi, const int *ilo_psi_gb, const int *ihi_psi_gb, const int *jlo_psi_gb, const int *jhi_psi_gb, const double *psi_x_plus, const double *psi_y_plus, const int *ilo_grad_psi_plus_gb, const int *ihi_grad_psi_plus_gb, const int *jlo_grad_psi_plus_gb, const int *jhi_grad_psi_plus_gb, const double *psi_x_minus, const double *psi_y_minus, const int *ilo_grad_psi_minus_gb, const int *ihi_grad_psi_minus_gb, const int *jlo_grad_psi_minus_gb, const int *jhi_grad_psi_minus_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcomputeorthogonalizationeqnrhs_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_psi_gb, ihi_psi_gb, jlo_psi_gb, jhi_psi_gb);
  L_.box(ilo_grad_psi_plus_gb, ihi_grad_psi_plus_gb, jlo_grad_psi_plus_gb, jhi_grad_psi_plus_gb);
  L_.box(ilo_grad_psi_minus_gb, ihi_grad_psi_minus_gb, jlo_grad_psi_minus_gb, jhi_grad_psi_minus_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsmgpu_orthogonalization_rhs_unit_sgn_smoothing(ortho_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, psi, ilo_psi_gb, ihi_psi_gb, jlo_psi_gb, jhi_psi_gb, &L_.k0, &L_.k0, psi_x_plus, psi_y_plus, L_.zero(), ilo_grad_psi_plus_gb, ihi_grad_psi_plus_gb, jlo_grad_psi_plus_gb, jhi_grad_psi_plus_gb, &L_.k0, &L_.k0, psi_x_minus, psi_y_minus, L_.zero(), ilo_grad_psi_minus_gb, ihi_grad_psi_minus_gb, jlo_grad_psi_minus_gb, jhi_grad_psi_minus_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/reinitialization/lsm_reinitialization2d_local.f.in:284
void lsm2dcomputeorthogonalizationeqnrhslocal_(double *ortho_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *psi, const int *ilo_psi_gb, const int *ihi_psi_gb, const int *jlo_psi_gb, const int *jhi_psi_gb, const double *psi_x_plus, const double *psi_y_plus, const int *ilo_grad_psi_plus_gb, const int *ihi_grad_psi_plus_gb, const int *jlo_grad_psi_plus_gb, const int *jhi_grad_psi_plus_gb, const double *psi_x_minus, const double *psi_y_minus, const int *ilo_grad_psi_minus_gb, const int *ihi_grad_psi_minus_gb, const int *jlo_grad_psi_minus_gb, const int *jhi_grad_psi_minus_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputeorthogonalizationeqnrhslocal_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_psi_gb, ihi_psi_gb, jlo_psi_gb, jhi_psi_gb);
  L_.box(ilo_grad_psi_plus_gb, ihi_grad_psi_plus_gb, jlo_grad_psi_plus_gb, jhi_grad_psi_plus_gb);
  L_.box(ilo_grad_psi_minus_gb, ihi_grad_psi_minus_gb, jlo_grad_psi_minus_gb, jhi_grad_psi_minus_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local(ortho_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, psi, ilo_psi_gb, ihi_psi_gb, jlo_psi_gb, jhi_psi_gb, &L_.k0, &L_.k0, psi_x_plus, psi_y_plus, L_.zero(), ilo_grad_psi_plus_gb, ihi_grad_psi_plus_gb, jlo_grad_psi_plus_gb, jhi_grad_psi_plus_gb, &L_.k0, &L_.k0, psi_x_minus, psi_y_minus, L_.zero(), ilo_grad_psi_minus_gb, ihi_grad_psi_minus_gb, jlo_grad_psi_minus_gb, jhi_grad_psi_minus_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/reinitialization/lsm_reinitialization2d.f.in:48
void lsm2dcomputereinitializationeqnrhs_(double *reinit_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi0, const int *ilo_phi0_gb, const int *ihi_phi0_gb, const int *jlo_phi0_gb, const int *jhi_phi0_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy, const int *use_phi0_for_sgn) {
  Lift L_(2, "lsm2dcomputereinitializationeqnrhs_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcomputereinitializationeqnrhs_(reinit_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi0, ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx, use_phi0_for_sgn);
}

// src/reinitialization/lsm_reinitialization2d_local.f.in:49
void lsm2dcomputereinitializationeqnrhslocal_(double *reinit_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi0, const int *ilo_phi0_gb, const int *ihi_phi0_gb, const int *jlo_phi0_gb, const int *jhi_phi0_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *dx, const double *dy, const int *use_phi0_for_sgn, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputereinitializationeqnrhslocal_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputereinitializationeqnrhslocal_(reinit_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi0, ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, dx, dy, dx, use_phi0_for_sgn, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/reinitialization/lsm_reinitialization2d.f.in:468
void lsm2dcomputereinitializationeqnrhssubcellfixorder1_(double *reinit_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi0, const double *distance0, const int *ilo_phi0_gb, const int *ihi_phi0_gb, const int *jlo_phi0_gb, const int *jhi_phi0_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dcomputereinitializationeqnrhssubcellfixorder1_");
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcomputereinitializationeqnrhssubcellfixorder1_(reinit_rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi0, distance0, ilo_phi0_gb, ihi_phi0_gb, jlo_phi0_gb, jhi_phi0_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_math_utils2d.f.in:218
void lsm2dcomputestableadvectiondt_(double *dt, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestableadvectiondt_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondt_(dt, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d.f.in:868
void lsm2dcomputestableadvectiondtcontrolvolume_(double *dt, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestableadvectiondtcontrolvolume_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondtcontrolvolume_(dt, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d_local.f.in:165
void lsm2dcomputestableadvectiondtlocal_(double *dt, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const double *dx, const double *dy, const double *cfl_number, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputestableadvectiondtlocal_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondtlocal_(dt, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, dx, dy, dx, cfl_number, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_math_utils2d.f.in:382
void lsm2dcomputestableconstnormalveldt_(double *dt, const double *vel_n, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestableconstnormalveldt_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableconstnormalveldt_(dt, vel_n, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d.f.in:1102
void lsm2dcomputestableconstnormalveldtcontrolvolume_(double *dt, const double *vel_n, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestableconstnormalveldtcontrolvolume_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableconstnormalveldtcontrolvolume_(dt, vel_n, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d_local.f.in:360
void lsm2dcomputestableconstnormalveldtlocal_(double *dt, const double *vel_n, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *dx, const double *dy, const double *cfl_number, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputestableconstnormalveldtlocal_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputestableconstnormalveldtlocal_(dt, vel_n, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, dx, dy, dx, cfl_number, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_math_utils2d.f.in:285
void lsm2dcomputestablenormalveldt_(double *dt, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestablenormalveldt_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestablenormalveldt_(dt, vel_n, ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d.f.in:966
void lsm2dcomputestablenormalveldtcontrolvolume_(double *dt, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *cfl_number) {
  Lift L_(2, "lsm2dcomputestablenormalveldtcontrolvolume_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestablenormalveldtcontrolvolume_(dt, vel_n, ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, dx, cfl_number);
}

// src/toolbox/lsm_math_utils2d_local.f.in:246
void lsm2dcomputestablenormalveldtlocal_(double *dt, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const double *phi_x_plus, const double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, const double *phi_x_minus, const double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *dx, const double *dy, const double *cfl_number, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dcomputestablenormalveldtlocal_");
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dcomputestablenormalveldtlocal_(dt, vel_n, ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, phi_x_plus, phi_y_plus, L_.zero(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.zero(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, dx, dy, dx, cfl_number, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_localization2d.f:833
void lsm2dcopydatalocal_(double *dest, const int *ilo_dest_gb, const int *ihi_dest_gb, const int *jlo_dest_gb, const int *jhi_dest_gb, const double *src, const int *ilo_src_gb, const int *ihi_src_gb, const int *jlo_src_gb, const int *jhi_src_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index) {
  Lift L_(2, "lsm2dcopydatalocal_");
  L_.box(ilo_dest_gb, ihi_dest_gb, jlo_dest_gb, jhi_dest_gb);
  L_.box(ilo_src_gb, ihi_src_gb, jlo_src_gb, jhi_src_gb);
  L_.list(nlo_index, nhi_index);
  if (!L_.ready()) return;
  lsm3dcopydatalocal_(dest, ilo_dest_gb, ihi_dest_gb, jlo_dest_gb, jhi_dest_gb, &L_.k0, &L_.k0, src, ilo_src_gb, ihi_src_gb, jlo_src_gb, jhi_src_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:264
void lsm2dcopyextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dcopyextrapolation_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dcopyextrapolation_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_calculus_toolbox2d.f.in:16
void lsm2ddeltafunctionorder1_(const double *phi, double *delta, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const double *norm_phi_x, const double *norm_phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2ddeltafunctionorder1_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3ddeltafunctionorder1_(phi, delta, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, norm_phi_x, norm_phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_localization2d.f:139
void lsm2ddeterminenarrowband_(const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, int *index_x, int *index_y, const int *nlo_index, const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer, const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus, int *nhi_outer_minus, const double *width, const double *width_inner, const int *level) {
  Lift L_(2, "lsm2ddeterminenarrowband_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  L_.list(nlo_index, nhi_index);
  L_.list(nlo_index_outer, nhi_index_outer);
  if (!L_.ready()) return;
  lsmgpu_determine_narrow_band_2d_bookkeeping(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, index_x, index_y, (int *)L_.junk(), nlo_index, nhi_index, n_lo, n_hi, index_outer, nlo_index_outer, nhi_index_outer, nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus, width, width_inner, level);
}

// src/toolbox/lsm_localization2d.f:365
void lsm2ddeterminenarrowbandawayfrommask_(const double *phi, const double *mask, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, int *index_x, int *index_y, const int *nlo_index, const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer, const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus, int *nhi_outer_minus, const double *width, const double *width_inner, const int *level, const double *dx, const double *dy) {
  Lift L_(2, "lsm2ddeterminenarrowbandawayfrommask_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  L_.list(nlo_index, nhi_index);
  L_.list(nlo_index_outer, nhi_index_outer);
  if (!L_.ready()) return;
  lsm3ddeterminenarrowbandawayfrommask_(phi, mask, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, index_x, index_y, (int *)L_.junk(), nlo_index, nhi_index, n_lo, n_hi, index_outer, nlo_index_outer, nhi_index_outer, nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus, width, width_inner, level, dx, dy, dx);
}

// src/toolbox/lsm_localization2d.f:539
void lsm2ddeterminenarrowbandfrommask_(const double *mask, const int *ilo_mask_gb, const int *ihi_mask_gb, const int *jlo_mask_gb, const int *jhi_mask_gb, unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, int *index_x, int *index_y, const int *nlo_index, const int *nhi_index, int *n_lo, int *n_hi, const int *level, const int *use_mask_sign) {
  Lift L_(2, "lsm2ddeterminenarrowbandfrommask_");
  L_.box(ilo_mask_gb, ihi_mask_gb, jlo_mask_gb, jhi_mask_gb);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  L_.list(nlo_index, nhi_index);
  if (!L_.ready()) return;
  lsm3ddeterminenarrowbandfrommask_(mask, ilo_mask_gb, ihi_mask_gb, jlo_mask_gb, jhi_mask_gb, &L_.k0, &L_.k0, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, index_x, index_y, (int *)L_.junk(), nlo_index, nhi_index, n_lo, n_hi, level, use_mask_sign);
}

// src/toolbox/lsm_localization2d.f:248
void lsm2ddeterminenarrowbandfromtwolevelsets_(const double *phi, const double *psi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, int *index_x, int *index_y, const int *nlo_index, const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer, const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus, int *nhi_outer_minus, const double *width, const double *width_inner, const int *level) {
  Lift L_(2, "lsm2ddeterminenarrowbandfromtwolevelsets_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  L_.list(nlo_index, nhi_index);
  L_.list(nlo_index_outer, nhi_index_outer);
  if (!L_.ready()) return;
  lsm3ddeterminenarrowbandfromtwolevelsets_(phi, psi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, index_x, index_y, (int *)L_.junk(), nlo_index, nhi_index, n_lo, n_hi, index_outer, nlo_index_outer, nhi_index_outer, nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus, width, width_inner, level);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2395
void lsm2dgradientmagnitude_(const double *phi_x, const double *phi_y, double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2dgradientmagnitude_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dgradientmagnitude_(phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1689
void lsm2dgradientmagnitudelocal_(const double *phi_x, const double *phi_y, double *grad_phi_mag, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dgradientmagnitudelocal_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dgradientmagnitudelocal_(phi_x, phi_y, L_.zero(), grad_phi_mag, ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:165
void lsm2dhjeno1_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dhjeno1_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno1_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:133
void lsm2dhjeno1local_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index0, const int *nhi_index0, const int *nlo_index1, const int *nhi_index1, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const unsigned char *mark_d1) {
  Lift L_(2, "lsm2dhjeno1local_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.list(nlo_index0, nhi_index0);
  L_.list(nlo_index1, nhi_index1);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dhjeno1local_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index0, nhi_index0, nlo_index1, nhi_index1, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, mark_d1);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:296
void lsm2dhjeno2_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dhjeno2_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno2_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:280
void lsm2dhjeno2local_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index0, const int *nhi_index0, const int *nlo_index1, const int *nhi_index1, const int *nlo_index2, const int *nhi_index2, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const unsigned char *mark_d1, const unsigned char *mark_d2) {
  Lift L_(2, "lsm2dhjeno2local_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.list(nlo_index0, nhi_index0);
  L_.list(nlo_index1, nhi_index1);
  L_.list(nlo_index2, nhi_index2);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dhjeno2local_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index0, nhi_index0, nlo_index1, nhi_index1, nlo_index2, nhi_index2, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, mark_d1, mark_d2);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:479
void lsm2dhjeno3_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, double *d3, const int *ilo_d3_gb, const int *ihi_d3_gb, const int *jlo_d3_gb, const int *jhi_d3_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dhjeno3_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.box(ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhjeno3_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, d3, ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:498
void lsm2dhjeno3local_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, double *d3, const int *ilo_d3_gb, const int *ihi_d3_gb, const int *jlo_d3_gb, const int *jhi_d3_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index0, const int *nhi_index0, const int *nlo_index1, const int *nhi_index1, const int *nlo_index2, const int *nhi_index2, const int *nlo_index3, const int *nhi_index3, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const unsigned char *mark_d1, const unsigned char *mark_d2, const unsigned char *mark_d3) {
  Lift L_(2, "lsm2dhjeno3local_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.box(ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb);
  L_.list(nlo_index0, nhi_index0);
  L_.list(nlo_index1, nhi_index1);
  L_.list(nlo_index2, nhi_index2);
  L_.list(nlo_index3, nhi_index3);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dhjeno3local_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, d3, ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index0, nhi_index0, nlo_index1, nhi_index1, nlo_index2, nhi_index2, nlo_index3, nhi_index3, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, mark_d1, mark_d2, mark_d3);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:756
void lsm2dhjweno5_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dhjweno5_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhjweno5_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:816
void lsm2dhjweno5local_(double *phi_x_plus, double *phi_y_plus, const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb, double *phi_x_minus, double *phi_y_minus, const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index0, const int *nhi_index0, const int *nlo_index1, const int *nhi_index1, const int *nlo_index2, const int *nhi_index2, const int *nlo_index3, const int *nhi_index3, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const unsigned char *mark_d1) {
  Lift L_(2, "lsm2dhjweno5local_");
  L_.box(ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb);
  L_.box(ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.list(nlo_index0, nhi_index0);
  L_.list(nlo_index1, nhi_index1);
  L_.list(nlo_index2, nhi_index2);
  L_.list(nlo_index3, nhi_index3);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dhjweno5local_(phi_x_plus, phi_y_plus, L_.junk(), ilo_grad_phi_plus_gb, ihi_grad_phi_plus_gb, jlo_grad_phi_plus_gb, jhi_grad_phi_plus_gb, &L_.k0, &L_.k0, phi_x_minus, phi_y_minus, L_.junk(), ilo_grad_phi_minus_gb, ihi_grad_phi_minus_gb, jlo_grad_phi_minus_gb, jhi_grad_phi_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index0, nhi_index0, nlo_index1, nhi_index1, nlo_index2, nhi_index2, nlo_index3, nhi_index3, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, mark_d1);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:360
void lsm2dhomogeneousneumanneno1_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dhomogeneousneumanneno1_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno1_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:403
void lsm2dhomogeneousneumanneno2_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dhomogeneousneumanneno2_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno2_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:446
void lsm2dhomogeneousneumanneno3_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dhomogeneousneumanneno3_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumanneno3_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:489
void lsm2dhomogeneousneumannweno5_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dhomogeneousneumannweno5_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dhomogeneousneumannweno5_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_localization2d.f:778
void lsm2dimposemasklocal_(double *dest, const int *ilo_dest_gb, const int *ihi_dest_gb, const int *jlo_dest_gb, const int *jhi_dest_gb, const double *src, const int *ilo_src_gb, const int *ihi_src_gb, const int *jlo_src_gb, const int *jhi_src_gb, const double *mask, const int *ilo_mask_gb, const int *ihi_mask_gb, const int *jlo_mask_gb, const int *jhi_mask_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index) {
  Lift L_(2, "lsm2dimposemasklocal_");
  L_.box(ilo_dest_gb, ihi_dest_gb, jlo_dest_gb, jhi_dest_gb);
  L_.box(ilo_src_gb, ihi_src_gb, jlo_src_gb, jhi_src_gb);
  L_.box(ilo_mask_gb, ihi_mask_gb, jlo_mask_gb, jhi_mask_gb);
  L_.list(nlo_index, nhi_index);
  if (!L_.ready()) return;
  lsm3dimposemasklocal_(dest, ilo_dest_gb, ihi_dest_gb, jlo_dest_gb, jhi_dest_gb, &L_.k0, &L_.k0, src, ilo_src_gb, ihi_src_gb, jlo_src_gb, jhi_src_gb, &L_.k0, &L_.k0, mask, ilo_mask_gb, ihi_mask_gb, jlo_mask_gb, jhi_mask_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2091
void lsm2dlaplacianorder2_(double *laplacian_phi, const int *ilo_laplacian_phi_gb, const int *ihi_laplacian_phi_gb, const int *jlo_laplacian_phi_gb, const int *jhi_laplacian_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dlaplacianorder2_");
  L_.box(ilo_laplacian_phi_gb, ihi_laplacian_phi_gb, jlo_laplacian_phi_gb, jhi_laplacian_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dlaplacianorder2_(laplacian_phi, ilo_laplacian_phi_gb, ihi_laplacian_phi_gb, jlo_laplacian_phi_gb, jhi_laplacian_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1542
void lsm2dlaplacianorder2local_(double *laplacian_phi, const int *ilo_laplacian_phi_gb, const int *ihi_laplacian_phi_gb, const int *jlo_laplacian_phi_gb, const int *jhi_laplacian_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dlaplacianorder2local_");
  L_.box(ilo_laplacian_phi_gb, ihi_laplacian_phi_gb, jlo_laplacian_phi_gb, jhi_laplacian_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dlaplacianorder2local_(laplacian_phi, ilo_laplacian_phi_gb, ihi_laplacian_phi_gb, jlo_laplacian_phi_gb, jhi_laplacian_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:44
void lsm2dlinearextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dlinearextrapolation_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dlinearextrapolation_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_localization2d.f:486
void lsm2dmarknarrowbandboundarylayer_(unsigned char *narrow_band, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const unsigned char *mark_boundary_layer) {
  Lift L_(2, "lsm2dmarknarrowbandboundarylayer_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dmarknarrowbandboundarylayer_(narrow_band, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, mark_boundary_layer);
}

// src/toolbox/lsm_localization2d.f:48
void lsm2dmarknarrowbandneighbors_(unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, int *index_x, int *index_y, const int *nlo_index, const int *nhi_index, int *n_lo, int *n_hi, const int *level) {
  Lift L_(2, "lsm2dmarknarrowbandneighbors_");
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  L_.list(nlo_index, nhi_index);
  if (!L_.ready()) return;
  lsm3dmarknarrowbandneighbors_(narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, index_x, index_y, (int *)L_.junk(), nlo_index, nhi_index, n_lo, n_hi, level);
}

// src/toolbox/lsm_math_utils2d.f.in:15
void lsm2dmaxnormdiff_(double *max_norm_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const int *jlo_field1_gb, const int *jhi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const int *jlo_field2_gb, const int *jhi_field2_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dmaxnormdiff_");
  L_.box(ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dmaxnormdiff_(max_norm_diff, field1, ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils2d.f.in:777
void lsm2dmaxnormdiffcontrolvolume_(double *max_norm_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const int *jlo_field1_gb, const int *jhi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const int *jlo_field2_gb, const int *jhi_field2_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dmaxnormdiffcontrolvolume_");
  L_.box(ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dmaxnormdiffcontrolvolume_(max_norm_diff, field1, ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils2d_local.f.in:16
void lsm2dmaxnormdifflocal_(double *max_norm_diff, const double *field1, const int *ilo_field1_gb, const int *ihi_field1_gb, const int *jlo_field1_gb, const int *jhi_field1_gb, const double *field2, const int *ilo_field2_gb, const int *ihi_field2_gb, const int *jlo_field2_gb, const int *jhi_field2_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dmaxnormdifflocal_");
  L_.box(ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb);
  L_.box(ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dmaxnormdifflocal_(max_norm_diff, field1, ilo_field1_gb, ihi_field1_gb, jlo_field1_gb, jhi_field1_gb, &L_.k0, &L_.k0, field2, ilo_field2_gb, ihi_field2_gb, jlo_field2_gb, jhi_field2_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_localization2d.f:621
void lsm2dmultiplycutofflserhslocal_(const double *phi, double *lse_rhs, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const double *beta, const double *gamma) {
  Lift L_(2, "lsm2dmultiplycutofflserhslocal_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dmultiplycutofflserhslocal_(phi, lse_rhs, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, beta, gamma);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:2166
void lsm2dphiupwindgradf_(double *f_x, double *f_y, const int *ilo_grad_f_gb, const int *ihi_grad_f_gb, const int *jlo_grad_f_gb, const int *jhi_grad_f_gb, const double *f_x_plus, const double *f_y_plus, const int *ilo_grad_f_plus_gb, const int *ihi_grad_f_plus_gb, const int *jlo_grad_f_plus_gb, const int *jhi_grad_f_plus_gb, const double *f_x_minus, const double *f_y_minus, const int *ilo_grad_f_minus_gb, const int *ihi_grad_f_minus_gb, const int *jlo_grad_f_minus_gb, const int *jhi_grad_f_minus_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb) {
  Lift L_(2, "lsm2dphiupwindgradf_");
  L_.box(ilo_grad_f_gb, ihi_grad_f_gb, jlo_grad_f_gb, jhi_grad_f_gb);
  L_.box(ilo_grad_f_plus_gb, ihi_grad_f_plus_gb, jlo_grad_f_plus_gb, jhi_grad_f_plus_gb);
  L_.box(ilo_grad_f_minus_gb, ihi_grad_f_minus_gb, jlo_grad_f_minus_gb, jhi_grad_f_minus_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dphiupwindgradf_(f_x, f_y, L_.junk(), ilo_grad_f_gb, ihi_grad_f_gb, jlo_grad_f_gb, jhi_grad_f_gb, &L_.k0, &L_.k0, f_x_plus, f_y_plus, L_.zero(), ilo_grad_f_plus_gb, ihi_grad_f_plus_gb, jlo_grad_f_plus_gb, jhi_grad_f_plus_gb, &L_.k0, &L_.k0, f_x_minus, f_y_minus, L_.zero(), ilo_grad_f_minus_gb, ihi_grad_f_minus_gb, jlo_grad_f_minus_gb, jhi_grad_f_minus_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:32
void lsm2drk1step_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2drk1step_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3drk1step_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:33
void lsm2drk1steplocal_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2drk1steplocal_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3drk1steplocal_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/boundary_conditions/lsm_boundary_conditions2d.f:149
void lsm2dsignedlinearextrapolation_(double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *bdry_location_idx) {
  Lift L_(2, "lsm2dsignedlinearextrapolation_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dsignedlinearextrapolation_(phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, bdry_location_idx);
}

// src/toolbox/lsm_math_utils2d.f.in:625
void lsm2dsurfaceintegral_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dsurfaceintegral_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dsurfaceintegral_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils2d.f.in:1472
void lsm2dsurfaceintegralcontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *phi_x, const double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dsurfaceintegralcontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dsurfaceintegralcontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, phi_x, phi_y, L_.zero(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:96
void lsm2dtvdrk2stage1_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2dtvdrk2stage1_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage1_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:123
void lsm2dtvdrk2stage1local_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dtvdrk2stage1local_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage1local_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:160
void lsm2dtvdrk2stage2_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2dtvdrk2stage2_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage2_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:212
void lsm2dtvdrk2stage2local_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dtvdrk2stage2local_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dtvdrk2stage2local_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:232
void lsm2dtvdrk3stage1_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2dtvdrk3stage1_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage1_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:308
void lsm2dtvdrk3stage1local_(double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dtvdrk3stage1local_");
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage1local_(u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:296
void lsm2dtvdrk3stage2_(double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const int *jlo_u_stage2_gb, const int *jhi_u_stage2_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2dtvdrk3stage2_");
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage2_(u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:396
void lsm2dtvdrk3stage2local_(double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const int *jlo_u_stage2_gb, const int *jhi_u_stage2_gb, const double *u_stage1, const int *ilo_u_stage1_gb, const int *ihi_u_stage1_gb, const int *jlo_u_stage1_gb, const int *jhi_u_stage1_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dtvdrk3stage2local_");
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb);
  L_.box(ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage2local_(u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb, &L_.k0, &L_.k0, u_stage1, ilo_u_stage1_gb, ihi_u_stage1_gb, jlo_u_stage1_gb, jhi_u_stage1_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_tvd_runge_kutta2d.f:366
void lsm2dtvdrk3stage3_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const int *jlo_u_stage2_gb, const int *jhi_u_stage2_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dt) {
  Lift L_(2, "lsm2dtvdrk3stage3_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage3_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dt);
}

// src/toolbox/lsm_tvd_runge_kutta2d_local.f:491
void lsm2dtvdrk3stage3local_(double *u_next, const int *ilo_u_next_gb, const int *ihi_u_next_gb, const int *jlo_u_next_gb, const int *jhi_u_next_gb, const double *u_stage2, const int *ilo_u_stage2_gb, const int *ihi_u_stage2_gb, const int *jlo_u_stage2_gb, const int *jhi_u_stage2_gb, const double *u_cur, const int *ilo_u_cur_gb, const int *ihi_u_cur_gb, const int *jlo_u_cur_gb, const int *jhi_u_cur_gb, const double *rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb, const int *jhi_rhs_gb, const double *dt, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb) {
  Lift L_(2, "lsm2dtvdrk3stage3local_");
  L_.box(ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb);
  L_.box(ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb);
  L_.box(ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb);
  L_.box(ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb);
  L_.list(nlo_index, nhi_index);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dtvdrk3stage3local_(u_next, ilo_u_next_gb, ihi_u_next_gb, jlo_u_next_gb, jhi_u_next_gb, &L_.k0, &L_.k0, u_stage2, ilo_u_stage2_gb, ihi_u_stage2_gb, jlo_u_stage2_gb, jhi_u_stage2_gb, &L_.k0, &L_.k0, u_cur, ilo_u_cur_gb, ihi_u_cur_gb, jlo_u_cur_gb, jhi_u_cur_gb, &L_.k0, &L_.k0, rhs, ilo_rhs_gb, ihi_rhs_gb, jlo_rhs_gb, jhi_rhs_gb, &L_.k0, &L_.k0, dt, index_x, index_y, L_.zero_int(), nlo_index, nhi_index, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:1069
void lsm2dupwindhjeno1_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dupwindhjeno1_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno1_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:1214
void lsm2dupwindhjeno2_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dupwindhjeno2_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno2_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d_local.f.in:1160
void lsm2dupwindhjeno2local_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, const double *dx, const double *dy, const int *index_x, const int *index_y, const int *nlo_index0, const int *nhi_index0, const int *nlo_index1, const int *nhi_index1, const int *nlo_index2, const int *nhi_index2, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const unsigned char *mark_fb, const unsigned char *mark_d1, const unsigned char *mark_d2) {
  Lift L_(2, "lsm2dupwindhjeno2local_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.list(nlo_index0, nhi_index0);
  L_.list(nlo_index1, nhi_index1);
  L_.list(nlo_index2, nhi_index2);
  L_.box(ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno2local_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, dx, dy, dx, index_x, index_y, L_.zero_int(), nlo_index0, nhi_index0, nlo_index1, nhi_index1, nlo_index2, nhi_index2, narrow_band, ilo_nb_gb, ihi_nb_gb, jlo_nb_gb, jhi_nb_gb, &L_.k0, &L_.k0, mark_fb, mark_d1, mark_d2);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:1416
void lsm2dupwindhjeno3_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, double *d2, const int *ilo_d2_gb, const int *ihi_d2_gb, const int *jlo_d2_gb, const int *jhi_d2_gb, double *d3, const int *ilo_d3_gb, const int *ihi_d3_gb, const int *jlo_d3_gb, const int *jhi_d3_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dupwindhjeno3_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb);
  L_.box(ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjeno3_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, d2, ilo_d2_gb, ihi_d2_gb, jlo_d2_gb, jhi_d2_gb, &L_.k0, &L_.k0, d3, ilo_d3_gb, ihi_d3_gb, jlo_d3_gb, jhi_d3_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_spatial_derivatives2d.f.in:1699
void lsm2dupwindhjweno5_(double *phi_x, double *phi_y, const int *ilo_grad_phi_gb, const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *vel_x, const double *vel_y, const int *ilo_vel_gb, const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, double *d1, const int *ilo_d1_gb, const int *ihi_d1_gb, const int *jlo_d1_gb, const int *jhi_d1_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const double *dx, const double *dy) {
  Lift L_(2, "lsm2dupwindhjweno5_");
  L_.box(ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb);
  L_.box(ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb);
  L_.box(ilo_fb, ihi_fb, jlo_fb, jhi_fb);
  if (!L_.ready()) return;
  lsm3dupwindhjweno5_(phi_x, phi_y, L_.junk(), ilo_grad_phi_gb, ihi_grad_phi_gb, jlo_grad_phi_gb, jhi_grad_phi_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, vel_x, vel_y, L_.zero(), ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, &L_.k0, &L_.k0, d1, ilo_d1_gb, ihi_d1_gb, jlo_d1_gb, jhi_d1_gb, &L_.k0, &L_.k0, ilo_fb, ihi_fb, jlo_fb, jhi_fb, &L_.k0, &L_.k0, dx, dy, dx);
}

// src/toolbox/lsm_math_utils2d.f.in:549
void lsm2dvolumeintegralphigreaterthanzero_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dvolumeintegralphigreaterthanzero_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphigreaterthanzero_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils2d.f.in:1353
void lsm2dvolumeintegralphigreaterthanzerocontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dvolumeintegralphigreaterthanzerocontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphigreaterthanzerocontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils2d.f.in:473
void lsm2dvolumeintegralphilessthanzero_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dvolumeintegralphilessthanzero_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphilessthanzero_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils2d.f.in:1234
void lsm2dvolumeintegralphilessthanzerocontrolvolume_(double *int_f, const double *f, const int *ilo_f_gb, const int *ihi_f_gb, const int *jlo_f_gb, const int *jhi_f_gb, const double *phi, const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const double *dx, const double *dy, const double *epsilon) {
  Lift L_(2, "lsm2dvolumeintegralphilessthanzerocontrolvolume_");
  L_.box(ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb);
  L_.box(ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvolumeintegralphilessthanzerocontrolvolume_(int_f, f, ilo_f_gb, ihi_f_gb, jlo_f_gb, jhi_f_gb, &L_.k0, &L_.k0, phi, ilo_phi_gb, ihi_phi_gb, jlo_phi_gb, jhi_phi_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0, dx, dy, &L_.one, epsilon);
}

// src/toolbox/lsm_math_utils2d.f.in:132
void lsm2dvoxelcountgreaterthanzero_(int *count, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dvoxelcountgreaterthanzero_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvoxelcountgreaterthanzero_(count, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils2d.f.in:1604
void lsm2dvoxelcountgreaterthanzerocontrolvolume_(int *count, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dvoxelcountgreaterthanzerocontrolvolume_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvoxelcountgreaterthanzerocontrolvolume_(count, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils2d.f.in:175
void lsm2dvoxelcountlessthanzero_(int *count, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dvoxelcountlessthanzero_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvoxelcountlessthanzero_(count, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_math_utils2d.f.in:1674
void lsm2dvoxelcountlessthanzerocontrolvolume_(int *count, const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const double *control_vol, const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *jlo_control_vol_gb, const int *jhi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib) {
  Lift L_(2, "lsm2dvoxelcountlessthanzerocontrolvolume_");
  L_.box(ilo_gb, ihi_gb, jlo_gb, jhi_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib, jlo_ib, jhi_ib);
  if (!L_.ready()) return;
  lsm3dvoxelcountlessthanzerocontrolvolume_(count, phi, ilo_gb, ihi_gb, jlo_gb, jhi_gb, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb, ihi_control_vol_gb, jlo_control_vol_gb, jhi_control_vol_gb, &L_.k0, &L_.k0, control_vol_sgn, ilo_ib, ihi_ib, jlo_ib, jhi_ib, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d.f.in:16
void lsm2dzerooutlevelseteqnrhs_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb) {
  Lift L_(2, "lsm2dzerooutlevelseteqnrhs_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  if (!L_.ready()) return;
  lsm3dzerooutlevelseteqnrhs_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0);
}

// src/toolbox/lsm_level_set_evolution2d_local.f.in:16
void lsm2dzerooutlevelseteqnrhslocal_(double *lse_rhs, const int *ilo_lse_rhs_gb, const int *ihi_lse_rhs_gb, const int *jlo_lse_rhs_gb, const int *jhi_lse_rhs_gb, const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index) {
  Lift L_(2, "lsm2dzerooutlevelseteqnrhslocal_");
  L_.box(ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb);
  L_.list(nlo_index, nhi_index);
  if (!L_.ready()) return;
  lsm3dzerooutlevelseteqnrhslocal_(lse_rhs, ilo_lse_rhs_gb, ihi_lse_rhs_gb, jlo_lse_rhs_gb, jhi_lse_rhs_gb, &L_.k0, &L_.k0, index_x, index_y, L_.zero_int(), nlo_index, nhi_index);
}

}  // extern "C"
