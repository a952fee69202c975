/*
 * lsmgpu drop-in entry points for LSMLIB's 1D toolbox.
 *
 * Same conventions as lsmgpu_toolbox3d.h: LSMLIB's symbol names and
 * argument lists, column-major arrays over the ghost box given by the
 * bounds that follow them, double precision.  Each routine runs the 3D
 * kernels on its arrays (one cell along the missing axes, stride 0) and
 * matches the reference routine bit for bit.
 */
#ifndef LSMGPU_TOOLBOX1D_H
#define LSMGPU_TOOLBOX1D_H

#ifdef __cplusplus
extern "C" {
#endif

/* 1D form: rhs -= u . grad(phi).
 * Replaces src/toolbox/lsm_level_set_evolution1d.f.in:65; C declaration src/toolbox/lsm_level_set_evolution1d.h:83.
 */
void lsm1daddadvectiontermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *ilo_fb,
  const int *ihi_fb);

/* 1D form: rhs -= Vn |grad phi| (Godunov), Vn a field.
 * Replaces src/toolbox/lsm_level_set_evolution1d.f.in:118; C declaration src/toolbox/lsm_level_set_evolution1d.h:120.
 */
void lsm1daddnormalveltermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *ilo_fb,
  const int *ihi_fb);

/* 1D form: average of plus and minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1471; C declaration src/toolbox/lsm_spatial_derivatives1d.h:576.
 */
void lsm1daveragegradphi_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb);

/* 1D form: second-order central gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1198; C declaration src/toolbox/lsm_spatial_derivatives1d.h:432.
 */
void lsm1dcentralgradorder2_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: fourth-order central gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1250; C declaration src/toolbox/lsm_spatial_derivatives1d.h:466.
 */
void lsm1dcentralgradorder4_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: n-th undivided difference along dir (1e10 outside the fill range).
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:49.
 */
void lsm1dcomputedn_(
  double *dn,
  const int *ilo_dn_gb,
  const int *ihi_dn_gb,
  const double *dn_minus_one,
  const int *ilo_dn_minus_one_gb,
  const int *ihi_dn_minus_one_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *n);

/* 1D form: reinitialization RHS sgn(phi)(1 - |grad phi|), Godunov.
 * Replaces src/reinitialization/lsm_reinitialization1d.f.in:48; C declaration src/reinitialization/lsm_reinitialization1d.h:71.
 */
void lsm1dcomputereinitializationeqnrhs_(
  double *reinit_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *phi0,
  const int *ilo_phi0_gb,
  const int *ihi_phi0_gb,
  const double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx,
  const int *use_phi0_for_sgn);

/* 1D form: CFL-stable dt for advection.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:81; C declaration src/toolbox/lsm_math_utils1d.h:101.
 */
void lsm1dcomputestableadvectiondt_(
  double *dt,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *cfl_number);

/* 1D form: CFL-stable advection dt over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:542; C declaration src/toolbox/lsm_math_utils1d.h:310.
 */
void lsm1dcomputestableadvectiondtcontrolvolume_(
  double *dt,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *cfl_number);

/* 1D form: CFL-stable dt for a normal velocity: max |vel_n| / dx.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:157; C declaration src/toolbox/lsm_math_utils1d.h:136.
 */
void lsm1dcomputestablenormalveldt_(
  double *dt,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *cfl_number);

/* 1D form: CFL-stable dt for a normal velocity over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:633; C declaration src/toolbox/lsm_math_utils1d.h:355.
 */
void lsm1dcomputestablenormalveldtcontrolvolume_(
  double *dt,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *cfl_number);

/* 1D form: copy extrapolation into the ghost cells of one face.
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:169; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:123.
 */
void lsm1dcopyextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: first-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:135; C declaration src/toolbox/lsm_spatial_derivatives1d.h:80.
 */
void lsm1dhjeno1_(
  double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: second-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:228; C declaration src/toolbox/lsm_spatial_derivatives1d.h:128.
 */
void lsm1dhjeno2_(
  double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: third-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:344; C declaration src/toolbox/lsm_spatial_derivatives1d.h:180.
 */
void lsm1dhjeno3_(
  double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  double *d3,
  const int *ilo_d3_gb,
  const int *ihi_d3_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: fifth-order HJ WENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:499; C declaration src/toolbox/lsm_spatial_derivatives1d.h:233.
 */
void lsm1dhjweno5_(
  double *phi_x_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  double *phi_x_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: homogeneous Neumann fill for ENO1 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:225; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:145.
 */
void lsm1dhomogeneousneumanneno1_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: homogeneous Neumann fill for ENO2 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:268; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:166.
 */
void lsm1dhomogeneousneumanneno2_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: homogeneous Neumann fill for ENO3 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:311; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:187.
 */
void lsm1dhomogeneousneumanneno3_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: homogeneous Neumann fill for WENO5 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:354; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:208.
 */
void lsm1dhomogeneousneumannweno5_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: second-order Laplacian.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1305; C declaration src/toolbox/lsm_spatial_derivatives1d.h:500.
 */
void lsm1dlaplacianorder2_(
  double *laplacian_phi,
  const int *ilo_laplacian_phi_gb,
  const int *ihi_laplacian_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: linear extrapolation into the ghost cells of one face.
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:42; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:67.
 */
void lsm1dlinearextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: max |field1 - field2| over an index box.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:27; C declaration src/toolbox/lsm_math_utils1d.h:75.
 */
void lsm1dmaxnormdiff_(
  double *max_norm_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *ilo_ib,
  const int *ihi_ib);

/* 1D form: max |field1 - field2| over cells of one control-volume sign (seeded with the box corner).
 * Replaces src/toolbox/lsm_math_utils1d.f.in:470; C declaration src/toolbox/lsm_math_utils1d.h:274.
 */
void lsm1dmaxnormdiffcontrolvolume_(
  double *max_norm_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib);

/* 1D form: gradient of F upwinded by the local extremum of phi.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1369; C declaration src/toolbox/lsm_spatial_derivatives1d.h:540.
 */
void lsm1dphiupwindgradf_(
  double *f_x,
  const int *ilo_grad_f_gb,
  const int *ihi_grad_f_gb,
  const double *f_x_plus,
  const int *ilo_grad_f_plus_gb,
  const int *ihi_grad_f_plus_gb,
  const double *f_x_minus,
  const int *ilo_grad_f_minus_gb,
  const int *ihi_grad_f_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb);

/* 1D form: forward Euler step u_next = u + dt*L.
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:32; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:59.
 */
void lsm1drk1step_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: signed linear extrapolation, sign from the cell next to the edge.
 * Replaces src/boundary_conditions/lsm_boundary_conditions1d.f:103; C declaration src/boundary_conditions/lsm_boundary_conditions1d.h:103.
 */
void lsm1dsignedlinearextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *bdry_location_idx);

/* 1D form: integral of F over {phi = 0} with a smoothed delta.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:390; C declaration src/toolbox/lsm_math_utils1d.h:238.
 */
void lsm1dsurfaceintegral_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: surface integral restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:924; C declaration src/toolbox/lsm_math_utils1d.h:487.
 */
void lsm1dsurfaceintegralcontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: TVD RK2 stage 1 (an Euler step).
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:85; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:92.
 */
void lsm1dtvdrk2stage1_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: TVD RK2 stage 2: 0.5*(u + u1 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:137; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:122.
 */
void lsm1dtvdrk2stage2_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: TVD RK3 stage 1 (an Euler step).
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:195; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:158.
 */
void lsm1dtvdrk3stage1_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: TVD RK3 stage 2: 0.75*u + 0.25*(u1 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:247; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:188.
 */
void lsm1dtvdrk3stage2_(
  double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: TVD RK3 stage 3: u/3 + 2/3*(u2 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta1d.f:303; C declaration src/toolbox/lsm_tvd_runge_kutta1d.h:221.
 */
void lsm1dtvdrk3stage3_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dt);

/* 1D form: first-order upwind HJ ENO gradient for a velocity field.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:680; C declaration src/toolbox/lsm_spatial_derivatives1d.h:270.
 */
void lsm1dupwindhjeno1_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: second-order upwind HJ ENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:771; C declaration src/toolbox/lsm_spatial_derivatives1d.h:308.
 */
void lsm1dupwindhjeno2_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: third-order upwind HJ ENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:888; C declaration src/toolbox/lsm_spatial_derivatives1d.h:350.
 */
void lsm1dupwindhjeno3_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  double *d3,
  const int *ilo_d3_gb,
  const int *ihi_d3_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: fifth-order upwind HJ WENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives1d.f.in:1042; C declaration src/toolbox/lsm_spatial_derivatives1d.h:393.
 */
void lsm1dupwindhjweno5_(
  double *phi_x,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *vel_x,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const double *dx);

/* 1D form: integral of F over {phi > 0} with a smoothed Heaviside.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:315; C declaration src/toolbox/lsm_math_utils1d.h:205.
 */
void lsm1dvolumeintegralphigreaterthanzero_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: volume integral over {phi > 0} restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:828; C declaration src/toolbox/lsm_math_utils1d.h:444.
 */
void lsm1dvolumeintegralphigreaterthanzerocontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: integral of F over {phi < 0} with a smoothed Heaviside.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:238; C declaration src/toolbox/lsm_math_utils1d.h:172.
 */
void lsm1dvolumeintegralphilessthanzero_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: volume integral over {phi < 0} restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils1d.f.in:732; C declaration src/toolbox/lsm_math_utils1d.h:401.
 */
void lsm1dvolumeintegralphilessthanzerocontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const double *dx,
  const double *epsilon);

/* 1D form: zero the level set equation RHS over its ghost box.
 * Replaces src/toolbox/lsm_level_set_evolution1d.f.in:25; C declaration src/toolbox/lsm_level_set_evolution1d.h:57.
 */
void lsm1dzerooutlevelseteqnrhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb);

#ifdef __cplusplus
}
#endif

#endif /* LSMGPU_TOOLBOX1D_H */
