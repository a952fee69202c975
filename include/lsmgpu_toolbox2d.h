/*
 * lsmgpu drop-in entry points for LSMLIB's 2D toolbox.
 *
 * Same conventions as lsmgpu_toolbox3d.h: LSMLIB's symbol names and
 * argument lists, column-major arrays over the ghost box given by the
 * bounds that follow them, double precision.  Each routine runs the 3D
 * kernels on its arrays (one cell along the missing axes, stride 0) and
 * matches the reference routine bit for bit.
 */
#ifndef LSMGPU_TOOLBOX2D_H
#define LSMGPU_TOOLBOX2D_H

#ifdef __cplusplus
extern "C" {
#endif

/* 2D form: rhs -= u . grad(phi).
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:47; C declaration src/toolbox/lsm_level_set_evolution2d.h:92.
 */
void lsm2daddadvectiontermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: advection term on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:55; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:106.
 */
void lsm2daddadvectiontermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: rhs += b * kappa |grad phi| from first and second derivatives.
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:273; C declaration src/toolbox/lsm_level_set_evolution2d.h:243.
 */
void lsm2daddconstcurvtermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi_xx,
  const double *phi_xy,
  const double *phi_yy,
  const int *ilo_grad2_phi_gb,
  const int *ihi_grad2_phi_gb,
  const int *jlo_grad2_phi_gb,
  const int *jhi_grad2_phi_gb,
  const double *b,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: curvature term on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:320; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:289.
 */
void lsm2daddconstcurvtermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi_xx,
  const double *phi_xy,
  const double *phi_yy,
  const int *ilo_grad2_phi_gb,
  const int *ihi_grad2_phi_gb,
  const int *jlo_grad2_phi_gb,
  const int *jhi_grad2_phi_gb,
  const double *b,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: rhs -= Vn |grad phi| (Godunov), Vn constant.
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:189; C declaration src/toolbox/lsm_level_set_evolution2d.h:193.
 */
void lsm2daddconstnormalveltermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: normal velocity term (constant) on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:227; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:226.
 */
void lsm2daddconstnormalveltermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: rhs += b * kappa * |grad phi| (loops k,j from the fill box to the ghost box end and i over the ghost box, as the reference does).
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:345; C declaration src/toolbox/lsm_level_set_evolution2d.h:288.
 */
void lsm2daddconstprecomputedcurvtermtolserhs_(
  double *lse_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *b,
  const int *ilo_rhs_fb,
  const int *ihi_rhs_fb,
  const int *jlo_rhs_fb,
  const int *jhi_rhs_fb);

/* 2D form: rhs += b * kappa * |grad phi| on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:408; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:47.
 */
void lsm2daddconstprecomputedcurvtermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *grad_phi_mag,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *b,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: rhs -= u . grad(phi) + Vn |grad phi| over the fill box, combined Godunov upwinding.
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:399; C declaration src/toolbox/lsm_level_set_evolution2d.h:341.
 */
void lsm2daddexternalandnormalveltermtolserhs_(
  double *lse_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *ilo_rhs_fb,
  const int *ihi_rhs_fb,
  const int *jlo_rhs_fb,
  const int *jhi_rhs_fb);

/* 2D form: external plus normal velocity term with the combined Godunov upwinding on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:474; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:414.
 */
void lsm2daddexternalandnormalveltermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: rhs -= Vn |grad phi| (Godunov), Vn a field.
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:101; C declaration src/toolbox/lsm_level_set_evolution2d.h:139.
 */
void lsm2daddnormalveltermtolserhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: normal velocity term (field) on band cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:126; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:163.
 */
void lsm2daddnormalveltermtolserhslocal_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: mean |field1 - field2| over an index box.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:69; C declaration src/toolbox/lsm_math_utils2d.h:121.
 */
void lsm2daveabsdiff_(
  double *ave_abs_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const int *jlo_field1_gb,
  const int *jhi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *jlo_field2_gb,
  const int *jhi_field2_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: average of plus and minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2322; C declaration src/toolbox/lsm_spatial_derivatives2d.h:739.
 */
void lsm2daveragegradphi_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: second-order central gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:1957; C declaration src/toolbox/lsm_spatial_derivatives2d.h:557.
 */
void lsm2dcentralgradorder2_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: second-order central gradient on band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1392; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:426.
 */
void lsm2dcentralgradorder2local_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: fourth-order central gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2021; C declaration src/toolbox/lsm_spatial_derivatives2d.h:599.
 */
void lsm2dcentralgradorder4_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: fourth-order central gradient on band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1465; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:469.
 */
void lsm2dcentralgradorder4local_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: second-order central Hessian.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2500; C declaration src/toolbox/lsm_spatial_derivatives2d.h:829.
 */
void lsm2dcentralhessian_(
  double *phi_xx,
  double *phi_xy,
  double *phi_yy,
  const int *ilo_hessian_gb,
  const int *ihi_hessian_gb,
  const int *jlo_hessian_gb,
  const int *jhi_hessian_gb,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: 1 when the outer band layer holds both signs of phi.
 * Replaces src/toolbox/lsm_localization2d.f:693; C declaration src/toolbox/lsm_localization2d.h:403.
 */
void lsm2dcheckouternarrowbandlayer_(
  int *change_sign,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const int *index_outer,
  const int *nlo_index_outer,
  const int *nhi_index_outer,
  const int *nlo_outer_plus,
  const int *nhi_outer_plus,
  const int *nlo_outer_minus,
  const int *nhi_outer_minus);

/* 2D form: average |grad phi| over band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1616; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:555.
 */
void lsm2dcomputeavegradphilocal_(
  double *grad_phi_ave,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: distance estimate for the subcell fix (2 phi0 / delta).
 * Replaces src/reinitialization/lsm_reinitialization2d.f.in:392; C declaration src/reinitialization/lsm_reinitialization2d.h:216.
 */
void lsm2dcomputedistanceforsubcellfix_(
  double *distance0,
  const double *phi0,
  const int *ilo_phi0_gb,
  const int *ihi_phi0_gb,
  const int *jlo_phi0_gb,
  const int *jhi_phi0_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: n-th undivided difference along dir (1e10 outside the fill range).
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:49.
 */
void lsm2dcomputedn_(
  double *dn,
  const int *ilo_dn_gb,
  const int *ihi_dn_gb,
  const int *jlo_dn_gb,
  const int *jhi_dn_gb,
  const double *dn_minus_one,
  const int *ilo_dn_minus_one_gb,
  const int *ihi_dn_minus_one_gb,
  const int *jlo_dn_minus_one_gb,
  const int *jhi_dn_minus_one_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *n,
  const int *dir);

/* 2D form: n-th undivided differences over an index list.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:43.
 */
void lsm2dcomputednlocal_(
  double *dn,
  const int *ilo_dn_gb,
  const int *ihi_dn_gb,
  const int *jlo_dn_gb,
  const int *jhi_dn_gb,
  const double *dn_minus_one,
  const int *ilo_dn_minus_one_gb,
  const int *ihi_dn_minus_one_gb,
  const int *jlo_dn_minus_one_gb,
  const int *jhi_dn_minus_one_gb,
  const int *n,
  const int *dir,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: second-order mean curvature.
 * Replaces src/geometry/lsm_curvature2d.f.in:15; C declaration src/geometry/lsm_curvature2d.h:59.
 */
void lsm2dcomputemeancurvatureorder2_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: second-order mean curvature on band cells.
 * Replaces src/geometry/lsm_curvature2d_local.f.in:15; C declaration src/geometry/lsm_curvature2d_local.h:64.
 */
void lsm2dcomputemeancurvatureorder2local_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: fourth-order mean curvature (cross derivatives from the first derivatives).
 * Replaces src/geometry/lsm_curvature2d.f.in:252; C declaration src/geometry/lsm_curvature2d.h:175.
 */
void lsm2dcomputemeancurvatureorder4_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: fourth-order mean curvature on band cells.
 * Replaces src/geometry/lsm_curvature2d_local.f.in:299; C declaration src/geometry/lsm_curvature2d_local.h:207.
 */
void lsm2dcomputemeancurvatureorder4local_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: orthogonalization RHS (sgn(psi) smoothed with max(dx)^2).
 * Replaces src/reinitialization/lsm_reinitialization2d.f.in:255; C declaration src/reinitialization/lsm_reinitialization2d.h:149.
 */
void lsm2dcomputeorthogonalizationeqnrhs_(
  double *ortho_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *psi,
  const int *ilo_psi_gb,
  const int *ihi_psi_gb,
  const int *jlo_psi_gb,
  const int *jhi_psi_gb,
  const double *psi_x_plus,
  const double *psi_y_plus,
  const int *ilo_grad_psi_plus_gb,
  const int *ihi_grad_psi_plus_gb,
  const int *jlo_grad_psi_plus_gb,
  const int *jhi_grad_psi_plus_gb,
  const double *psi_x_minus,
  const double *psi_y_minus,
  const int *ilo_grad_psi_minus_gb,
  const int *ihi_grad_psi_minus_gb,
  const int *jlo_grad_psi_minus_gb,
  const int *jhi_grad_psi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: orthogonalization RHS on band cells (sgn(psi) smoothed with max(dx)^2).
 * Replaces src/reinitialization/lsm_reinitialization2d_local.f.in:284; C declaration src/reinitialization/lsm_reinitialization2d_local.h:84.
 */
void lsm2dcomputeorthogonalizationeqnrhslocal_(
  double *ortho_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *psi,
  const int *ilo_psi_gb,
  const int *ihi_psi_gb,
  const int *jlo_psi_gb,
  const int *jhi_psi_gb,
  const double *psi_x_plus,
  const double *psi_y_plus,
  const int *ilo_grad_psi_plus_gb,
  const int *ihi_grad_psi_plus_gb,
  const int *jlo_grad_psi_plus_gb,
  const int *jhi_grad_psi_plus_gb,
  const double *psi_x_minus,
  const double *psi_y_minus,
  const int *ilo_grad_psi_minus_gb,
  const int *ihi_grad_psi_minus_gb,
  const int *jlo_grad_psi_minus_gb,
  const int *jhi_grad_psi_minus_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: reinitialization RHS sgn(phi)(1 - |grad phi|), Godunov.
 * Replaces src/reinitialization/lsm_reinitialization2d.f.in:48; C declaration src/reinitialization/lsm_reinitialization2d.h:78.
 */
void lsm2dcomputereinitializationeqnrhs_(
  double *reinit_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi0,
  const int *ilo_phi0_gb,
  const int *ihi_phi0_gb,
  const int *jlo_phi0_gb,
  const int *jhi_phi0_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy,
  const int *use_phi0_for_sgn);

/* 2D form: reinitialization RHS on band cells.
 * Replaces src/reinitialization/lsm_reinitialization2d_local.f.in:49; C declaration src/reinitialization/lsm_reinitialization2d_local.h:41.
 */
void lsm2dcomputereinitializationeqnrhslocal_(
  double *reinit_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi0,
  const int *ilo_phi0_gb,
  const int *ihi_phi0_gb,
  const int *jlo_phi0_gb,
  const int *jhi_phi0_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *dx,
  const double *dy,
  const int *use_phi0_for_sgn,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: first-order reinitialization RHS with the Russo-Smereka subcell fix.
 * Replaces src/reinitialization/lsm_reinitialization2d.f.in:468; C declaration src/reinitialization/lsm_reinitialization2d.h:259.
 */
void lsm2dcomputereinitializationeqnrhssubcellfixorder1_(
  double *reinit_rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi0,
  const double *distance0,
  const int *ilo_phi0_gb,
  const int *ihi_phi0_gb,
  const int *jlo_phi0_gb,
  const int *jhi_phi0_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: CFL-stable dt for advection.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:218; C declaration src/toolbox/lsm_math_utils2d.h:204.
 */
void lsm2dcomputestableadvectiondt_(
  double *dt,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable advection dt over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:868; C declaration src/toolbox/lsm_math_utils2d.h:548.
 */
void lsm2dcomputestableadvectiondtcontrolvolume_(
  double *dt,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable advection dt over band cells.
 * Replaces src/toolbox/lsm_math_utils2d_local.f.in:165; C declaration src/toolbox/lsm_math_utils2d_local.h:146.
 */
void lsm2dcomputestableadvectiondtlocal_(
  double *dt,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const double *dx,
  const double *dy,
  const double *cfl_number,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: CFL-stable dt for a constant normal velocity.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:382; C declaration src/toolbox/lsm_math_utils2d.h:297.
 */
void lsm2dcomputestableconstnormalveldt_(
  double *dt,
  const double *vel_n,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable constant normal-velocity dt over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1102; C declaration src/toolbox/lsm_math_utils2d.h:665.
 */
void lsm2dcomputestableconstnormalveldtcontrolvolume_(
  double *dt,
  const double *vel_n,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable constant normal-velocity dt over band cells (the reference routine reads two unassigned variables; this computes the dense routine's formula).
 * Replaces src/toolbox/lsm_math_utils2d_local.f.in:360; C declaration src/toolbox/lsm_math_utils2d_local.h:257.
 */
void lsm2dcomputestableconstnormalveldtlocal_(
  double *dt,
  const double *vel_n,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *dx,
  const double *dy,
  const double *cfl_number,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: CFL-stable dt for a normal velocity field.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:285; C declaration src/toolbox/lsm_math_utils2d.h:245.
 */
void lsm2dcomputestablenormalveldt_(
  double *dt,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable normal-velocity dt over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:966; C declaration src/toolbox/lsm_math_utils2d.h:601.
 */
void lsm2dcomputestablenormalveldtcontrolvolume_(
  double *dt,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *cfl_number);

/* 2D form: CFL-stable normal-velocity dt over band cells.
 * Replaces src/toolbox/lsm_math_utils2d_local.f.in:246; C declaration src/toolbox/lsm_math_utils2d_local.h:196.
 */
void lsm2dcomputestablenormalveldtlocal_(
  double *dt,
  const double *vel_n,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  const double *phi_x_plus,
  const double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  const double *phi_x_minus,
  const double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *dx,
  const double *dy,
  const double *cfl_number,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: dest = src on listed cells.
 * Replaces src/toolbox/lsm_localization2d.f:833; C declaration src/toolbox/lsm_localization2d.h:491.
 */
void lsm2dcopydatalocal_(
  double *dest,
  const int *ilo_dest_gb,
  const int *ihi_dest_gb,
  const int *jlo_dest_gb,
  const int *jhi_dest_gb,
  const double *src,
  const int *ilo_src_gb,
  const int *ihi_src_gb,
  const int *jlo_src_gb,
  const int *jhi_src_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index);

/* 2D form: copy extrapolation into the ghost cells of one face.
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:264; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:129.
 */
void lsm2dcopyextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: first-order delta function from sign changes (z terms use norm_phi_x and 1/dx, as the reference does).
 * Replaces src/toolbox/lsm_calculus_toolbox2d.f.in:16; C declaration src/toolbox/lsm_calculus_toolbox2d.h:45.
 */
void lsm2ddeltafunctionorder1_(
  const double *phi,
  double *delta,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const double *norm_phi_x,
  const double *norm_phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: build the narrow band: level-0 list in sweep order, outer lists, BFS levels.
 * Replaces src/toolbox/lsm_localization2d.f:139; C declaration src/toolbox/lsm_localization2d.h:94.
 */
void lsm2ddeterminenarrowband_(
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  int *index_x,
  int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  int *n_lo,
  int *n_hi,
  int *index_outer,
  const int *nlo_index_outer,
  const int *nhi_index_outer,
  int *nlo_outer_plus,
  int *nhi_outer_plus,
  int *nlo_outer_minus,
  int *nhi_outer_minus,
  const double *width,
  const double *width_inner,
  const int *level);

/* 2D form: build a narrow band of cells near phi = 0 and away from a mask (|phi - mask| > max dx).
 * Replaces src/toolbox/lsm_localization2d.f:365; C declaration src/toolbox/lsm_localization2d.h:237.
 */
void lsm2ddeterminenarrowbandawayfrommask_(
  const double *phi,
  const double *mask,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  int *index_x,
  int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  int *n_lo,
  int *n_hi,
  int *index_outer,
  const int *nlo_index_outer,
  const int *nhi_index_outer,
  int *nlo_outer_plus,
  int *nhi_outer_plus,
  int *nlo_outer_minus,
  int *nhi_outer_minus,
  const double *width,
  const double *width_inner,
  const int *level,
  const double *dx,
  const double *dy);

/* 2D form: build a narrow band from the sign of a mask.
 * Replaces src/toolbox/lsm_localization2d.f:539; C declaration src/toolbox/lsm_localization2d.h:328.
 */
void lsm2ddeterminenarrowbandfrommask_(
  const double *mask,
  const int *ilo_mask_gb,
  const int *ihi_mask_gb,
  const int *jlo_mask_gb,
  const int *jhi_mask_gb,
  unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  int *index_x,
  int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  int *n_lo,
  int *n_hi,
  const int *level,
  const int *use_mask_sign);

/* 2D form: build a narrow band of cells near the zero sets of both phi and psi.
 * Replaces src/toolbox/lsm_localization2d.f:248; C declaration src/toolbox/lsm_localization2d.h:165.
 */
void lsm2ddeterminenarrowbandfromtwolevelsets_(
  const double *phi,
  const double *psi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  int *index_x,
  int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  int *n_lo,
  int *n_hi,
  int *index_outer,
  const int *nlo_index_outer,
  const int *nhi_index_outer,
  int *nlo_outer_plus,
  int *nhi_outer_plus,
  int *nlo_outer_minus,
  int *nhi_outer_minus,
  const double *width,
  const double *width_inner,
  const int *level);

/* 2D form: |grad phi| with the reference's 1e-8 clamps.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2395; C declaration src/toolbox/lsm_spatial_derivatives2d.h:774.
 */
void lsm2dgradientmagnitude_(
  const double *phi_x,
  const double *phi_y,
  double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: |grad phi| on band cells (zero_tol clamps).
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1689; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:591.
 */
void lsm2dgradientmagnitudelocal_(
  const double *phi_x,
  const double *phi_y,
  double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: first-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:165; C declaration src/toolbox/lsm_spatial_derivatives2d.h:84.
 */
void lsm2dhjeno1_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: HJ ENO1 plus/minus gradients on level-0 band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:133; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:77.
 */
void lsm2dhjeno1local_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index0,
  const int *nhi_index0,
  const int *nlo_index1,
  const int *nhi_index1,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const unsigned char *mark_d1);

/* 2D form: second-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:296; C declaration src/toolbox/lsm_spatial_derivatives2d.h:147.
 */
void lsm2dhjeno2_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: HJ ENO2 plus/minus gradients on level-0 band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:280; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:145.
 */
void lsm2dhjeno2local_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index0,
  const int *nhi_index0,
  const int *nlo_index1,
  const int *nhi_index1,
  const int *nlo_index2,
  const int *nhi_index2,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const unsigned char *mark_d1,
  const unsigned char *mark_d2);

/* 2D form: third-order HJ ENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:479; C declaration src/toolbox/lsm_spatial_derivatives2d.h:216.
 */
void lsm2dhjeno3_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  double *d3,
  const int *ilo_d3_gb,
  const int *ihi_d3_gb,
  const int *jlo_d3_gb,
  const int *jhi_d3_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: HJ ENO3 plus/minus gradients on level-0 band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:498; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:220.
 */
void lsm2dhjeno3local_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  double *d3,
  const int *ilo_d3_gb,
  const int *ihi_d3_gb,
  const int *jlo_d3_gb,
  const int *jhi_d3_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index0,
  const int *nhi_index0,
  const int *nlo_index1,
  const int *nhi_index1,
  const int *nlo_index2,
  const int *nhi_index2,
  const int *nlo_index3,
  const int *nhi_index3,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const unsigned char *mark_d1,
  const unsigned char *mark_d2,
  const unsigned char *mark_d3);

/* 2D form: fifth-order HJ WENO plus/minus gradients.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:756; C declaration src/toolbox/lsm_spatial_derivatives2d.h:287.
 */
void lsm2dhjweno5_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: HJ WENO5 plus/minus gradients on level-0 band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:816; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:301.
 */
void lsm2dhjweno5local_(
  double *phi_x_plus,
  double *phi_y_plus,
  const int *ilo_grad_phi_plus_gb,
  const int *ihi_grad_phi_plus_gb,
  const int *jlo_grad_phi_plus_gb,
  const int *jhi_grad_phi_plus_gb,
  double *phi_x_minus,
  double *phi_y_minus,
  const int *ilo_grad_phi_minus_gb,
  const int *ihi_grad_phi_minus_gb,
  const int *jlo_grad_phi_minus_gb,
  const int *jhi_grad_phi_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index0,
  const int *nhi_index0,
  const int *nlo_index1,
  const int *nhi_index1,
  const int *nlo_index2,
  const int *nhi_index2,
  const int *nlo_index3,
  const int *nhi_index3,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const unsigned char *mark_d1);

/* 2D form: homogeneous Neumann fill for ENO1 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:360; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:153.
 */
void lsm2dhomogeneousneumanneno1_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: homogeneous Neumann fill for ENO2 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:403; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:176.
 */
void lsm2dhomogeneousneumanneno2_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: homogeneous Neumann fill for ENO3 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:446; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:199.
 */
void lsm2dhomogeneousneumanneno3_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: homogeneous Neumann fill for WENO5 (copy extrapolation).
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:489; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:222.
 */
void lsm2dhomogeneousneumannweno5_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: dest = max(mask, src) on listed cells.
 * Replaces src/toolbox/lsm_localization2d.f:778; C declaration src/toolbox/lsm_localization2d.h:421.
 */
void lsm2dimposemasklocal_(
  double *dest,
  const int *ilo_dest_gb,
  const int *ihi_dest_gb,
  const int *jlo_dest_gb,
  const int *jhi_dest_gb,
  const double *src,
  const int *ilo_src_gb,
  const int *ihi_src_gb,
  const int *jlo_src_gb,
  const int *jhi_src_gb,
  const double *mask,
  const int *ilo_mask_gb,
  const int *ihi_mask_gb,
  const int *jlo_mask_gb,
  const int *jhi_mask_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index);

/* 2D form: second-order Laplacian.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2091; C declaration src/toolbox/lsm_spatial_derivatives2d.h:643.
 */
void lsm2dlaplacianorder2_(
  double *laplacian_phi,
  const int *ilo_laplacian_phi_gb,
  const int *ihi_laplacian_phi_gb,
  const int *jlo_laplacian_phi_gb,
  const int *jhi_laplacian_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: second-order Laplacian on band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1542; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:512.
 */
void lsm2dlaplacianorder2local_(
  double *laplacian_phi,
  const int *ilo_laplacian_phi_gb,
  const int *ihi_laplacian_phi_gb,
  const int *jlo_laplacian_phi_gb,
  const int *jhi_laplacian_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: linear extrapolation into the ghost cells of one face.
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:44; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:69.
 */
void lsm2dlinearextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: mark the one-cell faces of a fill box.
 * Replaces src/toolbox/lsm_localization2d.f:486; C declaration src/toolbox/lsm_localization2d.h:283.
 */
void lsm2dmarknarrowbandboundarylayer_(
  unsigned char *narrow_band,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const unsigned char *mark_boundary_layer);

/* 2D form: breadth-first neighbour levels of a narrow band.
 * Replaces src/toolbox/lsm_localization2d.f:48.
 */
void lsm2dmarknarrowbandneighbors_(
  unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  int *index_x,
  int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  int *n_lo,
  int *n_hi,
  const int *level);

/* 2D form: max |field1 - field2| over an index box.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:15; C declaration src/toolbox/lsm_math_utils2d.h:90.
 */
void lsm2dmaxnormdiff_(
  double *max_norm_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const int *jlo_field1_gb,
  const int *jhi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *jlo_field2_gb,
  const int *jhi_field2_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: max |field1 - field2| over cells of one control-volume sign (seeded with the box corner).
 * Replaces src/toolbox/lsm_math_utils2d.f.in:777; C declaration src/toolbox/lsm_math_utils2d.h:505.
 */
void lsm2dmaxnormdiffcontrolvolume_(
  double *max_norm_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const int *jlo_field1_gb,
  const int *jhi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *jlo_field2_gb,
  const int *jhi_field2_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: max |field1 - field2| over band cells (starts at 0).
 * Replaces src/toolbox/lsm_math_utils2d_local.f.in:16; C declaration src/toolbox/lsm_math_utils2d_local.h:64.
 */
void lsm2dmaxnormdifflocal_(
  double *max_norm_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const int *jlo_field1_gb,
  const int *jhi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *jlo_field2_gb,
  const int *jhi_field2_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: cubic cut-off of the RHS between beta and gamma.
 * Replaces src/toolbox/lsm_localization2d.f:621; C declaration src/toolbox/lsm_localization2d.h:367.
 */
void lsm2dmultiplycutofflserhslocal_(
  const double *phi,
  double *lse_rhs,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const double *beta,
  const double *gamma);

/* 2D form: gradient of F upwinded by the local extremum of phi.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2166; C declaration src/toolbox/lsm_spatial_derivatives2d.h:690.
 */
void lsm2dphiupwindgradf_(
  double *f_x,
  double *f_y,
  const int *ilo_grad_f_gb,
  const int *ihi_grad_f_gb,
  const int *jlo_grad_f_gb,
  const int *jhi_grad_f_gb,
  const double *f_x_plus,
  const double *f_y_plus,
  const int *ilo_grad_f_plus_gb,
  const int *ihi_grad_f_plus_gb,
  const int *jlo_grad_f_plus_gb,
  const int *jhi_grad_f_plus_gb,
  const double *f_x_minus,
  const double *f_y_minus,
  const int *ilo_grad_f_minus_gb,
  const int *ihi_grad_f_minus_gb,
  const int *jlo_grad_f_minus_gb,
  const int *jhi_grad_f_minus_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb);

/* 2D form: forward Euler step u_next = u + dt*L.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:32; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:59.
 */
void lsm2drk1step_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: Euler step on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:33; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:35.
 */
void lsm2drk1steplocal_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: signed linear extrapolation into the ghost cells of one face.
 * Replaces src/boundary_conditions/lsm_boundary_conditions2d.f:149; C declaration src/boundary_conditions/lsm_boundary_conditions2d.h:107.
 */
void lsm2dsignedlinearextrapolation_(
  double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const int *bdry_location_idx);

/* 2D form: integral of F over {phi = 0} with a smoothed delta.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:625; C declaration src/toolbox/lsm_math_utils2d.h:418.
 */
void lsm2dsurfaceintegral_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: surface integral restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1472; C declaration src/toolbox/lsm_math_utils2d.h:821.
 */
void lsm2dsurfaceintegralcontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *phi_x,
  const double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: TVD RK2 stage 1 (an Euler step).
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:96; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:100.
 */
void lsm2dtvdrk2stage1_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: TVD RK2 stage 1 on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:123; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:64.
 */
void lsm2dtvdrk2stage1local_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: TVD RK2 stage 2: 0.5*(u + u1 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:160; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:138.
 */
void lsm2dtvdrk2stage2_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: TVD RK2 stage 2 on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:212; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:93.
 */
void lsm2dtvdrk2stage2local_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: TVD RK3 stage 1 (an Euler step).
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:232; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:184.
 */
void lsm2dtvdrk3stage1_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: TVD RK3 stage 1 on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:308; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:127.
 */
void lsm2dtvdrk3stage1local_(
  double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: TVD RK3 stage 2: 0.75*u + 0.25*(u1 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:296; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:222.
 */
void lsm2dtvdrk3stage2_(
  double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const int *jlo_u_stage2_gb,
  const int *jhi_u_stage2_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: TVD RK3 stage 2 on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:396; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:156.
 */
void lsm2dtvdrk3stage2local_(
  double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const int *jlo_u_stage2_gb,
  const int *jhi_u_stage2_gb,
  const double *u_stage1,
  const int *ilo_u_stage1_gb,
  const int *ihi_u_stage1_gb,
  const int *jlo_u_stage1_gb,
  const int *jhi_u_stage1_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: TVD RK3 stage 3: u/3 + 2/3*(u2 + dt*L).
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d.f:366; C declaration src/toolbox/lsm_tvd_runge_kutta2d.h:265.
 */
void lsm2dtvdrk3stage3_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const int *jlo_u_stage2_gb,
  const int *jhi_u_stage2_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dt);

/* 2D form: TVD RK3 stage 3 on band cells.
 * Replaces src/toolbox/lsm_tvd_runge_kutta2d_local.f:491; C declaration src/toolbox/lsm_tvd_runge_kutta2d_local.h:189.
 */
void lsm2dtvdrk3stage3local_(
  double *u_next,
  const int *ilo_u_next_gb,
  const int *ihi_u_next_gb,
  const int *jlo_u_next_gb,
  const int *jhi_u_next_gb,
  const double *u_stage2,
  const int *ilo_u_stage2_gb,
  const int *ihi_u_stage2_gb,
  const int *jlo_u_stage2_gb,
  const int *jhi_u_stage2_gb,
  const double *u_cur,
  const int *ilo_u_cur_gb,
  const int *ihi_u_cur_gb,
  const int *jlo_u_cur_gb,
  const int *jhi_u_cur_gb,
  const double *rhs,
  const int *ilo_rhs_gb,
  const int *ihi_rhs_gb,
  const int *jlo_rhs_gb,
  const int *jhi_rhs_gb,
  const double *dt,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D form: first-order upwind HJ ENO gradient for a velocity field.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:1069; C declaration src/toolbox/lsm_spatial_derivatives2d.h:337.
 */
void lsm2dupwindhjeno1_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: second-order upwind HJ ENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:1214; C declaration src/toolbox/lsm_spatial_derivatives2d.h:388.
 */
void lsm2dupwindhjeno2_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: upwind HJ ENO2 gradient for a velocity field on level-0 band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1160; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:361.
 */
void lsm2dupwindhjeno2local_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index0,
  const int *nhi_index0,
  const int *nlo_index1,
  const int *nhi_index1,
  const int *nlo_index2,
  const int *nhi_index2,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb,
  const unsigned char *mark_d1,
  const unsigned char *mark_d2);

/* 2D form: third-order upwind HJ ENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:1416; C declaration src/toolbox/lsm_spatial_derivatives2d.h:445.
 */
void lsm2dupwindhjeno3_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  double *d2,
  const int *ilo_d2_gb,
  const int *ihi_d2_gb,
  const int *jlo_d2_gb,
  const int *jhi_d2_gb,
  double *d3,
  const int *ilo_d3_gb,
  const int *ihi_d3_gb,
  const int *jlo_d3_gb,
  const int *jhi_d3_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: fifth-order upwind HJ WENO gradient.
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:1699; C declaration src/toolbox/lsm_spatial_derivatives2d.h:505.
 */
void lsm2dupwindhjweno5_(
  double *phi_x,
  double *phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *vel_x,
  const double *vel_y,
  const int *ilo_vel_gb,
  const int *ihi_vel_gb,
  const int *jlo_vel_gb,
  const int *jhi_vel_gb,
  double *d1,
  const int *ilo_d1_gb,
  const int *ihi_d1_gb,
  const int *jlo_d1_gb,
  const int *jhi_d1_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D form: integral of F over {phi > 0} with a smoothed Heaviside.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:549; C declaration src/toolbox/lsm_math_utils2d.h:379.
 */
void lsm2dvolumeintegralphigreaterthanzero_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: volume integral over {phi > 0} restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1353; C declaration src/toolbox/lsm_math_utils2d.h:770.
 */
void lsm2dvolumeintegralphigreaterthanzerocontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: integral of F over {phi < 0} with a smoothed Heaviside.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:473; C declaration src/toolbox/lsm_math_utils2d.h:340.
 */
void lsm2dvolumeintegralphilessthanzero_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: volume integral over {phi < 0} restricted to one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1234; C declaration src/toolbox/lsm_math_utils2d.h:719.
 */
void lsm2dvolumeintegralphilessthanzerocontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy,
  const double *epsilon);

/* 2D form: number of cells with phi > 0.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:132; C declaration src/toolbox/lsm_math_utils2d.h:152.
 */
void lsm2dvoxelcountgreaterthanzero_(
  int *count,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: number of cells with phi > 0 and the selected control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1604; C declaration src/toolbox/lsm_math_utils2d.h:866.
 */
void lsm2dvoxelcountgreaterthanzerocontrolvolume_(
  int *count,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: number of cells with phi < 0.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:175; C declaration src/toolbox/lsm_math_utils2d.h:178.
 */
void lsm2dvoxelcountlessthanzero_(
  int *count,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: number of cells with phi < 0 and the selected control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1674; C declaration src/toolbox/lsm_math_utils2d.h:897.
 */
void lsm2dvoxelcountlessthanzerocontrolvolume_(
  int *count,
  const double *phi,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib);

/* 2D form: zero the level set equation RHS over its ghost box.
 * Replaces src/toolbox/lsm_level_set_evolution2d.f.in:16; C declaration src/toolbox/lsm_level_set_evolution2d.h:64.
 */
void lsm2dzerooutlevelseteqnrhs_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb);

/* 2D form: zero the RHS on listed cells.
 * Replaces src/toolbox/lsm_level_set_evolution2d_local.f.in:16; C declaration src/toolbox/lsm_level_set_evolution2d_local.h:70.
 */
void lsm2dzerooutlevelseteqnrhslocal_(
  double *lse_rhs,
  const int *ilo_lse_rhs_gb,
  const int *ihi_lse_rhs_gb,
  const int *jlo_lse_rhs_gb,
  const int *jhi_lse_rhs_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index);

/* 2D: mean curvature from a 9-point stencil (face gradients).
 * Replaces src/geometry/lsm_curvature2d.f.in:98; C declaration src/geometry/lsm_curvature2d.h:102.
 */
void lsm2dcomputemeancurvature9stencil_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D: mean curvature from a 9-point stencil on band cells.
 * Replaces src/geometry/lsm_curvature2d_local.f.in:115; C declaration src/geometry/lsm_curvature2d_local.h:116.
 */
void lsm2dcomputemeancurvature9stencillocal_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D: mean curvature of a signed distance function, Laplacian / (1 - phi Laplacian).
 * Replaces src/geometry/lsm_curvature2d.f.in:178; C declaration src/geometry/lsm_curvature2d.h:140.
 */
void lsm2dcomputemeancurvaturesgndist_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D: signed-distance mean curvature on band cells (dx where the denominator vanishes, as the reference).
 * Replaces src/geometry/lsm_curvature2d_local.f.in:211; C declaration src/geometry/lsm_curvature2d_local.h:162.
 */
void lsm2dcomputemeancurvaturesgndistlocal_(
  double *kappa,
  const int *ilo_kappa_gb,
  const int *ihi_kappa_gb,
  const int *jlo_kappa_gb,
  const int *jhi_kappa_gb,
  const double *phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D: second-order central divergence of (fx, fy).
 * Replaces src/toolbox/lsm_spatial_derivatives2d.f.in:2452; C declaration src/toolbox/lsm_spatial_derivatives2d.h:799.
 */
void lsm2ddivergencecentral_(
  double *divf,
  const int *ilo_divf_gb,
  const int *ihi_divf_gb,
  const int *jlo_divf_gb,
  const int *jhi_divf_gb,
  const double *fx,
  const double *fy,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D: second-order central divergence on band cells.
 * Replaces src/toolbox/lsm_spatial_derivatives2d_local.f.in:1769; C declaration src/toolbox/lsm_spatial_derivatives2d_local.h:628.
 */
void lsm2ddivergencecentrallocal_(
  double *divf,
  const int *ilo_divf_gb,
  const int *ihi_divf_gb,
  const int *jlo_divf_gb,
  const int *jhi_divf_gb,
  const double *fx,
  const double *fy,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const double *dx,
  const double *dy,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

/* 2D: second-order delta function (Smereka) from phi and the unit normal.
 * Replaces src/toolbox/lsm_calculus_toolbox2d.f.in:100; C declaration src/toolbox/lsm_calculus_toolbox2d.h:83.
 */
void lsm2ddeltafunctionorder2_(
  const double *phi,
  double *delta,
  const int *ilo_gb,
  const int *ihi_gb,
  const int *jlo_gb,
  const int *jhi_gb,
  const double *norm_phi_x,
  const double *norm_phi_y,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_fb,
  const int *ihi_fb,
  const int *jlo_fb,
  const int *jhi_fb,
  const double *dx,
  const double *dy);

/* 2D: integral of F delta |grad phi| dV over an index box (index box from the C declaration).
 * Replaces src/toolbox/lsm_math_utils2d.f.in:713; C declaration src/toolbox/lsm_math_utils2d.h:462.
 */
void lsm2dsurfaceintegralprecomputeddelta_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *delta_phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy);

/* 2D: integral of F delta |grad phi| dV over cells of one control-volume sign.
 * Replaces src/toolbox/lsm_math_utils2d.f.in:1744; C declaration src/toolbox/lsm_math_utils2d.h:938.
 */
void lsm2dsurfaceintegralprecomputeddeltacontrolvolume_(
  double *int_f,
  const double *f,
  const int *ilo_f_gb,
  const int *ihi_f_gb,
  const int *jlo_f_gb,
  const int *jhi_f_gb,
  const double *delta_phi,
  const int *ilo_phi_gb,
  const int *ihi_phi_gb,
  const int *jlo_phi_gb,
  const int *jhi_phi_gb,
  const double *grad_phi_mag,
  const int *ilo_grad_phi_gb,
  const int *ihi_grad_phi_gb,
  const int *jlo_grad_phi_gb,
  const int *jhi_grad_phi_gb,
  const double *control_vol,
  const int *ilo_control_vol_gb,
  const int *ihi_control_vol_gb,
  const int *jlo_control_vol_gb,
  const int *jhi_control_vol_gb,
  const int *control_vol_sgn,
  const int *ilo_ib,
  const int *ihi_ib,
  const int *jlo_ib,
  const int *jhi_ib,
  const double *dx,
  const double *dy);

/* 2D: mean |field1 - field2| over band cells (0 when none).
 * Replaces src/toolbox/lsm_math_utils2d_local.f.in:86; C declaration src/toolbox/lsm_math_utils2d_local.h:106.
 */
void lsm2daveabsdifflocal_(
  double *ave_abs_diff,
  const double *field1,
  const int *ilo_field1_gb,
  const int *ihi_field1_gb,
  const int *jlo_field1_gb,
  const int *jhi_field1_gb,
  const double *field2,
  const int *ilo_field2_gb,
  const int *ihi_field2_gb,
  const int *jlo_field2_gb,
  const int *jhi_field2_gb,
  const int *index_x,
  const int *index_y,
  const int *nlo_index,
  const int *nhi_index,
  const unsigned char *narrow_band,
  const int *ilo_nb_gb,
  const int *ihi_nb_gb,
  const int *jlo_nb_gb,
  const int *jhi_nb_gb,
  const unsigned char *mark_fb);

#ifdef __cplusplus
}
#endif

#endif /* LSMGPU_TOOLBOX2D_H */
