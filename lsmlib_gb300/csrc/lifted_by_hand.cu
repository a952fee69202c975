// LSMLIB's 1D normal-velocity dt routines on the 3D advection dt kernels.
//
// lsm1dComputeStableNormalVelDt (math_utils1d.f.in:157) and its control-volume
// form (:633) take phi_x_plus / phi_x_minus but read only |vel_n| / dx: dt =
// cfl / (max over the box of |vel_n| / dx + 1e-36), the maximum starting at
// -1.  That is the 3D advection dt (math_utils3d.f.in:253, :1887) with
// vel_x = vel_n and zero y and z velocities: |vel_n| / dx + 0 / dx + 0 / dx is
// |vel_n| / dx exactly.  The gradient arguments are accepted and not read.
// The control-volume form takes a cell where control_vol_sgn * control_vol > 0
// (math_utils1d.f.in:686), which is the 3D selection for the documented signs
// 1 and -1.
// Declared in include/lsmgpu_toolbox1d.h.
#include "lift.cuh"
#include "../../include/lsmgpu_toolbox3d.h"
#include "../../include/lsmgpu_toolbox1d.h"

using lsmgpu::Lift;

extern "C" {

void lsm1dcomputestablenormalveldt_(double *dt, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb,
                                    const double *phi_x_plus, const int *ilo_grad_phi_plus_gb,
                                    const int *ihi_grad_phi_plus_gb, const double *phi_x_minus,
                                    const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb,
                                    const int *ilo_ib, const int *ihi_ib, const double *dx,
                                    const double *cfl_number) {
  (void)phi_x_plus; (void)ilo_grad_phi_plus_gb; (void)ihi_grad_phi_plus_gb;
  (void)phi_x_minus; (void)ilo_grad_phi_minus_gb; (void)ihi_grad_phi_minus_gb;
  Lift L_(1, "lsm1dcomputestablenormalveldt_");
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondt_(dt, vel_n, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0, &L_.k0, &L_.k0,
                                 &L_.k0, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx, dx, dx, cfl_number);
}

void lsm1dcomputestablenormalveldtcontrolvolume_(
    double *dt, const double *vel_n, const int *ilo_vel_gb, const int *ihi_vel_gb, const double *phi_x_plus,
    const int *ilo_grad_phi_plus_gb, const int *ihi_grad_phi_plus_gb, const double *phi_x_minus,
    const int *ilo_grad_phi_minus_gb, const int *ihi_grad_phi_minus_gb, const double *control_vol,
    const int *ilo_control_vol_gb, const int *ihi_control_vol_gb, const int *control_vol_sgn, const int *ilo_ib,
    const int *ihi_ib, const double *dx, const double *cfl_number) {
  (void)phi_x_plus; (void)ilo_grad_phi_plus_gb; (void)ihi_grad_phi_plus_gb;
  (void)phi_x_minus; (void)ilo_grad_phi_minus_gb; (void)ihi_grad_phi_minus_gb;
  Lift L_(1, "lsm1dcomputestablenormalveldtcontrolvolume_");
  L_.box(ilo_vel_gb, ihi_vel_gb);
  L_.box(ilo_control_vol_gb, ihi_control_vol_gb);
  L_.box(ilo_ib, ihi_ib);
  if (!L_.ready()) return;
  lsm3dcomputestableadvectiondtcontrolvolume_(dt, vel_n, L_.zero(), L_.zero(), ilo_vel_gb, ihi_vel_gb, &L_.k0,
                                              &L_.k0, &L_.k0, &L_.k0, control_vol, ilo_control_vol_gb,
                                              ihi_control_vol_gb, &L_.k0, &L_.k0, &L_.k0, &L_.k0,
                                              control_vol_sgn, ilo_ib, ihi_ib, &L_.k0, &L_.k0, &L_.k0, &L_.k0, dx,
                                              dx, dx, cfl_number);
}

}  // extern "C"
