// extern "C" entry points of the advection adjoint for one precision;
// included by adjoint_f64.cu (double, FP64 arithmetic without contraction)
// and adjoint_f32.cu (float, FP32 arithmetic).
#pragma once
#include "adjoint_driver.cuh"

#define LSMGPU_ACAT2(a, b) a##b
#define LSMGPU_ACAT(a, b) LSMGPU_ACAT2(a, b)

using namespace lsmgpu;

static Box adj_box6(const int *b) {
  Box r;
  r.lo[0] = b[0]; r.hi[0] = b[1];
  r.lo[1] = b[2]; r.hi[1] = b[3];
  r.lo[2] = b[4]; r.hi[2] = b[5];
  return r;
}

extern "C" int LSMGPU_ACAT(lsmgpu_advect_adjoint_weno5_tvdrk3_, LSMGPU_ADJ_SUFFIX)(
    const LSMGPU_ADJ_R *phi, const int *gb, const int *fb, const LSMGPU_ADJ_R *vel_x,
    const LSMGPU_ADJ_R *vel_y, const LSMGPU_ADJ_R *vel_z, const int *vel_gb, const LSMGPU_ADJ_R *phi_target,
    LSMGPU_ADJ_R dx, LSMGPU_ADJ_R dy, LSMGPU_ADJ_R dz, LSMGPU_ADJ_R dt, int n_steps, int checkpoint_every,
    double heaviside_eps, double *J, LSMGPU_ADJ_R *grad_phi, LSMGPU_ADJ_R *grad_vel_x,
    LSMGPU_ADJ_R *grad_vel_y, LSMGPU_ADJ_R *grad_vel_z) {
  clear_error();
  if (!phi || !gb || !fb || !vel_x || !vel_y || !vel_z || !vel_gb || !phi_target) {
    set_error(LSMGPU_ERR_ARGUMENT, "lsmgpu_advect_adjoint_weno5_tvdrk3: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  adj::AdjSpec sp{};
  sp.n_steps = n_steps;
  sp.ckpt = checkpoint_every;
  sp.dt = dt; sp.dx = dx; sp.dy = dy; sp.dz = dz;
  sp.eps = heaviside_eps;
  const LSMGPU_ADJ_R *vel[3] = {vel_x, vel_y, vel_z};
  LSMGPU_ADJ_R *gvel[3] = {grad_vel_x, grad_vel_y, grad_vel_z};
  return adj::run<LSMGPU_ADJ_R, LSMGPU_ADJ_EXACT>("lsmgpu_advect_adjoint_weno5_tvdrk3", phi, adj_box6(gb),
                                                  adj_box6(fb), vel, adj_box6(vel_gb), phi_target, sp, J,
                                                  grad_phi, gvel);
}
