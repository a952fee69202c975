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
  sp.mode = adj::ADJ_MODE_ADVECT;
  sp.n_steps = n_steps;
  sp.ckpt = checkpoint_every;
  sp.dt = dt; sp.dx = dx; sp.dy = dy; sp.dz = dz;
  sp.eps = heaviside_eps;
  adj::AdjIO<LSMGPU_ADJ_R> io{};
  io.phi = phi;
  io.vel[0] = vel_x; io.vel[1] = vel_y; io.vel[2] = vel_z;
  io.tgt = phi_target;
  io.J = J;
  io.gphi = grad_phi;
  io.gvel[0] = grad_vel_x; io.gvel[1] = grad_vel_y; io.gvel[2] = grad_vel_z;
  return adj::run<LSMGPU_ADJ_R, LSMGPU_ADJ_EXACT>("lsmgpu_advect_adjoint_weno5_tvdrk3", adj_box6(gb), adj_box6(fb),
                                                  adj_box6(vel_gb), sp, io);
}

extern "C" int LSMGPU_ACAT(lsmgpu_advect_vjp_weno5_tvdrk3_, LSMGPU_ADJ_SUFFIX)(
    const LSMGPU_ADJ_R *phi, const int *gb, const int *fb, const LSMGPU_ADJ_R *vel_x,
    const LSMGPU_ADJ_R *vel_y, const LSMGPU_ADJ_R *vel_z, const int *vel_gb, LSMGPU_ADJ_R dx, LSMGPU_ADJ_R dy,
    LSMGPU_ADJ_R dz, LSMGPU_ADJ_R dt, int n_steps, int checkpoint_every, const LSMGPU_ADJ_R *grad_out,
    LSMGPU_ADJ_R *phi_out, LSMGPU_ADJ_R *grad_phi, LSMGPU_ADJ_R *grad_vel_x, LSMGPU_ADJ_R *grad_vel_y,
    LSMGPU_ADJ_R *grad_vel_z) {
  clear_error();
  if (!phi || !gb || !fb || !vel_x || !vel_y || !vel_z || !vel_gb || (grad_phi && !grad_out)) {
    set_error(LSMGPU_ERR_ARGUMENT, "lsmgpu_advect_vjp_weno5_tvdrk3: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  adj::AdjSpec sp{};
  sp.mode = adj::ADJ_MODE_ADVECT;
  sp.n_steps = n_steps;
  sp.ckpt = checkpoint_every;
  sp.dt = dt; sp.dx = dx; sp.dy = dy; sp.dz = dz;
  adj::AdjIO<LSMGPU_ADJ_R> io{};
  io.phi = phi;
  io.vel[0] = vel_x; io.vel[1] = vel_y; io.vel[2] = vel_z;
  io.grad_out = grad_out;
  io.phi_out = phi_out;
  io.gphi = grad_phi;
  io.gvel[0] = grad_vel_x; io.gvel[1] = grad_vel_y; io.gvel[2] = grad_vel_z;
  return adj::run<LSMGPU_ADJ_R, LSMGPU_ADJ_EXACT>("lsmgpu_advect_vjp_weno5_tvdrk3", adj_box6(gb), adj_box6(fb),
                                                  adj_box6(vel_gb), sp, io);
}

extern "C" int LSMGPU_ACAT(lsmgpu_reinit_vjp_weno5_tvdrk3_, LSMGPU_ADJ_SUFFIX)(
    const LSMGPU_ADJ_R *phi, const int *gb, const int *fb, LSMGPU_ADJ_R dx, LSMGPU_ADJ_R dy, LSMGPU_ADJ_R dz,
    LSMGPU_ADJ_R dtau, int n_iter, int checkpoint_every, const LSMGPU_ADJ_R *grad_out, LSMGPU_ADJ_R *phi_out,
    LSMGPU_ADJ_R *grad_phi) {
  clear_error();
  if (!phi || !gb || !fb || (grad_phi && !grad_out)) {
    set_error(LSMGPU_ERR_ARGUMENT, "lsmgpu_reinit_vjp_weno5_tvdrk3: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  adj::AdjSpec sp{};
  sp.mode = adj::ADJ_MODE_REINIT;
  sp.n_steps = n_iter;
  sp.ckpt = checkpoint_every;
  sp.dt = dtau; sp.dx = dx; sp.dy = dy; sp.dz = dz;
  adj::AdjIO<LSMGPU_ADJ_R> io{};
  io.phi = phi;
  io.grad_out = grad_out;
  io.phi_out = phi_out;
  io.gphi = grad_phi;
  return adj::run<LSMGPU_ADJ_R, LSMGPU_ADJ_EXACT>("lsmgpu_reinit_vjp_weno5_tvdrk3", adj_box6(gb), adj_box6(fb),
                                                  Box{}, sp, io);
}
