// extern "C" entry points of the fused steppers for one precision; included
// by fused_f64.cu (LSMGPU_FUSED_R = double, parity arithmetic) and
// fused_f32.cu (float, fast arithmetic).
#pragma once
#include "fused_driver.cuh"
#include "curvature_fused.cuh"

#define LSMGPU_CAT2(a, b) a##b
#define LSMGPU_CAT(a, b) LSMGPU_CAT2(a, b)

using namespace lsmgpu;
using namespace lsmgpu::fused;

static Box box6(const int *b) {
  Box r;
  r.lo[0] = b[0]; r.hi[0] = b[1];
  r.lo[1] = b[2]; r.hi[1] = b[3];
  r.lo[2] = b[4]; r.hi[2] = b[5];
  return r;
}

extern "C" {

int LSMGPU_CAT(lsmgpu_reinit_weno5_tvdrk3_, LSMGPU_FUSED_SUFFIX)(
    LSMGPU_FUSED_R *phi, const int *gb, const int *fb, LSMGPU_FUSED_R dx, LSMGPU_FUSED_R dy,
    LSMGPU_FUSED_R dz, LSMGPU_FUSED_R dtau, int n_iter, int use_phi0_for_sgn, int bc) {
  if (!phi || !gb || !fb) {
    set_error(LSMGPU_ERR_ARGUMENT, "reinit: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  RunSpec rs{};
  rs.mode = REINIT;
  rs.n_steps = n_iter;
  rs.bc = bc;
  rs.use0 = (use_phi0_for_sgn == 1);
  rs.dt = dtau; rs.dx = dx; rs.dy = dy; rs.dz = dz;
  return run<LSMGPU_FUSED_R, LSMGPU_FUSED_EXACT>("lsmgpu_reinit_weno5_tvdrk3", phi, box6(gb), box6(fb),
                                                 nullptr, nullptr, nullptr, Box{}, rs);
}

int LSMGPU_CAT(lsmgpu_advect_weno5_tvdrk3_, LSMGPU_FUSED_SUFFIX)(
    LSMGPU_FUSED_R *phi, const int *gb, const int *fb, const LSMGPU_FUSED_R *vel_x,
    const LSMGPU_FUSED_R *vel_y, const LSMGPU_FUSED_R *vel_z, const int *vel_gb,
    const LSMGPU_FUSED_R *vel_const, LSMGPU_FUSED_R dx, LSMGPU_FUSED_R dy, LSMGPU_FUSED_R dz,
    LSMGPU_FUSED_R dt, int n_steps, int bc) {
  if (!phi || !gb || !fb || (!vel_x && !vel_const) || (vel_x && (!vel_y || !vel_z || !vel_gb))) {
    set_error(LSMGPU_ERR_ARGUMENT, "advect: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  RunSpec rs{};
  rs.mode = vel_x ? ADV_FIELD : ADV_CONST;
  rs.n_steps = n_steps;
  rs.bc = bc;
  rs.dt = dt; rs.dx = dx; rs.dy = dy; rs.dz = dz;
  if (!vel_x) {
    rs.vconst[0] = vel_const[0]; rs.vconst[1] = vel_const[1]; rs.vconst[2] = vel_const[2];
  }
  return run<LSMGPU_FUSED_R, LSMGPU_FUSED_EXACT>("lsmgpu_advect_weno5_tvdrk3", phi, box6(gb), box6(fb),
                                                 vel_x, vel_y, vel_z, vel_x ? box6(vel_gb) : Box{}, rs);
}

int LSMGPU_CAT(lsmgpu_mean_curvature_o2_, LSMGPU_FUSED_SUFFIX)(
    LSMGPU_FUSED_R *kappa, const int *kappa_gb, const LSMGPU_FUSED_R *phi, const int *phi_gb,
    LSMGPU_FUSED_R *grad_phi_mag, const int *fb, LSMGPU_FUSED_R dx, LSMGPU_FUSED_R dy,
    LSMGPU_FUSED_R dz) {
  if (!kappa || !kappa_gb || !phi || !phi_gb || !fb) {
    set_error(LSMGPU_ERR_ARGUMENT, "mean curvature: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  return lsmgpu::curv::run<LSMGPU_FUSED_R>("lsmgpu_mean_curvature_o2", kappa, box6(kappa_gb), phi,
                                           box6(phi_gb), grad_phi_mag, box6(fb), dx, dy, dz);
}

}  // extern "C"
