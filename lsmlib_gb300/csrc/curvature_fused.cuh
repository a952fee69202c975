// Fused second-order mean curvature: the LSMLIB sequence
//   lsm3dCentralGradOrder2 -> lsm3dGradientMagnitude -> lsm3dComputeMeanCurvatureOrder2
// (spatial_derivatives3d.f.in:3016-3077, :3586-3659; curvature3d.f.in:15-128)
// in one kernel: each cell reads its 19-point neighbourhood once and writes
// kappa (and, optionally, the gradient magnitude).  Included by the FP64
// parity unit and the FP32 unit.
#pragma once

#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"

namespace lsmgpu {
namespace curv {

template <class R>
struct CurvArgs {
  View<const R> phi;
  View<R> kappa;
  View<R> mag;      // p == nullptr: not written
  Box fb;
  R gx, gy, gz;     // 0.5/dx ...
  R fxx, fyy, fzz, fxy, fxz, fyz;
};

template <class R>
__global__ void k_mean_curvature(CurvArgs<R> a) {
  LSMGPU_CELL_INDEX(a.fb, i, j, k);
  const R *c = a.phi.p + a.phi.off(i, j, k);
  const long long sx = 1, sy = a.phi.s1, sz = a.phi.s2;
  // central gradient
  const R px = (c[sx] - c[-sx]) * a.gx;
  const R py = (c[sy] - c[-sy]) * a.gy;
  const R pz = (c[sz] - c[-sz]) * a.gz;
  // gradient magnitude with the reference's 1e-8 clamps
  const R tol = R(1.e-8);
  R x2 = px * px, y2 = py * py, z2 = pz * pz;
  if (x2 < tol) x2 = R(0);
  if (y2 < tol) y2 = R(0);
  if (z2 < tol) z2 = R(0);
  const R t = sqrt(x2 + y2 + z2);
  const R g = (t < tol) ? R(0) : t;
  if (a.mag.p) a.mag(i, j, k) = g;
  // second derivatives and curvature
  const R xx = (c[sx] - R(2.0) * c[0] + c[-sx]) * a.fxx;
  const R yy = (c[sy] - R(2.0) * c[0] + c[-sy]) * a.fyy;
  const R zz = (c[sz] - R(2.0) * c[0] + c[-sz]) * a.fzz;
  const R xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * a.fxy;
  const R xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * a.fxz;
  const R yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * a.fyz;
  const R den = g * g * g;
  R out;
  if (den < R(Consts<double>::zero_tol))
    out = R(0);
  else
    out = curv_numerator(xx, yy, zz, xy, xz, yz, px, py, pz) / den;
  a.kappa(i, j, k) = out;
}

template <class R>
int run(const char *name, R *kappa, const Box &kb, const R *phi, const Box &pb, R *mag, const Box &fb,
        R dx, R dy, R dz) {
  Call call(name);
  if (!pb.contains(fb, 1, 1, 1)) call.fail("phi ghost box must hold 1 ghost cell around the fill box");
  if (!kb.contains(fb, 0, 0, 0)) call.fail("kappa ghost box does not cover the fill box");
  if (!call.ok()) return LSMGPU_ERR_BOUNDS;
  if (fb.empty()) return LSMGPU_OK;
  CurvArgs<R> a{};
  a.phi = view((const R *)call.in(phi, pb.size()), pb);
  // kappa and |grad phi| are written on every fill-box cell and nowhere else
  a.kappa = view(call.out_region(kappa, kb, fb), kb);
  a.mag = mag ? view(call.out_region(mag, kb, fb), kb) : View<R>{};
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  a.fb = fb;
  a.gx = R(0.5) / dx; a.gy = R(0.5) / dy; a.gz = R(0.5) / dz;
  a.fxx = R(1.0) / dx / dx; a.fyy = R(1.0) / dy / dy; a.fzz = R(1.0) / dz / dz;
  a.fxy = R(0.25) / dx / dy; a.fxz = R(0.25) / dx / dz; a.fyz = R(0.25) / dy / dz;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_mean_curvature<R>, g.grid, g.block, 0, a);
  call.finish();
  return lsmgpu_get_last_error(nullptr, 0);
}

}  // namespace curv
}  // namespace lsmgpu
