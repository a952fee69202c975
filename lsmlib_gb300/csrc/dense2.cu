// Further drop-in dense entry points: central Hessian, averaged and upwinded
// gradients, the two LSE terms whose loops mix the fill box and the ghost box,
// and the ghost-cell boundary conditions.  FP64 parity form (compiled with
// -fmad=false).
#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

namespace lsmgpu {
namespace {

typedef double R;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)

template <class F>
__global__ void k_box(F f, Box b) {
  LSMGPU_CELL_INDEX(b, i, j, k);
  f(i, j, k);
}
template <class F>
void for_box(const Box &b, F f) {
  if (b.empty()) return;
  Grid3 g = cover(b);
  LSMGPU_LAUNCH(k_box<F>, g.grid, g.block, 0, f, b);
}

View<const R> vin(Call &c, const R *p, const Box &b) { return view((const R *)c.in(p, b.size()), b); }
View<R> vio(Call &c, R *p, const Box &b) { return view(c.inout(p, b.size()), b); }
// an output written on every cell of `fb` and nowhere else
View<R> vout(Call &c, R *p, const Box &b, const Box &fb) { return view(c.out_region(p, b, fb), b); }

// boundary conditions (boundary_conditions3d.f:46-639)
// BC_SIGNED_INNER: the 1D routine's form, the sign taken from the cell next
// to the edge (boundary_conditions1d.f:103-140) instead of the edge cell
enum { BC_LINEAR, BC_SIGNED, BC_COPY, BC_SIGNED_INNER };

void face_extrapolate(const char *name, R *phi, const Box &gb, const Box &fb, int face, int kind) {
  Call call(name);
  if (face < 0 || face > 5) return;  // the reference does nothing for other values
  const int axis = face / 2, upper = face % 2;
  const int edge = upper ? fb.hi[axis] : fb.lo[axis];
  const int inner = upper ? edge - 1 : edge + 1;
  if (edge < gb.lo[axis] || edge > gb.hi[axis] || (kind != BC_COPY && (inner < gb.lo[axis] || inner > gb.hi[axis])))
    call.fail("fill-box edge outside the ghost box");
  if (!call.ok()) return;
  View<R> P = vio(call, phi, gb);
  if (!call.ok()) return;
  Box plane = gb;  // one thread per line through the face
  plane.lo[axis] = plane.hi[axis] = 0;
  const int first = upper ? edge + 1 : gb.lo[axis];
  const int last = upper ? gb.hi[axis] : edge - 1;
  if (last < first) return;
  for_box(plane, [=] __device__(int i, int j, int k) {
    int c[3] = {i, j, k};
    c[axis] = edge;
    const R e = P(c[0], c[1], c[2]);
    R slope = R(0);
    if (kind != BC_COPY) {
      c[axis] = inner;
      const R nx = P(c[0], c[1], c[2]);
      slope = (kind == BC_LINEAR) ? e - nx : copysign(R(1.0), kind == BC_SIGNED_INNER ? nx : e) * fabs(e - nx);
    }
    for (int m = first; m <= last; m++) {
      c[axis] = m;
      if (kind == BC_COPY)
        P(c[0], c[1], c[2]) = e;
      else
        P(c[0], c[1], c[2]) = e + slope * (R)(upper ? m - edge : edge - m);
    }
  });
  call.finish();
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

// orthogonalization equation RHS (reinitialization3d.f.in:296-470); SGN3 =
// false gives the 2D routine's smoothing of sgn(psi) (see ortho_rhs)
template <bool SGN3>
void ortho_dense(const char *name, R *ortho_rhs, const Box &rb, const R *phi_x_plus, const R *phi_y_plus,
                 const R *phi_z_plus, const Box &pb, const R *phi_x_minus, const R *phi_y_minus,
                 const R *phi_z_minus, const Box &mb, const R *psi, const Box &sb, const R *psi_x_plus,
                 const R *psi_y_plus, const R *psi_z_plus, const Box &spb, const R *psi_x_minus,
                 const R *psi_y_minus, const R *psi_z_minus, const Box &smb, const Box &fb, R dx, R dy, R dz) {
  Call call(name);
  if (!rb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0) ||
      !sb.contains(fb, 0, 0, 0) || !spb.contains(fb, 0, 0, 0) || !smb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.out_region(ortho_rhs, rb, fb), rb);
  View<const R> XP = vin(call, phi_x_plus, pb), YP = vin(call, phi_y_plus, pb), ZP = vin(call, phi_z_plus, pb);
  View<const R> XM = vin(call, phi_x_minus, mb), YM = vin(call, phi_y_minus, mb), ZM = vin(call, phi_z_minus, mb);
  View<const R> S = vin(call, psi, sb);
  View<const R> SXP = vin(call, psi_x_plus, spb), SYP = vin(call, psi_y_plus, spb), SZP = vin(call, psi_z_plus, spb);
  View<const R> SXM = vin(call, psi_x_minus, smb), SYM = vin(call, psi_y_minus, smb),
                SZM = vin(call, psi_z_minus, smb);
  if (!call.ok()) return;
  R dx_sq = rmax(rmax(dx, dy), dz);
  dx_sq = dx_sq * dx_sq;
  for_box(fb, [=] __device__(int i, int j, int k) {
    const R psp[3] = {SXP(i, j, k), SYP(i, j, k), SZP(i, j, k)}, psm[3] = {SXM(i, j, k), SYM(i, j, k), SZM(i, j, k)};
    const R pp[3] = {XP(i, j, k), YP(i, j, k), ZP(i, j, k)}, pm[3] = {XM(i, j, k), YM(i, j, k), ZM(i, j, k)};
    O(i, j, k) = lsmgpu::ortho_rhs<R, SGN3>(S(i, j, k), psp, psm, pp, pm, dx_sq);
  });
  call.finish();
}

// distance estimate for the subcell fix (reinitialization3d.f.in:477-575;
// HALF = false: the 2D routine's form, see subcell_distance); distance0 and
// phi0 share phi0's ghost box
template <bool HALF>
void subcell_distance_dense(const char *name, R *distance0, const R *phi0, const Box &zb, const Box &fb, R dx,
                            R dy, R dz) {
  Call call(name);
  if (!zb.contains(fb, 1, 1, 1)) call.fail("phi0 ghost box must hold 1 ghost cell around the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> D = view(call.out_region(distance0, zb, fb), zb);
  View<const R> P0 = vin(call, phi0, zb);
  if (!call.ok()) return;
  const R flag = R(-1000.0) * rmax(rmax(dx, dy), dz);
  for_box(fb, [=] __device__(int i, int j, int k) {
    const long long st[3] = {1, P0.s1, P0.s2};
    D(i, j, k) = subcell_distance<R, HALF>(P0.p + P0.off(i, j, k), st, flag);
  });
  call.finish();
}

// rhs -= u . grad(phi) + Vn |grad phi| with the combined Godunov selection
// (level_set_evolution3d.f.in:532-718).  FILL_BOX = false: the 3D routine's
// loop (k, j from the fill box to the ghost box end, i over the ghost box,
// :620) and its branches (the advection part alone where |Vn| or |grad phi|^2
// is below zero_tol); FILL_BOX = true: the 2D routine's form
// (level_set_evolution2d.f.in:399-520): the fill box, and nothing added where
// |Vn| < zero_tol
template <bool FILL_BOX>
void external_normal(const char *name, R *lse_rhs, const Box &rb, const R *phi_x_plus, const R *phi_y_plus,
                     const R *phi_z_plus, const Box &pb, const R *phi_x_minus, const R *phi_y_minus,
                     const R *phi_z_minus, const Box &mb, const R *vel_n, const R *vel_x, const R *vel_y,
                     const R *vel_z, const Box &vb, const Box &fb) {
  Call call(name);
  Box loop = fb;
  if (!FILL_BOX) {
    loop = rb;
    loop.lo[1] = fb.lo[1];
    loop.lo[2] = fb.lo[2];
  }
  if (!rb.contains(loop, 0, 0, 0) || !pb.contains(loop, 0, 0, 0) || !mb.contains(loop, 0, 0, 0) ||
      !vb.contains(loop, 0, 0, 0))
    call.fail("ghost box does not cover the loop range");
  if (!call.ok() || loop.empty()) return;
  View<R> O = vio(call, lse_rhs, rb);
  View<const R> XP = vin(call, phi_x_plus, pb), YP = vin(call, phi_y_plus, pb), ZP = vin(call, phi_z_plus, pb);
  View<const R> XM = vin(call, phi_x_minus, mb), YM = vin(call, phi_y_minus, mb), ZM = vin(call, phi_z_minus, mb);
  View<const R> VN = vin(call, vel_n, vb), VX = vin(call, vel_x, vb), VY = vin(call, vel_y, vb), VZ = vin(call, vel_z, vb);
  if (!call.ok()) return;
  for_box(loop, [=] __device__(int i, int j, int k) {
    const R w = VN(i, j, k), ux = VX(i, j, k), uy = VY(i, j, k), uz = VZ(i, j, k);
    const R gx = ext_pick<R>(ux, w, XP(i, j, k), XM(i, j, k));
    const R gy = ext_pick<R>(uy, w, YP(i, j, k), YM(i, j, k));
    const R gz = ext_pick<R>(uz, w, ZP(i, j, k), ZM(i, j, k));
    const R n2 = gx * gx + gy * gy + gz * gz;
    if (FILL_BOX) {
      if (fabs(w) >= Consts<R>::zero_tol) O(i, j, k) = O(i, j, k) - ux * gx - uy * gy - uz * gz - w * sqrt(n2);
    } else if (fabs(w) >= Consts<R>::zero_tol && n2 >= Consts<R>::zero_tol) {
      O(i, j, k) = O(i, j, k) - ux * gx - uy * gy - uz * gz - w * sqrt(n2);
    } else {
      O(i, j, k) = O(i, j, k) - ux * gx - uy * gy - uz * gz;
    }
  });
  call.finish();
}

extern "C" {

void lsm3dcentralhessian_(R *phi_xx, R *phi_xy, R *phi_xz, R *phi_yy, R *phi_yz, R *phi_zz, BOXARG(h),
                          const R *phi, BOXARG(g), BOXARG(fb), const R *dx, const R *dy, const R *dz) {
  Call call("lsm3dcentralhessian_");
  Box hb = BOXOF(h), gb = BOXOF(g), fb = BOXOF(fb);
  if (!gb.contains(fb, 1, 1, 1) || !hb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> XX = vout(call, phi_xx, hb, fb), XY = vout(call, phi_xy, hb, fb), XZ = vout(call, phi_xz, hb, fb),
          YY = vout(call, phi_yy, hb, fb), YZ = vout(call, phi_yz, hb, fb), ZZ = vout(call, phi_zz, hb, fb);
  View<const R> F = vin(call, phi, gb);
  if (!call.ok()) return;
  const R ddx = *dx, ddy = *dy, ddz = *dz;
  for_box(fb, [=] __device__(int i, int j, int k) {
    const R *c = F.p + F.off(i, j, k);
    const long long sx = 1, sy = F.s1, sz = F.s2;
    XX(i, j, k) = (c[sx] - 2 * c[0] + c[-sx]) / (ddx * ddx);
    XY(i, j, k) = R(0.25) * (c[sx + sy] - c[-sx + sy] - c[sx - sy] + c[-sx - sy]) / (ddx * ddy);
    XZ(i, j, k) = R(0.25) * (c[sx + sz] - c[-sx + sz] - c[sx - sz] + c[-sx - sz]) / (ddx * ddz);
    YY(i, j, k) = (c[sy] - 2 * c[0] + c[-sy]) / (ddy * ddy);
    YZ(i, j, k) = R(0.25) * (c[sy + sz] - c[-sy + sz] - c[sy - sz] + c[-sy - sz]) / (ddy * ddz);
    ZZ(i, j, k) = (c[sz] - 2 * c[0] + c[-sz]) / (ddz * ddz);
  });
  call.finish();
}

void lsm3daveragegradphi_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi_x_plus, const R *phi_y_plus,
                          const R *phi_z_plus, BOXARG(p), const R *phi_x_minus, const R *phi_y_minus,
                          const R *phi_z_minus, BOXARG(m), BOXARG(fb)) {
  Call call("lsm3daveragegradphi_");
  Box gb = BOXOF(g), pb = BOXOF(p), mb = BOXOF(m), fb = BOXOF(fb);
  if (!gb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> X = vout(call, phi_x, gb, fb), Y = vout(call, phi_y, gb, fb), Z = vout(call, phi_z, gb, fb);
  View<const R> XP = vin(call, phi_x_plus, pb), YP = vin(call, phi_y_plus, pb), ZP = vin(call, phi_z_plus, pb);
  View<const R> XM = vin(call, phi_x_minus, mb), YM = vin(call, phi_y_minus, mb), ZM = vin(call, phi_z_minus, mb);
  if (!call.ok()) return;
  for_box(fb, [=] __device__(int i, int j, int k) {
    X(i, j, k) = R(0.5) * (XP(i, j, k) + XM(i, j, k));
    Y(i, j, k) = R(0.5) * (YP(i, j, k) + YM(i, j, k));
    Z(i, j, k) = R(0.5) * (ZP(i, j, k) + ZM(i, j, k));
  });
  call.finish();
}

void lsm3dphiupwindgradf_(R *F_x, R *F_y, R *F_z, BOXARG(g), const R *F_x_plus, const R *F_y_plus,
                          const R *F_z_plus, BOXARG(p), const R *F_x_minus, const R *F_y_minus,
                          const R *F_z_minus, BOXARG(m), const R *phi, BOXARG(f), BOXARG(fb)) {
  Call call("lsm3dphiupwindgradf_");
  Box gb = BOXOF(g), pb = BOXOF(p), mb = BOXOF(m), phb = BOXOF(f), fb = BOXOF(fb);
  if (!gb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0) ||
      !phb.contains(fb, 1, 1, 1))
    call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> O[3] = {vio(call, F_x, gb), vio(call, F_y, gb), vio(call, F_z, gb)};
  View<const R> PL[3] = {vin(call, F_x_plus, pb), vin(call, F_y_plus, pb), vin(call, F_z_plus, pb)};
  View<const R> MI[3] = {vin(call, F_x_minus, mb), vin(call, F_y_minus, mb), vin(call, F_z_minus, mb)};
  View<const R> PH = vin(call, phi, phb);
  if (!call.ok()) return;
  View<R> O0 = O[0], O1 = O[1], O2 = O[2];
  View<const R> P0 = PL[0], P1 = PL[1], P2 = PL[2], M0 = MI[0], M1 = MI[1], M2 = MI[2];
  // spatial_derivatives3d.f.in:3355-3459
  for_box(fb, [=] __device__(int i, int j, int k) {
    const R *c = PH.p + PH.off(i, j, k);
    const R pc = c[0];
    const long long s[3] = {1, PH.s1, PH.s2};
    for (int d = 0; d < 3; d++) {
      const View<R> &o = d == 0 ? O0 : (d == 1 ? O1 : O2);
      const View<const R> &pl = d == 0 ? P0 : (d == 1 ? P1 : P2);
      const View<const R> &mi = d == 0 ? M0 : (d == 1 ? M1 : M2);
      const R nm = c[-s[d]], np = c[s[d]];
      if (pc > R(0)) {
        if (nm <= pc) o(i, j, k) = (np < nm) ? pl(i, j, k) : mi(i, j, k);
        else if (np <= pc) o(i, j, k) = pl(i, j, k);
        else o(i, j, k) = R(0);
      } else if (pc < R(0)) {
        if (nm >= pc) o(i, j, k) = (np > nm) ? pl(i, j, k) : mi(i, j, k);
        else if (np >= pc) o(i, j, k) = pl(i, j, k);
        else o(i, j, k) = R(0);
      }
    }
  });
  call.finish();
}

// level_set_evolution3d.f.in:514-521: k from klo_fb to khi_gb, j from jlo_fb to
// jhi_gb, i over the whole ghost box of the rhs
void lsm3daddconstprecomputedcurvtermtolserhs_(R *lse_rhs, BOXARG(r), const R *kappa, BOXARG(k),
                                               const R *grad_phi_mag, BOXARG(g), const R *b, BOXARG(fb)) {
  Call call("lsm3daddconstprecomputedcurvtermtolserhs_");
  Box rb = BOXOF(r), kb = BOXOF(k), gb = BOXOF(g), fb = BOXOF(fb);
  Box loop = rb;
  loop.lo[1] = fb.lo[1];
  loop.lo[2] = fb.lo[2];
  if (!kb.contains(loop, 0, 0, 0) || !gb.contains(loop, 0, 0, 0)) call.fail("kappa / grad_phi_mag ghost box does not cover the loop range");
  if (!call.ok() || loop.empty()) return;
  View<R> O = vio(call, lse_rhs, rb);
  View<const R> K = vin(call, kappa, kb), G = vin(call, grad_phi_mag, gb);
  if (!call.ok()) return;
  const R bb = *b;
  for_box(loop, [=] __device__(int i, int j, int k) { O(i, j, k) = O(i, j, k) + bb * K(i, j, k) * G(i, j, k); });
  call.finish();
}

#define EXT_ARGS                                                                                          \
  R *lse_rhs, BOXARG(r), const R *phi_x_plus, const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),        \
      const R *phi_x_minus, const R *phi_y_minus, const R *phi_z_minus, BOXARG(m), const R *vel_n,         \
      const R *vel_x, const R *vel_y, const R *vel_z, BOXARG(v), BOXARG(fb)
#define EXT_PASS                                                                                          \
  lse_rhs, BOXOF(r), phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, \
      BOXOF(m), vel_n, vel_x, vel_y, vel_z, BOXOF(v), BOXOF(fb)

void lsm3daddexternalandnormalveltermtolserhs_(EXT_ARGS) {
  external_normal<false>("lsm3daddexternalandnormalveltermtolserhs_", EXT_PASS);
}
void lsmgpu_external_normal_vel_term_fill_box(EXT_ARGS) {
  external_normal<true>("lsmgpu_external_normal_vel_term_fill_box", EXT_PASS);
}

#define BCARGS R *phi, BOXARG(g), BOXARG(fb), const int *bdry_location_idx
void lsm3dlinearextrapolation_(BCARGS) {
  face_extrapolate("lsm3dlinearextrapolation_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_LINEAR);
}
void lsm3dsignedlinearextrapolation_(BCARGS) {
  face_extrapolate("lsm3dsignedlinearextrapolation_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_SIGNED);
}
void lsmgpu_signed_linear_extrapolation_inner_sign(BCARGS) {
  face_extrapolate("lsmgpu_signed_linear_extrapolation_inner_sign", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx,
                   BC_SIGNED_INNER);
}
void lsm3dcopyextrapolation_(BCARGS) {
  face_extrapolate("lsm3dcopyextrapolation_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_COPY);
}
void lsm3dhomogeneousneumanneno1_(BCARGS) {
  face_extrapolate("lsm3dhomogeneousneumanneno1_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_COPY);
}
void lsm3dhomogeneousneumanneno2_(BCARGS) {
  face_extrapolate("lsm3dhomogeneousneumanneno2_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_COPY);
}
void lsm3dhomogeneousneumanneno3_(BCARGS) {
  face_extrapolate("lsm3dhomogeneousneumanneno3_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_COPY);
}
void lsm3dhomogeneousneumannweno5_(BCARGS) {
  face_extrapolate("lsm3dhomogeneousneumannweno5_", phi, BOXOF(g), BOXOF(fb), *bdry_location_idx, BC_COPY);
}

// n-th undivided difference along dir (spatial_derivatives3d.f.in:49-176):
// odd n face-centred, Dn(c) = Dm(c) - Dm(c - 1) over the fill box grown by one
// cell along dir; even n, Dn(c) = -(Dm(c) - Dm(c + 1)) over the fill box;
// every other cell of Dn's ghost box holds 1e10.  The dense derivative
// routines form these differences in registers; this is the routine itself.
void lsm3dcomputedn_(R *Dn, BOXARG(d), const R *Dn_minus_one, BOXARG(m), const int *ilo_fb, const int *ihi_fb,
                     const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb, const int *n,
                     const int *dir) {
  Call call("lsm3dcomputedn_");
  if (*dir < 1 || *dir > 3) call.fail("dir must be 1, 2 or 3");
  if (!call.ok()) return;
  const Box db = BOXOF(d), mb = BOXOF(m);
  const int ax = *dir - 1;
  const bool odd = (*n % 2) != 0;
  Box cb = mkbox(ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb);  // cells with a difference
  if (odd) cb.hi[ax] += 1;
  // Dm(c) and Dm(c - 1) (odd) or Dm(c + 1) (even) along dir
  Box need = cb;
  if (odd) need.lo[ax] -= 1; else need.hi[ax] += 1;
  if (!db.contains(cb, 0, 0, 0) || !mb.contains(need, 0, 0, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || db.empty()) return;
  View<R> D = view(call.inout(Dn, db.size()), db);
  View<const R> Mv = vin(call, Dn_minus_one, mb);
  if (!call.ok()) return;
  const int o0 = ax == 0 ? (odd ? 1 : -1) : 0, o1 = ax == 1 ? (odd ? 1 : -1) : 0, o2 = ax == 2 ? (odd ? 1 : -1) : 0;
  const R sgn = odd ? R(1) : R(-1);
  for_box(db, [=] __device__(int i, int j, int k) {
    if (inbox(cb, i, j, k))
      D(i, j, k) = sgn * (Mv(i, j, k) - Mv(i - o0, j - o1, k - o2));
    else
      D(i, j, k) = R(1.0e10);
  });
  call.finish();
}

// First-order delta function from sign changes along each axis
// (calculus_toolbox3d.f.in:15-130).  The reference's z terms use norm_phi_x
// and 1/dx (:103-115); kept, so the results are the reference's.
void lsm3ddeltafunctionorder1_(const R *phi, R *delta, BOXARG(g), const R *norm_phi_x, const R *norm_phi_y,
                               const R *norm_phi_z, BOXARG(n), const int *ilo_fb, const int *ihi_fb,
                               const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb,
                               const R *dx, const R *dy, const R *dz) {
  Call call("lsm3ddeltafunctionorder1_");
  const Box gb = BOXOF(g), nb = BOXOF(n), fb = mkbox(ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb);
  if (!gb.contains(fb, 1, 1, 1) || !nb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<const R> P = vin(call, phi, gb);
  View<R> D = vio(call, delta, gb);
  View<const R> NX = vin(call, norm_phi_x, nb), NY = vin(call, norm_phi_y, nb);
  (void)norm_phi_z;
  if (!call.ok()) return;
  const R ox = R(1.0) / *dx, oy = R(1.0) / *dy;
  for_box(fb, [=] __device__(int i, int j, int k) {
    const R c = P(i, j, k);
    auto side = [&](R nbr, R n, R o) {
      if (nbr * c <= R(0)) return nbr * n * o / (nbr - c);
      return R(0);
    };
    const R nx = NX(i, j, k), ny = NY(i, j, k);
    const R xp = side(P(i + 1, j, k), nx, ox), xm = side(P(i - 1, j, k), nx, ox);
    const R yp = side(P(i, j + 1, k), ny, oy), ym = side(P(i, j - 1, k), ny, oy);
    const R zp = side(P(i, j, k + 1), nx, ox), zm = side(P(i, j, k - 1), nx, ox);
    D(i, j, k) = fabs(xp) + fabs(xm) + fabs(yp) + fabs(ym) + fabs(zp) + fabs(zm);
  });
  call.finish();
}

#define ORTHO_ARGS                                                                                       \
  R *ortho_rhs, BOXARG(r), const R *phi_x_plus, const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),     \
      const R *phi_x_minus, const R *phi_y_minus, const R *phi_z_minus, BOXARG(m), const R *psi, BOXARG(s), \
      const R *psi_x_plus, const R *psi_y_plus, const R *psi_z_plus, BOXARG(sp), const R *psi_x_minus,    \
      const R *psi_y_minus, const R *psi_z_minus, BOXARG(sm), BOXARG(fb), const R *dx, const R *dy,       \
      const R *dz
#define ORTHO_PASS                                                                                       \
  ortho_rhs, BOXOF(r), phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, \
      BOXOF(m), psi, BOXOF(s), psi_x_plus, psi_y_plus, psi_z_plus, BOXOF(sp), psi_x_minus, psi_y_minus,    \
      psi_z_minus, BOXOF(sm), BOXOF(fb), *dx, *dy, *dz

void lsm3dcomputeorthogonalizationeqnrhs_(ORTHO_ARGS) {
  ortho_dense<true>("lsm3dcomputeorthogonalizationeqnrhs_", ORTHO_PASS);
}
void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing(ORTHO_ARGS) {
  ortho_dense<false>("lsmgpu_orthogonalization_rhs_unit_sgn_smoothing", ORTHO_PASS);
}

void lsm3dcomputedistanceforsubcellfix_(R *distance0, const R *phi0, BOXARG(z), BOXARG(fb), const R *dx,
                                        const R *dy, const R *dz) {
  subcell_distance_dense<true>("lsm3dcomputedistanceforsubcellfix_", distance0, phi0, BOXOF(z), BOXOF(fb), *dx,
                               *dy, *dz);
}
void lsmgpu_distance_for_subcell_fix_full_central(R *distance0, const R *phi0, BOXARG(z), BOXARG(fb),
                                                  const R *dx, const R *dy, const R *dz) {
  subcell_distance_dense<false>("lsmgpu_distance_for_subcell_fix_full_central", distance0, phi0, BOXOF(z),
                                BOXOF(fb), *dx, *dy, *dz);
}

// first-order reinitialization RHS with the subcell fix
// (reinitialization3d.f.in:586-757)
void lsm3dcomputereinitializationeqnrhssubcellfixorder1_(R *reinit_rhs, BOXARG(r), const R *phi, BOXARG(f),
                                                         const R *phi0, const R *distance0, BOXARG(z),
                                                         const R *phi_x_plus, const R *phi_y_plus,
                                                         const R *phi_z_plus, BOXARG(p), const R *phi_x_minus,
                                                         const R *phi_y_minus, const R *phi_z_minus, BOXARG(m),
                                                         BOXARG(fb), const R *dx, const R *dy, const R *dz) {
  Call call("lsm3dcomputereinitializationeqnrhssubcellfixorder1_");
  const Box rb = BOXOF(r), phb = BOXOF(f), zb = BOXOF(z), pb = BOXOF(p), mb = BOXOF(m), fb = BOXOF(fb);
  if (!rb.contains(fb, 0, 0, 0) || !phb.contains(fb, 0, 0, 0) || !zb.contains(fb, 0, 0, 0) ||
      !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.out_region(reinit_rhs, rb, fb), rb);
  View<const R> PH = vin(call, phi, phb), P0 = vin(call, phi0, zb), D0 = vin(call, distance0, zb);
  View<const R> XP = vin(call, phi_x_plus, pb), YP = vin(call, phi_y_plus, pb), ZP = vin(call, phi_z_plus, pb);
  View<const R> XM = vin(call, phi_x_minus, mb), YM = vin(call, phi_y_minus, mb), ZM = vin(call, phi_z_minus, mb);
  if (!call.ok()) return;
  const R max_dx = rmax(rmax(*dx, *dy), *dz);
  const R flag = R(-1000.0) * max_dx;
  for_box(fb, [=] __device__(int i, int j, int k) {
    const R gp[3] = {XP(i, j, k), YP(i, j, k), ZP(i, j, k)}, gm[3] = {XM(i, j, k), YM(i, j, k), ZM(i, j, k)};
    O(i, j, k) = subcell_rhs<R>(PH(i, j, k), P0(i, j, k), D0(i, j, k), gp, gm, flag, max_dx);
  });
  call.finish();
}

}  // extern "C"
