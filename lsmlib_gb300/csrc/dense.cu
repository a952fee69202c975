// Drop-in dense-grid entry points: LSMLIB's 3D toolbox routines with LSMLIB's
// symbol names and argument lists (see include/lsmgpu_toolbox3d.h for the
// reference citation of each).
//
// Each routine is one kernel with one thread per fill-box cell.  The
// reference's two-sweep structure (undivided differences into scratch D1/D2/D3,
// then a pass that reads them) collapses into a single pass: the differences
// a cell needs are formed in registers from phi, with the same subtractions,
// so the outputs are bit-identical and no scratch array is read or written.
//
// This translation unit is compiled with -fmad=false (FP64 parity form).
#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

namespace lsmgpu {
namespace {

typedef double R;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)
#define FBARGS const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb
#define FBOX mkbox(ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb)

enum Scheme { ENO1 = 1, ENO2 = 2, ENO3 = 3, WENO5 = 5 };

template <int S> struct SchemeInfo;
template <> struct SchemeInfo<ENO1> { static constexpr int reach = 1, order = 1; };
template <> struct SchemeInfo<ENO2> { static constexpr int reach = 2, order = 2; };
template <> struct SchemeInfo<ENO3> { static constexpr int reach = 3, order = 3; };
template <> struct SchemeInfo<WENO5> { static constexpr int reach = 3, order = 1; };

template <int S>
__device__ __forceinline__ void side_values(const Diffs<R> &d, R inv, R &plus, R &minus) {
  if (S == ENO1) { plus = eno1_plus(d, inv); minus = eno1_minus(d, inv); }
  if (S == ENO2) { plus = eno2_plus(d, inv); minus = eno2_minus(d, inv); }
  if (S == ENO3) { plus = eno3_plus(d, inv); minus = eno3_minus(d, inv); }
  if (S == WENO5) { plus = weno5_plus(d, inv); minus = weno5_minus(d, inv); }
}
template <int S>
__device__ __forceinline__ R side_value(const Diffs<R> &d, R inv, bool use_minus) {
  if (S == ENO1) return use_minus ? eno1_minus(d, inv) : eno1_plus(d, inv);
  if (S == ENO2) return use_minus ? eno2_minus(d, inv) : eno2_plus(d, inv);
  if (S == ENO3) return use_minus ? eno3_minus(d, inv) : eno3_plus(d, inv);
  return use_minus ? weno5_minus(d, inv) : weno5_plus(d, inv);
}

// load phi(c-3..c+3) along stride s (only the reach the scheme needs)
template <int REACH>
__device__ __forceinline__ void load_line(R a[7], const R *c, long long s) {
#pragma unroll
  for (int m = 0; m < 7; m++) {
    const int o = m - 3;
    a[m] = (o >= -REACH && o <= REACH) ? __ldg(c + o * s) : R(0);
  }
}

struct Out3 { View<R> x, y, z; };

template <int S>
__global__ void k_hj_pm(Out3 plus, Out3 minus, View<const R> phi, Box fb, R ix, R iy, R iz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  const R inv[3] = {ix, iy, iz};
  const long long st[3] = {1, phi.s1, phi.s2};
  R pv[3], mv[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    R a[7];
    load_line<SchemeInfo<S>::reach>(a, c, st[d]);
    Diffs<R> df;
    make_diffs<R, SchemeInfo<S>::order>(df, a);
    side_values<S>(df, inv[d], pv[d], mv[d]);
  }
  plus.x(i, j, k) = pv[0]; plus.y(i, j, k) = pv[1]; plus.z(i, j, k) = pv[2];
  minus.x(i, j, k) = mv[0]; minus.y(i, j, k) = mv[1]; minus.z(i, j, k) = mv[2];
}

template <int S>
__global__ void k_hj_upwind(Out3 g, View<const R> phi, View<const R> vx, View<const R> vy,
                            View<const R> vz, Box fb, R ix, R iy, R iz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  const R inv[3] = {ix, iy, iz};
  const long long st[3] = {1, phi.s1, phi.s2};
  const R vel[3] = {vx(i, j, k), vy(i, j, k), vz(i, j, k)};
  R out[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    // spatial_derivatives3d.f.in:2756-2812: |v| < zero_tol gives 0, v > 0
    // takes the backward (minus) stencil, otherwise the forward one
    if (fabs(vel[d]) < Consts<R>::zero_tol) {
      out[d] = R(0);
    } else {
      R a[7];
      load_line<SchemeInfo<S>::reach>(a, c, st[d]);
      Diffs<R> df;
      make_diffs<R, SchemeInfo<S>::order>(df, a);
      out[d] = side_value<S>(df, inv[d], vel[d] > R(0));
    }
  }
  g.x(i, j, k) = out[0]; g.y(i, j, k) = out[1]; g.z(i, j, k) = out[2];
}

template <int S>
void hj_pm(const char *name, R *pxp, R *pyp, R *pzp, const Box &pb, R *pxm, R *pym, R *pzm,
           const Box &mb, const R *phi, const Box &phb, const Box &fb, R dx, R dy, R dz) {
  Call call(name);
  const int r = SchemeInfo<S>::reach;
  if (!phb.contains(fb, r, r, r)) call.fail("phi ghost box does not cover the fill box plus the stencil");
  if (!pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0)) call.fail("output ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  // outputs written on every fill-box cell and nowhere else (host arrays:
  // no copy in, the fill box copied back)
  Out3 P{view(call.out_region(pxp, pb, fb), pb), view(call.out_region(pyp, pb, fb), pb),
         view(call.out_region(pzp, pb, fb), pb)};
  Out3 M{view(call.out_region(pxm, mb, fb), mb), view(call.out_region(pym, mb, fb), mb),
         view(call.out_region(pzm, mb, fb), mb)};
  View<const R> ph = view((const R *)call.in(phi, phb.size()), phb);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_hj_pm<S>, g.grid, g.block, 0, P, M, ph, fb, R(1.0) / dx, R(1.0) / dy, R(1.0) / dz);
  call.finish();
}

template <int S>
void hj_upwind(const char *name, R *px, R *py, R *pz, const Box &gb, const R *phi, const Box &phb,
               const R *vx, const R *vy, const R *vz, const Box &vb, const Box &fb, R dx, R dy, R dz) {
  Call call(name);
  const int r = SchemeInfo<S>::reach;
  if (!phb.contains(fb, r, r, r)) call.fail("phi ghost box does not cover the fill box plus the stencil");
  if (!gb.contains(fb, 0, 0, 0) || !vb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  const long long nv = vb.size();
  Out3 G{view(call.out_region(px, gb, fb), gb), view(call.out_region(py, gb, fb), gb),
         view(call.out_region(pz, gb, fb), gb)};
  View<const R> ph = view((const R *)call.in(phi, phb.size()), phb);
  View<const R> VX = view((const R *)call.in(vx, nv), vb);
  View<const R> VY = view((const R *)call.in(vy, nv), vb);
  View<const R> VZ = view((const R *)call.in(vz, nv), vb);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_hj_upwind<S>, g.grid, g.block, 0, G, ph, VX, VY, VZ, fb, R(1.0) / dx, R(1.0) / dy,
                R(1.0) / dz);
  call.finish();
}

// ---- central differences ---------------------------------------------------
__global__ void k_central2(Out3 g, View<const R> phi, Box fb, R fx, R fy, R fz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  g.x(i, j, k) = (c[1] - c[-1]) * fx;
  g.y(i, j, k) = (c[phi.s1] - c[-phi.s1]) * fy;
  g.z(i, j, k) = (c[phi.s2] - c[-phi.s2]) * fz;
}

__global__ void k_central4(Out3 g, View<const R> phi, Box fb, R fx, R fy, R fz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  const R e = R(8.0);
  const long long s[3] = {1, phi.s1, phi.s2};
  const R f[3] = {fx, fy, fz};
  R o[3];
#pragma unroll
  for (int d = 0; d < 3; d++)
    o[d] = (-c[2 * s[d]] + e * c[s[d]] + c[-2 * s[d]] - e * c[-s[d]]) * f[d];
  g.x(i, j, k) = o[0]; g.y(i, j, k) = o[1]; g.z(i, j, k) = o[2];
}

__global__ void k_laplacian2(View<R> lap, View<const R> phi, Box fb, R ix, R iy, R iz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  const long long sy = phi.s1, sz = phi.s2;
  lap(i, j, k) = ix * (c[1] - R(2.0) * c[0] + c[-1]) + iy * (c[sy] - R(2.0) * c[0] + c[-sy]) +
                 iz * (c[sz] - R(2.0) * c[0] + c[-sz]);
}

__global__ void k_gradmag(View<const R> px, View<const R> py, View<const R> pz, View<R> mag, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R tol = R(1.e-8);
  R x = px(i, j, k), y = py(i, j, k), z = pz(i, j, k);
  R x2 = x * x, y2 = y * y, z2 = z * z;
  if (x2 < tol) x2 = R(0);
  if (y2 < tol) y2 = R(0);
  if (z2 < tol) z2 = R(0);
  const R t = sqrt(x2 + y2 + z2);
  mag(i, j, k) = (t < tol) ? R(0) : t;
}

// ---- RK stages ---------------------------------------------------------------
// kind 0: u1 = u + dt*L (tvd_runge_kutta3d.f:78)
// kind 1: un = 0.5*(u + u1 + dt*L) (:240-241)
// kind 2: u2 = 0.75*u + 0.25*(u1 + dt*L) (:403-404)
// kind 3: un = u/3 + 2/3*(u2 + dt*L) (:490-492)
template <int KIND>
__global__ void k_rk(View<R> out, View<const R> a, View<const R> u, View<const R> rhs, Box fb, R dt) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R L = rhs(i, j, k);
  R v;
  if (KIND == 0) v = u(i, j, k) + dt * L;
  if (KIND == 1) v = R(0.5) * (u(i, j, k) + a(i, j, k) + dt * L);
  if (KIND == 2) v = R(0.75) * u(i, j, k) + R(0.25) * (a(i, j, k) + dt * L);
  if (KIND == 3) v = R(1.0 / 3.0) * u(i, j, k) + R(2.0 / 3.0) * (a(i, j, k) + dt * L);
  out(i, j, k) = v;
}

template <int KIND>
void rk(const char *name, R *out, const Box &ob, const R *a, const Box &ab, const R *u, const Box &ub,
        const R *rhs, const Box &rb, const Box &fb, R dt) {
  Call call(name);
  if (!ob.contains(fb, 0, 0, 0) || !ub.contains(fb, 0, 0, 0) || !rb.contains(fb, 0, 0, 0) ||
      (KIND != 0 && !ab.contains(fb, 0, 0, 0)))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.out_region(out, ob, fb), ob);
  View<const R> A = (KIND != 0) ? view((const R *)call.in(a, ab.size()), ab) : View<const R>{};
  View<const R> U = view((const R *)call.in(u, ub.size()), ub);
  View<const R> L = view((const R *)call.in(rhs, rb.size()), rb);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_rk<KIND>, g.grid, g.block, 0, O, A, U, L, fb, dt);
  call.finish();
}

// ---- level set RHS terms ------------------------------------------------------
__global__ void k_fill(View<R> a, Box b, R v) {
  LSMGPU_CELL_INDEX(b, i, j, k);
  a(i, j, k) = v;
}

__global__ void k_add_advection(View<R> rhs, View<const R> px, View<const R> py, View<const R> pz,
                                View<const R> vx, View<const R> vy, View<const R> vz, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  rhs(i, j, k) = rhs(i, j, k) - (vx(i, j, k) * px(i, j, k) + vy(i, j, k) * py(i, j, k) +
                                 vz(i, j, k) * pz(i, j, k));
}

// vn field (const_vn == false) or constant (const_vn == true)
__global__ void k_add_normal(View<R> rhs, View<const R> pxp, View<const R> pyp, View<const R> pzp,
                             View<const R> pxm, View<const R> pym, View<const R> pzm,
                             View<const R> vn, bool const_vn, R vn_const, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R w = const_vn ? vn_const : vn(i, j, k);
  if (!(fabs(w) >= Consts<R>::zero_tol)) return;
  const R p[3] = {pxp(i, j, k), pyp(i, j, k), pzp(i, j, k)};
  const R m[3] = {pxm(i, j, k), pym(i, j, k), pzm(i, j, k)};
  rhs(i, j, k) = rhs(i, j, k) - w * sqrt(godunov_normal_sq(w > R(0), p, m));
}

__global__ void k_add_const_curv(View<R> rhs, View<const R> px, View<const R> py, View<const R> pz,
                                 View<const R> pxx, View<const R> pxy, View<const R> pxz,
                                 View<const R> pyy, View<const R> pyz, View<const R> pzz, R b, Box fb) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R x = px(i, j, k), y = py(i, j, k), z = pz(i, j, k);
  const R m2 = x * x + y * y + z * z;
  R curv;
  if (m2 < Consts<R>::zero_tol) {
    curv = R(0);
  } else {
    curv = curv_numerator(pxx(i, j, k), pyy(i, j, k), pzz(i, j, k), pxy(i, j, k), pxz(i, j, k),
                          pyz(i, j, k), x, y, z);
    curv = curv / m2;
  }
  rhs(i, j, k) = rhs(i, j, k) + b * curv;
}

// ---- reinitialization --------------------------------------------------------
__global__ void k_reinit_rhs(View<R> rhs, View<const R> phi, View<const R> phi0, View<const R> pxp,
                             View<const R> pyp, View<const R> pzp, View<const R> pxm,
                             View<const R> pym, View<const R> pzm, Box fb, R dx_sq, bool use0) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R pc = use0 ? phi0(i, j, k) : phi(i, j, k);
  const R gp[3] = {pxp(i, j, k), pyp(i, j, k), pzp(i, j, k)};
  const R gm[3] = {pxm(i, j, k), pym(i, j, k), pzm(i, j, k)};
  rhs(i, j, k) = reinit_rhs(pc, gp, gm, dx_sq, use0);
}

// ---- mean curvature -----------------------------------------------------------
__global__ void k_mean_curv2(View<R> kappa, View<const R> phi, View<const R> px, View<const R> py,
                             View<const R> pz, View<const R> mag, Box fb, R fxx, R fyy, R fzz, R fxy,
                             R fxz, R fyz) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const R *c = phi.p + phi.off(i, j, k);
  const long long sx = 1, sy = phi.s1, sz = phi.s2;
  const R xx = (c[sx] - R(2.0) * c[0] + c[-sx]) * fxx;
  const R yy = (c[sy] - R(2.0) * c[0] + c[-sy]) * fyy;
  const R zz = (c[sz] - R(2.0) * c[0] + c[-sz]) * fzz;
  const R xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * fxy;
  const R xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * fxz;
  const R yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * fyz;
  const R g = mag(i, j, k);
  const R den = g * g * g;
  R out;
  if (den < Consts<R>::zero_tol)
    out = R(0);
  else
    out = curv_numerator(xx, yy, zz, xy, xz, yz, px(i, j, k), py(i, j, k), pz(i, j, k)) / den;
  kappa(i, j, k) = out;
}

// Gaussian curvature (order 2, 4) and mean curvature (order 4): the order-2
// form differences phi, the order-4 forms take phi_xy, phi_yz, phi_zx from the
// first derivatives (curvature3d.f.in:136-508)
template <int K>
__global__ void k_curv_variant(View<R> kappa, View<const R> phi, View<const R> px, View<const R> py,
                               View<const R> pz, View<const R> mag, Box fb, CurvFactors<R> F) {
  LSMGPU_CELL_INDEX(fb, i, j, k);
  const long long o = px.off(i, j, k);
  kappa(i, j, k) = curvature_variant<R, K>(phi.p + phi.off(i, j, k), phi.s1, phi.s2, px.p + o, py.p + o, pz.p + o,
                                           px.s1, px.s2, mag(i, j, k), F);
}

// ---- max reductions ---------------------------------------------------------------
// An order-preserving map of doubles onto unsigned 64-bit keys, so a max over
// cells becomes atomicMax on keys.  Max is exact and order independent, so the
// result equals the reference's serial scan.
__device__ __forceinline__ unsigned long long okey(R v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ R okey_inv(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}

__device__ __forceinline__ void block_max_commit(R v, unsigned long long *key) {
  for (int o = 16; o > 0; o >>= 1) v = rmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __shared__ R part[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nt = blockDim.x * blockDim.y * blockDim.z;
  if ((t & 31) == 0) part[t >> 5] = v;
  __syncthreads();
  if (t < 32) {
    R w = (t < (nt + 31) / 32) ? part[t] : R(-1.0e308);
    for (int o = 16; o > 0; o >>= 1) w = rmax(w, __shfl_xor_sync(0xffffffffu, w, o));
    if (t == 0) atomicMax(key, okey(w));
  }
}

// mode 0: advection (math_utils3d.f.in:309-315)
// mode 1: normal velocity field (:421-438), mode 2: constant normal velocity (:537-556)
// mode 3: max |f1 - f2| (:56-71)
// The control-volume variants (math_utils3d.f.in:852-1416) take a cell only
// when control_vol > 0 (cv_sgn > 0) or control_vol < 0 (cv_sgn < 0); cv_sgn 0
// takes every cell.  Max-norm seeds with the (ilo, jlo, klo) corner whatever
// its control volume (:908-909), so mode 3 always takes that cell.
struct RedArgs {
  View<const R> a, b, c;         // vel_x,y,z | (unused) | f1,f2
  View<const R> pxp, pyp, pzp, pxm, pym, pzm;
  View<const R> vn;
  View<const R> cv;
  int cv_sgn;
  R vn_const, ix, iy, iz, max_dx_sq;
};

template <int MODE>
__global__ void k_reduce_max(RedArgs A, Box ib, unsigned long long *key) {
  const int i = ib.lo[0] + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = ib.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = ib.lo[2] + blockIdx.z * blockDim.z + threadIdx.z;
  R v = R(-1.0e308);
  bool take = i <= ib.hi[0] && j <= ib.hi[1] && k <= ib.hi[2];
  if (take && A.cv_sgn != 0 && !(MODE == 3 && i == ib.lo[0] && j == ib.lo[1] && k == ib.lo[2])) {
    const R c = A.cv(i, j, k);
    take = A.cv_sgn > 0 ? c > R(0) : c < R(0);
  }
  if (take) {
    if (MODE == 0) {
      v = fabs(A.a(i, j, k)) * A.ix + fabs(A.b(i, j, k)) * A.iy + fabs(A.c(i, j, k)) * A.iz;
    } else if (MODE == 3) {
      v = fabs(A.a(i, j, k) - A.b(i, j, k));
    } else {
      const R avn = (MODE == 2) ? fabs(A.vn_const) : fabs(A.vn(i, j, k));
      const R cx = rmax(fabs(A.pxp(i, j, k)), fabs(A.pxm(i, j, k)));
      const R cy = rmax(fabs(A.pyp(i, j, k)), fabs(A.pym(i, j, k)));
      const R cz = rmax(fabs(A.pzp(i, j, k)), fabs(A.pzm(i, j, k)));
      const R ng = sqrt(cx * cx + cy * cy + cz * cz + A.max_dx_sq);
      v = avn / ng * (cx * A.ix + cy * A.iy + cz * A.iz);
    }
  }
  block_max_commit(v, key);
}

// final scalar: mode 0-2 give dt = cfl/(max + tiny) with the running max
// starting at -1 (math_utils3d.f.in:297, :323); mode 3 gives the max itself
__global__ void k_finish_scalar(const unsigned long long *key, R *out, int mode, R cfl, R init) {
  R m = okey_inv(*key);
  if (m < init) m = init;
  if (mode == 3)
    *out = m;
  else
    *out = cfl / (m + Consts<R>::tiny);
}

__global__ void k_set_key(unsigned long long *key, R v) { *key = okey(v); }

template <int MODE>
void reduce_max(Call &call, RedArgs &A, const Box &ib, R *out, R cfl, R init) {
  unsigned long long *key = call.temp<unsigned long long>(1);
  R *dout = call.scalar_out(out);
  if (!call.ok()) return;
  LSMGPU_LAUNCH(k_set_key, 1, 1, 0, key, init);
  if (!ib.empty()) {
    Grid3 g = cover(ib);
    LSMGPU_LAUNCH(k_reduce_max<MODE>, g.grid, g.block, 0, A, ib, key);
  }
  LSMGPU_LAUNCH(k_finish_scalar, 1, 1, 0, key, dout, MODE, cfl, init);
  call.finish();
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

// ============================================================================
// C entry points
// ============================================================================
template <int K>
void curv_variant(const char *name, R *kappa, const Box &kb, const R *phi, const Box &phb, const R *phi_x,
                  const R *phi_y, const R *phi_z, const R *grad_phi_mag, const Box &gb, const Box &fb, R dxv, R dyv,
                  R dzv) {
  Call call(name);
  const int rp = (K == CURV_GAUSS2) ? 1 : 2, rg = (K == CURV_GAUSS2) ? 0 : 2;
  if (!kb.contains(fb, 0, 0, 0) || !gb.contains(fb, rg, rg, rg) || !phb.contains(fb, rp, rp, rp))
    call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> KA = view(call.out_region(kappa, kb, fb), kb);
  View<const R> PH = view((const R *)call.in(phi, phb.size()), phb);
  const long long ng = gb.size();
  View<const R> X = view((const R *)call.in(phi_x, ng), gb), Y = view((const R *)call.in(phi_y, ng), gb),
                Z = view((const R *)call.in(phi_z, ng), gb), G = view((const R *)call.in(grad_phi_mag, ng), gb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_curv_variant<K>, g3.grid, g3.block, 0, KA, PH, X, Y, Z, G, fb,
                curvature_factors<R, K>(dxv, dyv, dzv));
  call.finish();
}

extern "C" void lsm3dcomputedn_(R *Dn, const int *, const int *, const int *, const int *, const int *,
                                const int *, const R *Dn_minus_one, const int *, const int *, const int *,
                                const int *, const int *, const int *, const int *ilo_fb, const int *ihi_fb,
                                const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb,
                                const int *n, const int *dir);

// Exact side-effect mode: the lsm3dComputeDn calls a derivative routine of
// LSMLIB makes, in its order (per direction x, y, z: D1 from phi, then D2 from
// D1, D3 from D2, over the fill box grown along that direction by `grow`;
// spatial_derivatives3d.f.in:281-341 ENO1, :487-635 ENO2, :795-1066 ENO3,
// :1266-1511 WENO5, and the same in the upwind routines), so the scratch
// arrays end as LSMLIB leaves them.  Runs after the derivative call (each
// replayed call is an entry point of its own) and only if it succeeded; a 2D
// or 1D routine running on the 3D one replays its own directions only.
static void replay_scratch(int scheme, const R *phi, const Box &fphi, R *const D[3], const Box db[3],
                           const Box &fb) {
  if (!exact_side_effects() || lsmgpu_get_last_error(nullptr, 0) != LSMGPU_OK) return;
  const int orders = scheme == ENO2 ? 2 : (scheme == ENO3 ? 3 : 1);
  const int grow[3] = {scheme == ENO1 ? 0 : (scheme == ENO2 ? 1 : 2), scheme == ENO2 ? 1 : 2, 1};
  for (int ax = 0; ax < g_lift_dims; ax++)
    for (int n = 1; n <= orders; n++) {
      Box cb = fb;
      cb.lo[ax] -= grow[n - 1];
      cb.hi[ax] += grow[n - 1];
      const Box &ob = db[n - 1], &sb = n == 1 ? fphi : db[n - 2];
      const R *src = n == 1 ? phi : D[n - 2];
      const int dir = ax + 1;
      lsm3dcomputedn_(D[n - 1], &ob.lo[0], &ob.hi[0], &ob.lo[1], &ob.hi[1], &ob.lo[2], &ob.hi[2], src, &sb.lo[0],
                      &sb.hi[0], &sb.lo[1], &sb.hi[1], &sb.lo[2], &sb.hi[2], &cb.lo[0], &cb.hi[0], &cb.lo[1],
                      &cb.hi[1], &cb.lo[2], &cb.hi[2], &n, &dir);
      if (lsmgpu_get_last_error(nullptr, 0) != LSMGPU_OK) return;
    }
}

extern "C" {

#define PM_PARAMS                                                                        \
  R *phi_x_plus, R *phi_y_plus, R *phi_z_plus, BOXARG(p), R *phi_x_minus, R *phi_y_minus, \
      R *phi_z_minus, BOXARG(m), const R *phi, BOXARG(f)
#define SCR(n) R *n, BOXARG(n)
#define DXP const R *dx, const R *dy, const R *dz

void lsm3dhjeno1_(PM_PARAMS, SCR(D1), FBARGS, DXP) {
  hj_pm<ENO1>("lsm3dhjeno1_", phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus,
              phi_z_minus, BOXOF(m), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, nullptr, nullptr};
    const Box db[3] = {BOXOF(D1), Box{}, Box{}};
    replay_scratch(ENO1, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dhjeno2_(PM_PARAMS, SCR(D1), SCR(D2), FBARGS, DXP) {
  hj_pm<ENO2>("lsm3dhjeno2_", phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus,
              phi_z_minus, BOXOF(m), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, D2, nullptr};
    const Box db[3] = {BOXOF(D1), BOXOF(D2), Box{}};
    replay_scratch(ENO2, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dhjeno3_(PM_PARAMS, SCR(D1), SCR(D2), SCR(D3), FBARGS, DXP) {
  hj_pm<ENO3>("lsm3dhjeno3_", phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus,
              phi_z_minus, BOXOF(m), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, D2, D3};
    const Box db[3] = {BOXOF(D1), BOXOF(D2), BOXOF(D3)};
    replay_scratch(ENO3, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dhjweno5_(PM_PARAMS, SCR(D1), FBARGS, DXP) {
  hj_pm<WENO5>("lsm3dhjweno5_", phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus,
               phi_y_minus, phi_z_minus, BOXOF(m), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, nullptr, nullptr};
    const Box db[3] = {BOXOF(D1), Box{}, Box{}};
    replay_scratch(WENO5, phi, BOXOF(f), D, db, FBOX);
  }
}

#define UP_PARAMS                                                                     \
  R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f), const R *vel_x, \
      const R *vel_y, const R *vel_z, BOXARG(v)

void lsm3dupwindhjeno1_(UP_PARAMS, SCR(D1), FBARGS, DXP) {
  hj_upwind<ENO1>("lsm3dupwindhjeno1_", phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), vel_x, vel_y,
                  vel_z, BOXOF(v), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, nullptr, nullptr};
    const Box db[3] = {BOXOF(D1), Box{}, Box{}};
    replay_scratch(ENO1, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dupwindhjeno2_(UP_PARAMS, SCR(D1), SCR(D2), FBARGS, DXP) {
  hj_upwind<ENO2>("lsm3dupwindhjeno2_", phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), vel_x, vel_y,
                  vel_z, BOXOF(v), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, D2, nullptr};
    const Box db[3] = {BOXOF(D1), BOXOF(D2), Box{}};
    replay_scratch(ENO2, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dupwindhjeno3_(UP_PARAMS, SCR(D1), SCR(D2), SCR(D3), FBARGS, DXP) {
  hj_upwind<ENO3>("lsm3dupwindhjeno3_", phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), vel_x, vel_y,
                  vel_z, BOXOF(v), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, D2, D3};
    const Box db[3] = {BOXOF(D1), BOXOF(D2), BOXOF(D3)};
    replay_scratch(ENO3, phi, BOXOF(f), D, db, FBOX);
  }
}
void lsm3dupwindhjweno5_(UP_PARAMS, SCR(D1), FBARGS, DXP) {
  hj_upwind<WENO5>("lsm3dupwindhjweno5_", phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), vel_x, vel_y,
                   vel_z, BOXOF(v), FBOX, *dx, *dy, *dz);
  {
    R *const D[3] = {D1, nullptr, nullptr};
    const Box db[3] = {BOXOF(D1), Box{}, Box{}};
    replay_scratch(WENO5, phi, BOXOF(f), D, db, FBOX);
  }
}

static void central(const char *name, int order, R *px, R *py, R *pz, const Box &gb, const R *phi,
                    const Box &fb_phi, const Box &fb, R dx, R dy, R dz) {
  Call call(name);
  const int r = order == 2 ? 1 : 2;
  if (!fb_phi.contains(fb, r, r, r)) call.fail("phi ghost box does not cover the fill box plus the stencil");
  if (!gb.contains(fb, 0, 0, 0)) call.fail("output ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  Out3 G{view(call.out_region(px, gb, fb), gb), view(call.out_region(py, gb, fb), gb),
         view(call.out_region(pz, gb, fb), gb)};
  View<const R> ph = view((const R *)call.in(phi, fb_phi.size()), fb_phi);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  if (order == 2) {
    LSMGPU_LAUNCH(k_central2, g.grid, g.block, 0, G, ph, fb, R(0.5) / dx, R(0.5) / dy, R(0.5) / dz);
  } else {
    const R c = R(0.0833333333333333333333);
    LSMGPU_LAUNCH(k_central4, g.grid, g.block, 0, G, ph, fb, c / dx, c / dy, c / dz);
  }
  call.finish();
}

void lsm3dcentralgradorder2_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f),
                             FBARGS, DXP) {
  central("lsm3dcentralgradorder2_", 2, phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
}
void lsm3dcentralgradorder4_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f),
                             FBARGS, DXP) {
  central("lsm3dcentralgradorder4_", 4, phi_x, phi_y, phi_z, BOXOF(g), phi, BOXOF(f), FBOX, *dx, *dy, *dz);
}

void lsm3dlaplacianorder2_(R *lap, BOXARG(l), const R *phi, BOXARG(f), FBARGS, DXP) {
  Call call("lsm3dlaplacianorder2_");
  Box lb = BOXOF(l), phb = BOXOF(f), fb = FBOX;
  if (!phb.contains(fb, 1, 1, 1) || !lb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> L = view(call.out_region(lap, lb, fb), lb);
  View<const R> ph = view((const R *)call.in(phi, phb.size()), phb);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_laplacian2, g.grid, g.block, 0, L, ph, fb, R(1.0) / *dx / *dx, R(1.0) / *dy / *dy,
                R(1.0) / *dz / *dz);
  call.finish();
}

void lsm3dgradientmagnitude_(const R *phi_x, const R *phi_y, const R *phi_z, R *grad_phi_mag,
                             BOXARG(g), const int *ilo_fb, const int *ihi_fb, const int *jlo_fb,
                             const int *jhi_fb, const int *klo_fb, const int *khi_fb) {
  Call call("lsm3dgradientmagnitude_");
  Box gb = BOXOF(g), fb = FBOX;
  if (!gb.contains(fb, 0, 0, 0)) call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  const long long n = gb.size();
  View<const R> X = view((const R *)call.in(phi_x, n), gb), Y = view((const R *)call.in(phi_y, n), gb),
                Z = view((const R *)call.in(phi_z, n), gb);
  View<R> M = view(call.out_region(grad_phi_mag, gb, fb), gb);
  if (!call.ok()) return;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_gradmag, g.grid, g.block, 0, X, Y, Z, M, fb);
  call.finish();
}

// RK stages -------------------------------------------------------------------
void lsm3drk1step_(R *u_next, BOXARG(a), const R *u_cur, BOXARG(b), const R *rhs, BOXARG(c), FBARGS,
                   const R *dt) {
  rk<0>("lsm3drk1step_", u_next, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), FBOX, *dt);
}
void lsm3dtvdrk2stage1_(R *u_stage1, BOXARG(a), const R *u_cur, BOXARG(b), const R *rhs, BOXARG(c),
                        FBARGS, const R *dt) {
  rk<0>("lsm3dtvdrk2stage1_", u_stage1, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), FBOX, *dt);
}
void lsm3dtvdrk3stage1_(R *u_stage1, BOXARG(a), const R *u_cur, BOXARG(b), const R *rhs, BOXARG(c),
                        FBARGS, const R *dt) {
  rk<0>("lsm3dtvdrk3stage1_", u_stage1, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), FBOX, *dt);
}
void lsm3dtvdrk2stage2_(R *u_next, BOXARG(a), const R *u_stage1, BOXARG(b), const R *u_cur, BOXARG(c),
                        const R *rhs, BOXARG(d), FBARGS, const R *dt) {
  rk<1>("lsm3dtvdrk2stage2_", u_next, BOXOF(a), u_stage1, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), FBOX, *dt);
}
void lsm3dtvdrk3stage2_(R *u_stage2, BOXARG(a), const R *u_stage1, BOXARG(b), const R *u_cur,
                        BOXARG(c), const R *rhs, BOXARG(d), FBARGS, const R *dt) {
  rk<2>("lsm3dtvdrk3stage2_", u_stage2, BOXOF(a), u_stage1, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), FBOX, *dt);
}
void lsm3dtvdrk3stage3_(R *u_next, BOXARG(a), const R *u_stage2, BOXARG(b), const R *u_cur, BOXARG(c),
                        const R *rhs, BOXARG(d), FBARGS, const R *dt) {
  rk<3>("lsm3dtvdrk3stage3_", u_next, BOXOF(a), u_stage2, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), FBOX, *dt);
}

// level set equation RHS -----------------------------------------------------------
void lsm3dzerooutlevelseteqnrhs_(R *lse_rhs, BOXARG(r)) {
  Call call("lsm3dzerooutlevelseteqnrhs_");
  Box rb = BOXOF(r);
  if (rb.empty()) return;
  View<R> O = view(call.out(lse_rhs, rb.size()), rb);
  if (!call.ok()) return;
  Grid3 g = cover(rb);
  LSMGPU_LAUNCH(k_fill, g.grid, g.block, 0, O, rb, R(0));
  call.finish();
}

void lsm3daddadvectiontermtolserhs_(R *lse_rhs, BOXARG(r), const R *phi_x, const R *phi_y,
                                    const R *phi_z, BOXARG(g), const R *vel_x, const R *vel_y,
                                    const R *vel_z, BOXARG(v), FBARGS) {
  Call call("lsm3daddadvectiontermtolserhs_");
  Box rb = BOXOF(r), gb = BOXOF(g), vb = BOXOF(v), fb = FBOX;
  if (!rb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0) || !vb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.inout(lse_rhs, rb.size()), rb);
  const long long ng = gb.size(), nv = vb.size();
  View<const R> X = view((const R *)call.in(phi_x, ng), gb), Y = view((const R *)call.in(phi_y, ng), gb),
                Z = view((const R *)call.in(phi_z, ng), gb);
  View<const R> VX = view((const R *)call.in(vel_x, nv), vb), VY = view((const R *)call.in(vel_y, nv), vb),
                VZ = view((const R *)call.in(vel_z, nv), vb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_add_advection, g3.grid, g3.block, 0, O, X, Y, Z, VX, VY, VZ, fb);
  call.finish();
}

static void add_normal(const char *name, R *rhs, const Box &rb, const R *pxp, const R *pyp,
                       const R *pzp, const Box &pb, const R *pxm, const R *pym, const R *pzm,
                       const Box &mb, const R *vn, const Box &vb, bool const_vn, R vn_const,
                       const Box &fb) {
  Call call(name);
  if (!rb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0) ||
      (!const_vn && !vb.contains(fb, 0, 0, 0)))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  if (const_vn && !(fabs(vn_const) >= Consts<R>::zero_tol)) return;  // f.in:308
  View<R> O = view(call.inout(rhs, rb.size()), rb);
  const long long np = pb.size(), nm = mb.size();
  View<const R> XP = view((const R *)call.in(pxp, np), pb), YP = view((const R *)call.in(pyp, np), pb),
                ZP = view((const R *)call.in(pzp, np), pb);
  View<const R> XM = view((const R *)call.in(pxm, nm), mb), YM = view((const R *)call.in(pym, nm), mb),
                ZM = view((const R *)call.in(pzm, nm), mb);
  View<const R> V = const_vn ? View<const R>{} : view((const R *)call.in(vn, vb.size()), vb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_add_normal, g3.grid, g3.block, 0, O, XP, YP, ZP, XM, YM, ZM, V, const_vn, vn_const, fb);
  call.finish();
}

void lsm3daddnormalveltermtolserhs_(R *lse_rhs, BOXARG(r), const R *phi_x_plus, const R *phi_y_plus,
                                    const R *phi_z_plus, BOXARG(p), const R *phi_x_minus,
                                    const R *phi_y_minus, const R *phi_z_minus, BOXARG(m),
                                    const R *vel_n, BOXARG(v), FBARGS) {
  add_normal("lsm3daddnormalveltermtolserhs_", lse_rhs, BOXOF(r), phi_x_plus, phi_y_plus, phi_z_plus,
             BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), vel_n, BOXOF(v), false, R(0), FBOX);
}

void lsm3daddconstnormalveltermtolserhs_(R *lse_rhs, BOXARG(r), const R *phi_x_plus,
                                         const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                         const R *phi_x_minus, const R *phi_y_minus,
                                         const R *phi_z_minus, BOXARG(m), const R *vel_n, FBARGS) {
  add_normal("lsm3daddconstnormalveltermtolserhs_", lse_rhs, BOXOF(r), phi_x_plus, phi_y_plus,
             phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), nullptr, Box{},
             true, *vel_n, FBOX);
}

void lsm3daddconstcurvtermtolserhs_(R *lse_rhs, BOXARG(r), const R *phi_x, const R *phi_y,
                                    const R *phi_z, BOXARG(g), const R *phi_xx, const R *phi_xy,
                                    const R *phi_xz, const R *phi_yy, const R *phi_yz,
                                    const R *phi_zz, BOXARG(h), const R *b, FBARGS) {
  Call call("lsm3daddconstcurvtermtolserhs_");
  Box rb = BOXOF(r), gb = BOXOF(g), hb = BOXOF(h), fb = FBOX;
  if (!rb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0) || !hb.contains(fb, 0, 0, 0))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.inout(lse_rhs, rb.size()), rb);
  const long long ng = gb.size(), nh = hb.size();
  View<const R> X = view((const R *)call.in(phi_x, ng), gb), Y = view((const R *)call.in(phi_y, ng), gb),
                Z = view((const R *)call.in(phi_z, ng), gb);
  View<const R> XX = view((const R *)call.in(phi_xx, nh), hb), XY = view((const R *)call.in(phi_xy, nh), hb),
                XZ = view((const R *)call.in(phi_xz, nh), hb), YY = view((const R *)call.in(phi_yy, nh), hb),
                YZ = view((const R *)call.in(phi_yz, nh), hb), ZZ = view((const R *)call.in(phi_zz, nh), hb);
  if (!call.ok()) return;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_add_const_curv, g3.grid, g3.block, 0, O, X, Y, Z, XX, XY, XZ, YY, YZ, ZZ, *b, fb);
  call.finish();
}

void lsm3dcomputereinitializationeqnrhs_(R *reinit_rhs, BOXARG(r), const R *phi, BOXARG(f),
                                         const R *phi0, BOXARG(z), const R *phi_x_plus,
                                         const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                         const R *phi_x_minus, const R *phi_y_minus,
                                         const R *phi_z_minus, BOXARG(m), FBARGS, DXP,
                                         const int *use_phi0_for_sgn) {
  Call call("lsm3dcomputereinitializationeqnrhs_");
  Box rb = BOXOF(r), phb = BOXOF(f), zb = BOXOF(z), pb = BOXOF(p), mb = BOXOF(m), fb = FBOX;
  const bool use0 = (*use_phi0_for_sgn == 1);
  if (!rb.contains(fb, 0, 0, 0) || !pb.contains(fb, 0, 0, 0) || !mb.contains(fb, 0, 0, 0) ||
      (use0 ? !zb.contains(fb, 0, 0, 0) : !phb.contains(fb, 0, 0, 0)))
    call.fail("ghost box does not cover the fill box");
  if (!call.ok() || fb.empty()) return;
  View<R> O = view(call.out_region(reinit_rhs, rb, fb), rb);
  View<const R> PH = use0 ? View<const R>{} : view((const R *)call.in(phi, phb.size()), phb);
  View<const R> P0 = use0 ? view((const R *)call.in(phi0, zb.size()), zb) : View<const R>{};
  const long long np = pb.size(), nm = mb.size();
  View<const R> XP = view((const R *)call.in(phi_x_plus, np), pb), YP = view((const R *)call.in(phi_y_plus, np), pb),
                ZP = view((const R *)call.in(phi_z_plus, np), pb);
  View<const R> XM = view((const R *)call.in(phi_x_minus, nm), mb), YM = view((const R *)call.in(phi_y_minus, nm), mb),
                ZM = view((const R *)call.in(phi_z_minus, nm), mb);
  if (!call.ok()) return;
  R dx_sq = rmax(rmax(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_reinit_rhs, g3.grid, g3.block, 0, O, PH, P0, XP, YP, ZP, XM, YM, ZM, fb, dx_sq, use0);
  call.finish();
}

void lsm3dcomputemeancurvatureorder2_(R *kappa, BOXARG(k), const R *phi, BOXARG(f), const R *phi_x,
                                      const R *phi_y, const R *phi_z, const R *grad_phi_mag,
                                      BOXARG(g), BOXARG(kf), DXP) {
  Call call("lsm3dcomputemeancurvatureorder2_");
  Box kb = BOXOF(k), phb = BOXOF(f), gb = BOXOF(g), fb = BOXOF(kf);
  if (!kb.contains(fb, 0, 0, 0) || !gb.contains(fb, 0, 0, 0) || !phb.contains(fb, 1, 1, 1))
    call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> K = view(call.out_region(kappa, kb, fb), kb);
  View<const R> PH = view((const R *)call.in(phi, phb.size()), phb);
  const long long ng = gb.size();
  View<const R> X = view((const R *)call.in(phi_x, ng), gb), Y = view((const R *)call.in(phi_y, ng), gb),
                Z = view((const R *)call.in(phi_z, ng), gb), G = view((const R *)call.in(grad_phi_mag, ng), gb);
  if (!call.ok()) return;
  const R dxv = *dx, dyv = *dy, dzv = *dz;
  Grid3 g3 = cover(fb);
  LSMGPU_LAUNCH(k_mean_curv2, g3.grid, g3.block, 0, K, PH, X, Y, Z, G, fb, R(1.0) / dxv / dxv,
                R(1.0) / dyv / dyv, R(1.0) / dzv / dzv, R(0.25) / dxv / dyv, R(0.25) / dxv / dzv,
                R(0.25) / dyv / dzv);
  call.finish();
}

#define CURV_ARGS                                                                                         \
  R *kappa, BOXARG(k), const R *phi, BOXARG(f), const R *phi_x, const R *phi_y, const R *phi_z,         \
      const R *grad_phi_mag, BOXARG(g), BOXARG(kf), DXP
#define CURV_PASS kappa, BOXOF(k), phi, BOXOF(f), phi_x, phi_y, phi_z, grad_phi_mag, BOXOF(g), BOXOF(kf), *dx, *dy, *dz

void lsm3dcomputegaussiancurvatureorder2_(CURV_ARGS) {
  curv_variant<CURV_GAUSS2>("lsm3dcomputegaussiancurvatureorder2_", CURV_PASS);
}
void lsm3dcomputemeancurvatureorder4_(CURV_ARGS) {
  curv_variant<CURV_MEAN4>("lsm3dcomputemeancurvatureorder4_", CURV_PASS);
}
void lsm3dcomputegaussiancurvatureorder4_(CURV_ARGS) {
  curv_variant<CURV_GAUSS4>("lsm3dcomputegaussiancurvatureorder4_", CURV_PASS);
}

// reductions ---------------------------------------------------------------------------
#define IBARGS const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib
#define IBOX mkbox(ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib)

void lsm3dmaxnormdiff_(R *max_norm_diff, const R *field1, BOXARG(a), const R *field2, BOXARG(b), IBARGS) {
  Call call("lsm3dmaxnormdiff_");
  Box ab = BOXOF(a), bb = BOXOF(b), ib = IBOX;
  // the reference reads the (ilo_ib, jlo_ib, klo_ib) corner even for an
  // empty box (math_utils3d.f.in:56)
  Box corner = ib;
  corner.hi[0] = corner.lo[0]; corner.hi[1] = corner.lo[1]; corner.hi[2] = corner.lo[2];
  if (!ab.contains(corner, 0, 0, 0) || !bb.contains(corner, 0, 0, 0) || !ab.contains(ib, 0, 0, 0) ||
      !bb.contains(ib, 0, 0, 0))
    call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  RedArgs A{};
  A.a = view((const R *)call.in(field1, ab.size()), ab);
  A.b = view((const R *)call.in(field2, bb.size()), bb);
  if (!call.ok()) return;
  // seed with the corner value, then max over the box
  Box seedbox = ib.empty() ? corner : ib;
  reduce_max<3>(call, A, seedbox, max_norm_diff, R(0), R(-1.0e308));
}

void lsm3dcomputestableadvectiondt_(R *dt, const R *vel_x, const R *vel_y, const R *vel_z, BOXARG(v),
                                    IBARGS, DXP, const R *cfl_number) {
  Call call("lsm3dcomputestableadvectiondt_");
  Box vb = BOXOF(v), ib = IBOX;
  if (!vb.contains(ib, 0, 0, 0)) call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  RedArgs A{};
  const long long n = vb.size();
  A.a = view((const R *)call.in(vel_x, n), vb);
  A.b = view((const R *)call.in(vel_y, n), vb);
  A.c = view((const R *)call.in(vel_z, n), vb);
  A.ix = R(1.0) / *dx; A.iy = R(1.0) / *dy; A.iz = R(1.0) / *dz;
  if (!call.ok()) return;
  reduce_max<0>(call, A, ib, dt, *cfl_number, R(-1.0));
}

static void normal_dt(const char *name, bool const_vn, R *dt, const R *vn, const Box &vb, R vn_const,
                      const R *pxp, const R *pyp, const R *pzp, const Box &pb, const R *pxm,
                      const R *pym, const R *pzm, const Box &mb, const Box &ib, R dx, R dy, R dz,
                      R cfl, const R *cv = nullptr, const Box &cb = Box{}, int cv_sgn = 0) {
  Call call(name);
  if (!pb.contains(ib, 0, 0, 0) || !mb.contains(ib, 0, 0, 0) || (!const_vn && !vb.contains(ib, 0, 0, 0)) ||
      (cv_sgn != 0 && !cb.contains(ib, 0, 0, 0)))
    call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  RedArgs A{};
  if (cv_sgn != 0) {
    A.cv = view((const R *)call.in(cv, cb.size()), cb);
    A.cv_sgn = cv_sgn;
  }
  const long long np = pb.size(), nm = mb.size();
  A.pxp = view((const R *)call.in(pxp, np), pb); A.pyp = view((const R *)call.in(pyp, np), pb);
  A.pzp = view((const R *)call.in(pzp, np), pb);
  A.pxm = view((const R *)call.in(pxm, nm), mb); A.pym = view((const R *)call.in(pym, nm), mb);
  A.pzm = view((const R *)call.in(pzm, nm), mb);
  if (!const_vn) A.vn = view((const R *)call.in(vn, vb.size()), vb);
  A.vn_const = vn_const;
  A.ix = R(1.0) / dx; A.iy = R(1.0) / dy; A.iz = R(1.0) / dz;
  const R mx = rmax(rmax(dx, dy), dz);
  A.max_dx_sq = mx * mx;
  if (!call.ok()) return;
  if (const_vn)
    reduce_max<2>(call, A, ib, dt, cfl, R(-1.0));
  else
    reduce_max<1>(call, A, ib, dt, cfl, R(-1.0));
}

void lsm3dcomputestablenormalveldt_(R *dt, const R *vel_n, BOXARG(v), const R *phi_x_plus,
                                    const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                    const R *phi_x_minus, const R *phi_y_minus, const R *phi_z_minus,
                                    BOXARG(m), IBARGS, DXP, const R *cfl_number) {
  normal_dt("lsm3dcomputestablenormalveldt_", false, dt, vel_n, BOXOF(v), R(0), phi_x_plus, phi_y_plus,
            phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), IBOX, *dx, *dy, *dz,
            *cfl_number);
}

void lsm3dcomputestableconstnormalveldt_(R *dt, const R *vel_n, const R *phi_x_plus,
                                         const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                         const R *phi_x_minus, const R *phi_y_minus,
                                         const R *phi_z_minus, BOXARG(m), IBARGS, DXP,
                                         const R *cfl_number) {
  normal_dt("lsm3dcomputestableconstnormalveldt_", true, dt, nullptr, Box{}, *vel_n, phi_x_plus,
            phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), IBOX, *dx,
            *dy, *dz, *cfl_number);
}


// ---- control-volume variants (math_utils3d.f.in:852-1416) ------------------------
#define CVARGS const R *control_vol, BOXARG(c), const int *control_vol_sgn
#define CVSGN (*control_vol_sgn > 0 ? 1 : -1)

void lsm3dmaxnormdiffcontrolvolume_(R *max_norm_diff, const R *field1, BOXARG(a), const R *field2, BOXARG(b),
                                    CVARGS, IBARGS) {
  Call call("lsm3dmaxnormdiffcontrolvolume_");
  Box ab = BOXOF(a), bb = BOXOF(b), cb = BOXOF(c), ib = IBOX;
  Box corner = ib;
  corner.hi[0] = corner.lo[0]; corner.hi[1] = corner.lo[1]; corner.hi[2] = corner.lo[2];
  if (!ab.contains(corner, 0, 0, 0) || !bb.contains(corner, 0, 0, 0) || !ab.contains(ib, 0, 0, 0) ||
      !bb.contains(ib, 0, 0, 0) || !cb.contains(ib, 0, 0, 0))
    call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  RedArgs A{};
  A.a = view((const R *)call.in(field1, ab.size()), ab);
  A.b = view((const R *)call.in(field2, bb.size()), bb);
  A.cv = view((const R *)call.in(control_vol, cb.size()), cb);
  A.cv_sgn = CVSGN;
  if (!call.ok()) return;
  reduce_max<3>(call, A, ib.empty() ? corner : ib, max_norm_diff, R(0), R(-1.0e308));
}

void lsm3dcomputestableadvectiondtcontrolvolume_(R *dt, const R *vel_x, const R *vel_y, const R *vel_z,
                                                 BOXARG(v), CVARGS, IBARGS, DXP, const R *cfl_number) {
  Call call("lsm3dcomputestableadvectiondtcontrolvolume_");
  Box vb = BOXOF(v), cb = BOXOF(c), ib = IBOX;
  if (!vb.contains(ib, 0, 0, 0) || !cb.contains(ib, 0, 0, 0)) call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  RedArgs A{};
  const long long n = vb.size();
  A.a = view((const R *)call.in(vel_x, n), vb);
  A.b = view((const R *)call.in(vel_y, n), vb);
  A.c = view((const R *)call.in(vel_z, n), vb);
  A.cv = view((const R *)call.in(control_vol, cb.size()), cb);
  A.cv_sgn = CVSGN;
  A.ix = R(1.0) / *dx; A.iy = R(1.0) / *dy; A.iz = R(1.0) / *dz;
  if (!call.ok()) return;
  reduce_max<0>(call, A, ib, dt, *cfl_number, R(-1.0));
}

void lsm3dcomputestablenormalveldtcontrolvolume_(R *dt, const R *vel_n, BOXARG(v), const R *phi_x_plus,
                                                 const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                                 const R *phi_x_minus, const R *phi_y_minus,
                                                 const R *phi_z_minus, BOXARG(m), CVARGS, IBARGS, DXP,
                                                 const R *cfl_number) {
  normal_dt("lsm3dcomputestablenormalveldtcontrolvolume_", false, dt, vel_n, BOXOF(v), R(0), phi_x_plus,
            phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), IBOX, *dx, *dy,
            *dz, *cfl_number, control_vol, BOXOF(c), CVSGN);
}

void lsm3dcomputestableconstnormalveldtcontrolvolume_(R *dt, const R *vel_n, const R *phi_x_plus,
                                                      const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                                      const R *phi_x_minus, const R *phi_y_minus,
                                                      const R *phi_z_minus, BOXARG(m), CVARGS, IBARGS, DXP,
                                                      const R *cfl_number) {
  normal_dt("lsm3dcomputestableconstnormalveldtcontrolvolume_", true, dt, nullptr, Box{}, *vel_n, phi_x_plus,
            phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), IBOX, *dx, *dy,
            *dz, *cfl_number, control_vol, BOXOF(c), CVSGN);
}

}  // extern "C"
