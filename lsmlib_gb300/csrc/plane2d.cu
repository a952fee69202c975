// LSMLIB's 2D routines that have no 3D counterpart to run on: the 9-point and
// signed-distance mean curvatures (curvature2d.f.in:98, :178 and their list
// forms, curvature2d_local.f.in:115, :211), the central divergence
// (spatial_derivatives2d.f.in:2452, spatial_derivatives2d_local.f.in:1769)
// Smereka's second-order delta function (calculus_toolbox2d.f.in:100), the
// surface integrals with a precomputed delta function (math_utils2d.f.in:713,
// :1744) and the list mean absolute difference (math_utils2d_local.f.in:86).
// LSMLIB's symbol names and argument lists (include/lsmgpu_toolbox2d.h); a
// 2D array phi(ilo:ihi, jlo:jhi) is the 3D array phi(ilo:ihi, jlo:jhi, 0:0).
// One thread per fill-box cell or list entry, the reference's operation
// order, compiled without FMA contraction (FP64 parity form).
#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu_toolbox2d.h"

namespace lsmgpu {
namespace {

typedef double R;
typedef unsigned char U8;

const int kZero = 0;

#define B2ARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi
#define B2OF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, &kZero, &kZero)

template <class F>
__global__ void k_plane(F f, Box b) {
  LSMGPU_CELL_INDEX(b, i, j, k);
  f(i, j);
}
template <class F>
void for_plane(const Box &b, F f) {
  if (b.empty()) return;
  Grid3 g = cover(b);
  LSMGPU_LAUNCH(k_plane<F>, g.grid, g.block, 0, f, b);
}

// one thread per list entry l in [lo, hi] (index_x(nlo:nhi), entry l at
// element l - lo); the cell takes part when it lies in `safe` and in the
// narrow_band array and narrow_band(i, j) <= mark (INTEGER*1, signed)
struct Plane2List {
  const int *ix, *iy;
  int lo, hi;
  View<const U8> nb;
  Box nbb, safe;
  signed char mark;
  __device__ __forceinline__ bool take(int i, int j) const {
    return inbox(safe, i, j, 0) && inbox(nbb, i, j, 0) && (signed char)nb(i, j, 0) <= mark;
  }
};
template <class F>
__global__ void k_plane_list(F f, Plane2List L) {
  const long long l = (long long)L.lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (l > L.hi) return;
  const int i = L.ix[l - L.lo], j = L.iy[l - L.lo];
  if (L.take(i, j)) f(i, j);
}
template <class F>
void for_plane_list(const Plane2List &L, F f) {
  if (L.hi < L.lo) return;
  const long long n = (long long)L.hi - L.lo + 1;
  LSMGPU_LAUNCH(k_plane_list<F>, (unsigned)((n + 255) / 256), 256, 0, f, L);
}

Plane2List plane_list(Call &c, const int *ix, const int *iy, const int *nlo, const int *nhi, const U8 *nb,
                      const Box &nbb, const U8 *mark, const Box &safe) {
  Plane2List L{};
  L.lo = *nlo;
  L.hi = *nhi;
  const long long n = (long long)L.hi - L.lo + 1;
  if (n > 0) {
    L.ix = c.in(ix, n);
    L.iy = c.in(iy, n);
  }
  L.nb = view((const U8 *)c.in(nb, nbb.size()), nbb);
  L.nbb = nbb;
  L.safe = safe;
  L.mark = (signed char)*mark;
  return L;
}

View<const R> vin(Call &c, const R *p, const Box &b) { return view((const R *)c.in(p, b.size()), b); }

// 9-point mean curvature at (i, j) (curvature2d.f.in:130-165): face
// gradients with the tangential difference averaged over two cells
__device__ __forceinline__ R curv9(const View<const R> &P, int i, int j, R dx, R dy) {
  const R c = R(1.0) / R(16.0), tol = Consts<R>::zero_tol;
  auto p = [&](int a, int b) { return P(i + a, j + b, 0); };
  const R xp = (p(1, 0) - p(0, 0)) / dx;
  R t = (p(0, 1) - p(0, -1) + p(1, 1) - p(1, -1)) / dy;
  const R nxp = sqrt(xp * xp + c * t * t);
  const R xm = (p(0, 0) - p(-1, 0)) / dx;
  t = (p(0, 1) - p(0, -1) + p(-1, 1) - p(-1, -1)) / dy;
  const R nxm = sqrt(xm * xm + c * t * t);
  const R yp = (p(0, 1) - p(0, 0)) / dy;
  t = (p(1, 0) - p(-1, 0) + p(1, 1) - p(-1, 1)) / dx;
  const R nyp = sqrt(yp * yp + c * t * t);
  const R ym = (p(0, 0) - p(0, -1)) / dy;
  t = (p(1, 0) - p(-1, 0) + p(1, -1) - p(-1, -1)) / dx;
  const R nym = sqrt(ym * ym + c * t * t);
  if (nxp < tol || nxm < tol || nyp < tol || nym < tol) return R(0);
  return (xp / nxp - xm / nxm) / dx + (yp / nyp - ym / nym) / dy;
}

// mean curvature of a signed distance function (curvature2d.f.in:210-232):
// Laplacian / (1 - phi Laplacian), `fallback` where the denominator is
// below zero_tol (1 in the dense routine, dx in the list routine,
// curvature2d_local.f.in:258)
__device__ __forceinline__ R curv_sgndist(const View<const R> &P, int i, int j, R ix2, R iy2, R fallback) {
  const R tol = Consts<R>::zero_tol, c = P(i, j, 0);
  R lap = ix2 * (P(i + 1, j, 0) - R(2.0) * c + P(i - 1, j, 0)) + iy2 * (P(i, j + 1, 0) - R(2.0) * c + P(i, j - 1, 0));
  if (fabs(lap) < tol) lap = R(0);
  R den = R(1.0) - c * lap;
  if (fabs(den) < tol) den = fallback;
  return lap / den;
}

// Smereka's second-order delta function at (i, j) (calculus_toolbox2d.f.in:150-290)
struct DeltaConsts {
  R half_dx, half_dy, odx, ody, o2dx, o2dy, odxsq, odysq, o2dxsq, o2dysq, dx, dy;
};
__device__ __forceinline__ R interface_distance(R sum1, R sum2, R diff, R od, R o2dsq) {
  const R pc = (R(1.0) / R(16.0)) * (R(9.0) * sum1 - sum2);
  const R dpc = diff * od;
  const R d2pc = (sum2 - sum1) * o2dsq;
  return -(pc / dpc) - R(0.5) * (d2pc * pc * pc) / (dpc * dpc * dpc);
}
__device__ R delta2(const View<const R> &P, const View<const R> &NX, const View<const R> &NY, int i, int j,
                    const DeltaConsts &K) {
  auto p = [&](int a, int b) { return P(i + a, j + b, 0); };
  const R zero = R(0);
  const R nx = NX(i, j, 0), ny = NY(i, j, 0);
  const R sx = -ny, sy = nx;
  const R dxsx = K.o2dx * (-NY(i + 1, j, 0) + NY(i - 1, j, 0));
  const R dysx = K.o2dy * (-NY(i, j + 1, 0) + NY(i, j - 1, 0));
  const R dxsy = K.o2dx * (NX(i + 1, j, 0) - NX(i - 1, j, 0));
  const R dysy = K.o2dy * (NX(i, j + 1, 0) - NX(i, j - 1, 0));
  const R tmpx = dxsx * sx + dysx * sy;
  const R tmpy = dxsy * sx + dysy * sy;
  const R D = -((sx * ny + sy * nx) * (nx * tmpx + ny * tmpy));
  const R jx = -D * copysign(R(1.0), nx);
  const R jy = D * copysign(R(1.0), ny);
  const R c = p(0, 0);
  R dxp = zero, dxm = zero, dyp = zero, dym = zero;
  if (p(1, 0) * c <= zero) {
    const R diff = p(1, 0) - c;
    const R pi = interface_distance(c + p(1, 0), p(-1, 0) + p(2, 0), diff, K.odx, K.o2dxsq);
    const R h = (fabs(pi) < K.half_dx) ? K.half_dx - pi : fabs(K.dx * p(1, 0) / diff);
    dxp = h * (fabs(nx) + R(0.5) * h * jx);
  }
  if (p(-1, 0) * c < zero) {
    const R diff = c - p(-1, 0);
    const R pi = interface_distance(p(-1, 0) + c, p(-2, 0) + p(1, 0), diff, K.odx, K.o2dxsq);
    const R h = (fabs(pi) < K.half_dx) ? K.half_dx + pi : fabs(K.dx * p(-1, 0) / diff);
    dxm = (fabs(nx) - R(0.5) * h * jx) * h;
  }
  if (p(0, 1) * c <= zero) {
    const R diff = p(0, 1) - c;
    const R pi = interface_distance(c + p(0, 1), p(0, -1) + p(0, 2), diff, K.ody, K.o2dysq);
    const R h = (fabs(pi) < K.half_dy) ? K.half_dy - pi : fabs(K.dy * p(0, 1) / diff);
    dyp = h * (fabs(ny) + R(0.5) * h * jy);
  }
  if (p(0, -1) * c < zero) {
    const R diff = c - p(0, -1);
    const R pi = interface_distance(p(0, -1) + c, p(0, -2) + p(0, 1), diff, K.ody, K.o2dysq);
    const R h = (fabs(pi) < K.half_dy) ? K.half_dy + pi : fabs(K.dy * p(0, -1) / diff);
    dym = (fabs(ny) - R(0.5) * h * jy) * h;
  }
  return (dxp + dxm) * K.odxsq + (dyp + dym) * K.odysq;
}

// ---- deterministic sums ------------------------------------------------------
// LSMLIB adds its terms serially.  Here the n terms (cells of an index box in
// memory order, or list entries) are split into kSumBlocks fixed contiguous
// chunks; a block adds its chunk lane-strided and in a fixed tree, one block
// adds the chunk sums in a fixed tree.  The result depends on the data only,
// within (n + 16) 2^-53 sum|term| of the serial sum.  Counts are exact.
constexpr int kSumBlocks = 304;  // two per SM
constexpr int kSumThreads = 256;

template <class F>
__global__ void __launch_bounds__(kSumThreads) k_plane_sum(F term, long long n, R *part_sum,
                                                           unsigned long long *part_cnt) {
  __shared__ R ss[kSumThreads];
  __shared__ unsigned long long sc[kSumThreads];
  const int t = threadIdx.x;
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long long b0 = (long long)blockIdx.x * chunk;
  const long long b1 = b0 + chunk < n ? b0 + chunk : n;
  R sum = R(0);
  unsigned long long cnt = 0;
  for (long long q = b0 + t; q < b1; q += kSumThreads) {
    R v;
    if (term(q, v)) {
      sum = sum + v;
      cnt++;
    }
  }
  ss[t] = sum;
  sc[t] = cnt;
  __syncthreads();
  for (int w = kSumThreads / 2; w > 0; w >>= 1) {
    if (t < w) {
      ss[t] = ss[t] + ss[t + w];
      sc[t] += sc[t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
    part_sum[blockIdx.x] = ss[0];
    part_cnt[blockIdx.x] = sc[0];
  }
}

// AVERAGE: sum / count (0 when nothing was counted), else the sum
template <bool AVERAGE>
__global__ void __launch_bounds__(kSumThreads) k_plane_sum_final(const R *part_sum,
                                                                 const unsigned long long *part_cnt, int np,
                                                                 R *out) {
  __shared__ R ss[kSumThreads];
  __shared__ unsigned long long sc[kSumThreads];
  const int t = threadIdx.x;
  R sum = R(0);
  unsigned long long cnt = 0;
  for (int q = t; q < np; q += kSumThreads) {
    sum = sum + part_sum[q];
    cnt += part_cnt[q];
  }
  ss[t] = sum;
  sc[t] = cnt;
  __syncthreads();
  for (int w = kSumThreads / 2; w > 0; w >>= 1) {
    if (t < w) {
      ss[t] = ss[t] + ss[t + w];
      sc[t] += sc[t + w];
    }
    __syncthreads();
  }
  if (t == 0) *out = AVERAGE ? (sc[0] > 0 ? ss[0] / (R)sc[0] : R(0)) : ss[0];
}

template <bool AVERAGE, class F>
void plane_sum(Call &call, F term, long long n, R *out) {
  R *dout = call.scalar_out(out);
  R *ps = call.temp<R>(kSumBlocks);
  unsigned long long *pc = call.temp<unsigned long long>(kSumBlocks);
  if (!call.ok()) return;
  LSMGPU_LAUNCH(k_plane_sum<F>, kSumBlocks, kSumThreads, 0, term, n, ps, pc);
  LSMGPU_LAUNCH(k_plane_sum_final<AVERAGE>, 1, kSumThreads, 0, ps, pc, kSumBlocks, dout);
  call.finish();
}

// integral of F delta |grad phi| dV over an index box, optionally over the
// cells of one control-volume sign (math_utils2d.f.in:713-770, :1744-1830)
struct DeltaIntegral {
  View<const R> f, dl, gm, cv;
  int cv_sgn;  // 0: every cell; > 0: control_vol > 0; < 0: control_vol < 0
  Box ib;
  R dv;
  __device__ __forceinline__ bool operator()(long long q, R &v) const {
    const long long nx = ib.n(0);
    const int i = ib.lo[0] + (int)(q % nx), j = ib.lo[1] + (int)(q / nx);
    if (cv_sgn > 0 && !(cv(i, j, 0) > R(0))) return false;
    if (cv_sgn < 0 && !(cv(i, j, 0) < R(0))) return false;
    v = dl(i, j, 0) * gm(i, j, 0) * f(i, j, 0) * dv;
    return true;
  }
};

// |field1 - field2| on the gated entries of a list (math_utils2d_local.f.in:86-150)
struct ListAbsDiff {
  const int *ix, *iy;
  View<const R> a, b;
  View<const U8> nb;
  Box nbb, safe;
  signed char mark;
  __device__ __forceinline__ bool operator()(long long q, R &v) const {
    const int i = ix[q], j = iy[q];
    if (!(inbox(safe, i, j, 0) && inbox(nbb, i, j, 0) && (signed char)nb(i, j, 0) <= mark)) return false;
    v = fabs(a(i, j, 0) - b(i, j, 0));
    return true;
  }
};

void delta_integral(const char *name, R *int_f, const R *f, const Box &fbx, const R *delta_phi, const Box &pb,
                    const R *grad_phi_mag, const Box &gb, const R *control_vol, const Box &cb, int cv_sgn,
                    const Box &ib, R dx, R dy) {
  Call call(name);
  if (!fbx.contains(ib, 0, 0, 0) || !pb.contains(ib, 0, 0, 0) || !gb.contains(ib, 0, 0, 0) ||
      (control_vol && !cb.contains(ib, 0, 0, 0)))
    call.fail("ghost box does not cover the index box");
  if (!call.ok()) return;
  DeltaIntegral T{};
  T.f = vin(call, f, fbx);
  T.dl = vin(call, delta_phi, pb);
  T.gm = vin(call, grad_phi_mag, gb);
  if (control_vol) T.cv = vin(call, control_vol, cb);
  T.cv_sgn = control_vol ? (cv_sgn > 0 ? 1 : -1) : 0;
  T.ib = ib;
  T.dv = dx * dy;
  if (!call.ok()) return;
  plane_sum<false>(call, T, ib.empty() ? 0 : ib.size(), int_f);
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

void lsm2dcomputemeancurvature9stencil_(R *kappa, B2ARG(k), const R *phi, B2ARG(f), B2ARG(fb), const R *dx,
                                        const R *dy) {
  Call call("lsm2dcomputemeancurvature9stencil_");
  const Box kb = B2OF(k), pb = B2OF(f), fb = B2OF(fb);
  if (!kb.contains(fb, 0, 0, 0) || !pb.contains(fb, 1, 1, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> K = view(call.out_region(kappa, kb, fb), kb);
  View<const R> P = vin(call, phi, pb);
  if (!call.ok()) return;
  const R dxv = *dx, dyv = *dy;
  for_plane(fb, [=] __device__(int i, int j) { K(i, j, 0) = curv9(P, i, j, dxv, dyv); });
  call.finish();
}

void lsm2dcomputemeancurvature9stencillocal_(R *kappa, B2ARG(k), const R *phi, B2ARG(f), const R *dx, const R *dy,
                                             const int *index_x, const int *index_y, const int *nlo_index,
                                             const int *nhi_index, const U8 *narrow_band, B2ARG(nb),
                                             const U8 *mark_fb) {
  Call call("lsm2dcomputemeancurvature9stencillocal_");
  const Box kb = B2OF(k), pb = B2OF(f);
  Box safe = isect(kb, pb);
  safe.lo[0] = pb.lo[0] + 1; safe.hi[0] = pb.hi[0] - 1;
  safe.lo[1] = pb.lo[1] + 1; safe.hi[1] = pb.hi[1] - 1;
  safe = isect(safe, kb);
  Plane2List L = plane_list(call, index_x, index_y, nlo_index, nhi_index, narrow_band, B2OF(nb), mark_fb, safe);
  View<R> K = view(call.inout(kappa, kb.size()), kb);
  View<const R> P = vin(call, phi, pb);
  if (!call.ok()) return;
  const R dxv = *dx, dyv = *dy;
  for_plane_list(L, [=] __device__(int i, int j) { K(i, j, 0) = curv9(P, i, j, dxv, dyv); });
  call.finish();
}

void lsm2dcomputemeancurvaturesgndist_(R *kappa, B2ARG(k), const R *phi, B2ARG(f), B2ARG(fb), const R *dx,
                                       const R *dy) {
  Call call("lsm2dcomputemeancurvaturesgndist_");
  const Box kb = B2OF(k), pb = B2OF(f), fb = B2OF(fb);
  if (!kb.contains(fb, 0, 0, 0) || !pb.contains(fb, 1, 1, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> K = view(call.out_region(kappa, kb, fb), kb);
  View<const R> P = vin(call, phi, pb);
  if (!call.ok()) return;
  const R ix2 = R(1.0) / *dx / *dx, iy2 = R(1.0) / *dy / *dy;
  for_plane(fb, [=] __device__(int i, int j) { K(i, j, 0) = curv_sgndist(P, i, j, ix2, iy2, R(1.0)); });
  call.finish();
}

void lsm2dcomputemeancurvaturesgndistlocal_(R *kappa, B2ARG(k), const R *phi, B2ARG(f), const R *dx, const R *dy,
                                            const int *index_x, const int *index_y, const int *nlo_index,
                                            const int *nhi_index, const U8 *narrow_band, B2ARG(nb),
                                            const U8 *mark_fb) {
  Call call("lsm2dcomputemeancurvaturesgndistlocal_");
  const Box kb = B2OF(k), pb = B2OF(f);
  Box safe = pb;
  safe.lo[0] += 1; safe.hi[0] -= 1;
  safe.lo[1] += 1; safe.hi[1] -= 1;
  safe = isect(safe, kb);
  Plane2List L = plane_list(call, index_x, index_y, nlo_index, nhi_index, narrow_band, B2OF(nb), mark_fb, safe);
  View<R> K = view(call.inout(kappa, kb.size()), kb);
  View<const R> P = vin(call, phi, pb);
  if (!call.ok()) return;
  const R ix2 = R(1.0) / *dx / *dx, iy2 = R(1.0) / *dy / *dy, dxv = *dx;
  for_plane_list(L, [=] __device__(int i, int j) { K(i, j, 0) = curv_sgndist(P, i, j, ix2, iy2, dxv); });
  call.finish();
}

void lsm2ddivergencecentral_(R *divf, B2ARG(d), const R *fx, const R *fy, B2ARG(g), B2ARG(fb), const R *dx,
                             const R *dy) {
  Call call("lsm2ddivergencecentral_");
  const Box db = B2OF(d), gb = B2OF(g), fb = B2OF(fb);
  if (!db.contains(fb, 0, 0, 0) || !gb.contains(fb, 1, 1, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<R> D = view(call.out_region(divf, db, fb), db);
  View<const R> FX = vin(call, fx, gb), FY = vin(call, fy, gb);
  if (!call.ok()) return;
  const R fxf = R(0.5) / *dx, fyf = R(0.5) / *dy;
  for_plane(fb, [=] __device__(int i, int j) {
    D(i, j, 0) = (FX(i + 1, j, 0) - FX(i - 1, j, 0)) * fxf + (FY(i, j + 1, 0) - FY(i, j - 1, 0)) * fyf;
  });
  call.finish();
}

void lsm2ddivergencecentrallocal_(R *divf, B2ARG(d), const R *fx, const R *fy, B2ARG(g), const R *dx, const R *dy,
                                  const int *index_x, const int *index_y, const int *nlo_index,
                                  const int *nhi_index, const U8 *narrow_band, B2ARG(nb), const U8 *mark_fb) {
  Call call("lsm2ddivergencecentrallocal_");
  const Box db = B2OF(d), gb = B2OF(g);
  Box safe = gb;
  safe.lo[0] += 1; safe.hi[0] -= 1;
  safe.lo[1] += 1; safe.hi[1] -= 1;
  safe = isect(safe, db);
  Plane2List L = plane_list(call, index_x, index_y, nlo_index, nhi_index, narrow_band, B2OF(nb), mark_fb, safe);
  View<R> D = view(call.inout(divf, db.size()), db);
  View<const R> FX = vin(call, fx, gb), FY = vin(call, fy, gb);
  if (!call.ok()) return;
  const R fxf = R(0.5) / *dx, fyf = R(0.5) / *dy;
  for_plane_list(L, [=] __device__(int i, int j) {
    D(i, j, 0) = (FX(i + 1, j, 0) - FX(i - 1, j, 0)) * fxf + (FY(i, j + 1, 0) - FY(i, j - 1, 0)) * fyf;
  });
  call.finish();
}

void lsm2ddeltafunctionorder2_(const R *phi, R *delta, B2ARG(g), const R *norm_phi_x, const R *norm_phi_y,
                               B2ARG(n), B2ARG(fb), const R *dx, const R *dy) {
  Call call("lsm2ddeltafunctionorder2_");
  const Box gb = B2OF(g), nb = B2OF(n), fb = B2OF(fb);
  if (!gb.contains(fb, 2, 2, 0) || !nb.contains(fb, 1, 1, 0)) call.fail("ghost box does not cover the stencil");
  if (!call.ok() || fb.empty()) return;
  View<const R> P = vin(call, phi, gb);
  View<R> D = view(call.out_region(delta, gb, fb), gb);
  View<const R> NX = vin(call, norm_phi_x, nb), NY = vin(call, norm_phi_y, nb);
  if (!call.ok()) return;
  const R dxv = *dx, dyv = *dy;
  DeltaConsts K;
  K.dx = dxv; K.dy = dyv;
  K.half_dx = R(0.5) * dxv; K.half_dy = R(0.5) * dyv;
  K.odx = R(1.0) / dxv; K.ody = R(1.0) / dyv;
  K.o2dx = R(0.5) / dxv; K.o2dy = R(0.5) / dyv;
  K.odxsq = R(1.0) / dxv / dxv; K.odysq = R(1.0) / dyv / dyv;
  K.o2dxsq = R(0.5) / dxv / dxv; K.o2dysq = R(0.5) / dyv / dyv;
  for_plane(fb, [=] __device__(int i, int j) { D(i, j, 0) = delta2(P, NX, NY, i, j, K); });
  call.finish();
}

void lsm2dsurfaceintegralprecomputeddelta_(R *int_f, const R *f, B2ARG(f), const R *delta_phi, B2ARG(p),
                                           const R *grad_phi_mag, B2ARG(g), B2ARG(ib), const R *dx, const R *dy) {
  delta_integral("lsm2dsurfaceintegralprecomputeddelta_", int_f, f, B2OF(f), delta_phi, B2OF(p), grad_phi_mag,
                 B2OF(g), nullptr, Box{}, 0, B2OF(ib), *dx, *dy);
}

void lsm2dsurfaceintegralprecomputeddeltacontrolvolume_(R *int_f, const R *f, B2ARG(f), const R *delta_phi,
                                                        B2ARG(p), const R *grad_phi_mag, B2ARG(g),
                                                        const R *control_vol, B2ARG(c), const int *control_vol_sgn,
                                                        B2ARG(ib), const R *dx, const R *dy) {
  delta_integral("lsm2dsurfaceintegralprecomputeddeltacontrolvolume_", int_f, f, B2OF(f), delta_phi, B2OF(p),
                 grad_phi_mag, B2OF(g), control_vol, B2OF(c), *control_vol_sgn, B2OF(ib), *dx, *dy);
}

void lsm2daveabsdifflocal_(R *ave_abs_diff, const R *field1, B2ARG(a), const R *field2, B2ARG(b),
                           const int *index_x, const int *index_y, const int *nlo_index, const int *nhi_index,
                           const U8 *narrow_band, B2ARG(nb), const U8 *mark_fb) {
  Call call("lsm2daveabsdifflocal_");
  const Box ab = B2OF(a), bb = B2OF(b), nbb = B2OF(nb);
  ListAbsDiff T{};
  const long long n = (long long)*nhi_index - *nlo_index + 1;
  if (n > 0) {
    T.ix = call.in(index_x, n);
    T.iy = call.in(index_y, n);
  }
  T.a = vin(call, field1, ab);
  T.b = vin(call, field2, bb);
  T.nb = view((const U8 *)call.in(narrow_band, nbb.size()), nbb);
  T.nbb = nbb;
  T.safe = isect(ab, bb);
  T.mark = (signed char)*mark_fb;
  if (!call.ok()) return;
  plane_sum<true>(call, T, n > 0 ? n : 0, ave_abs_diff);
}

}  // extern "C"
