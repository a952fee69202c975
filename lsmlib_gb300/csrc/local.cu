// Drop-in narrow-band (index-list) entry points: LSMLIB's *_local routines
// with LSMLIB's symbol names and argument lists, one thread per list entry.
//
// Conventions kept from the reference (spatial_derivatives3d_local.f.in and
// the other *_local files):
//  - the lists are declared index_x(nlo:nhi) with the routine's first lower
//    bound, so entry l is element l - nlo of the array passed in;
//  - a cell takes part when narrow_band(i,j,k) <= mark (INTEGER*1, signed);
//  - the derivative routines first fill the caller's scratch D1 (D2, D3) over
//    the listed cells (1e10 where the cell's mark exceeds the scratch mark)
//    and then read it, so scratch contents are an observable input and output
//    exactly as in the reference.
// This translation unit is compiled with -fmad=false (FP64 parity form).
#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

namespace lsmgpu {
namespace {

typedef double R;
typedef unsigned char U8;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)

struct List {
  const int *ix, *iy, *iz;
  int decl;  // declared lower bound of the arrays
};

// cells outside the narrow_band array, or whose stencil would leave an array's
// ghost box, are skipped (LSMLIB reads outside the arrays there)
struct Gate {
  View<const U8> nb;
  Box nbb;   // narrow_band's ghost box
  Box safe;  // cells whose stencil stays inside every array this routine touches
  signed char mark;
  __device__ __forceinline__ bool ok(int i, int j, int k) const { return inbox(safe, i, j, k) && inbox(nbb, i, j, k); }
  __device__ __forceinline__ bool pass(int i, int j, int k) const { return (signed char)nb(i, j, k) <= mark; }
  __device__ __forceinline__ bool operator()(int i, int j, int k) const { return ok(i, j, k) && pass(i, j, k); }
  Gate with(const Box &s, unsigned char m) const {
    Gate g = *this;
    g.safe = s;
    g.mark = (signed char)m;
    return g;
  }
};

inline Box everything() {
  Box b;
  for (int d = 0; d < 3; d++) { b.lo[d] = -2147483647; b.hi[d] = 2147483647; }
  return b;
}

// one thread per list entry l in [lo, hi]
template <class F>
__global__ void k_list(F f, List L, int lo, int hi) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long l = (long long)lo + t;
  if (l > hi) return;
  const long long e = l - L.decl;
  f(L.ix[e], L.iy[e], L.iz[e]);
}

template <class F>
void for_list(const List &L, int lo, int hi, F f) {
  if (hi < lo) return;
  const long long n = (long long)hi - lo + 1;
  const int bs = 256;
  LSMGPU_LAUNCH(k_list<F>, (unsigned)((n + bs - 1) / bs), bs, 0, f, L, lo, hi);
}

// staging helpers -----------------------------------------------------------
struct LocalCall {
  Call c;
  explicit LocalCall(const char *name) : c(name) {}
  List list(const int *ix, const int *iy, const int *iz, int decl_lo, int decl_hi) {
    List L;
    const long long n = (long long)decl_hi - decl_lo + 1;
    L.decl = decl_lo;
    if (n <= 0) {
      L.ix = L.iy = L.iz = nullptr;
      return L;
    }
    L.ix = c.in(ix, n);
    L.iy = c.in(iy, n);
    L.iz = c.in(iz, n);
    return L;
  }
  Gate gate(const unsigned char *nb, const Box &b, unsigned char mark) {
    Gate g;
    g.nb = view((const U8 *)c.in(nb, b.size()), b);
    g.nbb = b;
    g.safe = everything();
    g.mark = (signed char)mark;
    return g;
  }
  View<const R> in(const R *p, const Box &b) { return view((const R *)c.in(p, b.size()), b); }
  View<R> inout(R *p, const Box &b) { return view(c.inout(p, b.size()), b); }
};

// undivided differences over a list (spatial_derivatives3d_local.f.in:43-138)
void dn_local(View<R> dn, const Box &db, View<const R> dm, const Box &mb, int n, int dir, const List &L, int lo,
              int hi, Gate g) {
  // Dn(i) reads Dm(i) and Dm(i - 1) (odd n) or Dm(i + 1) (even n) along dir
  g.safe = isect(g.safe, isect(db, inner_axis(mb, dir, n % 2 == 1 ? 1 : 0, n % 2 == 1 ? 0 : 1)));
  int o0 = 0, o1 = 0, o2 = 0;
  const int off = (n % 2 == 1) ? 1 : -1;
  const R sgn = (n % 2 == 1) ? R(1.0) : R(-1.0);
  if (dir == 0) o0 = off;
  if (dir == 1) o1 = off;
  if (dir == 2) o2 = off;
  for_list(L, lo, hi, [=] __device__(int i, int j, int k) {
    if (!g.ok(i, j, k)) return;
    if (g.pass(i, j, k))
      dn(i, j, k) = sgn * (dm(i, j, k) - dm(i - o0, j - o1, k - o2));
    else
      dn(i, j, k) = R(1.0e10);
  });
}

struct PM3 { View<R> x, y, z; __device__ View<R> operator[](int d) const { return d == 0 ? x : (d == 1 ? y : z); } };

__device__ __forceinline__ long long dstride(const View<R> &v, int d) { return d == 0 ? 1 : (d == 1 ? v.s1 : v.s2); }

// WENO5 with the local routines' epsilon floor 1e-35
// (spatial_derivatives2d_local.f.in:892)
__device__ __forceinline__ R weno5_local(R v1, R v2, R v3, R v4, R v5) {
  const R c13 = 1.0 / 3.0, c76 = 7.0 / 6.0, c116 = 11.0 / 6.0, c16 = 1.0 / 6.0, c56 = 5.0 / 6.0;
  const R c1312 = 13.0 / 12.0, c14 = 0.25;
  R m = v1 * v1;
  m = rmax(m, v2 * v2);
  m = rmax(m, v3 * v3);
  m = rmax(m, v4 * v4);
  m = rmax(m, v5 * v5);
  const R eps = R(1e-6) * m + R(1.e-35);
  const R p1 = c13 * v1 - c76 * v2 + c116 * v3;
  const R p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  const R p3 = c13 * v3 + c56 * v4 - c16 * v5;
  R t = v1 - R(2.0) * v2 + v3, u = v1 - R(4.0) * v2 + R(3.0) * v3;
  const R S1 = c1312 * (t * t) + c14 * (u * u);
  t = v2 - R(2.0) * v3 + v4; u = v2 - v4;
  const R S2 = c1312 * (t * t) + c14 * (u * u);
  t = v3 - R(2.0) * v4 + v5; u = R(3.0) * v3 - R(4.0) * v4 + v5;
  const R S3 = c1312 * (t * t) + c14 * (u * u);
  R a1 = R(0.1) / ((S1 + eps) * (S1 + eps));
  R a2 = R(0.6) / ((S2 + eps) * (S2 + eps));
  R a3 = R(0.3) / ((S3 + eps) * (S3 + eps));
  const R is = R(1.0) / (a1 + a2 + a3);
  a1 = a1 * is; a2 = a2 * is; a3 = a3 * is;
  return a1 * p1 + a2 * p2 + a3 * p3;
}

// ---- max / sum reductions over lists ----------------------------------------
__device__ __forceinline__ unsigned long long okey(R v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ R okey_inv(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}
__global__ void k_init_key(unsigned long long *key, R v) { *key = okey(v); }
// mode 0: dt = cfl/(max + tiny); mode 1: the max itself
__global__ void k_key_result(const unsigned long long *key, R *out, int mode, R cfl) {
  const R m = okey_inv(*key);
  *out = mode == 1 ? m : cfl / (m + Consts<R>::tiny);
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

#define IDX3 const int *index_x, const int *index_y, const int *index_z
#define NBARG const unsigned char *narrow_band, BOXARG(nb)
#define DXP const R *dx, const R *dy, const R *dz

// Gaussian curvature (order 2, 4) and curvature order 4 over lists
// (curvature3d_local.f.in:151-574).  The reference's 3D MeanCurvatureOrder4
// local routine evaluates the Gaussian-curvature formula (numerator and
// |grad phi|^4 denominator, curvature3d_local.f.in:385-410); its entry point
// keeps that, and lsmgpu_mean_curvature_order4_local evaluates the mean
// curvature the dense routine and the 2D local routine compute.
template <int K>
void curv_variant_local(const char *name, R *kappa, const Box &kb, const R *phi, const Box &fb, const R *phi_x,
                        const R *phi_y, const R *phi_z, const R *grad_phi_mag, const Box &gb, R dxv, R dyv, R dzv,
                        const int *index_x, const int *index_y, const int *index_z, const int *nlo,
                        const int *nhi, const unsigned char *narrow_band, const Box &nbb,
                        const unsigned char *mark_fb) {
  LocalCall lc(name);
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  Gate g = lc.gate(narrow_band, nbb, *mark_fb);
  View<R> KA = lc.inout(kappa, kb);
  View<const R> F = lc.in(phi, fb);
  View<const R> X = lc.in(phi_x, gb), Y = lc.in(phi_y, gb), Z = lc.in(phi_z, gb), G = lc.in(grad_phi_mag, gb);
  const int rp = (K == CURV_GAUSS2) ? 1 : 2, rg = (K == CURV_GAUSS2) ? 0 : 2;
  g.safe = isect(isect(kb, inner(gb, rg, rg, rg, rg, rg, rg)), inner(fb, rp, rp, rp, rp, rp, rp));
  if (!lc.c.ok()) return;
  const CurvFactors<R> cf = curvature_factors<R, K>(dxv, dyv, dzv);
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const long long o = X.off(i, j, k);
    KA(i, j, k) = curvature_variant<R, K>(F.p + F.off(i, j, k), F.s1, F.s2, X.p + o, Y.p + o, Z.p + o, X.s1, X.s2,
                                          G(i, j, k), cf);
  });
  lc.c.finish();
}

// orthogonalization equation RHS on listed cells
// (reinitialization3d_local.f.in:326-480); SGN3 = false gives the 2D
// routine's smoothing of sgn(psi) (reinitialization2d_local.f.in:406)
template <bool SGN3>
void ortho_local(const char *name, R *ortho_rhs, const Box &rb, const R *phi_x_plus, const R *phi_y_plus,
                 const R *phi_z_plus, const Box &pb, const R *phi_x_minus, const R *phi_y_minus,
                 const R *phi_z_minus, const Box &mb, const R *psi, const Box &sb, const R *psi_x_plus,
                 const R *psi_y_plus, const R *psi_z_plus, const Box &spb, const R *psi_x_minus,
                 const R *psi_y_minus, const R *psi_z_minus, const Box &smb, R dx, R dy, R dz,
                 const int *index_x, const int *index_y, const int *index_z, const int *nlo, const int *nhi,
                 const unsigned char *narrow_band, const Box &nbb, const unsigned char *mark_fb) {
  LocalCall lc(name);
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  Gate g = lc.gate(narrow_band, nbb, *mark_fb);
  View<R> O = lc.inout(ortho_rhs, rb);
  View<const R> XP = lc.in(phi_x_plus, pb), YP = lc.in(phi_y_plus, pb), ZP = lc.in(phi_z_plus, pb);
  View<const R> XM = lc.in(phi_x_minus, mb), YM = lc.in(phi_y_minus, mb), ZM = lc.in(phi_z_minus, mb);
  View<const R> S = lc.in(psi, sb);
  View<const R> SXP = lc.in(psi_x_plus, spb), SYP = lc.in(psi_y_plus, spb), SZP = lc.in(psi_z_plus, spb);
  View<const R> SXM = lc.in(psi_x_minus, smb), SYM = lc.in(psi_y_minus, smb), SZM = lc.in(psi_z_minus, smb);
  g.safe = isect(isect(isect(rb, sb), isect(pb, mb)), isect(spb, smb));
  if (!lc.c.ok()) return;
  R dx_sq = rmax(rmax(dx, dy), dz);
  dx_sq = dx_sq * dx_sq;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R psp[3] = {SXP(i, j, k), SYP(i, j, k), SZP(i, j, k)}, psm[3] = {SXM(i, j, k), SYM(i, j, k), SZM(i, j, k)};
    const R pp[3] = {XP(i, j, k), YP(i, j, k), ZP(i, j, k)}, pm[3] = {XM(i, j, k), YM(i, j, k), ZM(i, j, k)};
    O(i, j, k) = lsmgpu::ortho_rhs<R, SGN3>(S(i, j, k), psp, psm, pp, pm, dx_sq);
  });
  lc.c.finish();
}

extern "C" {

void lsm3dcomputednlocal_(R *dn, BOXARG(d), const R *dm, BOXARG(m), const int *n, const int *dir, IDX3,
                          const int *nlo, const int *nhi, NBARG, const unsigned char *mark_fb) {
  LocalCall lc("lsm3dcomputednlocal_");
  Box db = BOXOF(d), mb = BOXOF(m), nbb = BOXOF(nb);
  if (*dir < 1 || *dir > 3) { lc.c.fail("dir must be 1, 2 or 3"); return; }
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  Gate g = lc.gate(narrow_band, nbb, *mark_fb);
  View<R> D = lc.inout(dn, db);
  View<const R> M = lc.in(dm, mb);
  if (!lc.c.ok()) return;
  dn_local(D, db, M, mb, *n, *dir - 1, L, *nlo, *nhi, g);
  lc.c.finish();
}

#define PMARGS R *phi_x_plus, R *phi_y_plus, R *phi_z_plus, BOXARG(p), R *phi_x_minus, R *phi_y_minus, R *phi_z_minus, BOXARG(m), const R *phi, BOXARG(f)

void lsm3dhjeno1local_(PMARGS, R *d1, BOXARG(d1), DXP, IDX3, const int *nlo0, const int *nhi0,
                       const int *nlo1, const int *nhi1, NBARG, const unsigned char *mark_fb,
                       const unsigned char *mark_d1) {
  LocalCall lc("lsm3dhjeno1local_");
  Box pb = BOXOF(p), mb = BOXOF(m);
  List L = lc.list(index_x, index_y, index_z, *nlo0, *nhi1);
  Gate gfb = lc.gate(narrow_band, BOXOF(nb), *mark_fb);
  Gate gd1 = gfb; gd1.mark = (signed char)*mark_d1;
  PM3 P{lc.inout(phi_x_plus, pb), lc.inout(phi_y_plus, pb), lc.inout(phi_z_plus, pb)};
  PM3 M{lc.inout(phi_x_minus, mb), lc.inout(phi_y_minus, mb), lc.inout(phi_z_minus, mb)};
  View<const R> F = lc.in(phi, BOXOF(f));
  View<R> D1 = lc.inout(d1, BOXOF(d1));
  if (!lc.c.ok()) return;
  const R inv[3] = {R(1.0) / *dx, R(1.0) / *dy, R(1.0) / *dz};
  const Box d1b = BOXOF(d1), fbx = BOXOF(f), outb = isect(pb, mb);
  for (int d = 0; d < 3; d++) {
    dn_local(D1, d1b, F, fbx, 1, d, L, *nlo0, *nhi1, gd1);
    const R w = inv[d];
    const Gate gd = gfb.with(isect(outb, inner_axis(d1b, d, 0, 1)), *mark_fb);
    for_list(L, *nlo0, *nhi0, [=] __device__(int i, int j, int k) {
      if (!gd(i, j, k)) return;
      const long long c = D1.off(i, j, k), s = dstride(D1, d);
      P[d](i, j, k) = D1.p[c + s] * w;
      M[d](i, j, k) = D1.p[c] * w;
    });
  }
  lc.c.finish();
}

void lsm3dhjeno2local_(PMARGS, R *d1, BOXARG(d1), R *d2, BOXARG(d2), DXP, IDX3, const int *nlo0,
                       const int *nhi0, const int *nlo1, const int *nhi1, const int *nlo2,
                       const int *nhi2, NBARG, const unsigned char *mark_fb,
                       const unsigned char *mark_d1, const unsigned char *mark_d2) {
  LocalCall lc("lsm3dhjeno2local_");
  Box pb = BOXOF(p), mb = BOXOF(m);
  List L = lc.list(index_x, index_y, index_z, *nlo0, *nhi2);
  Gate gfb = lc.gate(narrow_band, BOXOF(nb), *mark_fb);
  Gate g1 = gfb, g2 = gfb;
  g1.mark = (signed char)*mark_d1;
  g2.mark = (signed char)*mark_d2;
  PM3 P{lc.inout(phi_x_plus, pb), lc.inout(phi_y_plus, pb), lc.inout(phi_z_plus, pb)};
  PM3 M{lc.inout(phi_x_minus, mb), lc.inout(phi_y_minus, mb), lc.inout(phi_z_minus, mb)};
  View<const R> F = lc.in(phi, BOXOF(f));
  View<R> D1 = lc.inout(d1, BOXOF(d1)), D2 = lc.inout(d2, BOXOF(d2));
  if (!lc.c.ok()) return;
  const R inv[3] = {R(1.0) / *dx, R(1.0) / *dy, R(1.0) / *dz};
  const Box d1b = BOXOF(d1), d2b = BOXOF(d2), fbx = BOXOF(f), outb = isect(pb, mb);
  for (int d = 0; d < 3; d++) {
    dn_local(D1, d1b, F, fbx, 1, d, L, *nlo0, *nhi2, g1);
    View<const R> D1c{D1.p, D1.lo0, D1.lo1, D1.lo2, D1.s1, D1.s2};
    dn_local(D2, d2b, D1c, d1b, 2, d, L, *nlo0, *nhi1, g2);
    const R w = inv[d];
    const Gate gd = gfb.with(isect(outb, isect(inner_axis(d1b, d, 0, 1), inner_axis(d2b, d, 1, 1))), *mark_fb);
    for_list(L, *nlo0, *nhi0, [=] __device__(int i, int j, int k) {
      if (!gd(i, j, k)) return;
      const long long a = D1.off(i, j, k), b = D2.off(i, j, k);
      const long long s1 = dstride(D1, d), s2 = dstride(D2, d);
      const R *q = D2.p;
      R c = (fabs(q[b]) < fabs(q[b + s2])) ? q[b] : q[b + s2];
      P[d](i, j, k) = (D1.p[a + s1] - R(0.5) * c) * w;
      c = (fabs(q[b - s2]) < fabs(q[b])) ? q[b - s2] : q[b];
      M[d](i, j, k) = (D1.p[a] + R(0.5) * c) * w;
    });
  }
  lc.c.finish();
}

// 3D upwind HJ ENO2 over lists: no 3D original in LSMLIB; follows the 2D
// lsm2dUpwindHJENO2LOCAL (spatial_derivatives2d_local.f.in:1160-1390): D1
// over levels 0-2, D2 over 0-1, then on level-0 cells 0 where |vel| <
// zero_tol, the minus-side ENO2 value where vel > 0, the plus side otherwise
void lsm3dupwindhjeno2local_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f), const R *vel_x,
                             const R *vel_y, const R *vel_z, BOXARG(v), R *d1, BOXARG(d1), R *d2, BOXARG(d2),
                             DXP, IDX3, const int *nlo0, const int *nhi0, const int *nlo1, const int *nhi1,
                             const int *nlo2, const int *nhi2, NBARG, const unsigned char *mark_fb,
                             const unsigned char *mark_d1, const unsigned char *mark_d2) {
  LocalCall lc("lsm3dupwindhjeno2local_");
  (void)nlo1;
  (void)nlo2;
  Box gb = BOXOF(g), vb = BOXOF(v);
  List L = lc.list(index_x, index_y, index_z, *nlo0, *nhi2);
  Gate gfb = lc.gate(narrow_band, BOXOF(nb), *mark_fb);
  Gate g1 = gfb, g2 = gfb;
  g1.mark = (signed char)*mark_d1;
  g2.mark = (signed char)*mark_d2;
  PM3 G{lc.inout(phi_x, gb), lc.inout(phi_y, gb), lc.inout(phi_z, gb)};
  View<const R> F = lc.in(phi, BOXOF(f));
  const View<const R> V[3] = {lc.in(vel_x, vb), lc.in(vel_y, vb), lc.in(vel_z, vb)};
  View<R> D1 = lc.inout(d1, BOXOF(d1)), D2 = lc.inout(d2, BOXOF(d2));
  if (!lc.c.ok()) return;
  const R inv[3] = {R(1.0) / *dx, R(1.0) / *dy, R(1.0) / *dz};
  const Box d1b = BOXOF(d1), d2b = BOXOF(d2), fbx = BOXOF(f), outb = isect(gb, vb);
  for (int d = 0; d < 3; d++) {
    dn_local(D1, d1b, F, fbx, 1, d, L, *nlo0, *nhi2, g1);
    View<const R> D1c{D1.p, D1.lo0, D1.lo1, D1.lo2, D1.s1, D1.s2};
    dn_local(D2, d2b, D1c, d1b, 2, d, L, *nlo0, *nhi1, g2);
    const R w = inv[d];
    const View<const R> U = V[d];
    const View<R> O = d == 0 ? G.x : (d == 1 ? G.y : G.z);
    const Gate gd = gfb.with(isect(outb, isect(inner_axis(d1b, d, 0, 1), inner_axis(d2b, d, 1, 1))), *mark_fb);
    for_list(L, *nlo0, *nhi0, [=] __device__(int i, int j, int k) {
      if (!gd(i, j, k)) return;
      const R u = U(i, j, k);
      const long long a = D1.off(i, j, k), b = D2.off(i, j, k);
      const long long s1 = dstride(D1, d), s2 = dstride(D2, d);
      const R *q = D2.p;
      R r;
      if (fabs(u) < Consts<R>::zero_tol) {
        r = R(0);
      } else if (u > R(0)) {
        const R c = (fabs(q[b - s2]) < fabs(q[b])) ? q[b - s2] : q[b];
        r = (D1.p[a] + R(0.5) * c) * w;
      } else {
        const R c = (fabs(q[b]) < fabs(q[b + s2])) ? q[b] : q[b + s2];
        r = (D1.p[a + s1] - R(0.5) * c) * w;
      }
      O(i, j, k) = r;
    });
  }
  lc.c.finish();
}

void lsm3dhjeno3local_(PMARGS, R *d1, BOXARG(d1), R *d2, BOXARG(d2), R *d3, BOXARG(d3), DXP, IDX3,
                       const int *nlo0, const int *nhi0, const int *nlo1, const int *nhi1,
                       const int *nlo2, const int *nhi2, const int *nlo3, const int *nhi3, NBARG,
                       const unsigned char *mark_fb, const unsigned char *mark_d1,
                       const unsigned char *mark_d2, const unsigned char *mark_d3) {
  LocalCall lc("lsm3dhjeno3local_");
  Box pb = BOXOF(p), mb = BOXOF(m);
  List L = lc.list(index_x, index_y, index_z, *nlo0, *nhi3);
  Gate gfb = lc.gate(narrow_band, BOXOF(nb), *mark_fb);
  Gate g1 = gfb, g2 = gfb, g3 = gfb;
  g1.mark = (signed char)*mark_d1;
  g2.mark = (signed char)*mark_d2;
  g3.mark = (signed char)*mark_d3;
  PM3 P{lc.inout(phi_x_plus, pb), lc.inout(phi_y_plus, pb), lc.inout(phi_z_plus, pb)};
  PM3 M{lc.inout(phi_x_minus, mb), lc.inout(phi_y_minus, mb), lc.inout(phi_z_minus, mb)};
  View<const R> F = lc.in(phi, BOXOF(f));
  View<R> D1 = lc.inout(d1, BOXOF(d1)), D2 = lc.inout(d2, BOXOF(d2)), D3 = lc.inout(d3, BOXOF(d3));
  if (!lc.c.ok()) return;
  const R inv[3] = {R(1.0) / *dx, R(1.0) / *dy, R(1.0) / *dz};
  const Box d1b = BOXOF(d1), d2b = BOXOF(d2), d3b = BOXOF(d3), fbx = BOXOF(f), outb = isect(pb, mb);
  for (int d = 0; d < 3; d++) {
    dn_local(D1, d1b, F, fbx, 1, d, L, *nlo0, *nhi3, g1);
    dn_local(D2, d2b, View<const R>{D1.p, D1.lo0, D1.lo1, D1.lo2, D1.s1, D1.s2}, d1b, 2, d, L, *nlo0, *nhi2, g2);
    dn_local(D3, d3b, View<const R>{D2.p, D2.lo0, D2.lo1, D2.lo2, D2.s1, D2.s2}, d2b, 3, d, L, *nlo0, *nhi1, g3);
    const R w = inv[d];
    const Gate gd = gfb.with(isect(outb, isect(inner_axis(d1b, d, 0, 1), isect(inner_axis(d2b, d, 1, 1),
                                                                               inner_axis(d3b, d, 1, 2)))),
                             *mark_fb);
    for_list(L, *nlo0, *nhi0, [=] __device__(int i, int j, int k) {
      if (!gd(i, j, k)) return;
      const R third = R(1.0 / 3.0), sixth = R(1.0 / 6.0), h = R(0.5);
      const long long a = D1.off(i, j, k), b = D2.off(i, j, k), c3 = D3.off(i, j, k);
      const long long s1 = dstride(D1, d), s2 = dstride(D2, d), s3 = dstride(D3, d);
      const R *q2 = D2.p, *q3 = D3.p;
      R x = D1.p[a + s1];
      if (fabs(q2[b]) < fabs(q2[b + s2])) {
        x = x - h * q2[b];
        x = (fabs(q3[c3]) < fabs(q3[c3 + s3])) ? x - sixth * q3[c3] : x - sixth * q3[c3 + s3];
      } else {
        x = x - h * q2[b + s2];
        x = (fabs(q3[c3 + s3]) < fabs(q3[c3 + 2 * s3])) ? x + third * q3[c3 + s3] : x + third * q3[c3 + 2 * s3];
      }
      P[d](i, j, k) = x * w;
      x = D1.p[a];
      if (fabs(q2[b - s2]) < fabs(q2[b])) {
        x = x + h * q2[b - s2];
        x = (fabs(q3[c3 - s3]) < fabs(q3[c3])) ? x + third * q3[c3 - s3] : x + third * q3[c3];
      } else {
        x = x + h * q2[b];
        x = (fabs(q3[c3]) < fabs(q3[c3 + s3])) ? x - sixth * q3[c3] : x - sixth * q3[c3 + s3];
      }
      M[d](i, j, k) = x * w;
    });
  }
  lc.c.finish();
}

void lsm3dhjweno5local_(PMARGS, R *d1, BOXARG(d1), DXP, IDX3, const int *nlo0, const int *nhi0,
                        const int *nlo1, const int *nhi1, const int *nlo2, const int *nhi2,
                        const int *nlo3, const int *nhi3, NBARG, const unsigned char *mark_fb,
                        const unsigned char *mark_d1) {
  LocalCall lc("lsm3dhjweno5local_");
  Box pb = BOXOF(p), mb = BOXOF(m);
  List L = lc.list(index_x, index_y, index_z, *nlo0, *nhi3);
  Gate gfb = lc.gate(narrow_band, BOXOF(nb), *mark_fb);
  Gate g1 = gfb;
  g1.mark = (signed char)*mark_d1;
  PM3 P{lc.inout(phi_x_plus, pb), lc.inout(phi_y_plus, pb), lc.inout(phi_z_plus, pb)};
  PM3 M{lc.inout(phi_x_minus, mb), lc.inout(phi_y_minus, mb), lc.inout(phi_z_minus, mb)};
  View<const R> F = lc.in(phi, BOXOF(f));
  View<R> D1 = lc.inout(d1, BOXOF(d1));
  if (!lc.c.ok()) return;
  const R inv[3] = {R(1.0) / *dx, R(1.0) / *dy, R(1.0) / *dz};
  const Box d1b = BOXOF(d1), fbx = BOXOF(f), outb = isect(pb, mb);
  for (int d = 0; d < 3; d++) {
    dn_local(D1, d1b, F, fbx, 1, d, L, *nlo0, *nhi3, g1);
    const R w = inv[d];
    const Gate gd = gfb.with(isect(outb, inner_axis(d1b, d, 2, 3)), *mark_fb);
    for_list(L, *nlo0, *nhi0, [=] __device__(int i, int j, int k) {
      if (!gd(i, j, k)) return;
      const long long c = D1.off(i, j, k), s = dstride(D1, d);
      const R *q = D1.p;
      P[d](i, j, k) = weno5_local(q[c + 3 * s] * w, q[c + 2 * s] * w, q[c + s] * w, q[c] * w, q[c - s] * w);
      M[d](i, j, k) = weno5_local(q[c - 2 * s] * w, q[c - s] * w, q[c] * w, q[c + s] * w, q[c + 2 * s] * w);
    });
  }
  lc.c.finish();
}

#define LTAIL IDX3, const int *nlo, const int *nhi, NBARG, const unsigned char *mark_fb
#define LSETUP(name)                                         \
  LocalCall lc(name);                                        \
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);   \
  Gate g = lc.gate(narrow_band, BOXOF(nb), *mark_fb);

void lsm3dcentralgradorder2local_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f), DXP,
                                  LTAIL) {
  LSETUP("lsm3dcentralgradorder2local_")
  Box gb = BOXOF(g);
  View<R> X = lc.inout(phi_x, gb), Y = lc.inout(phi_y, gb), Z = lc.inout(phi_z, gb);
  View<const R> F = lc.in(phi, BOXOF(f));
  g.safe = isect(gb, inner(BOXOF(f), 1, 1, 1, 1, 1, 1));
  if (!lc.c.ok()) return;
  const R fx = R(0.5) / *dx, fy = R(0.5) / *dy, fz = R(0.5) / *dz;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R *c = F.p + F.off(i, j, k);
    X(i, j, k) = (c[1] - c[-1]) * fx;
    Y(i, j, k) = (c[F.s1] - c[-F.s1]) * fy;
    Z(i, j, k) = (c[F.s2] - c[-F.s2]) * fz;
  });
  lc.c.finish();
}

void lsm3dcentralgradorder4local_(R *phi_x, R *phi_y, R *phi_z, BOXARG(g), const R *phi, BOXARG(f), DXP,
                                  LTAIL) {
  LSETUP("lsm3dcentralgradorder4local_")
  Box gb = BOXOF(g);
  View<R> X = lc.inout(phi_x, gb), Y = lc.inout(phi_y, gb), Z = lc.inout(phi_z, gb);
  View<const R> F = lc.in(phi, BOXOF(f));
  g.safe = isect(gb, inner(BOXOF(f), 2, 2, 2, 2, 2, 2));
  if (!lc.c.ok()) return;
  const R c12 = R(0.0833333333333333333333);
  const R fx = c12 / *dx, fy = c12 / *dy, fz = c12 / *dz;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R *c = F.p + F.off(i, j, k);
    const R e = R(8.0);
    const long long s[3] = {1, F.s1, F.s2};
    const R f[3] = {fx, fy, fz};
    R o[3];
    for (int d = 0; d < 3; d++) o[d] = (-c[2 * s[d]] + e * c[s[d]] + c[-2 * s[d]] - e * c[-s[d]]) * f[d];
    X(i, j, k) = o[0]; Y(i, j, k) = o[1]; Z(i, j, k) = o[2];
  });
  lc.c.finish();
}

void lsm3dlaplacianorder2local_(R *lap, BOXARG(g), const R *phi, BOXARG(f), DXP, LTAIL) {
  LSETUP("lsm3dlaplacianorder2local_")
  View<R> O = lc.inout(lap, BOXOF(g));
  View<const R> F = lc.in(phi, BOXOF(f));
  g.safe = isect(BOXOF(g), inner(BOXOF(f), 1, 1, 1, 1, 1, 1));
  if (!lc.c.ok()) return;
  const R a = R(1.0) / *dx / *dx, b = R(1.0) / *dy / *dy, e = R(1.0) / *dz / *dz;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R *c = F.p + F.off(i, j, k);
    const long long sy = F.s1, sz = F.s2;
    O(i, j, k) = a * (c[1] - R(2.0) * c[0] + c[-1]) + b * (c[sy] - R(2.0) * c[0] + c[-sy]) +
                 e * (c[sz] - R(2.0) * c[0] + c[-sz]);
  });
  lc.c.finish();
}

// the reference sums serially (spatial_derivatives3d_local.f.in:1143-1164);
// here each block sums its entries and a one-block pass adds the block sums in
// block order: deterministic, and within a few ulps of the serial sum
__global__ void k_avegrad_partial(View<const R> F, Gate g, List L, int lo, int hi, R fx, R fy, R fz,
                                  R *psum, int *pcnt) {
  __shared__ R ss[256];
  __shared__ int sc[256];
  const long long l = (long long)lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  R v = R(0);
  int cnt = 0;
  if (l <= hi) {
    const long long e = l - L.decl;
    const int i = L.ix[e], j = L.iy[e], k = L.iz[e];
    if (g(i, j, k)) {
      const R *c = F.p + F.off(i, j, k);
      const R px = (c[1] - c[-1]) * fx, py = (c[F.s1] - c[-F.s1]) * fy, pz = (c[F.s2] - c[-F.s2]) * fz;
      v = sqrt(px * px + py * py + pz * pz);
      cnt = 1;
    }
  }
  ss[threadIdx.x] = v;
  sc[threadIdx.x] = cnt;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      ss[threadIdx.x] += ss[threadIdx.x + s];
      sc[threadIdx.x] += sc[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    psum[blockIdx.x] = ss[0];
    pcnt[blockIdx.x] = sc[0];
  }
}

__global__ void k_avegrad_final(const R *psum, const int *pcnt, int nb, R *out) {
  __shared__ R ss[1024];
  __shared__ long long sc[1024];
  R v = R(0);
  long long c = 0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    v += psum[b];
    c += pcnt[b];
  }
  ss[threadIdx.x] = v;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      ss[threadIdx.x] += ss[threadIdx.x + s];
      sc[threadIdx.x] += sc[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sc[0] > 0 ? ss[0] / (R)sc[0] : ss[0];
}

void lsm3dcomputeavegradphilocal_(R *grad_phi_ave, const R *phi, BOXARG(f), DXP, LTAIL) {
  LSETUP("lsm3dcomputeavegradphilocal_")
  View<const R> F = lc.in(phi, BOXOF(f));
  g.safe = inner(BOXOF(f), 1, 1, 1, 1, 1, 1);
  R *out = lc.c.scalar_out(grad_phi_ave);
  const long long n = (long long)*nhi - *nlo + 1;
  const int nb = n > 0 ? (int)((n + 255) / 256) : 1;
  R *ps = lc.c.temp<R>(nb);
  int *pc = lc.c.temp<int>(nb);
  if (!lc.c.ok()) return;
  cudaMemsetAsync(ps, 0, sizeof(R) * nb, stream());
  cudaMemsetAsync(pc, 0, sizeof(int) * nb, stream());
  if (n > 0) LSMGPU_LAUNCH(k_avegrad_partial, nb, 256, 0, F, g, L, *nlo, *nhi, R(0.5) / *dx, R(0.5) / *dy, R(0.5) / *dz, ps, pc);
  LSMGPU_LAUNCH(k_avegrad_final, 1, 1024, 0, ps, pc, nb, out);
  lc.c.finish();
}

void lsm3dgradientmagnitudelocal_(const R *phi_x, const R *phi_y, const R *phi_z, R *grad_phi_mag,
                                  BOXARG(g), LTAIL) {
  LSETUP("lsm3dgradientmagnitudelocal_")
  Box gb = BOXOF(g);
  View<const R> X = lc.in(phi_x, gb), Y = lc.in(phi_y, gb), Z = lc.in(phi_z, gb);
  View<R> O = lc.inout(grad_phi_mag, gb);
  g.safe = gb;
  if (!lc.c.ok()) return;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R tol = Consts<R>::zero_tol;
    R x2 = X(i, j, k) * X(i, j, k), y2 = Y(i, j, k) * Y(i, j, k), z2 = Z(i, j, k) * Z(i, j, k);
    if (x2 < tol) x2 = R(0);
    if (y2 < tol) y2 = R(0);
    if (z2 < tol) z2 = R(0);
    const R t = sqrt(x2 + y2 + z2);
    O(i, j, k) = (t < tol) ? R(0) : t;
  });
  lc.c.finish();
}

// ---- RK stages over lists -------------------------------------------------------
static void rk_local(const char *name, int kind, R *out, const Box &ob, const R *a, const Box &ab,
                     const R *u, const Box &ub, const R *rhs, const Box &rb, R dt, IDX3,
                     const int *nlo, const int *nhi, NBARG, const unsigned char *mark_fb) {
  LSETUP(name)
  View<R> O = lc.inout(out, ob);
  View<const R> A = kind ? lc.in(a, ab) : View<const R>{};
  View<const R> U = lc.in(u, ub), Lr = lc.in(rhs, rb);
  g.safe = isect(isect(ob, ub), kind ? isect(rb, ab) : rb);
  if (!lc.c.ok()) return;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R r = Lr(i, j, k);
    if (kind == 0) O(i, j, k) = U(i, j, k) + dt * r;
    else if (kind == 1) O(i, j, k) = R(0.5) * (U(i, j, k) + A(i, j, k) + dt * r);
    else if (kind == 2) O(i, j, k) = R(0.75) * U(i, j, k) + R(0.25) * (A(i, j, k) + dt * r);
    else O(i, j, k) = R(1.0 / 3.0) * U(i, j, k) + R(2.0 / 3.0) * (A(i, j, k) + dt * r);
  });
  lc.c.finish();
}

#define RKL3 R *u_next, BOXARG(a), const R *u_cur, BOXARG(b), const R *rhs, BOXARG(c), const R *dt, LTAIL
#define RKL4 R *u_next, BOXARG(a), const R *u_s, BOXARG(b), const R *u_cur, BOXARG(c), const R *rhs, BOXARG(d), const R *dt, LTAIL
#define LPASS index_x, index_y, index_z, nlo, nhi, narrow_band, nb_ilo, nb_ihi, nb_jlo, nb_jhi, nb_klo, nb_khi, mark_fb

void lsm3drk1steplocal_(RKL3) {
  rk_local("lsm3drk1steplocal_", 0, u_next, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), *dt, LPASS);
}
void lsm3dtvdrk2stage1local_(RKL3) {
  rk_local("lsm3dtvdrk2stage1local_", 0, u_next, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), *dt, LPASS);
}
void lsm3dtvdrk3stage1local_(RKL3) {
  rk_local("lsm3dtvdrk3stage1local_", 0, u_next, BOXOF(a), nullptr, Box{}, u_cur, BOXOF(b), rhs, BOXOF(c), *dt, LPASS);
}
void lsm3dtvdrk2stage2local_(RKL4) {
  rk_local("lsm3dtvdrk2stage2local_", 1, u_next, BOXOF(a), u_s, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), *dt, LPASS);
}
void lsm3dtvdrk3stage2local_(RKL4) {
  rk_local("lsm3dtvdrk3stage2local_", 2, u_next, BOXOF(a), u_s, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), *dt, LPASS);
}
void lsm3dtvdrk3stage3local_(RKL4) {
  rk_local("lsm3dtvdrk3stage3local_", 3, u_next, BOXOF(a), u_s, BOXOF(b), u_cur, BOXOF(c), rhs, BOXOF(d), *dt, LPASS);
}

// ---- LSE right-hand sides over lists ---------------------------------------------
void lsm3dzerooutlevelseteqnrhslocal_(R *lse_rhs, BOXARG(r), IDX3, const int *nlo, const int *nhi) {
  LocalCall lc("lsm3dzerooutlevelseteqnrhslocal_");
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  View<R> O = lc.inout(lse_rhs, BOXOF(r));
  if (!lc.c.ok()) return;
  const Box rb = BOXOF(r);
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (inbox(rb, i, j, k)) O(i, j, k) = R(0);
  });
  lc.c.finish();
}

void lsm3daddadvectiontermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *phi_x, const R *phi_y,
                                         const R *phi_z, BOXARG(g), const R *vel_x, const R *vel_y,
                                         const R *vel_z, BOXARG(v), LTAIL) {
  LSETUP("lsm3daddadvectiontermtolserhslocal_")
  Box gb = BOXOF(g), vb = BOXOF(v);
  View<R> O = lc.inout(lse_rhs, BOXOF(r));
  View<const R> X = lc.in(phi_x, gb), Y = lc.in(phi_y, gb), Z = lc.in(phi_z, gb);
  View<const R> VX = lc.in(vel_x, vb), VY = lc.in(vel_y, vb), VZ = lc.in(vel_z, vb);
  g.safe = isect(BOXOF(r), isect(gb, vb));
  if (!lc.c.ok()) return;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    O(i, j, k) = O(i, j, k) - (VX(i, j, k) * X(i, j, k) + VY(i, j, k) * Y(i, j, k) + VZ(i, j, k) * Z(i, j, k));
  });
  lc.c.finish();
}

static void normal_local(const char *name, R *rhs, const Box &rb, const R *pxp, const R *pyp, const R *pzp,
                         const Box &pb, const R *pxm, const R *pym, const R *pzm, const Box &mb, const R *vn,
                         const Box &vb, bool cst, R vc, IDX3, const int *nlo, const int *nhi, NBARG,
                         const unsigned char *mark_fb) {
  LSETUP(name)
  View<R> O = lc.inout(rhs, rb);
  View<const R> XP = lc.in(pxp, pb), YP = lc.in(pyp, pb), ZP = lc.in(pzp, pb);
  View<const R> XM = lc.in(pxm, mb), YM = lc.in(pym, mb), ZM = lc.in(pzm, mb);
  View<const R> V = cst ? View<const R>{} : lc.in(vn, vb);
  g.safe = isect(rb, isect(pb, cst ? mb : isect(mb, vb)));
  if (!lc.c.ok()) return;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R w = cst ? vc : V(i, j, k);
    const R p[3] = {XP(i, j, k), YP(i, j, k), ZP(i, j, k)}, m[3] = {XM(i, j, k), YM(i, j, k), ZM(i, j, k)};
    const R s = godunov_normal_sq(w > R(0), p, m);
    if (fabs(w) >= Consts<R>::zero_tol) O(i, j, k) = O(i, j, k) - w * sqrt(s);
  });
  lc.c.finish();
}

void lsm3daddnormalveltermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *phi_x_plus, const R *phi_y_plus,
                                         const R *phi_z_plus, BOXARG(p), const R *phi_x_minus,
                                         const R *phi_y_minus, const R *phi_z_minus, BOXARG(m),
                                         const R *vel_n, BOXARG(v), LTAIL) {
  normal_local("lsm3daddnormalveltermtolserhslocal_", lse_rhs, BOXOF(r), phi_x_plus, phi_y_plus, phi_z_plus,
               BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), vel_n, BOXOF(v), false, R(0), LPASS);
}

void lsm3daddconstnormalveltermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *phi_x_plus,
                                              const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                              const R *phi_x_minus, const R *phi_y_minus,
                                              const R *phi_z_minus, BOXARG(m), const R *vel_n, LTAIL) {
  normal_local("lsm3daddconstnormalveltermtolserhslocal_", lse_rhs, BOXOF(r), phi_x_plus, phi_y_plus,
               phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), nullptr, Box{}, true,
               *vel_n, LPASS);
}

void lsm3daddconstcurvtermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *phi_x, const R *phi_y,
                                         const R *phi_z, BOXARG(g), const R *phi_xx, const R *phi_xy,
                                         const R *phi_xz, const R *phi_yy, const R *phi_yz,
                                         const R *phi_zz, BOXARG(h), const R *b, LTAIL) {
  LSETUP("lsm3daddconstcurvtermtolserhslocal_")
  Box gb = BOXOF(g), hb = BOXOF(h);
  View<R> O = lc.inout(lse_rhs, BOXOF(r));
  View<const R> X = lc.in(phi_x, gb), Y = lc.in(phi_y, gb), Z = lc.in(phi_z, gb);
  View<const R> XX = lc.in(phi_xx, hb), XY = lc.in(phi_xy, hb), XZ = lc.in(phi_xz, hb),
                YY = lc.in(phi_yy, hb), YZ = lc.in(phi_yz, hb), ZZ = lc.in(phi_zz, hb);
  g.safe = isect(BOXOF(r), isect(gb, hb));
  if (!lc.c.ok()) return;
  const R bb = *b;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R x = X(i, j, k), y = Y(i, j, k), z = Z(i, j, k);
    const R m2 = x * x + y * y + z * z;
    R curv = R(0);
    if (!(m2 < Consts<R>::zero_tol))
      curv = curv_numerator(XX(i, j, k), YY(i, j, k), ZZ(i, j, k), XY(i, j, k), XZ(i, j, k), YZ(i, j, k), x, y, z) / m2;
    O(i, j, k) = O(i, j, k) + bb * curv;
  });
  lc.c.finish();
}

void lsm3dcomputereinitializationeqnrhslocal_(R *reinit_rhs, BOXARG(r), const R *phi, BOXARG(f),
                                              const R *phi0, BOXARG(z), const R *phi_x_plus,
                                              const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                              const R *phi_x_minus, const R *phi_y_minus,
                                              const R *phi_z_minus, BOXARG(m), DXP,
                                              const int *use_phi0_for_sgn, LTAIL) {
  LSETUP("lsm3dcomputereinitializationeqnrhslocal_")
  const bool use0 = (*use_phi0_for_sgn == 1);
  Box pb = BOXOF(p), mb = BOXOF(m);
  View<R> O = lc.inout(reinit_rhs, BOXOF(r));
  View<const R> PH = use0 ? View<const R>{} : lc.in(phi, BOXOF(f));
  View<const R> P0 = use0 ? lc.in(phi0, BOXOF(z)) : View<const R>{};
  View<const R> XP = lc.in(phi_x_plus, pb), YP = lc.in(phi_y_plus, pb), ZP = lc.in(phi_z_plus, pb);
  View<const R> XM = lc.in(phi_x_minus, mb), YM = lc.in(phi_y_minus, mb), ZM = lc.in(phi_z_minus, mb);
  g.safe = isect(isect(BOXOF(r), use0 ? BOXOF(z) : BOXOF(f)), isect(pb, mb));
  if (!lc.c.ok()) return;
  R dx_sq = rmax(rmax(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R pc = use0 ? P0(i, j, k) : PH(i, j, k);
    const R gp[3] = {XP(i, j, k), YP(i, j, k), ZP(i, j, k)}, gm[3] = {XM(i, j, k), YM(i, j, k), ZM(i, j, k)};
    O(i, j, k) = lsmgpu::reinit_rhs<R>(pc, gp, gm, dx_sq, use0);
  });
  lc.c.finish();
}

void lsm3dcomputemeancurvatureorder2local_(R *kappa, BOXARG(k), const R *phi, BOXARG(f), const R *phi_x,
                                           const R *phi_y, const R *phi_z, const R *grad_phi_mag,
                                           BOXARG(g), DXP, LTAIL) {
  LSETUP("lsm3dcomputemeancurvatureorder2local_")
  Box gb = BOXOF(g);
  View<R> K = lc.inout(kappa, BOXOF(k));
  View<const R> F = lc.in(phi, BOXOF(f));
  View<const R> X = lc.in(phi_x, gb), Y = lc.in(phi_y, gb), Z = lc.in(phi_z, gb), G = lc.in(grad_phi_mag, gb);
  g.safe = isect(isect(BOXOF(k), gb), inner(BOXOF(f), 1, 1, 1, 1, 1, 1));
  if (!lc.c.ok()) return;
  const R dxv = *dx, dyv = *dy, dzv = *dz;
  const R fxx = R(1.0) / dxv / dxv, fyy = R(1.0) / dyv / dyv, fzz = R(1.0) / dzv / dzv;
  const R fxy = R(0.25) / dxv / dyv, fxz = R(0.25) / dxv / dzv, fyz = R(0.25) / dyv / dzv;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R *c = F.p + F.off(i, j, k);
    const long long sx = 1, sy = F.s1, sz = F.s2;
    const R xx = (c[sx] - R(2.0) * c[0] + c[-sx]) * fxx;
    const R yy = (c[sy] - R(2.0) * c[0] + c[-sy]) * fyy;
    const R zz = (c[sz] - R(2.0) * c[0] + c[-sz]) * fzz;
    const R xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * fxy;
    const R xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * fxz;
    const R yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * fyz;
    const R gg = G(i, j, k);
    const R den = gg * gg * gg;
    K(i, j, k) = (den < Consts<R>::zero_tol)
                     ? R(0)
                     : curv_numerator(xx, yy, zz, xy, xz, yz, X(i, j, k), Y(i, j, k), Z(i, j, k)) / den;
  });
  lc.c.finish();
}

#define CURVL_ARGS                                                                                        \
  R *kappa, BOXARG(k), const R *phi, BOXARG(f), const R *phi_x, const R *phi_y, const R *phi_z,         \
      const R *grad_phi_mag, BOXARG(g), DXP, LTAIL
#define CURVL_PASS                                                                                        \
  kappa, BOXOF(k), phi, BOXOF(f), phi_x, phi_y, phi_z, grad_phi_mag, BOXOF(g), *dx, *dy, *dz, index_x, index_y, \
      index_z, nlo, nhi, narrow_band, BOXOF(nb), mark_fb

void lsm3dcomputegaussiancurvatureorder2local_(CURVL_ARGS) {
  curv_variant_local<CURV_GAUSS2>("lsm3dcomputegaussiancurvatureorder2local_", CURVL_PASS);
}
void lsm3dcomputemeancurvatureorder4local_(CURVL_ARGS) {
  curv_variant_local<CURV_GAUSS4>("lsm3dcomputemeancurvatureorder4local_", CURVL_PASS);
}
void lsm3dcomputegaussiancurvatureorder4local_(CURVL_ARGS) {
  curv_variant_local<CURV_GAUSS4>("lsm3dcomputegaussiancurvatureorder4local_", CURVL_PASS);
}
void lsmgpu_mean_curvature_order4_local(CURVL_ARGS) {
  curv_variant_local<CURV_MEAN4>("lsmgpu_mean_curvature_order4_local", CURVL_PASS);
}

// rhs += b * kappa * |grad phi| on listed cells
// (level_set_evolution3d_local.f.in:530-607)
void lsm3daddconstprecomputedcurvtermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *kappa, BOXARG(k),
                                                    const R *grad_phi_mag, BOXARG(g), const R *b, LTAIL) {
  LSETUP("lsm3daddconstprecomputedcurvtermtolserhslocal_")
  View<R> O = lc.inout(lse_rhs, BOXOF(r));
  View<const R> KA = lc.in(kappa, BOXOF(k)), G = lc.in(grad_phi_mag, BOXOF(g));
  g.safe = isect(BOXOF(r), isect(BOXOF(k), BOXOF(g)));
  if (!lc.c.ok()) return;
  const R bb = *b;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    O(i, j, k) = O(i, j, k) + bb * KA(i, j, k) * G(i, j, k);
  });
  lc.c.finish();
}

// rhs -= u . grad(phi) + Vn |grad phi| with the combined Godunov selection on
// listed cells (level_set_evolution3d_local.f.in:612-812)
void lsm3daddexternalandnormalveltermtolserhslocal_(R *lse_rhs, BOXARG(r), const R *phi_x_plus,
                                                    const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                                    const R *phi_x_minus, const R *phi_y_minus,
                                                    const R *phi_z_minus, BOXARG(m), const R *vel_n,
                                                    const R *vel_x, const R *vel_y, const R *vel_z, BOXARG(v),
                                                    LTAIL) {
  LSETUP("lsm3daddexternalandnormalveltermtolserhslocal_")
  Box pb = BOXOF(p), mb = BOXOF(m), vb = BOXOF(v);
  View<R> O = lc.inout(lse_rhs, BOXOF(r));
  View<const R> XP = lc.in(phi_x_plus, pb), YP = lc.in(phi_y_plus, pb), ZP = lc.in(phi_z_plus, pb);
  View<const R> XM = lc.in(phi_x_minus, mb), YM = lc.in(phi_y_minus, mb), ZM = lc.in(phi_z_minus, mb);
  View<const R> VN = lc.in(vel_n, vb), VX = lc.in(vel_x, vb), VY = lc.in(vel_y, vb), VZ = lc.in(vel_z, vb);
  g.safe = isect(isect(BOXOF(r), vb), isect(pb, mb));
  if (!lc.c.ok()) return;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R w = VN(i, j, k), ux = VX(i, j, k), uy = VY(i, j, k), uz = VZ(i, j, k);
    const R gx = ext_pick<R>(ux, w, XP(i, j, k), XM(i, j, k));
    const R gy = ext_pick<R>(uy, w, YP(i, j, k), YM(i, j, k));
    const R gz = ext_pick<R>(uz, w, ZP(i, j, k), ZM(i, j, k));
    const R n2 = gx * gx + gy * gy + gz * gz;
    if (fabs(w) >= Consts<R>::zero_tol && n2 >= Consts<R>::zero_tol)
      O(i, j, k) = O(i, j, k) - ux * gx - uy * gy - uz * gz - w * sqrt(n2);
    else
      O(i, j, k) = O(i, j, k) - ux * gx - uy * gy - uz * gz;
  });
  lc.c.finish();
}

#define ORTHOL_ARGS                                                                                      \
  R *ortho_rhs, BOXARG(r), const R *phi_x_plus, const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),     \
      const R *phi_x_minus, const R *phi_y_minus, const R *phi_z_minus, BOXARG(m), const R *psi, BOXARG(s), \
      const R *psi_x_plus, const R *psi_y_plus, const R *psi_z_plus, BOXARG(sp), const R *psi_x_minus,    \
      const R *psi_y_minus, const R *psi_z_minus, BOXARG(sm), DXP, LTAIL
#define ORTHOL_PASS                                                                                      \
  ortho_rhs, BOXOF(r), phi_x_plus, phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, \
      BOXOF(m), psi, BOXOF(s), psi_x_plus, psi_y_plus, psi_z_plus, BOXOF(sp), psi_x_minus, psi_y_minus,    \
      psi_z_minus, BOXOF(sm), *dx, *dy, *dz, index_x, index_y, index_z, nlo, nhi, narrow_band, BOXOF(nb),  \
      mark_fb

void lsm3dcomputeorthogonalizationeqnrhslocal_(ORTHOL_ARGS) {
  ortho_local<true>("lsm3dcomputeorthogonalizationeqnrhslocal_", ORTHOL_PASS);
}
void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local(ORTHOL_ARGS) {
  ortho_local<false>("lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local", ORTHOL_PASS);
}

}  // extern "C"

// ---- reductions over lists ----------------------------------------------------
// mode 0: advection dt, 1: normal velocity dt (skips norm_grad_phi <= tol),
// 2: constant normal velocity dt, 3: max |f1 - f2|
// cv_sgn != 0 (control-volume variants, math_utils3d_local.f.in:98, :432):
// take a cell only when control_vol > 0 (cv_sgn > 0) or < 0 (cv_sgn < 0)
struct LRed {
  View<const R> a, b, c, xp, yp, zp, xm, ym, zm, vn, cv;
  int cv_sgn;
  R vc, ix, iy, iz, mdx2;
};

template <int MODE>
__global__ void k_list_max(LRed A, Gate g, List L, int lo, int hi, unsigned long long *key) {
  const long long l = (long long)lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  R v = R(-1.0e308);
  if (l <= hi) {
    const long long e = l - L.decl;
    const int i = L.ix[e], j = L.iy[e], k = L.iz[e];
    bool take = g(i, j, k);
    if (take && A.cv_sgn != 0) take = A.cv_sgn > 0 ? A.cv(i, j, k) > R(0) : A.cv(i, j, k) < R(0);
    if (take) {
      if (MODE == 0) {
        v = fabs(A.a(i, j, k)) * A.ix + fabs(A.b(i, j, k)) * A.iy + fabs(A.c(i, j, k)) * A.iz;
      } else if (MODE == 3) {
        v = fabs(A.a(i, j, k) - A.b(i, j, k));
      } else {
        const R cx = rmax(fabs(A.xp(i, j, k)), fabs(A.xm(i, j, k)));
        const R cy = rmax(fabs(A.yp(i, j, k)), fabs(A.ym(i, j, k)));
        const R cz = rmax(fabs(A.zp(i, j, k)), fabs(A.zm(i, j, k)));
        const R ng = sqrt(cx * cx + cy * cy + cz * cz + A.mdx2);
        const R avn = MODE == 2 ? fabs(A.vc) : fabs(A.vn(i, j, k));
        if (MODE == 2 || ng > Consts<R>::zero_tol) v = avn / ng * (cx * A.ix + cy * A.iy + cz * A.iz);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) v = rmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(key, okey(v));
}

template <int MODE>
static void list_max(LocalCall &lc, LRed &A, Gate g, List L, int lo, int hi, R *out, R init, int result_mode,
                     R cfl) {
  unsigned long long *key = lc.c.temp<unsigned long long>(1);
  R *dout = lc.c.scalar_out(out);
  if (!lc.c.ok()) return;
  LSMGPU_LAUNCH(k_init_key, 1, 1, 0, key, init);
  if (hi >= lo) {
    const long long n = (long long)hi - lo + 1;
    LSMGPU_LAUNCH(k_list_max<MODE>, (unsigned)((n + 255) / 256), 256, 0, A, g, L, lo, hi, key);
  }
  LSMGPU_LAUNCH(k_key_result, 1, 1, 0, key, dout, result_mode, cfl);
  lc.c.finish();
}

extern "C" {

void lsm3dmaxnormdifflocal_(R *max_norm_diff, const R *field1, BOXARG(a), const R *field2, BOXARG(b), LTAIL) {
  LSETUP("lsm3dmaxnormdifflocal_")
  LRed A{};
  A.a = lc.in(field1, BOXOF(a));
  A.b = lc.in(field2, BOXOF(b));
  g.safe = isect(BOXOF(a), BOXOF(b));
  list_max<3>(lc, A, g, L, *nlo, *nhi, max_norm_diff, R(0.0), 1, R(0));  // starts at 0 (:72)
}

void lsm3dcomputestableadvectiondtlocal_(R *dt, const R *vel_x, const R *vel_y, const R *vel_z, BOXARG(v),
                                         DXP, const R *cfl_number, LTAIL) {
  LSETUP("lsm3dcomputestableadvectiondtlocal_")
  Box vb = BOXOF(v);
  LRed A{};
  A.a = lc.in(vel_x, vb); A.b = lc.in(vel_y, vb); A.c = lc.in(vel_z, vb);
  g.safe = vb;
  A.ix = R(1.0) / *dx; A.iy = R(1.0) / *dy; A.iz = R(1.0) / *dz;
  list_max<0>(lc, A, g, L, *nlo, *nhi, dt, R(-1.0), 0, *cfl_number);
}

}  // extern "C"

static void normal_dt_local(const char *name, int mode, R *dt, const R *vn, const Box &vb, R vc,
                            const R *pxp, const R *pyp, const R *pzp, const Box &pb, const R *pxm,
                            const R *pym, const R *pzm, const Box &mb, R dx, R dy, R dz, R cfl,
                            bool max3, IDX3, const int *nlo, const int *nhi, NBARG,
                            const unsigned char *mark_fb) {
  LSETUP(name)
  LRed A{};
  A.xp = lc.in(pxp, pb); A.yp = lc.in(pyp, pb); A.zp = lc.in(pzp, pb);
  A.xm = lc.in(pxm, mb); A.ym = lc.in(pym, mb); A.zm = lc.in(pzm, mb);
  if (mode == 1) A.vn = lc.in(vn, vb);
  g.safe = isect(isect(pb, mb), mode == 1 ? vb : pb);
  A.vc = vc;
  A.ix = R(1.0) / dx; A.iy = R(1.0) / dy; A.iz = R(1.0) / dz;
  R mx = max3 ? rmax(rmax(dx, dy), dz) : rmax(rmax(dx, dy), dz);
  A.mdx2 = mx * mx;
  if (mode == 1)
    list_max<1>(lc, A, g, L, *nlo, *nhi, dt, R(-1.0), 0, cfl);
  else
    list_max<2>(lc, A, g, L, *nlo, *nhi, dt, R(-1.0), 0, cfl);
}

extern "C" {

void lsm3dcomputestablenormalveldtlocal_(R *dt, const R *vel_n, BOXARG(v), const R *phi_x_plus,
                                         const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                         const R *phi_x_minus, const R *phi_y_minus, const R *phi_z_minus,
                                         BOXARG(m), DXP, const R *cfl_number, LTAIL) {
  normal_dt_local("lsm3dcomputestablenormalveldtlocal_", 1, dt, vel_n, BOXOF(v), R(0), phi_x_plus, phi_y_plus,
                  phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), *dx, *dy, *dz,
                  *cfl_number, true, LPASS);
}

// starts at 0 and takes listed cells with a negative control volume: the
// routine has no control_vol_sgn argument (math_utils3d_local.f.in:98-190)
void lsm3dmaxnormdiffcontrolvolumelocal_(R *max_norm_diff, const R *field1, BOXARG(a), const R *field2,
                                         BOXARG(b), const R *control_vol, BOXARG(c), LTAIL) {
  LSETUP("lsm3dmaxnormdiffcontrolvolumelocal_")
  LRed A{};
  A.a = lc.in(field1, BOXOF(a));
  A.b = lc.in(field2, BOXOF(b));
  A.cv = lc.in(control_vol, BOXOF(c));
  A.cv_sgn = -1;
  g.safe = isect(isect(BOXOF(a), BOXOF(b)), BOXOF(c));
  list_max<3>(lc, A, g, L, *nlo, *nhi, max_norm_diff, R(0.0), 1, R(0));
}

// math_utils3d_local.f.in:432-624 (norm_grad_phi <= zero_tol skipped, :138)
void lsm3dcomputestablenormalveldtcontrolvolumelocal_(R *dt, const R *vel_n, BOXARG(v), const R *phi_x_plus,
                                                      const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                                      const R *phi_x_minus, const R *phi_y_minus,
                                                      const R *phi_z_minus, BOXARG(m), const R *control_vol,
                                                      BOXARG(c), const int *control_vol_sgn, DXP,
                                                      const R *cfl_number, LTAIL) {
  LSETUP("lsm3dcomputestablenormalveldtcontrolvolumelocal_")
  const Box vb = BOXOF(v), pb = BOXOF(p), mb = BOXOF(m), cb = BOXOF(c);
  LRed A{};
  A.xp = lc.in(phi_x_plus, pb); A.yp = lc.in(phi_y_plus, pb); A.zp = lc.in(phi_z_plus, pb);
  A.xm = lc.in(phi_x_minus, mb); A.ym = lc.in(phi_y_minus, mb); A.zm = lc.in(phi_z_minus, mb);
  A.vn = lc.in(vel_n, vb);
  A.cv = lc.in(control_vol, cb);
  A.cv_sgn = *control_vol_sgn > 0 ? 1 : -1;
  g.safe = isect(isect(isect(pb, mb), vb), cb);
  A.ix = R(1.0) / *dx; A.iy = R(1.0) / *dy; A.iz = R(1.0) / *dz;
  const R mx = rmax(rmax(*dx, *dy), *dz);
  A.mdx2 = mx * mx;
  list_max<1>(lc, A, g, L, *nlo, *nhi, dt, R(-1.0), 0, *cfl_number);
}

// LSMLIB's routine (math_utils3d_local.f.in:628-752) reads two unassigned
// locals; this computes the dense routine's formula over the listed cells
void lsm3dcomputestableconstnormalveldtlocal_(R *dt, const R *vel_n, const R *phi_x_plus,
                                              const R *phi_y_plus, const R *phi_z_plus, BOXARG(p),
                                              const R *phi_x_minus, const R *phi_y_minus,
                                              const R *phi_z_minus, BOXARG(m), DXP, const R *cfl_number,
                                              LTAIL) {
  normal_dt_local("lsm3dcomputestableconstnormalveldtlocal_", 2, dt, nullptr, Box{}, *vel_n, phi_x_plus,
                  phi_y_plus, phi_z_plus, BOXOF(p), phi_x_minus, phi_y_minus, phi_z_minus, BOXOF(m), *dx, *dy,
                  *dz, *cfl_number, false, LPASS);
}

// ---- list utilities (localization3d.f) -------------------------------------------
void lsm3dmultiplycutofflserhslocal_(const R *phi, R *lse_rhs, BOXARG(g), LTAIL, const R *beta, const R *gamma) {
  LSETUP("lsm3dmultiplycutofflserhslocal_")
  Box gb = BOXOF(g);
  View<const R> F = lc.in(phi, gb);
  View<R> O = lc.inout(lse_rhs, gb);
  g.safe = gb;
  if (!lc.c.ok()) return;
  const R bt = *beta, gm = *gamma;
  const R c1 = gm - 3 * bt;
  R c2 = (gm - bt);
  c2 = c2 * c2 * c2;
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (!g(i, j, k)) return;
    const R a = fabs(F(i, j, k));
    R co;
    if (a <= bt) {
      co = R(1);
    } else if (a <= gm) {
      const R t = a - gm;
      co = (t * t * (2 * a + c1)) / c2;
    } else {
      co = R(0);
    }
    O(i, j, k) = co * O(i, j, k);
  });
  lc.c.finish();
}

void lsm3dimposemasklocal_(R *dest, BOXARG(d), const R *src, BOXARG(s), const R *mask, BOXARG(m), IDX3,
                           const int *nlo, const int *nhi) {
  LocalCall lc("lsm3dimposemasklocal_");
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  View<R> D = lc.inout(dest, BOXOF(d));
  View<const R> S = lc.in(src, BOXOF(s)), M = lc.in(mask, BOXOF(m));
  if (!lc.c.ok()) return;
  const Box sb = isect(BOXOF(d), isect(BOXOF(s), BOXOF(m)));
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (inbox(sb, i, j, k)) D(i, j, k) = rmax(M(i, j, k), S(i, j, k));
  });
  lc.c.finish();
}

void lsm3dcopydatalocal_(R *dest, BOXARG(d), const R *src, BOXARG(s), IDX3, const int *nlo, const int *nhi) {
  LocalCall lc("lsm3dcopydatalocal_");
  List L = lc.list(index_x, index_y, index_z, *nlo, *nhi);
  View<R> D = lc.inout(dest, BOXOF(d));
  View<const R> S = lc.in(src, BOXOF(s));
  if (!lc.c.ok()) return;
  const Box sb = isect(BOXOF(d), BOXOF(s));
  for_list(L, *nlo, *nhi, [=] __device__(int i, int j, int k) {
    if (inbox(sb, i, j, k)) D(i, j, k) = S(i, j, k);
  });
  lc.c.finish();
}

}  // extern "C"
