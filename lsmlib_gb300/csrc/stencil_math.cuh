// Per-cell stencil arithmetic shared by the drop-in kernels and the fused
// stage kernels.
//
// Every routine here evaluates one LSMLIB formula on values already in
// registers, with the operations in the order LSMLIB's Fortran performs them:
// translation units that include this header for the FP64 parity form are
// compiled with -fmad=false, so each product and sum rounds exactly as the
// reference's does and the results are bit-identical to it.
//
// Index convention (LSMLIB spatial_derivatives3d.f.in:19-45): the first
// undivided difference D1(i) = phi(i) - phi(i-1) sits on the face between
// cells i-1 and i.  For a cell c, `a[m]` holds phi(c + m - 3), m = 0..6, so
// D1(c+f) = a[f+3] - a[f+2].
#pragma once

namespace lsmgpu {

template <class R>
__host__ __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <class R>
__host__ __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }

// LSMLIB template constants for the FP64 build (src/CMakeLists.txt:10-20).
template <class R> struct Consts;
template <> struct Consts<double> {
  static constexpr double zero_tol = 1.e-11;
  static constexpr double tiny = 1.e-36;
};
template <> struct Consts<float> {
  static constexpr float zero_tol = 1.e-5f;
  static constexpr float tiny = 1.e-36f;
};

// Undivided differences around one cell along one axis.
template <class R>
struct Diffs {
  R d1[6];  // D1(c+f), f = -2..3
  R d2[5];  // D2(c+f), f = -2..2
  R d3[4];  // D3(c+f), f = -1..2
  __device__ __forceinline__ R D1(int f) const { return d1[f + 2]; }
  __device__ __forceinline__ R D2(int f) const { return d2[f + 2]; }
  __device__ __forceinline__ R D3(int f) const { return d3[f + 1]; }
};

// order: 1 (D1 only), 2 (D1, D2), 3 (D1, D2, D3).  lsm3dComputeDn
// (spatial_derivatives3d.f.in:49-176): odd n subtracts the left neighbour,
// even n negates (Dn-1(i) - Dn-1(i+1)), which equals Dn-1(i+1) - Dn-1(i)
// exactly.
template <class R, int ORDER>
__device__ __forceinline__ void make_diffs(Diffs<R> &d, const R a[7]) {
#pragma unroll
  for (int f = -2; f <= 3; f++) d.d1[f + 2] = a[f + 3] - a[f + 2];
  if (ORDER >= 2) {
#pragma unroll
    for (int f = -2; f <= 2; f++) d.d2[f + 2] = d.d1[f + 3] - d.d1[f + 2];
  }
  if (ORDER >= 3) {
#pragma unroll
    for (int f = -1; f <= 2; f++) d.d3[f + 1] = d.d2[f + 2] - d.d2[f + 1];
  }
}

// ENO1 (spatial_derivatives3d.f.in:299-300)
template <class R> __device__ __forceinline__ R eno1_plus(const Diffs<R> &d, R inv) { return d.D1(1) * inv; }
template <class R> __device__ __forceinline__ R eno1_minus(const Diffs<R> &d, R inv) { return d.D1(0) * inv; }

// ENO2 (spatial_derivatives3d.f.in:520-535)
template <class R>
__device__ __forceinline__ R eno2_plus(const Diffs<R> &d, R inv) {
  const R h = R(0.5);
  R c = (fabs(d.D2(0)) < fabs(d.D2(1))) ? d.D2(0) : d.D2(1);
  return (d.D1(1) - h * c) * inv;
}
template <class R>
__device__ __forceinline__ R eno2_minus(const Diffs<R> &d, R inv) {
  const R h = R(0.5);
  R c = (fabs(d.D2(-1)) < fabs(d.D2(0))) ? d.D2(-1) : d.D2(0);
  return (d.D1(0) + h * c) * inv;
}

// ENO3 (spatial_derivatives3d.f.in:842-896)
template <class R>
__device__ __forceinline__ R eno3_plus(const Diffs<R> &d, R inv) {
  const R third = R(1.0 / 3.0), sixth = R(1.0 / 6.0), h = R(0.5);
  R x = d.D1(1);
  if (fabs(d.D2(0)) < fabs(d.D2(1))) {
    x = x - h * d.D2(0);
    R c = (fabs(d.D3(0)) < fabs(d.D3(1))) ? d.D3(0) : d.D3(1);
    x = x - sixth * c;
  } else {
    x = x - h * d.D2(1);
    R c = (fabs(d.D3(1)) < fabs(d.D3(2))) ? d.D3(1) : d.D3(2);
    x = x + third * c;
  }
  return x * inv;
}
template <class R>
__device__ __forceinline__ R eno3_minus(const Diffs<R> &d, R inv) {
  const R third = R(1.0 / 3.0), sixth = R(1.0 / 6.0), h = R(0.5);
  R x = d.D1(0);
  if (fabs(d.D2(-1)) < fabs(d.D2(0))) {
    x = x + h * d.D2(-1);
    R c = (fabs(d.D3(-1)) < fabs(d.D3(0))) ? d.D3(-1) : d.D3(0);
    x = x + third * c;
  } else {
    x = x + h * d.D2(0);
    R c = (fabs(d.D3(0)) < fabs(d.D3(1))) ? d.D3(0) : d.D3(1);
    x = x - sixth * c;
  }
  return x * inv;
}

// WENO5-JS on five scaled first differences, in the exact form of
// spatial_derivatives3d.f.in:1296-1323 (parity form).
template <class R>
__device__ __forceinline__ R weno5_exact(R v1, R v2, R v3, R v4, R v5) {
  const R c13 = R(1.0 / 3.0), c76 = R(7.0 / 6.0), c116 = R(11.0 / 6.0);
  const R c16 = R(1.0 / 6.0), c56 = R(5.0 / 6.0), c1312 = R(13.0 / 12.0);
  const R c14 = R(0.25);
  R m = v1 * v1;
  m = rmax(m, v2 * v2);
  m = rmax(m, v3 * v3);
  m = rmax(m, v4 * v4);
  m = rmax(m, v5 * v5);
  const R eps = R(1e-6) * m + Consts<R>::tiny;
  const R p1 = c13 * v1 - c76 * v2 + c116 * v3;
  const R p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  const R p3 = c13 * v3 + c56 * v4 - c16 * v5;
  R t = v1 - R(2.0) * v2 + v3;
  R u = v1 - R(4.0) * v2 + R(3.0) * v3;
  const R S1 = c1312 * (t * t) + c14 * (u * u);
  t = v2 - R(2.0) * v3 + v4;
  u = v2 - v4;
  const R S2 = c1312 * (t * t) + c14 * (u * u);
  t = v3 - R(2.0) * v4 + v5;
  u = R(3.0) * v3 - R(4.0) * v4 + v5;
  const R S3 = c1312 * (t * t) + c14 * (u * u);
  R a1 = R(0.1) / ((S1 + eps) * (S1 + eps));
  R a2 = R(0.6) / ((S2 + eps) * (S2 + eps));
  R a3 = R(0.3) / ((S3 + eps) * (S3 + eps));
  const R inv_sum = R(1.0) / (a1 + a2 + a3);
  a1 = a1 * inv_sum;
  a2 = a2 * inv_sum;
  a3 = a3 * inv_sum;
  return a1 * p1 + a2 * p2 + a3 * p3;
}

// plus side: v = D1(c+3..c-1); minus side: v = D1(c-2..c+2)
// (spatial_derivatives3d.f.in:1286-1367)
template <class R>
__device__ __forceinline__ R weno5_plus(const Diffs<R> &d, R inv) {
  return weno5_exact<R>(d.D1(3) * inv, d.D1(2) * inv, d.D1(1) * inv, d.D1(0) * inv, d.D1(-1) * inv);
}
template <class R>
__device__ __forceinline__ R weno5_minus(const Diffs<R> &d, R inv) {
  return weno5_exact<R>(d.D1(-2) * inv, d.D1(-1) * inv, d.D1(0) * inv, d.D1(1) * inv, d.D1(2) * inv);
}

// Godunov |grad phi|^2 of level_set_evolution3d.f.in:210-223 for normal
// speed sign `pos` (vn > 0).
template <class R>
__device__ __forceinline__ R godunov_normal_sq(bool pos, const R p[3], const R m[3]) {
  R s = R(0);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    R a, b;
    if (pos) {
      a = rmax(m[d], R(0));
      b = rmin(p[d], R(0));
    } else {
      a = rmin(m[d], R(0));
      b = rmax(p[d], R(0));
    }
    const R t = rmax(a * a, b * b);
    s = (d == 0) ? t : s + t;
  }
  return s;
}

// Reinitialization right-hand side of reinitialization3d.f.in:159-199 (Peng
// form, use0 = false) and :217-256 (phi0 form, use0 = true).  `pc` is phi
// (or phi0) at the cell.
template <class R>
__device__ __forceinline__ R reinit_rhs(R pc, const R gp[3], const R gm[3], R dx_sq, bool use0) {
  R st[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    R u, w;
    if (pc > R(0)) {
      u = rmax(-gp[d], R(0));
      w = rmax(gm[d], R(0));
    } else {
      u = rmax(gp[d], R(0));
      w = rmax(-gm[d], R(0));
    }
    st[d] = rmax(u, w);
  }
  if (!(fabs(pc) >= Consts<R>::zero_tol)) return R(0);
  const R n2 = st[0] * st[0] + st[1] * st[1] + st[2] * st[2];
  const R sgn = use0 ? pc / sqrt(pc * pc + dx_sq) : pc / sqrt(pc * pc + n2 * dx_sq);
  return sgn * (R(1.0) - sqrt(n2));
}

// Curvature numerator in the term order of curvature3d.f.in:109-117.
template <class R>
__device__ __forceinline__ R curv_numerator(R xx, R yy, R zz, R xy, R xz, R yz, R x, R y, R z) {
  return xx * y * y + yy * x * x - R(2) * xy * x * y + xx * z * z + zz * x * x - R(2) * xz * x * z +
         yy * z * z + zz * y * y - R(2) * yz * y * z;
}

// one axis of the combined external + normal velocity Godunov selection
// (level_set_evolution3d.f.in:630-649, level_set_evolution3d_local.f.in:714-787)
template <class R>
__device__ __forceinline__ R ext_pick(R v, R vn, R p, R m) {
  const R hp = v + vn * p, hm = v + vn * m;
  if (hp > R(0)) return (hm > R(0)) ? m : -v / vn;
  if (hm < R(0)) return p;
  return (fabs(hp) > fabs(hm)) ? p : m;
}

// ---- orthogonalization and subcell fix (reinitialization3d.f.in:296-757) --------
// orthogonalization RHS at one cell: upwinding of grad(phi) along
// sgn(psi) grad(psi*), grad(psi*) the average of the plus and minus
// derivatives of psi (reinitialization3d.f.in:380-425)
// GRAD_SMOOTH: sgn(psi) = psi / sqrt(psi^2 + dx_sq |grad psi*|^2) as the 3D
// routine smooths it (reinitialization3d.f.in:439); otherwise
// psi / sqrt(psi^2 + dx_sq), the 2D routine's form (reinitialization2d.f.in:360)
template <class R, bool GRAD_SMOOTH = true>
__device__ __forceinline__ R ortho_rhs(R psi, const R psp[3], const R psm[3], const R pp[3], const R pm[3],
                                       R dx_sq) {
  R g[3];
  for (int d = 0; d < 3; d++) g[d] = R(0.5) * (psp[d] + psm[d]);
  R n = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  n = sqrt(n);
  if (!(fabs(psi) > Consts<R>::zero_tol && n > Consts<R>::zero_tol)) return R(0);
  const R s = GRAD_SMOOTH ? psi / sqrt(psi * psi + dx_sq * (n * n)) : psi / sqrt(psi * psi + dx_sq);
  R t = rmax(s * g[0], R(0)) * pm[0];
  t = t + rmin(s * g[0], R(0)) * pp[0];
  t = t + rmax(s * g[1], R(0)) * pm[1];
  t = t + rmin(s * g[1], R(0)) * pp[1];
  t = t + rmax(s * g[2], R(0)) * pm[2];
  t = t + rmin(s * g[2], R(0)) * pp[2];
  return -(R(1.0) / n * t);
}

// signed distance estimate near the interface for the subcell fix
// (Russo-Smereka): `flag` away from sign changes, else phi0 over the largest
// one-sided or central difference.  HALF_CENTRAL is the 3D routine's form
// (reinitialization3d.f.in:520-569: sign changes by comparisons, half the
// central difference, phi0 / delta); otherwise the 2D routine's
// (reinitialization2d.f.in:425-460: sign changes by negative products, the
// full central difference, 2 phi0 / delta)
template <class R, bool HALF_CENTRAL = true>
__device__ __forceinline__ R subcell_distance(const R *c, const long long s[3], R flag) {
  const R p = c[0], z = R(0);
  bool near = false;
  for (int d = 0; d < 3; d++) {
    const R a = c[s[d]], b = c[-s[d]];
    if (HALF_CENTRAL)
      near = near || (a > z && p <= z) || (a <= z && p > z) || (b > z && p <= z) || (b <= z && p > z);
    else
      near = near || (a * p < z) || (b * p < z);
  }
  if (!near) return flag;
  R delta = Consts<R>::zero_tol;
  for (int d = 0; d < 3; d++) {
    const R a = c[s[d]], b = c[-s[d]];
    const R central = HALF_CENTRAL ? fabs(a - b) / R(2.0) : fabs(a - b);
    const R m = rmax(rmax(central, fabs(a - p)), fabs(p - b));
    delta = rmax(m, delta);
  }
  return HALF_CENTRAL ? p / delta : R(2.0) * p / delta;
}

// first-order reinitialization RHS with the subcell fix
// (reinitialization3d.f.in:660-745)
template <class R>
__device__ __forceinline__ R subcell_rhs(R pc, R p0, R dist, const R gp[3], const R gm[3], R flag, R max_dx) {
  const R sgn0 = (fabs(p0) > Consts<R>::zero_tol) ? copysign(R(1.0), p0) : R(0);
  if (!(dist == flag)) return dist - sgn0 * fabs(pc) / max_dx;
  R st[3];
  for (int d = 0; d < 3; d++) {
    R u, w;
    if (pc > R(0)) {
      u = rmax(-gp[d], R(0));
      w = rmax(gm[d], R(0));
    } else {
      u = rmax(gp[d], R(0));
      w = rmax(-gm[d], R(0));
    }
    st[d] = rmax(u, w);
  }
  if (!(fabs(pc) > Consts<R>::zero_tol)) return R(0);
  const R n2 = st[0] * st[0] + st[1] * st[1] + st[2] * st[2];
  return sgn0 - sgn0 * sqrt(n2);
}

// ---- curvature variants (curvature3d.f.in:136-508, curvature3d_local.f.in:151-574)
enum CurvKind { CURV_GAUSS2 = 1, CURV_MEAN4 = 2, CURV_GAUSS4 = 3 };

// order 2: f = {1/dx^2, 1/dy^2, 1/dz^2, 1/(4 dx dy), 1/(4 dx dz), 1/(4 dy dz)};
// order 4: f = {1/(12 dx^2), 1/(12 dy^2), 1/(12 dz^2), 1/(12 dx), 1/(12 dy), 1/(12 dz)}
template <class R>
struct CurvFactors {
  R f[6];
};

// kappa at cell (i, j, k): c points at phi there (strides sy, sz), x, y, z
// and gm the first derivatives and |grad phi| there; for order 4 the cross
// derivatives come from the first derivatives (phi_x along y, phi_y along z,
// phi_z along x) through px, py, pz at the cell with strides pys, pzs.
template <class R, int K>
__device__ __forceinline__ R curvature_variant(const R *c, long long sy, long long sz, const R *px, const R *py,
                                               const R *pz, long long pys, long long pzs, R gm,
                                               const CurvFactors<R> &F) {
  R xx, yy, zz, xy, xz, yz;
  const R x = px[0], y = py[0], z = pz[0];
  if (K == CURV_GAUSS2) {
    xx = (c[1] - R(2.0) * c[0] + c[-1]) * F.f[0];
    yy = (c[sy] - R(2.0) * c[0] + c[-sy]) * F.f[1];
    zz = (c[sz] - R(2.0) * c[0] + c[-sz]) * F.f[2];
    xy = (c[1 + sy] - c[1 - sy] - c[-1 + sy] + c[-1 - sy]) * F.f[3];
    xz = (c[1 + sz] - c[1 - sz] - c[-1 + sz] + c[-1 - sz]) * F.f[4];
    yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * F.f[5];
  } else {
    const R sixteen = R(16), thirty = R(30), eight = R(8);
    xx = (-c[2] + sixteen * c[1] - thirty * c[0] - c[-2] + sixteen * c[-1]) * F.f[0];
    yy = (-c[2 * sy] + sixteen * c[sy] - thirty * c[0] - c[-2 * sy] + sixteen * c[-sy]) * F.f[1];
    zz = (-c[2 * sz] + sixteen * c[sz] - thirty * c[0] - c[-2 * sz] + sixteen * c[-sz]) * F.f[2];
    xy = (-px[2 * pys] + eight * px[pys] + px[-2 * pys] - eight * px[-pys]) * F.f[4];  // phi_x along y
    yz = (-py[2 * pzs] + eight * py[pzs] + py[-2 * pzs] - eight * py[-pzs]) * F.f[5];  // phi_y along z
    xz = (-pz[2] + eight * pz[1] + pz[-2] - eight * pz[-1]) * F.f[3];                  // phi_z along x
  }
  if (K == CURV_MEAN4) {
    const R den = gm * gm * gm;
    if (den < Consts<R>::zero_tol) return R(0);
    const R t = xx * y * y + yy * x * x - R(2) * xy * x * y + xx * z * z + zz * x * x - R(2) * xz * x * z +
                yy * z * z + zz * y * y - R(2) * yz * y * z;
    return t / den;
  }
  const R den = gm * gm * gm * gm;
  if (den < Consts<R>::zero_tol) return R(0);
  const R t = x * x * (yy * zz - yz * yz) + y * y * (xx * zz - xz * xz) + z * z * (xx * yy - xy * xy) +
              R(2) * (x * y * (xz * yz - xy * zz) + y * z * (xy * xz - yz * xx) + x * z * (xy * yz - xz * yy));
  return t / den;
}

template <class R, int K>
inline CurvFactors<R> curvature_factors(R dx, R dy, R dz) {
  CurvFactors<R> F;
  if (K == CURV_GAUSS2) {
    F.f[0] = R(1.0) / dx / dx; F.f[1] = R(1.0) / dy / dy; F.f[2] = R(1.0) / dz / dz;
    F.f[3] = R(0.25) / dx / dy; F.f[4] = R(0.25) / dx / dz; F.f[5] = R(0.25) / dy / dz;
  } else {
    const R c = R(0.0833333333333333333333);
    F.f[0] = c / dx / dx; F.f[1] = c / dy / dy; F.f[2] = c / dz / dz;
    F.f[3] = c / dx; F.f[4] = c / dy; F.f[5] = c / dz;
  }
  return F;
}

}  // namespace lsmgpu
