// Fused narrow-band curvature flow: phi_t + Vn |grad phi| = 0 with
// Vn = a_n - b_n * kappa, HJ WENO5 on a narrow band, TVD-RK3, the band rebuilt
// every `rebuild_every` steps.  It replaces the LSMLIB local call sequence
// per stage (on level-0 cells):
//   lsm3dCentralGradOrder2LOCAL -> lsm3dGradientMagnitudeLocal ->
//   lsm3dComputeMeanCurvatureOrder2Local -> Vn = a_n - b_n*kappa ->
//   HJ WENO5 LOCAL -> lsm3dZeroOut/AddNormalVelTermToLSERHSLOCAL ->
//   (stage 1: lsm3dComputeStableNormalVelDtLOCAL) ->
//   lsm3dMultiplyCutOffLSERHSLOCAL -> lsm3dTVDRK3StageNLOCAL
// with one gather kernel per stage (stage 1 is split at the dt reduction),
// and the band build of band.cuh.  Band levels 1..3 of the stage fields hold
// phi^n: they are refreshed at every rebuild and never written by a stage.
//
// LSMGPU_BANDFLOW_EXACT selects the FP64 parity arithmetic (this unit is
// compiled with -fmad=false); the FP32 form uses the fast WENO weights.
#pragma once
#include <vector>

#include "band.cuh"
#include "fused_stage.cuh"
#include "stencil_math.cuh"
#include "../../include/lsmgpu.h"

namespace lsmgpu {
namespace bandflow {

template <class R>
struct BandArgs {
  View<const R> src;      // stage source (phi^n, u1, u2)
  View<const R> phin;     // phi^n (stages 2, 3)
  View<R> out;            // stage output
  const int *ix, *iy, *iz;
  const int *off0;        // padded offset of each level-0 entry (written at each rebuild)
  int n0;                 // level-0 entries (list elements 0..n0-1)
  R dx, a_n, b_n, beta, gamma, cfl;
  // per-call constants of the stencils, divided on the host in R exactly as
  // the per-cell expressions would: 0.5/dx, 1/dx/dx, 0.25/dx/dx, 1/dx
  R f_half, f_xx, f_xy, inv_dx;
  R *rhs;                 // stage 1: the RHS per level-0 entry (FP32 form: a
                          // (src, src, rhs, rhs) record per entry pair)
  const R *dt;            // device scalar
  unsigned long long *key;
  int stage;
};

__device__ __forceinline__ unsigned long long okey(double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ double okey_inv(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
  return __longlong_as_double((long long)u);
}

// running maximum of the dt keys: the key only grows, so a warp whose key
// does not exceed the value it reads cannot raise it and skips the atomic
// (a stale read only costs an atomic); keeps tens of thousands of warps from
// queueing on one address
__device__ __forceinline__ void raise_key(unsigned long long *key, unsigned long long k) {
  if (k > __ldcg(key)) atomicMax(key, k);
}

// WENO5 with the local routines' epsilon floor (spatial_derivatives2d_local.f.in:892)
template <class R, bool EXACT>
__device__ __forceinline__ R weno_local(R v1, R v2, R v3, R v4, R v5) {
  if constexpr (EXACT) {
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
  } else {
    return (R)fused::weno5_fast((float)v1, (float)v2, (float)v3, (float)v4, (float)v5);
  }
}

// normal speed Vn = a_n - b_n kappa at a level-0 cell: central gradient,
// |grad phi| with zero_tol clamps, mean curvature
// (spatial_derivatives3d_local.f.in:825-839, :1251-1272; curvature3d_local.f.in)
template <class R>
__device__ __forceinline__ R cell_vn(const BandArgs<R> &a, const R *c, const long long s[3]) {
  const R f = a.f_half;
  const R g0 = (c[s[0]] - c[-s[0]]) * f, g1 = (c[s[1]] - c[-s[1]]) * f, g2 = (c[s[2]] - c[-s[2]]) * f;
  const R tol = Consts<double>::zero_tol;
  R x2 = g0 * g0, y2 = g1 * g1, z2 = g2 * g2;
  if (x2 < tol) x2 = R(0);
  if (y2 < tol) y2 = R(0);
  if (z2 < tol) z2 = R(0);
  const R t = sqrt(x2 + y2 + z2);
  const R mag = (t < tol) ? R(0) : t;
  const R fxx = a.f_xx, fxy = a.f_xy;
  const R xx = (c[s[0]] - R(2.0) * c[0] + c[-s[0]]) * fxx;
  const R yy = (c[s[1]] - R(2.0) * c[0] + c[-s[1]]) * fxx;
  const R zz = (c[s[2]] - R(2.0) * c[0] + c[-s[2]]) * fxx;
  const R xy = (c[s[0] + s[1]] - c[s[0] - s[1]] - c[-s[0] + s[1]] + c[-s[0] - s[1]]) * fxy;
  const R xz = (c[s[0] + s[2]] - c[s[0] - s[2]] - c[-s[0] + s[2]] + c[-s[0] - s[2]]) * fxy;
  const R yz = (c[s[1] + s[2]] - c[s[1] - s[2]] - c[-s[1] + s[2]] + c[-s[1] - s[2]]) * fxy;
  const R den = mag * mag * mag;
  const R kappa = (den < tol) ? R(0) : curv_numerator(xx, yy, zz, xy, xz, yz, g0, g1, g2) / den;
  return a.a_n - a.b_n * kappa;
}

// Godunov normal-velocity term (level_set_evolution3d_local.f.in:236-273) from
// the WENO5 plus/minus derivatives, and the cell's H/dx
// (math_utils3d_local.f.in:396-414)
template <class R>
__device__ __forceinline__ R godunov_rhs(const BandArgs<R> &a, R vn, const R gp[3], const R gm[3], R &h_over_dx) {
  const R tol = Consts<double>::zero_tol;
  const R sq = godunov_normal_sq<R>(vn > R(0), gp, gm);
  R rhs = R(0);
  if (fabs(vn) >= tol) rhs = rhs - vn * sqrt(sq);
  const R dx = a.dx, inv = a.inv_dx;
  const R mx2 = dx * dx;
  const R cx = rmax(fabs(gp[0]), fabs(gm[0])), cy = rmax(fabs(gp[1]), fabs(gm[1])), cz = rmax(fabs(gp[2]), fabs(gm[2]));
  const R ng = sqrt(cx * cx + cy * cy + cz * cz + mx2);
  h_over_dx = (ng > tol) ? fabs(vn) / ng * (cx * inv + cy * inv + cz * inv) : R(-1.0);
  return rhs;
}

// the RHS of one level-0 cell, before the cut-off; also the cell's H/dx for dt
template <class R, bool EXACT>
__device__ __forceinline__ R cell_rhs(const BandArgs<R> &a, int i, int j, int k, R &h_over_dx) {
  const R *c = a.src.p + a.src.off(i, j, k);
  const long long s[3] = {1, a.src.s1, a.src.s2};
  const R vn = cell_vn<R>(a, c, s);
  // HJ WENO5 plus/minus from the band values of src
  const R inv = a.inv_dx;
  R gp[3], gm[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    R v[6];
#pragma unroll
    for (int q = -2; q <= 3; q++) v[q + 2] = (c[q * s[d]] - c[(q - 1) * s[d]]) * inv;
    gp[d] = weno_local<R, EXACT>(v[5], v[4], v[3], v[2], v[1]);
    gm[d] = weno_local<R, EXACT>(v[0], v[1], v[2], v[3], v[4]);
  }
  return godunov_rhs<R>(a, vn, gp, gm, h_over_dx);
}

// cell_vn on two cells in packed FP32x2: the central gradient, the second
// differences and the curvature numerator (summed as
// xx (y^2 + z^2) + yy (x^2 + z^2) + zz (x^2 + y^2) - 2 (xy x y + xz x z + yz y z))
// run on the pair; the zero_tol clamps, |grad phi| and the division per cell
static __device__ __forceinline__ float2 cell_vn_x2(const BandArgs<float> &a, const float *c0, const float *c1,
                                                    const long long s[3]) {
  using fused::add2;
  using fused::fma2;
  using fused::mul2;
  using fused::sp;
  const auto at = [&](long long o) { return make_float2(c0[o], c1[o]); };
  const auto sub = [](float2 x, float2 y) { return fma2(y, sp(-1.f), x); };
  const float2 cc = at(0);
  const float2 xp = at(s[0]), xm = at(-s[0]), yp = at(s[1]), ym = at(-s[1]), zp = at(s[2]), zm = at(-s[2]);
  const float2 f = sp(a.f_half);
  const float2 gx = mul2(sub(xp, xm), f), gy = mul2(sub(yp, ym), f), gz = mul2(sub(zp, zm), f);
  const float tol = Consts<double>::zero_tol;
  const float2 sx = mul2(gx, gx), sy = mul2(gy, gy), sz = mul2(gz, gz);
  // |grad phi| with each square below zero_tol dropped
  const float2 q = add2(add2(make_float2(sx.x < tol ? 0.f : sx.x, sx.y < tol ? 0.f : sx.y),
                             make_float2(sy.x < tol ? 0.f : sy.x, sy.y < tol ? 0.f : sy.y)),
                        make_float2(sz.x < tol ? 0.f : sz.x, sz.y < tol ? 0.f : sz.y));
  float m0 = sqrtf(q.x), m1 = sqrtf(q.y);
  m0 = (m0 < tol) ? 0.f : m0;
  m1 = (m1 < tol) ? 0.f : m1;
  const float2 fxx = sp(a.f_xx), fxy = sp(a.f_xy), m2 = sp(-2.f);
  const float2 xx = mul2(add2(fma2(m2, cc, xp), xm), fxx);
  const float2 yy = mul2(add2(fma2(m2, cc, yp), ym), fxx);
  const float2 zz = mul2(add2(fma2(m2, cc, zp), zm), fxx);
  const float2 xy = mul2(add2(sub(sub(at(s[0] + s[1]), at(s[0] - s[1])), at(-s[0] + s[1])), at(-s[0] - s[1])), fxy);
  const float2 xz = mul2(add2(sub(sub(at(s[0] + s[2]), at(s[0] - s[2])), at(-s[0] + s[2])), at(-s[0] - s[2])), fxy);
  const float2 yz = mul2(add2(sub(sub(at(s[1] + s[2]), at(s[1] - s[2])), at(-s[1] + s[2])), at(-s[1] - s[2])), fxy);
  const float2 diag = fma2(xx, add2(sy, sz), fma2(yy, add2(sx, sz), mul2(zz, add2(sx, sy))));
  const float2 cross = fma2(mul2(xy, gx), gy, fma2(mul2(xz, gx), gz, mul2(mul2(yz, gy), gz)));
  const float2 num = fma2(m2, cross, diag);
  const float d0 = m0 * m0 * m0, d1 = m1 * m1 * m1;
  const float k0 = (d0 < tol) ? 0.f : num.x / d0, k1 = (d1 < tol) ? 0.f : num.y / d1;
  return make_float2(a.a_n - a.b_n * k0, a.a_n - a.b_n * k1);
}

// FP32 RHS of two level-0 cells (padded offsets o0, o1): the six WENO5
// reconstructions and the curvature run on the pair in Blackwell's packed
// FP32x2 arithmetic (WENO5: both sides of an axis together); the Godunov term
// per cell
static __device__ __forceinline__ float2 cell_rhs_x2(const BandArgs<float> &a, long long o0, long long o1, float2 &hd) {
  const float *c0 = a.src.p + o0, *c1 = a.src.p + o1;
  const long long s[3] = {1, a.src.s1, a.src.s2};
  const float2 vn = cell_vn_x2(a, c0, c1, s);
  const float vn0 = vn.x, vn1 = vn.y;
  const float2 inv = fused::sp(a.inv_dx);
  float gp0[3], gm0[3], gp1[3], gm1[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    float2 v[6];
#pragma unroll
    for (int q = -2; q <= 3; q++)
      v[q + 2] = fused::mul2(make_float2(c0[q * s[d]] - c0[(q - 1) * s[d]], c1[q * s[d]] - c1[(q - 1) * s[d]]), inv);
    float2 p, m;
    fused::weno5_pm_x2(v, p, m);
    gp0[d] = p.x; gp1[d] = p.y;
    gm0[d] = m.x; gm1[d] = m.y;
  }
  float h0, h1;
  const float r0 = godunov_rhs<float>(a, vn0, gp0, gm0, h0);
  const float r1 = godunov_rhs<float>(a, vn1, gp1, gm1, h1);
  hd = make_float2(h0, h1);
  return make_float2(r0, r1);
}

// cubic cut-off between beta and gamma (localization3d.f:527-553)
template <class R>
__device__ __forceinline__ R cutoff(R rhs, R phi, R beta, R gamma) {
  const R av = fabs(phi);
  R co;
  if (av <= beta) {
    co = R(1);
  } else if (av <= gamma) {
    const R c1 = gamma - 3 * beta;
    R c2 = (gamma - beta);
    c2 = c2 * c2 * c2;
    const R tt = av - gamma;
    co = (tt * tt * (2 * av + c1)) / c2;
  } else {
    co = R(0);
  }
  return co * rhs;
}

template <class R>
__device__ __forceinline__ R rk_update(int stage, R un, R us, R dt, R rhs) {
  if (stage == 1) return un + dt * rhs;
  if (stage == 2) return R(0.75) * un + R(0.25) * (us + dt * rhs);
  return R(1.0 / 3.0) * un + R(2.0 / 3.0) * (us + dt * rhs);
}

// stage 1, pass 1: RHS (cut off) per entry and the dt maximum
template <class R, bool EXACT>
__global__ void k_band_rhs(BandArgs<R> a) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  double h = -1.0e308;
  if (l < a.n0) {
    const int i = a.ix[l], j = a.iy[l], k = a.iz[l];
    R hd;
    const R r = cell_rhs<R, EXACT>(a, i, j, k, hd);
    h = (double)hd;
    a.rhs[l] = cutoff<R>(r, a.src(i, j, k), a.beta, a.gamma);
  }
  for (int o = 16; o > 0; o >>= 1) h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
  if ((threadIdx.x & 31) == 0) raise_key(a.key, okey(h));
}

template <class R>
__global__ void k_band_dt(const unsigned long long *key, R *dt, R cfl, double *dt_log) {
  double m = okey_inv(*key);
  if (m < -1.0) m = -1.0;  // the reference's running maximum starts at -1
  const R d = cfl / ((R)m + (R)Consts<double>::tiny);
  *dt = d;
  if (dt_log) *dt_log = (double)d;
}

// stage 1, pass 2: the update
template <class R>
__global__ void k_band_update1(BandArgs<R> a) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= a.n0) return;
  const long long o = a.off0[l];
  a.out.p[o] = rk_update<R>(1, a.src.p[o], a.src.p[o], *a.dt, a.rhs[l]);
}

// stages 2 and 3: RHS, cut-off and update in one pass
template <class R, bool EXACT>
__global__ void k_band_stage(BandArgs<R> a) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= a.n0) return;
  const int i = a.ix[l], j = a.iy[l], k = a.iz[l];
  R hd;
  const R us = a.src(i, j, k);
  const R r = cutoff<R>(cell_rhs<R, EXACT>(a, i, j, k, hd), us, a.beta, a.gamma);
  a.out(i, j, k) = rk_update<R>(a.stage, a.phin(i, j, k), us, *a.dt, r);
}

// FP32 forms of k_band_rhs and k_band_stage on pairs of consecutive list
// entries (the second of an odd tail repeats the first and is not written)
// offsets of the entry pair l0, l0 + 1 (the second repeats the first at an
// odd tail); off0 has an even number of elements, so the pair load is in bounds
static __device__ __forceinline__ void pair_offsets(const BandArgs<float> &a, int l0, bool two, long long &o0,
                                                    long long &o1) {
  const int2 p = *reinterpret_cast<const int2 *>(a.off0 + l0);
  o0 = p.x;
  o1 = two ? p.y : p.x;
}

// Stage 1 of the FP32 form stores, per entry pair p, the float4
// (src[l0], src[l1], rhs[l0], rhs[l1]) at a.rhs + 4p, so that the update
// after the dt reduction reads one contiguous record instead of gathering src.
// The dt maximum is taken in FP32 (a maximum is exact in either precision;
// the one conversion to FP64 per warp gives the same key) to keep the slow
// FP64 pipe out of the kernel.
static __global__ void __launch_bounds__(128, 8) k_band_rhs_x2(BandArgs<float> a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int l0 = 2 * p;
  float h = -INFINITY;
  if (l0 < a.n0) {
    const bool two = l0 + 1 < a.n0;
    long long o0, o1;
    pair_offsets(a, l0, two, o0, o1);
    float2 hd;
    const float2 r = cell_rhs_x2(a, o0, o1, hd);
    h = two ? fmaxf(hd.x, hd.y) : hd.x;
    const float s0 = a.src.p[o0], s1 = a.src.p[o1];
    reinterpret_cast<float4 *>(a.rhs)[p] =
        make_float4(s0, s1, cutoff<float>(r.x, s0, a.beta, a.gamma), cutoff<float>(r.y, s1, a.beta, a.gamma));
  }
  for (int o = 16; o > 0; o >>= 1) h = fmaxf(h, __shfl_xor_sync(0xffffffffu, h, o));
  if ((threadIdx.x & 31) == 0) raise_key(a.key, okey((double)h));
}

// stage 1, pass 2 of the FP32 form: one entry pair per thread from its record
static __global__ void k_band_update1_x2(BandArgs<float> a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int l0 = 2 * p;
  if (l0 >= a.n0) return;
  const bool two = l0 + 1 < a.n0;
  long long o0, o1;
  pair_offsets(a, l0, two, o0, o1);
  const float4 v = reinterpret_cast<const float4 *>(a.rhs)[p];
  const float dt = *a.dt;
  a.out.p[o0] = rk_update<float>(1, v.x, v.x, dt, v.z);
  if (two) a.out.p[o1] = rk_update<float>(1, v.y, v.y, dt, v.w);
}

static __global__ void k_band_stage_x2(BandArgs<float> a) {
  const int l0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (l0 >= a.n0) return;
  const bool two = l0 + 1 < a.n0;
  long long o0, o1;
  pair_offsets(a, l0, two, o0, o1);
  float2 hd;
  const float2 r = cell_rhs_x2(a, o0, o1, hd);
  const float dt = *a.dt;
  const float us0 = a.src.p[o0], us1 = a.src.p[o1];
  const float n0v = a.phin.p[o0], n1v = a.phin.p[o1];
  a.out.p[o0] = rk_update<float>(a.stage, n0v, us0, dt, cutoff<float>(r.x, us0, a.beta, a.gamma));
  if (two) a.out.p[o1] = rk_update<float>(a.stage, n1v, us1, dt, cutoff<float>(r.y, us1, a.beta, a.gamma));
}

// the padded offset of each level-0 entry, for the stage kernels (one 4-byte
// read per entry instead of three coordinates)
template <class R>
__global__ void k_band_offsets(View<const R> v, const int *ix, const int *iy, const int *iz, int n, int *off) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n) return;
  off[l] = (int)v.off(ix[l], iy[l], iz[l]);
}

// clears the marks of the listed cells (the previous band, before a rebuild)
// and copies the level-0 entries (the first n0) to ox, oy, oz
static __global__ void k_band_retire(U8 *nb, View<const U8> v, const int *ix, const int *iy, const int *iz, int n,
                                     int n0, int *ox, int *oy, int *oz) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n) return;
  const int i = ix[l], j = iy[l], k = iz[l];
  nb[v.off(i, j, k)] = 0;
  if (l < n0) {
    ox[l] = i;
    oy[l] = j;
    oz[l] = k;
  }
}

// phi -> u1, u2 at the listed cells
template <class R>
__global__ void k_copy_band(const R *phi, R *u1, R *u2, View<const R> v, const int *ix, const int *iy, const int *iz,
                            int n) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n) return;
  const long long o = v.off(ix[l], iy[l], iz[l]);
  const R p = phi[o];
  u1[o] = p;
  u2[o] = p;
}

template <class R, bool EXACT>
int run(const char *name, R *phi_user, const Box &gb, const Box &fb, R dx, R a_n, R b_n, R cfl, R gamma, R beta,
        int n_steps, int rebuild_every, double *dt_log, long long *band_log) {
  Call call(name);
  if (!gb.contains(fb, 0, 0, 0)) call.fail("fill box outside the ghost box");
  if (rebuild_every <= 0) call.fail("rebuild_every must be positive");
  if (gb.size() >= (1LL << 31)) call.fail("ghost box of 2^31 cells or more");
  if (!call.ok()) return LSMGPU_ERR_BOUNDS;
  if (n_steps <= 0) return LSMGPU_OK;
  const long long n = gb.size();
  R *phi = call.inout(phi_user, n);
  R *u1 = call.temp<R>(n), *u2 = call.temp<R>(n);
  U8 *nb = call.temp<U8>(n);
  int *ix = call.temp<int>(n), *iy = call.temp<int>(n), *iz = call.temp<int>(n), *outer = call.temp<int>(n);
  constexpr bool packed = !EXACT && sizeof(R) == 4;
  R *rhs = nullptr;  // per level-0 entry; sized at the first build
  int *off0 = call.temp<int>(n + 1);  // n + 1: the pair loads read an even count
  R *dt = call.temp<R>(1);
  unsigned long long *key = call.temp<unsigned long long>(1);
  double *dtl = dt_log ? call.temp<double>(n_steps) : nullptr;
  int *claim = new_claims(call, gb);  // reused by every rebuild (left unclaimed)
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  cudaStream_t s = stream();
  const int level = 3;
  std::vector<int> lo, hi;
  int ob[4];
  int n0 = 0, nrebuild = 0;
  // the previous level-0 list of a rebuild (the first build scans the grid)
  int *ox = nullptr, *oy = nullptr, *oz = nullptr;
  for (int step = 0; step < n_steps; step++) {
    if (step % rebuild_every == 0) {
      long long c0 = 0;
      PrevLevel0 prev;
      if (nrebuild > 0) {
        // phi changed only at level-0 cells since the last build: the new
        // band's level 0 is drawn from the old one (Level0List); the old
        // band's marks are cleared so the breadth-first levels start clean
        int nlist = 0;
        for (int lv = 0; lv <= level; lv++)
          if (hi[lv] + 1 > nlist) nlist = hi[lv] + 1;
        if (nlist > 0)
          LSMGPU_LAUNCH(k_band_retire, (unsigned)((nlist + 255) / 256), 256, 0, nb, view((const U8 *)nb, gb), ix, iy,
                        iz, nlist, n0, ox, oy, oz);
        prev.ox = ox;
        prev.oy = oy;
        prev.oz = oz;
        prev.n = n0;
      }
      if (!band_build<R>(call, phi, gb, nb, gb, ix, iy, iz, 0, (int)(n - 1), outer, 0, (int)(n - 1), (double)gamma,
                         (double)beta, level, lo, hi, ob, &c0, claim, true, BandForm<R>(), nullptr,
                         nrebuild > 0 ? &prev : nullptr))
        return lsmgpu_get_last_error(nullptr, 0);
      if (nrebuild == 0 && c0 > 0) {
        // later level-0 lists are sub-sequences of this one
        ox = call.temp<int>(c0);
        oy = call.temp<int>(c0);
        oz = call.temp<int>(c0);
        // the FP32 form keeps a 4-value record per entry pair
        rhs = call.temp<R>(packed ? 2 * c0 + 4 : c0);
        if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
      }
      n0 = (int)c0;
      if (band_log) band_log[nrebuild] = c0;
      nrebuild++;
      // stage fields hold phi^n on band levels 1..3 (every cell a level-0
      // stencil reads besides level 0); level-0 cells are written by each
      // stage before any stage reads them, so only levels 1..3 are copied
      int nlist = 0;
      for (int lv = 0; lv <= level; lv++)
        if (hi[lv] + 1 > nlist) nlist = hi[lv] + 1;
      if (n0 > 0)
        LSMGPU_LAUNCH(k_band_offsets<R>, (unsigned)((n0 + 255) / 256), 256, 0, view((const R *)phi, gb), ix, iy, iz,
                      n0, off0);
      const int first = n0;  // levels 1..3 follow level 0 in the lists
      if (n0 > 0 && nlist > first)
        LSMGPU_LAUNCH(k_copy_band<R>, (unsigned)((nlist - first + 255) / 256), 256, 0, (const R *)phi, u1, u2,
                      view((const R *)phi, gb), ix + first, iy + first, iz + first, nlist - first);
    }
    if (n0 == 0) continue;
    BandArgs<R> a{};
    a.ix = ix; a.iy = iy; a.iz = iz;
    a.off0 = off0;
    a.n0 = n0;
    a.dx = dx; a.a_n = a_n; a.b_n = b_n; a.beta = beta; a.gamma = gamma; a.cfl = cfl;
    a.f_half = R(0.5) / dx;
    a.f_xx = R(1.0) / dx / dx;
    a.f_xy = R(0.25) / dx / dx;
    a.inv_dx = R(1.0) / dx;
    a.rhs = rhs;
    a.dt = dt;
    a.key = key;
    const unsigned blocks = (unsigned)((n0 + 127) / 128);
    const unsigned blocks2 = (unsigned)((n0 + 255) / 256);  // pairs of entries
    // stage 1
    a.src = view((const R *)phi, gb);
    a.phin = a.src;
    a.out = view(u1, gb);
    a.stage = 1;
    cudaMemsetAsync(key, 0, sizeof(unsigned long long), s);
    if constexpr (packed) LSMGPU_LAUNCH(k_band_rhs_x2, blocks2, 128, 0, a);
    else LSMGPU_LAUNCH((k_band_rhs<R, EXACT>), blocks, 128, 0, a);
    LSMGPU_LAUNCH(k_band_dt<R>, 1, 1, 0, key, dt, cfl, dtl ? dtl + step : nullptr);
    if constexpr (packed) LSMGPU_LAUNCH(k_band_update1_x2, blocks2, 128, 0, a);
    else LSMGPU_LAUNCH(k_band_update1<R>, blocks, 128, 0, a);
    // stage 2
    a.src = view((const R *)u1, gb);
    a.out = view(u2, gb);
    a.phin = view((const R *)phi, gb);
    a.stage = 2;
    if constexpr (packed) LSMGPU_LAUNCH(k_band_stage_x2, blocks2, 128, 0, a);
    else LSMGPU_LAUNCH((k_band_stage<R, EXACT>), blocks, 128, 0, a);
    // stage 3 (in place on phi: each cell reads only its own phi^n)
    a.src = view((const R *)u2, gb);
    a.out = view(phi, gb);
    a.stage = 3;
    if constexpr (packed) LSMGPU_LAUNCH(k_band_stage_x2, blocks2, 128, 0, a);
    else LSMGPU_LAUNCH((k_band_stage<R, EXACT>), blocks, 128, 0, a);
  }
  if (dt_log) cudaMemcpyAsync(dt_log, dtl, sizeof(double) * n_steps, cudaMemcpyDeviceToHost, s);
  call.finish();
  cudaStreamSynchronize(s);
  return lsmgpu_get_last_error(nullptr, 0);
}

}  // namespace bandflow
}  // namespace lsmgpu
