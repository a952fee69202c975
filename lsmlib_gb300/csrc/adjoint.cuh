// Hand-written adjoint (reverse mode) of periodic WENO5 / TVD-RK3 advection.
//
// Forward map (per time step, LSMLIB's call sequence on a periodic grid):
//   L(s)_c = 0 - sum_d u_d(c) W_d(s)_c         upwind WENO5 derivative W_d
//   u1 = u + dt L(u);  u2 = 3/4 u + 1/4 (u1 + dt L(u1));
//   u' = 1/3 u + 2/3 (u2 + dt L(u2))           (tvd_runge_kutta3d.f:78, 403, 490)
// Objective J = sum_c (H(phi_T) - H(phi_target))^2 dx dy dz with LSMLIB's
// smoothed Heaviside (lsm_calculus_toolbox.h:41); dt is held fixed.
//
// Reverse step, given lam = dJ/du':
//   mu2 = 2/3 lam;  lam_u2 = mu2 + dt L_u2^T mu2;       (adjoint stage 3)
//   mu1 = 1/4 lam_u2;  lam_u1 = mu1 + dt L_u1^T mu1;    (adjoint stage 2)
//   lam_u = 1/3 lam + 3/4 lam_u2 + lam_u1 + dt L_u^T lam_u1   (adjoint stage 1)
//   grad_u_d += dt * mu * (-W_d)  at each of the three linearisation points.
//
// L_s^T mu.  Along axis d, cell c reads five first differences V(f) =
// (s_f - s_{f-1})/dx_d at faces f = c-2..c+2 (u_d > 0) or c-1..c+3 (u_d < 0).
// Reverse mode gives per cell six face slots G_m(c), m = 0..5 for faces
// c-2+m (one end slot is zero), G = dt mu_c (-u_d) / dx_d * dW/dv.  The
// adjoint of face f is Vbar(f) = sum_m G_m(f+2-m) and the adjoint of cell j
// is Vbar(j) - Vbar(j+1).  So each output cell needs the slots of the cells
// within 3 of it along each axis.
//
// Kernels (two per adjoint stage, neither uses shared memory or block
// barriers):
//   k_adj_xz: a warp owns a row segment of 32 cells along x, the middle 26 of
//     which it writes, and marches along z through a chunk of planes.  Each
//     lane keeps a 7-value window of s down its column and a ring of six
//     z-face sums (z slots of the cell 3 planes ahead); per output plane it
//     computes the x slots of its cell and the warp sums x faces with
//     shuffles.  It writes out = mu + dt (A_x + A_z) (+ P, Q terms).
//   k_adj_y: a thread owns an (x, z) column and marches along y through a
//     chunk with the same window / face-ring scheme; it adds dt A_y to out.
// Redundant slot work: x and z 32/26, y (chunk + 6)/chunk, z also
// (chunk + 6)/chunk.
//
// All indices wrap periodically, so the adjoint fields need no ghost cells;
// the forward states use the fused steppers' padded layout (their periodic
// ghost images are written by the forward stage kernels).
#pragma once

#include "fused_stage.cuh"
#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"

namespace lsmgpu {
namespace adj {

using fused::Layout;

constexpr int kSeg = 26;     // cells of a row segment written by one warp
constexpr int kRows = 8;     // warps (rows) per CTA of k_adj_xz, columns per CTA row of k_adj_y
// resident CTAs per SM the FP32 reverse kernels are compiled for (register
// caps).  Measured at 192^3 (reverse step, same box): k_adj_y capped for 4
// CTAs of 256 threads (61 registers, no spills) 0.858 ms against 0.904 ms
// uncapped (79 registers); 5 CTAs (48 registers) 0.861 ms; k_adj_xz_row for 4
// CTAs spills (64 registers) and ran 0.920 ms.
#ifndef LSMGPU_ADJ_ROW_CTAS
#define LSMGPU_ADJ_ROW_CTAS 3
#endif
#ifndef LSMGPU_ADJ_Y_CTAS
#define LSMGPU_ADJ_Y_CTAS 4
#endif
constexpr int kRowMax = 256; // longest x row k_adj_xz_row takes (one CTA per row)

// periodic image of index a in [0, n): one add or subtract for a in
// [-n, 2n), a remainder otherwise
__host__ __device__ __forceinline__ int wrapi(int a, int n) {
  if (a < 0) a += n;
  else if (a >= n) a -= n;
  if ((unsigned)a >= (unsigned)n) {
    a %= n;
    if (a < 0) a += n;
  }
  return a;
}

// WENO5 value and its partial derivatives dW/dv_q.
//
// With alpha_k = d_k/(S_k+eps)^2, w_k = alpha_k/sum(alpha), W = sum w_k p_k:
//   dW = sum_k w_k dp_k + sum_k beta_k (dS_k + deps),
//   beta_k = -2 w_k (p_k - W) / (S_k + eps),
// and deps = 2e-6 v_m dv_m for the index m that max(v^2) selects.
// EXACT: the FP64 form of spatial_derivatives3d.f.in:1296-1323.  Otherwise
// the FP32 epsilon-scaled form (q_k = S_k/eps + 1, weights d_k/q_k^2
// normalised, 1/(S_k+eps) = (1/eps)/q_k), which cannot under- or overflow.
template <class R, bool EXACT>
__device__ __forceinline__ R weno5_adj(const R v[5], R dv[5]) {
  const R c13 = R(1.0 / 3.0), c76 = R(7.0 / 6.0), c116 = R(11.0 / 6.0);
  const R c16 = R(1.0 / 6.0), c56 = R(5.0 / 6.0), c1312 = R(13.0 / 12.0), c136 = R(13.0 / 6.0);
  const R v1 = v[0], v2 = v[1], v3 = v[2], v4 = v[3], v5 = v[4];
  R m = v1 * v1;
  int am = 0;
#pragma unroll
  for (int q = 1; q < 5; q++) {
    const R sq = v[q] * v[q];
    if (!(m > sq)) am = q;
    m = rmax(m, sq);
  }
  const R p1 = c13 * v1 - c76 * v2 + c116 * v3;
  const R p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  const R p3 = c13 * v3 + c56 * v4 - c16 * v5;
  const R t1 = v1 - R(2) * v2 + v3, u1 = v1 - R(4) * v2 + R(3) * v3;
  const R t2 = v2 - R(2) * v3 + v4, u2 = v2 - v4;
  const R t3 = v3 - R(2) * v4 + v5, u3 = R(3) * v3 - R(4) * v4 + v5;
  const R S1 = c1312 * (t1 * t1) + R(0.25) * (u1 * u1);
  const R S2 = c1312 * (t2 * t2) + R(0.25) * (u2 * u2);
  const R S3 = c1312 * (t3 * t3) + R(0.25) * (u3 * u3);
  R w1, w2, w3, i1, i2, i3;  // normalised weights; 1/(S_k + eps)
  if constexpr (EXACT) {
    const R eps = R(1e-6) * m + Consts<R>::tiny;
    i1 = R(1) / (S1 + eps);
    i2 = R(1) / (S2 + eps);
    i3 = R(1) / (S3 + eps);
    const R a1 = R(0.1) * (i1 * i1), a2 = R(0.6) * (i2 * i2), a3 = R(0.3) * (i3 * i3);
    const R inv_sum = R(1) / (a1 + a2 + a3);
    w1 = a1 * inv_sum;
    w2 = a2 * inv_sum;
    w3 = a3 * inv_sum;
  } else {
    const R eps = R(1e-6) * m + R(1e-36);
    const R r = __fdividef(R(1), eps);
    const R q1 = S1 * r + R(1), q2 = S2 * r + R(1), q3 = S3 * r + R(1);
    const R q12 = q1 * q2, q13 = q1 * q3, q23 = q2 * q3;
    const R n1 = R(0.1) * (q23 * q23), n2 = R(0.6) * (q13 * q13), n3 = R(0.3) * (q12 * q12);
    const R inv_sum = __fdividef(R(1), n1 + n2 + n3);  // sum <= 3e31 < 2^126
    w1 = n1 * inv_sum;
    w2 = n2 * inv_sum;
    w3 = n3 * inv_sum;
    const R rq = __fdividef(r, q12 * q3);
    i1 = rq * q23;
    i2 = rq * q13;
    i3 = rq * q12;
  }
  const R W = w1 * p1 + w2 * p2 + w3 * p3;
  const R b1 = R(-2) * w1 * (p1 - W) * i1;
  const R b2 = R(-2) * w2 * (p2 - W) * i2;
  const R b3 = R(-2) * w3 * (p3 - W) * i3;
  const R T1 = c136 * t1 * b1, U1 = R(0.5) * u1 * b1;
  const R T2 = c136 * t2 * b2, U2 = R(0.5) * u2 * b2;
  const R T3 = c136 * t3 * b3, U3 = R(0.5) * u3 * b3;
  dv[0] = c13 * w1 + T1 + U1;
  dv[1] = -c76 * w1 - c16 * w2 - R(2) * T1 - R(4) * U1 + T2 + U2;
  dv[2] = c116 * w1 + c56 * w2 + c13 * w3 + T1 + R(3) * U1 - R(2) * T2 + T3 + R(3) * U3;
  dv[3] = c13 * w2 + c56 * w3 + T2 - U2 - R(2) * T3 - R(4) * U3;
  dv[4] = -c16 * w3 + T3 + U3;
  const R de = (b1 + b2 + b3) * R(2e-6);
#pragma unroll
  for (int q = 0; q < 5; q++)
    if (q == am) dv[q] += de * v[q];
  return W;
}

// Slots of one cell along one axis.  a[0..6] = s(c-3 .. c+3) along the axis,
// u = the velocity component, mu = the adjoint weight of the cell, inv = 1/dx_d.
// G[m] is the adjoint of face c-2+m (scaled by dt); the return value is the
// velocity adjoint dt * mu * (-W), zero where the forward set W to zero.
// FP32 slots with the adjoint weight folded in early: yb = dt mu kap / dx
// multiplies the weights and the beta_k once, so the five face adjoints come
// out of the derivative formulas directly.  kap = dL/dW for the WENO5 value W
// on side `minus`; returns W.
// D[0..5] = (s(c-2+f) - s(c-3+f)) / dx, the scaled differences of the cell
static __device__ __forceinline__ float lin_slots_f32(const float D[6], float kap, bool minus, float mu, float dt,
                                                      float inv, float G[6]) {
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float c136 = 13.f / 6.f;
  float v[5];
#pragma unroll
  for (int q = 0; q < 5; q++) v[q] = minus ? D[q] : D[5 - q];
  float m = v[0] * v[0];
  int am = 0;
#pragma unroll
  for (int q = 1; q < 5; q++) {
    const float sq = v[q] * v[q];
    const bool take = !(m > sq);  // the running max keeps the earlier value only when larger
    am = take ? q : am;
    m = take ? sq : m;
  }
  const float v1 = v[0], v2 = v[1], v3 = v[2], v4 = v[3], v5 = v[4];
  // q_k = (S_k + eps) r with r = 2^-e, 2^e <= eps < 2^(e+1) (exponent bits,
  // no reciprocal): the weights see only ratios of the q_k, and
  // 1/(S_k + eps) = r / q_k; S_k is kept as 4 S_k = 13/3 t^2 + u^2
  const float eps = fmaf(1e-6f, m, 1e-36f);
  const float r = fused::pow2_recip(eps);
  const float e = eps * r, r4 = 0.25f * r;
  const float p1 = fmaf(c13, v1, fmaf(-c76, v2, c116 * v3));
  const float p2 = fmaf(-c16, v2, fmaf(c56, v3, c13 * v4));
  const float p3 = fmaf(c13, v3, fmaf(c56, v4, -c16 * v5));
  const float t1 = fmaf(-2.f, v2, v1 + v3), u1 = fmaf(-4.f, v2, fmaf(3.f, v3, v1));
  const float t2 = fmaf(-2.f, v3, v2 + v4), u2 = v2 - v4;
  const float t3 = fmaf(-2.f, v4, v3 + v5), u3 = fmaf(-4.f, v4, fmaf(3.f, v3, v5));
  const float c133 = 13.f / 3.f;
  const float q1 = fmaf(fmaf(u1, u1, c133 * t1 * t1), r4, e);
  const float q2 = fmaf(fmaf(u2, u2, c133 * t2 * t2), r4, e);
  const float q3 = fmaf(fmaf(u3, u3, c133 * t3 * t3), r4, e);
  const float q12 = q1 * q2, q13 = q1 * q3, q23 = q2 * q3;
  // 10 d_k prod_{j != k} q_j^2 (the common factor cancels in the weights)
  const float n1 = q23 * q23, n2 = 6.f * q13 * q13, n3 = 3.f * q12 * q12;
  const float is = __fdividef(1.f, n1 + n2 + n3);  // sum <= 1e32 < 2^126
  const float w1 = n1 * is, w2 = n2 * is, w3 = n3 * is;
  const float W = fmaf(w1, p1, fmaf(w2, p2, w3 * p3));
  const float yb = dt * mu * kap * inv;
  // beta_k yb = -2 yb w_k (p_k - W) / (S_k + eps), 1/(S_k + eps) = r / (q1 q2 q3) * q_j q_l
  const float k0 = -2.f * yb * __fdividef(r, q12 * q3);
  const float b1 = k0 * w1 * (p1 - W) * q23, b2 = k0 * w2 * (p2 - W) * q13, b3 = k0 * w3 * (p3 - W) * q12;
  const float y1 = yb * w1, y2 = yb * w2, y3 = yb * w3;
  const float T1 = c136 * t1 * b1, U1 = 0.5f * u1 * b1;
  const float T2 = c136 * t2 * b2, U2 = 0.5f * u2 * b2;
  const float T3 = c136 * t3 * b3, U3 = 0.5f * u3 * b3;
  float g[5];
  g[0] = fmaf(c13, y1, T1 + U1);
  g[1] = fmaf(-c76, y1, fmaf(-c16, y2, fmaf(-2.f, T1, fmaf(-4.f, U1, T2 + U2))));
  g[2] = fmaf(c116, y1, fmaf(c56, y2, fmaf(c13, y3, fmaf(3.f, U1, fmaf(-2.f, T2, fmaf(3.f, U3, T1 + T3))))));
  g[3] = fmaf(c13, y2, fmaf(c56, y3, fmaf(-2.f, T3, fmaf(-4.f, U3, T2 - U2))));
  g[4] = fmaf(-c16, y3, T3 + U3);
  const float de = (b1 + b2 + b3) * 2e-6f;
#pragma unroll
  for (int q = 0; q < 5; q++) g[q] = (q == am) ? fmaf(de, v[q], g[q]) : g[q];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const float lo = (k < 5) ? g[k] : 0.f, hi = (k > 0) ? g[5 - k] : 0.f;
    G[k] = minus ? lo : hi;
  }
  return W;
}

// Face adjoints G[m] (faces c-2+m, scaled by dt) of one cell along one axis
// for the linearisation coefficient kap = dL/dW of the WENO5 value W on side
// `minus` (faces c-2..c+2) or plus (faces c-1..c+3); D[0..5] = the scaled
// differences (s(c-2+f) - s(c-3+f)) * inv along the axis, mu the adjoint
// weight of the cell, inv = 1/dx_d.  Returns W.
template <class R, bool EXACT>
__device__ __forceinline__ R lin_slots(const R D[6], R kap, bool minus, R mu, R dt, R inv, R G[6]) {
  if constexpr (!EXACT && sizeof(R) == 4) {
    return lin_slots_f32(D, kap, minus, mu, dt, inv, G);
  } else {
    R v[5], dv[5];
#pragma unroll
    for (int q = 0; q < 5; q++) v[q] = minus ? D[q] : D[5 - q];
    const R W = weno5_adj<R, EXACT>(v, dv);
    const R ybar = dt * mu * kap * inv;
    // minus: v_q on face c-2+q (slot q); plus: v_q on face c+3-q (slot 5-q)
#pragma unroll
    for (int m = 0; m < 6; m++) {
      const R lo = (m < 5) ? dv[m] : R(0);
      const R hi = (m > 0) ? dv[5 - m] : R(0);
      G[m] = ybar * (minus ? lo : hi);
    }
    return W;
  }
}

// Linearisation coefficient of one cell along one axis.
//   ADJ_ADV (advection, L = -sum_d u_d W_d): kap = -u_d, side from the sign of
//     u_d, none where |u_d| < zero_tol (spatial_derivatives3d.f.in:2756-2812);
//     the velocity adjoint of the cell is dt mu (-W).
//   ADJ_LIN: kap and side precomputed per cell (side bits 2d..2d+1: 0 none,
//     1 plus, 2 minus).
enum { ADJ_ADV = 0, ADJ_LIN = 1 };

template <class R>
struct Coef {
  R k;
  unsigned char side;
};

// D[0..5]: the cell's scaled differences along axis d (see lin_slots)
template <class R, bool EXACT, int MODE>
__device__ __forceinline__ R coef_slots_d(const R D[6], Coef<R> cf, int d, R mu, R dt, R inv, R G[6]) {
  if constexpr (MODE == ADJ_ADV) {
    const R u = cf.k;
    const bool on = !(fabs(u) < R(Consts<double>::zero_tol));
    const R W = lin_slots<R, EXACT>(D, on ? -u : R(0), u > R(0), mu, dt, inv, G);
    return on ? dt * mu * (-W) : R(0);
  } else {
    const int sb = (cf.side >> (2 * d)) & 3;
    lin_slots<R, EXACT>(D, sb ? cf.k : R(0), sb == 2, mu, dt, inv, G);
    return R(0);
  }
}

// the same from the values a[0..6] = s(c-3 .. c+3) along the axis
template <class R, bool EXACT, int MODE>
__device__ __forceinline__ R coef_slots(const R a[7], Coef<R> cf, int d, R mu, R dt, R inv, R G[6]) {
  R D[6];
#pragma unroll
  for (int f = 0; f < 6; f++) D[f] = (a[f + 1] - a[f]) * inv;
  return coef_slots_d<R, EXACT, MODE>(D, cf, d, mu, dt, inv, G);
}

template <class R>
struct AdjStageArgs {
  Layout L;
  const R *s;         // forward state the stage was linearised at
  const R *M;         // adjoint input; mu = mscale * M
  const R *P, *Q;     // optional pointwise terms pscale * P + qscale * Q
  R *out;             // mu + dt L_s^T mu (+ P, Q terms), interior cells
  const R *vel[3];     // ADJ_ADV: velocity components
  R *gvel[3];         // ADJ_ADV: velocity adjoint accumulators (nullptr: not wanted)
  const R *kap[3];    // ADJ_LIN: dL/dW per axis
  const unsigned char *side;  // ADJ_LIN: side bits per cell
  R mscale, pscale, qscale;
  R dt;
  R inv[3];
  int zchunk;         // planes per warp along z (k_adj_xz)
  int xchunk;         // planes per CTA of the x-face kernel of the two-line path
  int ychunk;         // rows per thread along y (k_adj_y)
};

// coefficient of axis d at padded index c
template <class R, int MODE>
__device__ __forceinline__ Coef<R> load_coef(const AdjStageArgs<R> &a, int d, long long c) {
  Coef<R> cf;
  if constexpr (MODE == ADJ_ADV) {
    cf.k = a.vel[d][c];
    cf.side = 0;
  } else {
    cf.k = a.kap[d][c];
    cf.side = a.side[c];
  }
  return cf;
}

// One step of the face-sum ring of a marching thread: add the slots of the
// cell `lead` (3 ahead of the output cell), and return A(lead - 3) =
// Vbar(lead - 3) - Vbar(lead - 2).
template <class R>
__device__ __forceinline__ R ring_step(R F[6], R &prevV, const R G[6]) {
#pragma unroll
  for (int m = 0; m < 6; m++) F[m] += G[m];
  const R A = prevV - F[0];
  prevV = F[0];
#pragma unroll
  for (int m = 0; m < 5; m++) F[m] = F[m + 1];
  F[5] = R(0);
  return A;
}

// Offset of plane p + c along a periodic axis of n planes and pitch `pitch`,
// from the offset `o` of plane p (0 <= p < n, -n <= c <= n).
__device__ __forceinline__ long long plane_add(long long o, int p, int c, int n, long long pitch) {
  long long r = o + (long long)c * pitch;
  const int q = p + c;
  if (q >= n) r -= (long long)n * pitch;
  else if (q < 0) r += (long long)n * pitch;
  return r;
}

template <class R, bool EXACT, int MODE>
__global__ void __launch_bounds__(32 * kRows, sizeof(R) == 4 ? 3 : 1) k_adj_xz(AdjStageArgs<R> a) {
  const Layout &L = a.L;
  const int lane = threadIdx.x;
  const int j = blockIdx.y * kRows + threadIdx.y;
  if (j >= L.ny) return;  // whole warp
  const int xs = blockIdx.x * kSeg;
  const int x = xs - 3 + lane;
  const int xw = wrapi(x, L.nx);
  const bool own = lane >= 3 && lane < 3 + kSeg && x < L.nx;
  const int z0 = blockIdx.z * a.zchunk;
  const int zend = min(z0 + a.zchunk, L.nz);
  const int nz = L.nz;
  const R dt = a.dt, msc = a.mscale, ix = a.inv[0], iz = a.inv[2];
  const long long pz = L.pz;
  const long long row = (long long)fused::GX + L.py * (j + fused::GY);
  // x offsets of the x stencil of this lane's cell, s(x-3 .. x+3), relative to the row
  int xo[7];
#pragma unroll
  for (int q = 0; q < 7; q++) xo[q] = wrapi(x - 3 + q, L.nx) - xw;
  const long long col = row + xw;  // this lane's column; plane offsets are added
  const R *s = a.s + col;
  const R *M = a.M + col;
  // plane cursor: offset of plane kk (wrapped) and its index
  int zk = wrapi(z0 - 3, nz);
  long long ok = pz * (long long)(zk + fused::GZ);

  // dw: the scaled differences along the march of the cell being linearised
  // (slid one face per step), last: the newest value they reach
  R dw[6], mring[4], F[6], last;
  R prevV = R(0);
  {
    R w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = s[plane_add(ok, zk, q - 3, nz, pz)];
      F[q] = R(0);
    }
    dw[0] = R(0);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = (w[f + 1] - w[f]) * iz;
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = R(0);
  R cs = s[plane_add(ok, zk, 3, nz, pz)], cm = M[ok];
  Coef<R> cv = load_coef<R, MODE>(a, 2, col + ok);
  R xsn[7];
  Coef<R> xvn;
  {
    const long long o = plane_add(ok, zk, 3, nz, pz);  // plane z0
#pragma unroll
    for (int q = 0; q < 7; q++) xsn[q] = s[o + xo[q]];
    xvn = load_coef<R, MODE>(a, 0, col + o);
  }

  for (int kk = z0 - 3; kk < zend + 3; kk++) {
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = (cs - last) * iz;
    last = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = msc * cm;
    const Coef<R> uz = cv;
    const long long okk = ok;  // plane kk
    const int zkk = zk;
    // advance the cursor to plane kk + 1 and prefetch the next column values
    ok = plane_add(ok, zk, 1, nz, pz);
    zk = (zk + 1 == nz) ? 0 : zk + 1;
    if (kk + 1 < zend + 3) {
      cs = s[plane_add(ok, zk, 3, nz, pz)];
      cm = M[ok];
      cv = load_coef<R, MODE>(a, 2, col + ok);
    }
    R G[6];
    const R gz = coef_slots_d<R, EXACT, MODE>(dw, uz, 2, mring[3], dt, iz, G);
    if (MODE == ADJ_ADV && a.gvel[2] && own && kk >= z0 && kk < zend) a.gvel[2][col + okk] += gz;
    const R Az = ring_step<R>(F, prevV, G);
    const int k = kk - 3;
    if (k < z0) continue;

    // x slots of (x, j, k); the warp sums the x faces with shuffles
    R w7[7];
#pragma unroll
    for (int q = 0; q < 7; q++) w7[q] = xsn[q];
    const Coef<R> ux = xvn;
    const long long ob = plane_add(okk, zkk, -3, nz, pz);  // plane k
    if (k + 1 < zend) {
      const long long o = plane_add(okk, zkk, -2, nz, pz);
#pragma unroll
      for (int q = 0; q < 7; q++) xsn[q] = s[o + xo[q]];
      xvn = load_coef<R, MODE>(a, 0, col + o);
    }
    const R gx = coef_slots<R, EXACT, MODE>(w7, ux, 0, mring[0], dt, ix, G);
    const long long c = col + ob;
    if (MODE == ADJ_ADV && a.gvel[0] && own) a.gvel[0][c] += gx;
    // Vbar(x) = sum_m G_m(x + 2 - m): lane + 2 - m; valid for lanes 3..29
    R V = R(0);
#pragma unroll
    for (int m = 0; m < 6; m++) V += __shfl_sync(0xffffffffu, G[m], (lane + 2 - m) & 31);
    const R Ax = V - __shfl_sync(0xffffffffu, V, (lane + 1) & 31);
    if (!own) continue;
    R o = mring[0] + (Ax + Az);
    if (a.P) o += a.pscale * a.P[c];
    if (a.Q) o += a.qscale * a.Q[c];
    a.out[c] = o;
  }
}

// Row form of k_adj_xz for rows of at most kRowMax cells: a CTA of
// ceil(nx/32) warps owns a whole x row (every cell of it written, no halo
// lanes) and marches along z; per output plane each lane puts its x slots in
// shared memory (two buffers, one barrier per plane) and sums its two x faces
// from its neighbours' slots with periodic wrap.
template <class R, bool EXACT, int MODE>
__global__ void __launch_bounds__(kRowMax, sizeof(R) == 4 ? LSMGPU_ADJ_ROW_CTAS : 1) k_adj_xz_row(AdjStageArgs<R> a) {
  extern __shared__ __align__(16) unsigned char xr_smem[];
  const Layout &L = a.L;
  const int nx = L.nx, nz = L.nz;
  const int npad = blockDim.y * 32;
  R *buf = reinterpret_cast<R *>(xr_smem);  // [2][6][npad]
  const int lane = threadIdx.x;
  const int x = threadIdx.y * 32 + lane;
  const bool own = x < nx;
  const int j = blockIdx.x;
  const int z0 = blockIdx.y * a.zchunk;
  const int zend = min(z0 + a.zchunk, nz);
  const R dt = a.dt, msc = a.mscale, ix = a.inv[0], iz = a.inv[2];
  const long long pz = L.pz;
  const long long row = (long long)fused::GX + L.py * (j + fused::GY);
  const int xc = own ? x : nx - 1;  // idle lanes shadow the last cell
  int xo[7], xn[7];  // stencil offsets relative to the cell; wrapped neighbour cells x-3 .. x+3
#pragma unroll
  for (int q = 0; q < 7; q++) {
    xn[q] = wrapi(xc - 3 + q, nx);
    xo[q] = xn[q] - xc;
  }
  const long long col = row + xc;
  const R *s = a.s + col;
  const R *M = a.M + col;
  int zk = wrapi(z0 - 3, nz);
  long long ok = pz * (long long)(zk + fused::GZ);

  // dw: the scaled differences along the march of the cell being linearised
  // (slid one face per step), last: the newest value they reach
  R dw[6], mring[4], F[6], last;
  R prevV = R(0);
  {
    R w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = s[plane_add(ok, zk, q - 3, nz, pz)];
      F[q] = R(0);
    }
    dw[0] = R(0);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = (w[f + 1] - w[f]) * iz;
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = R(0);
  R cs = s[plane_add(ok, zk, 3, nz, pz)], cm = M[ok];
  Coef<R> cv = load_coef<R, MODE>(a, 2, col + ok);
  R xsn[7];
  Coef<R> xvn;
  {
    const long long o = plane_add(ok, zk, 3, nz, pz);  // plane z0
#pragma unroll
    for (int q = 0; q < 7; q++) xsn[q] = s[o + xo[q]];
    xvn = load_coef<R, MODE>(a, 0, col + o);
  }
  int b = 0;
  for (int kk = z0 - 3; kk < zend + 3; kk++) {
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = (cs - last) * iz;
    last = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = msc * cm;
    const Coef<R> uz = cv;
    const long long okk = ok;
    const int zkk = zk;
    ok = plane_add(ok, zk, 1, nz, pz);
    zk = (zk + 1 == nz) ? 0 : zk + 1;
    if (kk + 1 < zend + 3) {
      cs = s[plane_add(ok, zk, 3, nz, pz)];
      cm = M[ok];
      cv = load_coef<R, MODE>(a, 2, col + ok);
    }
    // accumulators' old values and the P / Q terms are loaded ahead of the
    // slot evaluations that precede their use (distinct arrays)
    const bool gzw = MODE == ADJ_ADV && a.gvel[2] && own && kk >= z0 && kk < zend;
    const R gz_old = gzw ? a.gvel[2][col + okk] : R(0);
    R G[6];
    const R gz = coef_slots_d<R, EXACT, MODE>(dw, uz, 2, mring[3], dt, iz, G);
    if (gzw) a.gvel[2][col + okk] = gz_old + gz;
    const R Az = ring_step<R>(F, prevV, G);
    const int k = kk - 3;
    if (k < z0) continue;  // uniform over the CTA

    R w7[7];
#pragma unroll
    for (int q = 0; q < 7; q++) w7[q] = xsn[q];
    const Coef<R> ux = xvn;
    const long long ob = plane_add(okk, zkk, -3, nz, pz);  // plane k
    if (k + 1 < zend) {
      const long long o = plane_add(okk, zkk, -2, nz, pz);
#pragma unroll
      for (int q = 0; q < 7; q++) xsn[q] = s[o + xo[q]];
      xvn = load_coef<R, MODE>(a, 0, col + o);
    }
    const long long c = col + ob;
    const bool gxw = MODE == ADJ_ADV && a.gvel[0] && own;
    const R gx_old = gxw ? a.gvel[0][c] : R(0);
    const R p_c = (a.P && own) ? a.P[c] : R(0), q_c = (a.Q && own) ? a.Q[c] : R(0);
    const R gx = coef_slots<R, EXACT, MODE>(w7, ux, 0, mring[0], dt, ix, G);
    if (gxw) a.gvel[0][c] = gx_old + gx;
    R *bb = buf + b * 6 * npad;
    if (own) {
#pragma unroll
      for (int m = 0; m < 6; m++) bb[m * npad + x] = G[m];
    }
    __syncthreads();
    // Vbar(x) - Vbar(x+1) = sum_m G_m(x + 2 - m) - G_m(x + 3 - m)
    R Ax = R(0);
#pragma unroll
    for (int m = 0; m < 6; m++) Ax += bb[m * npad + xn[5 - m]] - bb[m * npad + xn[6 - m]];
    b ^= 1;
    if (!own) continue;
    R o = mring[0] + (Ax + Az);
    if (a.P) o += a.pscale * p_c;
    if (a.Q) o += a.qscale * q_c;
    a.out[c] = o;
  }
}

template <class R, bool EXACT, int MODE>
__global__ void __launch_bounds__(32 * kRows, sizeof(R) == 4 ? LSMGPU_ADJ_Y_CTAS : 1) k_adj_y(AdjStageArgs<R> a) {
  const Layout &L = a.L;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int k = blockIdx.y * kRows + threadIdx.y;
  if (i >= L.nx || k >= L.nz) return;
  const int y0 = blockIdx.z * a.ychunk;
  const int yend = min(y0 + a.ychunk, L.ny);
  const int ny = L.ny;
  const R dt = a.dt, msc = a.mscale, iy = a.inv[1];
  const long long py = L.py;
  const long long base = (long long)(i + fused::GX) + L.pz * (long long)(k + fused::GZ);
  const R *s = a.s + base, *M = a.M + base;
  int yk = wrapi(y0 - 3, ny);
  long long ok = py * (long long)(yk + fused::GY);

  // dw: the scaled differences along the march of the cell being linearised
  // (slid one face per step), last: the newest value they reach
  R dw[6], mring[4], F[6], last;
  R prevV = R(0);
  {
    R w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = s[plane_add(ok, yk, q - 3, ny, py)];
      F[q] = R(0);
    }
    dw[0] = R(0);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = (w[f + 1] - w[f]) * iy;
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = R(0);
  R cs = s[plane_add(ok, yk, 3, ny, py)], cm = M[ok];
  Coef<R> cv = load_coef<R, MODE>(a, 1, base + ok);
  for (int jj = y0 - 3; jj < yend + 3; jj++) {
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = (cs - last) * iy;
    last = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = msc * cm;
    const Coef<R> uy = cv;
    const long long ojj = ok;
    const int yjj = yk;
    ok = plane_add(ok, yk, 1, ny, py);
    yk = (yk + 1 == ny) ? 0 : yk + 1;
    if (jj + 1 < yend + 3) {
      cs = s[plane_add(ok, yk, 3, ny, py)];
      cm = M[ok];
      cv = load_coef<R, MODE>(a, 1, base + ok);
    }
    // the accumulators' old values are loaded before the slot evaluation so
    // their latency overlaps it (out, gvel and the state arrays are distinct)
    const bool gw = MODE == ADJ_ADV && a.gvel[1] && jj >= y0 && jj < yend;
    const bool ow = jj - 3 >= y0;
    const long long tgt = base + plane_add(ojj, yjj, -3, ny, py);
    const R g_old = gw ? a.gvel[1][base + ojj] : R(0);
    const R o_old = ow ? a.out[tgt] : R(0);
    R G[6];
    const R gy = coef_slots_d<R, EXACT, MODE>(dw, uy, 1, mring[3], dt, iy, G);
    if (gw) a.gvel[1][base + ojj] = g_old + gy;
    const R Ay = ring_step<R>(F, prevV, G);
    if (!ow) continue;
    a.out[tgt] = o_old + Ay;
  }
}

// Linearisation of the reinitialization RHS (phi0 sign form, use_phi0_for_sgn
// = 1; reinitialization3d.f.in:217-256) at state s, one thread per interior
// cell.  L = sgn (1 - |grad s|_G), sgn = phi0 / sqrt(phi0^2 + dx^2),
// |grad s|_G^2 = sum_d max(u_d, w_d)^2 with u, w from the WENO5 plus/minus
// values.  Per axis the derivative follows the branch the forward's maxima
// take to exactly one of the two WENO5 values (or none): kap_d = dL/dW and
// the side bits.  The sign source's sensitivity dL/dphi0 = (1 - |grad s|_G)
// dx^2 / (phi0^2 + dx^2)^(3/2) is accumulated (times dt mu) into gp0.
template <class R, bool EXACT>
__global__ void __launch_bounds__(256) k_reinit_lin(const R *s, const R *phi0, const R *M, R mscale, R dt,
                                                    R dx_sq, R ix, R iy, R iz, Layout L, R *kx, R *ky, R *kz,
                                                    unsigned char *side, R *gp0) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= L.nx || j >= L.ny || k >= L.nz) return;
  const long long c = L.idx(i, j, k);
  const long long st[3] = {1, L.py, L.pz};
  const R inv[3] = {ix, iy, iz};
  const R pc = phi0[c];
  R kap[3] = {R(0), R(0), R(0)};
  unsigned char sb = 0;
  const bool live = EXACT ? (fabs(pc) >= Consts<double>::zero_tol) : !(fabs(pc) < R(1e-11));
  if (live) {
    R star[3], sel[3];
    int which[3];
    for (int d = 0; d < 3; d++) {
      R v[6];  // scaled D1(c-2 .. c+3)
#pragma unroll
      for (int f = -2; f <= 3; f++) v[f + 2] = (s[c + f * st[d]] - s[c + (f - 1) * st[d]]) * inv[d];
      const R gp = fused::weno<R, EXACT>(v[5], v[4], v[3], v[2], v[1]);
      const R gm = fused::weno<R, EXACT>(v[0], v[1], v[2], v[3], v[4]);
      R u, w, du, dw;
      if (pc > R(0)) {
        u = rmax(-gp, R(0)); du = (-gp > R(0)) ? R(-1) : R(0);
        w = rmax(gm, R(0));  dw = (gm > R(0)) ? R(1) : R(0);
      } else {
        u = rmax(gp, R(0));  du = (gp > R(0)) ? R(1) : R(0);
        w = rmax(-gm, R(0)); dw = (-gm > R(0)) ? R(-1) : R(0);
      }
      if (u > w) {
        star[d] = u; sel[d] = du; which[d] = du != R(0) ? 1 : 0;
      } else {
        star[d] = w; sel[d] = dw; which[d] = dw != R(0) ? 2 : 0;
      }
    }
    const R n2 = star[0] * star[0] + star[1] * star[1] + star[2] * star[2];
    const R nrm = sqrt(n2);
    const R den = pc * pc + dx_sq;
    const R sq = sqrt(den);
    const R sgn = pc / sq;
    const R mu = mscale * M[c];
    gp0[c] += dt * mu * (R(1) - nrm) * dx_sq / (den * sq);
    if (nrm > R(0)) {
      for (int d = 0; d < 3; d++) {
        if (!which[d]) continue;
        kap[d] = -sgn * star[d] / nrm * sel[d];
        sb |= (unsigned char)(which[d] << (2 * d));
      }
    }
  }
  kx[c] = kap[0];
  ky[c] = kap[1];
  kz[c] = kap[2];
  side[c] = sb;
}

template <class R>
__global__ void k_add_interior(R *dst, const R *src, Layout L) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= L.nx || j >= L.ny || k >= L.nz) return;
  const long long c = L.idx(i, j, k);
  dst[c] += src[c];
}

// Objective terms per interior cell (in FP64): h = H(phi_T) - H(phi_target),
// lam = 2 h delta(phi_T) dV; per-block sums of h^2 in a fixed order.
static __device__ __forceinline__ double heaviside(double x, double eps) {
  // LSM_HEAVISIDE, lsm_calculus_toolbox.h:41-45
  if (x < -eps) return 0.0;
  if (x > eps) return 1.0;
  return 0.5 * (1 + x / eps + 1 / M_PI * sin(M_PI * x / eps));
}
static __device__ __forceinline__ double delta_fn(double x, double eps) {
  // LSM_DELTA_FUNCTION, lsm_calculus_toolbox.h:58-62
  if (x < -eps) return 0.0;
  if (x > eps) return 0.0;
  return 0.5 / eps * (1 + cos(M_PI * x / eps));
}

constexpr int kObjThreads = 256;

// FP32 forms of H and delta for FP32 states (the sums stay FP64)
static __device__ __forceinline__ float heaviside_f(float x, float eps) {
  if (x < -eps) return 0.f;
  if (x > eps) return 1.f;
  return 0.5f * (1.f + x / eps + (1.f / 3.14159265358979f) * sinf(3.14159265358979f * x / eps));
}
static __device__ __forceinline__ float delta_f(float x, float eps) {
  if (x < -eps) return 0.f;
  if (x > eps) return 0.f;
  return 0.5f / eps * (1.f + cosf(3.14159265358979f * x / eps));
}

template <class R>
__global__ void __launch_bounds__(kObjThreads) k_objective(const R *phiT, const R *tgt, Layout L, double eps,
                                                           double vol, R *lam, double *partial) {
  const long long n = (long long)L.nx * L.ny * L.nz;
  const long long e = (long long)blockIdx.x * kObjThreads + threadIdx.x;
  double h2 = 0.0;
  if (e < n) {
    const int i = (int)(e % L.nx);
    const int j = (int)((e / L.nx) % L.ny);
    const int k = (int)(e / ((long long)L.nx * L.ny));
    const long long c = L.idx(i, j, k);
    double h, dl;
    if constexpr (sizeof(R) == 4) {
      // FP32 state: H and delta in FP32 (FP64 sin/cos would dominate the
      // forward pass on this GPU), h^2 and the sum in FP64
      const float p = (float)phiT[c], ef = (float)eps;
      h = (double)(heaviside_f(p, ef) - heaviside_f((float)tgt[c], ef));
      dl = (double)delta_f(p, ef);
    } else {
      const double p = (double)phiT[c];
      h = heaviside(p, eps) - heaviside((double)tgt[c], eps);
      dl = delta_fn(p, eps);
    }
    h2 = h * h;
    if (lam) lam[c] = (R)(2.0 * h * dl * vol);
  }
  for (int o = 16; o > 0; o >>= 1) h2 += __shfl_xor_sync(0xffffffffu, h2, o);
  __shared__ double ws[kObjThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = h2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int w = 0; w < kObjThreads / 32; w++) b += ws[w];
    partial[blockIdx.x] = b;
  }
}

static __global__ void __launch_bounds__(1024) k_objective_fold(const double *partial, int nblocks, double vol,
                                                         double *J) {
  __shared__ double s[1024];
  double b = 0.0;
  for (int q = threadIdx.x; q < nblocks; q += blockDim.x) b += partial[q];
  s[threadIdx.x] = b;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) *J = s[0] * vol;
}

// periodic images in the 3 ghost layers of a padded-layout field
template <class R>
__global__ void k_fill_periodic(R *f, Layout L) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 3;
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y) - 3;
  const int k = (int)(blockIdx.z * blockDim.z + threadIdx.z) - 3;
  if (i > L.nx + 2 || j > L.ny + 2 || k > L.nz + 2) return;
  if (i >= 0 && i < L.nx && j >= 0 && j < L.ny && k >= 0 && k < L.nz) return;
  f[L.idx(i, j, k)] = f[L.idx(wrapi(i, L.nx), wrapi(j, L.ny), wrapi(k, L.nz))];
}

// caller's ghost-box array <- interior of a padded-layout field; every other
// entry of the caller's array is set to zero
template <class R>
__global__ void k_unpack_interior(View<R> dst, Box gb, const R *src, Layout L, int ilo, int jlo, int klo) {
  const int gi = gb.lo[0] + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int gj = gb.lo[1] + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int gk = gb.lo[2] + (int)(blockIdx.z * blockDim.z + threadIdx.z);
  if (gi > gb.hi[0] || gj > gb.hi[1] || gk > gb.hi[2]) return;
  const int i = gi - ilo, j = gj - jlo, k = gk - klo;
  R v = R(0);
  if (i >= 0 && i < L.nx && j >= 0 && j < L.ny && k >= 0 && k < L.nz) v = src[L.idx(i, j, k)];
  dst(gi, gj, gk) = v;
}

}  // namespace adj
}  // namespace lsmgpu
