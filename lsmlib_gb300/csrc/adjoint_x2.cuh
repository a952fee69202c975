// FP32 reverse stages on two lines at once (Blackwell's packed FP32x2
// instructions), for grids whose x rows fit one CTA (nx <= kRowMax).
//
// The arithmetic is that of k_adj_xz_row / k_adj_y in adjoint.cuh (same
// slots, same face sums) evaluated for two independent lines per thread,
// one in each lane of a float2.  Three launches per reverse stage:
//   k_adj_x_x2: a CTA owns two x rows (j, j+1) and a chunk of planes; per
//     plane the rows' values are staged in shared memory (scaled by 1/dx,
//     with periodic copies at the row ends) and the x slots exchanged there;
//     writes out = mu + A_x (+ P, Q terms).  No state is carried between
//     planes, so the kernel needs few registers and no warm-up planes.
//   k_adj_march_x2<AX>: a thread owns two lines along y (AX = 1, the lines
//     at z = k, k+1) or z (AX = 2, at y = j, j+1) and marches them with a
//     register window and a face-sum ring; adds A_AX to out.
// The slot evaluation (lin_slots_x2) is the FP32 epsilon-scaled WENO5
// derivative of lin_slots_f32 written for packed lanes: per lane only the
// stencil orientation, the epsilon maximum and its argument are selected.
#pragma once

#include "adjoint.cuh"
#include "reinit_x2.cuh"

namespace lsmgpu {
namespace adj {

using fused::add2;
using fused::fma2;
using fused::max3f;
using fused::mul2;
using fused::rcp2;
using fused::sp;
using fused::sub2;

// Face adjoints G[m] (faces c-2+m) of one cell on each of two lines.
// D[f] = (s(c-2+f) - s(c-3+f)) / dx along the axis, yb = dt mu kap / dx per
// line (zero where the cell has no term), mx / my = minus side of each line's
// cell.  Returns the WENO5 value W of each line.
//
// With q_k = S_k / eps + 1 and alpha_k ~ d_k / q_k^2 the weights are
// w_k = n_k / sum(n), n = (q2 q3)^2, 6 (q1 q3)^2, 3 (q1 q2)^2, and
//   dW/dv = sum_k w_k dp_k/dv + sum_k beta_k (dS_k/dv + deps/dv),
//   beta_k = -2 w_k (p_k - W) / (S_k + eps) = -8 s w_k (p_k - W) q_jl / (q1 q2 q3)
// with s = 1 / (4 eps); the adjoint weight yb is folded in before the
// indicator derivatives (bh_k = yb beta_k / 2).  eps = 1e-6 max v^2 + 1e-36;
// its derivative goes to the last index of the maximum, as in the FP64 form.
// ORIENT: 0 = per lane (mx, my), 1 = both lanes minus, 2 = both lanes plus.
template <int ORIENT>
__device__ __forceinline__ float2 lin_slots_x2(const float2 D[6], float2 yb, bool mx, bool my, float2 G[6]) {
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float c133 = 13.f / 3.f;
  // the minus-side value a or the plus-side value b of each lane
  auto pick = [&](float2 a, float2 b) {
    if constexpr (ORIENT == 1) return a;
    else if constexpr (ORIENT == 2) return b;
    else return make_float2(mx ? a.x : b.x, my ? a.y : b.y);
  };
  float2 v[5], sq[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    v[q] = pick(D[q], D[5 - q]);
    sq[q] = mul2(v[q], v[q]);
  }
  const float2 m = make_float2(max3f(max3f(sq[0].x, sq[1].x, sq[2].x), sq[3].x, sq[4].x),
                               max3f(max3f(sq[0].y, sq[1].y, sq[2].y), sq[3].y, sq[4].y));
  // s4n = -4 s = -1 / eps
  const float2 s4 = rcp2(fma2(sp(4e-6f), m, sp(4e-36f)));
  const float2 p1 = fma2(sp(c13), v[0], fma2(sp(-c76), v[1], mul2(sp(c116), v[2])));
  const float2 p2 = fma2(sp(-c16), v[1], fma2(sp(c56), v[2], mul2(sp(c13), v[3])));
  const float2 p3 = fma2(sp(c13), v[2], fma2(sp(c56), v[3], mul2(sp(-c16), v[4])));
  // second differences t_k and the asymmetric parts u_k of the indicators:
  // u1 = v1 - 4 v2 + 3 v3 = 2 t1 + (v3 - v1), u2 = v2 - v4,
  // u3 = 3 v3 - 4 v4 + v5 = 2 t3 - (v5 - v3)
  const float2 t1 = fma2(sp(-2.f), v[1], add2(v[0], v[2]));
  const float2 t2 = fma2(sp(-2.f), v[2], add2(v[1], v[3]));
  const float2 t3 = fma2(sp(-2.f), v[3], add2(v[2], v[4]));
  const float2 u1 = fma2(sp(2.f), t1, sub2(v[2], v[0]));
  const float2 u2 = sub2(v[1], v[3]);
  const float2 u3 = fma2(sp(2.f), t3, sub2(v[2], v[4]));
  const float2 tc1 = mul2(sp(c133), t1), tc2 = mul2(sp(c133), t2), tc3 = mul2(sp(c133), t3);
  // q_k = 4 S_k s + 1, 4 S_k = 13/3 t_k^2 + u_k^2
  const float2 q1 = fma2(fma2(tc1, t1, mul2(u1, u1)), s4, sp(1.f));
  const float2 q2 = fma2(fma2(tc2, t2, mul2(u2, u2)), s4, sp(1.f));
  const float2 q3 = fma2(fma2(tc3, t3, mul2(u3, u3)), s4, sp(1.f));
  const float2 q23 = mul2(q2, q3), q13 = mul2(q1, q3), q12 = mul2(q1, q2);
  const float2 n1 = mul2(q23, q23), n2 = mul2(mul2(sp(6.f), q13), q13), n3 = mul2(mul2(sp(3.f), q12), q12);
  const float2 is = rcp2(add2(add2(n1, n2), n3));  // sum <= 1e32 < 2^126
  const float2 w1 = mul2(n1, is), w2 = mul2(n2, is), w3 = mul2(n3, is);
  const float2 W = fma2(w1, p1, fma2(w2, p2, mul2(w3, p3)));
  // bh_k = yb beta_k / 2 = k0 w_k q_jl (p_k - W), k0 = -4 yb s / (q1 q2 q3)
  const float2 k0 = mul2(mul2(mul2(sp(-4.f), yb), s4), rcp2(mul2(q12, q3)));
  const float2 b1 = mul2(mul2(k0, mul2(w1, q23)), sub2(p1, W));
  const float2 b2 = mul2(mul2(k0, mul2(w2, q13)), sub2(p2, W));
  const float2 b3 = mul2(mul2(k0, mul2(w3, q12)), sub2(p3, W));
  const float2 y1 = mul2(yb, w1), y2 = mul2(yb, w2), y3 = mul2(yb, w3);
  // yb beta_k dS_k = T_k dt_k + U_k du_k with T_k = 13/3 t_k bh_k, U_k = u_k bh_k
  const float2 T1 = mul2(tc1, b1), U1 = mul2(u1, b1);
  const float2 T2 = mul2(tc2, b2), U2 = mul2(u2, b2);
  const float2 T3 = mul2(tc3, b3), U3 = mul2(u3, b3);
  float2 g[5];
  g[0] = fma2(sp(c13), y1, add2(T1, U1));
  g[1] = fma2(sp(-c76), y1, fma2(sp(-c16), y2, fma2(sp(-2.f), T1, fma2(sp(-4.f), U1, add2(T2, U2)))));
  g[2] = fma2(sp(c116), y1, fma2(sp(c56), y2, fma2(sp(c13), y3,
             fma2(sp(3.f), U1, fma2(sp(-2.f), T2, fma2(sp(3.f), U3, add2(T1, T3)))))));
  g[3] = fma2(sp(c13), y2, fma2(sp(c56), y3, fma2(sp(-2.f), T3, fma2(sp(-4.f), U3, sub2(T2, U2)))));
  g[4] = fma2(sp(-c16), y3, add2(T3, U3));
  // yb beta_k deps, deps = 2e-6 v_am dv_am at the last index of the maximum
  const float2 de = mul2(sp(4e-6f), add2(add2(b1, b2), b3));
  bool fx = false, fy = false;
#pragma unroll
  for (int q = 4; q >= 0; q--) {
    const bool hx = !fx && sq[q].x == m.x, hy = !fy && sq[q].y == m.y;
    fx = fx || hx;
    fy = fy || hy;
    const float2 e = mul2(de, v[q]);
    g[q].x = hx ? g[q].x + e.x : g[q].x;
    g[q].y = hy ? g[q].y + e.y : g[q].y;
  }
  // minus: v_q on face c-2+q (slot q); plus: v_q on face c+3-q (slot 5-q)
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const float2 lo = k < 5 ? g[k] : sp(0.f), hi = k > 0 ? g[5 - k] : sp(0.f);
    G[k] = pick(lo, hi);
  }
  return W;
}

// lin_slots_x2 with the orientation resolved per warp where all its lanes
// take the same side (the common case: the upwind side follows the sign of a
// smooth coefficient field), per lane otherwise
__device__ __forceinline__ float2 lin_slots_x2_any(const float2 D[6], float2 yb, bool mx, bool my, float2 G[6]) {
  const unsigned act = __activemask();
  if (!__any_sync(act, !(mx && my))) return lin_slots_x2<1>(D, yb, mx, my, G);
  if (!__any_sync(act, mx || my)) return lin_slots_x2<2>(D, yb, mx, my, G);
  return lin_slots_x2<0>(D, yb, mx, my, G);
}

// Coefficients of one cell on two lines along axis d: the adjoint weight
// yb = dt mu kap / dx, the sides, and (advection) whether the velocity term
// is on (the forward sets W to zero where |u_d| < zero_tol).
template <int MODE>
struct Coef2 {
  float2 k;           // ADJ_ADV: u_d; ADJ_LIN: kap_d
  unsigned sx, sy;    // ADJ_LIN: side bytes
};

template <int MODE>
__device__ __forceinline__ Coef2<MODE> load_coef2(const AdjStageArgs<float> &a, int d, long long c0, long long c1) {
  Coef2<MODE> cf;
  if constexpr (MODE == ADJ_ADV) {
    cf.k = make_float2(a.vel[d][c0], a.vel[d][c1]);
    cf.sx = cf.sy = 0;
  } else {
    cf.k = make_float2(a.kap[d][c0], a.kap[d][c1]);
    cf.sx = a.side[c0];
    cf.sy = a.side[c1];
  }
  return cf;
}

// Slots of the cells of two lines along axis d; returns the velocity adjoint
// dt mu (-W) of each (advection; zero where the term is off).
// WARP_SIDES: resolve the stencil side per warp where possible
// (lin_slots_x2_any); otherwise per lane
// live: some cell of the warp has a nonzero adjoint weight mu (warp_live).
// Where mu is zero in every cell of the warp (the adjoint field spreads from
// the objective's support by the stencil reach per stage) every slot and
// velocity adjoint is exactly zero and the evaluation is skipped.
__device__ __forceinline__ bool warp_live(float2 mu) {
  return __any_sync(__activemask(), mu.x != 0.f || mu.y != 0.f);
}

template <int MODE, bool WARP_SIDES>
__device__ __forceinline__ float2 coef_slots_x2(const float2 D[6], const Coef2<MODE> &cf, int d, float2 mu,
                                                float2 dt_inv, float dt, float2 G[6], bool live) {
  if (!live) {
#pragma unroll
    for (int m = 0; m < 6; m++) G[m] = sp(0.f);
    return sp(0.f);
  }
  auto slots = [&](float2 yb, bool mx, bool my) {
    if constexpr (WARP_SIDES) return lin_slots_x2_any(D, yb, mx, my, G);
    else return lin_slots_x2<0>(D, yb, mx, my, G);
  };
  if constexpr (MODE == ADJ_ADV) {
    const bool onx = !(fabsf(cf.k.x) < 1e-11f), ony = !(fabsf(cf.k.y) < 1e-11f);
    const float2 kap = make_float2(onx ? -cf.k.x : 0.f, ony ? -cf.k.y : 0.f);
    const float2 yb = mul2(mul2(dt_inv, mu), kap);
    const float2 W = slots(yb, cf.k.x > 0.f, cf.k.y > 0.f);
    const float2 gv = mul2(mul2(sp(-dt), mu), W);
    return make_float2(onx ? gv.x : 0.f, ony ? gv.y : 0.f);
  } else {
    const unsigned bx = (cf.sx >> (2 * d)) & 3u, by = (cf.sy >> (2 * d)) & 3u;
    const float2 kap = make_float2(bx ? cf.k.x : 0.f, by ? cf.k.y : 0.f);
    slots(mul2(mul2(dt_inv, mu), kap), bx == 2u, by == 2u);
    return sp(0.f);
  }
}

// face-sum ring of a marching thread (ring_step of adjoint.cuh on two lines)
__device__ __forceinline__ float2 ring_step2(float2 F[6], float2 &prevV, const float2 G[6]) {
#pragma unroll
  for (int m = 0; m < 6; m++) F[m] = add2(F[m], G[m]);
  const float2 A = sub2(prevV, F[0]);
  prevV = F[0];
#pragma unroll
  for (int m = 0; m < 5; m++) F[m] = F[m + 1];
  F[5] = sp(0.f);
  return A;
}

// A plane (or row) of a periodic axis of n cells and its element offset in
// the padded layout (g ghost layers); the two-line kernels index with 32-bit
// element offsets (grids of fewer than 2^31 padded elements).
struct Cursor {
  int p;
  unsigned off;
};
// cursor at p, -n <= p < 2n
__device__ __forceinline__ Cursor cursor_at(int p, int n, unsigned pitch, int g) {
  p = p < 0 ? p + n : (p >= n ? p - n : p);
  return Cursor{p, pitch * (unsigned)(p + g)};
}
__device__ __forceinline__ Cursor cursor_next(Cursor c, int n, unsigned pitch) {
  c.p++;
  c.off += pitch;
  if (c.p == n) {
    c.p = 0;
    c.off -= (unsigned)n * pitch;
  }
  return c;
}

// shared memory of k_adj_x_x2: two buffers of both rows' s / dx and two of
// the six x slots, each row of nx + 6 float2 (3 periodic copies per end)
__host__ __device__ constexpr size_t adj_x_x2_smem(int nx) { return (size_t)(2 + 2 * 6) * (nx + 6) * sizeof(float2); }
#ifndef LSMGPU_ADJ_X_X2_NREG
#define LSMGPU_ADJ_X_X2_NREG 80
#endif

// x faces of a chunk of planes of two x rows (j, j+1): per plane each thread
// stages its column value (times 1/dx) with periodic copies at the row ends,
// evaluates its cell's x slots from the staged row and exchanges them; one
// barrier per plane (the staging of plane k+1 and the slots of plane k share
// it).  Writes out = mu + A_x (+ P, Q terms).
template <int MODE>
__global__ void __maxnreg__(LSMGPU_ADJ_X_X2_NREG) k_adj_x_x2(AdjStageArgs<float> a) {
  extern __shared__ __align__(16) unsigned char x2_smem[];
  const Layout &L = a.L;
  const int nx = L.nx, nz = L.nz;
  const int hp = nx + 6;
  float2 *sbuf = reinterpret_cast<float2 *>(x2_smem);  // [2][hp]
  float2 *gbuf = sbuf + 2 * hp;                        // [2][6][hp]
  const int x = threadIdx.y * 32 + threadIdx.x;
  const bool own = x < nx;
  const int xc = own ? x : nx - 1;  // idle lanes shadow the last cell
  const int j0 = 2 * blockIdx.x;
  const int j1 = j0 + 1 < L.ny ? j0 + 1 : j0;  // odd ny: the last CTA's second row repeats the first
  const bool two = j1 != j0;
  const int z0 = blockIdx.y * a.xchunk;
  if (z0 >= nz) return;  // whole CTA, before any barrier
  const int zend = min(z0 + a.xchunk, nz);
  const float dt = a.dt;
  const float2 msc = sp(a.mscale), ix = sp(a.inv[0]), dtix = sp(a.dt * a.inv[0]);
  const unsigned pz = (unsigned)L.pz;
  const unsigned col0 = (unsigned)(fused::GX + xc) + (unsigned)L.py * (unsigned)(j0 + fused::GY);
  const unsigned col1 = (unsigned)(fused::GX + xc) + (unsigned)L.py * (unsigned)(j1 + fused::GY);
  const int p_main = xc + 3;
  const int p_copy = xc < 3 ? nx + 3 + xc : (xc >= nx - 3 ? xc - (nx - 3) : -1);
  auto ld2 = [&](const float *p, unsigned o) { return make_float2(p[col0 + o], p[col1 + o]); };
  auto stage_s = [&](float2 *row, float2 v) {
    if (own) {
      const float2 sv = mul2(v, ix);
      row[p_main] = sv;
      if (p_copy >= 0) row[p_copy] = sv;
    }
  };

  unsigned ok = pz * (unsigned)(z0 + fused::GZ);
  stage_s(sbuf + (z0 & 1) * hp, ld2(a.s, ok));  // plane k is read from buffer k & 1
  // the next plane's values are loaded one plane ahead
  float2 sn = sp(0.f), mn = ld2(a.M, ok);
  Coef2<MODE> cn = load_coef2<MODE>(a, 0, col0 + ok, col1 + ok);
  if (z0 + 1 < zend) sn = ld2(a.s, ok + pz);
  __syncthreads();
  for (int k = z0; k < zend; k++) {
    const int b = k & 1;
    const float2 mu = mul2(msc, mn);
    const Coef2<MODE> ux = cn;
    const float2 s_next = sn;
    const unsigned okn = ok + pz;
    const bool more = k + 1 < zend;
    if (more) {
      mn = ld2(a.M, okn);
      cn = load_coef2<MODE>(a, 0, col0 + okn, col1 + okn);
      if (k + 2 < zend) sn = ld2(a.s, okn + pz);
    }
    const bool live = warp_live(mu);
    const bool gxw = MODE == ADJ_ADV && a.gvel[0] && own && live;
    float2 gx_old = sp(0.f), pq = sp(0.f);
    if (gxw) gx_old = ld2(a.gvel[0], ok);
    if (own) {
      if (a.P) pq = mul2(sp(a.pscale), ld2(a.P, ok));
      if (a.Q) pq = fma2(sp(a.qscale), ld2(a.Q, ok), pq);
    }
    float2 D[6];
    {
      const float2 *rw = sbuf + b * hp + xc;
      float2 w7[7];
#pragma unroll
      for (int q = 0; q < 7; q++) w7[q] = rw[q];
#pragma unroll
      for (int f = 0; f < 6; f++) D[f] = sub2(w7[f + 1], w7[f]);
    }
    float2 G[6];
    const float2 gx = coef_slots_x2<MODE, true>(D, ux, 0, mu, dtix, dt, G, live);
    if (gxw) {
      a.gvel[0][col0 + ok] = gx_old.x + gx.x;
      if (two) a.gvel[0][col1 + ok] = gx_old.y + gx.y;
    }
    float2 *bb = gbuf + b * 6 * hp;
    if (own) {
#pragma unroll
      for (int m = 0; m < 6; m++) {
        bb[m * hp + p_main] = G[m];
        if (p_copy >= 0) bb[m * hp + p_copy] = G[m];
      }
    }
    if (more) stage_s(sbuf + (b ^ 1) * hp, s_next);
    __syncthreads();
    // A(x) = Vbar(x) - Vbar(x+1) = sum_m G_m(x + 2 - m) - G_m(x + 3 - m)
    float2 Ax = sp(0.f);
#pragma unroll
    for (int m = 0; m < 6; m++) Ax = add2(Ax, sub2(bb[m * hp + xc + 5 - m], bb[m * hp + xc + 6 - m]));
    if (own) {
      const float2 o = add2(add2(mu, Ax), pq);
      a.out[col0 + ok] = o.x;
      if (two) a.out[col1 + ok] = o.y;
    }
    ok = okn;
  }
}

// CTAs of 32 x kMarchRows threads (line pairs), LSMGPU_ADJ_MARCH_X2_CTAS
// resident per SM
constexpr int kMarchRows = 4;
#ifndef LSMGPU_ADJ_MARCH_X2_CTAS
#define LSMGPU_ADJ_MARCH_X2_CTAS 4
#endif
// per-warp stencil sides in the march kernels (with per-lane sides only, the
// kernels fit 96 registers, five CTAs per SM; measured at 192^3, the per-warp
// sides at four CTAs are faster)
#ifndef LSMGPU_ADJ_MARCH_WARP_SIDES
#define LSMGPU_ADJ_MARCH_WARP_SIDES 1
#endif
// lead values and coefficients loaded this many cells ahead (1 or 2)
#ifndef LSMGPU_ADJ_MARCH_PREFETCH
#define LSMGPU_ADJ_MARCH_PREFETCH 1
#endif

// Faces along axis AX (1: y, 2: z) of a chunk of the march: a thread owns two
// lines along AX at (i, the pair 2p, 2p+1 of the remaining axis) and marches
// them with the window / face-ring scheme of k_adj_y; adds dt A_AX to out.
template <int MODE, int AX>
__global__ void __launch_bounds__(32 * kMarchRows, LSMGPU_ADJ_MARCH_X2_CTAS) k_adj_march_x2(AdjStageArgs<float> a) {
  static_assert(AX == 1 || AX == 2, "march along y or z");
  const Layout &L = a.L;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int n_pair = AX == 1 ? L.nz : L.ny;  // the axis the pairs run along
  const int q0 = 2 * (blockIdx.y * kMarchRows + threadIdx.y);
  if (i >= L.nx || q0 >= n_pair) return;
  const int q1 = q0 + 1 < n_pair ? q0 + 1 : q0;  // odd count: the last pair's second line repeats the first
  const bool two = q1 != q0;
  const int n = AX == 1 ? L.ny : L.nz;         // march length
  const int g = AX == 1 ? fused::GY : fused::GZ;
  const unsigned pm = (unsigned)(AX == 1 ? L.py : L.pz);       // march pitch
  const unsigned pq_ = (unsigned)(AX == 1 ? L.pz : L.py);      // pair pitch
  const int gq = AX == 1 ? fused::GZ : fused::GY;
  const int y0 = blockIdx.z * (AX == 1 ? a.ychunk : a.zchunk);
  const int yend = min(y0 + (AX == 1 ? a.ychunk : a.zchunk), n);
  const float dt = a.dt;
  const float2 msc = sp(a.mscale), iy = sp(a.inv[AX]), dtiy = sp(a.dt * a.inv[AX]);
  const unsigned b0 = (unsigned)(i + fused::GX) + pq_ * (unsigned)(q0 + gq);
  const unsigned b1 = (unsigned)(i + fused::GX) + pq_ * (unsigned)(q1 + gq);
  auto ld2 = [&](const float *p, unsigned o) { return make_float2(p[b0 + o], p[b1 + o]); };

  float2 dw[6], mring[4], F[6], last, prevV = sp(0.f);
  int quiet = 0;
  {
    float2 w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = ld2(a.s, cursor_at(y0 - 6 + q, n, pm, g).off);
      F[q] = sp(0.f);
    }
    dw[0] = sp(0.f);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = mul2(sub2(w[f + 1], w[f]), iy);
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = sp(0.f);
  // cursors: cell jj of the march, the cell jj + P whose values are loaded
  // (P = LSMGPU_ADJ_MARCH_PREFETCH cells ahead) and its lead cell jj + P + 3,
  // the output cell jj - 3
  constexpr int P = LSMGPU_ADJ_MARCH_PREFETCH;
  static_assert(P == 1 || P == 2, "prefetch distance 1 or 2");
  Cursor cj = cursor_at(y0 - 3, n, pm, g);
  Cursor cp = cursor_at(y0 - 3 + P, n, pm, g);
  Cursor cl = cursor_at(y0 + P, n, pm, g);
  Cursor co = cursor_at(y0, n, pm, g);
  // [0]: the values of the next step, [1]: of the step after (P = 2)
  float2 cs[P], cm[P];
  Coef2<MODE> cv[P];
  cs[0] = ld2(a.s, co.off);  // cell y0 = jj + 3 of the first step
  cm[0] = ld2(a.M, cj.off);
  cv[0] = load_coef2<MODE>(a, AX, b0 + cj.off, b1 + cj.off);
  if constexpr (P == 2) {
    const unsigned o1 = cursor_next(cj, n, pm).off;
    cs[1] = ld2(a.s, cursor_next(co, n, pm).off);
    cm[1] = ld2(a.M, o1);
    cv[1] = load_coef2<MODE>(a, AX, b0 + o1, b1 + o1);
  }
  for (int jj = y0 - 3; jj < yend + 3; jj++) {
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = mul2(sub2(cs[0], last), iy);
    last = cs[0];
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = mul2(msc, cm[0]);
    const Coef2<MODE> uy = cv[0];
    const unsigned ojj = cj.off;
    cj = cursor_next(cj, n, pm);
#pragma unroll
    for (int q = 0; q + 1 < P; q++) {
      cs[q] = cs[q + 1];
      cm[q] = cm[q + 1];
      cv[q] = cv[q + 1];
    }
    if (jj + P < yend + 3) {
      cs[P - 1] = ld2(a.s, cl.off);
      cm[P - 1] = ld2(a.M, cp.off);
      cv[P - 1] = load_coef2<MODE>(a, AX, b0 + cp.off, b1 + cp.off);
    }
    cp = cursor_next(cp, n, pm);
    cl = cursor_next(cl, n, pm);
    // warp-uniform: some cell has a nonzero weight; quiet counts the steps
    // since one had (after 7 the face ring holds only zeros and A_AX = 0)
    const bool live = warp_live(mring[3]);
    quiet = live ? 0 : quiet + 1;
    // the accumulators' old values are loaded before the slot evaluation so
    // their latency overlaps it (out, gvel and the state arrays are distinct)
    const bool gw = MODE == ADJ_ADV && a.gvel[AX] && jj >= y0 && jj < yend && live;
    const bool ow = jj - 3 >= y0;
    const bool orw = ow && quiet < 7;
    const unsigned otg = co.off;
    if (ow) co = cursor_next(co, n, pm);
    float2 g_old = sp(0.f), o_old = sp(0.f);
    if (gw) g_old = ld2(a.gvel[AX], ojj);
    if (orw) o_old = ld2(a.out, otg);
    float2 G[6];
    const float2 gy =
        coef_slots_x2<MODE, LSMGPU_ADJ_MARCH_WARP_SIDES != 0>(dw, uy, AX, mring[3], dtiy, dt, G, live);
    if (gw) {
      a.gvel[AX][b0 + ojj] = g_old.x + gy.x;
      if (two) a.gvel[AX][b1 + ojj] = g_old.y + gy.y;
    }
    const float2 Ay = ring_step2(F, prevV, G);
    if (!orw) continue;
    a.out[b0 + otg] = o_old.x + Ay.x;
    if (two) a.out[b1 + otg] = o_old.y + Ay.y;
  }
}

}  // namespace adj
}  // namespace lsmgpu
