// FP32 reverse stages on two lines at once (Blackwell's packed FP32x2
// instructions), for grids whose x rows fit one CTA (nx <= kRowMax).
//
// The arithmetic is that of k_adj_xz_row / k_adj_y in adjoint.cuh (same
// slots, same face sums) evaluated for two independent lines per thread,
// one in each lane of a float2:
//   k_adj_xz_x2: a CTA owns two x rows (j, j+1) and marches along z; lane x
//     of the pair is row j, lane y row j+1.  The x stencils come from a ring
//     of the last eight planes of both rows in shared memory (each thread
//     stores the column value it loads for the z march, scaled by 1/dx, with
//     periodic copies at the row ends), and the x slots are exchanged through
//     shared memory as in the scalar row kernel: one barrier per plane.
//   k_adj_y_x2: a thread owns the columns (i, k) and (i, k+1) and marches
//     along y.
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
__device__ __forceinline__ float2 lin_slots_x2(const float2 D[6], float2 yb, bool mx, bool my, float2 G[6]) {
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float c133 = 13.f / 3.f;
  float2 v[5], sq[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    v[q] = make_float2(mx ? D[q].x : D[5 - q].x, my ? D[q].y : D[5 - q].y);
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
    G[k] = make_float2(mx ? lo.x : hi.x, my ? lo.y : hi.y);
  }
  return W;
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
template <int MODE>
__device__ __forceinline__ float2 coef_slots_x2(const float2 D[6], const Coef2<MODE> &cf, int d, float2 mu,
                                                float2 dt_inv, float dt, float2 G[6]) {
  if constexpr (MODE == ADJ_ADV) {
    const bool onx = !(fabsf(cf.k.x) < 1e-11f), ony = !(fabsf(cf.k.y) < 1e-11f);
    const float2 kap = make_float2(onx ? -cf.k.x : 0.f, ony ? -cf.k.y : 0.f);
    const float2 yb = mul2(mul2(dt_inv, mu), kap);
    const float2 W = lin_slots_x2(D, yb, cf.k.x > 0.f, cf.k.y > 0.f, G);
    const float2 gv = mul2(mul2(sp(-dt), mu), W);
    return make_float2(onx ? gv.x : 0.f, ony ? gv.y : 0.f);
  } else {
    const unsigned bx = (cf.sx >> (2 * d)) & 3u, by = (cf.sy >> (2 * d)) & 3u;
    const float2 kap = make_float2(bx ? cf.k.x : 0.f, by ? cf.k.y : 0.f);
    lin_slots_x2(D, mul2(mul2(dt_inv, mu), kap), bx == 2u, by == 2u, G);
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

// shared memory of k_adj_xz_x2: an 8-plane ring of both rows' s / dx and two
// buffers of the six x slots, each row of nx + 6 float2 (3 periodic copies
// per end)
__host__ __device__ constexpr size_t adj_xz_x2_smem(int nx) { return (size_t)(8 + 2 * 6) * (nx + 6) * sizeof(float2); }

// register cap of k_adj_xz_x2: 112 per thread keeps three 192-thread CTAs
// (a 192-cell row) resident per SM without spills
#ifndef LSMGPU_ADJ_XZ_X2_NREG
#define LSMGPU_ADJ_XZ_X2_NREG 112
#endif
#define LSMGPU_ADJ_XZ_X2_BOUNDS __maxnreg__(LSMGPU_ADJ_XZ_X2_NREG)

template <int MODE>
__global__ void LSMGPU_ADJ_XZ_X2_BOUNDS k_adj_xz_x2(AdjStageArgs<float> a) {
  extern __shared__ __align__(16) unsigned char xz2_smem[];
  const Layout &L = a.L;
  const int nx = L.nx, nz = L.nz;
  const int hp = nx + 6;
  float2 *ring = reinterpret_cast<float2 *>(xz2_smem);  // [8][hp]
  float2 *gbuf = ring + 8 * hp;                        // [2][6][hp]
  const int x = threadIdx.y * 32 + threadIdx.x;
  const bool own = x < nx;
  const int xc = own ? x : nx - 1;  // idle lanes shadow the last cell
  const int j0 = 2 * blockIdx.x;
  const int j1 = j0 + 1 < L.ny ? j0 + 1 : j0;  // odd ny: the last CTA's second row repeats the first
  const bool two = j1 != j0;
  const int z0 = blockIdx.y * a.zchunk;
  const int zend = min(z0 + a.zchunk, nz);
  const float dt = a.dt;
  const float2 msc = sp(a.mscale), ix = sp(a.inv[0]), iz = sp(a.inv[2]);
  const float2 dtix = sp(a.dt * a.inv[0]), dtiz = sp(a.dt * a.inv[2]);
  const unsigned pz = (unsigned)L.pz;
  const unsigned col0 = (unsigned)(fused::GX + xc) + (unsigned)L.py * (unsigned)(j0 + fused::GY);
  const unsigned col1 = (unsigned)(fused::GX + xc) + (unsigned)L.py * (unsigned)(j1 + fused::GY);
  // shared-memory positions this thread writes: its cell and a periodic copy
  const int p_main = xc + 3;
  const int p_copy = xc < 3 ? nx + 3 + xc : (xc >= nx - 3 ? xc - (nx - 3) : -1);
  const bool wr = own;
  auto ld2 = [&](const float *p, unsigned o) { return make_float2(p[col0 + o], p[col1 + o]); };

  float2 dw[6], mring[4], F[6], last, prevV = sp(0.f);
  {
    float2 w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = ld2(a.s, cursor_at(z0 - 6 + q, nz, pz, fused::GZ).off);
      F[q] = sp(0.f);
    }
    dw[0] = sp(0.f);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = mul2(sub2(w[f + 1], w[f]), iz);
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = sp(0.f);
  // cursors: plane kk of the march, its lead plane kk + 4, the output plane kk - 3
  Cursor ck = cursor_at(z0 - 3, nz, pz, fused::GZ);
  Cursor cl = cursor_at(z0 + 1, nz, pz, fused::GZ);
  Cursor co = cursor_at(z0, nz, pz, fused::GZ);
  float2 cs = ld2(a.s, co.off);  // plane z0 = kk + 3 of the first step
  float2 cm = ld2(a.M, ck.off);
  Coef2<MODE> cv = load_coef2<MODE>(a, 2, col0 + ck.off, col1 + ck.off);
  // x coefficient of the next output plane, loaded one plane ahead
  Coef2<MODE> cx = load_coef2<MODE>(a, 0, col0 + co.off, col1 + co.off);
  int b = 0;
  for (int kk = z0 - 3; kk < zend + 3; kk++) {
    const int k = kk - 3;
    const bool xs = k >= z0;  // an output plane (uniform over the CTA)
    const unsigned ok = co.off;
    // the x accumulator and the P / Q terms of plane k are loaded before the
    // z slot evaluation, which hides their latency
    const bool gxw = MODE == ADJ_ADV && a.gvel[0] && own && xs;
    float2 gx_old = sp(0.f), pq = sp(0.f);
    if (gxw) gx_old = ld2(a.gvel[0], ok);
    if (own && xs) {
      if (a.P) pq = mul2(sp(a.pscale), ld2(a.P, ok));
      if (a.Q) pq = fma2(sp(a.qscale), ld2(a.Q, ok), pq);
    }
    // plane kk + 3 of both rows, scaled by 1/dx, for the x stencils of plane kk + 3
    if (wr && kk + 3 < zend) {
      const float2 sv = mul2(cs, ix);
      float2 *rp = ring + ((kk + 3) & 7) * hp;
      rp[p_main] = sv;
      if (p_copy >= 0) rp[p_copy] = sv;
    }
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = mul2(sub2(cs, last), iz);
    last = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = mul2(msc, cm);
    const Coef2<MODE> uz = cv;
    const unsigned okk = ck.off;
    ck = cursor_next(ck, nz, pz);
    if (kk + 1 < zend + 3) {
      cs = ld2(a.s, cl.off);
      cm = ld2(a.M, ck.off);
      cv = load_coef2<MODE>(a, 2, col0 + ck.off, col1 + ck.off);
    }
    cl = cursor_next(cl, nz, pz);
    const bool gzw = MODE == ADJ_ADV && a.gvel[2] && own && kk >= z0 && kk < zend;
    float2 gz_old = sp(0.f);
    if (gzw) gz_old = ld2(a.gvel[2], okk);
    float2 G[6];
    const float2 gz = coef_slots_x2<MODE>(dw, uz, 2, mring[3], dtiz, dt, G);
    if (gzw) {
      a.gvel[2][col0 + okk] = gz_old.x + gz.x;
      if (two) a.gvel[2][col1 + okk] = gz_old.y + gz.y;
    }
    const float2 Az = ring_step2(F, prevV, G);
    if (!xs) continue;
    if (k == z0) __syncthreads();  // the ring's first planes were written without a barrier since

    // x slots of plane k from the ring
    const float2 *rw = ring + (k & 7) * hp + xc;
    float2 D[6];
    {
      float2 w7[7];
#pragma unroll
      for (int q = 0; q < 7; q++) w7[q] = rw[q];
#pragma unroll
      for (int f = 0; f < 6; f++) D[f] = sub2(w7[f + 1], w7[f]);
    }
    const Coef2<MODE> ux = cx;
    co = cursor_next(co, nz, pz);
    if (k + 1 < zend) cx = load_coef2<MODE>(a, 0, col0 + co.off, col1 + co.off);
    const float2 gx = coef_slots_x2<MODE>(D, ux, 0, mring[0], dtix, dt, G);
    if (gxw) {
      a.gvel[0][col0 + ok] = gx_old.x + gx.x;
      if (two) a.gvel[0][col1 + ok] = gx_old.y + gx.y;
    }
    float2 *bb = gbuf + b * 6 * hp;
    if (wr) {
#pragma unroll
      for (int m = 0; m < 6; m++) {
        bb[m * hp + p_main] = G[m];
        if (p_copy >= 0) bb[m * hp + p_copy] = G[m];
      }
    }
    __syncthreads();
    // A(x) = Vbar(x) - Vbar(x+1) = sum_m G_m(x + 2 - m) - G_m(x + 3 - m)
    float2 Ax = sp(0.f);
#pragma unroll
    for (int m = 0; m < 6; m++) Ax = add2(Ax, sub2(bb[m * hp + xc + 5 - m], bb[m * hp + xc + 6 - m]));
    b ^= 1;
    if (!own) continue;
    const float2 o = add2(add2(mring[0], add2(Ax, Az)), pq);
    a.out[col0 + ok] = o.x;
    if (two) a.out[col1 + ok] = o.y;
  }
}

// CTAs of 32 x kYRows threads (column pairs), kYCtas resident per SM
constexpr int kYRows = 4;
#ifndef LSMGPU_ADJ_Y_X2_CTAS
#define LSMGPU_ADJ_Y_X2_CTAS 5
#endif

template <int MODE>
__global__ void __launch_bounds__(32 * kYRows, LSMGPU_ADJ_Y_X2_CTAS) k_adj_y_x2(AdjStageArgs<float> a) {
  const Layout &L = a.L;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int k0 = 2 * (blockIdx.y * kYRows + threadIdx.y);
  if (i >= L.nx || k0 >= L.nz) return;
  const int k1 = k0 + 1 < L.nz ? k0 + 1 : k0;  // odd nz: the last pair's second column repeats the first
  const bool two = k1 != k0;
  const int y0 = blockIdx.z * a.ychunk;
  const int yend = min(y0 + a.ychunk, L.ny);
  const int ny = L.ny;
  const float dt = a.dt;
  const float2 msc = sp(a.mscale), iy = sp(a.inv[1]), dtiy = sp(a.dt * a.inv[1]);
  const unsigned py = (unsigned)L.py;
  const unsigned b0 = (unsigned)(i + fused::GX) + (unsigned)L.pz * (unsigned)(k0 + fused::GZ);
  const unsigned b1 = (unsigned)(i + fused::GX) + (unsigned)L.pz * (unsigned)(k1 + fused::GZ);
  auto ld2 = [&](const float *p, unsigned o) { return make_float2(p[b0 + o], p[b1 + o]); };

  float2 dw[6], mring[4], F[6], last, prevV = sp(0.f);
  {
    float2 w[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      w[q] = ld2(a.s, cursor_at(y0 - 6 + q, ny, py, fused::GY).off);
      F[q] = sp(0.f);
    }
    dw[0] = sp(0.f);
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f + 1] = mul2(sub2(w[f + 1], w[f]), iy);
    last = w[5];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = sp(0.f);
  // cursors: row jj of the march, its lead row jj + 4, the output row jj - 3
  Cursor cj = cursor_at(y0 - 3, ny, py, fused::GY);
  Cursor cl = cursor_at(y0 + 1, ny, py, fused::GY);
  Cursor co = cursor_at(y0, ny, py, fused::GY);
  float2 cs = ld2(a.s, co.off);  // row y0 = jj + 3 of the first step
  float2 cm = ld2(a.M, cj.off);
  Coef2<MODE> cv = load_coef2<MODE>(a, 1, b0 + cj.off, b1 + cj.off);
  for (int jj = y0 - 3; jj < yend + 3; jj++) {
#pragma unroll
    for (int f = 0; f < 5; f++) dw[f] = dw[f + 1];
    dw[5] = mul2(sub2(cs, last), iy);
    last = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = mul2(msc, cm);
    const Coef2<MODE> uy = cv;
    const unsigned ojj = cj.off;
    cj = cursor_next(cj, ny, py);
    if (jj + 1 < yend + 3) {
      cs = ld2(a.s, cl.off);
      cm = ld2(a.M, cj.off);
      cv = load_coef2<MODE>(a, 1, b0 + cj.off, b1 + cj.off);
    }
    cl = cursor_next(cl, ny, py);
    // the accumulators' old values are loaded before the slot evaluation so
    // their latency overlaps it (out, gvel and the state arrays are distinct)
    const bool gw = MODE == ADJ_ADV && a.gvel[1] && jj >= y0 && jj < yend;
    const bool ow = jj - 3 >= y0;
    const unsigned otg = co.off;
    if (ow) co = cursor_next(co, ny, py);
    float2 g_old = sp(0.f), o_old = sp(0.f);
    if (gw) g_old = ld2(a.gvel[1], ojj);
    if (ow) o_old = ld2(a.out, otg);
    float2 G[6];
    const float2 gy = coef_slots_x2<MODE>(dw, uy, 1, mring[3], dtiy, dt, G);
    if (gw) {
      a.gvel[1][b0 + ojj] = g_old.x + gy.x;
      if (two) a.gvel[1][b1 + ojj] = g_old.y + gy.y;
    }
    const float2 Ay = ring_step2(F, prevV, G);
    if (!ow) continue;
    a.out[b0 + otg] = o_old.x + Ay.x;
    if (two) a.out[b1 + otg] = o_old.y + Ay.y;
  }
}

}  // namespace adj
}  // namespace lsmgpu
