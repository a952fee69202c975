// FP32 reinitialization stage kernel with WENO5 windows shared between
// neighbouring cells.
//
// LSMLIB's HJ WENO5 (spatial_derivatives3d.f.in:1161-1611) reconstructs, per
// axis and cell c, a minus value from the five first differences
// D(c-2 .. c+2) and a plus value from D(c+3 .. c-1) (D(s) = phi(s) -
// phi(s-1)).  The plus window of c holds the same five differences as the
// minus window of c+1, reversed: both have the same smoothness indicators
// (permuted), the same epsilon and therefore the same weight products.  Here
// each such window W(c) = D(c-2 .. c+2) is evaluated once and feeds both
// minus(c) and plus(c-1):
//  * z: each thread marches up its column and carries the quantities of the
//    previous windows in registers (one new window per cell);
//  * x: a thread owns two x-neighbouring cells (i, i+1) as the two lanes of
//    Blackwell's packed FP32x2 instructions and evaluates W(i+1), W(i+2); the
//    minus(i+2) it produces is minus(i') of the next lane, and the indicator
//    forms of triples i-1, i come from the previous lane (warp shuffles); the
//    first lane of a row takes them from a per-tile prologue;
//  * y: each warp is one row of the tile; a thread evaluates W(j+1) and hands
//    minus(j+1) to the row above through shared memory (one barrier per
//    plane); the tile's first row takes minus(y0) from the prologue.
// The weights use the epsilon-scaled form of fused_stage.cuh (no under- or
// overflow on near-flat data), and the reconstruction is written as the
// central candidate plus third-difference corrections,
//   minus(c) = p2 + w1 (p1 - p2) + w3 (p3 - p2),
//   p1 - p2 = TD(c-2) / 3,  p3 - p2 = TD(c-1) / 6,
//   TD(s) = D(s) - 3 D(s+1) + 3 D(s+2) - D(s+3),
// which is LSMLIB's w1 p1 + w2 p2 + w3 p3 rearranged (the weights sum to 1).
// Differences are not divided by dx: WENO5 is homogeneous of degree one in
// them, so the reconstructed derivatives are scaled once at the end.
//
// Tile: 64 x 8 x RZ cells per CTA of 32 x 8 threads; the tile plus its halo
// (72 x 14 x (RZ + 6)) is staged by one TMA load.  With extrapolation
// boundary conditions the ghost cells the stencils read are computed in
// shared memory from the tile's interior cells (fill_face_ghosts in
// fused_stage.cuh), so the stage needs no separate ghost-fill launch.
#pragma once

#include "fused_stage.cuh"

namespace lsmgpu {
namespace fused {

constexpr int RX = 64, RY = 8;    // cells of a tile in x and y
constexpr int RSX = RX + 8, RSY = RY + 6;  // staged tile in x and y
constexpr int RZ = 8;             // planes of a tile (the depth the steppers launch)
// staged tile of a TILE_Z-plane tile: 72 x 14 x (TILE_Z + 6) floats
constexpr size_t reinit_x2_smem(int tile_z) { return (size_t)RSX * RSY * (tile_z + 6) * sizeof(float); }
// CTAs per SM the kernel is built for: three 8-plane tiles fit the SM's
// shared memory (67 KB each with the static arrays) and registers (80 per
// thread); a 16-plane tile needs 100 KB, so two.
constexpr int reinit_x2_ctas(int tile_z) { return tile_z <= 8 ? 3 : 2; }

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return fma2(b, sp(-1.f), a); }
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float2 rcp2(float2 x) { return make_float2(rcp_approx(x.x), rcp_approx(x.y)); }
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// A triple of consecutive differences (d0, d1, d2): its second difference t
// and the three smoothness-indicator forms it takes in a window, times 4:
//   first triple of a window:  13/3 t^2 + (d0 - 4 d1 + 3 d2)^2
//   middle triple:             13/3 t^2 + (d0 - d2)^2
//   last triple:               13/3 t^2 + (3 d0 - 4 d1 + d2)^2
// (spatial_derivatives3d.f.in:1306-1311; the outer ones are the middle form
// plus 4 t^2 -/+ 4 t (d0 - d2)).
struct Tri {
  float2 t, s1, s2, s3;
};
__device__ __forceinline__ Tri tri_forms(float2 d0, float2 d1, float2 d2) {
  Tri r;
  r.t = fma2(sp(-2.f), d1, add2(d0, d2));
  const float2 nb = sub2(d2, d0);  // -(d0 - d2)
  const float2 tt = mul2(sp(13.f / 3.f), r.t);
  r.s2 = fma2(tt, r.t, mul2(nb, nb));
  const float2 t4 = mul2(sp(4.f), r.t);
  const float2 x = fma2(t4, r.t, r.s2);
  const float2 y = mul2(t4, nb);  // -4 t (d0 - d2)
  r.s1 = add2(x, y);
  r.s3 = sub2(x, y);
  return r;
}

// Weight products of a window from its three indicator forms (x4) and the
// maximum squared difference m: q_k = 4 S_k / (4 eps) + 1 = (S_k + eps) / eps,
// eps = 1e-6 m + 1e-36 (LSMLIB's, spatial_derivatives3d.f.in:1296, in units
// of the unscaled differences); only ratios of the q_k enter the weights.
// 1 <= q_k < 4e7, so the squared products stay below 3e30.
struct WQ {
  float2 q23, q13, q12;  // (q2 q3)^2, (q1 q3)^2, (q1 q2)^2
};
__device__ __forceinline__ WQ window_q(float2 s1, float2 s2, float2 s3, float2 m) {
  const float2 s = rcp2(fma2(sp(4e-6f), m, sp(4e-36f)));  // 1 / (4 eps), finite: 4 eps >= 4e-36
  const float2 q1 = fma2(s1, s, sp(1.f)), q2 = fma2(s2, s, sp(1.f)), q3 = fma2(s3, s, sp(1.f));
  const float2 a = mul2(q2, q3), b = mul2(q1, q3), c = mul2(q1, q2);
  return {mul2(a, a), mul2(b, b), mul2(c, c)};
}

// minus(c) of window W(c):  p2 + (2 q23 TD(c-2) + 3 q12 TD(c-1)) / (6 (q23 + 6 q13 + 3 q12))
__device__ __forceinline__ float2 side_minus(const WQ &w, float2 tda, float2 tdb, float2 p2) {
  const float2 num = fma2(sp(2.f), mul2(w.q23, tda), mul2(sp(3.f), mul2(w.q12, tdb)));
  const float2 den = fma2(sp(6.f), w.q23, fma2(sp(36.f), w.q13, mul2(sp(18.f), w.q12)));
  return fma2(num, rcp2(den), p2);
}

// both sides of one window W(c): minus(c) as above and
// plus(c-1) = p2' - (2 q12 TD(c-1) + 3 q23 TD(c-2)) / (6 (q12 + 6 q13 + 3 q23))
__device__ __forceinline__ void sides_both(const WQ &w, float2 tda, float2 tdb, float2 p2m, float2 p2p,
                                           float2 &minus, float2 &plus) {
  const float2 u = mul2(w.q23, tda), v = mul2(w.q12, tdb);
  const float2 g = mul2(sp(36.f), w.q13);
  const float2 num_m = fma2(sp(2.f), u, mul2(sp(3.f), v));
  const float2 num_p = fma2(sp(3.f), u, mul2(sp(2.f), v));
  const float2 den_m = fma2(sp(6.f), w.q23, fma2(sp(18.f), w.q12, g));
  const float2 den_p = fma2(sp(6.f), w.q12, fma2(sp(18.f), w.q23, g));
  minus = fma2(num_m, rcp2(den_m), p2m);
  plus = fma2(sp(-1.f), mul2(num_p, rcp2(den_p)), p2p);
}

__device__ __forceinline__ float2 max5(float2 a, float2 b, float2 c, float2 d, float2 e) {
  return make_float2(max3f(max3f(a.x, b.x, c.x), d.x, e.x), max3f(max3f(a.y, b.y, c.y), d.y, e.y));
}

// minus(c) of the window W(c) = D[0..4] = D(c-2 .. c+2), per lane
__device__ __forceinline__ float2 minus_of_window(const float2 D[5], Tri *mid = nullptr, Tri *last = nullptr) {
  const Tri a0 = tri_forms(D[0], D[1], D[2]), a1 = tri_forms(D[1], D[2], D[3]), a2 = tri_forms(D[2], D[3], D[4]);
  float2 sq[5];
#pragma unroll
  for (int q = 0; q < 5; q++) sq[q] = mul2(D[q], D[q]);
  const WQ wq = window_q(a0.s1, a1.s2, a2.s3, max5(sq[0], sq[1], sq[2], sq[3], sq[4]));
  const float2 p2m = fma2(sp(-1.f / 6.f), a1.t, mul2(sp(0.5f), add2(D[2], D[3])));
  if (mid) *mid = a1;
  if (last) *last = a2;
  return side_minus(wq, sub2(a0.t, a1.t), sub2(a1.t, a2.t), p2m);
}

// periodic images of a cell's new value in the 3 ghost layers (faces, edges,
// corners), written by the thread that computes the cell (not inlined: the
// stage loop then keeps none of its index arithmetic when it is not used)
static __device__ __noinline__ void write_periodic_images(float *out, const Layout &L, int i, int j, int k, float val) {
  const int oi = i < 3 ? L.nx : (i >= L.nx - 3 ? -L.nx : 0);
  const int oj = j < 3 ? L.ny : (j >= L.ny - 3 ? -L.ny : 0);
  const int ok = k < 3 ? L.nz : (k >= L.nz - 3 ? -L.nz : 0);
  if (!(oi | oj | ok)) return;
  const long long c = L.idx(i, j, k), sx = oi, sy = L.py * oj, sz = L.pz * ok;
  if (oi) out[c + sx] = val;
  if (oj) out[c + sy] = val;
  if (ok) out[c + sz] = val;
  if (oi && oj) out[c + sx + sy] = val;
  if (oi && ok) out[c + sx + sz] = val;
  if (oj && ok) out[c + sy + sz] = val;
  if (oi && oj && ok) out[c + sx + sy + sz] = val;
}

// (a template so that each translation unit including this header has its
// own instance, as with the other stage kernels)
template <int TILE_Z = RZ>
__global__ void __launch_bounds__(256, reinit_x2_ctas(TILE_Z))
    k_reinit_x2(const __grid_constant__ CUtensorMap tm, StageArgs<float> a) {
  static_assert(TILE_Z % 2 == 0 && TILE_Z % RY == 0, "the prologues pack plane pairs and cover the planes by rows");
  constexpr int RZ = TILE_Z, RSZ = TILE_Z + 6;
  constexpr size_t kReinitX2Smem = reinit_x2_smem(TILE_Z);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *tile = reinterpret_cast<float *>(smem_raw);
  __shared__ __align__(8) uint64_t bar;
  // tile-edge values of the neighbouring lanes / rows that do not exist:
  // x: per (plane, row) minus(x0) and the forms of triples x0-1, x0;
  // y: per (plane, x pair) minus(y0)
  __shared__ float xedge[6][RZ][RY];
  __shared__ float2 yedge[RZ][32];
  __shared__ float2 yx[2][RY][32];  // minus(j+1) handed to the next row, by plane parity
  const int lane = threadIdx.x, w = threadIdx.y;
  const int tid = lane + 32 * w;
  const int x0 = blockIdx.x * RX, y0 = blockIdx.y * RY, z0 = blockIdx.z * RZ;
  const Layout &L = a.L;

  if (tid == 0) {
    prefetch_tmap(&tm);
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar, (uint32_t)kReinitX2Smem);
    tma_load_3d(tile, &tm, x0 + GX - 4, y0 + GY - 3, z0 + GZ - 3, &bar);
  }
  if (!mbar_wait(&bar, 0, kMaxPolls)) {
    if (tid == 0) atomicExch(a.err, LSMGPU_ERR_TIMEOUT);
    mbar_wait(&bar, 0, kMaxPolls);  // let an in-flight copy land before exit
    return;
  }
  if (a.ghost) {
    fill_face_ghosts<float>(tile, RSX, RSY, RSZ, x0 - 4, y0 - 3, z0 - 3, L, a.ghost);
    __syncthreads();
  }

  const int st_y = RSX, st_z = RSX * RSY;
  // ---- prologue: the tile-edge values, two planes per thread as a pair ------
  if (tid < RY * RZ / 2) {
    const int pw = tid % RY, pz = 2 * (tid / RY);
    const float *r0 = tile + ((pz + 3) * RSY + pw + 3) * RSX, *r1 = r0 + st_z;
    float2 p[6];  // phi(x0-3 .. x0+2)
#pragma unroll
    for (int q = 0; q < 6; q++) p[q] = make_float2(r0[q + 1], r1[q + 1]);
    float2 D[5];  // D(x0-2 .. x0+2)
#pragma unroll
    for (int q = 0; q < 5; q++) D[q] = sub2(p[q + 1], p[q]);
    Tri a1, a2;
    const float2 mv = minus_of_window(D, &a1, &a2);  // a1 = tri(x0-1), a2 = tri(x0)
    const float2 v[6] = {mv, a1.s1, a2.s1, a2.s2, a1.t, a2.t};
#pragma unroll
    for (int q = 0; q < 6; q++) {
      xedge[q][pz][pw] = v[q].x;
      xedge[q][pz + 1][pw] = v[q].y;
    }
  }
  {
    // minus(y0) of each x pair, planes w and w + RY
#pragma unroll 1
    for (int tz = w; tz < RZ; tz += RY) {
      const float *c = tile + (tz + 3) * st_z + 2 * lane + 4;
      float2 p[6];  // phi(y0-3 .. y0+2)
#pragma unroll
      for (int q = 0; q < 6; q++) p[q] = *reinterpret_cast<const float2 *>(c + q * st_y);
      float2 D[5];
#pragma unroll
      for (int q = 0; q < 5; q++) D[q] = sub2(p[q + 1], p[q]);
      yedge[tz][lane] = minus_of_window(D);
    }
  }
  __syncthreads();

  // Every warp runs every plane (the y hand-over needs one barrier per
  // plane); rows and lanes outside the grid compute on tile padding and
  // store nothing.
  const int i = x0 + 2 * lane, j = y0 + w;
  const bool row_live = j < L.ny;
  const bool two = i + 1 < L.nx;
  const bool live = row_live && i < L.nx;
  const int sx = 2 * lane + 4, sy = w + 3;
  const int kmax = min(RZ, L.nz - z0);
  const float *col = tile + sy * st_y + sx;  // (i, j) column, plane index sz
  auto ld2 = [&](int sz, int dx, int dy) {
    return *reinterpret_cast<const float2 *>(col + sz * st_z + dy * st_y + dx);
  };
  const float2 iv2[3] = {sp(a.inv[0] * a.inv[0]), sp(a.inv[1] * a.inv[1]), sp(a.inv[2] * a.inv[2])};

  // ---- z march warm-up: the carried state for cell z0 ---------------------
  float2 fz2, dz1, dz2, s1p, s1c, s2c, tk, tdk1, sumk, gmz, pb1, pb2, sqk1, sqk2;
  {
    float2 p[6];  // phi(z0-3 .. z0+2)
#pragma unroll
    for (int q = 0; q < 6; q++) p[q] = ld2(q, 0, 0);
    float2 D[5];  // D(z0-2 .. z0+2)
#pragma unroll
    for (int q = 0; q < 5; q++) D[q] = sub2(p[q + 1], p[q]);
    Tri a1, a2;
    gmz = minus_of_window(D, &a1, &a2);  // minus(z0); a1 = tri(z0-1), a2 = tri(z0)
    float2 sq[5];
#pragma unroll
    for (int q = 0; q < 5; q++) sq[q] = mul2(D[q], D[q]);
    fz2 = p[5];
    dz1 = D[3];
    dz2 = D[4];
    s1p = a1.s1;
    s1c = a2.s1;
    s2c = a2.s2;
    tk = a2.t;
    tdk1 = sub2(a1.t, a2.t);  // TD(z0-1)
    sumk = add2(D[2], D[3]);  // D(z0) + D(z0+1)
    sqk1 = sq[3];
    sqk2 = sq[4];
    pb2 = make_float2(fmaxf(sq[1].x, sq[2].x), fmaxf(sq[1].y, sq[2].y));  // max sq(z0-1), sq(z0)
    pb1 = make_float2(fmaxf(sq[2].x, sq[3].x), fmaxf(sq[2].y, sq[3].y));  // max sq(z0), sq(z0+1)
  }

  // phi0 and phi^n at the cell pair are read from global memory one plane
  // ahead of their use, so their latency overlaps a plane of arithmetic
  const float *pc_src = a.use0 ? a.phi0 : nullptr;
  const float *un_src = a.stage == 1 ? nullptr : a.phi_n;
  const long long cell0 = L.idx(live ? i : 0, row_live ? j : 0, z0);
  float2 pc_next = pc_src ? *reinterpret_cast<const float2 *>(pc_src + cell0) : sp(0.f);
  float2 un_next = un_src ? *reinterpret_cast<const float2 *>(un_src + cell0) : sp(0.f);

  for (int tz = 0; tz < kmax; tz++) {
    const int k = z0 + tz;
    const int sz = tz + 3;
    const long long cell = cell0 + (long long)tz * L.pz;
    const float2 pc_ld = pc_next, un = un_next;
    if (tz + 1 < kmax) {
      if (pc_src) pc_next = *reinterpret_cast<const float2 *>(pc_src + cell + L.pz);
      if (un_src) un_next = *reinterpret_cast<const float2 *>(un_src + cell + L.pz);
    }
    // ---- y: window W(j+1) -> plus(j), minus(j+1) (handed to row j+1) --------
    const float2 u0 = ld2(sz, 0, 0);  // phi(i), phi(i+1)
    float2 gpy, gmy;
    {
      float2 r[6];  // phi(j-2 .. j+3)
#pragma unroll
      for (int q = 0; q < 6; q++) r[q] = (q == 2) ? u0 : ld2(sz, 0, q - 2);
      float2 D[5];  // D(j-1 .. j+3)
#pragma unroll
      for (int q = 0; q < 5; q++) D[q] = sub2(r[q + 1], r[q]);
      const Tri b = tri_forms(D[0], D[1], D[2]), c = tri_forms(D[1], D[2], D[3]), d = tri_forms(D[2], D[3], D[4]);
      float2 sq[5];
#pragma unroll
      for (int q = 0; q < 5; q++) sq[q] = mul2(D[q], D[q]);
      const WQ wq = window_q(b.s1, c.s2, d.s3, max5(sq[0], sq[1], sq[2], sq[3], sq[4]));
      const float2 c6 = mul2(sp(-1.f / 6.f), c.t);               // t(j) / -6
      const float2 p2m = fma2(sp(0.5f), add2(D[2], D[3]), c6);  // minus(j+1)
      const float2 p2p = fma2(sp(0.5f), add2(D[1], D[2]), c6);  // plus(j)
      float2 mn;
      sides_both(wq, sub2(b.t, c.t), sub2(c.t, d.t), p2m, p2p, mn, gpy);
      yx[tz & 1][w][lane] = mn;
    }
    // ---- z: window W(k+1) -> plus(k), minus(k+1) -----------------------------
    const float2 gmz_cur = gmz;  // minus(k), from the previous window
    float2 gpz;
    {
      const float2 f3 = ld2(sz + 3, 0, 0);
      const float2 d3 = sub2(f3, fz2);
      const float2 sq3 = mul2(d3, d3);
      const Tri n = tri_forms(dz1, dz2, d3);  // tri(k+1)
      const float2 tdk = sub2(tk, n.t);       // TD(k)
      const float2 pbn = make_float2(fmaxf(sqk1.x, sqk2.x), fmaxf(sqk1.y, sqk2.y));
      const float2 m = make_float2(max3f(pb2.x, pbn.x, sq3.x), max3f(pb2.y, pbn.y, sq3.y));
      const WQ wq = window_q(s1p, s2c, n.s3, m);
      const float2 sumn = add2(dz1, dz2);  // D(k+1) + D(k+2)
      const float2 c6 = mul2(sp(-1.f / 6.f), tk);
      const float2 p2m = fma2(sp(0.5f), sumn, c6), p2p = fma2(sp(0.5f), sumk, c6);
      sides_both(wq, tdk1, tdk, p2m, p2p, gmz, gpz);  // minus(k+1), plus(k)
      fz2 = f3;
      dz1 = dz2;
      dz2 = d3;
      s1p = s1c;
      s1c = n.s1;
      s2c = n.s2;
      tk = n.t;
      tdk1 = tdk;
      sumk = sumn;
      pb2 = pb1;
      pb1 = pbn;
      sqk1 = sqk2;
      sqk2 = sq3;
    }
    // ---- x: windows W(i+1), W(i+2); triples i-1, i from the previous lane ----
    float2 gpx, gmx;
    {
      const float2 e0 = ld2(sz, -2, 0), e2 = ld2(sz, 2, 0), e3 = ld2(sz, 4, 0);
      // odd pairs (phi(s), phi(s+1)) for s = i-1, i+1, i+3
      const float2 o0 = make_float2(e0.y, u0.x), o1 = make_float2(u0.y, e2.x), o2 = make_float2(e2.y, e3.x);
      // P_s = (D(s), D(s+1)) for s = i-1 .. i+3
      const float2 P0 = sub2(o0, e0), P1 = sub2(u0, o0), P2 = sub2(o1, u0), P3 = sub2(e2, o1), P4 = sub2(o2, e2);
      const Tri C = tri_forms(P2, P3, P4);  // (tri(i+1), tri(i+2))
      // (tri(i-1), tri(i)) are the previous lane's C
      float a_s1x = __shfl_up_sync(0xffffffffu, C.s1.x, 1), a_s1y = __shfl_up_sync(0xffffffffu, C.s1.y, 1);
      float a_s2y = __shfl_up_sync(0xffffffffu, C.s2.y, 1);
      float a_tx = __shfl_up_sync(0xffffffffu, C.t.x, 1), a_ty = __shfl_up_sync(0xffffffffu, C.t.y, 1);
      if (lane == 0) {
        a_s1x = xedge[1][tz][w];
        a_s1y = xedge[2][tz][w];
        a_s2y = xedge[3][tz][w];
        a_tx = xedge[4][tz][w];
        a_ty = xedge[5][tz][w];
      }
      const float2 As1 = make_float2(a_s1x, a_s1y), At = make_float2(a_tx, a_ty);
      const float2 Bs2 = make_float2(a_s2y, C.s2.x), Bt = make_float2(a_ty, C.t.x);
      const float2 q0 = mul2(P0, P0), q2 = mul2(P2, P2), q4 = mul2(P4, P4);  // sq(i-1 .. i+4)
      const float inner = fmaxf(max3f(q0.y, q2.x, q2.y), q4.x);             // sq(i .. i+3)
      const float2 m = make_float2(fmaxf(inner, q0.x), fmaxf(inner, q4.y));
      const WQ wq = window_q(As1, Bs2, C.s3, m);
      const float2 tda = sub2(At, Bt), tdb = sub2(Bt, C.t);
      const float2 c6 = mul2(sp(-1.f / 6.f), Bt);
      const float2 p2m = fma2(sp(0.5f), add2(P2, P3), c6);  // cells i+1, i+2
      const float2 p2p = fma2(sp(0.5f), add2(P1, P2), c6);  // cells i, i+1
      float2 mn;
      sides_both(wq, tda, tdb, p2m, p2p, mn, gpx);
      float prev = __shfl_up_sync(0xffffffffu, mn.y, 1);
      if (lane == 0) prev = xedge[0][tz][w];
      gmx = make_float2(prev, mn.x);
    }
    __syncthreads();  // minus(j+1) of every row is in yx
    gmy = (w == 0) ? yedge[tz][lane] : yx[tz & 1][w - 1][lane];
    // ---- reinitialization RHS (reinitialization3d.f.in:170-251) and stage ----
    const float2 pc = pc_src ? pc_ld : u0;
    float2 n2 = sp(0.f);
    {
      // Godunov: pc > 0: max(-g+, g-, 0); else max(g+, -g-, 0), i.e.
      // max(-s g+, s g-, 0) with s = sign of pc
      const float2 sg = make_float2(pc.x > 0.f ? 1.f : -1.f, pc.y > 0.f ? 1.f : -1.f);
      const float2 g[3][2] = {{gpx, gmx}, {gpy, gmy}, {gpz, gmz_cur}};
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const float2 ap = mul2(g[d][0], sg), am = mul2(g[d][1], sg);
        const float2 st = make_float2(max3f(-ap.x, am.x, 0.f), max3f(-ap.y, am.y, 0.f));
        n2 = fma2(mul2(st, iv2[d]), st, n2);
      }
    }
    const float2 den = a.use0 ? fma2(pc, pc, sp(a.dx_sq)) : fma2(pc, pc, mul2(n2, sp(a.dx_sq)));
    const float2 sgn = mul2(pc, make_float2(rsqrt_approx(den.x), rsqrt_approx(den.y)));
    const float2 gn = make_float2(sqrt_approx(n2.x), sqrt_approx(n2.y));
    float2 rhs = fma2(sp(-1.f), mul2(sgn, gn), sgn);  // sgn (1 - |grad phi|)
    if (!(fabsf(pc.x) >= 1e-11f)) rhs.x = 0.f;
    if (!(fabsf(pc.y) >= 1e-11f)) rhs.y = 0.f;
    float2 u;
    if (a.stage == 1) {
      u = fma2(sp(a.dt), rhs, u0);  // tvd_runge_kutta3d.f:78
    } else if (a.stage == 2) {
      u = fma2(sp(0.75f), un, mul2(sp(0.25f), fma2(sp(a.dt), rhs, u0)));  // :403-404
    } else {
      u = fma2(sp(1.f / 3.f), un, mul2(sp(2.f / 3.f), fma2(sp(a.dt), rhs, u0)));  // :490-492
    }
    if (live) {
      if (two) {
        *reinterpret_cast<float2 *>(a.out + cell) = u;
      } else {
        a.out[cell] = u.x;
      }
      // (the writer returns at once for a cell with no image; a boundary
      // test here measured 5% slower stages, through the loop's code)
      if (a.periodic) {
        write_periodic_images(a.out, L, i, j, k, u.x);
        if (two) write_periodic_images(a.out, L, i + 1, j, k, u.y);
      }
    }
  }
}

}  // namespace fused
}  // namespace lsmgpu
