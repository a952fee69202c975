// Fused TVD Runge-Kutta stage kernels: one kernel per stage computes the
// HJ WENO5 derivatives, the level-set right-hand side (advection, or the
// reinitialization Hamiltonian) and the stage update in a single pass, with
// the periodic ghost images of the result written in the same pass.
//
// Work layout in HBM (one buffer per stage field): interior cells (0..nx-1,
// 0..ny-1, 0..nz-1) with GX = 4 ghost cells below x and 3 above, 3 ghost
// layers in y and z; rows padded to a multiple of 32 elements so each row
// starts on a 128-byte boundary.  A CTA of 32 x 8 threads owns a 32 x 8 x 8
// tile and stages the tile plus its 3-cell halo (40 x 14 x 14 elements) into
// shared memory with one 3D TMA load; the x origin of the box is the tile's
// 32-aligned row offset, which satisfies TMA's 16-byte rule for both element
// sizes.  Each thread then walks the 8 cells of its z column.
//
// EXACT selects the FP64 parity arithmetic (LSMLIB's operation order; the
// including unit is compiled with -fmad=false).  Otherwise the FP32 form runs
// with FMA contraction and an epsilon-scaled WENO weight formula that cannot
// under- or overflow in single precision (see weno5_fast).
#pragma once

#include <type_traits>

#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"
#include "tma.cuh"

namespace lsmgpu {
namespace fused {

constexpr int GX = 4, GY = 3, GZ = 3;
constexpr int TX = 32, TY = 8, TZ = 8;
constexpr int SX = TX + 8, SY = TY + 6, SZ = TZ + 6;
constexpr uint32_t kMaxPolls = 1u << 22;

struct Layout {
  int nx, ny, nz;
  long long py, pz;  // element pitches of y and z
  __host__ __device__ long long idx(int i, int j, int k) const {
    return (long long)(i + GX) + py * (long long)(j + GY) + pz * (long long)(k + GZ);
  }
  __host__ long long elems() const { return pz * (long long)(nz + 2 * GZ); }
};

inline Layout make_layout(int nx, int ny, int nz) {
  Layout L;
  L.nx = nx; L.ny = ny; L.nz = nz;
  L.py = ((long long)nx + GX + 3 + 31) / 32 * 32;
  L.pz = L.py * (long long)(ny + 2 * GY);
  return L;
}

enum Mode { ADV_CONST = 0, ADV_FIELD = 1, REINIT = 2 };

template <class R>
struct StageArgs {
  Layout L;
  const R *phi_n;    // u^n at the cell (stages 2 and 3)
  const R *phi0;     // sign source of the phi0 reinitialization form
  const R *vel[3];   // velocity fields (ADV_FIELD)
  R *out;
  R vconst[3];       // constant velocity (ADV_CONST)
  R inv[3];          // 1/dx, 1/dy, 1/dz
  R dt, dx_sq;
  int stage;         // 1, 2 or 3
  int use0;          // reinitialization sign from phi0
  int periodic;      // write periodic ghost images of the result
  int ghost;         // 0, or the LSMGPU_BC_* extrapolation whose face ghosts
                     // the kernel computes in shared memory from the tile
  int *err;
};

// One-axis extrapolation of LSMLIB's ghost-cell routines
// (boundary_conditions3d.f:46-462) at distance g from the edge value e, with
// n the value next inside: linear (slope e - n), signed linear (slope
// sign(e) |e - n|, :203-206) or copy (homogeneous Neumann).
template <class R>
__device__ __forceinline__ R extrap(R e, R n, int g, int kind) {
  if (kind == LSMGPU_BC_COPY) return e;
  const R s = (kind == LSMGPU_BC_SIGNED_LINEAR) ? copysign(R(1.0), e) * fabs(e - n) : e - n;
  return e + s * R(g);
}

// The ghost cells a stage's stencils read (face ghosts: one coordinate in
// the 3-cell layer, the other two interior) that lie in a staged tile,
// computed from the tile's interior cells with LSMLIB's extrapolation
// (boundary_conditions3d.f:46-462): identical values to a fill of the
// stored array, whose faces are written x, then y, then z, because a face
// ghost of an axis is written only by that axis' pass from interior cells.
// (Edge and corner ghosts are read by no axis-aligned stencil.)  Tile cell
// (a, b, c) holds interior cell (ox + a, oy + b, oz + c).
// The faces write disjoint cells and read only interior ones, so they are
// filled in any order; a tile inside the domain on every axis has none (one
// uniform test).  Threads cover each face plane in 2D (x along threadIdx.x,
// the other axis along threadIdx.y) and walk the ghost layers, so no index
// is decomposed by division.  Not inlined, so the stage kernels' register
// allocation does not depend on it.
template <class R>
__device__ __noinline__ void fill_face_ghosts(R *tile, int sdx, int sdy, int sdz, int ox, int oy, int oz, const Layout &L,
                                 int kind) {
  if (ox >= 0 && ox + sdx <= L.nx && oy >= 0 && oy + sdy <= L.ny && oz >= 0 && oz + sdz <= L.nz) return;
  const int sxy = sdx * sdy;
  // one face: ghost layers 1..3 of axis AX below (up = 0) or above (up = 1)
  auto face = [&](auto ax_tag, int up) {
    constexpr int AX = decltype(ax_tag)::value;
    const int n0 = L.nx, n1 = L.ny, n2 = L.nz;
    const int nax = AX == 0 ? n0 : (AX == 1 ? n1 : n2);
    // ranges: ghost layers along AX, interior along the other two, clipped to the tile
    int lo0 = AX == 0 ? (up ? n0 : -3) : 0, hi0 = AX == 0 ? (up ? n0 + 2 : -1) : n0 - 1;
    int lo1 = AX == 1 ? (up ? n1 : -3) : 0, hi1 = AX == 1 ? (up ? n1 + 2 : -1) : n1 - 1;
    int lo2 = AX == 2 ? (up ? n2 : -3) : 0, hi2 = AX == 2 ? (up ? n2 + 2 : -1) : n2 - 1;
    lo0 = max(lo0, ox); hi0 = min(hi0, ox + sdx - 1);
    lo1 = max(lo1, oy); hi1 = min(hi1, oy + sdy - 1);
    lo2 = max(lo2, oz); hi2 = min(hi2, oz + sdz - 1);
    if (lo0 > hi0 || lo1 > hi1 || lo2 > hi2) return;
    const int e_at = up ? nax - 1 : 0, n_at = up ? nax - 2 : 1;
    const int st = AX == 0 ? 1 : (AX == 1 ? sdx : sxy);
    // plane axes: (1, 2) for an x face, (0, 2) for y, (0, 1) for z
    constexpr int PA = AX == 0 ? 1 : 0, PB = AX == 2 ? 1 : 2;
    const int loA = PA == 0 ? lo0 : lo1, hiA = PA == 0 ? hi0 : hi1;
    const int loB = PB == 1 ? lo1 : lo2, hiB = PB == 1 ? hi1 : hi2;
    const int loG = AX == 0 ? lo0 : (AX == 1 ? lo1 : lo2), hiG = AX == 0 ? hi0 : (AX == 1 ? hi1 : hi2);
    for (int pa = loA + (int)threadIdx.x; pa <= hiA; pa += blockDim.x)
      for (int pb = loB + (int)threadIdx.y; pb <= hiB; pb += blockDim.y)
        for (int g = loG; g <= hiG; g++) {
          const int c0 = AX == 0 ? g : pa;
          const int c1 = AX == 1 ? g : (PA == 1 ? pa : pb);
          const int c2 = AX == 2 ? g : pb;
          const int at = (c0 - ox) + (c1 - oy) * sdx + (c2 - oz) * sxy;
          const int d = up ? g - e_at : -g;
          tile[at] = extrap(tile[at + (e_at - g) * st], tile[at + (n_at - g) * st], d, kind);
        }
  };
  // only the faces the tile crosses
  if (ox < 0) face(std::integral_constant<int, 0>{}, 0);
  if (ox + sdx > L.nx) face(std::integral_constant<int, 0>{}, 1);
  if (oy < 0) face(std::integral_constant<int, 1>{}, 0);
  if (oy + sdy > L.ny) face(std::integral_constant<int, 1>{}, 1);
  if (oz < 0) face(std::integral_constant<int, 2>{}, 0);
  if (oz + sdz > L.nz) face(std::integral_constant<int, 2>{}, 1);
}

// ---------------------------------------------------------------------------
// FP32 arithmetic
// ---------------------------------------------------------------------------
// WENO5-JS with the nonlinear weights rewritten as
//   w_k = d_k prod_{j != k} q_j / sum_i d_i prod_{j != i} q_j,
//   q_k = (S_k / eps + 1)^2,
// which equals d_k/(S_k+eps)^2 normalised.  S_k <= 64 max v^2 and
// eps >= 1e-6 max v^2, so 1 <= q_k <= 4.2e15 and every product stays below
// 2e31: no underflow to 0/0 on near-flat data (where the direct form's
// (S+eps)^2 underflows in FP32) and no overflow, with two reciprocals
// instead of four divisions.
__device__ __forceinline__ float weno5_fast(float v1, float v2, float v3, float v4, float v5) {
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float c1312 = 13.f / 12.f;
  const float m = fmaxf(fmaxf(fmaxf(v1 * v1, v2 * v2), fmaxf(v3 * v3, v4 * v4)), v5 * v5);
  const float eps = fmaf(1e-6f, m, 1e-36f);
  const float p1 = fmaf(c13, v1, fmaf(-c76, v2, c116 * v3));
  const float p2 = fmaf(-c16, v2, fmaf(c56, v3, c13 * v4));
  const float p3 = fmaf(c13, v3, fmaf(c56, v4, -c16 * v5));
  float t = v1 - 2.f * v2 + v3, u = v1 - 4.f * v2 + 3.f * v3;
  const float S1 = fmaf(c1312 * t, t, 0.25f * u * u);
  t = v2 - 2.f * v3 + v4; u = v2 - v4;
  const float S2 = fmaf(c1312 * t, t, 0.25f * u * u);
  t = v3 - 2.f * v4 + v5; u = 3.f * v3 - 4.f * v4 + v5;
  const float S3 = fmaf(c1312 * t, t, 0.25f * u * u);
  const float r = __fdividef(1.f, eps);
  float q1 = fmaf(S1, r, 1.f), q2 = fmaf(S2, r, 1.f), q3 = fmaf(S3, r, 1.f);
  q1 *= q1; q2 *= q2; q3 *= q3;
  const float n1 = 0.1f * (q2 * q3), n2 = 0.6f * (q1 * q3), n3 = 0.3f * (q1 * q2);
  return __fdividef(fmaf(n1, p1, fmaf(n2, p2, n3 * p3)), n1 + n2 + n3);
}

template <class R, bool EXACT>
__device__ __forceinline__ R weno(R v1, R v2, R v3, R v4, R v5) {
  if constexpr (EXACT) return weno5_exact<R>(v1, v2, v3, v4, v5);
  else return (R)weno5_fast((float)v1, (float)v2, (float)v3, (float)v4, (float)v5);
}

// reinitialization RHS; the FP32 form keeps the FP64 zero tolerance so it
// approximates the FP64 computation, and uses reciprocal square roots
template <class R, bool EXACT>
__device__ __forceinline__ R reinit_term(R pc, const R gp[3], const R gm[3], R dx_sq, bool use0) {
  if constexpr (EXACT) {
    return reinit_rhs<R>(pc, gp, gm, dx_sq, use0);
  } else {
    float st[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const float u = (pc > 0.f) ? fmaxf(-gp[d], 0.f) : fmaxf(gp[d], 0.f);
      const float w = (pc > 0.f) ? fmaxf(gm[d], 0.f) : fmaxf(-gm[d], 0.f);
      st[d] = fmaxf(u, w);
    }
    if (!(fabsf(pc) >= 1e-11f)) return 0.f;
    const float n2 = fmaf(st[0], st[0], fmaf(st[1], st[1], st[2] * st[2]));
    const float den = use0 ? fmaf(pc, pc, (float)dx_sq) : fmaf(pc, pc, n2 * (float)dx_sq);
    const float sgn = pc * rsqrtf(den);
    return sgn * (1.f - sqrtf(n2));
  }
}

// ---------------------------------------------------------------------------
// the stage kernel
// ---------------------------------------------------------------------------
template <class R, int MODE, bool EXACT>
__global__ void __launch_bounds__(TX * TY) k_stage(const __grid_constant__ CUtensorMap tm, StageArgs<R> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  R *tile = reinterpret_cast<R *>(smem_raw);
  __shared__ __align__(8) uint64_t bar;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = tx + TX * ty;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ;

  if (tid == 0) {
    prefetch_tmap(&tm);
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar, (uint32_t)(SX * SY * SZ * sizeof(R)));
    // padded coordinates of interior cell (x0 - 4, y0 - 3, z0 - 3)
    tma_load_3d(tile, &tm, x0 + GX - 4, y0 + GY - 3, z0 + GZ - 3, &bar);
  }
  if (!mbar_wait(&bar, 0, kMaxPolls)) {
    if (tid == 0) atomicExch(a.err, LSMGPU_ERR_TIMEOUT);
    mbar_wait(&bar, 0, kMaxPolls);  // let an in-flight copy land before exit
    return;
  }
  if (a.ghost) {
    fill_face_ghosts<R>(tile, SX, SY, SZ, x0 - 4, y0 - 3, z0 - 3, a.L, a.ghost);
    __syncthreads();
  }

  const Layout &L = a.L;
  const int i = x0 + tx, j = y0 + ty;
  if (i >= L.nx || j >= L.ny) return;
  const int sx = tx + 4, sy = ty + 3;
  const int kmax = min(TZ, L.nz - z0);

  for (int tz = 0; tz < kmax; tz++) {
    const int k = z0 + tz;
    const int sz = tz + 3;
    const R *c = tile + (sz * SY + sy) * SX + sx;
    const int st[3] = {1, SX, SX * SY};
    R rhs;
    if (MODE == REINIT) {
      R gp[3], gm[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        R v[6];  // scaled D1(c-2 .. c+3)
#pragma unroll
        for (int f = -2; f <= 3; f++) v[f + 2] = (c[f * st[d]] - c[(f - 1) * st[d]]) * a.inv[d];
        gp[d] = weno<R, EXACT>(v[5], v[4], v[3], v[2], v[1]);
        gm[d] = weno<R, EXACT>(v[0], v[1], v[2], v[3], v[4]);
      }
      const long long cell = L.idx(i, j, k);
      const R pc = a.use0 ? a.phi0[cell] : c[0];
      rhs = reinit_term<R, EXACT>(pc, gp, gm, a.dx_sq, a.use0 != 0);
    } else {
      R g[3], vel[3];
      const long long cell = L.idx(i, j, k);
#pragma unroll
      for (int d = 0; d < 3; d++) vel[d] = (MODE == ADV_CONST) ? a.vconst[d] : a.vel[d][cell];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        // spatial_derivatives3d.f.in:2756-2812
        if (fabs(vel[d]) < Consts<double>::zero_tol) {
          g[d] = R(0);
        } else if (vel[d] > R(0)) {
          R v[5];
#pragma unroll
          for (int f = -2; f <= 2; f++) v[f + 2] = (c[f * st[d]] - c[(f - 1) * st[d]]) * a.inv[d];
          g[d] = weno<R, EXACT>(v[0], v[1], v[2], v[3], v[4]);
        } else {
          R v[5];
#pragma unroll
          for (int f = -1; f <= 3; f++) v[f + 1] = (c[f * st[d]] - c[(f - 1) * st[d]]) * a.inv[d];
          g[d] = weno<R, EXACT>(v[4], v[3], v[2], v[1], v[0]);
        }
      }
      // lsm3dZeroOutLevelSetEqnRHS then lsm3dAddAdvectionTermToLSERHS
      // (level_set_evolution3d.f.in:38, :113-116)
      rhs = R(0) - (vel[0] * g[0] + vel[1] * g[1] + vel[2] * g[2]);
    }

    const long long cell = L.idx(i, j, k);
    R u;
    if (a.stage == 1) {
      u = c[0] + a.dt * rhs;  // tvd_runge_kutta3d.f:78
    } else if (a.stage == 2) {
      u = R(0.75) * a.phi_n[cell] + R(0.25) * (c[0] + a.dt * rhs);  // :403-404
    } else {
      u = R(1.0 / 3.0) * a.phi_n[cell] + R(2.0 / 3.0) * (c[0] + a.dt * rhs);  // :490-492
    }
    a.out[cell] = u;

    if (a.periodic) {
      // periodic images in the ghost layers (3 cells per side)
      int oi[2] = {0, 0}, oj[2] = {0, 0}, ok_[2] = {0, 0};
      int ni = 1, nj = 1, nk = 1;
      if (i < 3) oi[ni++] = L.nx; else if (i >= L.nx - 3) oi[ni++] = -L.nx;
      if (j < 3) oj[nj++] = L.ny; else if (j >= L.ny - 3) oj[nj++] = -L.ny;
      if (k < 3) ok_[nk++] = L.nz; else if (k >= L.nz - 3) ok_[nk++] = -L.nz;
      if (ni + nj + nk > 3) {
        for (int p = 0; p < ni; p++)
          for (int q = 0; q < nj; q++)
            for (int r = 0; r < nk; r++)
              if (p | q | r) a.out[L.idx(i + oi[p], j + oj[q], k + ok_[r])] = u;
      }
    }
  }
}

}  // namespace fused
}  // namespace lsmgpu

// ---------------------------------------------------------------------------
// FP32 stage kernel on cell pairs: each thread advances cells (z, z+1) of its
// column together, one cell per lane of Blackwell's packed FP32x2
// instructions (FADD2 / FMUL2 / FFMA2), which halves the issued instructions
// of the WENO5 arithmetic.  Comparisons, selections and the reciprocals stay
// per lane.
// ---------------------------------------------------------------------------
namespace lsmgpu {
namespace fused {

__device__ __forceinline__ float2 sp(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// 2^-floor(log2 x) for a positive normal float x, from the exponent bits (no
// reciprocal instruction).  x * pow2_recip(x) lies in [1, 2).
__device__ __forceinline__ float pow2_recip(float x) {
  return __int_as_float(0x7f000000 - (__float_as_int(x) & 0x7f800000));
}
__device__ __forceinline__ float2 pow2_recip2(float2 x) { return make_float2(pow2_recip(x.x), pow2_recip(x.y)); }

// WENO5-JS on two cells at once, the epsilon-scaled weight form of
// weno5_fast with the common factors folded: only S/eps enters the weights,
// so the smoothness indicators are kept as 4 S and epsilon as 12 eps (the
// factor 3 goes into the scale), and the weights as 10 d_k prod q_j^2.
__device__ __forceinline__ float2 weno5_x2(float2 v1, float2 v2, float2 v3, float2 v4, float2 v5) {
  const float2 q1s = mul2(v1, v1), q2s = mul2(v2, v2), q3s = mul2(v3, v3), q4s = mul2(v4, v4), q5s = mul2(v5, v5);
  float2 m;
  m.x = fmaxf(fmaxf(fmaxf(q1s.x, q2s.x), fmaxf(q3s.x, q4s.x)), q5s.x);
  m.y = fmaxf(fmaxf(fmaxf(q1s.y, q2s.y), fmaxf(q3s.y, q4s.y)), q5s.y);
  const float2 eps = fma2(sp(12e-6f), m, sp(12e-36f));  // 12 eps
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float2 P1 = fma2(sp(c13), v1, fma2(sp(-c76), v2, mul2(sp(c116), v3)));
  const float2 P2 = fma2(sp(-c16), v2, fma2(sp(c56), v3, mul2(sp(c13), v4)));
  const float2 P3 = fma2(sp(c13), v3, fma2(sp(c56), v4, mul2(sp(-c16), v5)));
  // 4 * smoothness indicators: 13/3 t^2 + u^2
  const float c133 = 13.f / 3.f;
  float2 t = fma2(sp(-2.f), v2, add2(v1, v3));
  float2 u = fma2(sp(-4.f), v2, fma2(sp(3.f), v3, v1));
  const float2 S1 = fma2(u, u, mul2(mul2(sp(c133), t), t));
  t = fma2(sp(-2.f), v3, add2(v2, v4));
  u = fma2(sp(-1.f), v4, v2);
  const float2 S2 = fma2(u, u, mul2(mul2(sp(c133), t), t));
  t = fma2(sp(-2.f), v4, add2(v3, v5));
  u = fma2(sp(-4.f), v4, fma2(sp(3.f), v3, v5));
  const float2 S3 = fma2(u, u, mul2(mul2(sp(c133), t), t));
  // q_k = (S_k + eps) 2^-e with 2^e <= eps < 2^(e+1): the weights only see
  // ratios of the q_k, so any common scale of S + eps gives the same weights
  // as (S_k / eps + 1); with eps 2^-e in [1, 2), 1 <= q_k < 7e7 and the
  // products below stay under 1e32
  const float2 r = pow2_recip2(eps);
  const float2 e = mul2(eps, r), r3 = mul2(sp(3.f), r);
  const float2 q1 = fma2(S1, r3, e), q2 = fma2(S2, r3, e), q3 = fma2(S3, r3, e);
  const float2 q23 = mul2(q2, q3), q13 = mul2(q1, q3), q12 = mul2(q1, q2);
  // 10 d_k prod_{j != k} q_j^2 (the common factor cancels)
  const float2 n1 = mul2(q23, q23);
  const float2 n2 = mul2(mul2(sp(6.f), q13), q13);
  const float2 n3 = mul2(mul2(sp(3.f), q12), q12);
  const float2 num = fma2(n1, P1, fma2(n2, P2, mul2(n3, P3)));
  const float2 den = add2(add2(n1, n2), n3);
  return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
}

// Both one-sided WENO5 values of one axis for two cells: minus side on
// D(c-2 .. c+2), plus side on D(c+3 .. c-1), given D[0..5] = D(c-2 .. c+3).
// The two sides share two of their three candidate stencils (plus P2 = minus
// P3, plus P3 = minus P2), the second differences t of their middle and outer
// smoothness indicators (plus t2 = minus t3, plus t3 = minus t2), and four of
// the five squared differences of the epsilon maximum; each is computed once.
__device__ __forceinline__ void weno5_pm_x2(const float2 D[6], float2 &gp, float2 &gm) {
  float2 sq[6];
#pragma unroll
  for (int i = 0; i < 6; i++) sq[i] = mul2(D[i], D[i]);
  const float cx = fmaxf(fmaxf(sq[1].x, sq[2].x), fmaxf(sq[3].x, sq[4].x));
  const float cy = fmaxf(fmaxf(sq[1].y, sq[2].y), fmaxf(sq[3].y, sq[4].y));
  // 12 eps of each side, its power-of-two scale r and 12 eps r in [1, 2)
  const float2 em = fma2(sp(12e-6f), make_float2(fmaxf(cx, sq[0].x), fmaxf(cy, sq[0].y)), sp(12e-36f));
  const float2 ep = fma2(sp(12e-6f), make_float2(fmaxf(cx, sq[5].x), fmaxf(cy, sq[5].y)), sp(12e-36f));
  const float2 rm = pow2_recip2(em), rp = pow2_recip2(ep);
  const float2 emr = mul2(em, rm), epr = mul2(ep, rp);
  const float2 rm3 = mul2(sp(3.f), rm), rp3 = mul2(sp(3.f), rp);
  // candidate stencils
  const float c13 = 1.f / 3.f, c76 = 7.f / 6.f, c116 = 11.f / 6.f, c16 = 1.f / 6.f, c56 = 5.f / 6.f;
  const float2 P1m = fma2(sp(c13), D[0], fma2(sp(-c76), D[1], mul2(sp(c116), D[2])));
  const float2 A = fma2(sp(-c16), D[1], fma2(sp(c56), D[2], mul2(sp(c13), D[3])));  // minus p2, plus p3
  const float2 B = fma2(sp(c13), D[2], fma2(sp(c56), D[3], mul2(sp(-c16), D[4])));  // minus p3, plus p2
  const float2 P1p = fma2(sp(c13), D[5], fma2(sp(-c76), D[4], mul2(sp(c116), D[3])));
  // second differences t and the asymmetric parts u of the indicators
  const float2 t1m = fma2(sp(-2.f), D[1], add2(D[0], D[2]));
  const float2 t2 = fma2(sp(-2.f), D[2], add2(D[1], D[3]));  // minus t2, plus t3
  const float2 t3 = fma2(sp(-2.f), D[3], add2(D[2], D[4]));  // minus t3, plus t2
  const float2 t1p = fma2(sp(-2.f), D[4], add2(D[5], D[3]));
  const float2 u1m = fma2(sp(-4.f), D[1], fma2(sp(3.f), D[2], D[0]));
  const float2 u2m = fma2(sp(-1.f), D[3], D[1]);
  const float2 u3m = fma2(sp(-4.f), D[3], fma2(sp(3.f), D[2], D[4]));
  const float2 u1p = fma2(sp(-4.f), D[4], fma2(sp(3.f), D[3], D[5]));
  const float2 u2p = fma2(sp(-1.f), D[2], D[4]);
  const float2 u3p = fma2(sp(-4.f), D[2], fma2(sp(3.f), D[3], D[1]));
  // 4 * smoothness indicators, 13/3 t^2 + u^2 (times 3 r below gives 12 S r)
  const float c133 = 13.f / 3.f;
  const float2 T1m = mul2(mul2(sp(c133), t1m), t1m), T2 = mul2(mul2(sp(c133), t2), t2);
  const float2 T3 = mul2(mul2(sp(c133), t3), t3), T1p = mul2(mul2(sp(c133), t1p), t1p);
  const float2 q1m = fma2(fma2(u1m, u1m, T1m), rm3, emr);
  const float2 q2m = fma2(fma2(u2m, u2m, T2), rm3, emr);
  const float2 q3m = fma2(fma2(u3m, u3m, T3), rm3, emr);
  const float2 q1p = fma2(fma2(u1p, u1p, T1p), rp3, epr);
  const float2 q2p = fma2(fma2(u2p, u2p, T3), rp3, epr);
  const float2 q3p = fma2(fma2(u3p, u3p, T2), rp3, epr);
  // weights 10 d_k prod_{j != k} q_j^2 (the common factor cancels)
  auto combine = [](float2 q1, float2 q2, float2 q3, float2 p1, float2 p2, float2 p3) {
    const float2 q23 = mul2(q2, q3), q13 = mul2(q1, q3), q12 = mul2(q1, q2);
    const float2 n1 = mul2(q23, q23);
    const float2 n2 = mul2(mul2(sp(6.f), q13), q13);
    const float2 n3 = mul2(mul2(sp(3.f), q12), q12);
    const float2 num = fma2(n1, p1, fma2(n2, p2, mul2(n3, p3)));
    const float2 den = add2(add2(n1, n2), n3);  // <= 1e32 < 2^126
    return make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
  };
  gm = combine(q1m, q2m, q3m, P1m, A, B);
  gp = combine(q1p, q2p, q3p, P1p, B, A);
}

// Computes one TX_ x TY_ x TZ_ tile whose haloed input ((TX_ + 8) x (TY_ + 6)
// x (TZ_ + 6)) is in `tile`, the calling thread at (tx, ty) of the tile;
// shared by the single-grid kernel (32 x 8 tiles) and the batched persistent
// kernel (32 x 8 or 16 x 16 tiles per grid, TZ_ from its autotuner).
template <int MODE, int TZ_ = TZ, int TX_ = TX, int TY_ = TY>
__device__ __forceinline__ void f32_tile(const float *tile, const StageArgs<float> &a, int x0, int y0, int z0,
                                         int tx, int ty) {
  constexpr int SX_ = TX_ + 8, SY_ = TY_ + 6;
  const Layout &L = a.L;
  const int i = x0 + tx, j = y0 + ty;
  if (i >= L.nx || j >= L.ny) return;
  const int sx = tx + 4, sy = ty + 3;
  const int kmax = min(TZ_, L.nz - z0);
  const int st[3] = {1, SX_, SX_ * SY_};
  const float2 inv[3] = {sp(a.inv[0]), sp(a.inv[1]), sp(a.inv[2])};

  for (int tz = 0; tz < kmax; tz += 2) {
    const bool two = tz + 1 < kmax;  // the second lane is a real cell
    const float *c0 = tile + ((tz + 3) * SY_ + sy) * SX_ + sx;
    const float *c1 = two ? c0 + SX_ * SY_ : c0;
    const int k0 = z0 + tz, k1 = two ? k0 + 1 : k0;
    const long long cell0 = L.idx(i, j, k0), cell1 = L.idx(i, j, k1);
    float2 rhs;
    if (MODE == REINIT) {
      float gp0[3], gp1[3], gm0[3], gm1[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        float2 a7[7], v[6];  // phi / dx at c-3 .. c+3; scaled D1(c-2 .. c+3) for both cells
#pragma unroll
        for (int q = -3; q <= 3; q++) a7[q + 3] = mul2(make_float2(c0[q * st[d]], c1[q * st[d]]), inv[d]);
#pragma unroll
        for (int f = 0; f < 6; f++) v[f] = fma2(sp(-1.f), a7[f], a7[f + 1]);
        float2 p, m;
        weno5_pm_x2(v, p, m);
        gp0[d] = p.x; gp1[d] = p.y;
        gm0[d] = m.x; gm1[d] = m.y;
      }
      const float pc0 = a.use0 ? a.phi0[cell0] : c0[0];
      const float pc1 = a.use0 ? a.phi0[cell1] : c1[0];
      rhs.x = reinit_term<float, false>(pc0, gp0, gm0, a.dx_sq, a.use0 != 0);
      rhs.y = reinit_term<float, false>(pc1, gp1, gm1, a.dx_sq, a.use0 != 0);
    } else {
      float vel0[3], vel1[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        vel0[d] = (MODE == ADV_CONST) ? a.vconst[d] : a.vel[d][cell0];
        vel1[d] = (MODE == ADV_CONST) ? a.vconst[d] : a.vel[d][cell1];
      }
      float2 dot = sp(0.f);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        // per lane: the backward stencil D1(c-2..c+2) for v > 0, the forward
        // stencil D1(c+3..c-1) otherwise (spatial_derivatives3d.f.in:2756-2812);
        // the six differences are loaded at fixed offsets and the lane's
        // stencil is selected in registers
        float2 a7[7], D[6];
#pragma unroll
        for (int q = -3; q <= 3; q++) a7[q + 3] = mul2(make_float2(c0[q * st[d]], c1[q * st[d]]), inv[d]);
#pragma unroll
        for (int f = 0; f < 6; f++) D[f] = fma2(sp(-1.f), a7[f], a7[f + 1]);
        if constexpr (MODE == ADV_CONST) {
          // one velocity for the whole grid: the side and the zero cut are
          // uniform, so the stencil is chosen by a (non-divergent) branch
          const float u = a.vconst[d];
          if (fabsf(u) < 1e-11f) continue;
          const float2 g = u > 0.f ? weno5_x2(D[0], D[1], D[2], D[3], D[4]) : weno5_x2(D[5], D[4], D[3], D[2], D[1]);
          dot = fma2(sp(u), g, dot);
        } else {
          const bool b0 = vel0[d] > 0.f, b1 = vel1[d] > 0.f;
          float2 v[5];
#pragma unroll
          for (int q = 0; q < 5; q++) {
            v[q].x = b0 ? D[q].x : D[5 - q].x;
            v[q].y = b1 ? D[q].y : D[5 - q].y;
          }
          float2 g = weno5_x2(v[0], v[1], v[2], v[3], v[4]);
          if (fabsf(vel0[d]) < 1e-11f) g.x = 0.f;
          if (fabsf(vel1[d]) < 1e-11f) g.y = 0.f;
          dot = fma2(make_float2(vel0[d], vel1[d]), g, dot);
        }
      }
      rhs = make_float2(-dot.x, -dot.y);
    }
    const float2 u0 = make_float2(c0[0], c1[0]);
    float2 u;
    if (a.stage == 1) {
      u = fma2(sp(a.dt), rhs, u0);
    } else {
      const float2 un = make_float2(a.phi_n[cell0], a.phi_n[cell1]);
      if (a.stage == 2)
        u = fma2(sp(0.75f), un, mul2(sp(0.25f), fma2(sp(a.dt), rhs, u0)));
      else
        u = fma2(sp(1.f / 3.f), un, mul2(sp(2.f / 3.f), fma2(sp(a.dt), rhs, u0)));
    }
    for (int lane = 0; lane < (two ? 2 : 1); lane++) {
      const int k = lane ? k1 : k0;
      const float val = lane ? u.y : u.x;
      const long long c = L.idx(i, j, k);
      a.out[c] = val;
      if (a.periodic) {
        // the cell's periodic images in the ghost layers (up to 7: each
        // combination of the axes along which it lies within 3 of a face)
        const int oi = i < 3 ? L.nx : (i >= L.nx - 3 ? -L.nx : 0);
        const int oj = j < 3 ? L.ny : (j >= L.ny - 3 ? -L.ny : 0);
        const int ok = k < 3 ? L.nz : (k >= L.nz - 3 ? -L.nz : 0);
        if (oi | oj | ok) {
          const long long sx = oi, sy = L.py * oj, sz = L.pz * ok;
          if (oi) a.out[c + sx] = val;
          if (oj) a.out[c + sy] = val;
          if (ok) a.out[c + sz] = val;
          if (oi && oj) a.out[c + sx + sy] = val;
          if (oi && ok) a.out[c + sx + sz] = val;
          if (oj && ok) a.out[c + sy + sz] = val;
          if (oi && oj && ok) a.out[c + sx + sy + sz] = val;
        }
      }
    }
  }
}

// 32 x 8 x TZ_ tiles; the steppers launch TZ_ = 8, or 4 where 4-plane tiles
// fill the machine's waves better (fused_driver.cuh, stage_tz_f32)
template <int MODE, int TZ_ = TZ>
__global__ void __launch_bounds__(TX * TY) k_stage_f32(const __grid_constant__ CUtensorMap tm, StageArgs<float> a) {
  constexpr int SZ_ = TZ_ + 6;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float *tile = reinterpret_cast<float *>(smem_raw);
  __shared__ __align__(8) uint64_t bar;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = tx + TX * ty;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * TZ_;
  if (tid == 0) {
    prefetch_tmap(&tm);
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar, (uint32_t)(SX * SY * SZ_ * sizeof(float)));
    tma_load_3d(tile, &tm, x0 + GX - 4, y0 + GY - 3, z0 + GZ - 3, &bar);
  }
  if (!mbar_wait(&bar, 0, kMaxPolls)) {
    if (tid == 0) atomicExch(a.err, LSMGPU_ERR_TIMEOUT);
    mbar_wait(&bar, 0, kMaxPolls);
    return;
  }
  if (a.ghost) {
    fill_face_ghosts<float>(tile, SX, SY, SZ_, x0 - 4, y0 - 3, z0 - 3, a.L, a.ghost);
    __syncthreads();
  }
  f32_tile<MODE, TZ_>(tile, a, x0, y0, z0, tx, ty);
}

}  // namespace fused
}  // namespace lsmgpu
