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
// Kernel (one per adjoint stage): a CTA of 32 x 16 threads owns a 32 x 16
// column of cells and marches along z through a chunk of planes.
//   z: each thread keeps a 7-value window of s down its own column and a ring
//      of six face sums, computing the slots of the cell 3 planes ahead;
//   x, y: per plane the CTA stages the plane's s (a cross of 44 x 16 and
//      32 x 28 cells) in shared memory, computes the slots of the 38 x 16
//      x-extended and 32 x 22 y-extended cells into shared memory, then each
//      thread gathers its two faces per axis.
// Redundant slot work: x 38/32, y 22/16, z (chunk + 6)/chunk.
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

constexpr int AX = 32, AY = 16;              // threads / cells per plane
constexpr int HX = AX + 12, HY = AY + 12;    // staged s plane: 44 x 28 (cross)
constexpr int GXN = AX + 6, GYN = AY + 6;    // slot cells: 38 x 16 (x), 32 x 22 (y)
constexpr int NJX = GXN * AY, NJY = AX * GYN;  // 608 x-slot and 704 y-slot cells
constexpr int NCROSS = HX * AY + AX * 12;      // 704 + 384 staged s values per plane

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
template <class R, bool EXACT>
__device__ __forceinline__ R adv_slots(const R a[7], R u, R mu, R dt, R inv, R G[6]) {
#pragma unroll
  for (int m = 0; m < 6; m++) G[m] = R(0);
  // spatial_derivatives3d.f.in:2756-2812: no derivative where |u| < zero_tol
  if (fabs(u) < R(Consts<double>::zero_tol)) return R(0);
  R D[6];  // D(c+f) for f = -2..3
#pragma unroll
  for (int f = 0; f < 6; f++) D[f] = (a[f + 1] - a[f]) * inv;
  const bool minus = u > R(0);
  R v[5], dv[5];
#pragma unroll
  for (int q = 0; q < 5; q++) v[q] = minus ? D[q] : D[5 - q];
  const R W = weno5_adj<R, EXACT>(v, dv);
  const R ybar = dt * mu * (-u) * inv;
  // minus: v_q on face c-2+q (slot q); plus: v_q on face c+3-q (slot 5-q)
#pragma unroll
  for (int m = 0; m < 6; m++) {
    const R lo = (m < 5) ? dv[m] : R(0);
    const R hi = (m > 0) ? dv[5 - m] : R(0);
    G[m] = ybar * (minus ? lo : hi);
  }
  return dt * mu * (-W);
}

template <class R>
struct AdjStageArgs {
  Layout L;
  const R *s;         // forward state the stage was linearised at
  const R *M;         // adjoint input; mu = mscale * M
  const R *P, *Q;     // optional pointwise terms pscale * P + qscale * Q
  R *out;             // mu + dt L_s^T mu (+ P, Q terms), interior cells
  const R *vel[3];
  R *gvel[3];         // velocity adjoint accumulators (nullptr: not wanted)
  R mscale, pscale, qscale;
  R dt;
  R inv[3];
  int zchunk;
};

template <class R>
__device__ __forceinline__ long long widx(const Layout &L, int i, int j, int k) {
  return L.idx(wrapi(i, L.nx), wrapi(j, L.ny), wrapi(k, L.nz));
}

constexpr int kSmemElems = HY * HX + 6 * AY * GXN + 6 * GYN * AX;
constexpr int kPer = (NJX + NJY + AX * AY - 1) / (AX * AY);  // slot cells per thread per plane (3)

template <class R, bool EXACT>
__global__ void __launch_bounds__(AX * AY) k_adj_stage(AdjStageArgs<R> a) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  R (*sS)[HX] = reinterpret_cast<R (*)[HX]>(adj_smem);
  R (*sGx)[AY][GXN] = reinterpret_cast<R (*)[AY][GXN]>(adj_smem + sizeof(R) * HY * HX);
  R (*sGy)[GYN][AX] = reinterpret_cast<R (*)[GYN][AX]>(adj_smem + sizeof(R) * (HY * HX + 6 * AY * GXN));
  const Layout &L = a.L;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + AX * ty;
  const int x0 = blockIdx.x * AX, y0 = blockIdx.y * AY;
  const int z0 = blockIdx.z * a.zchunk;
  const int zend = min(z0 + a.zchunk, L.nz);
  const int i = x0 + tx, j = y0 + ty;
  const bool mine = i < L.nx && j < L.ny;
  const R dt = a.dt;
  // x/y part of the padded index of (wrapped) interior cell (x, y)
  auto planar = [&](int x, int y) { return (x + fused::GX) + (int)L.py * (y + fused::GY); };
  // z part for plane z (wrapped)
  auto zoff = [&](int z) { return L.pz * (long long)(wrapi(z, L.nz) + fused::GZ); };

  // cells this thread stages and computes slots for, in every plane
  int stg_off[kPer], stg_pos[kPer], job_off[kPer], job_code[kPer];
#pragma unroll
  for (int r = 0; r < kPer; r++) {
    const int e = tid + r * AX * AY;
    stg_off[r] = -1;
    if (e < NCROSS) {
      int lx, ly;
      if (e < HX * AY) {
        ly = 6 + e / HX;
        lx = e % HX;
      } else {
        const int q = e - HX * AY, row = q / AX;
        ly = row < 6 ? row : row + AY;
        lx = 6 + q % AX;
      }
      stg_off[r] = planar(wrapi(x0 - 6 + lx, L.nx), wrapi(y0 - 6 + ly, L.ny));
      stg_pos[r] = ly * HX + lx;
    }
    job_code[r] = -1;
    if (e < NJX) {  // x slots of cell (x0 - 3 + lx, y0 + ly)
      const int ly = e / GXN, lx = e % GXN, cx = x0 - 3 + lx, cy = y0 + ly;
      job_off[r] = planar(wrapi(cx, L.nx), wrapi(cy, L.ny));
      const bool own = lx >= 3 && lx < 3 + AX && cx < L.nx && cy < L.ny;
      job_code[r] = lx | (ly << 6) | (own << 12);
    } else if (e < NJX + NJY) {  // y slots of cell (x0 + lx, y0 - 3 + ly)
      const int q = e - NJX, ly = q / AX, lx = q % AX, cx = x0 + lx, cy = y0 - 3 + ly;
      job_off[r] = planar(wrapi(cx, L.nx), wrapi(cy, L.ny));
      const bool own = ly >= 3 && ly < 3 + AY && cx < L.nx && cy < L.ny;
      job_code[r] = lx | (ly << 6) | (own << 12) | (1 << 13);
    }
  }
  const int col = planar(wrapi(i, L.nx), wrapi(j, L.ny));

  // plane data, loaded one plane ahead: staged s, and mu and the velocity
  // component of each slot cell
  R stg[kPer], jm[kPer], jv[kPer];
  auto load_plane = [&](int k) {
    const long long zb = zoff(k);
#pragma unroll
    for (int r = 0; r < kPer; r++) {
      if (stg_off[r] >= 0) stg[r] = a.s[zb + stg_off[r]];
      if (job_code[r] >= 0) {
        jm[r] = a.M[zb + job_off[r]];
        jv[r] = (job_code[r] >> 13) ? a.vel[1][zb + job_off[r]] : a.vel[0][zb + job_off[r]];
      }
    }
  };
  load_plane(z0);

  R win[7];      // s(i, j, kk-3 .. kk+3)
  R mring[4];    // mu(i, j, kk-3 .. kk)
  R F[6];        // z-face sums for faces kk-2 .. kk+3
  R prevV = R(0);
#pragma unroll
  for (int q = 0; q < 6; q++) {
    win[q + 1] = a.s[zoff(z0 - 6 + q) + col];
    F[q] = R(0);
  }
#pragma unroll
  for (int q = 0; q < 4; q++) mring[q] = R(0);
  // column values of the next iteration: s(kk+3), M(kk), vel_z(kk)
  R cs = a.s[zoff(z0) + col], cm = a.M[zoff(z0 - 3) + col], cv = a.vel[2][zoff(z0 - 3) + col];

  for (int kk = z0 - 3; kk < zend + 3; kk++) {
    // ---- z: slots of cell (i, j, kk) from the column window ----------------
#pragma unroll
    for (int q = 0; q < 6; q++) win[q] = win[q + 1];
    win[6] = cs;
#pragma unroll
    for (int q = 0; q < 3; q++) mring[q] = mring[q + 1];
    mring[3] = a.mscale * cm;
    const R vz = cv;
    const long long zk = zoff(kk);
    if (kk + 1 < zend + 3) {
      cs = a.s[zoff(kk + 4) + col];
      cm = a.M[zoff(kk + 1) + col];
      cv = a.vel[2][zoff(kk + 1) + col];
    }
    R Az;
    {
      R G[6];
      const R gz = adv_slots<R, EXACT>(win, vz, mring[3], dt, a.inv[2], G);
      if (a.gvel[2] && mine && kk >= z0 && kk < zend) a.gvel[2][zk + col] += gz;
#pragma unroll
      for (int m = 0; m < 6; m++) F[m] += G[m];
      Az = prevV - F[0];  // Vbar(kk-3) - Vbar(kk-2)
      prevV = F[0];
#pragma unroll
      for (int m = 0; m < 5; m++) F[m] = F[m + 1];
      F[5] = R(0);
    }
    const int k = kk - 3;
    if (k < z0) continue;  // warm-up planes (uniform over the CTA)

    // ---- x, y: stage plane k of s, slots into shared memory ---------------
    __syncthreads();  // previous plane's gathers are done
    R *sflat = &sS[0][0];
#pragma unroll
    for (int r = 0; r < kPer; r++)
      if (stg_off[r] >= 0) sflat[stg_pos[r]] = stg[r];
    R m_cur[kPer], v_cur[kPer];
#pragma unroll
    for (int r = 0; r < kPer; r++) {
      m_cur[r] = jm[r];
      v_cur[r] = jv[r];
    }
    __syncthreads();
    if (k + 1 < zend) load_plane(k + 1);  // lands while this plane computes
    const long long zb = zoff(k);
#pragma unroll
    for (int r = 0; r < kPer; r++) {
      const int code = job_code[r];
      if (code < 0) continue;
      const int lx = code & 63, ly = (code >> 6) & 63;
      const bool own = (code >> 12) & 1, ydir = (code >> 13) & 1;
      R w7[7], G[6];
      if (!ydir) {
#pragma unroll
        for (int q = 0; q < 7; q++) w7[q] = sS[ly + 6][lx + q];
      } else {
#pragma unroll
        for (int q = 0; q < 7; q++) w7[q] = sS[ly + q][lx + 6];
      }
      const R g = adv_slots<R, EXACT>(w7, v_cur[r], a.mscale * m_cur[r], dt, a.inv[ydir], G);
      if (!ydir) {
#pragma unroll
        for (int m = 0; m < 6; m++) sGx[m][ly][lx] = G[m];
      } else {
#pragma unroll
        for (int m = 0; m < 6; m++) sGy[m][ly][lx] = G[m];
      }
      if (own && a.gvel[ydir]) a.gvel[ydir][zb + job_off[r]] += g;
    }
    __syncthreads();

    // ---- gather and write ---------------------------------------------------
    if (!mine) continue;
    R Ax = R(0), Ay = R(0);
#pragma unroll
    for (int m = 0; m < 6; m++) {
      Ax += sGx[m][ty][tx + 5 - m] - sGx[m][ty][tx + 6 - m];
      Ay += sGy[m][ty + 5 - m][tx] - sGy[m][ty + 6 - m][tx];
    }
    const long long c = zb + col;
    R o = mring[0] + ((Ax + Ay) + Az);
    if (a.P) o += a.pscale * a.P[c];
    if (a.Q) o += a.qscale * a.Q[c];
    a.out[c] = o;
  }
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
    const double p = (double)phiT[c];
    const double h = heaviside(p, eps) - heaviside((double)tgt[c], eps);
    h2 = h * h;
    if (lam) lam[c] = (R)(2.0 * h * delta_fn(p, eps) * vol);
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
