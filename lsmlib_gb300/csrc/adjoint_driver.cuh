// Host driver of the adjoints (periodic advection; periodic reinitialization
// in the phi0 sign form): forward sweep with checkpoints, the objective or the
// caller's dJ/dphi_T, then per checkpoint segment a forward recomputation that
// keeps every stage state and the reverse sweep over it.
//
// Memory (padded layout, E elements per field): 3 forward fields, one
// checkpoint per `ckpt` steps, 3*ckpt - 1 segment stage states, 3 adjoint
// fields; advection: 3 velocity fields and 3 velocity accumulators;
// reinitialization: 3 linearisation coefficients, side bits and the sign
// source's accumulator.
#pragma once

#include <vector>

#include <type_traits>

#include "adjoint.cuh"
#include "adjoint_x2.cuh"
#include "fused_driver.cuh"

namespace lsmgpu {
namespace adj {

enum { ADJ_MODE_ADVECT = 0, ADJ_MODE_REINIT = 1 };

struct AdjSpec {
  int mode;          // ADJ_MODE_ADVECT / ADJ_MODE_REINIT (phi0 sign form)
  int n_steps, ckpt;
  double dt, dx, dy, dz, eps;
};

// Arrays of one call (host or device; any output may be null)
template <class R>
struct AdjIO {
  const R *phi;          // initial state over gb (fill-box values used)
  const R *vel[3];       // advection velocity over vb
  const R *tgt;          // objective target over gb (objective form)
  const R *grad_out;     // dJ/dphi_T over gb (vector-Jacobian form)
  double *J;             // objective value (objective form)
  R *phi_out;            // final state over gb
  R *gphi;               // dJ/dphi over gb
  R *gvel[3];            // dJ/dvel over vb
};

// march threads per SM the chunk lengths aim at (z march of k_adj_xz_row,
// y march of k_adj_y)
#ifndef LSMGPU_ADJ_Z_THREADS
#define LSMGPU_ADJ_Z_THREADS 2048
#endif
#ifndef LSMGPU_ADJ_Y_THREADS
#define LSMGPU_ADJ_Y_THREADS 4096
#endif

// march length per thread: enough chunks for `per_sm` threads per SM (each
// march also computes 6 cells before its first output), at least 16 cells
inline int pick_chunk(int n_march, long long threads_per_chunk, int per_sm) {
  int sms = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (long long)per_sm * sms;
  long long chunks = (want + threads_per_chunk - 1) / threads_per_chunk;
  if (chunks < 1) chunks = 1;
  int c = (int)((n_march + chunks - 1) / chunks);
  if (c < 16) c = 16;
  if (c > n_march) c = n_march;
  return c;
}

// march length per CTA for kernels whose every CTA marches a chunk of n_march
// cells (plus `warm` warm-up cells) and `items` CTAs cover one chunk: the
// length that minimises waves x (chunk + warm), with `slots` CTAs resident at
// once (a partly filled last wave costs a whole one); the longest such chunk
inline int pick_chunk_waves(int n_march, long long items, long long slots, int warm) {
  int best = n_march;
  long long best_cost = -1;
  for (int c = n_march; c >= 8; c--) {
    const long long n = ((long long)n_march + c - 1) / c;
    const long long waves = (items * n + slots - 1) / slots;
    const long long cost = waves * (c + warm);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = c;
    }
  }
  return best;
}

// the FP32 reverse stages run the two-line kernels of adjoint_x2.cuh where
// the x rows fit one CTA
template <class R, bool EXACT>
constexpr bool adj_x2_kernels() {
  return std::is_same<R, float>::value && !EXACT;
}
inline bool adj_x2_fits(const Layout &L) { return L.nx <= kRowMax && L.elems() < (1LL << 31); }

// one reverse stage: x and z faces (writes out), then y faces (adds to out);
// internal linkage, so the shared-memory limit is set on this unit's kernel
template <class R, bool EXACT, int MODE>
static void launch_adj_stage(const AdjStageArgs<R> &a) {
  const Layout &L = a.L;
  dim3 blk(32, kRows);
  if constexpr (adj_x2_kernels<R, EXACT>()) {
    if (adj_x2_fits(L)) {
      const int w = (L.nx + 31) / 32;
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(k_adj_x_x2<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)adj_x_x2_smem(kRowMax));
        attr = true;
      }
      dim3 g1((unsigned)((L.ny + 1) / 2), (unsigned)((L.nz + a.xchunk - 1) / a.xchunk));
      k_adj_x_x2<MODE><<<g1, dim3(32, w), adj_x_x2_smem(L.nx), stream()>>>(a);
      note_launch();
      dim3 g2((unsigned)((L.nx + 31) / 32), (unsigned)((L.ny + 2 * kMarchRows - 1) / (2 * kMarchRows)),
              (unsigned)((L.nz + a.zchunk - 1) / a.zchunk));
      k_adj_march_x2<MODE, 2><<<g2, dim3(32, kMarchRows), 0, stream()>>>(a);
      note_launch();
      dim3 g3((unsigned)((L.nx + 31) / 32), (unsigned)((L.nz + 2 * kMarchRows - 1) / (2 * kMarchRows)),
              (unsigned)((L.ny + a.ychunk - 1) / a.ychunk));
      k_adj_march_x2<MODE, 1><<<g3, dim3(32, kMarchRows), 0, stream()>>>(a);
      note_launch();
      return;
    }
  }
  if (L.nx <= kRowMax) {
    // one CTA per x row
    const int w = (L.nx + 31) / 32;
    const size_t smem = 2 * 6 * (size_t)w * 32 * sizeof(R);
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_adj_xz_row<R, EXACT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(2 * 6 * kRowMax * sizeof(R)));
      attr = true;
    }
    dim3 g1((unsigned)L.ny, (unsigned)((L.nz + a.zchunk - 1) / a.zchunk));
    k_adj_xz_row<R, EXACT, MODE><<<g1, dim3(32, w), smem, stream()>>>(a);
  } else {
    dim3 g1((unsigned)((L.nx + kSeg - 1) / kSeg), (unsigned)((L.ny + kRows - 1) / kRows),
            (unsigned)((L.nz + a.zchunk - 1) / a.zchunk));
    k_adj_xz<R, EXACT, MODE><<<g1, blk, 0, stream()>>>(a);
  }
  note_launch();
  dim3 g2((unsigned)((L.nx + 31) / 32), (unsigned)((L.nz + kRows - 1) / kRows),
          (unsigned)((L.ny + a.ychunk - 1) / a.ychunk));
  k_adj_y<R, EXACT, MODE><<<g2, blk, 0, stream()>>>(a);
  note_launch();
}

// checkpoint_every = 0: the largest spacing K <= n_steps whose stored fields
// (3K segment stages, n_steps / K checkpoints, ~16 work fields) fit in half
// of the free device memory; K = n_steps keeps the whole trajectory and
// recomputes nothing.
inline int auto_checkpoint(int n_steps, long long field_bytes, bool want_grad) {
  if (n_steps <= 1 || !want_grad) return n_steps > 1 ? n_steps : 1;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return 8 < n_steps ? 8 : n_steps;
  }
  const double budget = 0.5 * (double)free_b;
  for (int k = n_steps; k > 1; k--) {
    const long long fields = 3LL * k + (n_steps + k - 1) / k + 16;
    if ((double)fields * (double)field_bytes <= budget) return k;
  }
  return 1;
}

template <class R, bool EXACT>
int run(const char *name, const Box &gb, const Box &fb, const Box &vb, const AdjSpec &sp, const AdjIO<R> &io) {
  using fused::StageArgs;
  const bool advect = sp.mode == ADJ_MODE_ADVECT;
  Call call(name);
  if (!gb.contains(fb, 3, 3, 3)) call.fail("ghost box must hold 3 ghost cells around the fill box");
  if (advect && !vb.contains(fb, 0, 0, 0)) call.fail("velocity ghost box does not cover the fill box");
  const int nx = (int)fb.n(0), ny = (int)fb.n(1), nz = (int)fb.n(2);
  if (fb.empty() || nx < 6 || ny < 6 || nz < 6) call.fail("fill box must be at least 6 cells per axis");
  if (!call.ok()) return LSMGPU_ERR_BOUNDS;
  const int ngv = advect ? (io.gvel[0] != nullptr) + (io.gvel[1] != nullptr) + (io.gvel[2] != nullptr) : 0;
  const bool objective = io.tgt != nullptr;
  if (sp.n_steps < 0 || sp.ckpt < 0 || (objective && !(sp.eps > 0.0)) || (ngv != 0 && ngv != 3) ||
      (ngv == 3 && !io.gphi) || (io.gphi && !objective && !io.grad_out)) {
    set_error(LSMGPU_ERR_ARGUMENT,
              "%s: need n_steps >= 0, checkpoint_every >= 0, heaviside_eps > 0, a gradient source, and "
              "velocity gradients either all three (with grad_phi) or none",
              name);
    return LSMGPU_ERR_ARGUMENT;
  }
  const bool want_grad = io.gphi != nullptr, want_gvel = ngv == 3;

  const R *phi_d = call.in(io.phi, gb.size());
  const R *tgt_d = objective ? call.in(io.tgt, gb.size()) : nullptr;
  const R *gout_d = (!objective && want_grad) ? call.in(io.grad_out, gb.size()) : nullptr;
  const R *vel_d[3] = {nullptr, nullptr, nullptr};
  if (advect)
    for (int d = 0; d < 3; d++) vel_d[d] = call.in(io.vel[d], vb.size());
  R *gphi_d = want_grad ? call.out(io.gphi, gb.size()) : nullptr;
  R *gvel_d[3] = {nullptr, nullptr, nullptr};
  if (want_gvel)
    for (int d = 0; d < 3; d++) gvel_d[d] = call.out(io.gvel[d], vb.size());
  R *phi_out_d = io.phi_out ? call.inout(io.phi_out, gb.size()) : nullptr;
  double *J_d = (objective && io.J) ? call.scalar_out(io.J) : nullptr;

  const Layout L = fused::make_layout(nx, ny, nz);
  const long long ne = L.elems();
  const int K = sp.ckpt > 0 ? sp.ckpt : auto_checkpoint(sp.n_steps, ne * (long long)sizeof(R), want_grad);
  const int nck = sp.n_steps > 0 ? (sp.n_steps + K - 1) / K : 1;
  R *X = call.temp<R>(ne), *T1 = call.temp<R>(ne), *T2 = call.temp<R>(ne);
  R *TG = objective ? call.temp<R>(ne) : nullptr;
  R *V[3] = {nullptr, nullptr, nullptr};
  if (advect)
    for (int d = 0; d < 3; d++) V[d] = call.temp<R>(ne);
  std::vector<R *> ck(nck);
  for (int c = 0; c < nck; c++) ck[c] = call.temp<R>(ne);
  const long long ncell = (long long)nx * ny * nz;
  const int nblk = (int)((ncell + kObjThreads - 1) / kObjThreads);
  double *partial = objective ? call.temp<double>(nblk) : nullptr;
  double *Jdev = objective ? call.temp<double>(1) : nullptr;
  int *err = call.temp<int>(1);
  R *LA = nullptr, *LB = nullptr, *LC = nullptr, *GV[3] = {nullptr, nullptr, nullptr};
  R *KAP[3] = {nullptr, nullptr, nullptr}, *GP0 = nullptr;
  unsigned char *SIDE = nullptr;
  std::vector<R *> U;
  if (want_grad) {
    LA = call.temp<R>(ne);
    LB = call.temp<R>(ne);
    LC = call.temp<R>(ne);
    if (want_gvel)
      for (int d = 0; d < 3; d++) GV[d] = call.temp<R>(ne);
    if (!advect) {
      for (int d = 0; d < 3; d++) KAP[d] = call.temp<R>(ne);
      SIDE = call.temp<unsigned char>(ne);
      GP0 = call.temp<R>(ne);
    }
    U.assign(3 * K, nullptr);
    for (int m = 1; m < 3 * K; m++) U[m] = call.temp<R>(ne);
  }
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);

  cudaStream_t s = stream();
  cudaMemsetAsync(err, 0, sizeof(int), s);
  const dim3 pblk = fused::pack_block(), pgrd = fused::pack_grid(nx, ny, nz, fused::GX);
  LSMGPU_LAUNCH(fused::k_pack<R>, pgrd, pblk, 0, ck[0], L, view(phi_d, gb), gb, fb.lo[0], fb.lo[1], fb.lo[2]);
  if (objective)
    LSMGPU_LAUNCH(fused::k_pack<R>, pgrd, pblk, 0, TG, L, view(tgt_d, gb), gb, fb.lo[0], fb.lo[1], fb.lo[2]);
  for (int d = 0; d < 3 && advect; d++)
    LSMGPU_LAUNCH(fused::k_pack<R>, pgrd, pblk, 0, V[d], L, view(vel_d[d], vb), vb, fb.lo[0], fb.lo[1], fb.lo[2]);
  {
    const dim3 fblk(32, 4, 2);
    dim3 gf((unsigned)((nx + 6 + 31) / 32), (unsigned)((ny + 6 + 3) / 4), (unsigned)((nz + 6 + 1) / 2));
    // the initial state is the periodic extension of the fill-box values
    LSMGPU_LAUNCH(k_fill_periodic<R>, gf, fblk, 0, ck[0], L);
  }
  cudaMemcpyAsync(X, ck[0], (size_t)ne * sizeof(R), cudaMemcpyDeviceToDevice, s);

  auto tmap = [&](const R *p, CUtensorMap *m) {
    return advect ? fused::encode_stage_tmap<R, fused::ADV_FIELD, EXACT>(m, p, L)
                  : fused::encode_stage_tmap<R, fused::REINIT, EXACT>(m, p, L);
  };
  CUtensorMap tX, tT1, tT2;
  if (!tmap(X, &tX) || !tmap(T1, &tT1) || !tmap(T2, &tT2)) {
    call.fail("tensor map encoding failed");
    return LSMGPU_ERR_CUDA;
  }

  StageArgs<R> fa{};
  fa.L = L;
  for (int d = 0; d < 3; d++) fa.vel[d] = V[d];
  fa.inv[0] = R(1.0) / (R)sp.dx;
  fa.inv[1] = R(1.0) / (R)sp.dy;
  fa.inv[2] = R(1.0) / (R)sp.dz;
  fa.dt = (R)sp.dt;
  {
    const R m = rmax(rmax((R)sp.dx, (R)sp.dy), (R)sp.dz);
    fa.dx_sq = m * m;
  }
  fa.phi0 = ck[0];  // reinitialization sign source: the initial state
  fa.use0 = 1;
  fa.periodic = 1;
  fa.err = err;
  auto stage = [&](const CUtensorMap &t, R *out, int st) {
    fa.stage = st;
    fa.out = out;
    if (advect) fused::launch_stage<R, fused::ADV_FIELD, EXACT>(t, fa);
    else fused::launch_stage<R, fused::REINIT, EXACT>(t, fa);
  };
  // one forward TVD-RK3 step: src -> o1 -> o2 -> dst (dst may be src)
  auto fwd_step = [&](const CUtensorMap &t_src, R *src, const CUtensorMap &t_o1, R *o1,
                      const CUtensorMap &t_o2, R *o2, R *dst) {
    fa.phi_n = src;
    stage(t_src, o1, 1);
    stage(t_o1, o2, 2);
    if (dst) stage(t_o2, dst, 3);
  };

  // stage states of a segment: U[3m] = state at step m, U[3m+1], U[3m+2] its
  // two intermediate stages (U[0] is the segment's checkpoint)
  std::vector<CUtensorMap> tU(want_grad ? 3 * K : 0);
  auto map_segment = [&](int seg) {
    U[0] = ck[seg];
    for (int m = 0; m < 3 * K; m++)
      if ((m == 0 || seg == nck - 1) && !tmap(U[m], &tU[m])) return false;
    return true;
  };
  if (want_grad && sp.n_steps > 0 && !map_segment(nck - 1)) {
    call.fail("tensor map encoding failed");
    return LSMGPU_ERR_CUDA;
  }

  // ---- forward sweep with checkpoints ----------------------------------------
  // The last segment's stage states are written straight into U, so the
  // reverse sweep does not recompute it (with checkpoint_every >= n_steps
  // nothing is recomputed).
  const int last0 = want_grad ? (nck - 1) * K : sp.n_steps;
  for (int n = 0; n < sp.n_steps; n++) {
    if (n < last0) {
      fwd_step(tX, X, tT1, T1, tT2, T2, X);
      if ((n + 1) % K == 0 && (n + 1) < sp.n_steps)
        cudaMemcpyAsync(ck[(n + 1) / K], X, (size_t)ne * sizeof(R), cudaMemcpyDeviceToDevice, s);
    } else {
      const int m = n - last0;
      R *dst = (n + 1 < sp.n_steps) ? U[3 * m + 3] : X;
      fwd_step(tU[3 * m], U[3 * m], tU[3 * m + 1], U[3 * m + 1], tU[3 * m + 2], U[3 * m + 2], dst);
    }
  }
  if (phi_out_d) {
    const dim3 blk = fused::pack_block(), grd = fused::pack_grid(nx, ny, nz, 3);
    LSMGPU_LAUNCH(fused::k_unpack<R>, grd, blk, 0, view(phi_out_d, gb), gb, X, L, fb.lo[0], fb.lo[1], fb.lo[2]);
  }
  if (objective) {
    const double vol = sp.dx * sp.dy * sp.dz;
    LSMGPU_LAUNCH(k_objective<R>, dim3((unsigned)nblk), dim3(kObjThreads), 0, X, TG, L, sp.eps, vol, LA,
                  partial);
    LSMGPU_LAUNCH(k_objective_fold, dim3(1), dim3(1024), 0, partial, nblk, vol, J_d ? J_d : Jdev);
  } else if (want_grad) {
    // dJ/dphi_T given by the caller
    LSMGPU_LAUNCH(fused::k_pack<R>, pgrd, pblk, 0, LA, L, view(gout_d, gb), gb, fb.lo[0], fb.lo[1], fb.lo[2]);
  }

  // ---- reverse sweep ------------------------------------------------------------
  if (want_grad) {
    if (want_gvel)
      for (int d = 0; d < 3; d++) cudaMemsetAsync(GV[d], 0, (size_t)ne * sizeof(R), s);
    if (GP0) cudaMemsetAsync(GP0, 0, (size_t)ne * sizeof(R), s);
    AdjStageArgs<R> aa{};
    aa.L = L;
    for (int d = 0; d < 3; d++) {
      aa.vel[d] = V[d];
      aa.gvel[d] = GV[d];
      aa.kap[d] = KAP[d];
    }
    aa.side = SIDE;
    aa.dt = (R)sp.dt;
    aa.inv[0] = fa.inv[0]; aa.inv[1] = fa.inv[1]; aa.inv[2] = fa.inv[2];
    // thread targets per SM measured best at 192^3 (more chunks than resident
    // threads: latency hiding outweighs the extra warm-up cells)
    if (adj_x2_kernels<R, EXACT>() && adj_x2_fits(L)) {
      // two lines per thread; chunks from the resident CTAs of each kernel
      int sms = 152, dev = 0, occ_x = 1, occ_m = 1;
      if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if constexpr (adj_x2_kernels<R, EXACT>()) {
        const int w = (nx + 31) / 32;
        auto occ = [&](auto kern, int threads, size_t smem) {
          int v = 0;
          if (smem) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adj_x_x2_smem(kRowMax));
          if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, threads, smem) != cudaSuccess || v < 1) {
            cudaGetLastError();
            v = 1;
          }
          return v;
        };
        occ_x = advect ? occ(k_adj_x_x2<ADJ_ADV>, 32 * w, adj_x_x2_smem(nx))
                       : occ(k_adj_x_x2<ADJ_LIN>, 32 * w, adj_x_x2_smem(nx));
        occ_m = advect ? occ(k_adj_march_x2<ADJ_ADV, 1>, 32 * kMarchRows, 0)
                       : occ(k_adj_march_x2<ADJ_LIN, 1>, 32 * kMarchRows, 0);
      }
      const long long cols = (nx + 31) / 32;
      // the x kernel carries nothing between planes: short chunks keep its
      // resident CTAs full to the end
      aa.xchunk = nz < 8 ? nz : 8;
      (void)occ_x;
      aa.zchunk = pick_chunk_waves(nz, cols * ((ny + 2 * kMarchRows - 1) / (2 * kMarchRows)), (long long)occ_m * sms, 6);
      aa.ychunk = pick_chunk_waves(ny, cols * ((nz + 2 * kMarchRows - 1) / (2 * kMarchRows)), (long long)occ_m * sms, 6);
    } else {
      aa.zchunk = pick_chunk(nz, nx <= kRowMax ? 32LL * ((nx + 31) / 32) * ny : 32LL * ((nx + kSeg - 1) / kSeg) * ny,
                             LSMGPU_ADJ_Z_THREADS);
      aa.ychunk = pick_chunk(ny, (long long)nx * nz, LSMGPU_ADJ_Y_THREADS);
    }
    const dim3 cgrid((unsigned)((nx + 31) / 32), (unsigned)((ny + 7) / 8), (unsigned)nz), cblk(32, 8);
    // one reverse stage at forward state `st`
    auto rstage = [&]() {
      if (advect) {
        launch_adj_stage<R, EXACT, ADJ_ADV>(aa);
      } else {
        LSMGPU_LAUNCH((k_reinit_lin<R, EXACT>), cgrid, cblk, 0, aa.s, (const R *)ck[0], aa.M, aa.mscale, aa.dt,
                      fa.dx_sq, aa.inv[0], aa.inv[1], aa.inv[2], L, KAP[0], KAP[1], KAP[2], SIDE, GP0);
        launch_adj_stage<R, EXACT, ADJ_LIN>(aa);
      }
    };
    for (int seg = nck - 1; seg >= 0 && sp.n_steps > 0; seg--) {
      const int s0 = seg * K, s1 = (s0 + K < sp.n_steps) ? s0 + K : sp.n_steps, ns = s1 - s0;
      if (seg != nck - 1) {  // the last segment is still in U from the forward sweep
        if (!map_segment(seg)) {
          call.fail("tensor map encoding failed");
          return LSMGPU_ERR_CUDA;
        }
        for (int m = 0; m < ns; m++)
          fwd_step(tU[3 * m], U[3 * m], tU[3 * m + 1], U[3 * m + 1], tU[3 * m + 2], U[3 * m + 2],
                   m + 1 < ns ? U[3 * m + 3] : nullptr);
      }
      for (int m = ns - 1; m >= 0; m--) {
        aa.s = U[3 * m + 2]; aa.M = LA; aa.mscale = R(2.0 / 3.0);
        aa.P = nullptr; aa.Q = nullptr; aa.out = LB;
        rstage();
        aa.s = U[3 * m + 1]; aa.M = LB; aa.mscale = R(0.25); aa.out = LC;
        rstage();
        aa.s = U[3 * m]; aa.M = LC; aa.mscale = R(1.0);
        aa.P = LA; aa.pscale = R(1.0 / 3.0); aa.Q = LB; aa.qscale = R(0.75); aa.out = LA;
        rstage();
      }
    }
    if (GP0) LSMGPU_LAUNCH(k_add_interior<R>, cgrid, cblk, 0, LA, (const R *)GP0, L);
    Grid3 gg = cover(gb);
    LSMGPU_LAUNCH(k_unpack_interior<R>, gg.grid, gg.block, 0, view(gphi_d, gb), gb, LA, L, fb.lo[0], fb.lo[1],
                  fb.lo[2]);
    if (want_gvel) {
      Grid3 gv = cover(vb);
      for (int d = 0; d < 3; d++)
        LSMGPU_LAUNCH(k_unpack_interior<R>, gv.grid, gv.block, 0, view(gvel_d[d], vb), vb, GV[d], L, fb.lo[0],
                      fb.lo[1], fb.lo[2]);
    }
  }
  int herr = 0;
  cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  call.finish();
  cudaStreamSynchronize(s);
  if (herr != 0) {
    set_error(herr, "%s: a bounded device wait gave up (TMA tile load)", name);
    return herr;
  }
  return lsmgpu_get_last_error(nullptr, 0);
}

}  // namespace adj
}  // namespace lsmgpu
