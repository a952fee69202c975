// Batched WENO5 / TVD-RK3 advection of many independent, unevenly sized grids.
//
// All grids live in one set of work buffers (the padded layout of the fused
// steppers, one region per grid).  Each RK stage is ONE persistent launch:
// CTAs (a fixed number per SM) pull 32 x 8 x TZ tiles of any grid from a
// global work counter, so small and large grids share the machine without a
// launch per grid; each CTA double-buffers its tiles in shared memory with
// TMA loads from per-grid tensor maps kept in global memory.  The n_steps x 3
// stage launches of a call are captured once into a CUDA graph and replayed.
// Each grid gets the tile shape (32 x 8 or 16 x 16 cells of a plane) that
// pads its x rows least: the 256 threads of a CTA cover one tile plane, and
// lanes past the row's end idle through the whole tile.  A table of
// (grid, tile position) per global tile index, built on the host, replaces
// any search or division in the kernel.  The tile depth TZ and the CTAs per
// SM come from a small autotuner that times the candidates on the batch at
// hand and keeps the choice per batch shape for the life of the process.
//
// For comparison the same batch can run as a loop of single-grid launches
// (one stage kernel per grid per stage), which is what calling the
// single-grid stepper grid by grid amounts to.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "fused_stage.cuh"
#include "lsmgpu_common.cuh"
#include "../../include/lsmgpu.h"

namespace lsmgpu {
namespace batch {

using fused::GX;
using fused::GY;
using fused::GZ;
using fused::Layout;
using fused::SX;
using fused::SY;
using fused::StageArgs;
using fused::TX;
using fused::TY;

struct GridDesc {
  Layout L;
  long long off;  // element offset of this grid's region in each work buffer
  float vconst[3], inv[3], dt;
  int tile_base;  // first global tile index of this grid
  int ntx, nty, ntz;
  int wide;       // 1: 32 x 8 tiles, 0: 16 x 16 tiles
};

// tile shapes: (32 x 8) and (16 x 16) cells per plane, 8 halo columns and 6
// halo rows; the shared-memory buffer holds the larger staged plane
constexpr int kWideSX = 32 + 8, kWideSY = 8 + 6, kNarrowSX = 16 + 8, kNarrowSY = 16 + 6;
constexpr int kPlaneMax = kWideSX * kWideSY > kNarrowSX * kNarrowSY ? kWideSX * kWideSY : kNarrowSX * kNarrowSY;

// one global tile: its grid and position (tiles per axis < 2^16 per grid)
struct TileRef {
  int g;
  unsigned short bx, by;
  unsigned short bz, pad;
};

template <int TZ_>
__global__ void __launch_bounds__(TX * TY) k_batch_stage(const GridDesc *__restrict__ gd,
                                                        const CUtensorMap *__restrict__ tmaps,
                                                        const TileRef *__restrict__ tiles_ref, int ntiles, int stage,
                                                        float *A, float *B, float *C, int *counter, int *err,
                                                        int periodic) {
  constexpr int SZ_ = TZ_ + 6;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // buffer b at tiles + b * kPlaneMax * SZ_ (no indexed pointer array: that
  // would live in local memory)
  float *const tiles = reinterpret_cast<float *>(smem_raw);
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int s_tile[2];
  const int tid = threadIdx.x + TX * threadIdx.y;
  const int in_buf = stage - 1;  // A, B, C
  float *outb = stage == 1 ? B : (stage == 2 ? C : A);

  auto issue = [&](int t, int b) {
    const TileRef r = tiles_ref[t];
    const int wide = gd[r.g].wide;
    const int tw = wide ? 32 : 16, th = wide ? 8 : 16;
    const CUtensorMap *m = tmaps + 3 * r.g + in_buf;
    const uint32_t bytes = (uint32_t)((wide ? kWideSX * kWideSY : kNarrowSX * kNarrowSY) * SZ_ * sizeof(float));
    // the maps live in global memory and are rewritten between calls
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"((uint64_t)m) : "memory");
    mbar_arrive_expect_tx(&bars[b], bytes);
    tma_load_3d(tiles + b * kPlaneMax * SZ_, m, r.bx * tw + GX - 4, r.by * th + GY - 3, r.bz * TZ_ + GZ - 3,
                &bars[b]);
  };

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_barrier_init();
    s_tile[0] = atomicAdd(counter, 1);
  }
  __syncthreads();
  int cur = 0;
  uint32_t phase = 0;  // bit b: the parity buffer b waits for next
  int t = s_tile[0];
  if (tid == 0 && t < ntiles) issue(t, 0);
  while (t < ntiles) {
    if (tid == 0) s_tile[cur ^ 1] = atomicAdd(counter, 1);
    __syncthreads();  // next index visible; buffer cur^1 no longer read
    const int tn = s_tile[cur ^ 1];
    if (tid == 0 && tn < ntiles) issue(tn, cur ^ 1);
    if (!mbar_wait(&bars[cur], (phase >> cur) & 1u, fused::kMaxPolls)) {
      if (tid == 0) atomicExch(err, LSMGPU_ERR_TIMEOUT);
      mbar_wait(&bars[cur], (phase >> cur) & 1u, fused::kMaxPolls);
      if (tn < ntiles) mbar_wait(&bars[cur ^ 1], (phase >> (cur ^ 1)) & 1u, fused::kMaxPolls);
      return;
    }
    phase ^= 1u << cur;
    const float *tile = tiles + cur * kPlaneMax * SZ_;
    const TileRef r = tiles_ref[t];
    const GridDesc &G = gd[r.g];
    StageArgs<float> a;
    a.L = G.L;
    a.phi_n = A + G.off;
    a.phi0 = nullptr;
    a.vel[0] = a.vel[1] = a.vel[2] = nullptr;
    a.out = outb + G.off;
    for (int d = 0; d < 3; d++) {
      a.vconst[d] = G.vconst[d];
      a.inv[d] = G.inv[d];
    }
    a.dt = G.dt;
    a.dx_sq = 0.f;
    a.stage = stage;
    a.use0 = 0;
    a.periodic = periodic;
    a.err = err;
    if (G.wide)
      fused::f32_tile<fused::ADV_CONST, TZ_, 32, 8>(tile, a, r.bx * 32, r.by * 8, r.bz * TZ_, tid & 31, tid >> 5);
    else
      fused::f32_tile<fused::ADV_CONST, TZ_, 16, 16>(tile, a, r.bx * 16, r.by * 16, r.bz * TZ_, tid & 15, tid >> 4);
    cur ^= 1;
    t = tn;
  }
}

// copies between the caller's packed LSMLIB arrays (3 ghost cells per side)
// and the padded work regions; blockIdx.y is the grid
__global__ void k_batch_pack(float *work, float *user, const GridDesc *gd, const long long *uoff, int unpack) {
  const GridDesc &G = gd[blockIdx.y];
  const Layout &L = G.L;
  const long long ux = L.nx + 6, uy = L.ny + 6, uz = L.nz + 6;
  const long long n = ux * uy * uz;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % ux) - 3, j = (int)((e / ux) % uy) - 3, k = (int)(e / (ux * uy)) - 3;
    const long long w = G.off + L.idx(i, j, k);
    if (unpack)
      user[uoff[blockIdx.y] + e] = work[w];
    else
      work[w] = user[uoff[blockIdx.y] + e];
  }
}

// autotuner memory: batch shape key -> (TZ, CTAs per SM)
std::mutex g_tune_lock;
std::map<std::tuple<int, long long, long long>, std::pair<int, int>> g_tuned;

struct Batch {
  int n = 0;
  std::vector<GridDesc> desc;
  long long total = 0;
  int ntiles = 0;
};

template <int TZ_>
void launch_batch_stage(const GridDesc *gd, const CUtensorMap *tm, const TileRef *tr, const Batch &b, int stage,
                        float *A, float *B, float *C, int *counter, int *err, int periodic, int blocks,
                        cudaStream_t s) {
  // the shared-memory attribute is set by max_blocks_per_sm() before any launch
  const size_t smem = 2 * (size_t)kPlaneMax * (TZ_ + 6) * sizeof(float);
  k_batch_stage<TZ_><<<blocks, dim3(TX, TY), smem, s>>>(gd, tm, tr, b.ntiles, stage, A, B, C, counter, err,
                                                        periodic);
  note_launch();
}

int max_blocks_per_sm(int tz) {
  int v = 1;
  const size_t smem = 2 * (size_t)kPlaneMax * (tz + 6) * sizeof(float);
  if (tz == 4) {
    cudaFuncSetAttribute(k_batch_stage<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_batch_stage<4>, TX * TY, smem);
  } else if (tz == 8) {
    cudaFuncSetAttribute(k_batch_stage<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_batch_stage<8>, TX * TY, smem);
  } else {
    cudaFuncSetAttribute(k_batch_stage<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_batch_stage<16>, TX * TY, smem);
  }
  return std::max(1, v);
}

}  // namespace batch
}  // namespace lsmgpu

using namespace lsmgpu;
using namespace lsmgpu::batch;

extern "C" int lsmgpu_advect_batch_weno5_tvdrk3_f32(float *phi, const long long *offsets, const int *dims,
                                                   int n_grids, const float *vel, const float *spacing,
                                                   const float *dt, int n_steps, int bc, int flags) {
  const char *name = "lsmgpu_advect_batch_weno5_tvdrk3_f32";
  Call call(name);
  if (!phi || !offsets || !dims || !vel || !spacing || !dt || n_grids <= 0) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument or no grids", name);
    return LSMGPU_ERR_ARGUMENT;
  }
  if (bc != LSMGPU_BC_PERIODIC) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: only periodic boundaries are supported for batches", name);
    return LSMGPU_ERR_ARGUMENT;
  }
  Batch b;
  b.n = n_grids;
  b.desc.resize(n_grids);
  long long user_total = 0;
  std::vector<long long> uoff(n_grids);
  for (int g = 0; g < n_grids; g++) {
    const int nx = dims[3 * g], ny = dims[3 * g + 1], nz = dims[3 * g + 2];
    if (nx < 6 || ny < 6 || nz < 6) {
      set_error(LSMGPU_ERR_BOUNDS, "%s: grid %d is smaller than 6 cells on an axis", name, g);
      return LSMGPU_ERR_BOUNDS;
    }
    // tile positions are 16-bit (16-cell tiles at the finest)
    if (nx > 65535 * 16 || ny > 65535 * 8 || nz > 65535 * 4) {
      set_error(LSMGPU_ERR_BOUNDS, "%s: grid %d has more than 65535 tiles along an axis", name, g);
      return LSMGPU_ERR_BOUNDS;
    }
    uoff[g] = offsets[g];
    user_total = std::max(user_total, offsets[g] + (long long)(nx + 6) * (ny + 6) * (nz + 6));
  }
  const int want_loop = flags & LSMGPU_BATCH_LOOP;
  const int use_graph = !(flags & LSMGPU_BATCH_NO_GRAPH);
  const int forced_tz = (flags >> 8) & 0xff;  // 0 = autotune

  float *user = call.inout(phi, user_total);
  long long *uoff_d = call.temp<long long>(n_grids);
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  cudaStream_t s = stream();

  std::vector<TileRef> tref;
  // force_wide: every grid on 32 x 8 tiles (the single-grid kernel's maps)
  auto build_desc = [&](int tz, bool force_wide = false) {
    long long off = 0;
    int tiles = 0;
    for (int g = 0; g < n_grids; g++) {
      GridDesc &G = b.desc[g];
      G.L = fused::make_layout(dims[3 * g], dims[3 * g + 1], dims[3 * g + 2]);
      G.off = off;
      off += (G.L.elems() + 31) / 32 * 32;
      for (int d = 0; d < 3; d++) {
        G.vconst[d] = vel[3 * g + d];
        G.inv[d] = 1.0f / spacing[3 * g + d];
      }
      G.dt = dt[g];
      // the shape that pads the x rows less (16-wide on a tie is no better)
      G.wide = (force_wide || (G.L.nx + 31) / 32 * 32 <= (G.L.nx + 15) / 16 * 16) ? 1 : 0;
      const int tw = G.wide ? 32 : 16, th = G.wide ? 8 : 16;
      G.ntx = (G.L.nx + tw - 1) / tw;
      G.nty = (G.L.ny + th - 1) / th;
      G.ntz = (G.L.nz + tz - 1) / tz;
      G.tile_base = tiles;
      tiles += G.ntx * G.nty * G.ntz;
    }
    b.total = off;
    b.ntiles = tiles;
    tref.resize((size_t)tiles);
    for (int g = 0; g < n_grids; g++) {
      const GridDesc &G = b.desc[g];
      int t = G.tile_base;
      for (int bz = 0; bz < G.ntz; bz++)
        for (int by = 0; by < G.nty; by++)
          for (int bx = 0; bx < G.ntx; bx++)
            tref[(size_t)t++] = TileRef{g, (unsigned short)bx, (unsigned short)by, (unsigned short)bz, 0};
    }
  };
  build_desc(8);
  // the tile table is sized for the smallest tile depth the autotuner tries
  long long max_tiles = 0;
  for (int g = 0; g < n_grids; g++) {
    const int nx = dims[3 * g], ny = dims[3 * g + 1], nz = dims[3 * g + 2];
    max_tiles += (long long)((nx + 15) / 16) * ((ny + 7) / 8) * ((nz + 3) / 4);
  }
  if (max_tiles > 0x7fffffffLL) {
    set_error(LSMGPU_ERR_CAPACITY, "%s: more than 2^31 tiles", name);
    return LSMGPU_ERR_CAPACITY;
  }
  float *A = call.temp<float>(b.total), *B = call.temp<float>(b.total), *C = call.temp<float>(b.total);
  GridDesc *gd = call.temp<GridDesc>(n_grids);
  TileRef *trd = call.temp<TileRef>(max_tiles);
  CUtensorMap *tm = (CUtensorMap *)call.temp<unsigned char>((long long)sizeof(CUtensorMap) * 3 * n_grids);
  int *counters = call.temp<int>(3 * (long long)std::max(n_steps, 1) + 64);
  int *err = call.temp<int>(1);
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  cudaMemcpyAsync(uoff_d, uoff.data(), sizeof(long long) * n_grids, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(err, 0, sizeof(int), s);
  cudaMemsetAsync(B, 0, sizeof(float) * b.total, s);
  cudaMemsetAsync(C, 0, sizeof(float) * b.total, s);

  std::vector<CUtensorMap> tmh(3 * (size_t)n_grids);
  auto encode_all = [&](int tz) -> bool {
    float *bufs[3] = {A, B, C};
    for (int g = 0; g < n_grids; g++) {
      const Layout &L = b.desc[g].L;
      for (int q = 0; q < 3; q++)
        if (!encode_tmap_3d(&tmh[3 * g + q], bufs[q] + b.desc[g].off, 4, (long long)L.nx + GX + 3,
                            (long long)L.ny + 2 * GY, (long long)L.nz + 2 * GZ, L.py, L.pz,
                            b.desc[g].wide ? kWideSX : kNarrowSX, b.desc[g].wide ? kWideSY : kNarrowSY, tz + 6))
          return false;
    }
    return cudaMemcpyAsync(tm, tmh.data(), sizeof(CUtensorMap) * tmh.size(), cudaMemcpyHostToDevice, s) ==
           cudaSuccess;
  };
  auto upload_desc = [&]() {
    cudaMemcpyAsync(gd, b.desc.data(), sizeof(GridDesc) * n_grids, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(trd, tref.data(), sizeof(TileRef) * tref.size(), cudaMemcpyHostToDevice, s);
  };
  upload_desc();
  {
    dim3 grd(64, n_grids);
    LSMGPU_LAUNCH(k_batch_pack, grd, 256, 0, A, user, gd, uoff_d, 0);
  }

  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);

  auto run_stage = [&](int tz, int stage, int *counter, int blocks) {
    if (tz == 4) launch_batch_stage<4>(gd, tm, trd, b, stage, A, B, C, counter, err, 1, blocks, s);
    else if (tz == 16) launch_batch_stage<16>(gd, tm, trd, b, stage, A, B, C, counter, err, 1, blocks, s);
    else launch_batch_stage<8>(gd, tm, trd, b, stage, A, B, C, counter, err, 1, blocks, s);
  };

  if (want_loop) {
    // comparison mode: one single-grid stage launch per grid per stage
    build_desc(8, true);
    if (!encode_all(8)) { call.fail("tensor map encoding failed"); return LSMGPU_ERR_CUDA; }
    const size_t smem = (size_t)SX * SY * fused::SZ * sizeof(float);
    cudaFuncSetAttribute(fused::k_stage_f32<fused::ADV_CONST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    for (int step = 0; step < n_steps; step++)
      for (int stage = 1; stage <= 3; stage++)
        for (int g = 0; g < n_grids; g++) {
          const GridDesc &G = b.desc[g];
          StageArgs<float> a{};
          a.L = G.L;
          a.phi_n = A + G.off;
          a.out = (stage == 1 ? B : (stage == 2 ? C : A)) + G.off;
          for (int d = 0; d < 3; d++) { a.vconst[d] = G.vconst[d]; a.inv[d] = G.inv[d]; }
          a.dt = G.dt;
          a.stage = stage;
          a.periodic = 1;
          a.err = err;
          dim3 grd(G.ntx, G.nty, G.ntz);
          fused::k_stage_f32<fused::ADV_CONST><<<grd, dim3(TX, TY), smem, s>>>(tmh[3 * g + stage - 1], a);
          note_launch();
        }
  } else {
    // autotune (TZ, CTAs per SM) once per batch shape
    int tz = 8, per_sm = 0;
    const auto key = std::make_tuple(n_grids, b.total, (long long)b.ntiles);
    {
      std::lock_guard<std::mutex> guard(g_tune_lock);
      auto it = g_tuned.find(key);
      if (it != g_tuned.end()) { tz = it->second.first; per_sm = it->second.second; }
    }
    if (forced_tz) { tz = forced_tz; per_sm = 0; }
    if (per_sm == 0 && !forced_tz) {
      float best = 1e30f;
      int bt = 8, bp = 1;
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      for (int cand_tz : {4, 8, 16}) {
        build_desc(cand_tz);
        upload_desc();
        if (!encode_all(cand_tz)) { call.fail("tensor map encoding failed"); return LSMGPU_ERR_CUDA; }
        const int maxb = max_blocks_per_sm(cand_tz);
        for (int p = 1; p <= maxb; p++) {
          // time stage 1 (reads A, writes B: the state is not advanced)
          cudaMemsetAsync(counters, 0, sizeof(int), s);
          run_stage(cand_tz, 1, counters, p * nsm);
          cudaMemsetAsync(counters, 0, sizeof(int), s);
          cudaEventRecord(e0, s);
          run_stage(cand_tz, 1, counters, p * nsm);
          cudaEventRecord(e1, s);
          cudaEventSynchronize(e1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (ms < best) { best = ms; bt = cand_tz; bp = p; }
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      tz = bt;
      per_sm = bp;
      std::lock_guard<std::mutex> guard(g_tune_lock);
      g_tuned[key] = {tz, per_sm};
    }
    {
      const int maxb = max_blocks_per_sm(tz);  // also sets the kernel's shared-memory attribute
      if (per_sm == 0 || per_sm > maxb) per_sm = maxb;
    }
    build_desc(tz);
    upload_desc();
    if (!encode_all(tz)) { call.fail("tensor map encoding failed"); return LSMGPU_ERR_CUDA; }
    const int blocks = per_sm * nsm;
    const long long ncounter = 3LL * n_steps;
    if (use_graph && n_steps > 0) {
      // capture on a private stream, ordered after the library stream
      cudaStream_t cs;
      cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
      cudaEvent_t ev;
      cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      cudaEventRecord(ev, s);
      cudaStreamWaitEvent(cs, ev, 0);
      cudaGraph_t graph;
      cudaGraphExec_t exec;
      cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      cudaMemsetAsync(counters, 0, sizeof(int) * ncounter, cs);
      for (int step = 0; step < n_steps; step++)
        for (int stage = 1; stage <= 3; stage++) {
          int *ctr = counters + 3 * step + stage - 1;
          if (tz == 4) launch_batch_stage<4>(gd, tm, trd, b, stage, A, B, C, ctr, err, 1, blocks, cs);
          else if (tz == 16) launch_batch_stage<16>(gd, tm, trd, b, stage, A, B, C, ctr, err, 1, blocks, cs);
          else launch_batch_stage<8>(gd, tm, trd, b, stage, A, B, C, ctr, err, 1, blocks, cs);
        }
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      if (ce != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaStreamDestroy(cs);
        call.fail("CUDA graph capture failed");
        return LSMGPU_ERR_CUDA;
      }
      cudaGraphLaunch(exec, cs);
      cudaEventRecord(ev, cs);
      cudaStreamWaitEvent(s, ev, 0);
      cudaStreamSynchronize(cs);
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      cudaEventDestroy(ev);
      cudaStreamDestroy(cs);
    } else {
      cudaMemsetAsync(counters, 0, sizeof(int) * ncounter, s);
      for (int step = 0; step < n_steps; step++)
        for (int stage = 1; stage <= 3; stage++) run_stage(tz, stage, counters + 3 * step + stage - 1, blocks);
    }
  }
  {
    dim3 grd(64, n_grids);
    LSMGPU_LAUNCH(k_batch_pack, grd, 256, 0, A, user, gd, uoff_d, 1);
  }
  int herr = 0;
  cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  call.finish();
  cudaStreamSynchronize(s);
  if (herr) {
    set_error(herr, "%s: a bounded device wait gave up (TMA tile load)", name);
    return herr;
  }
  return lsmgpu_get_last_error(nullptr, 0);
}
