// Host drivers of the fused WENO5 / TVD-RK3 time steppers (advection and
// reinitialization), shared by the FP64 parity unit and the FP32 unit.
//
// A call repacks the caller's array (LSMLIB ghost-box layout) into the padded
// work layout once, runs every stage kernel on the library stream, and
// unpacks the result.  Three work buffers rotate through the stages:
//   stage 1: A -> B,  stage 2: B (+ A at the cell) -> C,
//   stage 3: C (+ A at the cell) -> A   (in place: each cell reads only its
//   own A value, the stencil comes from C).
#pragma once

#include "fused_stage.cuh"
#include "reinit_x2.cuh"
#include "lsmgpu_common.cuh"
#include "../../include/lsmgpu.h"

namespace lsmgpu {
namespace fused {

// copy between the caller's ghost-box array and the padded layout over the
// region the layout holds (interior plus GX/3 ghost cells), clipped to the
// caller's box; cells of the layout outside the caller's box are zeroed
// Copies between a caller's array over its ghost box and the padded work
// layout: threads along x and y, each walking kPackZ planes with all its
// loads issued before its stores (one element in flight per thread leaves
// the copy far below the memory's rate).
constexpr int kPackZ = 8;

// dst2 (optional) receives the same values (the phi0 copy of the
// reinitialization's sign form)
template <class R>
__global__ void k_pack(R *dst, Layout L, View<const R> src, Box gb, int ilo, int jlo, int klo, R *dst2 = nullptr) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - GX;
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y) - GY;
  const int k0 = (int)(blockIdx.z * kPackZ) - GZ;
  if (i > L.nx + 2 || j > L.ny + 2) return;
  const int gi = i + ilo, gj = j + jlo;
  const bool in_xy = gi >= gb.lo[0] && gi <= gb.hi[0] && gj >= gb.lo[1] && gj <= gb.hi[1];
  R v[kPackZ];
#pragma unroll
  for (int q = 0; q < kPackZ; q++) {
    const int gk = k0 + q + klo;
    v[q] = (in_xy && gk >= gb.lo[2] && gk <= gb.hi[2]) ? src(gi, gj, gk) : R(0);
  }
#pragma unroll
  for (int q = 0; q < kPackZ; q++)
    if (k0 + q <= L.nz + 2) {
      const long long c = L.idx(i, j, k0 + q);
      dst[c] = v[q];
      if (dst2) dst2[c] = v[q];
    }
}

template <class R>
__global__ void k_unpack(View<R> dst, Box gb, const R *src, Layout L, int ilo, int jlo, int klo) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 3;
  const int j = (int)(blockIdx.y * blockDim.y + threadIdx.y) - 3;
  const int k0 = (int)(blockIdx.z * kPackZ) - 3;
  if (i > L.nx + 2 || j > L.ny + 2) return;
  const int gi = i + ilo, gj = j + jlo;
  if (!(gi >= gb.lo[0] && gi <= gb.hi[0] && gj >= gb.lo[1] && gj <= gb.hi[1])) return;
  R v[kPackZ];
#pragma unroll
  for (int q = 0; q < kPackZ; q++)
    if (k0 + q <= L.nz + 2) v[q] = src[L.idx(i, j, k0 + q)];
#pragma unroll
  for (int q = 0; q < kPackZ; q++) {
    const int gk = k0 + q + klo;
    if (k0 + q <= L.nz + 2 && gk >= gb.lo[2] && gk <= gb.hi[2]) dst(gi, gj, gk) = v[q];
  }
}

// launch geometry of k_pack / k_unpack over the padded box (x from -GX, y
// and z from -3) or the ghost box (from -3)
inline dim3 pack_block() { return dim3(32, 8, 1); }
inline dim3 pack_grid(int nx, int ny, int nz, int x_ghosts_below) {
  return dim3((unsigned)((nx + x_ghosts_below + 3 + 31) / 32), (unsigned)((ny + 6 + 7) / 8),
              (unsigned)((nz + 6 + kPackZ - 1) / kPackZ));
}

// Extrapolation into the 3 ghost layers along one axis: linear
// (boundary_conditions3d.f:46-169, phi(ghost) = phi(edge) + slope*dist with
// slope = phi(edge) - phi(next inside)), signed linear (:193-337) or copy
// (:352-462, the homogeneous Neumann fill).  Axes run x, y, z in turn over
// the full extent of the other two axes (ghosts included), as the
// reference's six face calls in that order do.
template <class R>
__global__ void k_linear_bc(R *phi, Layout L, int axis, int kind) {
  const int a = (int)(blockIdx.x * blockDim.x + threadIdx.x) - 3;
  const int b = (int)(blockIdx.y * blockDim.y + threadIdx.y) - 3;
  const int n[3] = {L.nx, L.ny, L.nz};
  const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;
  if (a > n[o1] + 2 || b > n[o2] + 2) return;
  int c[3];
  c[o1] = a;
  c[o2] = b;
  const int nn = n[axis];
  // lower face
  c[axis] = 0;
  const R e0 = phi[L.idx(c[0], c[1], c[2])];
  c[axis] = 1;
  const R n0 = phi[L.idx(c[0], c[1], c[2])];
  // upper face
  c[axis] = nn - 1;
  const R e1 = phi[L.idx(c[0], c[1], c[2])];
  c[axis] = nn - 2;
  const R n1 = phi[L.idx(c[0], c[1], c[2])];
  R s0 = e0 - n0, s1 = e1 - n1;
  if (kind == LSMGPU_BC_SIGNED_LINEAR) {
    // boundary_conditions3d.f:203-206: slope = sign(1, phi_edge)*|diff|
    s0 = copysign(R(1.0), e0) * fabs(e0 - n0);
    s1 = copysign(R(1.0), e1) * fabs(e1 - n1);
  }
#pragma unroll
  for (int g = 1; g <= 3; g++) {
    c[axis] = -g;
    phi[L.idx(c[0], c[1], c[2])] = (kind == LSMGPU_BC_COPY) ? e0 : e0 + s0 * R(g);
    c[axis] = nn - 1 + g;
    phi[L.idx(c[0], c[1], c[2])] = (kind == LSMGPU_BC_COPY) ? e1 : e1 + s1 * R(g);
  }
}

// The three passes above leave each ghost cell with a composition of at most
// three one-axis extrapolations of interior values: the x pass is final on
// x-ghost cells of interior (y, z) rows, the y pass (which reads x-ghost
// values at the y edge) on y-ghost cells of interior z planes, the z pass on
// every z-ghost cell.  k_ghost_fill evaluates that composition directly, one
// thread per ghost cell of the 3-layer shell, in one launch; every
// extrapolation is the same arithmetic as k_linear_bc's, so the values are
// identical to the three passes'.

template <class R>
struct GhostShell {
  const R *phi;
  Layout L;
  int kind;
  __device__ R at(int i, int j, int k) const { return phi[L.idx(i, j, k)]; }
  __device__ R X(int i, int j, int k) const {  // j, k interior
    if (i < 0) return extrap(at(0, j, k), at(1, j, k), -i, kind);
    if (i >= L.nx) return extrap(at(L.nx - 1, j, k), at(L.nx - 2, j, k), i - (L.nx - 1), kind);
    return at(i, j, k);
  }
  __device__ R Y(int i, int j, int k) const {  // k interior
    if (j < 0) return extrap(X(i, 0, k), X(i, 1, k), -j, kind);
    if (j >= L.ny) return extrap(X(i, L.ny - 1, k), X(i, L.ny - 2, k), j - (L.ny - 1), kind);
    return X(i, j, k);
  }
  __device__ R Z(int i, int j, int k) const {
    if (k < 0) return extrap(Y(i, j, 0), Y(i, j, 1), -k, kind);
    if (k >= L.nz) return extrap(Y(i, j, L.nz - 1), Y(i, j, L.nz - 2), k - (L.nz - 1), kind);
    return Y(i, j, k);
  }
};

// ghost shell: blockIdx.z picks a face (z below / above over the full x, y
// extent, y below / above over the full x extent and interior z, x below /
// above over interior y, z); a thread takes one line through the face,
// evaluates the edge value and its neighbour once and writes the 3 ghost
// cells of the line.  The values depend only on interior cells, so the
// threads' writes do not interfere.
template <class R>
__global__ void k_ghost_fill(R *phi, Layout L, int kind) {
  const int a = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int b = (int)(blockIdx.y * blockDim.y + threadIdx.y);
  const int face = (int)blockIdx.z, upper = face & 1;
  const GhostShell<R> G{phi, L, kind};
  R e, n;
  if (face < 2) {
    if (a >= L.nx + 6 || b >= L.ny + 6) return;
    const int i = a - 3, j = b - 3, k0 = upper ? L.nz - 1 : 0, k1 = upper ? L.nz - 2 : 1;
    e = G.Y(i, j, k0);
    n = G.Y(i, j, k1);
    for (int g = 1; g <= 3; g++) phi[L.idx(i, j, upper ? k0 + g : -g)] = extrap(e, n, g, kind);
  } else if (face < 4) {
    if (a >= L.nx + 6 || b >= L.nz) return;
    const int i = a - 3, k = b, j0 = upper ? L.ny - 1 : 0, j1 = upper ? L.ny - 2 : 1;
    e = G.X(i, j0, k);
    n = G.X(i, j1, k);
    for (int g = 1; g <= 3; g++) phi[L.idx(i, upper ? j0 + g : -g, k)] = extrap(e, n, g, kind);
  } else {
    if (a >= L.ny || b >= L.nz) return;
    const int j = a, k = b, i0 = upper ? L.nx - 1 : 0, i1 = upper ? L.nx - 2 : 1;
    e = G.at(i0, j, k);
    n = G.at(i1, j, k);
    for (int g = 1; g <= 3; g++) phi[L.idx(upper ? i0 + g : -g, j, k)] = extrap(e, n, g, kind);
  }
}

template <class R>
void launch_bc(R *buf, const Layout &L, int bc) {
  if (bc == LSMGPU_BC_PERIODIC) return;  // written by the stage kernel
  const int wa = (L.nx + 6 > L.ny ? L.nx + 6 : L.ny), wb = (L.ny + 6 > L.nz ? L.ny + 6 : L.nz);
  dim3 blk(32, 8);
  dim3 grd((unsigned)((wa + 31) / 32), (unsigned)((wb + 7) / 8), 6);
  LSMGPU_LAUNCH(k_ghost_fill<R>, grd, blk, 0, buf, L, bc);
}

// The FP32 reinitialization stage runs the window-sharing kernel of
// reinit_x2.cuh (64 x 8 x RZ tiles); every other form runs k_stage /
// k_stage_f32 (32 x 8 x TZ tiles).
template <class R, int MODE, bool EXACT>
constexpr bool uses_reinit_x2() {
  return !EXACT && sizeof(R) == 4 && MODE == REINIT;
}

// Tile depth of the FP32 k_stage_f32 launches of a grid: 8, or 4 where the
// 4-plane tiles fill whole waves of resident CTAs at least 10% better (a
// partly filled last wave costs a whole one; five CTAs per SM at either
// depth; a grid of less than one wave gets twice the CTAs).  At 128^3, 1024
// 8-plane tiles are 1.35 waves on 152 SMs, 2048 4-plane tiles 2.7; at 192^3
// and 256^3 both depths fill their waves equally and 8 is kept.
inline int stage_tz_f32(const Layout &L) {
  static int sms_of[64] = {};  // SM count per device, read once
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    if (sms_of[dev] == 0) {
      int v = 0;
      sms_of[dev] = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 152;
    }
    sms = sms_of[dev];
  } else {
    cudaGetLastError();
  }
  const long long slots = 5LL * sms;
  const long long cols = (long long)((L.nx + TX - 1) / TX) * ((L.ny + TY - 1) / TY);
  auto eff = [&](int tz) {
    const long long tiles = cols * ((L.nz + tz - 1) / tz);
    const long long waves = (tiles + slots - 1) / slots;
    return (double)L.nz / ((double)waves * slots * tz / (double)cols);  // used fraction of the wave slots
  };
  return eff(4) > 1.1 * eff(8) ? 4 : 8;
}

// Tensor map of a padded work buffer with the staged box of the stage kernel
// launch_stage<R, MODE, EXACT> runs.
template <class R, int MODE, bool EXACT>
bool encode_stage_tmap(CUtensorMap *m, const R *p, const Layout &L) {
  const long long ex = (long long)L.nx + GX + 3, ey = (long long)L.ny + 2 * GY, ez = (long long)L.nz + 2 * GZ;
  if constexpr (uses_reinit_x2<R, MODE, EXACT>())
    return encode_tmap_3d(m, p, sizeof(R), ex, ey, ez, L.py, L.pz, RSX, RSY, RZ + 6);
  if constexpr (!EXACT && sizeof(R) == 4)
    return encode_tmap_3d(m, p, sizeof(R), ex, ey, ez, L.py, L.pz, SX, SY, stage_tz_f32(L) + 6);
  return encode_tmap_3d(m, p, sizeof(R), ex, ey, ez, L.py, L.pz, SX, SY, SZ);
}

// Launches one stage kernel; with prepare_only it only sets the kernel's
// dynamic shared memory limit (done once, and before a launch is captured into
// a graph).  The function has internal linkage: each translation unit that
// launches a stage kernel has its own kernel instance, and its own copy of
// this function and of the flag below, so the limit is set on the instance
// the unit launches.  `tm` must come from encode_stage_tmap<R, MODE, EXACT>.
template <class R, int MODE, bool EXACT>
static void launch_stage(const CUtensorMap &tm, const StageArgs<R> &a, bool prepare_only = false) {
  const Layout &L = a.L;
  static bool attr_set = false;
  if constexpr (uses_reinit_x2<R, MODE, EXACT>()) {
    if (!attr_set) {
      cudaFuncSetAttribute(k_reinit_x2<RZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)reinit_x2_smem(RZ));
      attr_set = true;
    }
    if (prepare_only) return;
    dim3 grd((unsigned)((L.nx + RX - 1) / RX), (unsigned)((L.ny + RY - 1) / RY), (unsigned)((L.nz + RZ - 1) / RZ));
    k_reinit_x2<RZ><<<grd, dim3(32, RY), reinit_x2_smem(RZ), stream()>>>(tm, a);
    note_launch();
    return;
  }
  dim3 blk(TX, TY);
  if (!attr_set) {
    if constexpr (!EXACT && sizeof(R) == 4) {
      cudaFuncSetAttribute(k_stage_f32<MODE, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((size_t)SX * SY * 14 * sizeof(float)));
      cudaFuncSetAttribute(k_stage_f32<MODE, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((size_t)SX * SY * 10 * sizeof(float)));
    } else {
      cudaFuncSetAttribute(k_stage<R, MODE, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((size_t)SX * SY * SZ * sizeof(R)));
    }
    attr_set = true;
  }
  if (prepare_only) return;
  if constexpr (!EXACT && sizeof(R) == 4) {
    // FP32 form: the packed cell-pair kernel, tile depth per grid
    const int tz = stage_tz_f32(L);
    dim3 grd((unsigned)((L.nx + TX - 1) / TX), (unsigned)((L.ny + TY - 1) / TY), (unsigned)((L.nz + tz - 1) / tz));
    const size_t smem = (size_t)SX * SY * (tz + 6) * sizeof(float);
    if (tz == 4) k_stage_f32<MODE, 4><<<grd, blk, smem, stream()>>>(tm, a);
    else k_stage_f32<MODE, 8><<<grd, blk, smem, stream()>>>(tm, a);
  } else {
    dim3 grd((unsigned)((L.nx + TX - 1) / TX), (unsigned)((L.ny + TY - 1) / TY), (unsigned)((L.nz + TZ - 1) / TZ));
    k_stage<R, MODE, EXACT><<<grd, blk, (size_t)SX * SY * SZ * sizeof(R), stream()>>>(tm, a);
  }
  note_launch();
}

// The graph cache key of a stage-argument set, field by field (the structs
// have padding, whose bytes are unspecified and must not enter the key).
template <class R>
void add_stage_args(GraphKey &key, const StageArgs<R> &a) {
  key.add(a.L.nx); key.add(a.L.ny); key.add(a.L.nz); key.add(a.L.py); key.add(a.L.pz);
  key.add(a.phi_n); key.add(a.phi0);
  for (int d = 0; d < 3; d++) key.add(a.vel[d]);
  key.add(a.out);
  for (int d = 0; d < 3; d++) { key.add(a.vconst[d]); key.add(a.inv[d]); }
  key.add(a.dt); key.add(a.dx_sq);
  key.add(a.stage); key.add(a.use0); key.add(a.periodic); key.add(a.ghost);
  key.add(a.err);
}

struct RunSpec {
  int mode;          // ADV_CONST / ADV_FIELD / REINIT
  int n_steps;
  int bc;            // LSMGPU_BC_*
  int use0;
  double dt, dx, dy, dz;
  double vconst[3];
};

// Runs n_steps full TVD-RK3 steps on the caller's phi (device or host).
template <class R, bool EXACT>
int run(const char *name, R *phi_user, const Box &gb, const Box &fb, const R *vx, const R *vy, const R *vz,
        const Box &vb, const RunSpec &rs) {
  Call call(name);
  if (!gb.contains(fb, 3, 3, 3)) call.fail("ghost box must hold 3 ghost cells around the fill box");
  const int nx = (int)fb.n(0), ny = (int)fb.n(1), nz = (int)fb.n(2);
  if (fb.empty() || nx < 6 || ny < 6 || nz < 6) call.fail("fill box must be at least 6 cells per axis");
  if (rs.mode == ADV_FIELD && !vb.contains(fb, 0, 0, 0)) call.fail("velocity ghost box does not cover the fill box");
  if (rs.bc < LSMGPU_BC_PERIODIC || rs.bc > LSMGPU_BC_COPY) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: unknown boundary condition %d", name, rs.bc);
    return LSMGPU_ERR_ARGUMENT;
  }
  if (!call.ok()) return LSMGPU_ERR_BOUNDS;
  if (rs.n_steps <= 0) return LSMGPU_OK;

  R *phi_d = call.inout(phi_user, gb.size());
  const R *vel_d[3] = {nullptr, nullptr, nullptr};
  if (rs.mode == ADV_FIELD) {
    vel_d[0] = call.in(vx, vb.size());
    vel_d[1] = call.in(vy, vb.size());
    vel_d[2] = call.in(vz, vb.size());
  }
  Layout L = make_layout(nx, ny, nz);
  const long long ne = L.elems();
  R *A = call.temp<R>(ne), *B = call.temp<R>(ne), *C = call.temp<R>(ne);
  R *P0 = (rs.mode == REINIT && rs.use0) ? call.temp<R>(ne) : nullptr;
  R *V[3] = {nullptr, nullptr, nullptr};
  if (rs.mode == ADV_FIELD)
    for (int d = 0; d < 3; d++) V[d] = call.temp<R>(ne);
  int *err = call.temp<int>(1);
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);

  // B and C need no initial values: a stage writes every interior cell of
  // its output, and the ghost cells the next stage reads are either written
  // by the stage (periodic images) or computed by the next stage's loader
  cudaStream_t s = stream();
  cudaMemsetAsync(err, 0, sizeof(int), s);
  {
    const dim3 blk = pack_block(), grd = pack_grid(nx, ny, nz, GX);
    // the phi0 copy of the sign form (read at interior cells only) is
    // written by the same pass
    LSMGPU_LAUNCH(k_pack<R>, grd, blk, 0, A, L, view((const R *)phi_d, gb), gb, fb.lo[0], fb.lo[1], fb.lo[2], P0);
    if (rs.mode == ADV_FIELD)
      for (int d = 0; d < 3; d++)
        LSMGPU_LAUNCH(k_pack<R>, grd, blk, 0, V[d], L, view(vel_d[d], vb), vb, fb.lo[0], fb.lo[1], fb.lo[2]);
  }

  CUtensorMap tA, tB, tC;
  auto enc = [&](CUtensorMap *m, const R *p) {
    if (rs.mode == REINIT) return encode_stage_tmap<R, REINIT, EXACT>(m, p, L);
    if (rs.mode == ADV_CONST) return encode_stage_tmap<R, ADV_CONST, EXACT>(m, p, L);
    return encode_stage_tmap<R, ADV_FIELD, EXACT>(m, p, L);
  };
  if (!enc(&tA, A) || !enc(&tB, B) || !enc(&tC, C)) {
    call.fail("tensor map encoding failed");
    return LSMGPU_ERR_CUDA;
  }

  StageArgs<R> a{};
  a.L = L;
  a.phi0 = P0;
  for (int d = 0; d < 3; d++) a.vel[d] = V[d];
  a.vconst[0] = (R)rs.vconst[0]; a.vconst[1] = (R)rs.vconst[1]; a.vconst[2] = (R)rs.vconst[2];
  a.inv[0] = R(1.0) / (R)rs.dx; a.inv[1] = R(1.0) / (R)rs.dy; a.inv[2] = R(1.0) / (R)rs.dz;
  a.dt = (R)rs.dt;
  {
    R m = rmax(rmax((R)rs.dx, (R)rs.dy), (R)rs.dz);
    a.dx_sq = m * m;
  }
  a.use0 = rs.use0;
  a.periodic = rs.bc == LSMGPU_BC_PERIODIC;
  a.err = err;

  if (rs.mode == REINIT) launch_stage<R, REINIT, EXACT>(tA, a, true);
  else if (rs.mode == ADV_CONST) launch_stage<R, ADV_CONST, EXACT>(tA, a, true);
  else launch_stage<R, ADV_FIELD, EXACT>(tA, a, true);
  // The n_steps x 3 stage launches, replayed as one CUDA graph when the same
  // buffers, sizes and parameters come again.  With an extrapolation
  // boundary condition LSMLIB's drivers fill the ghost cells after every
  // stage; here each stage computes the face ghosts it reads from its input's
  // interior cells while staging its tile (the same values), except the very
  // first stage, which reads the caller's ghost cells as given, and one fill
  // of the stored result follows the last stage.
  const int ghost = a.periodic ? 0 : rs.bc;
  auto steps = [&]() {
    StageArgs<R> b = a;
    for (int step = 0; step < rs.n_steps; step++) {
      b.stage = 1; b.phi_n = A; b.out = B;
      b.ghost = step == 0 ? 0 : ghost;
      if (rs.mode == REINIT) launch_stage<R, REINIT, EXACT>(tA, b);
      else if (rs.mode == ADV_CONST) launch_stage<R, ADV_CONST, EXACT>(tA, b);
      else launch_stage<R, ADV_FIELD, EXACT>(tA, b);
      b.stage = 2; b.out = C;
      b.ghost = ghost;
      if (rs.mode == REINIT) launch_stage<R, REINIT, EXACT>(tB, b);
      else if (rs.mode == ADV_CONST) launch_stage<R, ADV_CONST, EXACT>(tB, b);
      else launch_stage<R, ADV_FIELD, EXACT>(tB, b);
      b.stage = 3; b.out = A;
      if (rs.mode == REINIT) launch_stage<R, REINIT, EXACT>(tC, b);
      else if (rs.mode == ADV_CONST) launch_stage<R, ADV_CONST, EXACT>(tC, b);
      else launch_stage<R, ADV_FIELD, EXACT>(tC, b);
    }
    launch_bc(A, L, rs.bc);
  };
  GraphKey key;
  key.add((int)sizeof(R));
  key.add((int)EXACT);
  key.add(rs.mode);
  key.add(rs.n_steps);
  key.add(rs.bc);
  key.add(A);
  key.add(B);
  key.add(C);
  add_stage_args(key, a);
  if (!graph_replay(key, steps)) steps();
  {
    const dim3 blk = pack_block(), grd = pack_grid(nx, ny, nz, 3);
    LSMGPU_LAUNCH(k_unpack<R>, grd, blk, 0, view(phi_d, gb), gb, A, L, fb.lo[0], fb.lo[1], fb.lo[2]);
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

}  // namespace fused
}  // namespace lsmgpu
