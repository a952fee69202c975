// Allocation-free variant of the CFL-stable advection time step.
//
// lsm3dcomputestableadvectiondt_ draws its reduction scratch (and, for host
// arrays, staging buffers) from the library's device arena, which grows with
// cudaMalloc.  Some callers cannot let a library allocate: a solver that runs
// inside another framework's memory pool, which owns every byte of device
// memory, and time-step loops that must not stall on the implicit device
// synchronisation cudaMalloc and cudaFree can cause.  This entry point
// computes the same dt with no allocation at all: its scratch is one
// file-scope __device__ array of fixed size, so it needs device-resident
// velocity arrays and handles at most kNoAllocMaxCells cells per call.
//
// Sharing rules: every call on a device uses the same scratch array, and a
// call overwrites what the previous call left there, so two calls that can
// overlap on the GPU (different streams, or different host threads) race on
// it and must be serialised by the caller.
#include <mutex>

#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"

namespace lsmgpu {
namespace noalloc {

typedef double R;

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 32;
constexpr long long kCellsPerBlock = (long long)kThreads * kCellsPerThread;  // 8192
constexpr int kMaxBlocks = 65536;
// 65536 blocks x 8192 cells = 536,870,912 cells (an 812^3 index box)
constexpr long long kNoAllocMaxCells = kCellsPerBlock * kMaxBlocks;

// per-block partial maxima, then one slot for the final dt: 512 KiB + 8 B
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 1];

// device address of g_noalloc_scratch per device, looked up once
static double *g_scratch_addr[64];
static std::mutex g_setup_lock;

static double *scratch_for_current_device(int *err) {
  int dev = 0;
  const cudaError_t ge = cudaGetDevice(&dev);
  if (ge != cudaSuccess || dev < 0 || dev >= 64) {
    if (ge != cudaSuccess) cudaGetLastError();
    set_error(LSMGPU_ERR_CUDA, "lsmgpu_compute_stable_advection_dt_noalloc: %s",
              ge != cudaSuccess ? cudaGetErrorString(ge) : "device index beyond the 64 this entry point tracks");
    *err = LSMGPU_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> guard(g_setup_lock);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(LSMGPU_ERR_CUDA, "lsmgpu_compute_stable_advection_dt_noalloc: cudaGetSymbolAddress: %s",
                cudaGetErrorString(e));
      *err = LSMGPU_ERR_CUDA;
      return nullptr;
    }
    g_scratch_addr[dev] = (double *)p;
  }
  return g_scratch_addr[dev];
}

// pass 1: each block writes the max of |u|/dx + |v|/dy + |w|/dz over its
// kCellsPerBlock cells (math_utils3d.f.in:305-319); a block with no cell
// writes -1, the reference's starting value
__global__ void __launch_bounds__(kThreads) k_partial_max(View<const R> vx, View<const R> vy, View<const R> vz,
                                                          Box ib, long long ncell, R ix, R iy, R iz,
                                                          double *partial) {
  const long long nx = ib.n(0), nxy = ib.n(0) * ib.n(1);
  const long long first = (long long)blockIdx.x * kCellsPerBlock;
  R m = R(-1.0);
  for (int q = 0; q < kCellsPerThread; q++) {
    const long long e = first + (long long)q * kThreads + threadIdx.x;
    if (e >= ncell) break;
    const int k = ib.lo[2] + (int)(e / nxy);
    const long long r = e % nxy;
    const int j = ib.lo[1] + (int)(r / nx);
    const int i = ib.lo[0] + (int)(r % nx);
    const R u = fabs(vx(i, j, k)) * ix + fabs(vy(i, j, k)) * iy + fabs(vz(i, j, k)) * iz;
    if (u > m) m = u;
  }
  for (int o = 16; o > 0; o >>= 1) m = rmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ R warp_max[kThreads / 32];
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    R b = warp_max[0];
    for (int w = 1; w < kThreads / 32; w++) b = rmax(b, warp_max[w]);
    partial[blockIdx.x] = b;
  }
}

// pass 2: one block folds the partials and writes dt = cfl / (max + tiny)
// (math_utils3d.f.in:323) into partial[kMaxBlocks]
__global__ void __launch_bounds__(1024) k_finish(double *partial, int nblocks, R cfl) {
  __shared__ R s[1024];
  R m = R(-1.0);
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) m = rmax(m, partial[b]);
  s[threadIdx.x] = m;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) s[threadIdx.x] = rmax(s[threadIdx.x], s[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[kMaxBlocks] = cfl / (s[0] + Consts<R>::tiny);
}

static cudaMemoryType memory_type(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return cudaMemoryTypeUnregistered;
  }
  return a.type;
}

static bool device_resident(const void *p) {
  const cudaMemoryType t = memory_type(p);
  return t == cudaMemoryTypeDevice || t == cudaMemoryTypeManaged;
}

}  // namespace noalloc
}  // namespace lsmgpu

using namespace lsmgpu;
using namespace lsmgpu::noalloc;

extern "C" int lsmgpu_compute_stable_advection_dt_noalloc(
    double *dt, const double *vel_x, const double *vel_y, const double *vel_z, const int *ilo_vel_gb,
    const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *klo_vel_gb,
    const int *khi_vel_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib,
    const int *klo_ib, const int *khi_ib, const double *dx, const double *dy, const double *dz,
    const double *cfl_number) {
  clear_error();
  const char *name = "lsmgpu_compute_stable_advection_dt_noalloc";
  if (!dt || !vel_x || !vel_y || !vel_z) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null pointer", name);
    return LSMGPU_ERR_ARGUMENT;
  }
  const Box vb = mkbox(ilo_vel_gb, ihi_vel_gb, jlo_vel_gb, jhi_vel_gb, klo_vel_gb, khi_vel_gb);
  const Box ib = mkbox(ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
  const long long ncell = ib.size();
  if (ncell > kNoAllocMaxCells) {
    set_error(LSMGPU_ERR_CAPACITY,
              "%s: index box has %lld cells; this entry point handles at most %lld (its fixed scratch holds "
              "%d block results); use lsm3dcomputestableadvectiondt_ for larger boxes",
              name, ncell, kNoAllocMaxCells, kMaxBlocks);
    return LSMGPU_ERR_CAPACITY;
  }
  if (!vb.contains(ib, 0, 0, 0)) {
    set_error(LSMGPU_ERR_BOUNDS, "%s: velocity ghost box does not cover the index box", name);
    return LSMGPU_ERR_BOUNDS;
  }
  if (!device_resident(vel_x) || !device_resident(vel_y) || !device_resident(vel_z)) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: velocity arrays must be in device memory (nothing is staged)", name);
    return LSMGPU_ERR_ARGUMENT;
  }
  int err = LSMGPU_OK;
  double *scratch = scratch_for_current_device(&err);
  if (!scratch) return err;
  cudaStream_t s = stream();
  const int nblocks = ncell > 0 ? (int)((ncell + kCellsPerBlock - 1) / kCellsPerBlock) : 0;
  if (nblocks > 0) {
    k_partial_max<<<nblocks, kThreads, 0, s>>>(view(vel_x, vb), view(vel_y, vb), view(vel_z, vb), ib, ncell,
                                               1.0 / *dx, 1.0 / *dy, 1.0 / *dz, scratch);
    note_launch();
  }
  // an empty box leaves no partial: the fold starts from -1 as the reference does
  k_finish<<<1, 1024, 0, s>>>(scratch, nblocks, *cfl_number);
  note_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(LSMGPU_ERR_CUDA, "%s: launch: %s", name, cudaGetErrorString(e));
    return LSMGPU_ERR_CUDA;
  }
  e = cudaMemcpyAsync(dt, scratch + kMaxBlocks, sizeof(double), cudaMemcpyDefault, s);
  // only a dt in device memory is left to the stream: host and managed
  // memory are read by host code, so the call waits for the copy
  if (e == cudaSuccess && memory_type(dt) != cudaMemoryTypeDevice) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(LSMGPU_ERR_CUDA, "%s: %s", name, cudaGetErrorString(e));
    return LSMGPU_ERR_CUDA;
  }
  return LSMGPU_OK;
}
