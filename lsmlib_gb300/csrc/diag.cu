// Diagnostics: a device scan for non-finite values (the GPU form of LSMLIB's
// EXAMINE_ARRAY, lsm_macros.h, which prints NaN / inf positions) and a
// self-test of the bounded device waits every TMA-staged kernel uses.
//
// The self-test makes one CTA wait on an mbarrier that nothing ever arrives
// on, with a small poll budget: the wait gives up, the kernel records
// LSMGPU_ERR_TIMEOUT in a status word and returns, and the host reads the
// status.  No copy is in flight and no thread spins without a limit, so the
// context stays usable; it is how the timeout path of the stage kernels is
// exercised without a fault.
#include "lsmgpu_common.cuh"
#include "tma.cuh"

namespace lsmgpu {
namespace {

constexpr unsigned kSelftestMaxPolls = 1u << 20;

__global__ void k_wait_for_nothing(unsigned polls, int *status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival expected; none is ever made
    fence_barrier_init();
  }
  __syncthreads();
  if (!mbar_wait(&bar, 0, polls) && threadIdx.x == 0) atomicExch(status, LSMGPU_ERR_TIMEOUT);
}

// non-finite: exponent bits all ones (NaN or +-inf)
__device__ __forceinline__ bool nonfinite(double v) {
  return (__double_as_longlong(v) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool nonfinite(float v) { return (__float_as_int(v) & 0x7f800000) == 0x7f800000; }

template <class T>
__global__ void k_nonfinite(View<const T> f, Box b, unsigned long long *count, unsigned long long *first) {
  LSMGPU_CELL_INDEX(b, i, j, k);
  if (!nonfinite(f(i, j, k))) return;
  atomicAdd(count, 1ULL);
  // position in the box's memory order, so the smallest is the first a
  // serial (k, j, i) sweep meets, whatever the launch order
  const unsigned long long pos = (unsigned long long)(i - b.lo[0]) +
                                 (unsigned long long)b.n(0) *
                                     ((unsigned long long)(j - b.lo[1]) + (unsigned long long)b.n(1) * (k - b.lo[2]));
  atomicMin(first, pos);
}

__global__ void k_init_scan(unsigned long long *count, unsigned long long *first) {
  *count = 0;
  *first = ~0ULL;
}

template <class T>
int count_nonfinite(const char *name, const T *field, const int *gb, const int *box, long long *count,
                    int *first) {
  Call call(name);
  if (!field || !gb || !box || !count) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", name);
    return LSMGPU_ERR_ARGUMENT;
  }
  const Box g = mkbox(gb, gb + 1, gb + 2, gb + 3, gb + 4, gb + 5);
  const Box b = mkbox(box, box + 1, box + 2, box + 3, box + 4, box + 5);
  if (!g.contains(b, 0, 0, 0)) call.fail("ghost box does not cover the scanned box");
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  View<const T> f = view((const T *)call.in(field, g.size()), g);
  unsigned long long *cnt = call.temp<unsigned long long>(1), *pos = call.temp<unsigned long long>(1);
  unsigned long long h[2] = {0, ~0ULL};
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  LSMGPU_LAUNCH(k_init_scan, 1, 1, 0, cnt, pos);
  if (!b.empty()) {
    Grid3 g3 = cover(b);
    LSMGPU_LAUNCH(k_nonfinite<T>, g3.grid, g3.block, 0, f, b, cnt, pos);
  }
  cuda_ok(cudaMemcpyAsync(&h[0], cnt, sizeof(h[0]), cudaMemcpyDeviceToHost, stream()), name);
  cuda_ok(cudaMemcpyAsync(&h[1], pos, sizeof(h[1]), cudaMemcpyDeviceToHost, stream()), name);
  call.finish();
  if (!cuda_ok(cudaStreamSynchronize(stream()), name)) return lsmgpu_get_last_error(nullptr, 0);
  *count = (long long)h[0];
  if (first) {
    if (h[0] == 0) {
      first[0] = b.lo[0] - 1;
      first[1] = b.lo[1] - 1;
      first[2] = b.lo[2] - 1;
    } else {
      const unsigned long long nx = (unsigned long long)b.n(0), ny = (unsigned long long)b.n(1);
      first[0] = b.lo[0] + (int)(h[1] % nx);
      first[1] = b.lo[1] + (int)((h[1] / nx) % ny);
      first[2] = b.lo[2] + (int)(h[1] / (nx * ny));
    }
  }
  return lsmgpu_get_last_error(nullptr, 0);
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

int lsmgpu_count_nonfinite_f64(const double *field, const int *gb, const int *box, long long *count, int *first) {
  return count_nonfinite("lsmgpu_count_nonfinite_f64", field, gb, box, count, first);
}

int lsmgpu_count_nonfinite_f32(const float *field, const int *gb, const int *box, long long *count, int *first) {
  return count_nonfinite("lsmgpu_count_nonfinite_f32", field, gb, box, count, first);
}

int lsmgpu_selftest_bounded_wait(unsigned int polls) {
  Call call("lsmgpu_selftest_bounded_wait");
  if (polls > kSelftestMaxPolls) {
    set_error(LSMGPU_ERR_CAPACITY, "lsmgpu_selftest_bounded_wait: at most %u polls", kSelftestMaxPolls);
    return LSMGPU_ERR_CAPACITY;
  }
  int *status = call.temp<int>(1);
  int h = 0;
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  cudaMemsetAsync(status, 0, sizeof(int), stream());
  LSMGPU_LAUNCH(k_wait_for_nothing, 1, 32, 0, polls, status);
  cuda_ok(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, stream()), "selftest");
  call.finish();
  if (!cuda_ok(cudaStreamSynchronize(stream()), "selftest")) return lsmgpu_get_last_error(nullptr, 0);
  if (h != 0) {
    set_error(h, "lsmgpu_selftest_bounded_wait: the device wait gave up after %u polls (as intended)", polls);
    return h;
  }
  return LSMGPU_OK;
}

}  // extern "C"
