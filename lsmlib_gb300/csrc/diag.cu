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

// Arithmetic-rate probes: every thread runs eight independent chains of
// fused multiply-adds (a = a * b + c with |b| < 1, so the values stay
// bounded) for a fixed number of iterations; the grid fills every SM
// several times over.  The result is the device's sustained rate of FP32
// lane operations through packed FFMA2 instructions and of FP64 FMAs.
constexpr int kProbeChains = 8;
constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads) k_probe_ffma2(float *out, int iters, float b, float c) {
  float2 acc[kProbeChains];
#pragma unroll
  for (int q = 0; q < kProbeChains; q++) acc[q] = make_float2(1e-3f * (threadIdx.x + q), 1e-3f * q);
  const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < kProbeChains; q++) acc[q] = __ffma2_rn(acc[q], b2, c2);
  }
  float r = 0.f;
#pragma unroll
  for (int q = 0; q < kProbeChains; q++) r += acc[q].x + acc[q].y;
  if (r == -1.f) out[blockIdx.x] = r;  // never true; keeps the chains live
}

__global__ void __launch_bounds__(kProbeThreads) k_probe_dfma(double *out, int iters, double b, double c) {
  double acc[kProbeChains];
#pragma unroll
  for (int q = 0; q < kProbeChains; q++) acc[q] = 1e-3 * (threadIdx.x + q);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < kProbeChains; q++) acc[q] = fma(acc[q], b, c);
  }
  double r = 0.0;
#pragma unroll
  for (int q = 0; q < kProbeChains; q++) r += acc[q];
  if (r == -1.0) out[blockIdx.x] = r;
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

int lsmgpu_measure_fma_rates(double *fp32_lane_ops_per_s, double *fp64_ops_per_s) {
  Call call("lsmgpu_measure_fma_rates");
  if (!fp32_lane_ops_per_s || !fp64_ops_per_s) {
    set_error(LSMGPU_ERR_ARGUMENT, "lsmgpu_measure_fma_rates: null argument");
    return LSMGPU_ERR_ARGUMENT;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = 8 * (sms > 0 ? sms : 1);
  void *sink = call.temp<double>(blocks);
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  cudaStream_t s = stream();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // best of three timed launches after one warm-up, per precision
  auto timed = [&](bool f64, int iters) {
    float best = 0.f;
    for (int rep = 0; rep < 4; rep++) {
      cudaEventRecord(e0, s);
      if (f64) k_probe_dfma<<<blocks, kProbeThreads, 0, s>>>((double *)sink, iters, 0.5, 1.0);
      else k_probe_ffma2<<<blocks, kProbeThreads, 0, s>>>((float *)sink, iters, 0.5f, 1.0f);
      note_launch();
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    return best;
  };
  const int it32 = 1 << 14, it64 = 1 << 9;
  const float ms32 = timed(false, it32), ms64 = timed(true, it64);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  call.finish();
  if (!cuda_ok(cudaGetLastError(), "lsmgpu_measure_fma_rates")) return lsmgpu_get_last_error(nullptr, 0);
  if (!(ms32 > 0.f) || !(ms64 > 0.f)) {
    set_error(LSMGPU_ERR_CUDA, "lsmgpu_measure_fma_rates: no timing");
    return LSMGPU_ERR_CUDA;
  }
  const double threads = (double)blocks * kProbeThreads;
  *fp32_lane_ops_per_s = threads * kProbeChains * 2.0 * it32 / (ms32 * 1e-3);
  *fp64_ops_per_s = threads * kProbeChains * (double)it64 / (ms64 * 1e-3);
  return LSMGPU_OK;
}

}  // extern "C"
