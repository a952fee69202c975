// Fused second-order mean curvature: the LSMLIB sequence
//   lsm3dCentralGradOrder2 -> lsm3dGradientMagnitude -> lsm3dComputeMeanCurvatureOrder2
// (spatial_derivatives3d.f.in:3016-3077, :3586-3659; curvature3d.f.in:15-128)
// in one kernel: each cell reads its 19-point neighbourhood once and writes
// kappa (and, optionally, the gradient magnitude).  Included by the FP64
// parity unit and the FP32 unit.
#pragma once

#include "lsmgpu_common.cuh"
#include "stencil_math.cuh"

namespace lsmgpu {
namespace curv {

template <class R>
struct CurvArgs {
  View<const R> phi;
  View<R> kappa;
  View<R> mag;      // p == nullptr: not written
  Box fb;
  R gx, gy, gz;     // 0.5/dx ...
  R fxx, fyy, fzz, fxy, fxz, fyz;
};

template <class R>
__global__ void k_mean_curvature(CurvArgs<R> a) {
  LSMGPU_CELL_INDEX(a.fb, i, j, k);
  const R *c = a.phi.p + a.phi.off(i, j, k);
  const long long sx = 1, sy = a.phi.s1, sz = a.phi.s2;
  // central gradient
  const R px = (c[sx] - c[-sx]) * a.gx;
  const R py = (c[sy] - c[-sy]) * a.gy;
  const R pz = (c[sz] - c[-sz]) * a.gz;
  // gradient magnitude with the reference's 1e-8 clamps
  const R tol = R(1.e-8);
  R x2 = px * px, y2 = py * py, z2 = pz * pz;
  if (x2 < tol) x2 = R(0);
  if (y2 < tol) y2 = R(0);
  if (z2 < tol) z2 = R(0);
  const R t = sqrt(x2 + y2 + z2);
  const R g = (t < tol) ? R(0) : t;
  if (a.mag.p) a.mag(i, j, k) = g;
  // second derivatives and curvature
  const R xx = (c[sx] - R(2.0) * c[0] + c[-sx]) * a.fxx;
  const R yy = (c[sy] - R(2.0) * c[0] + c[-sy]) * a.fyy;
  const R zz = (c[sz] - R(2.0) * c[0] + c[-sz]) * a.fzz;
  const R xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * a.fxy;
  const R xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * a.fxz;
  const R yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * a.fyz;
  const R den = g * g * g;
  R out;
  if (den < R(Consts<double>::zero_tol))
    out = R(0);
  else
    out = curv_numerator(xx, yy, zz, xy, xz, yz, px, py, pz) / den;
  a.kappa(i, j, k) = out;
}

inline bool pinned_host(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// Pinned host phi and kappa: the transfers overlap the kernel and each other.
// The fill box is cut into z slabs; phi's planes go to the device on copy
// stream 0 in order (each plane once: phi's planes are contiguous in its
// column-major layout), the kernel of a slab runs on the library stream once
// its planes and their one-plane halo are there, and the slab's kappa goes
// back on copy stream 1.  Returns false (nothing queued) when the streams or
// events are not available, so the caller stages the arrays whole instead.
template <class R>
bool run_pipelined(Call &call, CurvArgs<R> a, R *kappa, const Box &kb, const R *phi, const Box &pb,
                   const Box &fb) {
  constexpr int kSlabs = 8;
  cudaStream_t s = stream(), cin = copy_stream(0), cout = copy_stream(1);
  if (!cin || !cout || fb.n(2) < 2 * kSlabs) return false;
  R *phid = call.temp<R>(pb.size());
  R *kapd = call.temp<R>(kb.size());
  if (!call.ok()) return false;
  cudaEvent_t ev[2 * kSlabs + 2];
  int made = 0;
  for (; made < 2 * kSlabs + 2; made++)
    if (cudaEventCreateWithFlags(&ev[made], cudaEventDisableTiming) != cudaSuccess) break;
  bool ok = made == 2 * kSlabs + 2;
  if (ok) {
    // the copy streams start after the work already queued on the library stream
    ok = cuda_ok(cudaEventRecord(ev[2 * kSlabs], s), "cudaEventRecord") &&
         cuda_ok(cudaStreamWaitEvent(cin, ev[2 * kSlabs], 0), "cudaStreamWaitEvent") &&
         cuda_ok(cudaStreamWaitEvent(cout, ev[2 * kSlabs], 0), "cudaStreamWaitEvent");
  }
  a.phi = view((const R *)phid, pb);
  a.kappa = view(kapd, kb);
  const long long plane = pb.n(0) * pb.n(1);
  const long long nz = fb.n(2);
  int copied = pb.lo[2] - 1;  // last phi plane on the device
  for (int q = 0; q < kSlabs && ok; q++) {
    Box sb = fb;
    sb.lo[2] = fb.lo[2] + (int)(nz * q / kSlabs);
    sb.hi[2] = fb.lo[2] + (int)(nz * (q + 1) / kSlabs) - 1;
    const int need = sb.hi[2] + 1 < pb.hi[2] ? sb.hi[2] + 1 : pb.hi[2];
    if (need > copied) {
      const long long z0 = copied + 1 - pb.lo[2], n = (long long)(need - copied) * plane;
      ok = cuda_ok(cudaMemcpyAsync(phid + z0 * plane, phi + z0 * plane, (size_t)n * sizeof(R), cudaMemcpyHostToDevice,
                                   cin), "cudaMemcpyAsync(H2D slab)");
      copied = need;
    }
    ok = ok && cuda_ok(cudaEventRecord(ev[q], cin), "cudaEventRecord") &&
         cuda_ok(cudaStreamWaitEvent(s, ev[q], 0), "cudaStreamWaitEvent");
    if (!ok) break;
    a.fb = sb;
    Grid3 g = cover(sb);
    LSMGPU_LAUNCH(k_mean_curvature<R>, g.grid, g.block, 0, a);
    ok = cuda_ok(cudaEventRecord(ev[kSlabs + q], s), "cudaEventRecord") &&
         cuda_ok(cudaStreamWaitEvent(cout, ev[kSlabs + q], 0), "cudaStreamWaitEvent");
    if (!ok) break;
    // the slab's kappa rows: one 3D copy out of kappa's ghost-box layout
    cudaMemcpy3DParms m = {};
    const size_t pitch = (size_t)kb.n(0) * sizeof(R);
    m.srcPtr = make_cudaPitchedPtr(kapd, pitch, pitch, (size_t)kb.n(1));
    m.dstPtr = make_cudaPitchedPtr(kappa, pitch, pitch, (size_t)kb.n(1));
    m.srcPos = m.dstPos = make_cudaPos((size_t)(sb.lo[0] - kb.lo[0]) * sizeof(R), (size_t)(sb.lo[1] - kb.lo[1]),
                                       (size_t)(sb.lo[2] - kb.lo[2]));
    m.extent = make_cudaExtent((size_t)sb.n(0) * sizeof(R), (size_t)sb.n(1), (size_t)sb.n(2));
    m.kind = cudaMemcpyDeviceToHost;
    ok = cuda_ok(cudaMemcpy3DAsync(&m, cout), "cudaMemcpy3DAsync(D2H slab)");
  }
  // the library stream (and so the caller) waits for every copy; the call
  // returns once they are done, as a staged call does
  const bool joined = made == 2 * kSlabs + 2 && cuda_ok(cudaEventRecord(ev[2 * kSlabs + 1], cout), "cudaEventRecord") &&
                      cuda_ok(cudaStreamWaitEvent(s, ev[2 * kSlabs + 1], 0), "cudaStreamWaitEvent") &&
                      cuda_ok(cudaEventRecord(ev[2 * kSlabs], cin), "cudaEventRecord") &&
                      cuda_ok(cudaStreamWaitEvent(s, ev[2 * kSlabs], 0), "cudaStreamWaitEvent");
  const bool synced = cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  for (int e = 0; e < made; e++) cudaEventDestroy(ev[e]);
  if (!(ok && joined && synced)) call.fail("pipelined transfer failed");
  return true;
}

template <class R>
int run(const char *name, R *kappa, const Box &kb, const R *phi, const Box &pb, R *mag, const Box &fb,
        R dx, R dy, R dz) {
  Call call(name);
  if (!pb.contains(fb, 1, 1, 1)) call.fail("phi ghost box must hold 1 ghost cell around the fill box");
  if (!kb.contains(fb, 0, 0, 0)) call.fail("kappa ghost box does not cover the fill box");
  if (!call.ok()) return LSMGPU_ERR_BOUNDS;
  if (fb.empty()) return LSMGPU_OK;
  if (!phi || !kappa) {
    call.fail("null array pointer");
    return LSMGPU_ERR_ARGUMENT;
  }
  CurvArgs<R> a{};
  a.gx = R(0.5) / dx; a.gy = R(0.5) / dy; a.gz = R(0.5) / dz;
  a.fxx = R(1.0) / dx / dx; a.fyy = R(1.0) / dy / dy; a.fzz = R(1.0) / dz / dz;
  a.fxy = R(0.25) / dx / dy; a.fxz = R(0.25) / dx / dz; a.fyz = R(0.25) / dy / dz;
  if (!mag && pinned_host(phi) && pinned_host(kappa) && run_pipelined<R>(call, a, kappa, kb, phi, pb, fb)) {
    call.finish();
    return lsmgpu_get_last_error(nullptr, 0);
  }
  a.phi = view((const R *)call.in(phi, pb.size()), pb);
  // kappa and |grad phi| are written on every fill-box cell and nowhere else
  a.kappa = view(call.out_region(kappa, kb, fb), kb);
  a.mag = mag ? view(call.out_region(mag, kb, fb), kb) : View<R>{};
  if (!call.ok()) return lsmgpu_get_last_error(nullptr, 0);
  a.fb = fb;
  Grid3 g = cover(fb);
  LSMGPU_LAUNCH(k_mean_curvature<R>, g.grid, g.block, 0, a);
  call.finish();
  return lsmgpu_get_last_error(nullptr, 0);
}

}  // namespace curv
}  // namespace lsmgpu
