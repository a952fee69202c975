// lsmgpu — GB300-native level-set kernels behind LSMLIB's C interface.
//
// Common device/host helpers: column-major views with arbitrary lower bounds
// (LSMLIB's a(ilo:ihi, jlo:jhi, klo:khi) layout), launch geometry, and the
// per-call staging context that lets every C entry point accept either device
// pointers (used in place, asynchronous on the library stream) or host
// pointers (copied to device, computed, copied back, synchronous — the
// semantics LSMLIB's serial Fortran routines have).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>

#include "../../include/lsmgpu.h"

namespace lsmgpu {

// Dimension of the drop-in call running on this host thread: 3 normally; 2
// or 1 while a 2D / 1D entry point (lifted.cu) runs the 3D routine on its
// arrays, which are then 3D arrays with one cell along the missing axes.  In
// that state every view has stride 0 along those axes (a stencil reaching
// along them reads the centre cell, so its differences are exactly 0) and a
// stencil's reach along them is not required of the ghost boxes.
extern thread_local int g_lift_dims;

// ---------------------------------------------------------------------------
// index spaces
// ---------------------------------------------------------------------------
struct Box {
  int lo[3], hi[3];
  __host__ __device__ long long n(int d) const { return (long long)hi[d] - lo[d] + 1; }
  __host__ __device__ long long size() const {
    long long a = n(0), b = n(1), c = n(2);
    return (a > 0 && b > 0 && c > 0) ? a * b * c : 0;
  }
  __host__ __device__ bool empty() const { return hi[0] < lo[0] || hi[1] < lo[1] || hi[2] < lo[2]; }
  // true when `o` (grown by `g` cells per side along each axis) fits in this box
  __host__ bool contains(const Box &o, int gx, int gy, int gz) const {
    if (o.empty()) return true;
    if (g_lift_dims < 3) gz = 0;
    if (g_lift_dims < 2) gy = 0;
    return o.lo[0] - gx >= lo[0] && o.hi[0] + gx <= hi[0] && o.lo[1] - gy >= lo[1] &&
           o.hi[1] + gy <= hi[1] && o.lo[2] - gz >= lo[2] && o.hi[2] + gz <= hi[2];
  }
};

__host__ __device__ inline bool inbox(const Box &b, int i, int j, int k) {
  return i >= b.lo[0] && i <= b.hi[0] && j >= b.lo[1] && j <= b.hi[1] && k >= b.lo[2] && k <= b.hi[2];
}
inline Box isect(const Box &a, const Box &b) {
  Box r;
  for (int d = 0; d < 3; d++) {
    r.lo[d] = a.lo[d] > b.lo[d] ? a.lo[d] : b.lo[d];
    r.hi[d] = a.hi[d] < b.hi[d] ? a.hi[d] : b.hi[d];
  }
  return r;
}
// the cells c of b for which c - lo_reach .. c + hi_reach (per axis) stay in b
// (no reach is required along the missing axes of a 2D / 1D call)
inline Box inner(const Box &b, int rx0, int rx1, int ry0, int ry1, int rz0, int rz1) {
  if (g_lift_dims < 3) rz0 = rz1 = 0;
  if (g_lift_dims < 2) ry0 = ry1 = 0;
  Box r = b;
  r.lo[0] += rx0; r.hi[0] -= rx1;
  r.lo[1] += ry0; r.hi[1] -= ry1;
  r.lo[2] += rz0; r.hi[2] -= rz1;
  return r;
}
// (empty along a missing axis of a 2D / 1D call: work along it is skipped)
inline Box inner_axis(const Box &b, int axis, int lo_reach, int hi_reach) {
  Box r = b;
  r.lo[axis] += lo_reach;
  r.hi[axis] -= hi_reach;
  return r;
}

inline Box mkbox(const int *ilo, const int *ihi, const int *jlo, const int *jhi,
                 const int *klo, const int *khi) {
  Box b;
  b.lo[0] = *ilo; b.hi[0] = *ihi;
  b.lo[1] = *jlo; b.hi[1] = *jhi;
  b.lo[2] = *klo; b.hi[2] = *khi;
  return b;
}

#ifdef LSMGPU_BOUNDS_CHECK
// Bounds-check build: the device status word of the current device (count of
// out-of-range accesses, then the first one's i, j, k), allocated once.
int *bounds_word();
__device__ __forceinline__ void bounds_fail(int *w, int i, int j, int k) {
  if (!w) return;
  if (atomicAdd(&w[0], 1) == 0) {
    w[1] = i;
    w[2] = j;
    w[3] = k;
  }
}
#endif

// A device view of one column-major array.  In a build with
// LSMGPU_BOUNDS_CHECK defined every access checks the index against the
// array's box (along the axes with a stride: a 2D / 1D call's missing axes
// have none), records an out-of-range one in the status word
// (lsmgpu_bounds_check_read) and uses the array's first element instead.
template <class T>
struct View {
  T *p;
  int lo0, lo1, lo2;
  long long s1, s2;
#ifdef LSMGPU_BOUNDS_CHECK
  int hi0 = 0x7fffffff, hi1 = 0x7fffffff, hi2 = 0x7fffffff;
  int *oob = nullptr;
#endif
  __device__ __forceinline__ long long off(int i, int j, int k) const {
    return (long long)(i - lo0) + s1 * (long long)(j - lo1) + s2 * (long long)(k - lo2);
  }
  __device__ __forceinline__ T &operator()(int i, int j, int k) const {
#ifdef LSMGPU_BOUNDS_CHECK
    if (i < lo0 || i > hi0 || (s1 != 0 && (j < lo1 || j > hi1)) || (s2 != 0 && (k < lo2 || k > hi2))) {
      bounds_fail(oob, i, j, k);
      return p[0];
    }
#endif
    return p[off(i, j, k)];
  }
  __device__ __forceinline__ long long stride(int d) const { return d == 0 ? 1 : (d == 1 ? s1 : s2); }
};

template <class T>
inline View<T> view(T *p, const Box &b) {
  View<T> v;
  v.p = p;
  v.lo0 = b.lo[0]; v.lo1 = b.lo[1]; v.lo2 = b.lo[2];
  v.s1 = g_lift_dims < 2 ? 0 : b.n(0);
  v.s2 = g_lift_dims < 3 ? 0 : b.n(0) * b.n(1);
#ifdef LSMGPU_BOUNDS_CHECK
  v.hi0 = b.hi[0]; v.hi1 = b.hi[1]; v.hi2 = b.hi[2];
  v.oob = bounds_word();
#endif
  return v;
}

// ---------------------------------------------------------------------------
// launch geometry over a fill box: x fastest, one thread per cell
// ---------------------------------------------------------------------------
struct Grid3 {
  dim3 grid, block;
};
inline Grid3 cover(const Box &fb, int bx = 32, int by = 4, int bz = 2) {
  Grid3 g;
  g.block = dim3(bx, by, bz);
  g.grid = dim3((unsigned)((fb.n(0) + bx - 1) / bx), (unsigned)((fb.n(1) + by - 1) / by),
                (unsigned)((fb.n(2) + bz - 1) / bz));
  return g;
}

#define LSMGPU_CELL_INDEX(fb, i, j, k)                 \
  const int i = (fb).lo[0] + blockIdx.x * blockDim.x + threadIdx.x; \
  const int j = (fb).lo[1] + blockIdx.y * blockDim.y + threadIdx.y; \
  const int k = (fb).lo[2] + blockIdx.z * blockDim.z + threadIdx.z; \
  if (i > (fb).hi[0] || j > (fb).hi[1] || k > (fb).hi[2]) return;

// ---------------------------------------------------------------------------
// runtime (runtime.cu)
// ---------------------------------------------------------------------------
cudaStream_t stream();                      // library stream (lsmgpu_set_stream)
cudaStream_t copy_stream(int which);        // library copy streams 0 and 1 (nullptr if unavailable)
void note_launch();                         // counts kernels for lsmgpu_launch_count()

// Replays `body`'s stream work as a CUDA graph on the library stream.  The
// graph is captured (on a library-owned stream, thread-local capture mode)
// the first time a key is seen and kept for later calls with the same key;
// the key must hold every value the captured work depends on (buffers,
// sizes, scalars).  Returns false when capturing or launching fails (nothing
// was queued; the caller then runs `body` directly).
struct GraphKey {
  unsigned char bytes[512];
  size_t n = 0;
  template <class T>
  void add(const T &v) {  // appends v's bytes (T without padding, or zero-initialised)
    static_assert(sizeof(T) <= sizeof(bytes), "key part too large");
    if (n + sizeof(T) > sizeof(bytes)) {
      n = sizeof(bytes) + 1;  // marks the key unusable
      return;
    }
    memcpy(bytes + n, &v, sizeof(T));
    n += sizeof(T);
  }
};
bool graph_replay(const GraphKey &key, void (*body)(void *), void *ctx);
template <class F>
bool graph_replay(const GraphKey &key, F &body) {
  return graph_replay(key, [](void *c) { (*static_cast<F *>(c))(); }, &body);
}
// LSMLIB's scratch side effects requested (lsmgpu_set_exact_side_effects or
// LSMGPU_EXACT_SIDE_EFFECTS=1): the dense derivative routines then also leave
// D1 / D2 / D3 as LSMLIB's do
bool exact_side_effects();
void set_error(int code, const char *fmt, ...);
void clear_error();
bool cuda_ok(cudaError_t e, const char *what);  // records and returns false on error

// Per-call staging context.
class Call {
 public:
  explicit Call(const char *name);
  ~Call();
  // Array arguments.  `n` is the element count of the array's ghost box.
  // in():    read by the kernel
  // inout(): read and written (output arrays keep cells the kernel does not
  //          touch, so a host-resident output is copied both ways)
  // out():   written in full by the kernel (no copy in)
  template <class T> T *in(const T *p, long long n) { return (T *)stage(p, n * (long long)sizeof(T), true, false); }
  template <class T> T *inout(T *p, long long n) { return (T *)stage(p, n * (long long)sizeof(T), true, true); }
  template <class T> T *out(T *p, long long n) { return (T *)stage(p, n * (long long)sizeof(T), false, true); }
  // out_region(): written by the kernel over `region` only (a sub-box of the
  // array's ghost box gb); a host-resident array is neither copied in nor
  // copied back outside `region`, so its other cells keep their values
  template <class T> T *out_region(T *p, const Box &gb, const Box &region) {
    return (T *)stage_region(p, (long long)sizeof(T), gb, region);
  }
  // Device-only temporary memory for this call.
  template <class T> T *temp(long long n) { return (T *)arena_alloc(n * (long long)sizeof(T)); }
  // Scalar output written by a kernel into device memory and copied to *dst
  // (host or device) by finish().
  template <class T> T *scalar_out(T *dst) { return (T *)scalar(dst, sizeof(T)); }
  bool ok() const { return ok_; }
  bool host_staged() const { return host_staged_; }
  // Launch check + copies back + synchronisation when anything was staged.
  void finish();
  void fail(const char *msg);

 private:
  void *stage(const void *p, long long bytes, bool copy_in, bool copy_out);
  void *stage_region(void *p, long long elem, const Box &gb, const Box &region);
  void *scalar(void *dst, size_t bytes);
  void *arena_alloc(long long bytes);
  const char *name_;
  bool ok_ = true, host_staged_ = false, finished_ = false, need_sync_ = false;
  // bytes > 0: one linear copy; region.size() > 0 with bytes == 0: a 3D copy
  // of `region` out of arrays laid out over `gb` with `elem`-byte elements
  struct Back { void *host; void *dev; long long bytes; long long elem; Box gb, region; };
  Back backs_[64];
  int nback_ = 0;
  long long arena_mark_ = 0;
  bool locked_ = false;
};

// Launch `kern` on the library stream and count it.
#define LSMGPU_LAUNCH(kern, grid, block, smem, ...)                       \
  do {                                                                    \
    kern<<<(grid), (block), (smem), ::lsmgpu::stream()>>>(__VA_ARGS__);   \
    ::lsmgpu::note_launch();                                              \
  } while (0)

}  // namespace lsmgpu
