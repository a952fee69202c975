// Runtime services for the C entry points: status side channel, library
// stream, launch counting, a grow-only device arena for staged host arrays and
// temporaries, and the per-call staging context.
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "lsmgpu_common.cuh"

namespace lsmgpu {

thread_local int g_lift_dims = 3;

namespace {

thread_local int g_err = LSMGPU_OK;
thread_local char g_msg[512] = "";
std::atomic<cudaStream_t> g_stream{nullptr};
std::atomic<long long> g_launches{0};
std::atomic<long long> g_captures{0};     // graphs captured (cache misses)
std::atomic<long long> g_arena_bytes{0};  // device bytes the arena holds

// Device arena: a list of chunks per device, bump-allocated, reset at the
// start of each call.  All users run in the library stream's order, so memory
// handed out by one call may be reused by the next.
struct Chunk { char *p; long long cap; };
struct Arena {
  std::vector<Chunk> chunks;
  int cur = 0;
  long long used = 0;
};
std::mutex g_lock;
Arena g_arena[64];

}  // namespace

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

#ifdef LSMGPU_BOUNDS_CHECK
namespace {
int *g_oob_word[64] = {};
std::mutex g_oob_lock;
}  // namespace
int *bounds_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> guard(g_oob_lock);
  if (!g_oob_word[dev]) {
    void *p = nullptr;
    if (cudaMalloc(&p, 4 * sizeof(int)) != cudaSuccess || cudaMemset(p, 0, 4 * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    g_oob_word[dev] = (int *)p;
  }
  return g_oob_word[dev];
}
#endif

// exact side-effect mode: -1 until first asked, then the environment's
// LSMGPU_EXACT_SIDE_EFFECTS (unset or "0": off) unless set through the API
std::atomic<int> g_side_effects{-1};
bool exact_side_effects() {
  int v = g_side_effects.load();
  if (v < 0) {
    const char *e = getenv("LSMGPU_EXACT_SIDE_EFFECTS");
    v = (e && e[0] && !(e[0] == '0' && e[1] == 0)) ? 1 : 0;
    int expect = -1;
    g_side_effects.compare_exchange_strong(expect, v);
    v = g_side_effects.load();
  }
  return v == 1;
}

namespace {
thread_local cudaStream_t t_capture_stream = nullptr;  // set while a graph is captured

// cached executable graphs: key, graph, kernels per replay; per device
struct GraphEntry {
  int dev;
  GraphKey key;
  cudaGraphExec_t exec;
  long long kernels;
};
std::vector<GraphEntry> g_graphs;
constexpr size_t kMaxGraphs = 16;
cudaStream_t g_capture[64] = {};
}  // namespace

cudaStream_t stream() { return t_capture_stream ? t_capture_stream : g_stream.load(); }

// Two library-owned streams per device for host transfers that overlap the
// library stream's work (created on first use; used inside a Call, with the
// library lock held).
cudaStream_t copy_stream(int which) {
  static cudaStream_t streams[64][2] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || which < 0 || which > 1) {
    cudaGetLastError();
    return nullptr;
  }
  if (!streams[dev][which] && cudaStreamCreateWithFlags(&streams[dev][which], cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    streams[dev][which] = nullptr;
  }
  return streams[dev][which];
}

// Called with the library lock held (inside a Call), so the cache and the
// capture stream are not shared with another thread meanwhile.
bool graph_replay(const GraphKey &key, void (*body)(void *), void *ctx) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || key.n > sizeof(key.bytes)) {
    cudaGetLastError();
    return false;
  }
  for (size_t q = 0; q < g_graphs.size(); q++) {
    GraphEntry &e = g_graphs[q];
    if (e.dev == dev && e.key.n == key.n && memcmp(e.key.bytes, key.bytes, key.n) == 0) {
      if (cudaGraphLaunch(e.exec, g_stream.load()) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      g_launches.fetch_add(e.kernels, std::memory_order_relaxed);
      return true;
    }
  }
  if (!g_capture[dev] && cudaStreamCreateWithFlags(&g_capture[dev], cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    g_capture[dev] = nullptr;
    return false;
  }
  if (cudaStreamBeginCapture(g_capture[dev], cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const long long before = g_launches.load();
  g_captures.fetch_add(1, std::memory_order_relaxed);
  t_capture_stream = g_capture[dev];
  body(ctx);
  t_capture_stream = nullptr;
  const long long kernels = g_launches.load() - before;
  g_launches.fetch_sub(kernels, std::memory_order_relaxed);  // counted when replayed
  cudaGraph_t graph = nullptr;
  if (cudaStreamEndCapture(g_capture[dev], &graph) != cudaSuccess || !graph) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    return false;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (g_graphs.size() >= kMaxGraphs) {
    // the oldest entry goes; work it queued earlier keeps running (a graph
    // exec destroyed while launched completes its launches)
    cudaGraphExecDestroy(g_graphs.front().exec);
    g_graphs.erase(g_graphs.begin());
  }
  g_graphs.push_back({dev, key, exec, kernels});
  if (cudaGraphLaunch(exec, g_stream.load()) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  g_launches.fetch_add(kernels, std::memory_order_relaxed);
  return true;
}

void set_error(int code, const char *fmt, ...) {
  g_err = code;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
}

void clear_error() {
  g_err = LSMGPU_OK;
  g_msg[0] = 0;
}

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  set_error(LSMGPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}

// Every entry point is one NVTX range named after it (visible in Nsight
// timelines; without a tool attached a push / pop is a cheap no-op).
Call::Call(const char *name) : name_(name) {
  nvtxRangePushA(name);
  clear_error();
  g_lock.lock();
  locked_ = true;
  int dev = 0;
  cudaGetDevice(&dev);
  Arena &a = g_arena[dev & 63];
  a.cur = 0;
  a.used = 0;
}

Call::~Call() {
  if (!finished_) finish();
  if (locked_) g_lock.unlock();
  nvtxRangePop();
}

void Call::fail(const char *msg) {
  if (ok_) set_error(LSMGPU_ERR_BOUNDS, "%s: %s", name_, msg);
  ok_ = false;
}

void *Call::arena_alloc(long long bytes) {
  if (!ok_) return nullptr;
  int dev = 0;
  cudaGetDevice(&dev);
  Arena &a = g_arena[dev & 63];
  long long need = (bytes + 255) & ~255LL;
  if (need == 0) need = 256;
  while (a.cur < (int)a.chunks.size()) {
    Chunk &c = a.chunks[a.cur];
    if (a.used + need <= c.cap) {
      void *p = c.p + a.used;
      a.used += need;
      return p;
    }
    a.cur++;
    a.used = 0;
  }
  long long cap = need < (64LL << 20) ? (64LL << 20) : need;
  void *p = nullptr;
  if (!cuda_ok(cudaMalloc(&p, (size_t)cap), "cudaMalloc(arena)")) {
    ok_ = false;
    return nullptr;
  }
  a.chunks.push_back({(char *)p, cap});
  g_arena_bytes.fetch_add(cap, std::memory_order_relaxed);
  a.cur = (int)a.chunks.size() - 1;
  a.used = need;
  return p;
}

void *Call::stage(const void *p, long long bytes, bool copy_in, bool copy_out) {
  if (!ok_) return nullptr;
  if (p == nullptr) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null array pointer", name_);
    ok_ = false;
    return nullptr;
  }
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return (void *)p;
  // host memory: stage through the arena
  host_staged_ = true;
  need_sync_ = true;
  void *d = arena_alloc(bytes);
  if (!d) return nullptr;
  if (copy_in && bytes > 0) {
    if (!cuda_ok(cudaMemcpyAsync(d, p, (size_t)bytes, cudaMemcpyHostToDevice, stream()),
                 "cudaMemcpyAsync(H2D)")) {
      ok_ = false;
      return nullptr;
    }
  }
  if (copy_out) {
    if (nback_ >= 64) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: too many staged outputs", name_);
      ok_ = false;
      return nullptr;
    }
    backs_[nback_++] = {(void *)p, d, bytes, 0, Box{}, Box{}};
  }
  return d;
}

void *Call::stage_region(void *p, long long elem, const Box &gb, const Box &region) {
  if (!ok_) return nullptr;
  if (p == nullptr) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null array pointer", name_);
    ok_ = false;
    return nullptr;
  }
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return p;
  host_staged_ = true;
  need_sync_ = true;
  void *d = arena_alloc(gb.size() * elem);
  if (!d) return nullptr;
  const Box r = isect(gb, region);
  if (r.empty()) return d;
  if (nback_ >= 64) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: too many staged outputs", name_);
    ok_ = false;
    return nullptr;
  }
  backs_[nback_++] = {p, d, 0, elem, gb, r};
  return d;
}

void *Call::scalar(void *dst, size_t bytes) {
  if (!ok_) return nullptr;
  if (dst == nullptr) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null scalar output", name_);
    ok_ = false;
    return nullptr;
  }
  void *d = arena_alloc((long long)bytes);
  if (!d) return nullptr;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, dst);
  if (e != cudaSuccess) {
    cudaGetLastError();
    attr.type = cudaMemoryTypeUnregistered;
  }
  if (!(attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged)) need_sync_ = true;
  backs_[nback_++] = {dst, d, (long long)bytes, 0, Box{}, Box{}};
  return d;
}

void Call::finish() {
  if (finished_) return;
  finished_ = true;
  if (ok_) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(LSMGPU_ERR_CUDA, "%s: kernel launch: %s", name_, cudaGetErrorString(e));
      ok_ = false;
    }
  }
  if (ok_) {
    for (int b = 0; b < nback_; b++) {
      const Back &k = backs_[b];
      if (k.bytes <= 0 && k.elem > 0) {
        // the region's rows, one 3D copy (x extent in bytes, y rows, z planes)
        cudaMemcpy3DParms m = {};
        const size_t pitch = (size_t)(k.gb.n(0) * k.elem);
        m.srcPtr = make_cudaPitchedPtr(k.dev, pitch, pitch, (size_t)k.gb.n(1));
        m.dstPtr = make_cudaPitchedPtr(k.host, pitch, pitch, (size_t)k.gb.n(1));
        m.srcPos = m.dstPos = make_cudaPos((size_t)((k.region.lo[0] - k.gb.lo[0]) * k.elem),
                                           (size_t)(k.region.lo[1] - k.gb.lo[1]),
                                           (size_t)(k.region.lo[2] - k.gb.lo[2]));
        m.extent = make_cudaExtent((size_t)(k.region.n(0) * k.elem), (size_t)k.region.n(1), (size_t)k.region.n(2));
        m.kind = cudaMemcpyDefault;
        if (!cuda_ok(cudaMemcpy3DAsync(&m, stream()), "cudaMemcpy3DAsync(D2H region)")) {
          ok_ = false;
          break;
        }
        continue;
      }
      if (k.bytes <= 0) continue;
      if (!cuda_ok(cudaMemcpyAsync(k.host, k.dev, (size_t)k.bytes, cudaMemcpyDefault, stream()),
                   "cudaMemcpyAsync(D2H)")) {
        ok_ = false;
        break;
      }
    }
  }
  if (need_sync_) {
    cudaError_t e = cudaStreamSynchronize(stream());
    if (ok_ && e != cudaSuccess) {
      set_error(LSMGPU_ERR_CUDA, "%s: %s", name_, cudaGetErrorString(e));
      ok_ = false;
    }
  }
  if (locked_) {
    locked_ = false;
    g_lock.unlock();
  }
}

}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

int lsmgpu_get_last_error(char *msg, int len) {
  if (msg && len > 0) {
    strncpy(msg, g_msg, (size_t)len - 1);
    msg[len - 1] = 0;
  }
  return g_err;
}

void lsmgpu_set_stream(void *s) {
  cudaStream_t old = g_stream.load();
  if (old != (cudaStream_t)s) {
    // the arena is reused in stream order: drain the old stream first
    std::lock_guard<std::mutex> guard(g_lock);
    cudaStreamSynchronize(old);
    g_stream.store((cudaStream_t)s);
  }
}

void *lsmgpu_get_stream(void) { return (void *)g_stream.load(); }

int lsmgpu_synchronize(void) {
  clear_error();
  if (!cuda_ok(cudaStreamSynchronize(g_stream.load()), "cudaStreamSynchronize")) return g_err;
  return LSMGPU_OK;
}

long long lsmgpu_launch_count(void) { return g_launches.load(); }
void lsmgpu_reset_launch_count(void) { g_launches.store(0); }
long long lsmgpu_graph_capture_count(void) { return g_captures.load(); }

int lsmgpu_bounds_check_read(long long *count, int *first) {
#ifdef LSMGPU_BOUNDS_CHECK
  clear_error();
  int h[4] = {0, 0, 0, 0};
  int *w = bounds_word();
  if (!w) return lsmgpu_get_last_error(nullptr, 0);
  std::lock_guard<std::mutex> guard(g_lock);
  if (!cuda_ok(cudaStreamSynchronize(g_stream.load()), "lsmgpu_bounds_check_read") ||
      !cuda_ok(cudaMemcpy(h, w, sizeof(h), cudaMemcpyDeviceToHost), "lsmgpu_bounds_check_read") ||
      !cuda_ok(cudaMemset(w, 0, sizeof(h)), "lsmgpu_bounds_check_read"))
    return g_err;
  if (count) *count = h[0];
  if (first)
    for (int q = 0; q < 3; q++) first[q] = h[1 + q];
  return LSMGPU_OK;
#else
  (void)count;
  (void)first;
  set_error(LSMGPU_ERR_ARGUMENT, "lsmgpu_bounds_check_read: this library was built without LSMGPU_BOUNDS_CHECK");
  return LSMGPU_ERR_ARGUMENT;
#endif
}

void lsmgpu_set_exact_side_effects(int on) { g_side_effects.store(on ? 1 : 0); }
int lsmgpu_get_exact_side_effects(void) { return exact_side_effects() ? 1 : 0; }
long long lsmgpu_arena_bytes(void) { return g_arena_bytes.load(); }

const char *lsmgpu_version(void) { return "lsmgpu 0.1 (sm_103a)"; }

}  // extern "C"
