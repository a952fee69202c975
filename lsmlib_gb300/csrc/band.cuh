// Narrow-band construction machinery shared by the drop-in entry points
// (band.cu) and the fused narrow-band stepper (bandflow.cu).
//
// Bit-exact with the reference's serial order:
//  - level 0 lists cells with |phi| < width in the reference's (k, j, i) sweep
//    order, which is the column-major memory order of phi's ghost box, so an
//    ordered compaction (block counts -> scan -> block-local scan + scatter)
//    reproduces it; the outer-layer lists are compacted the same way, minus
//    cells ascending from the front, plus cells descending from the back;
//  - each breadth-first level visits parents in list order and their
//    neighbours in the order +x, -x, +y, -y, +z, -z; the first visit claims a
//    cell.  Candidate t = 6*(parent position) + direction is therefore a total
//    order, the winner for a cell is the smallest t that reaches it (an
//    atomicMin over the level's candidates), and an ordered compaction of the
//    winners in t order gives the reference's list.
// The distance test runs in FP64 whatever the field's precision.
#pragma once
#include <climits>
#include <vector>

#include "lsmgpu_common.cuh"

namespace lsmgpu {
namespace {

typedef double R;
typedef unsigned char U8;
constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 32;  // elements per thread
constexpr long long SCAN_TILE = (long long)SCAN_BLOCK * SCAN_ITEMS;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)

// ---- ordered compaction with up to three counters ---------------------------
// A "classifier" F provides  __device__ int flags(long long e) returning bits
// 0..2 for element e, and __device__ void emit(long long e, int bits,
// long long r0, long long r1, long long r2) called with each counter's rank.
// A block takes SCAN_TILE consecutive elements; warp w takes the WARP_SPAN
// elements from w * WARP_SPAN in SCAN_ITEMS rounds of 32 consecutive elements
// (coalesced loads), and ranks inside a round come from warp ballots, so the
// ranks follow element order.
constexpr int SCAN_WARPS = SCAN_BLOCK / 32;
constexpr int WARP_SPAN = 32 * SCAN_ITEMS;

// Classifiers split flags(e) into load(e) (the memory read) and
// classify(value, e); the kernels issue all of a thread's loads before the
// ballots (a ballot orders the memory operations around it, so loads and
// ballots interleaved one element at a time would expose each load's
// latency).
template <class F>
__device__ __forceinline__ void load_round(const F &f, long long base, long long n, typename F::V v[SCAN_ITEMS]) {
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const long long e = base + 32LL * q;
    if (e < n) v[q] = f.load(e);
  }
}

template <class F>
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_count(F f, long long n, int *counts) {
  __shared__ int s[3][SCAN_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)w * WARP_SPAN + lane;
  int c0 = 0, c1 = 0, c2 = 0;
  if constexpr (F::kPrefetch) {
    typename F::V v[SCAN_ITEMS];
    load_round(f, base, n, v);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
      const long long e = base + 32LL * q;
      const int b = (e < n) ? f.classify(v[q], e) : 0;
      if (e < n) f.counted(e, b);
      if (__ballot_sync(0xffffffffu, b) == 0) continue;  // most rounds of a sparse band hold nothing
      c0 += __popc(__ballot_sync(0xffffffffu, b & 1));
      c1 += __popc(__ballot_sync(0xffffffffu, b & 2));
      c2 += __popc(__ballot_sync(0xffffffffu, b & 4));
    }
  } else {
    for (int q = 0; q < SCAN_ITEMS; q++) {
      const long long e = base + 32LL * q;
      const int b = (e < n) ? f.flags(e) : 0;
      c0 += __popc(__ballot_sync(0xffffffffu, b & 1));
      c1 += __popc(__ballot_sync(0xffffffffu, b & 2));
      c2 += __popc(__ballot_sync(0xffffffffu, b & 4));
    }
  }
  if (lane == 0) {
    s[0][w] = c0;
    s[1][w] = c1;
    s[2][w] = c2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    int t = 0;
    for (int u = 0; u < SCAN_WARPS; u++) t += s[threadIdx.x][u];
    counts[3 * blockIdx.x + threadIdx.x] = t;
  }
}

// exclusive scan of the per-block counts (one block of 1024 threads: serial
// chunks per thread, then a warp-shuffle scan of the chunk totals);
// totals[r] at the end
__device__ __forceinline__ long long warp_incl_scan(long long v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(int *counts, int nblocks, long long *offsets,
                                                       long long *totals) {
  __shared__ long long wsum[3][32];
  const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5;
  const int per = (nblocks + nt - 1) / nt;
  const int b0 = t * per, b1 = min(nblocks, b0 + per);
  long long loc[3] = {0, 0, 0};
  for (int b = b0; b < b1; b++)
    for (int r = 0; r < 3; r++) loc[r] += counts[3 * b + r];
  long long incl[3];
  for (int r = 0; r < 3; r++) {
    incl[r] = warp_incl_scan(loc[r], lane);
    if (lane == 31) wsum[r][w] = incl[r];
  }
  __syncthreads();
  if (w == 0) {
    for (int r = 0; r < 3; r++) {
      const long long v = lane < nt / 32 ? wsum[r][lane] : 0;
      const long long x = warp_incl_scan(v, lane);
      wsum[r][lane] = x - v;  // exclusive prefix of the warp totals
      if (lane == 31) totals[r] = x;
    }
  }
  __syncthreads();
  long long run[3];
  for (int r = 0; r < 3; r++) run[r] = wsum[r][w] + incl[r] - loc[r];
  for (int b = b0; b < b1; b++)
    for (int r = 0; r < 3; r++) {
      offsets[3 * b + r] = run[r];
      run[r] += counts[3 * b + r];
    }
}

// An emit may change data a classify call reads (the breadth-first
// classifier marks the cell its winner claimed), but only for a cell whose one
// winner it is, so every element's flags in this pass equal the count pass's.
template <class F>
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_emit(F f, long long n, const long long *offsets,
                                                           const int *counts) {
  // a tile the count pass found empty has nothing to emit
  if ((counts[3 * blockIdx.x] | counts[3 * blockIdx.x + 1] | counts[3 * blockIdx.x + 2]) == 0) return;
  __shared__ int s[3][SCAN_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)w * WARP_SPAN + lane;
  int c[3] = {0, 0, 0};
  int bits[F::kPrefetch ? SCAN_ITEMS : 1];
  if constexpr (F::kPrefetch) {
    typename F::V v[SCAN_ITEMS];
    load_round(f, base, n, v);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS; q++) {
      const long long e = base + 32LL * q;
      bits[q] = (e < n) ? f.classify(v[q], e) : 0;
      if (__ballot_sync(0xffffffffu, bits[q]) == 0) continue;
#pragma unroll
      for (int r = 0; r < 3; r++) c[r] += __popc(__ballot_sync(0xffffffffu, (bits[q] >> r) & 1));
    }
  } else {
    for (int q = 0; q < SCAN_ITEMS; q++) {
      const long long e = base + 32LL * q;
      const int b = (e < n) ? f.flags(e) : 0;
#pragma unroll
      for (int r = 0; r < 3; r++) c[r] += __popc(__ballot_sync(0xffffffffu, (b >> r) & 1));
    }
  }
  if (lane == 0)
    for (int r = 0; r < 3; r++) s[r][w] = c[r];
  __syncthreads();
  long long run[3];
  for (int r = 0; r < 3; r++) {
    long long o = offsets[3 * blockIdx.x + r];
    for (int u = 0; u < w; u++) o += s[r][u];
    run[r] = o;
  }
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const long long e = base + 32LL * q;
    int b;
    if constexpr (F::kPrefetch) b = bits[q];
    else b = (e < n) ? f.flags(e) : 0;
    if (__ballot_sync(0xffffffffu, b) == 0) continue;
    const unsigned m0 = __ballot_sync(0xffffffffu, b & 1);
    const unsigned m1 = __ballot_sync(0xffffffffu, b & 2);
    const unsigned m2 = __ballot_sync(0xffffffffu, b & 4);
    if (b) f.emit(e, b, run[0] + __popc(m0 & below), run[1] + __popc(m1 & below), run[2] + __popc(m2 & below));
    run[0] += __popc(m0);
    run[1] += __popc(m1);
    run[2] += __popc(m2);
  }
}

// Ordered compaction in two calls: count() runs the per-block counts and the
// scan and returns the three totals (synchronous, so capacities can be
// checked before anything is written); emit() then writes every element's
// ranks using the same offsets.
struct Compaction {
  long long n = 0, nb = 0;
  int *counts = nullptr;
  long long *offs = nullptr, *tot = nullptr;

  template <class F>
  bool count(Call &call, F f, long long n_, long long totals_out[3]) {
    n = n_;
    nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    totals_out[0] = totals_out[1] = totals_out[2] = 0;
    if (nb == 0) return true;
    counts = call.temp<int>(3 * nb);
    offs = call.temp<long long>(3 * nb);
    tot = call.temp<long long>(3);
    if (!call.ok()) return false;
    LSMGPU_LAUNCH(k_scan_count<F>, (unsigned)nb, SCAN_BLOCK, 0, f, n, counts);
    LSMGPU_LAUNCH(k_scan_blocks, 1, 1024, 0, counts, (int)nb, offs, tot);
    return cuda_ok(cudaMemcpyAsync(totals_out, tot, 3 * sizeof(long long), cudaMemcpyDeviceToHost, stream()),
                   "cudaMemcpyAsync(totals)") &&
           cuda_ok(cudaStreamSynchronize(stream()), "cudaStreamSynchronize");
  }

  template <class F>
  void emit(F f) const {
    if (nb > 0) LSMGPU_LAUNCH(k_scan_emit<F>, (unsigned)nb, SCAN_BLOCK, 0, f, n, offs, counts);
  }
};

// count + emit in one go; returns the three totals
template <class F>
bool compact(Call &call, F f, long long n, long long totals_out[3]) {
  Compaction c;
  if (!c.count(call, f, n, totals_out)) return false;
  c.emit(f);
  return true;
}

// ---- level 0 -------------------------------------------------------------------
template <class T>
struct Level0T {
  View<const T> phi;      // over gb
  View<U8> nb;            // over the nb box
  Box gb;
  long long nx, nxy;
  R width, width_inner;
  int *ix, *iy, *iz;      // list arrays (element 0 = entry nlo_index)
  int *outer;             // index_outer (element 0 = entry nlo_outer)
  int nlo, nlo_outer, nhi_outer;
  int mode;               // 0: |phi| < width, 1: mask >= 0, 2: mask <= 0,
                          // 3: |phi| < width and |second| < width,
                          // 4: |phi| < width and |phi - second| > max_dx
  View<const T> second;   // over gb (modes 3, 4)
  R max_dx;
  __device__ void cell(long long e, int &i, int &j, int &k) const {
    if (nxy * (gb.hi[2] - gb.lo[2] + 1) <= 0x7fffffffLL) {  // 32-bit division when the box allows
      const unsigned u = (unsigned)e, uxy = (unsigned)nxy, ux = (unsigned)nx;
      const unsigned kk = u / uxy, r = u - kk * uxy, jj = r / ux;
      k = gb.lo[2] + (int)kk;
      j = gb.lo[1] + (int)jj;
      i = gb.lo[0] + (int)(r - jj * ux);
      return;
    }
    k = gb.lo[2] + (int)(e / nxy);
    const long long r = e % nxy;
    j = gb.lo[1] + (int)(r / nx);
    i = gb.lo[0] + (int)(r % nx);
  }
  // FP32 fields compare in FP32 against thresholds rounded so each decision
  // equals the FP64 one: for a float a, (double)a < width <=> a <= width_lt
  // (the largest float below width) and (double)a >= width_inner <=>
  // a >= inner_ge (the smallest float not below width_inner)
  float width_lt, inner_ge;
  // when set (nb box == phi's box): the count pass writes every cell's
  // classification bits into its mark byte (1 level 0, 2 outer minus, 4 outer
  // plus); the emit pass (Level0Marks) reads them back instead of phi and
  // leaves the final marks (1 in level 0, 0 elsewhere)
  U8 *mark_lin = nullptr;
  static constexpr bool kPrefetch = true;
  __device__ void counted(long long e, int bits) const {
    if (mark_lin) mark_lin[e] = (U8)bits;
  }
  typedef T V;
  __device__ T load(long long e) const { return phi.p[e]; }
  __device__ int flags(long long e) const { return classify(phi.p[e], e); }
  __device__ int classify(T raw, long long e) const {
    if (mode >= 3) {  // the 2D two-level-set / away-from-mask selections (localization2d.f:248-460)
      const R v = (R)raw, a = fabs(v), w = (R)second.p[e];
      if (!(a < width)) return 0;
      if (mode == 3 ? !(fabs(w) < width) : !(fabs(v - w) > max_dx)) return 0;
      if (a >= width_inner) return v <= R(0) ? 3 : 5;
      return 1;
    }
    if constexpr (sizeof(T) == 4) {
      const float v = (float)raw;
      if (mode == 1) return v >= 0.f ? 1 : 0;
      if (mode == 2) return v <= 0.f ? 1 : 0;
      const float a = fabsf(v);
      if (!(a <= width_lt)) return 0;
      if (a >= inner_ge) return v <= 0.f ? 3 : 5;
      return 1;
    } else {
      const R v = (R)raw;
      if (mode == 1) return v >= R(0) ? 1 : 0;
      if (mode == 2) return v <= R(0) ? 1 : 0;
      const R a = fabs(v);
      if (!(a < width)) return 0;
      if (a >= width_inner) return v <= R(0) ? 3 : 5;
      return 1;
    }
  }
  void set_widths(double w, double wi) {
    width = w;
    width_inner = wi;
    float f = (float)w;
    if ((double)f >= w) f = nextafterf(f, -INFINITY);
    width_lt = f;
    float g = (float)wi;
    if ((double)g < wi) g = nextafterf(g, INFINITY);
    inner_ge = g;
  }
  __device__ void emit(long long e, int bits, long long r0, long long r1, long long r2) const {
    int i, j, k;
    cell(e, i, j, k);
    const long long pos = r0;  // element of the list arrays
    ix[pos] = i;
    iy[pos] = j;
    iz[pos] = k;
    if (bits & 2) outer[r1] = nlo + (int)pos;
    if (bits & 4) outer[(nhi_outer - nlo_outer) - r2] = nlo + (int)pos;
  }
};

typedef Level0T<R> Level0;

// emit pass of a fused-marks level-0 build: the classification comes from the
// mark bytes the count pass wrote (a quarter of phi's bytes for FP32, an
// eighth for FP64); each listed cell's byte becomes its final mark 1
template <class T>
struct Level0Marks {
  Level0T<T> z;
  U8 *marks;
  static constexpr bool kPrefetch = true;
  typedef U8 V;
  __device__ U8 load(long long e) const { return marks[e]; }
  __device__ int classify(U8 raw, long long) const { return raw; }
  __device__ int flags(long long e) const { return marks[e]; }
  __device__ void counted(long long, int) const {}
  __device__ void emit(long long e, int bits, long long r0, long long r1, long long r2) const {
    z.emit(e, bits, r0, r1, r2);
    marks[e] = 1;
  }
};

// Level-0 pass of a rebuild inside the narrow-band flow over the previous
// level-0 list (ox, oy, oz) instead of the grid: between rebuilds the flow
// writes phi only at level-0 cells, so a cell outside the previous level 0
// still has |phi| >= width and the new level 0 (and its outer layer) is the
// ordered sub-sequence of the previous level-0 list whose cells pass the test
// (the previous list is in the reference's sweep order).  The caller clears
// the previous band's marks first; each listed cell gets mark 1.
template <class T>
struct Level0List {
  Level0T<T> z;
  const int *ox, *oy, *oz;
  static constexpr bool kPrefetch = true;
  typedef T V;
  __device__ T load(long long e) const { return z.phi.p[z.phi.off(ox[e], oy[e], oz[e])]; }
  __device__ int classify(T raw, long long) const { return z.classify(raw, 0); }
  __device__ int flags(long long e) const { return classify(load(e), e); }
  __device__ void counted(long long, int) const {}
  __device__ void emit(long long e, int bits, long long r0, long long r1, long long r2) const {
    const int i = ox[e], j = oy[e], k = oz[e];
    z.ix[r0] = i;
    z.iy[r0] = j;
    z.iz[r0] = k;
    if (bits & 2) z.outer[r1] = z.nlo + (int)r0;
    if (bits & 4) z.outer[(z.nhi_outer - z.nlo_outer) - r2] = z.nlo + (int)r0;
    z.nb(i, j, k) = 1;
  }
};

// every cell of phi's ghost box gets its level-0 mark (1 in the band, 0 out);
// threads along x and y, each walking kMarkZ planes
constexpr int kMarkZ = 16;
template <class T>
__global__ void k_mark0(Level0T<T> z) {
  const int i = z.gb.lo[0] + (int)(blockIdx.x * 32 + threadIdx.x);
  const int j = z.gb.lo[1] + (int)(blockIdx.y * 8 + threadIdx.y);
  const int k0 = z.gb.lo[2] + (int)blockIdx.z * kMarkZ;
  if (i > z.gb.hi[0] || j > z.gb.hi[1]) return;
  T v[kMarkZ];  // all loads before the stores (the arrays may alias for the compiler)
#pragma unroll
  for (int q = 0; q < kMarkZ; q++)
    if (k0 + q <= z.gb.hi[2]) v[q] = z.phi.p[z.phi.off(i, j, k0 + q)];
#pragma unroll
  for (int q = 0; q < kMarkZ; q++)
    if (k0 + q <= z.gb.hi[2]) z.nb(i, j, k0 + q) = (z.classify(v[q], z.phi.off(i, j, k0 + q)) & 1) ? 1 : 0;
}

// claim value of an unclaimed cell (a byte pattern, so a memset sets it)
constexpr int kUnclaimed = 0x7f7f7f7f;

// ---- breadth-first levels --------------------------------------------------------
struct Bfs {
  View<U8> nb;
  Box nbb;
  int *claim;             // over the nb box, kUnclaimed where unclaimed
  int *ix, *iy, *iz;      // list arrays, element 0 = entry nlo_index
  int nlo;                // list base
  int plo;                // first parent entry of this level
  int count0;             // first free entry
  U8 mark;
  __device__ long long cidx(int a, int b, int c) const { return nb.off(a, b, c); }
};

// A level runs with one thread per parent and its six candidates
// t = 6 p + d (parent p of the level, direction d): the claim (atomicMin of
// t), then an ordered compaction of the winners in t order whose count pass
// stores each parent's winner bits (one byte) and whose emit pass ranks a
// parent's winners by a warp scan of the bit counts, lists them, marks their
// cells with the level and releases the claims.
constexpr int BFS_ITEMS = 8;                         // parents per thread
constexpr long long BFS_TILE = (long long)SCAN_BLOCK * BFS_ITEMS;

__device__ __forceinline__ bool bfs_nbr6(const Bfs &f, int a, int b, int c, int d, int &x, int &y, int &z) {
  x = a; y = b; z = c;
  switch (d) {
    case 0: if (!(a < f.nbb.hi[0])) return false; x = a + 1; break;
    case 1: if (!(a > f.nbb.lo[0])) return false; x = a - 1; break;
    case 2: if (!(b < f.nbb.hi[1])) return false; y = b + 1; break;
    case 3: if (!(b > f.nbb.lo[1])) return false; y = b - 1; break;
    case 4: if (!(c < f.nbb.hi[2])) return false; z = c + 1; break;
    default: if (!(c > f.nbb.lo[2])) return false; z = c - 1; break;
  }
  return true;
}

__global__ void k_bfs_claim6(Bfs f, long long np) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const long long e = f.plo + p - f.nlo;
  const int a = f.ix[e], b = f.iy[e], c = f.iz[e];
#pragma unroll
  for (int d = 0; d < 6; d++) {
    int x, y, z;
    if (!bfs_nbr6(f, a, b, c, d, x, y, z)) continue;
    const long long o = f.cidx(x, y, z);
    if (f.nb.p[o] == 0) atomicMin(&f.claim[o], (int)(6 * p + d));
  }
}

// winner bits of parent p (bit d: candidate 6 p + d won its cell)
__device__ __forceinline__ unsigned bfs_winners6(const Bfs &f, long long p) {
  const long long e = f.plo + p - f.nlo;
  const int a = f.ix[e], b = f.iy[e], c = f.iz[e];
  unsigned m = 0;
#pragma unroll
  for (int d = 0; d < 6; d++) {
    int x, y, z;
    if (!bfs_nbr6(f, a, b, c, d, x, y, z)) continue;
    const long long o = f.cidx(x, y, z);
    if (f.nb.p[o] == 0 && f.claim[o] == (int)(6 * p + d)) m |= 1u << d;
  }
  return m;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_bfs_count6(Bfs f, long long np, int *counts, U8 *wm) {
  __shared__ int s[SCAN_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * BFS_TILE + (long long)w * 32 * BFS_ITEMS + lane;
  int cnt = 0;
#pragma unroll
  for (int q = 0; q < BFS_ITEMS; q++) {
    const long long p = base + 32LL * q;
    if (p < np) {
      const unsigned m = bfs_winners6(f, p);
      wm[p] = (U8)m;
      cnt += __popc(m);
    }
  }
  cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
  if (lane == 0) s[w] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int u = 0; u < SCAN_WARPS; u++) t += s[u];
    counts[3 * blockIdx.x] = t;
    counts[3 * blockIdx.x + 1] = 0;
    counts[3 * blockIdx.x + 2] = 0;
  }
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_bfs_emit6(Bfs f, long long np, const long long *offsets,
                                                          const int *counts, const U8 *wm) {
  if (counts[3 * blockIdx.x] == 0) return;
  __shared__ int s[SCAN_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * BFS_TILE + (long long)w * 32 * BFS_ITEMS + lane;
  unsigned m[BFS_ITEMS];
  int cnt = 0;
#pragma unroll
  for (int q = 0; q < BFS_ITEMS; q++) {
    const long long p = base + 32LL * q;
    m[q] = p < np ? wm[p] : 0u;
    cnt += __popc(m[q]);
  }
  cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
  if (lane == 0) s[w] = cnt;
  __syncthreads();
  long long run = offsets[3 * blockIdx.x];
  for (int u = 0; u < w; u++) run += s[u];
#pragma unroll
  for (int q = 0; q < BFS_ITEMS; q++) {
    const int c = __popc(m[q]);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (m[q]) {
      const long long p = base + 32LL * q;
      const long long e = f.plo + p - f.nlo;
      const int a = f.ix[e], b = f.iy[e], cc = f.iz[e];
      long long pos = (long long)f.count0 - f.nlo + run + incl - c;
      for (int d = 0; d < 6; d++) {
        if (!((m[q] >> d) & 1u)) continue;
        int x, y, z;
        bfs_nbr6(f, a, b, cc, d, x, y, z);
        f.ix[pos] = x;
        f.iy[pos] = y;
        f.iz[pos] = z;
        const long long o = f.cidx(x, y, z);
        f.nb.p[o] = f.mark;
        f.claim[o] = kUnclaimed;
        pos++;
      }
    }
    run += total;
  }
}

// claim array over the nb box, every entry kUnclaimed; bfs_levels leaves it so
int *new_claims(Call &call, const Box &nbb) {
  int *claim = call.temp<int>(nbb.size());
  if (call.ok()) cudaMemsetAsync(claim, 0x7f, (size_t)nbb.size() * sizeof(int), stream());
  return claim;
}

// Breadth-first levels 1..level from the lists already holding levels
// 0..(start-1); lo/hi are host copies of n_lo/n_hi, updated in place.
// `claim` (over the nb box) must hold kUnclaimed everywhere and is returned so.
bool bfs_levels(Call &call, View<U8> nb, const Box &nbb, int *ix, int *iy, int *iz, int nlo, int nhi,
                std::vector<int> &lo, std::vector<int> &hi, int level, int *claim) {
  if (!claim) return false;
  long long count = (long long)hi[0] + 1;
  for (int lv = 1; lv <= level; lv++) {
    // an empty parent level (-1, -1) yields an empty level; the reference
    // would index entry -1 here
    const long long np = (lo[lv - 1] >= 0 && hi[lv - 1] >= lo[lv - 1]) ? (long long)hi[lv - 1] - lo[lv - 1] + 1 : 0;
    long long added = 0;
    if (np > 0) {
      if (6 * np >= kUnclaimed) {
        set_error(LSMGPU_ERR_CAPACITY, "narrow band level too large for 32-bit candidate keys");
        return false;
      }
      Bfs f{nb, nbb, claim, ix, iy, iz, nlo, lo[lv - 1], (int)count, (U8)(lv + 1)};
      // one thread per parent (its six candidates in t order)
      const long long nbk = (np + BFS_TILE - 1) / BFS_TILE;
      U8 *wm = call.temp<U8>(np);
      int *counts = call.temp<int>(3 * nbk);
      long long *offs = call.temp<long long>(3 * nbk), *totd = call.temp<long long>(3);
      if (!call.ok()) return false;
      LSMGPU_LAUNCH(k_bfs_claim6, (unsigned)((np + 255) / 256), 256, 0, f, np);
      LSMGPU_LAUNCH(k_bfs_count6, (unsigned)nbk, SCAN_BLOCK, 0, f, np, counts, wm);
      LSMGPU_LAUNCH(k_scan_blocks, 1, 1024, 0, counts, (int)nbk, offs, totd);
      // the emit writes list entries count .. count+added-1; the total is
      // checked against the capacity before anything is written
      long long tot[3];
      if (!cuda_ok(cudaMemcpyAsync(tot, totd, 3 * sizeof(long long), cudaMemcpyDeviceToHost, stream()),
                   "cudaMemcpyAsync(totals)") ||
          !cuda_ok(cudaStreamSynchronize(stream()), "cudaStreamSynchronize"))
        return false;
      if (count + tot[0] - 1 > nhi) {
        set_error(LSMGPU_ERR_CAPACITY, "narrow band lists exceed nhi_index");
        return false;
      }
      LSMGPU_LAUNCH(k_bfs_emit6, (unsigned)nbk, SCAN_BLOCK, 0, f, np, offs, counts, wm);
      added = tot[0];
    }
    if (added > 0) {
      lo[lv] = hi[lv - 1] + 1;
      hi[lv] = (int)(count + added - 1);
    } else {
      lo[lv] = -1;
      hi[lv] = -1;
    }
    count += added;
  }
  return true;
}

// small integer outputs (n_lo, n_hi, outer-list bounds) may live in host or
// device memory
bool is_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
void get_ints(int *dst, const int *src, int n) {
  if (is_device(src)) {
    cudaStreamSynchronize(stream());
    cudaMemcpy(dst, src, sizeof(int) * n, cudaMemcpyDeviceToHost);
  } else {
    for (int q = 0; q < n; q++) dst[q] = src[q];
  }
}
void put_ints(int *dst, const int *src, int n) {
  if (is_device(dst)) {
    cudaStreamSynchronize(stream());
    cudaMemcpy(dst, src, sizeof(int) * n, cudaMemcpyHostToDevice);
  } else {
    for (int q = 0; q < n; q++) dst[q] = src[q];
  }
}


// Level-0 selection and list bookkeeping of a band build.
//  l0_mode: 0 |phi| < width; 3 also |second| < width; 4 also
//           |phi - second| > max_dx (second over phi's ghost box)
//  bookkeeping: 0 the 3D routines' (localization3d.f:274-292: an empty band
//           sets n_hi(0) = nlo and the outer bounds to their starts, and
//           writes level 0 only); 1 lsm2dDetermineNarrowBand's
//           (localization2d.f:225-240: n_hi(0) = count - 1 always, neighbour
//           levels only when level 0 holds two or more cells); 2 the 2D
//           two-level-set and away-from-mask routines' (:327-340: as 1, with
//           neighbour levels whenever level > 0)
template <class T>
struct BandForm {
  int l0_mode = 0;
  const T *second = nullptr;
  double max_dx = 0;
  int bookkeeping = 0;
};

// Builds the band of `phi` (device arrays) inside `call`: level-0 lists,
// outer lists and `level` neighbour levels.  lo/hi receive n_lo/n_hi, ob the
// outer-list bounds {plus lo, plus hi, minus lo, minus hi}, *nwrite (when
// set) the number of levels the reference writes.  Returns false after
// recording an error (capacity or CUDA).
// prev (optional, level-0 selection |phi| < width only): the previous
// level-0 list {ox, oy, oz, count} of a rebuild inside the narrow-band flow
// (Level0List); the caller has cleared that band's marks
struct PrevLevel0 {
  const int *ox = nullptr, *oy = nullptr, *oz = nullptr;
  long long n = 0;
};

template <class T>
bool band_build(Call &call, const T *phi, const Box &gb, U8 *nbd, const Box &nbb, int *ix, int *iy, int *iz,
                int nlo, int nhi, int *outer, int nlo_outer, int nhi_outer, double width, double width_inner,
                int level, std::vector<int> &lo, std::vector<int> &hi, int ob[4], long long *level0_count,
                int *claim, bool fuse_marks = false, const BandForm<T> &form = BandForm<T>(),
                int *nwrite = nullptr, const PrevLevel0 *prev = nullptr) {
  const long long cap = (long long)nhi - nlo + 1;
  const long long ocap = (long long)nhi_outer - nlo_outer + 1;
  Level0T<T> z;
  z.phi = view(phi, gb);
  z.nb = view(nbd, nbb);
  z.gb = gb;
  z.nx = gb.n(0);
  z.nxy = gb.n(0) * gb.n(1);
  z.set_widths(width, width_inner);
  z.ix = ix; z.iy = iy; z.iz = iz;
  z.outer = outer;
  z.nlo = nlo;
  z.nlo_outer = nlo_outer;
  z.nhi_outer = nhi_outer;
  z.mode = form.l0_mode;
  if (form.second) z.second = view(form.second, gb);
  z.max_dx = form.max_dx;
  const long long n = gb.size();
  long long tot[3];
  // fused marks: the count pass writes every cell's level-0 mark (the nb
  // array has phi's box); only for callers that own the arrays, since the
  // marks are then written before the capacity check
  const bool fused = fuse_marks && nbb.lo[0] == gb.lo[0] && nbb.hi[0] == gb.hi[0] && nbb.lo[1] == gb.lo[1] &&
                     nbb.hi[1] == gb.hi[1] && nbb.lo[2] == gb.lo[2] && nbb.hi[2] == gb.hi[2];
  const bool from_list = prev && prev->ox && form.l0_mode == 0;
  if (fused && !from_list) z.mark_lin = nbd;
  Compaction c0;
  if (from_list) {
    if (!c0.count(call, Level0List<T>{z, prev->ox, prev->oy, prev->oz}, prev->n, tot)) return false;
  } else if (!c0.count(call, z, n, tot)) {
    return false;
  }
  z.mark_lin = nullptr;
  if (tot[0] > cap || tot[1] + tot[2] > ocap) {
    set_error(LSMGPU_ERR_CAPACITY, "narrow band (%lld cells) or outer layer (%lld) exceeds the index arrays", tot[0],
              tot[1] + tot[2]);
    return false;
  }
  if (from_list) {
    c0.emit(Level0List<T>{z, prev->ox, prev->oy, prev->oz});
  } else if (fused) {
    c0.emit(Level0Marks<T>{z, nbd});
  } else {
    LSMGPU_LAUNCH(k_mark0<T>,
                  dim3((unsigned)((gb.n(0) + 31) / 32), (unsigned)((gb.n(1) + 7) / 8),
                       (unsigned)((gb.n(2) + kMarkZ - 1) / kMarkZ)),
                  dim3(32, 8), 0, z);
    c0.emit(z);
  }
  lo.assign(level + 1, -1);
  hi.assign(level + 1, -1);
  lo[0] = nlo;
  ob[0] = nhi_outer; ob[1] = nhi_outer; ob[2] = nlo_outer; ob[3] = nlo_outer;
  if (level0_count) *level0_count = tot[0];
  if (form.bookkeeping != 0) {
    hi[0] = (int)(nlo + tot[0] - 1);
    ob[2] = nlo_outer;
    ob[3] = (int)(nlo_outer + tot[1] - 1);
    ob[0] = (int)(nhi_outer - tot[2] + 1);
    ob[1] = nhi_outer;
    const bool levels = level > 0 && (form.bookkeeping == 2 || hi[0] > lo[0]);
    if (nwrite) *nwrite = levels ? level + 1 : 1;
    if (levels && !bfs_levels(call, z.nb, nbb, ix, iy, iz, nlo, nhi, lo, hi, level, claim)) return false;
    return true;
  }
  if (nwrite) *nwrite = tot[0] > 0 ? level + 1 : 1;
  if (tot[0] > 0) {
    hi[0] = (int)(nlo + tot[0] - 1);
    ob[2] = nlo_outer;
    ob[3] = (int)(nlo_outer + tot[1] - 1);
    ob[0] = (int)(nhi_outer - tot[2] + 1);
    ob[1] = nhi_outer;
    if (!bfs_levels(call, z.nb, nbb, ix, iy, iz, nlo, nhi, lo, hi, level, claim)) return false;
  } else {
    hi[0] = nlo;  // localization3d.f:289-292
  }
  return true;
}

}  // namespace
}  // namespace lsmgpu
