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
constexpr int SCAN_ITEMS = 16;  // elements per thread
constexpr long long SCAN_TILE = (long long)SCAN_BLOCK * SCAN_ITEMS;

#define BOXARG(b) const int *b##_ilo, const int *b##_ihi, const int *b##_jlo, const int *b##_jhi, const int *b##_klo, const int *b##_khi
#define BOXOF(b) mkbox(b##_ilo, b##_ihi, b##_jlo, b##_jhi, b##_klo, b##_khi)

// ---- ordered compaction with up to three counters ---------------------------
// A "classifier" F provides  __device__ int flags(long long e) returning bits
// 0..2 for element e, and __device__ void emit(long long e, int bits,
// long long r0, long long r1, long long r2) called with each counter's rank.
template <class F>
__global__ void k_scan_count(F f, long long n, int *counts) {
  __shared__ int s[3][SCAN_BLOCK];
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  int c0 = 0, c1 = 0, c2 = 0;
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const long long e = base + q;
    if (e < n) {
      const int b = f.flags(e);
      c0 += b & 1;
      c1 += (b >> 1) & 1;
      c2 += (b >> 2) & 1;
    }
  }
  s[0][threadIdx.x] = c0;
  s[1][threadIdx.x] = c1;
  s[2][threadIdx.x] = c2;
  __syncthreads();
  for (int st = SCAN_BLOCK / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int r = 0; r < 3; r++) s[r][threadIdx.x] += s[r][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int r = 0; r < 3; r++) counts[3 * blockIdx.x + r] = s[r][0];
}

// exclusive scan of the per-block counts (one block; serial chunks per
// thread, then a shared-memory scan of the chunk totals); totals[r] at the end
__global__ void k_scan_blocks(int *counts, int nblocks, long long *offsets, long long *totals) {
  __shared__ long long chunk[3][1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const int per = (nblocks + nt - 1) / nt;
  const int b0 = t * per, b1 = min(nblocks, b0 + per);
  long long loc[3] = {0, 0, 0};
  for (int b = b0; b < b1; b++)
    for (int r = 0; r < 3; r++) loc[r] += counts[3 * b + r];
  for (int r = 0; r < 3; r++) chunk[r][t] = loc[r];
  __syncthreads();
  if (t == 0) {
    long long acc[3] = {0, 0, 0};
    for (int u = 0; u < nt; u++)
      for (int r = 0; r < 3; r++) {
        const long long v = chunk[r][u];
        chunk[r][u] = acc[r];
        acc[r] += v;
      }
    for (int r = 0; r < 3; r++) totals[r] = acc[r];
  }
  __syncthreads();
  long long run[3] = {chunk[0][t], chunk[1][t], chunk[2][t]};
  for (int b = b0; b < b1; b++)
    for (int r = 0; r < 3; r++) {
      offsets[3 * b + r] = run[r];
      run[r] += counts[3 * b + r];
    }
}

template <class F>
__global__ void k_scan_emit(F f, long long n, const long long *offsets) {
  __shared__ int s[3][SCAN_BLOCK];
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  int bits[SCAN_ITEMS];
  int c[3] = {0, 0, 0};
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const long long e = base + q;
    bits[q] = (e < n) ? f.flags(e) : 0;
    for (int r = 0; r < 3; r++) c[r] += (bits[q] >> r) & 1;
  }
  for (int r = 0; r < 3; r++) s[r][threadIdx.x] = c[r];
  __syncthreads();
  // inclusive Hillis-Steele scan over the block's thread totals
  for (int st = 1; st < SCAN_BLOCK; st <<= 1) {
    int v[3] = {0, 0, 0};
    if ((int)threadIdx.x >= st)
      for (int r = 0; r < 3; r++) v[r] = s[r][threadIdx.x - st];
    __syncthreads();
    for (int r = 0; r < 3; r++) s[r][threadIdx.x] += v[r];
    __syncthreads();
  }
  long long rank[3];
  for (int r = 0; r < 3; r++) rank[r] = offsets[3 * blockIdx.x + r] + s[r][threadIdx.x] - c[r];
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const long long e = base + q;
    if (e >= n) break;
    if (bits[q]) f.emit(e, bits[q], rank[0], rank[1], rank[2]);
    for (int r = 0; r < 3; r++) rank[r] += (bits[q] >> r) & 1;
  }
}

// counts only (no emission), for capacity checks before anything is written
template <class F>
struct CountOnly {
  F f;
  __device__ int flags(long long e) const { return f.flags(e); }
  __device__ void emit(long long, int, long long, long long, long long) const {}
};

// runs the compaction; returns the three totals (synchronous)
template <class F>
bool compact(Call &call, F f, long long n, long long totals_out[3]) {
  const long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 0) {
    totals_out[0] = totals_out[1] = totals_out[2] = 0;
    return true;
  }
  int *counts = call.temp<int>(3 * nb);
  long long *offs = call.temp<long long>(3 * nb);
  long long *tot = call.temp<long long>(3);
  if (!call.ok()) return false;
  LSMGPU_LAUNCH(k_scan_count<F>, (unsigned)nb, SCAN_BLOCK, 0, f, n, counts);
  LSMGPU_LAUNCH(k_scan_blocks, 1, 1024, 0, counts, (int)nb, offs, tot);
  LSMGPU_LAUNCH(k_scan_emit<F>, (unsigned)nb, SCAN_BLOCK, 0, f, n, offs);
  if (!cuda_ok(cudaMemcpyAsync(totals_out, tot, 3 * sizeof(long long), cudaMemcpyDeviceToHost, stream()),
               "cudaMemcpyAsync(totals)") ||
      !cuda_ok(cudaStreamSynchronize(stream()), "cudaStreamSynchronize"))
    return false;
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
  int mode;               // 0: |phi| < width, 1: mask >= 0, 2: mask <= 0
  __device__ void cell(long long e, int &i, int &j, int &k) const {
    k = gb.lo[2] + (int)(e / nxy);
    const long long r = e % nxy;
    j = gb.lo[1] + (int)(r / nx);
    i = gb.lo[0] + (int)(r % nx);
  }
  __device__ int flags(long long e) const {
    const R v = (R)phi.p[e];
    if (mode == 1) return v >= R(0) ? 1 : 0;
    if (mode == 2) return v <= R(0) ? 1 : 0;
    const R a = fabs(v);
    if (!(a < width)) return 0;
    if (a >= width_inner) return v <= R(0) ? 3 : 5;
    return 1;
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

// every cell of phi's ghost box gets its level-0 mark (1 in the band, 0 out)
template <class T>
__global__ void k_mark0(Level0T<T> z, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int i, j, k;
  z.cell(e, i, j, k);
  z.nb(i, j, k) = (z.flags(e) & 1) ? 1 : 0;
}

// ---- breadth-first levels --------------------------------------------------------
struct Bfs {
  View<U8> nb;
  Box nbb;
  int *claim;             // over the nb box, INT_MAX where unclaimed
  int *ix, *iy, *iz;      // list arrays, element 0 = entry nlo_index
  int nlo;                // list base
  int plo;                // first parent entry of this level
  int count0;             // first free entry
  U8 mark;
  __device__ bool nbr(long long t, int &a, int &b, int &c) const {
    const long long m = plo + t / 6;
    const int q = (int)(t % 6);
    const long long e = m - nlo;
    a = ix[e]; b = iy[e]; c = iz[e];
    switch (q) {
      case 0: if (!(a < nbb.hi[0])) return false; a += 1; break;
      case 1: if (!(a > nbb.lo[0])) return false; a -= 1; break;
      case 2: if (!(b < nbb.hi[1])) return false; b += 1; break;
      case 3: if (!(b > nbb.lo[1])) return false; b -= 1; break;
      case 4: if (!(c < nbb.hi[2])) return false; c += 1; break;
      default: if (!(c > nbb.lo[2])) return false; c -= 1; break;
    }
    return true;
  }
  __device__ long long cidx(int a, int b, int c) const { return nb.off(a, b, c); }
  __device__ int flags(long long t) const {
    int a, b, c;
    if (!nbr(t, a, b, c)) return 0;
    const long long o = cidx(a, b, c);
    return (nb.p[o] == 0 && claim[o] == (int)t) ? 1 : 0;
  }
  __device__ void emit(long long t, int, long long r0, long long, long long) const {
    int a, b, c;
    nbr(t, a, b, c);
    const long long pos = (long long)count0 - nlo + r0;
    ix[pos] = a;
    iy[pos] = b;
    iz[pos] = c;
  }
};

__global__ void k_bfs_claim(Bfs f, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int a, b, c;
  if (!f.nbr(t, a, b, c)) return;
  const long long o = f.cidx(a, b, c);
  if (f.nb.p[o] == 0) atomicMin(&f.claim[o], (int)t);
}

// after the compaction: mark the new cells and release their claims
__global__ void k_bfs_mark(Bfs f, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int a, b, c;
  if (!f.nbr(t, a, b, c)) return;
  const long long o = f.cidx(a, b, c);
  if (f.nb.p[o] == 0 && f.claim[o] == (int)t) {
    f.nb.p[o] = f.mark;
    f.claim[o] = INT_MAX;
  }
}

// Breadth-first levels 1..level from the lists already holding levels
// 0..(start-1); lo/hi are host copies of n_lo/n_hi, updated in place.
bool bfs_levels(Call &call, View<U8> nb, const Box &nbb, int *ix, int *iy, int *iz, int nlo, int nhi,
                std::vector<int> &lo, std::vector<int> &hi, int level) {
  int *claim = call.temp<int>(nbb.size());
  if (!call.ok()) return false;
  cudaMemsetAsync(claim, 0x7f, (size_t)nbb.size() * sizeof(int), stream());
  long long count = (long long)hi[0] + 1;
  for (int lv = 1; lv <= level; lv++) {
    // an empty parent level (-1, -1) yields an empty level; the reference
    // would index entry -1 here
    const long long np = (lo[lv - 1] >= 0 && hi[lv - 1] >= lo[lv - 1]) ? (long long)hi[lv - 1] - lo[lv - 1] + 1 : 0;
    long long added = 0;
    if (np > 0) {
      if (6 * np >= INT_MAX) {
        set_error(LSMGPU_ERR_CAPACITY, "narrow band level too large for 32-bit candidate keys");
        return false;
      }
      Bfs f{nb, nbb, claim, ix, iy, iz, nlo, lo[lv - 1], (int)count, (U8)(lv + 1)};
      const long long n = 6 * np;
      const unsigned g = (unsigned)((n + 255) / 256);
      LSMGPU_LAUNCH(k_bfs_claim, g, 256, 0, f, n);
      // the compaction writes list entries count .. count+added-1; check the
      // capacity against the worst case first
      if (count + n - 1 > nhi) {
        // exact count needed: count winners first
        long long tot[3];
        if (!compact(call, CountOnly<Bfs>{f}, n, tot)) return false;
        if (count + tot[0] - 1 > nhi) {
          set_error(LSMGPU_ERR_CAPACITY, "narrow band lists exceed nhi_index");
          return false;
        }
      }
      long long tot[3];
      if (!compact(call, f, n, tot)) return false;
      LSMGPU_LAUNCH(k_bfs_mark, g, 256, 0, f, n);
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


// Builds the band of `phi` (device arrays) inside `call`: level-0 lists,
// outer lists and `level` neighbour levels.  lo/hi receive n_lo/n_hi, ob the
// outer-list bounds {plus lo, plus hi, minus lo, minus hi}.  Returns false
// after recording an error (capacity or CUDA).
template <class T>
bool band_build(Call &call, const T *phi, const Box &gb, U8 *nbd, const Box &nbb, int *ix, int *iy, int *iz,
                int nlo, int nhi, int *outer, int nlo_outer, int nhi_outer, double width, double width_inner,
                int level, std::vector<int> &lo, std::vector<int> &hi, int ob[4], long long *level0_count) {
  const long long cap = (long long)nhi - nlo + 1;
  const long long ocap = (long long)nhi_outer - nlo_outer + 1;
  Level0T<T> z;
  z.phi = view(phi, gb);
  z.nb = view(nbd, nbb);
  z.gb = gb;
  z.nx = gb.n(0);
  z.nxy = gb.n(0) * gb.n(1);
  z.width = width;
  z.width_inner = width_inner;
  z.ix = ix; z.iy = iy; z.iz = iz;
  z.outer = outer;
  z.nlo = nlo;
  z.nlo_outer = nlo_outer;
  z.nhi_outer = nhi_outer;
  z.mode = 0;
  const long long n = gb.size();
  long long tot[3];
  if (!compact(call, CountOnly<Level0T<T>>{z}, n, tot)) return false;
  if (tot[0] > cap || tot[1] + tot[2] > ocap) {
    set_error(LSMGPU_ERR_CAPACITY, "narrow band (%lld cells) or outer layer (%lld) exceeds the index arrays", tot[0],
              tot[1] + tot[2]);
    return false;
  }
  LSMGPU_LAUNCH(k_mark0<T>, (unsigned)((n + 255) / 256), 256, 0, z, n);
  if (!compact(call, z, n, tot)) return false;
  lo.assign(level + 1, -1);
  hi.assign(level + 1, -1);
  lo[0] = nlo;
  ob[0] = nhi_outer; ob[1] = nhi_outer; ob[2] = nlo_outer; ob[3] = nlo_outer;
  if (level0_count) *level0_count = tot[0];
  if (tot[0] > 0) {
    hi[0] = (int)(nlo + tot[0] - 1);
    ob[2] = nlo_outer;
    ob[3] = (int)(nlo_outer + tot[1] - 1);
    ob[0] = (int)(nhi_outer - tot[2] + 1);
    ob[1] = nhi_outer;
    if (!bfs_levels(call, z.nb, nbb, ix, iy, iz, nlo, nhi, lo, hi, level)) return false;
  } else {
    hi[0] = nlo;  // localization3d.f:289-292
  }
  return true;
}

}  // namespace
}  // namespace lsmgpu
