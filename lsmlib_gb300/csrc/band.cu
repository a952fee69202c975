// Narrow-band construction (localization3d.f) on the GPU, bit-exact with the
// reference's serial order:
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
#include <climits>
#include <vector>

#include "lsmgpu_common.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

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
struct Level0 {
  View<const R> phi;      // over gb
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
    const R v = phi.p[e];
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

// every cell of phi's ghost box gets its level-0 mark (1 in the band, 0 out)
__global__ void k_mark0(Level0 z, long long n) {
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

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

void lsm3ddeterminenarrowband_(const R *phi, BOXARG(g), unsigned char *narrow_band, BOXARG(nb), int *index_x,
                               int *index_y, int *index_z, const int *nlo_index, const int *nhi_index,
                               int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer,
                               const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus,
                               int *nlo_outer_minus, int *nhi_outer_minus, const R *width,
                               const R *width_inner, const int *level) {
  Call call("lsm3ddeterminenarrowband_");
  Box gb = BOXOF(g), nbb = BOXOF(nb);
  if (!nbb.contains(gb, 0, 0, 0)) call.fail("narrow_band ghost box must cover phi's ghost box");
  if (*level < 0) call.fail("level must be >= 0");
  const long long cap = (long long)*nhi_index - *nlo_index + 1;
  const long long ocap = (long long)*nhi_index_outer - *nlo_index_outer + 1;
  if (cap <= 0 || ocap <= 0) call.fail("empty index arrays");
  if (!call.ok()) return;
  const R *phd = call.in(phi, gb.size());
  U8 *nbd = call.inout(narrow_band, nbb.size());
  int *ix = call.inout(index_x, cap), *iy = call.inout(index_y, cap), *iz = call.inout(index_z, cap);
  int *outer = call.inout(index_outer, ocap);
  if (!call.ok()) return;
  Level0 z;
  z.phi = view(phd, gb);
  z.nb = view(nbd, nbb);
  z.gb = gb;
  z.nx = gb.n(0);
  z.nxy = gb.n(0) * gb.n(1);
  z.width = *width;
  z.width_inner = *width_inner;
  z.ix = ix; z.iy = iy; z.iz = iz;
  z.outer = outer;
  z.nlo = *nlo_index;
  z.nlo_outer = *nlo_index_outer;
  z.nhi_outer = *nhi_index_outer;
  z.mode = 0;
  const long long n = gb.size();
  // count first so an overflow is reported before anything is written
  long long tot[3];
  if (!compact(call, CountOnly<Level0>{z}, n, tot)) return;
  if (tot[0] > cap || tot[1] + tot[2] > ocap) {
    set_error(LSMGPU_ERR_CAPACITY, "lsm3ddeterminenarrowband_: band (%lld cells) or outer layer (%lld) exceeds the index arrays",
              tot[0], tot[1] + tot[2]);
    return;
  }
  LSMGPU_LAUNCH(k_mark0, (unsigned)((n + 255) / 256), 256, 0, z, n);
  if (!compact(call, z, n, tot)) return;
  std::vector<int> lo(*level + 1, -1), hi(*level + 1, -1);
  lo[0] = *nlo_index;
  int ob[4] = {*nlo_index_outer, *nhi_index_outer, *nlo_index_outer, *nhi_index_outer};  // plus lo/hi, minus lo/hi
  if (tot[0] > 0) {
    hi[0] = (int)(*nlo_index + tot[0] - 1);
    ob[2] = *nlo_index_outer;
    ob[3] = (int)(*nlo_index_outer + tot[1] - 1);
    ob[0] = (int)(*nhi_index_outer - tot[2] + 1);
    ob[1] = *nhi_index_outer;
    if (!bfs_levels(call, z.nb, nbb, ix, iy, iz, *nlo_index, *nhi_index, lo, hi, *level)) return;
    put_ints(n_lo, lo.data(), *level + 1);
    put_ints(n_hi, hi.data(), *level + 1);
  } else {
    // no band cell (localization3d.f:289-292): deeper levels are not written
    const int z0 = *nlo_index;
    put_ints(n_lo, &z0, 1);
    put_ints(n_hi, &z0, 1);
    ob[2] = *nlo_index_outer;
    ob[3] = *nlo_index_outer;
    ob[0] = *nhi_index_outer;
    ob[1] = *nhi_index_outer;
  }
  put_ints(nlo_outer_plus, &ob[0], 1);
  put_ints(nhi_outer_plus, &ob[1], 1);
  put_ints(nlo_outer_minus, &ob[2], 1);
  put_ints(nhi_outer_minus, &ob[3], 1);
  call.finish();
}

void lsm3dmarknarrowbandneighbors_(unsigned char *narrow_band, BOXARG(nb), int *index_x, int *index_y,
                                   int *index_z, const int *nlo_index, const int *nhi_index, int *n_lo,
                                   int *n_hi, const int *level) {
  Call call("lsm3dmarknarrowbandneighbors_");
  Box nbb = BOXOF(nb);
  const long long cap = (long long)*nhi_index - *nlo_index + 1;
  if (cap <= 0 || *level < 0) call.fail("empty index arrays or negative level");
  if (!call.ok()) return;
  U8 *nbd = call.inout(narrow_band, nbb.size());
  int *ix = call.inout(index_x, cap), *iy = call.inout(index_y, cap), *iz = call.inout(index_z, cap);
  if (!call.ok()) return;
  std::vector<int> lo(*level + 1), hi(*level + 1);
  get_ints(lo.data(), n_lo, *level + 1);
  get_ints(hi.data(), n_hi, *level + 1);
  if (!bfs_levels(call, view(nbd, nbb), nbb, ix, iy, iz, *nlo_index, *nhi_index, lo, hi, *level)) return;
  put_ints(n_lo, lo.data(), *level + 1);
  put_ints(n_hi, hi.data(), *level + 1);
  call.finish();
}

void lsm3ddeterminenarrowbandfrommask_(const R *mask, BOXARG(g), unsigned char *narrow_band, BOXARG(nb),
                                       int *index_x, int *index_y, int *index_z, const int *nlo_index,
                                       const int *nhi_index, int *n_lo, int *n_hi, const int *level,
                                       const int *use_mask_sign) {
  Call call("lsm3ddeterminenarrowbandfrommask_");
  Box gb = BOXOF(g), nbb = BOXOF(nb);
  if (!nbb.contains(gb, 0, 0, 0)) call.fail("narrow_band ghost box must cover the mask's ghost box");
  const long long cap = (long long)*nhi_index - *nlo_index + 1;
  if (cap <= 0 || *level < 0) call.fail("empty index arrays or negative level");
  if (!call.ok()) return;
  const R *md = call.in(mask, gb.size());
  U8 *nbd = call.inout(narrow_band, nbb.size());
  int *ix = call.inout(index_x, cap), *iy = call.inout(index_y, cap), *iz = call.inout(index_z, cap);
  if (!call.ok()) return;
  Level0 z{};
  z.phi = view(md, gb);
  z.nb = view(nbd, nbb);
  z.gb = gb;
  z.nx = gb.n(0);
  z.nxy = gb.n(0) * gb.n(1);
  z.ix = ix; z.iy = iy; z.iz = iz;
  z.nlo = *nlo_index;
  z.mode = (*use_mask_sign > 0) ? 1 : 2;
  const long long n = gb.size();
  long long tot[3];
  if (!compact(call, CountOnly<Level0>{z}, n, tot)) return;
  if (tot[0] > cap) {
    set_error(LSMGPU_ERR_CAPACITY, "lsm3ddeterminenarrowbandfrommask_: band exceeds the index arrays");
    return;
  }
  LSMGPU_LAUNCH(k_mark0, (unsigned)((n + 255) / 256), 256, 0, z, n);
  if (!compact(call, z, n, tot)) return;
  std::vector<int> lo(*level + 1, -1), hi(*level + 1, -1);
  lo[0] = *nlo_index;
  hi[0] = (int)(*nlo_index + tot[0] - 1);
  if (!bfs_levels(call, z.nb, nbb, ix, iy, iz, *nlo_index, *nhi_index, lo, hi, *level)) return;
  put_ints(n_lo, lo.data(), *level + 1);
  put_ints(n_hi, hi.data(), *level + 1);
  call.finish();
}

}  // extern "C"

// ---- boundary layer marks and outer-layer check ------------------------------------
namespace lsmgpu {
namespace {
__global__ void k_face_fill(View<U8> nb, Box face, U8 mark) {
  LSMGPU_CELL_INDEX(face, i, j, k);
  nb(i, j, k) = mark;
}

// counts positive and non-positive phi over a stretch of index_outer
__global__ void k_outer_signs(View<const R> v, const int *ix, const int *iy, const int *iz, int nlo,
                              const int *outer, int obase, int lo, int hi, int *pos_neg) {
  const long long m = (long long)lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m > hi) return;
  const int l = outer[m - obase];
  const int i = ix[l - nlo], j = iy[l - nlo], k = iz[l - nlo];
  if (v(i, j, k) > R(0))
    atomicOr(&pos_neg[0], 1);
  else
    atomicOr(&pos_neg[1], 1);
}
}  // namespace
}  // namespace lsmgpu

extern "C" {

void lsm3dmarknarrowbandboundarylayer_(unsigned char *narrow_band, BOXARG(g), const int *ilo_fb,
                                       const int *ihi_fb, const int *jlo_fb, const int *jhi_fb,
                                       const int *klo_fb, const int *khi_fb,
                                       const unsigned char *mark_boundary_layer) {
  Call call("lsm3dmarknarrowbandboundarylayer_");
  Box gb = BOXOF(g);
  const int f[6] = {*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb};
  for (int a = 0; a < 6; a++)
    if (f[a] < gb.lo[a / 2] || f[a] > gb.hi[a / 2]) call.fail("fill-box face outside the ghost box");
  if (!call.ok()) return;
  View<U8> nb = view(call.inout(narrow_band, gb.size()), gb);
  if (!call.ok()) return;
  // the six faces in the reference's order (localization3d.f:328-374)
  for (int face = 0; face < 6; face++) {
    Box b = gb;
    b.lo[face / 2] = b.hi[face / 2] = f[face];
    Grid3 g3 = cover(b);
    LSMGPU_LAUNCH(k_face_fill, g3.grid, g3.block, 0, nb, b, *mark_boundary_layer);
  }
  call.finish();
}

void lsm3dcheckouternarrowbandlayer_(int *change_sign, const R *phi, BOXARG(g), const int *index_x,
                                     const int *index_y, const int *index_z, const int *nlo_index,
                                     const int *nhi_index, const int *index_outer, const int *nlo_index_outer,
                                     const int *nhi_index_outer, const int *nlo_outer_plus,
                                     const int *nhi_outer_plus, const int *nlo_outer_minus,
                                     const int *nhi_outer_minus) {
  Call call("lsm3dcheckouternarrowbandlayer_");
  Box gb = BOXOF(g);
  const long long cap = (long long)*nhi_index - *nlo_index + 1;
  const long long ocap = (long long)*nhi_index_outer - *nlo_index_outer + 1;
  if (cap <= 0 || ocap <= 0) call.fail("empty index arrays");
  if (!call.ok()) return;
  const R *ph = call.in(phi, gb.size());
  const int *ix = call.in(index_x, cap), *iy = call.in(index_y, cap), *iz = call.in(index_z, cap);
  const int *outer = call.in(index_outer, ocap);
  int *flags = call.temp<int>(4);
  if (!call.ok()) return;
  cudaMemsetAsync(flags, 0, 4 * sizeof(int), stream());
  // the reference stops at the first sign change in each list; whether a list
  // holds both signs does not depend on the visiting order
  const int lists[2][2] = {{*nlo_outer_plus, *nhi_outer_plus}, {*nlo_outer_minus, *nhi_outer_minus}};
  for (int q = 0; q < 2; q++) {
    const long long n = (long long)lists[q][1] - lists[q][0] + 1;
    if (n <= 0) continue;
    LSMGPU_LAUNCH(k_outer_signs, (unsigned)((n + 255) / 256), 256, 0, view(ph, gb), ix, iy, iz, *nlo_index, outer,
                  *nlo_index_outer, lists[q][0], lists[q][1], flags + 2 * q);
  }
  int h[4] = {0, 0, 0, 0};
  cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, stream());
  call.finish();
  cudaStreamSynchronize(stream());
  *change_sign = ((h[0] && h[1]) || (h[2] && h[3])) ? 1 : 0;
}

}  // extern "C"
