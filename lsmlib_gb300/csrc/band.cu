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

#include "band.cuh"
#include "../../include/lsmgpu_toolbox3d.h"

namespace lsmgpu {
namespace {
}  // namespace
}  // namespace lsmgpu

namespace lsmgpu {
namespace {

// lsm3dDetermineNarrowBand (localization3d.f:174-302) and the forms of its
// 2D relatives (BandForm): level 0 in sweep order, outer lists, neighbour levels
void determine_band(const char *name, const R *phi, const Box &gb, const R *second, unsigned char *narrow_band,
                    const Box &nbb, int *index_x, int *index_y, int *index_z, const int *nlo_index,
                    const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer,
                    const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus,
                    int *nhi_outer_minus, R width, R width_inner, int level, BandForm<R> form) {
  Call call(name);
  if (!nbb.contains(gb, 0, 0, 0)) call.fail("narrow_band ghost box must cover phi's ghost box");
  if (level < 0) call.fail("level must be >= 0");
  const long long cap = (long long)*nhi_index - *nlo_index + 1;
  const long long ocap = (long long)*nhi_index_outer - *nlo_index_outer + 1;
  if (cap <= 0 || ocap <= 0) call.fail("empty index arrays");
  if (!call.ok()) return;
  const R *phd = call.in(phi, gb.size());
  if (second) form.second = call.in(second, gb.size());
  U8 *nbd = call.inout(narrow_band, nbb.size());
  int *ix = call.inout(index_x, cap), *iy = call.inout(index_y, cap), *iz = call.inout(index_z, cap);
  int *outer = call.inout(index_outer, ocap);
  if (!call.ok()) return;
  std::vector<int> lo, hi;
  int ob[4];
  int nwrite = 1;
  if (!band_build<R>(call, phd, gb, nbd, nbb, ix, iy, iz, *nlo_index, *nhi_index, outer, *nlo_index_outer,
                     *nhi_index_outer, width, width_inner, level, lo, hi, ob, nullptr, new_claims(call, nbb), false,
                     form, &nwrite))
    return;
  put_ints(n_lo, lo.data(), nwrite);
  put_ints(n_hi, hi.data(), nwrite);
  put_ints(nlo_outer_plus, &ob[0], 1);
  put_ints(nhi_outer_plus, &ob[1], 1);
  put_ints(nlo_outer_minus, &ob[2], 1);
  put_ints(nhi_outer_minus, &ob[3], 1);
  call.finish();
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

#define BAND_TAIL                                                                                         \
  unsigned char *narrow_band, BOXARG(nb), int *index_x, int *index_y, int *index_z, const int *nlo_index,   \
      const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer,            \
      const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus,         \
      int *nhi_outer_minus, const R *width, const R *width_inner, const int *level
#define BAND_PASS                                                                                         \
  narrow_band, BOXOF(nb), index_x, index_y, index_z, nlo_index, nhi_index, n_lo, n_hi, index_outer,         \
      nlo_index_outer, nhi_index_outer, nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus,   \
      *width, *width_inner, *level

void lsm3ddeterminenarrowband_(const R *phi, BOXARG(g), BAND_TAIL) {
  determine_band("lsm3ddeterminenarrowband_", phi, BOXOF(g), nullptr, BAND_PASS, BandForm<R>());
}

// the bookkeeping of lsm2dDetermineNarrowBand (localization2d.f:225-240) on
// 3D arrays: n_hi(0) = count - 1 even for an empty band, neighbour levels
// only when level 0 holds two or more cells
void lsmgpu_determine_narrow_band_2d_bookkeeping(const R *phi, BOXARG(g), BAND_TAIL) {
  BandForm<R> f;
  f.bookkeeping = 1;
  determine_band("lsmgpu_determine_narrow_band_2d_bookkeeping", phi, BOXOF(g), nullptr, BAND_PASS, f);
}

// no 3D original; follows lsm2dDetermineNarrowBandFromTwoLevelSets
// (localization2d.f:248-343): level 0 = cells with |phi| < width and
// |psi| < width, outer lists by phi
void lsm3ddeterminenarrowbandfromtwolevelsets_(const R *phi, const R *psi, BOXARG(g), BAND_TAIL) {
  BandForm<R> f;
  f.l0_mode = 3;
  f.bookkeeping = 2;
  determine_band("lsm3ddeterminenarrowbandfromtwolevelsets_", phi, BOXOF(g), psi, BAND_PASS, f);
}

// no 3D original; follows lsm2dDetermineNarrowBandAwayFromMask
// (localization2d.f:365-464): level 0 = cells with |phi| < width and
// |phi - mask| > max(dx, dy, dz)
void lsm3ddeterminenarrowbandawayfrommask_(const R *phi, const R *mask, BOXARG(g), BAND_TAIL, const R *dx,
                                           const R *dy, const R *dz) {
  BandForm<R> f;
  f.l0_mode = 4;
  f.bookkeeping = 2;
  const R m = *dx > *dy ? *dx : *dy;
  f.max_dx = m > *dz ? m : *dz;
  determine_band("lsm3ddeterminenarrowbandawayfrommask_", phi, BOXOF(g), mask, BAND_PASS, f);
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
  if (!bfs_levels(call, view(nbd, nbb), nbb, ix, iy, iz, *nlo_index, *nhi_index, lo, hi, *level,
                  new_claims(call, nbb)))
    return;
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
  Compaction c0;
  if (!c0.count(call, z, n, tot)) return;
  if (tot[0] > cap) {
    set_error(LSMGPU_ERR_CAPACITY, "lsm3ddeterminenarrowbandfrommask_: band exceeds the index arrays");
    return;
  }
  LSMGPU_LAUNCH(k_mark0, dim3((unsigned)((gb.n(0) + 31) / 32), (unsigned)((gb.n(1) + 7) / 8),
                             (unsigned)((gb.n(2) + kMarkZ - 1) / kMarkZ)),
                dim3(32, 8), 0, z);
  c0.emit(z);
  std::vector<int> lo(*level + 1, -1), hi(*level + 1, -1);
  lo[0] = *nlo_index;
  hi[0] = (int)(*nlo_index + tot[0] - 1);
  if (!bfs_levels(call, z.nb, nbb, ix, iy, iz, *nlo_index, *nhi_index, lo, hi, *level, new_claims(call, nbb)))
    return;
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
  // the six faces in the reference's order (localization3d.f:328-374); a 2D
  // call (lifted) has the four x and y faces only (localization2d.f)
  for (int face = 0; face < 2 * g_lift_dims; face++) {
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
