/*
 * CPU oracle, ghost-cell boundary conditions
 * (boundary_conditions3d.f:46-639).  TEST INFRASTRUCTURE ONLY.
 *
 * bdry_location_idx selects the face: 0/1 = x lower/upper, 2/3 = y, 4/5 = z.
 * Each face call fills every ghost layer of that face over the full ghost-box
 * extent of the other two axes.
 */
#include "oracle_common.h"

enum { EXTRAP_LINEAR, EXTRAP_SIGNED, EXTRAP_COPY };

static void extrapolate(real_t *phi, const gbox *g, const int fb[6], int face, int kind) {
  const int axis = face / 2, upper = face % 2;
  const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;
  const int edge = upper ? fb[2 * axis + 1] : fb[2 * axis];
  const int inner = upper ? edge - 1 : edge + 1;
  const int first = upper ? edge + 1 : g->lo[axis];
  const int last = upper ? g->hi[axis] : edge - 1;
  int c[3];
  for (int b = g->lo[o2]; b <= g->hi[o2]; b++)
    for (int a = g->lo[o1]; a <= g->hi[o1]; a++) {
      c[o1] = a;
      c[o2] = b;
      c[axis] = edge;
      const real_t e = phi[at(g, c[0], c[1], c[2])];
      c[axis] = inner;
      const real_t nx = phi[at(g, c[0], c[1], c[2])];
      real_t slope = 0.0;
      if (kind == EXTRAP_LINEAR) slope = e - nx;
      if (kind == EXTRAP_SIGNED) slope = copysign(1.0, e) * fabs(e - nx);
      for (int m = first; m <= last; m++) {
        c[axis] = m;
        if (kind == EXTRAP_COPY) {
          phi[at(g, c[0], c[1], c[2])] = e;
        } else {
          const real_t dist = (real_t)(upper ? m - edge : edge - m);
          phi[at(g, c[0], c[1], c[2])] = e + slope * dist;
        }
      }
    }
}

#define BC_ARGS                                                                \
  real_t *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb,        \
      const int *jhi_gb, const int *klo_gb, const int *khi_gb, const int *ilo_fb, \
      const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *klo_fb, \
      const int *khi_fb, const int *bdry_location_idx
#define BC_BODY(kind)                                                          \
  gbox g = mk_box(ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb);            \
  int fb[6] = {*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb};        \
  if (*bdry_location_idx < 0 || *bdry_location_idx > 5) return;              \
  extrapolate(phi, &g, fb, *bdry_location_idx, kind)

/* lsm3dLinearExtrapolation (boundary_conditions3d.f:46-169) */
void lsm3dlinearextrapolation_(BC_ARGS) { BC_BODY(EXTRAP_LINEAR); }
/* lsm3dSignedLinearExtrapolation (:193-337): slope = sign(1,phi_edge)*|diff| */
void lsm3dsignedlinearextrapolation_(BC_ARGS) { BC_BODY(EXTRAP_SIGNED); }
/* lsm3dCopyExtrapolation (:352-462) */
void lsm3dcopyextrapolation_(BC_ARGS) { BC_BODY(EXTRAP_COPY); }
/* lsm3dHomogeneousNeumannENO1/2/3/WENO5 (:486-638) are copy extrapolation */
void lsm3dhomogeneousneumanneno1_(BC_ARGS) { BC_BODY(EXTRAP_COPY); }
void lsm3dhomogeneousneumanneno2_(BC_ARGS) { BC_BODY(EXTRAP_COPY); }
void lsm3dhomogeneousneumanneno3_(BC_ARGS) { BC_BODY(EXTRAP_COPY); }
void lsm3dhomogeneousneumannweno5_(BC_ARGS) { BC_BODY(EXTRAP_COPY); }
