/*
 * CPU oracle, narrow-band (index-list) kernels and band construction.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_common.h).  Restates LSMLIB's
 * *_local.f(.in) routines and lsm_localization3d.f.  Conventions kept from the
 * reference:
 *  - index lists are declared index_x(nlo:nhi) with the routine's first lower
 *    bound, so list entry l sits at element l - nlo of the array passed in;
 *  - a cell takes part when narrow_band(i,j,k) <= mark (narrow_band is
 *    INTEGER*1, compared signed);
 *  - the local derivative routines fill the scratch array D1 (D2, D3) over
 *    the listed cells first (value 1e10 where the cell's mark exceeds the
 *    scratch mark) and then read it, exactly as the reference does, so their
 *    results depend on the scratch contents in the same way.
 */
#include "oracle_common.h"

typedef signed char mark_t;

#define LIST_ARGS const int *ix, const int *iy, const int *iz
#define NB_ARGS                                                            \
  const mark_t *nb, const int *nb_ilo, const int *nb_ihi, const int *nb_jlo, \
      const int *nb_jhi, const int *nb_klo, const int *nb_khi
#define NBBOX mk_box(nb_ilo, nb_ihi, nb_jlo, nb_jhi, nb_klo, nb_khi)
#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,             \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi
#define B3(n) mk_box(n##_ilo, n##_ihi, n##_jlo, n##_jhi, n##_klo, n##_khi)
#define DX_ARGS const real_t *dx, const real_t *dy, const real_t *dz

/* Cells outside an array's ghost box, or whose stencil would leave it, are
 * skipped: LSMLIB reads outside its arrays there (undefined behaviour), and
 * the GPU library skips the same cells. */
static int inb(const gbox *b, int i, int j, int k) {
  return i >= b->lo[0] && i <= b->hi[0] && j >= b->lo[1] && j <= b->hi[1] && k >= b->lo[2] &&
         k <= b->hi[2];
}
/* cell c with c-lo..c+hi along `axis` inside b */
static int inb_axis(const gbox *b, int axis, int lo, int hi, int i, int j, int k) {
  int c[3] = {i, j, k};
  for (int a = 0; a < 3; a++) {
    int l = (a == axis) ? lo : 0, h = (a == axis) ? hi : 0;
    if (c[a] - l < b->lo[a] || c[a] + h > b->hi[a]) return 0;
  }
  return 1;
}
/* cell with a reach of r on every axis inside b */
static int inb_r(const gbox *b, int r, int i, int j, int k) {
  return inb_axis(b, 0, r, r, i, j, k) && inb_axis(b, 1, r, r, i, j, k) && inb_axis(b, 2, r, r, i, j, k);
}

/* iterate list entries l = lo..hi of lists declared from `decl` */
#define FOR_LIST(decl, lo, hi)                                       \
  for (int l = (lo); l <= (hi); l++)                                   \
    for (int i = ix[l - (decl)], j = iy[l - (decl)], k = iz[l - (decl)], \
             once_ = 1; once_; once_ = 0)

/* ---- undivided differences over a list (spatial_derivatives3d_local.f.in:43-138) */
static void dn_local(real_t *dn, const gbox *db, const real_t *dm, const gbox *mb, int n, int dir,
                     const int *ix, const int *iy, const int *iz, int decl, int lo, int hi,
                     const mark_t *nb, const gbox *nbb, mark_t mark) {
  int off[3] = {0, 0, 0};
  real_t sgn;
  if (n % 2 == 1) {
    off[dir] = 1;
    sgn = 1.0;
  } else {
    off[dir] = -1;
    sgn = -1.0;
  }
  FOR_LIST(decl, lo, hi) {
    if (!inb(db, i, j, k) || !inb_axis(mb, dir, n % 2 == 1 ? 1 : 0, n % 2 == 1 ? 0 : 1, i, j, k) ||
        !inb(nbb, i, j, k))
      continue;
    if (nb[at(nbb, i, j, k)] <= mark)
      dn[at(db, i, j, k)] =
          sgn * (dm[at(mb, i, j, k)] - dm[at(mb, i - off[0], j - off[1], k - off[2])]);
    else
      dn[at(db, i, j, k)] = 1.0e10;
  }
}

void lsm3dcomputednlocal_(real_t *dn, A3(d), const real_t *dm, A3(m), const int *n, const int *dir,
                          LIST_ARGS, const int *nlo, const int *nhi, NB_ARGS, const mark_t *mark_fb) {
  gbox D = B3(d), M = B3(m), NB = NBBOX;
  dn_local(dn, &D, dm, &M, *n, *dir - 1, ix, iy, iz, *nlo, *nlo, *nhi, nb, &NB, *mark_fb);
}

#define PM_ARGS                                                                \
  real_t *pxp, real_t *pyp, real_t *pzp, A3(p), real_t *pxm, real_t *pym,      \
      real_t *pzm, A3(m), const real_t *phi, A3(f)
#define PM_SETUP                                                              \
  gbox P = B3(p), M = B3(m), F = B3(f), NB = NBBOX;                          \
  real_t *pp[3] = {pxp, pyp, pzp}, *pm[3] = {pxm, pym, pzm};                 \
  const real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz};                   \
  (void)F;

static long sh(const gbox *b, int dir, int s) { return (long)s * b->s[dir]; }

/* lsm3dHJENO1LOCAL (spatial_derivatives3d_local.f.in:170-381) */
void lsm3dhjeno1local_(PM_ARGS, real_t *d1, A3(d1), DX_ARGS, LIST_ARGS, const int *nlo0,
                       const int *nhi0, const int *nlo1, const int *nhi1, NB_ARGS,
                       const mark_t *mark_fb, const mark_t *mark_d1) {
  PM_SETUP
  gbox D1 = B3(d1);
  for (int d = 0; d < 3; d++) {
    dn_local(d1, &D1, phi, &F, 1, d, ix, iy, iz, *nlo0, *nlo0, *nhi1, nb, &NB, *mark_d1);
    FOR_LIST(*nlo0, *nlo0, *nhi0) {
      if (!inb(&P, i, j, k) || !inb(&M, i, j, k) || !inb(&NB, i, j, k) ||
          !inb_axis(&D1, d, 0, 1, i, j, k))
        continue;
      if (nb[at(&NB, i, j, k)] <= *mark_fb) {
        long c = at(&D1, i, j, k);
        pp[d][at(&P, i, j, k)] = d1[c + sh(&D1, d, 1)] * inv[d];
        pm[d][at(&M, i, j, k)] = d1[c] * inv[d];
      }
    }
  }
}

/* lsm3dHJENO2LOCAL (spatial_derivatives3d_local.f.in:414-735) */
void lsm3dhjeno2local_(PM_ARGS, real_t *d1, A3(d1), real_t *d2, A3(d2), DX_ARGS, LIST_ARGS,
                       const int *nlo0, const int *nhi0, const int *nlo1, const int *nhi1,
                       const int *nlo2, const int *nhi2, NB_ARGS, const mark_t *mark_fb,
                       const mark_t *mark_d1, const mark_t *mark_d2) {
  PM_SETUP
  gbox D1 = B3(d1), D2 = B3(d2);
  for (int d = 0; d < 3; d++) {
    dn_local(d1, &D1, phi, &F, 1, d, ix, iy, iz, *nlo0, *nlo0, *nhi2, nb, &NB, *mark_d1);
    dn_local(d2, &D2, d1, &D1, 2, d, ix, iy, iz, *nlo0, *nlo0, *nhi1, nb, &NB, *mark_d2);
    FOR_LIST(*nlo0, *nlo0, *nhi0) {
      if (!inb(&P, i, j, k) || !inb(&M, i, j, k) || !inb(&NB, i, j, k) ||
          !inb_axis(&D1, d, 0, 1, i, j, k) || !inb_axis(&D2, d, 1, 1, i, j, k))
        continue;
      if (nb[at(&NB, i, j, k)] <= *mark_fb) {
        long a = at(&D1, i, j, k), b = at(&D2, i, j, k);
        long s1 = sh(&D1, d, 1), s2 = sh(&D2, d, 1);
        real_t c = (fabs(d2[b]) < fabs(d2[b + s2])) ? d2[b] : d2[b + s2];
        pp[d][at(&P, i, j, k)] = (d1[a + s1] - 0.5 * c) * inv[d];
        c = (fabs(d2[b - s2]) < fabs(d2[b])) ? d2[b - s2] : d2[b];
        pm[d][at(&M, i, j, k)] = (d1[a] + 0.5 * c) * inv[d];
      }
    }
  }
}

/* 3D upwind HJ ENO2 on a band.  LSMLIB has no 3D version; this follows the
 * 2D lsm2dUpwindHJENO2LOCAL (spatial_derivatives2d_local.f.in:1160-1390):
 * D1 over levels 0-2, D2 over 0-1, then on level-0 cells 0 where
 * |vel| < zero_tol, the minus-side ENO2 value where vel > 0, the plus side
 * otherwise. */
void lsm3dupwindhjeno2local_(real_t *gx, real_t *gy, real_t *gz, A3(g), const real_t *phi, A3(f),
                             const real_t *vx, const real_t *vy, const real_t *vz, A3(v), real_t *d1,
                             A3(d1), real_t *d2, A3(d2), DX_ARGS, LIST_ARGS, const int *nlo0,
                             const int *nhi0, const int *nlo1, const int *nhi1, const int *nlo2,
                             const int *nhi2, NB_ARGS, const mark_t *mark_fb, const mark_t *mark_d1,
                             const mark_t *mark_d2) {
  gbox G = B3(g), F = B3(f), V = B3(v), NB = NBBOX, D1 = B3(d1), D2 = B3(d2);
  real_t *out[3] = {gx, gy, gz};
  const real_t *vel[3] = {vx, vy, vz};
  const real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz};
  (void)nlo1;
  for (int d = 0; d < 3; d++) {
    dn_local(d1, &D1, phi, &F, 1, d, ix, iy, iz, *nlo0, *nlo0, *nhi2, nb, &NB, *mark_d1);
    dn_local(d2, &D2, d1, &D1, 2, d, ix, iy, iz, *nlo0, *nlo0, *nhi1, nb, &NB, *mark_d2);
    FOR_LIST(*nlo0, *nlo0, *nhi0) {
      if (!inb(&G, i, j, k) || !inb(&V, i, j, k) || !inb(&NB, i, j, k) ||
          !inb_axis(&D1, d, 0, 1, i, j, k) || !inb_axis(&D2, d, 1, 1, i, j, k))
        continue;
      if (nb[at(&NB, i, j, k)] > *mark_fb) continue;
      real_t u = vel[d][at(&V, i, j, k)];
      long a = at(&D1, i, j, k), b = at(&D2, i, j, k);
      long s1 = sh(&D1, d, 1), s2 = sh(&D2, d, 1);
      real_t r;
      if (fabs(u) < ORACLE_ZERO_TOL) {
        r = 0.0;
      } else if (u > 0.0) {
        real_t c = (fabs(d2[b - s2]) < fabs(d2[b])) ? d2[b - s2] : d2[b];
        r = (d1[a] + 0.5 * c) * inv[d];
      } else {
        real_t c = (fabs(d2[b]) < fabs(d2[b + s2])) ? d2[b] : d2[b + s2];
        r = (d1[a + s1] - 0.5 * c) * inv[d];
      }
      out[d][at(&G, i, j, k)] = r;
    }
  }
}

/* 3D HJ ENO3 on a band.  LSMLIB has no 3D version; this follows the 2D
 * lsm2dHJENO3LOCAL (spatial_derivatives2d_local.f.in:498-813): D1 over levels
 * 0-3, D2 over 0-2, D3 over 0-1, then the dense ENO3 selection
 * (spatial_derivatives3d.f.in:842-896) on level-0 cells. */
void lsm3dhjeno3local_(PM_ARGS, real_t *d1, A3(d1), real_t *d2, A3(d2), real_t *d3, A3(d3),
                       DX_ARGS, LIST_ARGS, const int *nlo0, const int *nhi0, const int *nlo1,
                       const int *nhi1, const int *nlo2, const int *nhi2, const int *nlo3,
                       const int *nhi3, NB_ARGS, const mark_t *mark_fb, const mark_t *mark_d1,
                       const mark_t *mark_d2, const mark_t *mark_d3) {
  PM_SETUP
  gbox D1 = B3(d1), D2 = B3(d2), D3 = B3(d3);
  const real_t third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  for (int d = 0; d < 3; d++) {
    dn_local(d1, &D1, phi, &F, 1, d, ix, iy, iz, *nlo0, *nlo0, *nhi3, nb, &NB, *mark_d1);
    dn_local(d2, &D2, d1, &D1, 2, d, ix, iy, iz, *nlo0, *nlo0, *nhi2, nb, &NB, *mark_d2);
    dn_local(d3, &D3, d2, &D2, 3, d, ix, iy, iz, *nlo0, *nlo0, *nhi1, nb, &NB, *mark_d3);
    FOR_LIST(*nlo0, *nlo0, *nhi0) {
      if (!inb(&P, i, j, k) || !inb(&M, i, j, k) || !inb(&NB, i, j, k) ||
          !inb_axis(&D1, d, 0, 1, i, j, k) || !inb_axis(&D2, d, 1, 1, i, j, k) ||
          !inb_axis(&D3, d, 1, 2, i, j, k))
        continue;
      if (nb[at(&NB, i, j, k)] > *mark_fb) continue;
      long a = at(&D1, i, j, k), b = at(&D2, i, j, k), c3 = at(&D3, i, j, k);
      long s1 = sh(&D1, d, 1), s2 = sh(&D2, d, 1), s3 = sh(&D3, d, 1);
      real_t x = d1[a + s1];
      if (fabs(d2[b]) < fabs(d2[b + s2])) {
        x = x - 0.5 * d2[b];
        x = (fabs(d3[c3]) < fabs(d3[c3 + s3])) ? x - sixth * d3[c3] : x - sixth * d3[c3 + s3];
      } else {
        x = x - 0.5 * d2[b + s2];
        x = (fabs(d3[c3 + s3]) < fabs(d3[c3 + 2 * s3])) ? x + third * d3[c3 + s3]
                                                        : x + third * d3[c3 + 2 * s3];
      }
      pp[d][at(&P, i, j, k)] = x * inv[d];
      x = d1[a];
      if (fabs(d2[b - s2]) < fabs(d2[b])) {
        x = x + 0.5 * d2[b - s2];
        x = (fabs(d3[c3 - s3]) < fabs(d3[c3])) ? x + third * d3[c3 - s3] : x + third * d3[c3];
      } else {
        x = x + 0.5 * d2[b];
        x = (fabs(d3[c3]) < fabs(d3[c3 + s3])) ? x - sixth * d3[c3] : x - sixth * d3[c3 + s3];
      }
      pm[d][at(&M, i, j, k)] = x * inv[d];
    }
  }
}

/* WENO5 with the local routines' smaller epsilon floor 1e-35
 * (spatial_derivatives2d_local.f.in:892). */
static real_t weno5_local(real_t v1, real_t v2, real_t v3, real_t v4, real_t v5) {
  const real_t c13 = 1.0 / 3.0, c76 = 7.0 / 6.0, c116 = 11.0 / 6.0;
  const real_t c16 = 1.0 / 6.0, c56 = 5.0 / 6.0, c1312 = 13.0 / 12.0, c14 = 0.25;
  real_t m = v1 * v1;
  m = fmax2(m, v2 * v2);
  m = fmax2(m, v3 * v3);
  m = fmax2(m, v4 * v4);
  m = fmax2(m, v5 * v5);
  real_t eps = 1e-6 * m + 1.e-35;
  real_t p1 = c13 * v1 - c76 * v2 + c116 * v3;
  real_t p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  real_t p3 = c13 * v3 + c56 * v4 - c16 * v5;
  real_t t = v1 - 2.0 * v2 + v3, u = v1 - 4.0 * v2 + 3.0 * v3;
  real_t S1 = c1312 * (t * t) + c14 * (u * u);
  t = v2 - 2.0 * v3 + v4;
  u = v2 - v4;
  real_t S2 = c1312 * (t * t) + c14 * (u * u);
  t = v3 - 2.0 * v4 + v5;
  u = 3.0 * v3 - 4.0 * v4 + v5;
  real_t S3 = c1312 * (t * t) + c14 * (u * u);
  real_t a1 = 0.1 / ((S1 + eps) * (S1 + eps));
  real_t a2 = 0.6 / ((S2 + eps) * (S2 + eps));
  real_t a3 = 0.3 / ((S3 + eps) * (S3 + eps));
  real_t is = 1.0 / (a1 + a2 + a3);
  a1 = a1 * is;
  a2 = a2 * is;
  a3 = a3 * is;
  return a1 * p1 + a2 * p2 + a3 * p3;
}

/* 3D HJ WENO5 on a band.  LSMLIB has no 3D version; this follows the 2D
 * lsm2dHJWENO5LOCAL (spatial_derivatives2d_local.f.in:816-1154): D1 over
 * levels 0-3 (mark_D1), then the WENO5 plus/minus reconstruction on level-0
 * cells (mark_fb). */
void lsm3dhjweno5local_(PM_ARGS, real_t *d1, A3(d1), DX_ARGS, LIST_ARGS, const int *nlo0,
                        const int *nhi0, const int *nlo1, const int *nhi1, const int *nlo2,
                        const int *nhi2, const int *nlo3, const int *nhi3, NB_ARGS,
                        const mark_t *mark_fb, const mark_t *mark_d1) {
  PM_SETUP
  gbox D1 = B3(d1);
  for (int d = 0; d < 3; d++) {
    dn_local(d1, &D1, phi, &F, 1, d, ix, iy, iz, *nlo0, *nlo0, *nhi3, nb, &NB, *mark_d1);
    const long s = sh(&D1, d, 1);
    FOR_LIST(*nlo0, *nlo0, *nhi0) {
      if (!inb(&P, i, j, k) || !inb(&M, i, j, k) || !inb(&NB, i, j, k) ||
          !inb_axis(&D1, d, 2, 3, i, j, k))
        continue;
      if (nb[at(&NB, i, j, k)] > *mark_fb) continue;
      long c = at(&D1, i, j, k);
      real_t w = inv[d];
      pp[d][at(&P, i, j, k)] = weno5_local(d1[c + 3 * s] * w, d1[c + 2 * s] * w, d1[c + s] * w,
                                           d1[c] * w, d1[c - s] * w);
      pm[d][at(&M, i, j, k)] = weno5_local(d1[c - 2 * s] * w, d1[c - s] * w, d1[c] * w,
                                           d1[c + s] * w, d1[c + 2 * s] * w);
    }
  }
}

#define LOCAL_TAIL LIST_ARGS, const int *nlo, const int *nhi, NB_ARGS, const mark_t *mark_fb
#define GATE (inb(&NB, i, j, k) && nb[at(&NB, i, j, k)] <= *mark_fb)

/* lsm3dCentralGradOrder2LOCAL (spatial_derivatives3d_local.f.in:763-848) */
void lsm3dcentralgradorder2local_(real_t *px, real_t *py, real_t *pz, A3(g), const real_t *phi,
                                  A3(f), DX_ARGS, LOCAL_TAIL) {
  gbox G = B3(g), F = B3(f), NB = NBBOX;
  real_t fac[3] = {0.5 / *dx, 0.5 / *dy, 0.5 / *dz};
  real_t *o[3] = {px, py, pz};
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&G, i, j, k) && inb_r(&F, 1, i, j, k))) continue;
    const real_t *c = phi + at(&F, i, j, k);
    for (int d = 0; d < 3; d++) o[d][at(&G, i, j, k)] = (c[F.s[d]] - c[-F.s[d]]) * fac[d];
  }
}

/* lsm3dCentralGradOrder4LOCAL (:868-962) */
void lsm3dcentralgradorder4local_(real_t *px, real_t *py, real_t *pz, A3(g), const real_t *phi,
                                  A3(f), DX_ARGS, LOCAL_TAIL) {
  gbox G = B3(g), F = B3(f), NB = NBBOX;
  const real_t c12 = 0.0833333333333333333333;
  real_t fac[3] = {c12 / *dx, c12 / *dy, c12 / *dz};
  real_t *o[3] = {px, py, pz};
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&G, i, j, k) && inb_r(&F, 2, i, j, k))) continue;
    const real_t *c = phi + at(&F, i, j, k);
    for (int d = 0; d < 3; d++) {
      long s = F.s[d];
      o[d][at(&G, i, j, k)] = (-c[2 * s] + 8.0 * c[s] + c[-2 * s] - 8.0 * c[-s]) * fac[d];
    }
  }
}

/* lsm3dLaplacianOrder2LOCAL (:982-1066) */
void lsm3dlaplacianorder2local_(real_t *lap, A3(g), const real_t *phi, A3(f), DX_ARGS,
                                LOCAL_TAIL) {
  gbox G = B3(g), F = B3(f), NB = NBBOX;
  real_t a = 1.0 / *dx / *dx, b = 1.0 / *dy / *dy, e = 1.0 / *dz / *dz;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&G, i, j, k) && inb_r(&F, 1, i, j, k))) continue;
    const real_t *c = phi + at(&F, i, j, k);
    long sx = F.s[0], sy = F.s[1], sz = F.s[2];
    lap[at(&G, i, j, k)] = a * (c[sx] - 2.0 * c[0] + c[-sx]) + b * (c[sy] - 2.0 * c[0] + c[-sy]) +
                           e * (c[sz] - 2.0 * c[0] + c[-sz]);
  }
}

/* lsm3dComputeAveGradPhiLocal (:1089-1169): serial sum of |grad phi| */
void lsm3dcomputeavegradphilocal_(real_t *ave, const real_t *phi, A3(f), DX_ARGS, LOCAL_TAIL) {
  gbox F = B3(f), NB = NBBOX;
  real_t fac[3] = {0.5 / *dx, 0.5 / *dy, 0.5 / *dz};
  real_t s = 0.0;
  int count = 0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb_r(&F, 1, i, j, k))) continue;
    const real_t *c = phi + at(&F, i, j, k);
    real_t g[3];
    for (int d = 0; d < 3; d++) g[d] = (c[F.s[d]] - c[-F.s[d]]) * fac[d];
    s = s + sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    count++;
  }
  if (count > 0) s = s / (real_t)count;
  *ave = s;
}

/* lsm3dGradientMagnitudeLocal (:1186-1278): clamps at zero_tol, unlike the
 * dense routine's 1e-8 */
void lsm3dgradientmagnitudelocal_(const real_t *px, const real_t *py, const real_t *pz,
                                  real_t *mag, A3(g), LOCAL_TAIL) {
  gbox G = B3(g), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&G, i, j, k))) continue;
    long c = at(&G, i, j, k);
    real_t x2 = px[c] * px[c], y2 = py[c] * py[c], z2 = pz[c] * pz[c];
    if (x2 < ORACLE_ZERO_TOL) x2 = 0.0;
    if (y2 < ORACLE_ZERO_TOL) y2 = 0.0;
    if (z2 < ORACLE_ZERO_TOL) z2 = 0.0;
    real_t t = sqrt(x2 + y2 + z2);
    mag[c] = (t < ORACLE_ZERO_TOL) ? 0.0 : t;
  }
}

/* ---- RK stages over lists (tvd_runge_kutta3d_local.f) ------------------- */
void lsm3drk1steplocal_(real_t *un, A3(a), const real_t *u, A3(b), const real_t *rhs, A3(c),
                        const real_t *dt, LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), C = B3(c), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (GATE && inb(&A, i, j, k) && inb(&B, i, j, k) && inb(&C, i, j, k))
      un[at(&A, i, j, k)] = u[at(&B, i, j, k)] + *dt * rhs[at(&C, i, j, k)];
  }
}
void lsm3dtvdrk2stage1local_(real_t *un, A3(a), const real_t *u, A3(b), const real_t *rhs, A3(c),
                             const real_t *dt, LOCAL_TAIL) {
  lsm3drk1steplocal_(un, BOX6(a), u, BOX6(b), rhs, BOX6(c), dt, ix, iy, iz, nlo, nhi, nb, nb_ilo,
                     nb_ihi, nb_jlo, nb_jhi, nb_klo, nb_khi, mark_fb);
}
void lsm3dtvdrk3stage1local_(real_t *un, A3(a), const real_t *u, A3(b), const real_t *rhs, A3(c),
                             const real_t *dt, LOCAL_TAIL) {
  lsm3drk1steplocal_(un, BOX6(a), u, BOX6(b), rhs, BOX6(c), dt, ix, iy, iz, nlo, nhi, nb, nb_ilo,
                     nb_ihi, nb_jlo, nb_jhi, nb_klo, nb_khi, mark_fb);
}
void lsm3dtvdrk2stage2local_(real_t *un, A3(a), const real_t *u1, A3(b), const real_t *u, A3(c),
                             const real_t *rhs, A3(d), const real_t *dt, LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), C = B3(c), D = B3(d), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (GATE && inb(&A, i, j, k) && inb(&B, i, j, k) && inb(&C, i, j, k) && inb(&D, i, j, k))
      un[at(&A, i, j, k)] =
          0.5 * (u[at(&C, i, j, k)] + u1[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
  }
}
void lsm3dtvdrk3stage2local_(real_t *u2, A3(a), const real_t *u1, A3(b), const real_t *u, A3(c),
                             const real_t *rhs, A3(d), const real_t *dt, LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), C = B3(c), D = B3(d), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (GATE && inb(&A, i, j, k) && inb(&B, i, j, k) && inb(&C, i, j, k) && inb(&D, i, j, k))
      u2[at(&A, i, j, k)] = 0.75 * u[at(&C, i, j, k)] +
                            0.25 * (u1[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
  }
}
void lsm3dtvdrk3stage3local_(real_t *un, A3(a), const real_t *u2, A3(b), const real_t *u, A3(c),
                             const real_t *rhs, A3(d), const real_t *dt, LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), C = B3(c), D = B3(d), NB = NBBOX;
  const real_t c13 = 1.0 / 3.0, c23 = 2.0 / 3.0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (GATE && inb(&A, i, j, k) && inb(&B, i, j, k) && inb(&C, i, j, k) && inb(&D, i, j, k))
      un[at(&A, i, j, k)] = c13 * u[at(&C, i, j, k)] +
                            c23 * (u2[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
  }
}

/* ---- LSE right-hand sides over lists (level_set_evolution3d_local.f.in) - */
void lsm3dzerooutlevelseteqnrhslocal_(real_t *rhs, A3(r), LIST_ARGS, const int *nlo,
                                      const int *nhi) {
  gbox R = B3(r);
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (inb(&R, i, j, k)) rhs[at(&R, i, j, k)] = 0.0; /* no mark test (:44-50) */
  }
}

void lsm3daddadvectiontermtolserhslocal_(real_t *rhs, A3(r), const real_t *px, const real_t *py,
                                         const real_t *pz, A3(g), const real_t *vx,
                                         const real_t *vy, const real_t *vz, A3(v), LOCAL_TAIL) {
  gbox R = B3(r), G = B3(g), V = B3(v), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&R, i, j, k) && inb(&G, i, j, k) && inb(&V, i, j, k))) continue;
    long r = at(&R, i, j, k), g = at(&G, i, j, k), v = at(&V, i, j, k);
    rhs[r] = rhs[r] - (vx[v] * px[g] + vy[v] * py[g] + vz[v] * pz[g]);
  }
}

static real_t godunov_sq(real_t vn, real_t xp, real_t yp, real_t zp, real_t xm, real_t ym,
                         real_t zm) {
  const real_t p[3] = {xp, yp, zp}, m[3] = {xm, ym, zm};
  real_t s = 0.0;
  for (int d = 0; d < 3; d++) {
    real_t a = (vn > 0.0) ? fmax2(m[d], 0.0) : fmin2(m[d], 0.0);
    real_t b = (vn > 0.0) ? fmin2(p[d], 0.0) : fmax2(p[d], 0.0);
    real_t t = fmax2(a * a, b * b);
    s = (d == 0) ? t : s + t;
  }
  return s;
}

void lsm3daddnormalveltermtolserhslocal_(real_t *rhs, A3(r), const real_t *pxp, const real_t *pyp,
                                         const real_t *pzp, A3(p), const real_t *pxm,
                                         const real_t *pym, const real_t *pzm, A3(m),
                                         const real_t *vn, A3(v), LOCAL_TAIL) {
  gbox R = B3(r), P = B3(p), M = B3(m), V = B3(v), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&R, i, j, k) && inb(&P, i, j, k) && inb(&M, i, j, k) && inb(&V, i, j, k))) continue;
    real_t w = vn[at(&V, i, j, k)];
    long a = at(&P, i, j, k), b = at(&M, i, j, k), r = at(&R, i, j, k);
    real_t s = godunov_sq(w, pxp[a], pyp[a], pzp[a], pxm[b], pym[b], pzm[b]);
    if (fabs(w) >= ORACLE_ZERO_TOL) rhs[r] = rhs[r] - w * sqrt(s);
  }
}

void lsm3daddconstnormalveltermtolserhslocal_(real_t *rhs, A3(r), const real_t *pxp,
                                              const real_t *pyp, const real_t *pzp, A3(p),
                                              const real_t *pxm, const real_t *pym,
                                              const real_t *pzm, A3(m), const real_t *vel_n,
                                              LOCAL_TAIL) {
  gbox R = B3(r), P = B3(p), M = B3(m), NB = NBBOX;
  real_t w = *vel_n;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&R, i, j, k) && inb(&P, i, j, k) && inb(&M, i, j, k))) continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k), r = at(&R, i, j, k);
    real_t s = godunov_sq(w, pxp[a], pyp[a], pzp[a], pxm[b], pym[b], pzm[b]);
    if (fabs(w) >= ORACLE_ZERO_TOL) rhs[r] = rhs[r] - w * sqrt(s);
  }
}

static real_t curv_num(real_t xx, real_t yy, real_t zz, real_t xy, real_t xz, real_t yz, real_t x,
                       real_t y, real_t z) {
  return xx * y * y + yy * x * x - 2.0 * xy * x * y + xx * z * z + zz * x * x -
         2.0 * xz * x * z + yy * z * z + zz * y * y - 2.0 * yz * y * z;
}

void lsm3daddconstcurvtermtolserhslocal_(real_t *rhs, A3(r), const real_t *px, const real_t *py,
                                         const real_t *pz, A3(g), const real_t *pxx,
                                         const real_t *pxy, const real_t *pxz, const real_t *pyy,
                                         const real_t *pyz, const real_t *pzz, A3(h),
                                         const real_t *b, LOCAL_TAIL) {
  gbox R = B3(r), G = B3(g), H = B3(h), NB = NBBOX;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&R, i, j, k) && inb(&G, i, j, k) && inb(&H, i, j, k))) continue;
    long g = at(&G, i, j, k), h = at(&H, i, j, k), r = at(&R, i, j, k);
    real_t m2 = px[g] * px[g] + py[g] * py[g] + pz[g] * pz[g];
    real_t curv = 0.0;
    if (!(m2 < ORACLE_ZERO_TOL))
      curv = curv_num(pxx[h], pyy[h], pzz[h], pxy[h], pxz[h], pyz[h], px[g], py[g], pz[g]) / m2;
    rhs[r] = rhs[r] + *b * curv;
  }
}

/* ---- reinitialization over lists (reinitialization3d_local.f.in:50-324) */
void lsm3dcomputereinitializationeqnrhslocal_(
    real_t *rhs, A3(r), const real_t *phi, A3(f), const real_t *phi0, A3(z), const real_t *pxp,
    const real_t *pyp, const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
    const real_t *pzm, A3(m), DX_ARGS, const int *use_phi0_for_sgn, LOCAL_TAIL) {
  gbox R = B3(r), F = B3(f), Z = B3(z), P = B3(p), M = B3(m), NB = NBBOX;
  real_t dx_sq = fmax2(fmax2(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  const int use0 = (*use_phi0_for_sgn == 1);
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&R, i, j, k) && inb(use0 ? &Z : &F, i, j, k) && inb(&P, i, j, k) && inb(&M, i, j, k))) continue;
    real_t pc = use0 ? phi0[at(&Z, i, j, k)] : phi[at(&F, i, j, k)];
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t gp[3] = {pxp[a], pyp[a], pzp[a]}, gm[3] = {pxm[b], pym[b], pzm[b]}, st[3];
    for (int d = 0; d < 3; d++) {
      real_t u = (pc > 0.0) ? fmax2(-gp[d], 0.0) : fmax2(gp[d], 0.0);
      real_t w = (pc > 0.0) ? fmax2(gm[d], 0.0) : fmax2(-gm[d], 0.0);
      st[d] = fmax2(u, w);
    }
    real_t out = 0.0;
    if (fabs(pc) >= ORACLE_ZERO_TOL) {
      real_t n2 = st[0] * st[0] + st[1] * st[1] + st[2] * st[2];
      real_t sgn = use0 ? pc / sqrt(pc * pc + dx_sq) : pc / sqrt(pc * pc + n2 * dx_sq);
      out = sgn * (1.0 - sqrt(n2));
    }
    rhs[at(&R, i, j, k)] = out;
  }
}

/* ---- mean curvature over lists (curvature3d_local.f.in:15-150) ----------- */
void lsm3dcomputemeancurvatureorder2local_(real_t *kappa, A3(k), const real_t *phi, A3(f),
                                           const real_t *px, const real_t *py, const real_t *pz,
                                           const real_t *mag, A3(g), DX_ARGS, LOCAL_TAIL) {
  gbox K = B3(k), F = B3(f), G = B3(g), NB = NBBOX;
  real_t fxx = 1.0 / *dx / *dx, fyy = 1.0 / *dy / *dy, fzz = 1.0 / *dz / *dz;
  real_t fxy = 0.25 / *dx / *dy, fxz = 0.25 / *dx / *dz, fyz = 0.25 / *dy / *dz;
  long sx = F.s[0], sy = F.s[1], sz = F.s[2];
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&K, i, j, k) && inb(&G, i, j, k) && inb_r(&F, 1, i, j, k))) continue;
    const real_t *c = phi + at(&F, i, j, k);
    real_t xx = (c[sx] - 2.0 * c[0] + c[-sx]) * fxx;
    real_t yy = (c[sy] - 2.0 * c[0] + c[-sy]) * fyy;
    real_t zz = (c[sz] - 2.0 * c[0] + c[-sz]) * fzz;
    real_t xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * fxy;
    real_t xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * fxz;
    real_t yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * fyz;
    long g = at(&G, i, j, k);
    real_t den = mag[g] * mag[g] * mag[g];
    kappa[at(&K, i, j, k)] =
        (den < ORACLE_ZERO_TOL) ? 0.0 : curv_num(xx, yy, zz, xy, xz, yz, px[g], py[g], pz[g]) / den;
  }
}

/* ---- reductions over lists (math_utils3d_local.f.in) ------------------- */
void lsm3dmaxnormdifflocal_(real_t *out, const real_t *f1, A3(a), const real_t *f2, A3(b),
                            LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), NB = NBBOX;
  real_t m = 0.0; /* :72 */
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&A, i, j, k) && inb(&B, i, j, k))) continue;
    real_t d = fabs(f1[at(&A, i, j, k)] - f2[at(&B, i, j, k)]);
    if (d > m) m = d;
  }
  *out = m;
}

void lsm3dcomputestableadvectiondtlocal_(real_t *dt, const real_t *vx, const real_t *vy,
                                         const real_t *vz, A3(v), DX_ARGS, const real_t *cfl,
                                         LOCAL_TAIL) {
  gbox V = B3(v), NB = NBBOX;
  real_t ix_ = 1.0 / *dx, iy_ = 1.0 / *dy, iz_ = 1.0 / *dz, m = -1.0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&V, i, j, k))) continue;
    long c = at(&V, i, j, k);
    real_t u = fabs(vx[c]) * ix_ + fabs(vy[c]) * iy_ + fabs(vz[c]) * iz_;
    if (u > m) m = u;
  }
  *dt = *cfl / (m + ORACLE_TINY);
}

void lsm3dcomputestablenormalveldtlocal_(real_t *dt, const real_t *vn, A3(v), const real_t *pxp,
                                         const real_t *pyp, const real_t *pzp, A3(p),
                                         const real_t *pxm, const real_t *pym, const real_t *pzm,
                                         A3(m), DX_ARGS, const real_t *cfl, LOCAL_TAIL) {
  gbox V = B3(v), P = B3(p), M = B3(m), NB = NBBOX;
  real_t mx = fmax2(fmax2(*dx, *dy), *dz);
  real_t max_dx_sq = mx * mx;
  real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz}, best = -1.0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&V, i, j, k) && inb(&P, i, j, k) && inb(&M, i, j, k))) continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t cx = fmax2(fabs(pxp[a]), fabs(pxm[b]));
    real_t cy = fmax2(fabs(pyp[a]), fabs(pym[b]));
    real_t cz = fmax2(fabs(pzp[a]), fabs(pzm[b]));
    real_t ng = sqrt(cx * cx + cy * cy + cz * cz + max_dx_sq);
    if (ng > ORACLE_ZERO_TOL) { /* :404 */
      real_t h = fabs(vn[at(&V, i, j, k)]) / ng * (cx * inv[0] + cy * inv[1] + cz * inv[2]);
      if (h > best) best = h;
    }
  }
  *dt = *cfl / (best + ORACLE_TINY);
}

/* lsm3dMaxNormDiffControlVolumeLOCAL (math_utils3d_local.f.in:98-190): starts
 * at 0 and takes listed cells whose control volume is negative (the routine
 * has no control_vol_sgn argument) */
void lsm3dmaxnormdiffcontrolvolumelocal_(real_t *out, const real_t *f1, A3(a), const real_t *f2, A3(b),
                                         const real_t *cv, A3(c), LOCAL_TAIL) {
  gbox A = B3(a), B = B3(b), C = B3(c), NB = NBBOX;
  real_t m = 0.0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&A, i, j, k) && inb(&B, i, j, k) && inb(&C, i, j, k))) continue;
    if (!(cv[at(&C, i, j, k)] < 0.0)) continue;
    real_t d = fabs(f1[at(&A, i, j, k)] - f2[at(&B, i, j, k)]);
    if (d > m) m = d;
  }
  *out = m;
}

/* lsm3dComputeStableNormalVelDtControlVolumeLOCAL (math_utils3d_local.f.in:
 * 432-624): control_vol > 0 for control_vol_sgn > 0, else control_vol < 0;
 * cells with norm_grad_phi <= zero_tol are skipped (:138, :171) */
void lsm3dcomputestablenormalveldtcontrolvolumelocal_(real_t *dt, const real_t *vn, A3(v), const real_t *pxp,
                                                      const real_t *pyp, const real_t *pzp, A3(p),
                                                      const real_t *pxm, const real_t *pym,
                                                      const real_t *pzm, A3(m), const real_t *cv, A3(c),
                                                      const int *sgn, DX_ARGS, const real_t *cfl,
                                                      LOCAL_TAIL) {
  gbox V = B3(v), P = B3(p), M = B3(m), C = B3(c), NB = NBBOX;
  real_t mx = fmax2(fmax2(*dx, *dy), *dz);
  real_t max_dx_sq = mx * mx;
  real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz}, best = -1.0;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&V, i, j, k) && inb(&P, i, j, k) && inb(&M, i, j, k) && inb(&C, i, j, k))) continue;
    real_t c = cv[at(&C, i, j, k)];
    if (!(*sgn > 0 ? c > 0.0 : c < 0.0)) continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t cx = fmax2(fabs(pxp[a]), fabs(pxm[b]));
    real_t cy = fmax2(fabs(pyp[a]), fabs(pym[b]));
    real_t cz = fmax2(fabs(pzp[a]), fabs(pzm[b]));
    real_t ng = sqrt(cx * cx + cy * cy + cz * cz + max_dx_sq);
    if (ng > ORACLE_ZERO_TOL) {
      real_t h = fabs(vn[at(&V, i, j, k)]) / ng * (cx * inv[0] + cy * inv[1] + cz * inv[2]);
      if (h > best) best = h;
    }
  }
  *dt = *cfl / (best + ORACLE_TINY);
}

/* lsm3dComputeStableConstNormalVelDtLOCAL (math_utils3d_local.f.in:628-752)
 * reads two local variables it never assigns (abs_vel_n, norm_grad_phi).
 * The oracle implements the evident intent, the dense routine's formula
 * (math_utils3d.f.in:530-556) over the listed cells. */
void lsm3dcomputestableconstnormalveldtlocal_(real_t *dt, const real_t *vel_n, const real_t *pxp,
                                              const real_t *pyp, const real_t *pzp, A3(p),
                                              const real_t *pxm, const real_t *pym,
                                              const real_t *pzm, A3(m), DX_ARGS,
                                              const real_t *cfl, LOCAL_TAIL) {
  gbox P = B3(p), M = B3(m), NB = NBBOX;
  real_t mx = fmax2(*dx, *dy);
  mx = fmax2(mx, *dz);
  real_t max_dx_sq = mx * mx;
  real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz}, best = -1.0, avn = fabs(*vel_n);
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&P, i, j, k) && inb(&M, i, j, k))) continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t cx = fmax2(fabs(pxp[a]), fabs(pxm[b]));
    real_t cy = fmax2(fabs(pyp[a]), fabs(pym[b]));
    real_t cz = fmax2(fabs(pzp[a]), fabs(pzm[b]));
    real_t ng = sqrt(cx * cx + cy * cy + cz * cz + max_dx_sq);
    real_t h = avn / ng * (cx * inv[0] + cy * inv[1] + cz * inv[2]);
    if (h > best) best = h;
  }
  *dt = *cfl / (best + ORACLE_TINY);
}

/* ---- narrow band construction (localization3d.f) ---------------------- */

/* lsm3dMarkNarrowBandNeighbors (:48-167): breadth-first levels 1..level; the
 * neighbours of each parent are visited +x, -x, +y, -y, +z, -z and the first
 * visit claims a cell */
void lsm3dmarknarrowbandneighbors_(mark_t *nb, A3(g), int *ix_, int *iy_, int *iz_,
                                   const int *nlo_index, const int *nhi_index, int *n_lo,
                                   int *n_hi, const int *level) {
  gbox G = B3(g);
  const int base = *nlo_index;
  int count = n_hi[0] + 1;
  for (int lv = 1; lv <= *level; lv++) {
    mark_t mark = (mark_t)(lv + 1);
    for (int m = n_lo[lv - 1]; m <= n_hi[lv - 1]; m++) {
      const int i = ix_[m - base], j = iy_[m - base], k = iz_[m - base];
      const int nbr[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k},
                             {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
      const int ok[6] = {i < G.hi[0], i > G.lo[0], j < G.hi[1],
                         j > G.lo[1], k < G.hi[2], k > G.lo[2]};
      for (int q = 0; q < 6; q++) {
        if (!ok[q]) continue;
        long c = at(&G, nbr[q][0], nbr[q][1], nbr[q][2]);
        if (nb[c] == 0) {
          ix_[count - base] = nbr[q][0];
          iy_[count - base] = nbr[q][1];
          iz_[count - base] = nbr[q][2];
          nb[c] = mark;
          count++;
        }
      }
    }
    if (count > n_hi[lv - 1] + 1) {
      n_lo[lv] = n_hi[lv - 1] + 1;
      n_hi[lv] = count - 1;
    } else {
      n_lo[lv] = -1;
      n_hi[lv] = -1;
    }
  }
}

/* lsm3dDetermineNarrowBand (:174-297) */
void lsm3ddeterminenarrowband_(const real_t *phi, A3(g), mark_t *nb, A3(n), int *ix_, int *iy_,
                               int *iz_, const int *nlo_index, const int *nhi_index, int *n_lo,
                               int *n_hi, int *index_outer, const int *nlo_outer_idx,
                               const int *nhi_outer_idx, int *nlo_outer_plus, int *nhi_outer_plus,
                               int *nlo_outer_minus, int *nhi_outer_minus, const real_t *width,
                               const real_t *width_inner, const int *level) {
  gbox G = B3(g), N = B3(n);
  const int base = *nlo_index, obase = *nlo_outer_idx;
  int count = *nlo_index;
  n_lo[0] = *nlo_index;
  int cm = *nlo_outer_idx, cp = *nhi_outer_idx;
  *nlo_outer_minus = *nlo_outer_idx;
  *nhi_outer_plus = *nhi_outer_idx;
  FOR_BOX(G.lo[0], G.hi[0], G.lo[1], G.hi[1], G.lo[2], G.hi[2]) {
    real_t a = fabs(phi[at(&G, i, j, k)]);
    long c = at(&N, i, j, k);
    if (a < *width) {
      ix_[count - base] = i;
      iy_[count - base] = j;
      iz_[count - base] = k;
      nb[c] = 1;
      if (a >= *width_inner) {
        if (phi[at(&G, i, j, k)] <= 0.0)
          index_outer[(cm++) - obase] = count;
        else
          index_outer[(cp--) - obase] = count;
      }
      count++;
    } else {
      nb[c] = 0;
    }
  }
  if (count > *nlo_index) {
    n_hi[0] = count - 1;
    *nhi_outer_minus = cm - 1;
    *nlo_outer_plus = cp + 1;
    lsm3dmarknarrowbandneighbors_(nb, BOX6(n), ix_, iy_, iz_, nlo_index, nhi_index, n_lo, n_hi,
                                  level);
  } else {
    n_hi[0] = count;
    *nhi_outer_minus = cm;
    *nlo_outer_plus = cp;
  }
}

/* The 2D band builders' forms on 3D arrays (localization2d.f:174-464):
 * mode 0 |phi| < width; 3 also |second| < width (FromTwoLevelSets, :248);
 * 4 also |phi - second| > max_dx (AwayFromMask, :365).  bookkeeping 1
 * (DetermineNarrowBand, :225-240): n_hi(0) = count - 1 always, neighbour
 * levels when level > 0 and n_hi(0) > n_lo(0); 2 (:327-340): neighbour
 * levels whenever level > 0. */
static void determine_band_2dform(int mode, int bookkeeping, const real_t *phi, const real_t *second,
                                  real_t max_dx, const gbox *G, mark_t *nb, const int *n_lo_box, int *ix_,
                                  int *iy_, int *iz_, const int *nlo_index, const int *nhi_index, int *n_lo,
                                  int *n_hi, int *index_outer, const int *nlo_outer_idx,
                                  const int *nhi_outer_idx, int *nlo_outer_plus, int *nhi_outer_plus,
                                  int *nlo_outer_minus, int *nhi_outer_minus, real_t width,
                                  real_t width_inner, const int *level) {
  gbox N = mk_box(n_lo_box, n_lo_box + 1, n_lo_box + 2, n_lo_box + 3, n_lo_box + 4, n_lo_box + 5);
  const int base = *nlo_index, obase = *nlo_outer_idx;
  int count = *nlo_index;
  n_lo[0] = *nlo_index;
  int cm = *nlo_outer_idx, cp = *nhi_outer_idx;
  *nlo_outer_minus = *nlo_outer_idx;
  *nhi_outer_plus = *nhi_outer_idx;
  FOR_BOX(G->lo[0], G->hi[0], G->lo[1], G->hi[1], G->lo[2], G->hi[2]) {
    long g = at(G, i, j, k);
    real_t v = phi[g], a = fabs(v);
    int take = a < width;
    if (take && mode == 3) take = fabs(second[g]) < width;
    if (take && mode == 4) take = fabs(v - second[g]) > max_dx;
    long c = at(&N, i, j, k);
    if (take) {
      ix_[count - base] = i;
      iy_[count - base] = j;
      iz_[count - base] = k;
      nb[c] = 1;
      if (a >= width_inner) {
        if (v <= 0.0)
          index_outer[(cm++) - obase] = count;
        else
          index_outer[(cp--) - obase] = count;
      }
      count++;
    } else {
      nb[c] = 0;
    }
  }
  n_hi[0] = count - 1;
  *nhi_outer_minus = cm - 1;
  *nlo_outer_plus = cp + 1;
  if (*level > 0 && (bookkeeping == 2 || n_hi[0] > n_lo[0]))
    lsm3dmarknarrowbandneighbors_(nb, N.lo, N.hi, N.lo + 1, N.hi + 1, N.lo + 2, N.hi + 2, ix_, iy_, iz_,
                                  nlo_index, nhi_index, n_lo, n_hi, level);
}

#define BAND_ARGS                                                                                     \
  mark_t *nb, A3(n), int *ix_, int *iy_, int *iz_, const int *nlo_index, const int *nhi_index,          \
      int *n_lo, int *n_hi, int *index_outer, const int *nlo_outer_idx, const int *nhi_outer_idx,       \
      int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus, int *nhi_outer_minus,             \
      const real_t *width, const real_t *width_inner, const int *level
#define BAND_PASS                                                                                     \
  nb, nbox, ix_, iy_, iz_, nlo_index, nhi_index, n_lo, n_hi, index_outer, nlo_outer_idx, nhi_outer_idx, \
      nlo_outer_plus, nhi_outer_plus, nlo_outer_minus, nhi_outer_minus, *width, *width_inner, level

void lsmgpu_determine_narrow_band_2d_bookkeeping(const real_t *phi, A3(g), BAND_ARGS) {
  gbox G = B3(g);
  const int nbox[6] = {*n_ilo, *n_ihi, *n_jlo, *n_jhi, *n_klo, *n_khi};
  determine_band_2dform(0, 1, phi, NULL, 0.0, &G, BAND_PASS);
}

void lsm3ddeterminenarrowbandfromtwolevelsets_(const real_t *phi, const real_t *psi, A3(g), BAND_ARGS) {
  gbox G = B3(g);
  const int nbox[6] = {*n_ilo, *n_ihi, *n_jlo, *n_jhi, *n_klo, *n_khi};
  determine_band_2dform(3, 2, phi, psi, 0.0, &G, BAND_PASS);
}

void lsm3ddeterminenarrowbandawayfrommask_(const real_t *phi, const real_t *mask, A3(g), BAND_ARGS,
                                           const real_t *dx, const real_t *dy, const real_t *dz) {
  gbox G = B3(g);
  const int nbox[6] = {*n_ilo, *n_ihi, *n_jlo, *n_jhi, *n_klo, *n_khi};
  determine_band_2dform(4, 2, phi, mask, fmax2(fmax2(*dx, *dy), *dz), &G, BAND_PASS);
}

/* lsm3dMarkNarrowBandBoundaryLayer (:303-377): the six one-cell faces of the
 * fill box, over the ghost-box extent of the other axes */
void lsm3dmarknarrowbandboundarylayer_(mark_t *nb, A3(g), const int *ilo_fb, const int *ihi_fb,
                                       const int *jlo_fb, const int *jhi_fb, const int *klo_fb,
                                       const int *khi_fb, const mark_t *mark) {
  gbox G = B3(g);
  const int f[6] = {*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb};
  for (int face = 0; face < 6; face++) {
    int lo[3] = {G.lo[0], G.lo[1], G.lo[2]}, hi[3] = {G.hi[0], G.hi[1], G.hi[2]};
    lo[face / 2] = hi[face / 2] = f[face];
    FOR_BOX(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]) nb[at(&G, i, j, k)] = *mark;
  }
}

/* lsm3dDetermineNarrowBandFromMask (:385-475) */
void lsm3ddeterminenarrowbandfrommask_(const real_t *mask, A3(g), mark_t *nb, A3(n), int *ix_,
                                       int *iy_, int *iz_, const int *nlo_index,
                                       const int *nhi_index, int *n_lo, int *n_hi,
                                       const int *level, const int *use_mask_sign) {
  gbox G = B3(g), N = B3(n);
  const int base = *nlo_index;
  int count = *nlo_index;
  n_lo[0] = *nlo_index;
  FOR_BOX(G.lo[0], G.hi[0], G.lo[1], G.hi[1], G.lo[2], G.hi[2]) {
    real_t v = mask[at(&G, i, j, k)];
    int take = (*use_mask_sign > 0) ? (v >= 0.0) : (v <= 0.0);
    long c = at(&N, i, j, k);
    if (take) {
      ix_[count - base] = i;
      iy_[count - base] = j;
      iz_[count - base] = k;
      nb[c] = 1;
      count++;
    } else {
      nb[c] = 0;
    }
  }
  n_hi[0] = count - 1;
  lsm3dmarknarrowbandneighbors_(nb, BOX6(n), ix_, iy_, iz_, nlo_index, nhi_index, n_lo, n_hi,
                                level);
}

/* lsm3dMultiplyCutOffLSERHSLOCAL (:482-561): cubic cut-off between beta and
 * gamma */
void lsm3dmultiplycutofflserhslocal_(const real_t *phi, real_t *rhs, A3(g), LOCAL_TAIL,
                                     const real_t *beta, const real_t *gamma) {
  gbox G = B3(g), NB = NBBOX;
  real_t c1 = *gamma - 3 * *beta;
  real_t c2 = (*gamma - *beta);
  c2 = c2 * c2 * c2;
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (!GATE || !(inb(&G, i, j, k))) continue;
    long c = at(&G, i, j, k);
    real_t a = fabs(phi[c]), co;
    if (a <= *beta) {
      co = 1;
    } else if (a <= *gamma) {
      real_t t = a - *gamma;
      co = (t * t * (2 * a + c1)) / c2;
    } else {
      co = 0;
    }
    rhs[c] = co * rhs[c];
  }
}

/* lsm3dCheckOuterNarrowBandLayer (:568-653): 1 when the outer layer holds
 * both signs of phi, testing the plus list then the minus list */
void lsm3dcheckouternarrowbandlayer_(int *change_sign, const real_t *phi, A3(g), LIST_ARGS,
                                     const int *nlo, const int *nhi, const int *index_outer,
                                     const int *nlo_outer, const int *nhi_outer,
                                     const int *nlo_outer_plus, const int *nhi_outer_plus,
                                     const int *nlo_outer_minus, const int *nhi_outer_minus) {
  gbox G = B3(g);
  const int base = *nlo, obase = *nlo_outer;
  (void)nhi;
  (void)nhi_outer;
  int sp = 0, sm = 0, cs = 0;
  for (int m = *nlo_outer_plus; m <= *nhi_outer_plus; m++) {
    int l = index_outer[m - obase];
    if (phi[at(&G, ix[l - base], iy[l - base], iz[l - base])] > 0.0) sp = 1;
    else sm = 1;
    if (sp == 1 && sm == 1) {
      cs = 1;
      break;
    }
  }
  if (cs == 0) {
    sp = sm = 0;
    for (int m = *nlo_outer_minus; m <= *nhi_outer_minus; m++) {
      int l = index_outer[m - obase];
      if (phi[at(&G, ix[l - base], iy[l - base], iz[l - base])] > 0.0) sp = 1;
      else sm = 1;
      if (sp == 1 && sm == 1) {
        cs = 1;
        break;
      }
    }
  }
  *change_sign = cs;
}

/* lsm3dImposeMaskLocal (:660-719): dest = max(mask, src) on listed cells */
void lsm3dimposemasklocal_(real_t *dest, A3(d), const real_t *src, A3(s), const real_t *mask,
                           A3(m), LIST_ARGS, const int *nlo, const int *nhi) {
  gbox D = B3(d), S = B3(s), M = B3(m);
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (inb(&D, i, j, k) && inb(&S, i, j, k) && inb(&M, i, j, k))
      dest[at(&D, i, j, k)] = fmax2(mask[at(&M, i, j, k)], src[at(&S, i, j, k)]);
  }
}

/* lsm3dCopyDataLocal (:725-774) */
void lsm3dcopydatalocal_(real_t *dest, A3(d), const real_t *src, A3(s), LIST_ARGS, const int *nlo,
                         const int *nhi) {
  gbox D = B3(d), S = B3(s);
  FOR_LIST(*nlo, *nlo, *nhi) {
    if (inb(&D, i, j, k) && inb(&S, i, j, k)) dest[at(&D, i, j, k)] = src[at(&S, i, j, k)];
  }
}
