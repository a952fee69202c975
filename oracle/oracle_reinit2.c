/*
 * CPU oracle, orthogonalization and subcell-fix routines of the
 * reinitialization toolbox.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_common.h).  Restates
 *  - lsm3dComputeOrthogonalizationEqnRHS (reinitialization3d.f.in:296-470) and
 *    its list form (reinitialization3d_local.f.in:326-480);
 *  - lsm3dComputeDistanceForSubcellFix (reinitialization3d.f.in:477-575);
 *  - lsm3dComputeReinitializationEqnRHSSubcellFixOrder1
 *    (reinitialization3d.f.in:586-757).
 * MAX / MIN follow the reference translation: max(a, b) = a > b ? a : b,
 * folded left for more arguments.
 */
#include "oracle_common.h"

typedef signed char mark_t;

#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,             \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi
#define B3(n) mk_box(n##_ilo, n##_ihi, n##_jlo, n##_jhi, n##_klo, n##_khi)

static int inside(const gbox *b, int i, int j, int k) {
  return i >= b->lo[0] && i <= b->hi[0] && j >= b->lo[1] && j <= b->hi[1] && k >= b->lo[2] &&
         k <= b->hi[2];
}

/* reinitialization3d.f.in:380-425; unit_smooth: sgn(psi) smoothed with
 * dx_sq alone, as reinitialization2d.f.in:360 does */
static int unit_smooth = 0;
static real_t ortho_cell(real_t psi, real_t sxp, real_t syp, real_t szp, real_t sxm, real_t sym,
                         real_t szm, real_t pxp, real_t pyp, real_t pzp, real_t pxm, real_t pym,
                         real_t pzm, real_t dx_sq) {
  real_t gx = 0.5 * (sxp + sxm), gy = 0.5 * (syp + sym), gz = 0.5 * (szp + szm);
  real_t norm = sqrt(gx * gx + gy * gy + gz * gz);
  if (!(fabs(psi) > ORACLE_ZERO_TOL && norm > ORACLE_ZERO_TOL)) return 0.0;
  real_t sgn = unit_smooth ? psi / sqrt(psi * psi + dx_sq) : psi / sqrt(psi * psi + dx_sq * (norm * norm));
  real_t sum = fmax2(sgn * gx, 0.0) * pxm + fmin2(sgn * gx, 0.0) * pxp + fmax2(sgn * gy, 0.0) * pym +
               fmin2(sgn * gy, 0.0) * pyp + fmax2(sgn * gz, 0.0) * pzm + fmin2(sgn * gz, 0.0) * pzp;
  return -1.0 / norm * sum;
}

void lsm3dcomputeorthogonalizationeqnrhs_(real_t *out, A3(r), const real_t *pxp, const real_t *pyp,
                                          const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
                                          const real_t *pzm, A3(m), const real_t *psi, A3(s),
                                          const real_t *sxp, const real_t *syp, const real_t *szp, A3(sp),
                                          const real_t *sxm, const real_t *sym, const real_t *szm, A3(sm),
                                          A3(fb), const real_t *dx, const real_t *dy, const real_t *dz) {
  gbox R = B3(r), P = B3(p), M = B3(m), S = B3(s), SP = B3(sp), SM = B3(sm);
  real_t dx_sq = fmax2(fmax2(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    long a = at(&P, i, j, k), b = at(&M, i, j, k), c = at(&SP, i, j, k), d = at(&SM, i, j, k);
    out[at(&R, i, j, k)] = ortho_cell(psi[at(&S, i, j, k)], sxp[c], syp[c], szp[c], sxm[d], sym[d], szm[d],
                                      pxp[a], pyp[a], pzp[a], pxm[b], pym[b], pzm[b], dx_sq);
  }
}

void lsm3dcomputeorthogonalizationeqnrhslocal_(
    real_t *out, A3(r), const real_t *pxp, const real_t *pyp, const real_t *pzp, A3(p), const real_t *pxm,
    const real_t *pym, const real_t *pzm, A3(m), const real_t *psi, A3(s), const real_t *sxp,
    const real_t *syp, const real_t *szp, A3(sp), const real_t *sxm, const real_t *sym, const real_t *szm,
    A3(sm), const real_t *dx, const real_t *dy, const real_t *dz, const int *ix, const int *iy,
    const int *iz, const int *nlo, const int *nhi, const mark_t *nb, A3(nb), const mark_t *mark_fb) {
  gbox R = B3(r), P = B3(p), M = B3(m), S = B3(s), SP = B3(sp), SM = B3(sm), NB = B3(nb);
  real_t dx_sq = fmax2(fmax2(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  for (int l = *nlo; l <= *nhi; l++) {
    int i = ix[l - *nlo], j = iy[l - *nlo], k = iz[l - *nlo];
    if (!inside(&NB, i, j, k) || nb[at(&NB, i, j, k)] > *mark_fb) continue;
    if (!(inside(&R, i, j, k) && inside(&P, i, j, k) && inside(&M, i, j, k) && inside(&S, i, j, k) &&
          inside(&SP, i, j, k) && inside(&SM, i, j, k)))
      continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k), c = at(&SP, i, j, k), d = at(&SM, i, j, k);
    out[at(&R, i, j, k)] = ortho_cell(psi[at(&S, i, j, k)], sxp[c], syp[c], szp[c], sxm[d], sym[d], szm[d],
                                      pxp[a], pyp[a], pzp[a], pxm[b], pym[b], pzm[b], dx_sq);
  }
}

/* 1 when phi0 changes sign between the cell and a face neighbour: the 3D
 * routine's comparisons, or (full_central) the 2D routine's negative product
 * (reinitialization2d.f.in:425-434) */
static int full_central = 0;
static int crosses(real_t nbr, real_t c) {
  if (full_central) return nbr * c < 0.0;
  return (nbr > 0.0 && c <= 0.0) || (nbr <= 0.0 && c > 0.0);
}

void lsm3dcomputedistanceforsubcellfix_(real_t *dist, const real_t *phi0, A3(z), A3(fb), const real_t *dx,
                                        const real_t *dy, const real_t *dz) {
  gbox Z = B3(z);
  real_t flag = -1000.0 * fmax2(fmax2(*dx, *dy), *dz);
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    real_t c = phi0[at(&Z, i, j, k)];
    real_t xp = phi0[at(&Z, i + 1, j, k)], xm = phi0[at(&Z, i - 1, j, k)];
    real_t yp = phi0[at(&Z, i, j + 1, k)], ym = phi0[at(&Z, i, j - 1, k)];
    real_t zp = phi0[at(&Z, i, j, k + 1)], zm = phi0[at(&Z, i, j, k - 1)];
    int near = crosses(xp, c) || crosses(xm, c) || crosses(yp, c) || crosses(ym, c) || crosses(zp, c) ||
               crosses(zm, c);
    if (!near) {
      dist[at(&Z, i, j, k)] = flag;
      continue;
    }
    real_t h = full_central ? 1.0 : 2.0;
    real_t delta = fmax2(fmax2(fmax2(fabs(xp - xm) / h, fabs(xp - c)), fabs(c - xm)), ORACLE_ZERO_TOL);
    delta = fmax2(fmax2(fmax2(fabs(yp - ym) / h, fabs(yp - c)), fabs(c - ym)), delta);
    delta = fmax2(fmax2(fmax2(fabs(zp - zm) / h, fabs(zp - c)), fabs(c - zm)), delta);
    dist[at(&Z, i, j, k)] = full_central ? 2.0 * c / delta : c / delta;
  }
}

void lsm3dcomputereinitializationeqnrhssubcellfixorder1_(
    real_t *out, A3(r), const real_t *phi, A3(f), const real_t *phi0, const real_t *dist, A3(z),
    const real_t *pxp, const real_t *pyp, const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
    const real_t *pzm, A3(m), A3(fb), const real_t *dx, const real_t *dy, const real_t *dz) {
  gbox R = B3(r), F = B3(f), Z = B3(z), P = B3(p), M = B3(m);
  real_t max_dx = fmax2(fmax2(*dx, *dy), *dz);
  real_t flag = -1000.0 * max_dx;
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    real_t p0 = phi0[at(&Z, i, j, k)], d0 = dist[at(&Z, i, j, k)], pc = phi[at(&F, i, j, k)];
    real_t sgn0 = (fabs(p0) > ORACLE_ZERO_TOL) ? (p0 > 0.0 ? 1.0 : -1.0) : 0.0;
    long r = at(&R, i, j, k);
    if (d0 == flag) {
      long a = at(&P, i, j, k), b = at(&M, i, j, k);
      real_t plus[3] = {pxp[a], pyp[a], pzp[a]}, minus[3] = {pxm[b], pym[b], pzm[b]}, star[3];
      for (int d = 0; d < 3; d++) {
        real_t u = (pc > 0.0) ? fmax2(-plus[d], 0.0) : fmax2(plus[d], 0.0);
        real_t w = (pc > 0.0) ? fmax2(minus[d], 0.0) : fmax2(-minus[d], 0.0);
        star[d] = fmax2(u, w);
      }
      if (fabs(pc) > ORACLE_ZERO_TOL)
        out[r] = sgn0 - sgn0 * sqrt(star[0] * star[0] + star[1] * star[1] + star[2] * star[2]);
      else
        out[r] = 0.0;
    } else {
      out[r] = d0 - sgn0 * fabs(pc) / max_dx;
    }
  }
}

/* the 2D routines' forms on 3D arrays (the library's extension entry points) */
#define ORTHO_ARGS                                                                                       \
  real_t *out, A3(r), const real_t *pxp, const real_t *pyp, const real_t *pzp, A3(p), const real_t *pxm, \
      const real_t *pym, const real_t *pzm, A3(m), const real_t *psi, A3(s), const real_t *sxp,           \
      const real_t *syp, const real_t *szp, A3(sp), const real_t *sxm, const real_t *sym,                 \
      const real_t *szm, A3(sm)
#define ORTHO_PASS                                                                                       \
  out, r_ilo, r_ihi, r_jlo, r_jhi, r_klo, r_khi, pxp, pyp, pzp, p_ilo, p_ihi, p_jlo, p_jhi, p_klo, p_khi, \
      pxm, pym, pzm, m_ilo, m_ihi, m_jlo, m_jhi, m_klo, m_khi, psi, s_ilo, s_ihi, s_jlo, s_jhi, s_klo,    \
      s_khi, sxp, syp, szp, sp_ilo, sp_ihi, sp_jlo, sp_jhi, sp_klo, sp_khi, sxm, sym, szm, sm_ilo, sm_ihi, \
      sm_jlo, sm_jhi, sm_klo, sm_khi

void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing(ORTHO_ARGS, A3(fb), const real_t *dx, const real_t *dy,
                                                     const real_t *dz) {
  unit_smooth = 1;
  lsm3dcomputeorthogonalizationeqnrhs_(ORTHO_PASS, fb_ilo, fb_ihi, fb_jlo, fb_jhi, fb_klo, fb_khi, dx, dy, dz);
  unit_smooth = 0;
}

void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local(ORTHO_ARGS, const real_t *dx, const real_t *dy,
                                                           const real_t *dz, const int *ix, const int *iy,
                                                           const int *iz, const int *nlo, const int *nhi,
                                                           const mark_t *nb, A3(nb), const mark_t *mark_fb) {
  unit_smooth = 1;
  lsm3dcomputeorthogonalizationeqnrhslocal_(ORTHO_PASS, dx, dy, dz, ix, iy, iz, nlo, nhi, nb, nb_ilo, nb_ihi,
                                            nb_jlo, nb_jhi, nb_klo, nb_khi, mark_fb);
  unit_smooth = 0;
}

void lsmgpu_distance_for_subcell_fix_full_central(real_t *dist, const real_t *phi0, A3(z), A3(fb),
                                                  const real_t *dx, const real_t *dy, const real_t *dz) {
  full_central = 1;
  lsm3dcomputedistanceforsubcellfix_(dist, phi0, z_ilo, z_ihi, z_jlo, z_jhi, z_klo, z_khi, fb_ilo, fb_ihi,
                                     fb_jlo, fb_jhi, fb_klo, fb_khi, dx, dy, dz);
  full_central = 0;
}
