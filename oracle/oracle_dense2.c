/*
 * CPU oracle, further dense routines (TEST INFRASTRUCTURE ONLY): Hessian,
 * averaged and upwinded gradients, and the two LSE terms whose loops mix the
 * fill box and the ghost box.
 */
#include "oracle_common.h"

#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,             \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi
#define B3(n) mk_box(n##_ilo, n##_ihi, n##_jlo, n##_jhi, n##_klo, n##_khi)

/* lsm3dCentralHessian (spatial_derivatives3d.f.in:3664-3742) */
void lsm3dcentralhessian_(real_t *xx, real_t *xy, real_t *xz, real_t *yy, real_t *yz, real_t *zz,
                          A3(h), const real_t *phi, A3(f), A3(fb), const real_t *dx,
                          const real_t *dy, const real_t *dz) {
  gbox H = B3(h), F = B3(f);
  long sx = F.s[0], sy = F.s[1], sz = F.s[2];
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    const real_t *c = phi + at(&F, i, j, k);
    long o = at(&H, i, j, k);
    xx[o] = (c[sx] - 2 * c[0] + c[-sx]) / (*dx * *dx);
    xy[o] = 0.25 * (c[sx + sy] - c[-sx + sy] - c[sx - sy] + c[-sx - sy]) / (*dx * *dy);
    xz[o] = 0.25 * (c[sx + sz] - c[-sx + sz] - c[sx - sz] + c[-sx - sz]) / (*dx * *dz);
    yy[o] = (c[sy] - 2 * c[0] + c[-sy]) / (*dy * *dy);
    yz[o] = 0.25 * (c[sy + sz] - c[-sy + sz] - c[sy - sz] + c[-sy - sz]) / (*dy * *dz);
    zz[o] = (c[sz] - 2 * c[0] + c[-sz]) / (*dz * *dz);
  }
}

/* lsm3dAverageGradPhi (spatial_derivatives3d.f.in:3486-3571) */
void lsm3daveragegradphi_(real_t *px, real_t *py, real_t *pz, A3(g), const real_t *pxp,
                          const real_t *pyp, const real_t *pzp, A3(p), const real_t *pxm,
                          const real_t *pym, const real_t *pzm, A3(m), A3(fb)) {
  gbox G = B3(g), P = B3(p), M = B3(m);
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    long o = at(&G, i, j, k), a = at(&P, i, j, k), b = at(&M, i, j, k);
    px[o] = 0.5 * (pxp[a] + pxm[b]);
    py[o] = 0.5 * (pyp[a] + pym[b]);
    pz[o] = 0.5 * (pzp[a] + pzm[b]);
  }
}

/* lsm3dPhiUpwindGradF (spatial_derivatives3d.f.in:3270-3467): per axis, pick
 * the plus or minus derivative of F toward the neighbour of phi that lies on
 * the zero-level side; cells with phi = 0 are left untouched */
void lsm3dphiupwindgradf_(real_t *fx, real_t *fy, real_t *fz, A3(g), const real_t *fxp,
                          const real_t *fyp, const real_t *fzp, A3(p), const real_t *fxm,
                          const real_t *fym, const real_t *fzm, A3(m), const real_t *phi, A3(f),
                          A3(fb)) {
  gbox G = B3(g), P = B3(p), M = B3(m), F = B3(f);
  real_t *out[3] = {fx, fy, fz};
  const real_t *plus[3] = {fxp, fyp, fzp}, *minus[3] = {fxm, fym, fzm};
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    const real_t *c = phi + at(&F, i, j, k);
    real_t pc = c[0];
    long o = at(&G, i, j, k), a = at(&P, i, j, k), b = at(&M, i, j, k);
    for (int d = 0; d < 3; d++) {
      real_t nm = c[-F.s[d]], np = c[F.s[d]];
      if (pc > 0) {
        if (nm <= pc)
          out[d][o] = (np < nm) ? plus[d][a] : minus[d][b];
        else if (np <= pc)
          out[d][o] = plus[d][a];
        else
          out[d][o] = 0.0;
      } else if (pc < 0) {
        if (nm >= pc)
          out[d][o] = (np > nm) ? plus[d][a] : minus[d][b];
        else if (np >= pc)
          out[d][o] = plus[d][a];
        else
          out[d][o] = 0.0;
      }
    }
  }
}

/* lsm3dAddConstPrecomputedCurvTermToLSERHS (level_set_evolution3d.f.in:465-525):
 * k runs klo_fb..khi_gb, j jlo_fb..jhi_gb, i ilo_gb..ihi_gb (of the rhs), as
 * the reference loops */
void lsm3daddconstprecomputedcurvtermtolserhs_(real_t *rhs, A3(r), const real_t *kappa, A3(k),
                                               const real_t *mag, A3(g), const real_t *b,
                                               A3(fb)) {
  gbox R = B3(r), K = B3(k), G = B3(g);
  (void)fb_ilo; (void)fb_ihi; (void)fb_jhi; (void)fb_khi;
  FOR_BOX(R.lo[0], R.hi[0], *fb_jlo, R.hi[1], *fb_klo, R.hi[2]) {
    long o = at(&R, i, j, k);
    rhs[o] = rhs[o] + *b * kappa[at(&K, i, j, k)] * mag[at(&G, i, j, k)];
  }
}

/* one axis of the combined Godunov selection
 * (level_set_evolution3d.f.in:630-649) */
static real_t ext_normal_pick(real_t v, real_t vn, real_t p, real_t m) {
  real_t hp = v + vn * p, hm = v + vn * m;
  if (hp > 0.0) return (hm > 0.0) ? m : -v / vn;
  if (hm < 0.0) return p;
  return (fabs(hp) > fabs(hm)) ? p : m;
}

/* lsm3dAddExternalAndNormalVelTermToLSERHS (level_set_evolution3d.f.in:532-718),
 * same mixed loop bounds as above */
void lsm3daddexternalandnormalveltermtolserhs_(real_t *rhs, A3(r), const real_t *pxp,
                                               const real_t *pyp, const real_t *pzp, A3(p),
                                               const real_t *pxm, const real_t *pym,
                                               const real_t *pzm, A3(m), const real_t *vn,
                                               const real_t *vx, const real_t *vy,
                                               const real_t *vz, A3(v), A3(fb)) {
  gbox R = B3(r), P = B3(p), M = B3(m), V = B3(v);
  (void)fb_ilo; (void)fb_ihi; (void)fb_jhi; (void)fb_khi;
  FOR_BOX(R.lo[0], R.hi[0], *fb_jlo, R.hi[1], *fb_klo, R.hi[2]) {
    long vv = at(&V, i, j, k), a = at(&P, i, j, k), b = at(&M, i, j, k), o = at(&R, i, j, k);
    real_t w = vn[vv], ux = vx[vv], uy = vy[vv], uz = vz[vv];
    real_t gx = ext_normal_pick(ux, w, pxp[a], pxm[b]);
    real_t gy = ext_normal_pick(uy, w, pyp[a], pym[b]);
    real_t gz = ext_normal_pick(uz, w, pzp[a], pzm[b]);
    real_t n2 = gx * gx + gy * gy + gz * gz;
    if (fabs(w) >= ORACLE_ZERO_TOL && n2 >= ORACLE_ZERO_TOL)
      rhs[o] = rhs[o] - ux * gx - uy * gy - uz * gz - w * sqrt(n2);
    else
      rhs[o] = rhs[o] - ux * gx - uy * gy - uz * gz;
  }
}

/* lsm3dComputeDn (spatial_derivatives3d.f.in:49-176) */
void lsm3dcomputedn_(real_t *dn, A3(d), const real_t *dm, A3(m), const int *ilo_fb, const int *ihi_fb,
                     const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb, const int *n,
                     const int *dir) {
  gbox D = B3(d), M = B3(m);
  int off[3] = {0, 0, 0}, shift[3] = {0, 0, 0};
  real_t sgn;
  if (*n % 2 == 1) {
    off[*dir - 1] = 1;
    sgn = 1.0;
    shift[*dir - 1] = 1;
  } else {
    off[*dir - 1] = -1;
    sgn = -1.0;
  }
  FOR_BOX(*ilo_fb, *ihi_fb + shift[0], *jlo_fb, *jhi_fb + shift[1], *klo_fb, *khi_fb + shift[2])
    dn[at(&D, i, j, k)] = sgn * (dm[at(&M, i, j, k)] - dm[at(&M, i - off[0], j - off[1], k - off[2])]);
  /* cells outside that range hold big (:138-172) */
  FOR_BOX(D.lo[0], D.hi[0], D.lo[1], D.hi[1], D.lo[2], D.hi[2]) {
    int in = i >= *ilo_fb && i <= *ihi_fb + shift[0] && j >= *jlo_fb && j <= *jhi_fb + shift[1] &&
             k >= *klo_fb && k <= *khi_fb + shift[2];
    if (!in) dn[at(&D, i, j, k)] = 1.e10;
  }
}

/* lsm3dDeltaFunctionOrder1 (calculus_toolbox3d.f.in:15-130; its z terms use
 * norm_phi_x and 1/dx, :103-115) */
static real_t delta_side(real_t nbr, real_t c, real_t n, real_t o) {
  if (nbr * c <= 0.0) {
    real_t v = nbr * n * o;
    return v / (nbr - c);
  }
  return 0.0;
}
void lsm3ddeltafunctionorder1_(const real_t *phi, real_t *delta, A3(g), const real_t *nx, const real_t *ny,
                               const real_t *nz, A3(n), const int *ilo_fb, const int *ihi_fb, const int *jlo_fb,
                               const int *jhi_fb, const int *klo_fb, const int *khi_fb, const real_t *dx,
                               const real_t *dy, const real_t *dz) {
  gbox G = B3(g), N = B3(n);
  real_t ox = 1.0 / *dx, oy = 1.0 / *dy;
  (void)nz;
  (void)dz;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    real_t c = phi[at(&G, i, j, k)];
    long q = at(&N, i, j, k);
    real_t xp = delta_side(phi[at(&G, i + 1, j, k)], c, nx[q], ox);
    real_t xm = delta_side(phi[at(&G, i - 1, j, k)], c, nx[q], ox);
    real_t yp = delta_side(phi[at(&G, i, j + 1, k)], c, ny[q], oy);
    real_t ym = delta_side(phi[at(&G, i, j - 1, k)], c, ny[q], oy);
    real_t zp = delta_side(phi[at(&G, i, j, k + 1)], c, nx[q], ox);
    real_t zm = delta_side(phi[at(&G, i, j, k - 1)], c, nx[q], ox);
    delta[at(&G, i, j, k)] = fabs(xp) + fabs(xm) + fabs(yp) + fabs(ym) + fabs(zp) + fabs(zm);
  }
}
