/*
 * CPU oracle, curvature variants and two narrow-band LSE terms.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_common.h).  Restates
 *  - lsm3dComputeGaussianCurvatureOrder2, lsm3dComputeMeanCurvatureOrder4,
 *    lsm3dComputeGaussianCurvatureOrder4 (curvature3d.f.in:136-508) and their
 *    index-list forms (curvature3d_local.f.in:151-574);
 *  - lsm3dAddConstPrecomputedCurvTermToLSERHSLOCAL and
 *    lsm3dAddExternalAndNormalVelTermToLSERHSLOCAL
 *    (level_set_evolution3d_local.f.in:530-812);
 *  - the external + normal velocity term in the form of the 2D routine
 *    (level_set_evolution2d.f.in:399-520: fill box only, nothing added where
 *    |Vn| < zero_tol) on 3D arrays, the library's
 *    lsmgpu_external_normal_vel_term_fill_box.
 * The reference's MeanCurvatureOrder4 list routine evaluates the Gaussian
 * formula (curvature3d_local.f.in:385-410); so does this restatement.
 */
#include "oracle_common.h"

typedef signed char mark_t;

#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,             \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi
#define B3(n) mk_box(n##_ilo, n##_ihi, n##_jlo, n##_jhi, n##_klo, n##_khi)
#define DX_ARGS const real_t *dx, const real_t *dy, const real_t *dz
#define LOCAL_TAIL                                                                       \
  const int *ix, const int *iy, const int *iz, const int *nlo, const int *nhi,           \
      const mark_t *nb, const int *nb_ilo, const int *nb_ihi, const int *nb_jlo,        \
      const int *nb_jhi, const int *nb_klo, const int *nb_khi, const mark_t *mark_fb

enum { GAUSS2, MEAN4, GAUSS4 };

static int inside(const gbox *b, int r, int i, int j, int k) {
  return i - r >= b->lo[0] && i + r <= b->hi[0] && j - r >= b->lo[1] && j + r <= b->hi[1] &&
         k - r >= b->lo[2] && k + r <= b->hi[2];
}

/* kappa at (i, j, k); F = phi's box, G = the gradient box */
static real_t curvature_at(int kind, const real_t *phi, const gbox *F, const real_t *px,
                           const real_t *py, const real_t *pz, const real_t *mag, const gbox *G,
                           real_t dx, real_t dy, real_t dz, int i, int j, int k) {
#define P(a, b, c) phi[at(F, i + (a), j + (b), k + (c))]
  real_t xx, yy, zz, xy, xz, yz;
  long g = at(G, i, j, k);
  real_t x = px[g], y = py[g], z = pz[g];
  if (kind == GAUSS2) {
    xx = (P(1, 0, 0) - 2.0 * P(0, 0, 0) + P(-1, 0, 0)) * (1.0 / dx / dx);
    yy = (P(0, 1, 0) - 2.0 * P(0, 0, 0) + P(0, -1, 0)) * (1.0 / dy / dy);
    zz = (P(0, 0, 1) - 2.0 * P(0, 0, 0) + P(0, 0, -1)) * (1.0 / dz / dz);
    xy = (P(1, 1, 0) - P(1, -1, 0) - P(-1, 1, 0) + P(-1, -1, 0)) * (0.25 / dx / dy);
    xz = (P(1, 0, 1) - P(1, 0, -1) - P(-1, 0, 1) + P(-1, 0, -1)) * (0.25 / dx / dz);
    yz = (P(0, 1, 1) - P(0, 1, -1) - P(0, -1, 1) + P(0, -1, -1)) * (0.25 / dy / dz);
  } else {
    const real_t c12 = 0.0833333333333333333333;
    xx = (-P(2, 0, 0) + 16.0 * P(1, 0, 0) - 30.0 * P(0, 0, 0) - P(-2, 0, 0) + 16.0 * P(-1, 0, 0)) *
         (c12 / dx / dx);
    yy = (-P(0, 2, 0) + 16.0 * P(0, 1, 0) - 30.0 * P(0, 0, 0) - P(0, -2, 0) + 16.0 * P(0, -1, 0)) *
         (c12 / dy / dy);
    zz = (-P(0, 0, 2) + 16.0 * P(0, 0, 1) - 30.0 * P(0, 0, 0) - P(0, 0, -2) + 16.0 * P(0, 0, -1)) *
         (c12 / dz / dz);
    xy = (-px[at(G, i, j + 2, k)] + 8.0 * px[at(G, i, j + 1, k)] + px[at(G, i, j - 2, k)] -
          8.0 * px[at(G, i, j - 1, k)]) * (c12 / dy);
    yz = (-py[at(G, i, j, k + 2)] + 8.0 * py[at(G, i, j, k + 1)] + py[at(G, i, j, k - 2)] -
          8.0 * py[at(G, i, j, k - 1)]) * (c12 / dz);
    xz = (-pz[at(G, i + 2, j, k)] + 8.0 * pz[at(G, i + 1, j, k)] + pz[at(G, i - 2, j, k)] -
          8.0 * pz[at(G, i - 1, j, k)]) * (c12 / dx);
  }
#undef P
  real_t m = mag[g];
  if (kind == MEAN4) {
    real_t den = m * m * m;
    if (den < ORACLE_ZERO_TOL) return 0.0;
    return (xx * y * y + yy * x * x - 2.0 * xy * x * y + xx * z * z + zz * x * x - 2.0 * xz * x * z +
            yy * z * z + zz * y * y - 2.0 * yz * y * z) / den;
  }
  real_t den = m * m * m * m;
  if (den < ORACLE_ZERO_TOL) return 0.0;
  real_t t = x * x * (yy * zz - yz * yz) + y * y * (xx * zz - xz * xz) + z * z * (xx * yy - xy * xy) +
             2.0 * (x * y * (xz * yz - xy * zz) + y * z * (xy * xz - yz * xx) + x * z * (xy * yz - xz * yy));
  return t / den;
}

static void curvature_dense(int kind, real_t *kappa, const gbox *K, const real_t *phi, const gbox *F,
                            const real_t *px, const real_t *py, const real_t *pz, const real_t *mag,
                            const gbox *G, const int *fb, real_t dx, real_t dy, real_t dz) {
  FOR_BOX(fb[0], fb[1], fb[2], fb[3], fb[4], fb[5]) {
    kappa[at(K, i, j, k)] = curvature_at(kind, phi, F, px, py, pz, mag, G, dx, dy, dz, i, j, k);
  }
}

#define DENSE_CURV(sym, kind)                                                                    \
  void sym(real_t *kappa, A3(k), const real_t *phi, A3(f), const real_t *px, const real_t *py,   \
           const real_t *pz, const real_t *mag, A3(g), A3(kf), DX_ARGS) {                        \
    gbox K = B3(k), F = B3(f), G = B3(g);                                                        \
    int fb[6] = {*kf_ilo, *kf_ihi, *kf_jlo, *kf_jhi, *kf_klo, *kf_khi};                          \
    curvature_dense(kind, kappa, &K, phi, &F, px, py, pz, mag, &G, fb, *dx, *dy, *dz);           \
  }

DENSE_CURV(lsm3dcomputegaussiancurvatureorder2_, GAUSS2)
DENSE_CURV(lsm3dcomputemeancurvatureorder4_, MEAN4)
DENSE_CURV(lsm3dcomputegaussiancurvatureorder4_, GAUSS4)

/* list forms: cells outside an array, or whose stencil leaves one, are
 * skipped (the reference reads outside its arrays there) */
static void curvature_list(int kind, real_t *kappa, const gbox *K, const real_t *phi, const gbox *F,
                           const real_t *px, const real_t *py, const real_t *pz, const real_t *mag,
                           const gbox *G, real_t dx, real_t dy, real_t dz, const int *ix, const int *iy,
                           const int *iz, int lo, int hi, const mark_t *nb, const gbox *NB, mark_t mark) {
  int rp = (kind == GAUSS2) ? 1 : 2, rg = (kind == GAUSS2) ? 0 : 2;
  for (int l = lo; l <= hi; l++) {
    int i = ix[l - lo], j = iy[l - lo], k = iz[l - lo];
    if (!inside(NB, 0, i, j, k) || nb[at(NB, i, j, k)] > mark) continue;
    if (!inside(K, 0, i, j, k) || !inside(G, rg, i, j, k) || !inside(F, rp, i, j, k)) continue;
    kappa[at(K, i, j, k)] = curvature_at(kind, phi, F, px, py, pz, mag, G, dx, dy, dz, i, j, k);
  }
}

#define LOCAL_CURV(sym, kind)                                                                    \
  void sym(real_t *kappa, A3(k), const real_t *phi, A3(f), const real_t *px, const real_t *py,   \
           const real_t *pz, const real_t *mag, A3(g), DX_ARGS, LOCAL_TAIL) {                    \
    gbox K = B3(k), F = B3(f), G = B3(g), NB = B3(nb);                                           \
    curvature_list(kind, kappa, &K, phi, &F, px, py, pz, mag, &G, *dx, *dy, *dz, ix, iy, iz,     \
                   *nlo, *nhi, nb, &NB, *mark_fb);                                               \
  }

LOCAL_CURV(lsm3dcomputegaussiancurvatureorder2local_, GAUSS2)
LOCAL_CURV(lsm3dcomputemeancurvatureorder4local_, GAUSS4) /* the reference's formula */
LOCAL_CURV(lsm3dcomputegaussiancurvatureorder4local_, GAUSS4)
LOCAL_CURV(lsmgpu_mean_curvature_order4_local, MEAN4)

/* lsm3dAddConstPrecomputedCurvTermToLSERHSLOCAL (level_set_evolution3d_local.f.in:530-607) */
void lsm3daddconstprecomputedcurvtermtolserhslocal_(real_t *rhs, A3(r), const real_t *kappa, A3(k),
                                                    const real_t *mag, A3(g), const real_t *b,
                                                    LOCAL_TAIL) {
  gbox R = B3(r), K = B3(k), G = B3(g), NB = B3(nb);
  for (int l = *nlo; l <= *nhi; l++) {
    int i = ix[l - *nlo], j = iy[l - *nlo], k = iz[l - *nlo];
    if (!inside(&NB, 0, i, j, k) || nb[at(&NB, i, j, k)] > *mark_fb) continue;
    if (!inside(&R, 0, i, j, k) || !inside(&K, 0, i, j, k) || !inside(&G, 0, i, j, k)) continue;
    long r = at(&R, i, j, k);
    rhs[r] = rhs[r] + *b * kappa[at(&K, i, j, k)] * mag[at(&G, i, j, k)];
  }
}

/* Godunov choice of one gradient component for H = v.grad(phi) + vn |grad phi|
 * (level_set_evolution3d_local.f.in:714-787) */
static real_t godunov_ext(real_t v, real_t vn, real_t plus, real_t minus) {
  real_t h_plus = v + vn * plus, h_minus = v + vn * minus;
  if (h_plus > 0.0) {
    if (h_minus > 0.0) return minus;
    return -(v / vn);
  }
  if (h_minus < 0.0) return plus;
  if (fabs(h_plus) > fabs(h_minus)) return plus;
  return minus;
}

/* lsm3dAddExternalAndNormalVelTermToLSERHSLOCAL (level_set_evolution3d_local.f.in:612-812) */
void lsm3daddexternalandnormalveltermtolserhslocal_(real_t *rhs, A3(r), const real_t *pxp,
                                                    const real_t *pyp, const real_t *pzp, A3(p),
                                                    const real_t *pxm, const real_t *pym,
                                                    const real_t *pzm, A3(m), const real_t *vn,
                                                    const real_t *vx, const real_t *vy, const real_t *vz,
                                                    A3(v), LOCAL_TAIL) {
  gbox R = B3(r), P = B3(p), M = B3(m), V = B3(v), NB = B3(nb);
  for (int l = *nlo; l <= *nhi; l++) {
    int i = ix[l - *nlo], j = iy[l - *nlo], k = iz[l - *nlo];
    if (!inside(&NB, 0, i, j, k) || nb[at(&NB, i, j, k)] > *mark_fb) continue;
    if (!inside(&R, 0, i, j, k) || !inside(&P, 0, i, j, k) || !inside(&M, 0, i, j, k) ||
        !inside(&V, 0, i, j, k))
      continue;
    long a = at(&P, i, j, k), b = at(&M, i, j, k), c = at(&V, i, j, k), r = at(&R, i, j, k);
    real_t w = vn[c], ux = vx[c], uy = vy[c], uz = vz[c];
    real_t gx = godunov_ext(ux, w, pxp[a], pxm[b]);
    real_t gy = godunov_ext(uy, w, pyp[a], pym[b]);
    real_t gz = godunov_ext(uz, w, pzp[a], pzm[b]);
    real_t n2 = gx * gx + gy * gy + gz * gz;
    if (fabs(w) >= ORACLE_ZERO_TOL && n2 >= ORACLE_ZERO_TOL)
      rhs[r] = rhs[r] - ux * gx - uy * gy - uz * gz - w * sqrt(n2);
    else
      rhs[r] = rhs[r] - ux * gx - uy * gy - uz * gz;
  }
}

void lsmgpu_external_normal_vel_term_fill_box(real_t *rhs, A3(r), const real_t *pxp, const real_t *pyp,
                                              const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
                                              const real_t *pzm, A3(m), const real_t *vn, const real_t *vx,
                                              const real_t *vy, const real_t *vz, A3(v), A3(fb)) {
  gbox R = B3(r), P = B3(p), M = B3(m), V = B3(v);
  FOR_BOX(*fb_ilo, *fb_ihi, *fb_jlo, *fb_jhi, *fb_klo, *fb_khi) {
    long a = at(&P, i, j, k), b = at(&M, i, j, k), c = at(&V, i, j, k), r = at(&R, i, j, k);
    real_t w = vn[c];
    if (!(fabs(w) >= ORACLE_ZERO_TOL)) continue;
    real_t gx = godunov_ext(vx[c], w, pxp[a], pxm[b]);
    real_t gy = godunov_ext(vy[c], w, pyp[a], pym[b]);
    real_t gz = godunov_ext(vz[c], w, pzp[a], pzm[b]);
    rhs[r] = rhs[r] - vx[c] * gx - vy[c] * gy - vz[c] * gz - w * sqrt(gx * gx + gy * gy + gz * gz);
  }
}
