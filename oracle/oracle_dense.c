/*
 * CPU oracle, dense-grid kernels.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle_common.h).  Each function restates one
 * LSMLIB Fortran routine and exports the symbol name gfortran gives it, so the
 * oracle and the GPU library can be driven by the same caller.  File:line
 * citations are relative to the LSMLIB source tree.
 *
 * Design: instead of the reference's sweep-per-direction structure (compute
 * the undivided-difference array D1/D2/D3 over the whole box, then a second
 * sweep that reads it), every derivative here is evaluated per cell from phi
 * along one axis (stride s).  The undivided differences are formed with the
 * same subtractions the reference performs, so values are identical; the
 * scratch arrays D1/D2/D3 are accepted and left untouched.
 */
#include "oracle_common.h"

/* ---- undivided differences along one axis --------------------------------
 * lsm3dComputeDn (spatial_derivatives3d.f.in:49-176): for odd n,
 * Dn(i) = Dn-1(i) - Dn-1(i-1); for even n, Dn(i) = -(Dn-1(i) - Dn-1(i+1)).
 * -(a-b) equals b-a exactly in IEEE arithmetic, so D2(i) = D1(i+1) - D1(i).
 * Offsets are relative to the cell being evaluated; D1[f+2] holds D1(i+f). */
typedef struct {
  real_t d1[6]; /* f = -2..3  */
  real_t d2[5]; /* f = -2..2  */
  real_t d3[4]; /* f = -1..2  */
} diffs_t;

static void load_diffs(diffs_t *d, const real_t *p, long s, int order) {
  for (int f = -2; f <= 3; f++) d->d1[f + 2] = p[f * s] - p[(f - 1) * s];
  if (order >= 2)
    for (int f = -2; f <= 2; f++) d->d2[f + 2] = d->d1[f + 3] - d->d1[f + 2];
  if (order >= 3)
    for (int f = -1; f <= 2; f++) d->d3[f + 1] = d->d2[f + 2] - d->d2[f + 1];
}
#define D1(f) (d->d1[(f) + 2])
#define D2(f) (d->d2[(f) + 2])
#define D3(f) (d->d3[(f) + 1])

/* ENO2 plus/minus (spatial_derivatives3d.f.in:520-535) */
static real_t eno2_plus(const diffs_t *d, real_t inv) {
  if (fabs(D2(0)) < fabs(D2(1))) return (D1(1) - 0.5 * D2(0)) * inv;
  return (D1(1) - 0.5 * D2(1)) * inv;
}
static real_t eno2_minus(const diffs_t *d, real_t inv) {
  if (fabs(D2(-1)) < fabs(D2(0))) return (D1(0) + 0.5 * D2(-1)) * inv;
  return (D1(0) + 0.5 * D2(0)) * inv;
}

/* ENO3 plus/minus (spatial_derivatives3d.f.in:842-896) */
static real_t eno3_plus(const diffs_t *d, real_t inv) {
  const real_t third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  real_t x = D1(1);
  if (fabs(D2(0)) < fabs(D2(1))) {
    x = x - 0.5 * D2(0);
    x = (fabs(D3(0)) < fabs(D3(1))) ? x - sixth * D3(0) : x - sixth * D3(1);
  } else {
    x = x - 0.5 * D2(1);
    x = (fabs(D3(1)) < fabs(D3(2))) ? x + third * D3(1) : x + third * D3(2);
  }
  return x * inv;
}
static real_t eno3_minus(const diffs_t *d, real_t inv) {
  const real_t third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  real_t x = D1(0);
  if (fabs(D2(-1)) < fabs(D2(0))) {
    x = x + 0.5 * D2(-1);
    x = (fabs(D3(-1)) < fabs(D3(0))) ? x + third * D3(-1) : x + third * D3(0);
  } else {
    x = x + 0.5 * D2(0);
    x = (fabs(D3(0)) < fabs(D3(1))) ? x - sixth * D3(0) : x - sixth * D3(1);
  }
  return x * inv;
}

/* WENO5-JS reconstruction on five scaled differences
 * (spatial_derivatives3d.f.in:1296-1323). */
static real_t weno5(real_t v1, real_t v2, real_t v3, real_t v4, real_t v5) {
  const real_t c13 = 1.0 / 3.0, c76 = 7.0 / 6.0, c116 = 11.0 / 6.0;
  const real_t c16 = 1.0 / 6.0, c56 = 5.0 / 6.0, c1312 = 13.0 / 12.0;
  const real_t c14 = 0.25;
  real_t m = v1 * v1;
  m = fmax2(m, v2 * v2);
  m = fmax2(m, v3 * v3);
  m = fmax2(m, v4 * v4);
  m = fmax2(m, v5 * v5);
  real_t eps = 1e-6 * m + ORACLE_TINY;
  real_t p1 = c13 * v1 - c76 * v2 + c116 * v3;
  real_t p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  real_t p3 = c13 * v3 + c56 * v4 - c16 * v5;
  real_t t;
  t = v1 - 2.0 * v2 + v3;
  real_t S1 = c1312 * (t * t);
  t = v1 - 4.0 * v2 + 3.0 * v3;
  S1 = S1 + c14 * (t * t);
  t = v2 - 2.0 * v3 + v4;
  real_t S2 = c1312 * (t * t);
  t = v2 - v4;
  S2 = S2 + c14 * (t * t);
  t = v3 - 2.0 * v4 + v5;
  real_t S3 = c1312 * (t * t);
  t = 3.0 * v3 - 4.0 * v4 + v5;
  S3 = S3 + c14 * (t * t);
  real_t a1 = 0.1 / ((S1 + eps) * (S1 + eps));
  real_t a2 = 0.6 / ((S2 + eps) * (S2 + eps));
  real_t a3 = 0.3 / ((S3 + eps) * (S3 + eps));
  real_t inv_sum = 1.0 / (a1 + a2 + a3);
  a1 = a1 * inv_sum;
  a2 = a2 * inv_sum;
  a3 = a3 * inv_sum;
  return a1 * p1 + a2 * p2 + a3 * p3;
}
/* plus side uses D1(i+3..i-1), minus side D1(i-2..i+2) (f.in:1286-1367) */
static real_t weno5_plus(const diffs_t *d, real_t inv) {
  return weno5(D1(3) * inv, D1(2) * inv, D1(1) * inv, D1(0) * inv, D1(-1) * inv);
}
static real_t weno5_minus(const diffs_t *d, real_t inv) {
  return weno5(D1(-2) * inv, D1(-1) * inv, D1(0) * inv, D1(1) * inv, D1(2) * inv);
}

/* ---- plus/minus gradient drivers ---------------------------------------- */
typedef real_t (*side_fn)(const diffs_t *, real_t);

static void hj_pm(real_t *pp[3], const gbox *pb, real_t *pm[3], const gbox *mb,
                  const real_t *phi, const gbox *fb_phi, const int fb[6],
                  const real_t dxs[3], int order, side_fn fplus,
                  side_fn fminus) {
  for (int dir = 0; dir < 3; dir++) {
    const real_t inv = 1.0 / dxs[dir];
    const long s = fb_phi->s[dir];
    FOR_BOX(fb[0], fb[1], fb[2], fb[3], fb[4], fb[5]) {
      diffs_t d;
      load_diffs(&d, phi + at(fb_phi, i, j, k), s, order);
      pp[dir][at(pb, i, j, k)] = fplus(&d, inv);
      pm[dir][at(mb, i, j, k)] = fminus(&d, inv);
    }
  }
}

static real_t eno1_plus(const diffs_t *d, real_t inv) { return D1(1) * inv; }
static real_t eno1_minus(const diffs_t *d, real_t inv) { return D1(0) * inv; }

#define PM_ARGS                                                               \
  real_t *phi_x_plus, real_t *phi_y_plus, real_t *phi_z_plus,                 \
      const int *p_ilo, const int *p_ihi, const int *p_jlo, const int *p_jhi, \
      const int *p_klo, const int *p_khi, real_t *phi_x_minus,                \
      real_t *phi_y_minus, real_t *phi_z_minus, const int *m_ilo,             \
      const int *m_ihi, const int *m_jlo, const int *m_jhi, const int *m_klo, \
      const int *m_khi, const real_t *phi, const int *f_ilo,                  \
      const int *f_ihi, const int *f_jlo, const int *f_jhi, const int *f_klo, \
      const int *f_khi
#define SCRATCH_ARGS(n)                                                        \
  real_t *n, const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,      \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi
#define FB_ARGS                                                          \
  const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, \
      const int *klo_fb, const int *khi_fb
#define DX_ARGS const real_t *dx, const real_t *dy, const real_t *dz

#define PM_BODY(order, fp, fm)                                              \
  gbox pb = mk_box(BOX6(p)), mb = mk_box(BOX6(m)), phb = mk_box(BOX6(f));  \
  int fb[6] = {*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb};      \
  real_t dxs[3] = {*dx, *dy, *dz};                                         \
  real_t *pp[3] = {phi_x_plus, phi_y_plus, phi_z_plus};                    \
  real_t *pm[3] = {phi_x_minus, phi_y_minus, phi_z_minus};                 \
  hj_pm(pp, &pb, pm, &mb, phi, &phb, fb, dxs, order, fp, fm)

/* lsm3dHJENO1 (spatial_derivatives3d.f.in:199-368) */
void lsm3dhjeno1_(PM_ARGS, SCRATCH_ARGS(D1), FB_ARGS, DX_ARGS) {
  (void)D1; (void)D1_ilo; (void)D1_ihi; (void)D1_jlo; (void)D1_jhi; (void)D1_klo; (void)D1_khi;
  PM_BODY(1, eno1_plus, eno1_minus);
}
/* lsm3dHJENO2 (spatial_derivatives3d.f.in:393-663) */
void lsm3dhjeno2_(PM_ARGS, SCRATCH_ARGS(D1), SCRATCH_ARGS(D2), FB_ARGS, DX_ARGS) {
  (void)D1; (void)D2;
  PM_BODY(2, eno2_plus, eno2_minus);
}
/* lsm3dHJENO3 (spatial_derivatives3d.f.in:689-1137) */
void lsm3dhjeno3_(PM_ARGS, SCRATCH_ARGS(D1), SCRATCH_ARGS(D2), SCRATCH_ARGS(D3),
                  FB_ARGS, DX_ARGS) {
  (void)D1; (void)D2; (void)D3;
  PM_BODY(3, eno3_plus, eno3_minus);
}
/* lsm3dHJWENO5 (spatial_derivatives3d.f.in:1161-1611) */
void lsm3dhjweno5_(PM_ARGS, SCRATCH_ARGS(D1), FB_ARGS, DX_ARGS) {
  (void)D1;
  PM_BODY(1, weno5_plus, weno5_minus);
}

/* ---- upwind single gradient --------------------------------------------- */
static void hj_upwind(real_t *g[3], const gbox *gb, const real_t *phi,
                      const gbox *phb, const real_t *vel[3], const gbox *vb,
                      const int fb[6], const real_t dxs[3], int order,
                      side_fn fplus, side_fn fminus) {
  for (int dir = 0; dir < 3; dir++) {
    const real_t inv = 1.0 / dxs[dir];
    const long s = phb->s[dir];
    FOR_BOX(fb[0], fb[1], fb[2], fb[3], fb[4], fb[5]) {
      real_t v = vel[dir][at(vb, i, j, k)];
      real_t out;
      if (fabs(v) < ORACLE_ZERO_TOL) {
        out = 0.0;
      } else {
        diffs_t d;
        load_diffs(&d, phi + at(phb, i, j, k), s, order);
        out = (v > 0) ? fminus(&d, inv) : fplus(&d, inv);
      }
      g[dir][at(gb, i, j, k)] = out;
    }
  }
}

#define UP_ARGS                                                              \
  real_t *phi_x, real_t *phi_y, real_t *phi_z, const int *g_ilo,             \
      const int *g_ihi, const int *g_jlo, const int *g_jhi, const int *g_klo,\
      const int *g_khi, const real_t *phi, const int *f_ilo,                 \
      const int *f_ihi, const int *f_jlo, const int *f_jhi, const int *f_klo,\
      const int *f_khi, const real_t *vel_x, const real_t *vel_y,            \
      const real_t *vel_z, const int *v_ilo, const int *v_ihi,               \
      const int *v_jlo, const int *v_jhi, const int *v_klo, const int *v_khi
#define UP_BODY(order, fp, fm)                                              \
  gbox gb = mk_box(BOX6(g)), phb = mk_box(BOX6(f)), vb = mk_box(BOX6(v));  \
  int fb[6] = {*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb};      \
  real_t dxs[3] = {*dx, *dy, *dz};                                         \
  real_t *g[3] = {phi_x, phi_y, phi_z};                                    \
  const real_t *vel[3] = {vel_x, vel_y, vel_z};                            \
  hj_upwind(g, &gb, phi, &phb, vel, &vb, fb, dxs, order, fp, fm)

/* lsm3dUpwindHJENO1 (spatial_derivatives3d.f.in:1630-1834) */
void lsm3dupwindhjeno1_(UP_ARGS, SCRATCH_ARGS(D1), FB_ARGS, DX_ARGS) {
  (void)D1;
  UP_BODY(1, eno1_plus, eno1_minus);
}
/* lsm3dUpwindHJENO2 (spatial_derivatives3d.f.in:1854-2154) */
void lsm3dupwindhjeno2_(UP_ARGS, SCRATCH_ARGS(D1), SCRATCH_ARGS(D2), FB_ARGS, DX_ARGS) {
  (void)D1; (void)D2;
  UP_BODY(2, eno2_plus, eno2_minus);
}
/* lsm3dUpwindHJENO3 (spatial_derivatives3d.f.in:2174-2610) */
void lsm3dupwindhjeno3_(UP_ARGS, SCRATCH_ARGS(D1), SCRATCH_ARGS(D2),
                        SCRATCH_ARGS(D3), FB_ARGS, DX_ARGS) {
  (void)D1; (void)D2; (void)D3;
  UP_BODY(3, eno3_plus, eno3_minus);
}
/* lsm3dUpwindHJWENO5 (spatial_derivatives3d.f.in:2628-3000) */
void lsm3dupwindhjweno5_(UP_ARGS, SCRATCH_ARGS(D1), FB_ARGS, DX_ARGS) {
  (void)D1;
  UP_BODY(1, weno5_plus, weno5_minus);
}

/* ---- central differences ------------------------------------------------- */
#define G3_ARGS                                                              \
  real_t *phi_x, real_t *phi_y, real_t *phi_z, const int *g_ilo,             \
      const int *g_ihi, const int *g_jlo, const int *g_jhi, const int *g_klo,\
      const int *g_khi, const real_t *phi, const int *f_ilo,                 \
      const int *f_ihi, const int *f_jlo, const int *f_jhi, const int *f_klo,\
      const int *f_khi

/* lsm3dCentralGradOrder2 (spatial_derivatives3d.f.in:3016-3077) */
void lsm3dcentralgradorder2_(G3_ARGS, FB_ARGS, DX_ARGS) {
  gbox gb = mk_box(BOX6(g)), pb = mk_box(BOX6(f));
  real_t fac[3] = {0.5 / *dx, 0.5 / *dy, 0.5 / *dz};
  real_t *g[3] = {phi_x, phi_y, phi_z};
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    const real_t *c = phi + at(&pb, i, j, k);
    for (int d = 0; d < 3; d++)
      g[d][at(&gb, i, j, k)] = (c[pb.s[d]] - c[-pb.s[d]]) * fac[d];
  }
}

/* lsm3dCentralGradOrder4 (spatial_derivatives3d.f.in:3094-3163) */
void lsm3dcentralgradorder4_(G3_ARGS, FB_ARGS, DX_ARGS) {
  gbox gb = mk_box(BOX6(g)), pb = mk_box(BOX6(f));
  const real_t c12 = 0.0833333333333333333333;
  real_t fac[3] = {c12 / *dx, c12 / *dy, c12 / *dz};
  real_t *g[3] = {phi_x, phi_y, phi_z};
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    const real_t *c = phi + at(&pb, i, j, k);
    for (int d = 0; d < 3; d++) {
      long s = pb.s[d];
      g[d][at(&gb, i, j, k)] =
          (-c[2 * s] + 8.0 * c[s] + c[-2 * s] - 8.0 * c[-s]) * fac[d];
    }
  }
}

/* lsm3dLaplacianOrder2 (spatial_derivatives3d.f.in:3180-3243) */
void lsm3dlaplacianorder2_(real_t *lap, const int *g_ilo, const int *g_ihi,
                           const int *g_jlo, const int *g_jhi, const int *g_klo,
                           const int *g_khi, const real_t *phi, const int *f_ilo,
                           const int *f_ihi, const int *f_jlo, const int *f_jhi,
                           const int *f_klo, const int *f_khi, FB_ARGS, DX_ARGS) {
  gbox gb = mk_box(BOX6(g)), pb = mk_box(BOX6(f));
  real_t ix = 1.0 / *dx / *dx, iy = 1.0 / *dy / *dy, iz = 1.0 / *dz / *dz;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    const real_t *c = phi + at(&pb, i, j, k);
    long sx = pb.s[0], sy = pb.s[1], sz = pb.s[2];
    lap[at(&gb, i, j, k)] = ix * (c[sx] - 2.0 * c[0] + c[-sx]) +
                            iy * (c[sy] - 2.0 * c[0] + c[-sy]) +
                            iz * (c[sz] - 2.0 * c[0] + c[-sz]);
  }
}

/* lsm3dGradientMagnitude (spatial_derivatives3d.f.in:3586-3659): the four
 * arrays share one ghost box */
void lsm3dgradientmagnitude_(const real_t *phi_x, const real_t *phi_y,
                             const real_t *phi_z, real_t *mag, const int *g_ilo,
                             const int *g_ihi, const int *g_jlo, const int *g_jhi,
                             const int *g_klo, const int *g_khi, FB_ARGS) {
  gbox gb = mk_box(BOX6(g));
  const real_t tol = 1.e-8;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long c = at(&gb, i, j, k);
    real_t x2 = phi_x[c] * phi_x[c], y2 = phi_y[c] * phi_y[c],
           z2 = phi_z[c] * phi_z[c];
    if (x2 < tol) x2 = 0.0;
    if (y2 < tol) y2 = 0.0;
    if (z2 < tol) z2 = 0.0;
    real_t t = sqrt(x2 + y2 + z2);
    mag[c] = (t < tol) ? 0.0 : t;
  }
}

/* ---- TVD Runge-Kutta stages (tvd_runge_kutta3d.f) ------------------------ */
#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo,             \
      const int *n##_jhi, const int *n##_klo, const int *n##_khi

/* lsm3dRK1Step (tvd_runge_kutta3d.f:32-86): u_next = u + dt*L */
void lsm3drk1step_(real_t *u_next, A3(a), const real_t *u_cur, A3(b),
                   const real_t *rhs, A3(c), FB_ARGS, const real_t *dt) {
  gbox A = mk_box(BOX6(a)), B = mk_box(BOX6(b)), C = mk_box(BOX6(c));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb)
    u_next[at(&A, i, j, k)] = u_cur[at(&B, i, j, k)] + *dt * rhs[at(&C, i, j, k)];
}
/* lsm3dTVDRK2Stage1 (tvd_runge_kutta3d.f:107-166) and lsm3dTVDRK3Stage1
 * (:269-328) are both an RK1 step */
void lsm3dtvdrk2stage1_(real_t *u1, A3(a), const real_t *u, A3(b),
                        const real_t *rhs, A3(c), FB_ARGS, const real_t *dt) {
  lsm3drk1step_(u1, BOX6(a), u, BOX6(b), rhs, BOX6(c), ilo_fb, ihi_fb, jlo_fb,
                jhi_fb, klo_fb, khi_fb, dt);
}
void lsm3dtvdrk3stage1_(real_t *u1, A3(a), const real_t *u, A3(b),
                        const real_t *rhs, A3(c), FB_ARGS, const real_t *dt) {
  lsm3drk1step_(u1, BOX6(a), u, BOX6(b), rhs, BOX6(c), ilo_fb, ihi_fb, jlo_fb,
                jhi_fb, klo_fb, khi_fb, dt);
}
/* lsm3dTVDRK2Stage2 (tvd_runge_kutta3d.f:185-248):
 * u_next = 0.5*(u + u1 + dt*L) */
void lsm3dtvdrk2stage2_(real_t *un, A3(a), const real_t *u1, A3(b),
                        const real_t *u, A3(c), const real_t *rhs, A3(d),
                        FB_ARGS, const real_t *dt) {
  gbox A = mk_box(BOX6(a)), B = mk_box(BOX6(b)), C = mk_box(BOX6(c)),
       D = mk_box(BOX6(d));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb)
    un[at(&A, i, j, k)] =
        0.5 * (u[at(&C, i, j, k)] + u1[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
}
/* lsm3dTVDRK3Stage2 (tvd_runge_kutta3d.f:347-412):
 * u2 = 0.75*u + 0.25*(u1 + dt*L) */
void lsm3dtvdrk3stage2_(real_t *u2, A3(a), const real_t *u1, A3(b),
                        const real_t *u, A3(c), const real_t *rhs, A3(d),
                        FB_ARGS, const real_t *dt) {
  gbox A = mk_box(BOX6(a)), B = mk_box(BOX6(b)), C = mk_box(BOX6(c)),
       D = mk_box(BOX6(d));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb)
    u2[at(&A, i, j, k)] = 0.75 * u[at(&C, i, j, k)] +
                          0.25 * (u1[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
}
/* lsm3dTVDRK3Stage3 (tvd_runge_kutta3d.f:431-500):
 * u_next = u/3 + 2/3*(u2 + dt*L) */
void lsm3dtvdrk3stage3_(real_t *un, A3(a), const real_t *u2, A3(b),
                        const real_t *u, A3(c), const real_t *rhs, A3(d),
                        FB_ARGS, const real_t *dt) {
  gbox A = mk_box(BOX6(a)), B = mk_box(BOX6(b)), C = mk_box(BOX6(c)),
       D = mk_box(BOX6(d));
  const real_t c13 = 1.0 / 3.0, c23 = 2.0 / 3.0;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb)
    un[at(&A, i, j, k)] = c13 * u[at(&C, i, j, k)] +
                          c23 * (u2[at(&B, i, j, k)] + *dt * rhs[at(&D, i, j, k)]);
}

/* ---- level set equation right-hand sides (level_set_evolution3d.f.in) ---- */

/* lsm3dZeroOutLevelSetEqnRHS (:16-46) zeroes the whole ghost box */
void lsm3dzerooutlevelseteqnrhs_(real_t *rhs, A3(r)) {
  gbox R = mk_box(BOX6(r));
  FOR_BOX(R.lo[0], R.hi[0], R.lo[1], R.hi[1], R.lo[2], R.hi[2])
    rhs[at(&R, i, j, k)] = 0.0;
}

/* lsm3dAddAdvectionTermToLSERHS (:53-124): rhs -= u.grad(phi) */
void lsm3daddadvectiontermtolserhs_(real_t *rhs, A3(r), const real_t *px,
                                    const real_t *py, const real_t *pz, A3(g),
                                    const real_t *vx, const real_t *vy,
                                    const real_t *vz, A3(v), FB_ARGS) {
  gbox R = mk_box(BOX6(r)), G = mk_box(BOX6(g)), V = mk_box(BOX6(v));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long g = at(&G, i, j, k), v = at(&V, i, j, k), r = at(&R, i, j, k);
    rhs[r] = rhs[r] - (vx[v] * px[g] + vy[v] * py[g] + vz[v] * pz[g]);
  }
}

/* Godunov |grad phi|^2 for a normal speed of the given sign
 * (level_set_evolution3d.f.in:210-223) */
static real_t godunov_sq(real_t vn, const real_t p[3], const real_t m[3]) {
  real_t s = 0.0;
  for (int d = 0; d < 3; d++) {
    real_t a, b;
    if (vn > 0.0) {
      a = fmax2(m[d], 0.0);
      b = fmin2(p[d], 0.0);
    } else {
      a = fmin2(m[d], 0.0);
      b = fmax2(p[d], 0.0);
    }
    real_t t = fmax2(a * a, b * b);
    s = (d == 0) ? t : s + t;
  }
  return s;
}

/* lsm3dAddNormalVelTermToLSERHS (:131-241) */
void lsm3daddnormalveltermtolserhs_(real_t *rhs, A3(r), const real_t *pxp,
                                    const real_t *pyp, const real_t *pzp, A3(p),
                                    const real_t *pxm, const real_t *pym,
                                    const real_t *pzm, A3(m), const real_t *vn,
                                    A3(v), FB_ARGS) {
  gbox R = mk_box(BOX6(r)), P = mk_box(BOX6(p)), M = mk_box(BOX6(m)),
       V = mk_box(BOX6(v));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    real_t w = vn[at(&V, i, j, k)];
    if (fabs(w) >= ORACLE_ZERO_TOL) {
      long a = at(&P, i, j, k), b = at(&M, i, j, k), r = at(&R, i, j, k);
      real_t pp[3] = {pxp[a], pyp[a], pzp[a]}, mm[3] = {pxm[b], pym[b], pzm[b]};
      rhs[r] = rhs[r] - w * sqrt(godunov_sq(w, pp, mm));
    }
  }
}

/* lsm3dAddConstNormalVelTermToLSERHS (:248-349) */
void lsm3daddconstnormalveltermtolserhs_(real_t *rhs, A3(r), const real_t *pxp,
                                         const real_t *pyp, const real_t *pzp,
                                         A3(p), const real_t *pxm,
                                         const real_t *pym, const real_t *pzm,
                                         A3(m), const real_t *vel_n, FB_ARGS) {
  gbox R = mk_box(BOX6(r)), P = mk_box(BOX6(p)), M = mk_box(BOX6(m));
  real_t w = *vel_n;
  if (!(fabs(w) >= ORACLE_ZERO_TOL)) return;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long a = at(&P, i, j, k), b = at(&M, i, j, k), r = at(&R, i, j, k);
    real_t pp[3] = {pxp[a], pyp[a], pzp[a]}, mm[3] = {pxm[b], pym[b], pzm[b]};
    rhs[r] = rhs[r] - w * sqrt(godunov_sq(w, pp, mm));
  }
}

/* curvature numerator phi_xx phi_y^2 + ... - 2 phi_yz phi_y phi_z, in the
 * term order of level_set_evolution3d.f.in:439-447 and
 * curvature3d.f.in:109-117 */
static real_t curv_numerator(real_t xx, real_t yy, real_t zz, real_t xy,
                             real_t xz, real_t yz, real_t x, real_t y, real_t z) {
  return xx * y * y + yy * x * x - 2.0 * xy * x * y + xx * z * z + zz * x * x -
         2.0 * xz * x * z + yy * z * z + zz * y * y - 2.0 * yz * y * z;
}

/* lsm3dAddConstCurvTermToLSERHS (:356-459) */
void lsm3daddconstcurvtermtolserhs_(real_t *rhs, A3(r), const real_t *px,
                                    const real_t *py, const real_t *pz, A3(g),
                                    const real_t *pxx, const real_t *pxy,
                                    const real_t *pxz, const real_t *pyy,
                                    const real_t *pyz, const real_t *pzz, A3(h),
                                    const real_t *b, FB_ARGS) {
  gbox R = mk_box(BOX6(r)), G = mk_box(BOX6(g)), H = mk_box(BOX6(h));
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long g = at(&G, i, j, k), h = at(&H, i, j, k), r = at(&R, i, j, k);
    real_t m2 = px[g] * px[g] + py[g] * py[g] + pz[g] * pz[g];
    real_t curv;
    if (m2 < ORACLE_ZERO_TOL) {
      curv = 0.0;
    } else {
      curv = curv_numerator(pxx[h], pyy[h], pzz[h], pxy[h], pxz[h], pyz[h],
                            px[g], py[g], pz[g]);
      curv = curv / m2;
    }
    rhs[r] = rhs[r] + *b * curv;
  }
}

/* ---- reinitialization (reinitialization3d.f.in:48-267) ------------------- */
void lsm3dcomputereinitializationeqnrhs_(
    real_t *rhs, A3(r), const real_t *phi, A3(f), const real_t *phi0, A3(z),
    const real_t *pxp, const real_t *pyp, const real_t *pzp, A3(p),
    const real_t *pxm, const real_t *pym, const real_t *pzm, A3(m), FB_ARGS,
    DX_ARGS, const int *use_phi0_for_sgn) {
  gbox R = mk_box(BOX6(r)), F = mk_box(BOX6(f)), Z = mk_box(BOX6(z)),
       P = mk_box(BOX6(p)), M = mk_box(BOX6(m));
  real_t dx_sq = fmax2(fmax2(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  const int use0 = (*use_phi0_for_sgn == 1);
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    real_t pc = use0 ? phi0[at(&Z, i, j, k)] : phi[at(&F, i, j, k)];
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t gp[3] = {pxp[a], pyp[a], pzp[a]}, gm[3] = {pxm[b], pym[b], pzm[b]};
    real_t star[3];
    for (int d = 0; d < 3; d++) {
      real_t u, w;
      if (pc > 0.0) {
        u = fmax2(-gp[d], 0.0);
        w = fmax2(gm[d], 0.0);
      } else {
        u = fmax2(gp[d], 0.0);
        w = fmax2(-gm[d], 0.0);
      }
      star[d] = fmax2(u, w);
    }
    real_t out;
    if (fabs(pc) >= ORACLE_ZERO_TOL) {
      real_t n2 = star[0] * star[0] + star[1] * star[1] + star[2] * star[2];
      real_t sgn = use0 ? pc / sqrt(pc * pc + dx_sq)
                        : pc / sqrt(pc * pc + n2 * dx_sq);
      out = sgn * (1.0 - sqrt(n2));
    } else {
      out = 0.0;
    }
    rhs[at(&R, i, j, k)] = out;
  }
}

/* ---- mean curvature (curvature3d.f.in:15-128) ---------------------------- */
void lsm3dcomputemeancurvatureorder2_(
    real_t *kappa, A3(k), const real_t *phi, A3(f), const real_t *px,
    const real_t *py, const real_t *pz, const real_t *mag, A3(g),
    const int *kf_ilo, const int *kf_ihi, const int *kf_jlo, const int *kf_jhi,
    const int *kf_klo, const int *kf_khi, DX_ARGS) {
  gbox K = mk_box(BOX6(k)), F = mk_box(BOX6(f)), G = mk_box(BOX6(g));
  real_t fxx = 1.0 / *dx / *dx, fyy = 1.0 / *dy / *dy, fzz = 1.0 / *dz / *dz;
  real_t fxy = 0.25 / *dx / *dy, fxz = 0.25 / *dx / *dz, fyz = 0.25 / *dy / *dz;
  long sx = F.s[0], sy = F.s[1], sz = F.s[2];
  FOR_BOX(*kf_ilo, *kf_ihi, *kf_jlo, *kf_jhi, *kf_klo, *kf_khi) {
    const real_t *c = phi + at(&F, i, j, k);
    real_t xx = (c[sx] - 2.0 * c[0] + c[-sx]) * fxx;
    real_t yy = (c[sy] - 2.0 * c[0] + c[-sy]) * fyy;
    real_t zz = (c[sz] - 2.0 * c[0] + c[-sz]) * fzz;
    real_t xy = (c[sx + sy] - c[sx - sy] - c[-sx + sy] + c[-sx - sy]) * fxy;
    real_t xz = (c[sx + sz] - c[sx - sz] - c[-sx + sz] + c[-sx - sz]) * fxz;
    real_t yz = (c[sy + sz] - c[sy - sz] - c[-sy + sz] + c[-sy - sz]) * fyz;
    long g = at(&G, i, j, k);
    real_t den = mag[g] * mag[g] * mag[g];
    real_t out;
    if (den < ORACLE_ZERO_TOL)
      out = 0.0;
    else
      out = curv_numerator(xx, yy, zz, xy, xz, yz, px[g], py[g], pz[g]) / den;
    kappa[at(&K, i, j, k)] = out;
  }
}

/* ---- reductions (math_utils3d.f.in) -------------------------------------- */

/* lsm3dMaxNormDiff (:16-75) */
void lsm3dmaxnormdiff_(real_t *out, const real_t *f1, A3(a), const real_t *f2,
                       A3(b), const int *ilo_ib, const int *ihi_ib,
                       const int *jlo_ib, const int *jhi_ib, const int *klo_ib,
                       const int *khi_ib) {
  gbox A = mk_box(BOX6(a)), B = mk_box(BOX6(b));
  real_t m = fabs(f1[at(&A, *ilo_ib, *jlo_ib, *klo_ib)] -
                  f2[at(&B, *ilo_ib, *jlo_ib, *klo_ib)]);
  FOR_BOX(*ilo_ib, *ihi_ib, *jlo_ib, *jhi_ib, *klo_ib, *khi_ib) {
    real_t d = fabs(f1[at(&A, i, j, k)] - f2[at(&B, i, j, k)]);
    if (d > m) m = d;
  }
  *out = m;
}

/* lsm3dComputeStableAdvectionDt (:253-326) */
void lsm3dcomputestableadvectiondt_(real_t *dt, const real_t *vx,
                                    const real_t *vy, const real_t *vz, A3(v),
                                    const int *ilo_ib, const int *ihi_ib,
                                    const int *jlo_ib, const int *jhi_ib,
                                    const int *klo_ib, const int *khi_ib,
                                    DX_ARGS, const real_t *cfl) {
  gbox V = mk_box(BOX6(v));
  real_t ix = 1.0 / *dx, iy = 1.0 / *dy, iz = 1.0 / *dz;
  real_t m = -1.0;
  FOR_BOX(*ilo_ib, *ihi_ib, *jlo_ib, *jhi_ib, *klo_ib, *khi_ib) {
    long c = at(&V, i, j, k);
    real_t u = fabs(vx[c]) * ix + fabs(vy[c]) * iy + fabs(vz[c]) * iz;
    if (u > m) m = u;
  }
  *dt = *cfl / (m + ORACLE_TINY);
}

/* H/dx estimate shared by the two normal-velocity dt routines
 * (math_utils3d.f.in:421-434, :537-551) */
static real_t h_over_dx(real_t avn, const real_t p[3], const real_t m[3],
                        real_t max_dx_sq, const real_t inv[3]) {
  real_t c[3];
  for (int d = 0; d < 3; d++) c[d] = fmax2(fabs(p[d]), fabs(m[d]));
  real_t ng = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + max_dx_sq);
  return avn / ng * (c[0] * inv[0] + c[1] * inv[1] + c[2] * inv[2]);
}

/* lsm3dComputeStableNormalVelDt (:332-449) */
void lsm3dcomputestablenormalveldt_(
    real_t *dt, const real_t *vn, A3(v), const real_t *pxp, const real_t *pyp,
    const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
    const real_t *pzm, A3(m), const int *ilo_ib, const int *ihi_ib,
    const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib,
    DX_ARGS, const real_t *cfl) {
  gbox V = mk_box(BOX6(v)), P = mk_box(BOX6(p)), M = mk_box(BOX6(m));
  real_t mx = fmax2(fmax2(*dx, *dy), *dz);
  real_t max_dx_sq = mx * mx;
  real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz};
  real_t best = -1.0;
  FOR_BOX(*ilo_ib, *ihi_ib, *jlo_ib, *jhi_ib, *klo_ib, *khi_ib) {
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t pp[3] = {pxp[a], pyp[a], pzp[a]}, mm[3] = {pxm[b], pym[b], pzm[b]};
    real_t h = h_over_dx(fabs(vn[at(&V, i, j, k)]), pp, mm, max_dx_sq, inv);
    if (h > best) best = h;
  }
  *dt = *cfl / (best + ORACLE_TINY);
}

/* lsm3dComputeStableConstNormalVelDt (:455-567) */
void lsm3dcomputestableconstnormalveldt_(
    real_t *dt, const real_t *vel_n, const real_t *pxp, const real_t *pyp,
    const real_t *pzp, A3(p), const real_t *pxm, const real_t *pym,
    const real_t *pzm, A3(m), const int *ilo_ib, const int *ihi_ib,
    const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib,
    DX_ARGS, const real_t *cfl) {
  gbox P = mk_box(BOX6(p)), M = mk_box(BOX6(m));
  real_t mx = fmax2(fmax2(*dx, *dy), *dz);
  real_t max_dx_sq = mx * mx;
  real_t inv[3] = {1.0 / *dx, 1.0 / *dy, 1.0 / *dz};
  real_t avn = fabs(*vel_n);
  real_t best = -1.0;
  FOR_BOX(*ilo_ib, *ihi_ib, *jlo_ib, *jhi_ib, *klo_ib, *khi_ib) {
    long a = at(&P, i, j, k), b = at(&M, i, j, k);
    real_t pp[3] = {pxp[a], pyp[a], pzp[a]}, mm[3] = {pxm[b], pym[b], pzm[b]};
    real_t h = h_over_dx(avn, pp, mm, max_dx_sq, inv);
    if (h > best) best = h;
  }
  *dt = *cfl / (best + ORACLE_TINY);
}
