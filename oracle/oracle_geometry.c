/*
 * CPU oracle: geometry and integral reductions (TEST INFRASTRUCTURE ONLY).
 *
 * Restates, in the reference's serial (k, j, i) order and operation order:
 *  - lsm_math_utils3d.f.in: AveAbsDiff (:81), VoxelCount{Greater,Less}ThanZero
 *    (:154, :203), VolumeIntegralPhi{Less,Greater}ThanZero (:573, :659),
 *    SurfaceIntegral (:745) and the control-volume variants (:852-2008);
 *  - lsm_geometry3d_fort.f.in: ComputeUnitNormal (:27), ComputeSignedUnitNormal
 *    (:129), ComputeMeanCurvature (:274), VolumeRegionPhi{Less,Greater}ThanZero
 *    (:395, :484), SurfaceAreaZeroLevelSet (:574), SurfaceAreaZeroLevelSetDelta
 *    (:669) and the control-volume variants (:770-1330).
 * A control-volume variant includes a cell when control_vol > 0 for
 * control_vol_sgn > 0 and when control_vol < 0 otherwise.
 */
#include "oracle_common.h"

#define A3(n)                                                             \
  const int *n##_ilo, const int *n##_ihi, const int *n##_jlo, const int *n##_jhi, \
      const int *n##_klo, const int *n##_khi
#define B3(n) mk_box(n##_ilo, n##_ihi, n##_jlo, n##_jhi, n##_klo, n##_khi)
#define IB_ARGS                                                               \
  const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, \
      const int *klo_ib, const int *khi_ib
#define FOR_IB FOR_BOX(*ilo_ib, *ihi_ib, *jlo_ib, *jhi_ib, *klo_ib, *khi_ib)
#define DX_ARGS const real_t *dx, const real_t *dy, const real_t *dz

/* parameters of the reference routines (e.g. math_utils3d.f.in:616-619) */
static const real_t PI = 3.14159265358979323846;
static const real_t ONE_OVER_PI = 0.31830988618379;

static int cv_in(const real_t *cv, const gbox *C, int sgn, int i, int j, int k) {
  real_t v = cv[at(C, i, j, k)];
  return sgn > 0 ? v > 0.0 : v < 0.0;
}

/* smoothed 1 - H(phi) and H(phi) (math_utils3d.f.in:636-644, :722-730) */
static real_t one_minus_h(real_t p, real_t eps) {
  real_t q = p / eps;
  return 0.5 * (1.0 - q - ONE_OVER_PI * sin(PI * q));
}
static real_t h_of(real_t p, real_t eps) {
  real_t q = p / eps;
  return 0.5 * (1.0 + q + ONE_OVER_PI * sin(PI * q));
}
/* smoothed delta (math_utils3d.f.in:826-827) */
static real_t delta_of(real_t p, real_t one_over_eps) {
  return 0.5 * one_over_eps * (1.0 + cos(PI * p * one_over_eps));
}
static real_t norm3(const real_t *x, const real_t *y, const real_t *z, long c) {
  return sqrt(x[c] * x[c] + y[c] * y[c] + z[c] * z[c]);
}

/* ---- math_utils3d.f.in ------------------------------------------------------ */

/* lsm3dAveAbsDiff (:81-150) */
void lsm3daveabsdiff_(real_t *out, const real_t *f1, A3(a), const real_t *f2, A3(b), IB_ARGS) {
  gbox A = B3(a), B = B3(b);
  real_t s = 0.0, n = 0.0;
  FOR_IB {
    s = s + fabs(f1[at(&A, i, j, k)] - f2[at(&B, i, j, k)]);
    n = n + 1.0;
  }
  *out = n > 0.0 ? s / n : 0.0;
}

/* lsm3dVoxelCount{Greater,Less}ThanZero (:154-249) and the control-volume
 * variants (:1849-2008); sgn 0 selects the plain routine */
static int voxel_count(const real_t *phi, const gbox *G, const real_t *cv, const gbox *C, int sgn,
                       int greater, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib,
                       const int *jhi_ib, const int *klo_ib, const int *khi_ib) {
  int n = 0;
  FOR_IB {
    real_t p = phi[at(G, i, j, k)];
    if (!(greater ? p > 0.0 : p < 0.0)) continue;
    if (cv && !cv_in(cv, C, sgn, i, j, k)) continue;
    n = n + 1;
  }
  return n;
}

void lsm3dvoxelcountgreaterthanzero_(int *count, const real_t *phi, A3(g), IB_ARGS) {
  gbox G = B3(g);
  *count = voxel_count(phi, &G, 0, 0, 0, 1, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dvoxelcountlessthanzero_(int *count, const real_t *phi, A3(g), IB_ARGS) {
  gbox G = B3(g);
  *count = voxel_count(phi, &G, 0, 0, 0, 0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dvoxelcountgreaterthanzerocontrolvolume_(int *count, const real_t *phi, A3(g), const real_t *cv,
                                                  A3(c), const int *sgn, IB_ARGS) {
  gbox G = B3(g), C = B3(c);
  *count = voxel_count(phi, &G, cv, &C, *sgn > 0 ? 1 : -1, 1, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib,
                       khi_ib);
}
void lsm3dvoxelcountlessthanzerocontrolvolume_(int *count, const real_t *phi, A3(g), const real_t *cv,
                                               A3(c), const int *sgn, IB_ARGS) {
  gbox G = B3(g), C = B3(c);
  *count = voxel_count(phi, &G, cv, &C, *sgn > 0 ? 1 : -1, 0, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib,
                       khi_ib);
}

/* lsm3dVolumeIntegralPhi{Less,Greater}ThanZero (:573-655, :659-741) and their
 * control-volume variants (:1420-1552, :1556-1687) */
static real_t volume_integral(const real_t *F, const gbox *FB, const real_t *phi, const gbox *P,
                              const real_t *cv, const gbox *C, int sgn, int less, real_t dv,
                              real_t eps, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib,
                              const int *jhi_ib, const int *klo_ib, const int *khi_ib) {
  real_t s = 0.0;
  FOR_IB {
    if (cv && !cv_in(cv, C, sgn, i, j, k)) continue;
    real_t p = phi[at(P, i, j, k)];
    if (less) {
      if (p < -eps)
        s = s + F[at(FB, i, j, k)] * dv;
      else if (p < eps)
        s = s + one_minus_h(p, eps) * F[at(FB, i, j, k)] * dv;
    } else {
      if (p > eps)
        s = s + F[at(FB, i, j, k)] * dv;
      else if (p > -eps)
        s = s + h_of(p, eps) * F[at(FB, i, j, k)] * dv;
    }
  }
  return s;
}

void lsm3dvolumeintegralphilessthanzero_(real_t *out, const real_t *F, A3(f), const real_t *phi, A3(p),
                                         IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox FB = B3(f), P = B3(p);
  *out = volume_integral(F, &FB, phi, &P, 0, 0, 0, 1, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib,
                         jhi_ib, klo_ib, khi_ib);
}
void lsm3dvolumeintegralphigreaterthanzero_(real_t *out, const real_t *F, A3(f), const real_t *phi,
                                            A3(p), IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox FB = B3(f), P = B3(p);
  *out = volume_integral(F, &FB, phi, &P, 0, 0, 0, 0, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib,
                         jhi_ib, klo_ib, khi_ib);
}
void lsm3dvolumeintegralphilessthanzerocontrolvolume_(real_t *out, const real_t *F, A3(f), const real_t *phi,
                                                      A3(p), const real_t *cv, A3(c), const int *sgn,
                                                      IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox FB = B3(f), P = B3(p), C = B3(c);
  *out = volume_integral(F, &FB, phi, &P, cv, &C, *sgn > 0 ? 1 : -1, 1, *dx * *dy * *dz, *eps, ilo_ib,
                         ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dvolumeintegralphigreaterthanzerocontrolvolume_(real_t *out, const real_t *F, A3(f),
                                                         const real_t *phi, A3(p), const real_t *cv,
                                                         A3(c), const int *sgn, IB_ARGS, DX_ARGS,
                                                         const real_t *eps) {
  gbox FB = B3(f), P = B3(p), C = B3(c);
  *out = volume_integral(F, &FB, phi, &P, cv, &C, *sgn > 0 ? 1 : -1, 0, *dx * *dy * *dz, *eps, ilo_ib,
                         ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}

/* lsm3dSurfaceIntegral (:745-848) and its control-volume variant (:1691-1845) */
static real_t surface_integral(const real_t *F, const gbox *FB, const real_t *phi, const gbox *P,
                               const real_t *px, const real_t *py, const real_t *pz, const gbox *G,
                               const real_t *cv, const gbox *C, int sgn, real_t dv, real_t eps,
                               const int *ilo_ib, const int *ihi_ib, const int *jlo_ib,
                               const int *jhi_ib, const int *klo_ib, const int *khi_ib) {
  real_t one_over_eps = 1.0 / eps, s = 0.0;
  FOR_IB {
    if (cv && !cv_in(cv, C, sgn, i, j, k)) continue;
    real_t p = phi[at(P, i, j, k)];
    if (fabs(p) < eps) {
      real_t delta = delta_of(p, one_over_eps);
      real_t ng = norm3(px, py, pz, at(G, i, j, k));
      s = s + delta * ng * F[at(FB, i, j, k)] * dv;
    }
  }
  return s;
}

void lsm3dsurfaceintegral_(real_t *out, const real_t *F, A3(f), const real_t *phi, A3(p), const real_t *px,
                           const real_t *py, const real_t *pz, A3(g), IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox FB = B3(f), P = B3(p), G = B3(g);
  *out = surface_integral(F, &FB, phi, &P, px, py, pz, &G, 0, 0, 0, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib,
                          jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dsurfaceintegralcontrolvolume_(real_t *out, const real_t *F, A3(f), const real_t *phi, A3(p),
                                        const real_t *px, const real_t *py, const real_t *pz, A3(g),
                                        const real_t *cv, A3(c), const int *sgn, IB_ARGS, DX_ARGS,
                                        const real_t *eps) {
  gbox FB = B3(f), P = B3(p), G = B3(g), C = B3(c);
  *out = surface_integral(F, &FB, phi, &P, px, py, pz, &G, cv, &C, *sgn > 0 ? 1 : -1, *dx * *dy * *dz,
                          *eps, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}

/* lsm3dMaxNormDiffControlVolume (:852-956): seeded with the (ilo, jlo, klo)
 * corner whatever its control volume */
void lsm3dmaxnormdiffcontrolvolume_(real_t *out, const real_t *f1, A3(a), const real_t *f2, A3(b),
                                    const real_t *cv, A3(c), const int *sgn, IB_ARGS) {
  gbox A = B3(a), B = B3(b), C = B3(c);
  int s = *sgn > 0 ? 1 : -1;
  real_t m = fabs(f1[at(&A, *ilo_ib, *jlo_ib, *klo_ib)] - f2[at(&B, *ilo_ib, *jlo_ib, *klo_ib)]);
  FOR_IB {
    if (!cv_in(cv, &C, s, i, j, k)) continue;
    real_t d = fabs(f1[at(&A, i, j, k)] - f2[at(&B, i, j, k)]);
    if (d > m) m = d;
  }
  *out = m;
}

/* lsm3dComputeStableAdvectionDtControlVolume (:960-1076) */
void lsm3dcomputestableadvectiondtcontrolvolume_(real_t *dt, const real_t *vx, const real_t *vy,
                                                 const real_t *vz, A3(v), const real_t *cv, A3(c),
                                                 const int *sgn, IB_ARGS, DX_ARGS, const real_t *cfl) {
  gbox V = B3(v), C = B3(c);
  int s = *sgn > 0 ? 1 : -1;
  real_t ix = 1.0 / *dx, iy = 1.0 / *dy, iz = 1.0 / *dz, m = -1.0;
  FOR_IB {
    if (!cv_in(cv, &C, s, i, j, k)) continue;
    long q = at(&V, i, j, k);
    real_t u = fabs(vx[q]) * ix + fabs(vy[q]) * iy + fabs(vz[q]) * iz;
    if (u > m) m = u;
  }
  *dt = *cfl / (m + ORACLE_TINY);
}

/* H/dx of the normal-velocity dt routines (:1168-1181, :1340-1351) */
static real_t h_over_dx(real_t avn, long a, long b, const real_t *pxp, const real_t *pyp,
                        const real_t *pzp, const real_t *pxm, const real_t *pym, const real_t *pzm,
                        real_t max_dx_sq, real_t ix, real_t iy, real_t iz) {
  real_t cx = fmax2(fabs(pxp[a]), fabs(pxm[b]));
  real_t cy = fmax2(fabs(pyp[a]), fabs(pym[b]));
  real_t cz = fmax2(fabs(pzp[a]), fabs(pzm[b]));
  real_t ng = sqrt(cx * cx + cy * cy + cz * cz + max_dx_sq);
  return avn / ng * (cx * ix + cy * iy + cz * iz);
}

/* lsm3dComputeStable{,Const}NormalVelDtControlVolume (:1080-1251, :1255-1416) */
static void normal_dt_cv(real_t *dt, const real_t *vn, const gbox *V, real_t vconst, const real_t *pxp,
                         const real_t *pyp, const real_t *pzp, const gbox *P, const real_t *pxm,
                         const real_t *pym, const real_t *pzm, const gbox *M, const real_t *cv,
                         const gbox *C, int sgn, const int *ilo_ib, const int *ihi_ib,
                         const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib,
                         real_t dx, real_t dy, real_t dz, real_t cfl) {
  real_t mx = fmax2(fmax2(dx, dy), dz), max_dx_sq = mx * mx;
  real_t ix = 1.0 / dx, iy = 1.0 / dy, iz = 1.0 / dz, best = -1.0;
  int s = sgn > 0 ? 1 : -1;
  FOR_IB {
    if (!cv_in(cv, C, s, i, j, k)) continue;
    real_t avn = vn ? fabs(vn[at(V, i, j, k)]) : fabs(vconst);
    real_t h = h_over_dx(avn, at(P, i, j, k), at(M, i, j, k), pxp, pyp, pzp, pxm, pym, pzm, max_dx_sq, ix,
                         iy, iz);
    if (h > best) best = h;
  }
  *dt = cfl / (best + ORACLE_TINY);
}

void lsm3dcomputestablenormalveldtcontrolvolume_(real_t *dt, const real_t *vn, A3(v), const real_t *pxp,
                                                 const real_t *pyp, const real_t *pzp, A3(p),
                                                 const real_t *pxm, const real_t *pym, const real_t *pzm,
                                                 A3(m), const real_t *cv, A3(c), const int *sgn, IB_ARGS,
                                                 DX_ARGS, const real_t *cfl) {
  gbox V = B3(v), P = B3(p), M = B3(m), C = B3(c);
  normal_dt_cv(dt, vn, &V, 0.0, pxp, pyp, pzp, &P, pxm, pym, pzm, &M, cv, &C, *sgn, ilo_ib, ihi_ib, jlo_ib,
               jhi_ib, klo_ib, khi_ib, *dx, *dy, *dz, *cfl);
}
void lsm3dcomputestableconstnormalveldtcontrolvolume_(real_t *dt, const real_t *vel_n, const real_t *pxp,
                                                      const real_t *pyp, const real_t *pzp, A3(p),
                                                      const real_t *pxm, const real_t *pym,
                                                      const real_t *pzm, A3(m), const real_t *cv, A3(c),
                                                      const int *sgn, IB_ARGS, DX_ARGS, const real_t *cfl) {
  gbox P = B3(p), M = B3(m), C = B3(c);
  normal_dt_cv(dt, 0, 0, *vel_n, pxp, pyp, pzp, &P, pxm, pym, pzm, &M, cv, &C, *sgn, ilo_ib, ihi_ib, jlo_ib,
               jhi_ib, klo_ib, khi_ib, *dx, *dy, *dz, *cfl);
}

/* ---- geometry3d_fort.f.in ---------------------------------------------------- */

/* lsm3dComputeUnitNormal (:27-125) */
void lsm3dcomputeunitnormal_(real_t *nx, real_t *ny, real_t *nz, A3(n), const real_t *px, const real_t *py,
                             const real_t *pz, A3(g), const int *ilo_fb, const int *ihi_fb,
                             const int *jlo_fb, const int *jhi_fb, const int *klo_fb, const int *khi_fb) {
  gbox N = B3(n), G = B3(g);
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long g = at(&G, i, j, k), o = at(&N, i, j, k);
    real_t ng = norm3(px, py, pz, g);
    if (ng >= ORACLE_ZERO_TOL) {
      real_t inv = 1.0 / ng;
      nx[o] = px[g] * inv;
      ny[o] = py[g] * inv;
      nz[o] = pz[g] * inv;
    } else {
      nx[o] = 1.0;
      ny[o] = 0.0;
      nz[o] = 0.0;
    }
  }
}

/* lsm3dComputeSignedUnitNormal (:129-270) */
void lsm3dcomputesignedunitnormal_(real_t *nx, real_t *ny, real_t *nz, A3(n), const real_t *px,
                                   const real_t *py, const real_t *pz, A3(g), const real_t *phi, A3(f),
                                   const int *ilo_fb, const int *ihi_fb, const int *jlo_fb,
                                   const int *jhi_fb, const int *klo_fb, const int *khi_fb, DX_ARGS) {
  gbox N = B3(n), G = B3(g), F = B3(f);
  real_t dx_sq = fmax2(fmax2(*dx, *dy), *dz);
  dx_sq = dx_sq * dx_sq;
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long g = at(&G, i, j, k), o = at(&N, i, j, k);
    real_t p = phi[at(&F, i, j, k)];
    if (fabs(p) > ORACLE_ZERO_TOL) {
      real_t ngs = px[g] * px[g] + py[g] * py[g] + pz[g] * pz[g];
      if (ngs >= ORACLE_ZERO_TOL) {
        real_t sgn = p / sqrt(p * p + ngs * dx_sq);
        real_t inv = 1.0 / sqrt(ngs);
        nx[o] = sgn * px[g] * inv;
        ny[o] = sgn * py[g] * inv;
        nz[o] = sgn * pz[g] * inv;
      } else {
        nx[o] = 1.0;
        ny[o] = 0.0;
        nz[o] = 0.0;
      }
    } else {
      nx[o] = 0.0;
      ny[o] = 0.0;
      nz[o] = 0.0;
    }
  }
}

/* lsm3dComputeMeanCurvature (:274-391): numerator over |grad phi|^3 written as
 * norm_grad_phi_sq ** 1.5 */
void lsm3dcomputemeancurvature_(real_t *kappa, A3(k), const real_t *px, const real_t *py, const real_t *pz,
                                A3(g), const real_t *pxx, const real_t *pxy, const real_t *pxz,
                                const real_t *pyy, const real_t *pyz, const real_t *pzz, A3(h),
                                const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb,
                                const int *klo_fb, const int *khi_fb) {
  gbox K = B3(k), G = B3(g), H = B3(h);
  FOR_BOX(*ilo_fb, *ihi_fb, *jlo_fb, *jhi_fb, *klo_fb, *khi_fb) {
    long g = at(&G, i, j, k), h = at(&H, i, j, k);
    real_t x = px[g], y = py[g], z = pz[g];
    real_t ngs = x * x + y * y + z * z;
    if (ngs < ORACLE_ZERO_TOL) {
      kappa[at(&K, i, j, k)] = 0.0;
    } else {
      real_t num = pxx[h] * y * y - 2.0 * pxy[h] * x * y + pyy[h] * x * x + pxx[h] * z * z -
                   2.0 * pxz[h] * x * z + pzz[h] * x * x + pyy[h] * z * z - 2.0 * pyz[h] * y * z +
                   pzz[h] * y * y;
      kappa[at(&K, i, j, k)] = num / pow(ngs, 1.5);
    }
  }
}

/* lsm3dVolumeRegionPhi{Less,Greater}ThanZero (:395-480, :484-570) and the
 * control-volume variants (:770-912, :916-1057) */
static real_t volume_region(const real_t *phi, const gbox *P, const real_t *cv, const gbox *C, int sgn,
                            int less, real_t dv, real_t eps, const int *ilo_ib, const int *ihi_ib,
                            const int *jlo_ib, const int *jhi_ib, const int *klo_ib, const int *khi_ib) {
  real_t v = 0.0;
  FOR_IB {
    if (cv && !cv_in(cv, C, sgn, i, j, k)) continue;
    real_t p = phi[at(P, i, j, k)];
    if (less) {
      if (p < -eps)
        v = v + dv;
      else if (p < eps)
        v = v + one_minus_h(p, eps) * dv;
    } else {
      if (p > eps)
        v = v + dv;
      else if (p > -eps)
        v = v + h_of(p, eps) * dv;
    }
  }
  return v;
}

void lsm3dvolumeregionphilessthanzero_(real_t *out, const real_t *phi, A3(p), IB_ARGS, DX_ARGS,
                                       const real_t *eps) {
  gbox P = B3(p);
  *out = volume_region(phi, &P, 0, 0, 0, 1, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib,
                       khi_ib);
}
void lsm3dvolumeregionphigreaterthanzero_(real_t *out, const real_t *phi, A3(p), IB_ARGS, DX_ARGS,
                                          const real_t *eps) {
  gbox P = B3(p);
  *out = volume_region(phi, &P, 0, 0, 0, 0, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib,
                       khi_ib);
}
void lsm3dvolumeregionphilessthanzerocontrolvolume_(real_t *out, const real_t *phi, A3(p), const real_t *cv,
                                                    A3(c), const int *sgn, IB_ARGS, DX_ARGS,
                                                    const real_t *eps) {
  gbox P = B3(p), C = B3(c);
  *out = volume_region(phi, &P, cv, &C, *sgn > 0 ? 1 : -1, 1, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib,
                       jhi_ib, klo_ib, khi_ib);
}
void lsm3dvolumeregionphigreaterthanzerocontrolvolume_(real_t *out, const real_t *phi, A3(p),
                                                       const real_t *cv, A3(c), const int *sgn, IB_ARGS,
                                                       DX_ARGS, const real_t *eps) {
  gbox P = B3(p), C = B3(c);
  *out = volume_region(phi, &P, cv, &C, *sgn > 0 ? 1 : -1, 0, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib,
                       jhi_ib, klo_ib, khi_ib);
}

/* lsm3dSurfaceAreaZeroLevelSet{,Delta} (:574-665, :669-753) and the
 * control-volume variants (:1061-1205, :1209-1330).  The delta form reads a
 * precomputed delta function and includes cells where it is positive. */
static real_t surface_area(const real_t *phi, const gbox *P, int delta_form, const real_t *px,
                           const real_t *py, const real_t *pz, const gbox *G, const real_t *cv,
                           const gbox *C, int sgn, real_t dv, real_t eps, const int *ilo_ib,
                           const int *ihi_ib, const int *jlo_ib, const int *jhi_ib, const int *klo_ib,
                           const int *khi_ib) {
  real_t one_over_eps = delta_form ? 0.0 : 1.0 / eps, a = 0.0;
  FOR_IB {
    if (cv && !cv_in(cv, C, sgn, i, j, k)) continue;
    real_t p = phi[at(P, i, j, k)];
    if (delta_form) {
      if (p > 0.0) a = a + p * norm3(px, py, pz, at(G, i, j, k)) * dv;
    } else if (fabs(p) < eps) {
      real_t delta = delta_of(p, one_over_eps);
      a = a + delta * norm3(px, py, pz, at(G, i, j, k)) * dv;
    }
  }
  return a;
}

void lsm3dsurfaceareazerolevelset_(real_t *out, const real_t *phi, A3(p), const real_t *px, const real_t *py,
                                   const real_t *pz, A3(g), IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox P = B3(p), G = B3(g);
  *out = surface_area(phi, &P, 0, px, py, pz, &G, 0, 0, 0, *dx * *dy * *dz, *eps, ilo_ib, ihi_ib, jlo_ib,
                      jhi_ib, klo_ib, khi_ib);
}
void lsm3dsurfaceareazerolevelsetdelta_(real_t *out, const real_t *delta_phi, A3(p), const real_t *px,
                                        const real_t *py, const real_t *pz, A3(g), IB_ARGS, DX_ARGS) {
  gbox P = B3(p), G = B3(g);
  *out = surface_area(delta_phi, &P, 1, px, py, pz, &G, 0, 0, 0, *dx * *dy * *dz, 0.0, ilo_ib, ihi_ib,
                      jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dsurfaceareazerolevelsetcontrolvolume_(real_t *out, const real_t *phi, A3(p), const real_t *px,
                                                const real_t *py, const real_t *pz, A3(g), const real_t *cv,
                                                A3(c), const int *sgn, IB_ARGS, DX_ARGS, const real_t *eps) {
  gbox P = B3(p), G = B3(g), C = B3(c);
  *out = surface_area(phi, &P, 0, px, py, pz, &G, cv, &C, *sgn > 0 ? 1 : -1, *dx * *dy * *dz, *eps, ilo_ib,
                      ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}
void lsm3dsurfaceareazerolevelsetdeltacontrolvolume_(real_t *out, const real_t *delta_phi, A3(p),
                                                     const real_t *px, const real_t *py, const real_t *pz,
                                                     A3(g), const real_t *cv, A3(c), const int *sgn,
                                                     IB_ARGS, DX_ARGS) {
  gbox P = B3(p), G = B3(g), C = B3(c);
  *out = surface_area(delta_phi, &P, 1, px, py, pz, &G, cv, &C, *sgn > 0 ? 1 : -1, *dx * *dy * *dz, 0.0,
                      ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib);
}
