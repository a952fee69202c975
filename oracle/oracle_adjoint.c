/*
 * Reverse-mode gradients of periodic WENO5 / TVD-RK3 advection and
 * reinitialization, FP64, on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker for the GPU adjoint.  Nothing
 * in lsmlib_gb300/ includes or links it.
 *
 * LSMLIB has no adjoint.  The forward map here is LSMLIB's own call sequence
 * for one advection time step on a periodic grid:
 *   upwind WENO5 derivatives   lsm3dUpwindHJWENO5  (spatial_derivatives3d.f.in:2628-3000)
 *   advection RHS              lsm3dZeroOutLevelSetEqnRHS + lsm3dAddAdvectionTermToLSERHS
 *                              (level_set_evolution3d.f.in:38, :113-116)
 *   TVD RK3 stages             tvd_runge_kutta3d.f:78, :403-404, :490-492
 *   periodic ghost fill after every stage (and of the initial state)
 * and, for reinitialization, HJ WENO5 plus/minus with the reinitialization
 * RHS in its phi0 sign form (lsm3dComputeReinitializationEqnRHS,
 * reinitialization3d.f.in:217-256) in place of the advection terms,
 * with every operation in the order the oracle's dense routines use, so the
 * forward states are bit-identical to the oracle's LSMLIB composition.  The
 * objective is
 *   J = sum over interior cells of (H(phi_T) - H(phi_target))^2 * dx*dy*dz
 * with LSMLIB's smoothed Heaviside (lsm_calculus_toolbox.h:41) and its
 * derivative, the smoothed delta function (lsm_calculus_toolbox.h:58).
 *
 * The gradient is the exact derivative of that forward map (dt held fixed),
 * taken by hand in reverse mode: the WENO5 weights, the epsilon = 1e-6 max v^2
 * term (derivative routed to the index the max selects), the upwind switch
 * (derivative of the branch taken; the |v| < zero_tol cut gives zero), and
 * the RK3 stage combination.  The whole state trajectory is kept in memory
 * (this is for small grids).
 *
 * Arrays are compact and periodic: (nx, ny, nz) interior cells, column-major
 * (i fastest), no ghost cells.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_common.h"

/* LSM_HEAVISIDE (lsm_calculus_toolbox.h:41-45) */
double oracle_heaviside(double x, double eps) {
  if (x < -eps) return 0.0;
  if (x > eps) return 1.0;
  return 0.5 * (1 + x / eps + 1 / M_PI * sin(M_PI * x / eps));
}

/* LSM_DELTA_FUNCTION (lsm_calculus_toolbox.h:58-62) */
double oracle_delta(double x, double eps) {
  if (x < -eps) return 0.0;
  if (x > eps) return 0.0;
  return 0.5 / eps * (1 + cos(M_PI * x / eps));
}

typedef struct {
  int n[3];
  double inv[3];
} pgrid;

static inline long pwrap(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}
static inline long pidx(const pgrid *g, int i, int j, int k) {
  return pwrap(i, g->n[0]) + (long)g->n[0] * (pwrap(j, g->n[1]) + (long)g->n[1] * pwrap(k, g->n[2]));
}

/* WENO5 value in the operation order of the oracle's weno5 (the exact form
 * of spatial_derivatives3d.f.in:1296-1323); with dv != NULL also the partial
 * derivatives dW/dv_q.
 *
 * With alpha_k = d_k/(S_k+eps)^2, w_k = alpha_k/sum(alpha), W = sum w_k p_k:
 *   dW = sum_k w_k dp_k + sum_k beta_k (dS_k + deps),
 *   beta_k = -2 w_k (p_k - W) / (S_k + eps),
 * deps = 2e-6 v_m dv_m for the index m that max(v_q^2) selects (the running
 * max keeps the earlier value only when it is strictly larger). */
static double weno5_d(const double v[5], double dv[5]) {
  const double c13 = 1.0 / 3.0, c76 = 7.0 / 6.0, c116 = 11.0 / 6.0;
  const double c16 = 1.0 / 6.0, c56 = 5.0 / 6.0, c1312 = 13.0 / 12.0;
  const double c14 = 0.25;
  const double v1 = v[0], v2 = v[1], v3 = v[2], v4 = v[3], v5 = v[4];
  double m = v1 * v1;
  int am = 0;
  const double sq[5] = {v1 * v1, v2 * v2, v3 * v3, v4 * v4, v5 * v5};
  for (int q = 1; q < 5; q++) {
    if (!(m > sq[q])) am = q;
    m = fmax2(m, sq[q]);
  }
  const double eps = 1e-6 * m + ORACLE_TINY;
  const double p1 = c13 * v1 - c76 * v2 + c116 * v3;
  const double p2 = -(c16 * v2) + c56 * v3 + c13 * v4;
  const double p3 = c13 * v3 + c56 * v4 - c16 * v5;
  const double t1 = v1 - 2.0 * v2 + v3, u1 = v1 - 4.0 * v2 + 3.0 * v3;
  double S1 = c1312 * (t1 * t1);
  S1 = S1 + c14 * (u1 * u1);
  const double t2 = v2 - 2.0 * v3 + v4, u2 = v2 - v4;
  double S2 = c1312 * (t2 * t2);
  S2 = S2 + c14 * (u2 * u2);
  const double t3 = v3 - 2.0 * v4 + v5, u3 = 3.0 * v3 - 4.0 * v4 + v5;
  double S3 = c1312 * (t3 * t3);
  S3 = S3 + c14 * (u3 * u3);
  double a1 = 0.1 / ((S1 + eps) * (S1 + eps));
  double a2 = 0.6 / ((S2 + eps) * (S2 + eps));
  double a3 = 0.3 / ((S3 + eps) * (S3 + eps));
  const double inv_sum = 1.0 / (a1 + a2 + a3);
  a1 = a1 * inv_sum;
  a2 = a2 * inv_sum;
  a3 = a3 * inv_sum;
  const double W = a1 * p1 + a2 * p2 + a3 * p3;
  if (!dv) return W;

  const double b1 = -2.0 * a1 * (p1 - W) / (S1 + eps);
  const double b2 = -2.0 * a2 * (p2 - W) / (S2 + eps);
  const double b3 = -2.0 * a3 * (p3 - W) / (S3 + eps);
  /* dS/dv: S = 13/12 t^2 + 1/4 u^2 -> 13/6 t dt + 1/2 u du */
  const double T1 = 13.0 / 6.0 * t1 * b1, U1 = 0.5 * u1 * b1;
  const double T2 = 13.0 / 6.0 * t2 * b2, U2 = 0.5 * u2 * b2;
  const double T3 = 13.0 / 6.0 * t3 * b3, U3 = 0.5 * u3 * b3;
  dv[0] = c13 * a1 + T1 + U1;
  dv[1] = -c76 * a1 - c16 * a2 - 2.0 * T1 - 4.0 * U1 + T2 + U2;
  dv[2] = c116 * a1 + c56 * a2 + c13 * a3 + T1 + 3.0 * U1 - 2.0 * T2 + T3 + 3.0 * U3;
  dv[3] = c13 * a2 + c56 * a3 + T2 - U2 - 2.0 * T3 - 4.0 * U3;
  dv[4] = -c16 * a3 + T3 + U3;
  dv[am] += (b1 + b2 + b3) * 2e-6 * v[am];
  return W;
}

/* differences along axis d feeding the upwind WENO5 at cell (i,j,k):
 * minus side (vel > 0): v_q = D(c+q-2) for q = 0..4; plus side: v_q = D(c+3-q),
 * with D(f) = (s(f) - s(f-1)) / dx_d.  face[q] is the index offset f of v_q. */
static void upwind_stencil(const pgrid *g, const double *s, int i, int j, int k, int d, int minus,
                           double v[5], int face[5]) {
  for (int q = 0; q < 5; q++) {
    const int f = minus ? q - 2 : 3 - q;
    int a[3] = {i, j, k}, b[3] = {i, j, k};
    a[d] += f;
    b[d] += f - 1;
    v[q] = (s[pidx(g, a[0], a[1], a[2])] - s[pidx(g, b[0], b[1], b[2])]) * g->inv[d];
    face[q] = f;
  }
}

/* rhs = 0 - (u phi_x + v phi_y + w phi_z) with upwinded WENO5 derivatives */
static void adv_rhs(const pgrid *g, const double *s, const double *const vel[3], double *rhs) {
  FOR_BOX(0, g->n[0] - 1, 0, g->n[1] - 1, 0, g->n[2] - 1) {
    const long c = pidx(g, i, j, k);
    double gr[3];
    for (int d = 0; d < 3; d++) {
      const double u = vel[d][c];
      if (fabs(u) < ORACLE_ZERO_TOL) {
        gr[d] = 0.0;
      } else {
        double v[5];
        int face[5];
        upwind_stencil(g, s, i, j, k, d, u > 0.0, v, face);
        gr[d] = weno5_d(v, NULL);
      }
    }
    rhs[c] = 0.0 - (vel[0][c] * gr[0] + vel[1][c] * gr[1] + vel[2][c] * gr[2]);
  }
}

/* acc_s += dt * (dL/ds)^T mu ;  acc_v[d] += dt * (dL/dvel_d)^T mu  (L = rhs) */
static void adv_rhs_adjoint(const pgrid *g, const double *s, const double *const vel[3], const double *mu,
                            double dt, double *acc_s, double *const acc_v[3]) {
  FOR_BOX(0, g->n[0] - 1, 0, g->n[1] - 1, 0, g->n[2] - 1) {
    const long c = pidx(g, i, j, k);
    for (int d = 0; d < 3; d++) {
      const double u = vel[d][c];
      if (fabs(u) < ORACLE_ZERO_TOL) continue;
      double v[5], dv[5];
      int face[5];
      upwind_stencil(g, s, i, j, k, d, u > 0.0, v, face);
      const double W = weno5_d(v, dv);
      if (acc_v) acc_v[d][c] += dt * (mu[c] * -W);
      const double ybar = dt * mu[c] * -u * g->inv[d];
      for (int q = 0; q < 5; q++) {
        int a[3] = {i, j, k}, b[3] = {i, j, k};
        a[d] += face[q];
        b[d] += face[q] - 1;
        const double w = ybar * dv[q];
        acc_s[pidx(g, a[0], a[1], a[2])] += w;
        acc_s[pidx(g, b[0], b[1], b[2])] -= w;
      }
    }
  }
}

/* reinitialization RHS, phi0 sign form (use_phi0_for_sgn = 1), in the
 * operation order of lsm3dcomputereinitializationeqnrhs_
 * (reinitialization3d.f.in:217-256) with HJ WENO5 plus/minus derivatives */
static void reinit_rhs(const pgrid *g, const double *s, const double *phi0, double dx_sq, double *rhs) {
  FOR_BOX(0, g->n[0] - 1, 0, g->n[1] - 1, 0, g->n[2] - 1) {
    const long c = pidx(g, i, j, k);
    double gp[3], gm[3], star[3];
    for (int d = 0; d < 3; d++) {
      double v[5];
      int face[5];
      upwind_stencil(g, s, i, j, k, d, 0, v, face);
      gp[d] = weno5_d(v, NULL);
      upwind_stencil(g, s, i, j, k, d, 1, v, face);
      gm[d] = weno5_d(v, NULL);
    }
    const double pc = phi0[c];
    for (int d = 0; d < 3; d++) {
      double u, w;
      if (pc > 0.0) {
        u = fmax2(-gp[d], 0.0);
        w = fmax2(gm[d], 0.0);
      } else {
        u = fmax2(gp[d], 0.0);
        w = fmax2(-gm[d], 0.0);
      }
      star[d] = fmax2(u, w);
    }
    double out = 0.0;
    if (fabs(pc) >= ORACLE_ZERO_TOL) {
      const double n2 = star[0] * star[0] + star[1] * star[1] + star[2] * star[2];
      const double sgn = pc / sqrt(pc * pc + dx_sq);
      out = sgn * (1.0 - sqrt(n2));
    }
    rhs[c] = out;
  }
}

/* acc_s += dt * (dL/ds)^T mu ; acc_p0 += dt * (dL/dphi0)^T mu  (L = reinit RHS).
 * Per axis the Godunov selection passes the derivative to one of the two
 * WENO5 values (the branch the forward max takes); sgn = phi0/sqrt(phi0^2 +
 * dx^2) gives d sgn/d phi0 = dx^2 / (phi0^2 + dx^2)^(3/2). */
static void reinit_rhs_adjoint(const pgrid *g, const double *s, const double *phi0, double dx_sq, const double *mu,
                               double dt, double *acc_s, double *acc_p0) {
  FOR_BOX(0, g->n[0] - 1, 0, g->n[1] - 1, 0, g->n[2] - 1) {
    const long c = pidx(g, i, j, k);
    const double pc = phi0[c];
    if (!(fabs(pc) >= ORACLE_ZERO_TOL)) continue;
    double vp[3][5], vm[3][5], gp[3], gm[3], star[3];
    int fp[3][5], fm[3][5];
    int which[3]; /* 0: none, 1: plus side, 2: minus side */
    double sel[3];  /* d star / d (selected WENO value) */
    for (int d = 0; d < 3; d++) {
      upwind_stencil(g, s, i, j, k, d, 0, vp[d], fp[d]);
      gp[d] = weno5_d(vp[d], NULL);
      upwind_stencil(g, s, i, j, k, d, 1, vm[d], fm[d]);
      gm[d] = weno5_d(vm[d], NULL);
      double u, w, du, dw;
      if (pc > 0.0) {
        u = fmax2(-gp[d], 0.0); du = (-gp[d] > 0.0) ? -1.0 : 0.0;
        w = fmax2(gm[d], 0.0);  dw = (gm[d] > 0.0) ? 1.0 : 0.0;
      } else {
        u = fmax2(gp[d], 0.0);  du = (gp[d] > 0.0) ? 1.0 : 0.0;
        w = fmax2(-gm[d], 0.0); dw = (-gm[d] > 0.0) ? -1.0 : 0.0;
      }
      if (u > w) {
        star[d] = u; which[d] = du != 0.0 ? 1 : 0; sel[d] = du;
      } else {
        star[d] = w; which[d] = dw != 0.0 ? 2 : 0; sel[d] = dw;
      }
    }
    const double n2 = star[0] * star[0] + star[1] * star[1] + star[2] * star[2];
    const double nrm = sqrt(n2);
    const double den = pc * pc + dx_sq;
    const double sgn = pc / sqrt(den);
    if (acc_p0) acc_p0[c] += dt * mu[c] * (1.0 - nrm) * dx_sq / (den * sqrt(den));
    if (!(nrm > 0.0)) continue;
    for (int d = 0; d < 3; d++) {
      if (!which[d]) continue;
      const double kap = -sgn * star[d] / nrm * sel[d]; /* dL / d(selected WENO value) */
      const double *v = which[d] == 1 ? vp[d] : vm[d];
      const int *face = which[d] == 1 ? fp[d] : fm[d];
      double dv[5];
      weno5_d(v, dv);
      const double ybar = dt * mu[c] * kap * g->inv[d];
      for (int q = 0; q < 5; q++) {
        int a[3] = {i, j, k}, b[3] = {i, j, k};
        a[d] += face[q];
        b[d] += face[q] - 1;
        const double wq = ybar * dv[q];
        acc_s[pidx(g, a[0], a[1], a[2])] += wq;
        acc_s[pidx(g, b[0], b[1], b[2])] -= wq;
      }
    }
  }
}

typedef struct {
  int reinit;                  /* 0: advection, 1: reinitialization (phi0 form) */
  const double *const *vel;    /* advection velocity fields */
  const double *phi0;          /* reinitialization sign source */
  double dx_sq;
} rhs_t;

static void rhs_eval(const rhs_t *r, const pgrid *g, const double *s, double *rhs) {
  if (r->reinit) reinit_rhs(g, s, r->phi0, r->dx_sq, rhs);
  else adv_rhs(g, s, r->vel, rhs);
}

static void rhs_adj(const rhs_t *r, const pgrid *g, const double *s, const double *mu, double dt, double *acc_s,
                    double *const acc_v[3], double *acc_p0) {
  if (r->reinit) reinit_rhs_adjoint(g, s, r->phi0, r->dx_sq, mu, dt, acc_s, acc_p0);
  else adv_rhs_adjoint(g, s, r->vel, mu, dt, acc_s, acc_v);
}

/* one TVD-RK3 step u -> out, keeping u1 and u2 */
static void rk3_step(const rhs_t *r, const pgrid *g, const double *u, double dt, double *u1, double *u2,
                     double *out, double *rhs) {
  const long n = (long)g->n[0] * g->n[1] * g->n[2];
  rhs_eval(r, g, u, rhs);
  for (long c = 0; c < n; c++) u1[c] = u[c] + dt * rhs[c];
  rhs_eval(r, g, u1, rhs);
  for (long c = 0; c < n; c++) u2[c] = 0.75 * u[c] + 0.25 * (u1[c] + dt * rhs[c]);
  rhs_eval(r, g, u2, rhs);
  for (long c = 0; c < n; c++) out[c] = 1.0 / 3.0 * u[c] + 2.0 / 3.0 * (u2[c] + dt * rhs[c]);
}

/* Forward n_steps from phi0 (whole trajectory kept in traj); then, when lam
 * is not NULL, the reverse sweep from lam = dJ/dphi_T, leaving dJ/dphi_0 in
 * lam and the velocity gradients in acc_v (advection) or adding the sign
 * sensitivity to lam (reinitialization: phi0 is also the sign source). */
static void run(const rhs_t *r, const pgrid *g, double dt, int n_steps, double *traj, double *lam,
                double *const acc_v[3]) {
  const long n = (long)g->n[0] * g->n[1] * g->n[2];
  double *u1 = (double *)malloc(sizeof(double) * n), *u2 = (double *)malloc(sizeof(double) * n);
  double *rhs = (double *)malloc(sizeof(double) * n);
  for (int st = 0; st < n_steps; st++)
    rk3_step(r, g, traj + (size_t)st * n, dt, u1, u2, traj + (size_t)(st + 1) * n, rhs);
  if (lam) {
    double *lu1 = (double *)malloc(sizeof(double) * n), *lu2 = (double *)malloc(sizeof(double) * n);
    double *ln = (double *)malloc(sizeof(double) * n), *mu = (double *)malloc(sizeof(double) * n);
    double *p0 = r->reinit ? (double *)calloc((size_t)n, sizeof(double)) : NULL;
    if (acc_v)
      for (int d = 0; d < 3; d++) memset(acc_v[d], 0, sizeof(double) * n);
    for (int st = n_steps - 1; st >= 0; st--) {
      const double *u = traj + (size_t)st * n;
      double *tmp = traj + (size_t)(st + 1) * n; /* recomputed, identical */
      rk3_step(r, g, u, dt, u1, u2, tmp, rhs);
      /* stage 3: out = u/3 + 2/3 (u2 + dt L(u2)) */
      for (long c = 0; c < n; c++) {
        ln[c] = lam[c] / 3.0;
        mu[c] = 2.0 / 3.0 * lam[c];
        lu2[c] = mu[c];
      }
      rhs_adj(r, g, u2, mu, dt, lu2, acc_v, p0);
      /* stage 2: u2 = 3/4 u + 1/4 (u1 + dt L(u1)) */
      for (long c = 0; c < n; c++) {
        ln[c] += 0.75 * lu2[c];
        mu[c] = 0.25 * lu2[c];
        lu1[c] = mu[c];
      }
      rhs_adj(r, g, u1, mu, dt, lu1, acc_v, p0);
      /* stage 1: u1 = u + dt L(u) */
      for (long c = 0; c < n; c++) ln[c] += lu1[c];
      rhs_adj(r, g, u, lu1, dt, ln, acc_v, p0);
      memcpy(lam, ln, sizeof(double) * n);
    }
    if (p0)
      for (long c = 0; c < n; c++) lam[c] += p0[c];
    free(lu1); free(lu2); free(ln); free(mu); free(p0);
  }
  free(u1); free(u2); free(rhs);
}

static pgrid mk_pgrid(int nx, int ny, int nz, double dx, double dy, double dz) {
  pgrid g;
  g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
  g.inv[0] = 1.0 / dx; g.inv[1] = 1.0 / dy; g.inv[2] = 1.0 / dz;
  return g;
}

/* Objective J and (when g_phi is not NULL) its gradient with respect to the
 * initial phi and, when g_vel* are not NULL, the three velocity fields.
 * phi_T (the final state) is written to phi_final when it is not NULL. */
double oracle_advect_objective_adjoint(int nx, int ny, int nz, double dx, double dy, double dz, double dt,
                                       int n_steps, double heaviside_eps, const double *phi0,
                                       const double *vel_x, const double *vel_y, const double *vel_z,
                                       const double *phi_target, double *phi_final, double *g_phi,
                                       double *g_vel_x, double *g_vel_y, double *g_vel_z) {
  const pgrid g = mk_pgrid(nx, ny, nz, dx, dy, dz);
  const long n = (long)nx * ny * nz;
  const double *const vel[3] = {vel_x, vel_y, vel_z};
  const rhs_t r = {0, vel, NULL, 0.0};
  double *traj = (double *)malloc(sizeof(double) * n * (size_t)(n_steps + 1));
  memcpy(traj, phi0, sizeof(double) * n);
  run(&r, &g, dt, n_steps, traj, NULL, NULL);
  const double *phiT = traj + (size_t)n_steps * n;
  if (phi_final) memcpy(phi_final, phiT, sizeof(double) * n);
  const double vol = dx * dy * dz;
  double sum = 0.0;
  double *lam = (double *)calloc((size_t)n, sizeof(double));
  for (long c = 0; c < n; c++) {
    const double h = oracle_heaviside(phiT[c], heaviside_eps) - oracle_heaviside(phi_target[c], heaviside_eps);
    sum += h * h;
    lam[c] = 2.0 * h * oracle_delta(phiT[c], heaviside_eps) * vol;
  }
  const double J = sum * vol;
  if (g_phi) {
    double *const acc_v[3] = {g_vel_x, g_vel_y, g_vel_z};
    memcpy(traj, phi0, sizeof(double) * n);
    run(&r, &g, dt, n_steps, traj, lam, (g_vel_x && g_vel_y && g_vel_z) ? acc_v : NULL);
    memcpy(g_phi, lam, sizeof(double) * n);
  }
  free(lam);
  free(traj);
  return J;
}

/* Vector-Jacobian product of n_steps periodic advection steps:
 * g_phi = (d phi_T / d phi)^T grad_out, g_vel_d = (d phi_T / d vel_d)^T grad_out. */
void oracle_advect_vjp(int nx, int ny, int nz, double dx, double dy, double dz, double dt, int n_steps,
                       const double *phi, const double *vel_x, const double *vel_y, const double *vel_z,
                       const double *grad_out, double *phi_final, double *g_phi, double *g_vel_x,
                       double *g_vel_y, double *g_vel_z) {
  const pgrid g = mk_pgrid(nx, ny, nz, dx, dy, dz);
  const long n = (long)nx * ny * nz;
  const double *const vel[3] = {vel_x, vel_y, vel_z};
  const rhs_t r = {0, vel, NULL, 0.0};
  double *traj = (double *)malloc(sizeof(double) * n * (size_t)(n_steps + 1));
  memcpy(traj, phi, sizeof(double) * n);
  memcpy(g_phi, grad_out, sizeof(double) * n);
  double *const acc_v[3] = {g_vel_x, g_vel_y, g_vel_z};
  run(&r, &g, dt, n_steps, traj, g_phi, (g_vel_x && g_vel_y && g_vel_z) ? acc_v : NULL);
  if (phi_final) memcpy(phi_final, traj + (size_t)n_steps * n, sizeof(double) * n);
  free(traj);
}

/* Vector-Jacobian product of n_steps periodic reinitialization iterations
 * (phi0 sign form: the sign source is the initial phi, so its sensitivity is
 * part of the gradient); pseudo-time step dtau, dx_sq = max(dx, dy, dz)^2. */
void oracle_reinit_vjp(int nx, int ny, int nz, double dx, double dy, double dz, double dtau, int n_steps,
                       const double *phi, const double *grad_out, double *phi_final, double *g_phi) {
  const pgrid g = mk_pgrid(nx, ny, nz, dx, dy, dz);
  const long n = (long)nx * ny * nz;
  double m = fmax2(fmax2(dx, dy), dz);
  const rhs_t r = {1, NULL, phi, m * m};
  double *traj = (double *)malloc(sizeof(double) * n * (size_t)(n_steps + 1));
  memcpy(traj, phi, sizeof(double) * n);
  memcpy(g_phi, grad_out, sizeof(double) * n);
  run(&r, &g, dtau, n_steps, traj, g_phi, NULL);
  if (phi_final) memcpy(phi_final, traj + (size_t)n_steps * n, sizeof(double) * n);
  free(traj);
}
