/*
 * A C program written against LSMLIB's own headers, the way LSMLIB's example
 * drivers are (examples/curvature_driven_motion/curvature_model3d.c:484-625,
 * reinitializeMedium3d): a Grid from createGridSetDx, host arrays over its
 * ghost box, and a pseudo-time loop of HJ WENO5 plus/minus derivatives ->
 * reinitialization right-hand side -> TVD RK2 stages with signed linear
 * extrapolation on all six faces after each stage.  The level set is
 * (|x| - 0.5)(0.1 + (x-0.3)^2 + (y-0.3)^2 + (z+0.2)^2) on [-1, 1]^3.
 *
 * Built against LSMLIB's headers it links to any library that exports
 * LSMLIB's symbols (the reference's own objects, or liblsmgpu.so).  With
 * -DLSMGPU_HEADERS it is built against this library's headers instead,
 * which declare the same symbols; the names LSMLIB's headers define as
 * macros are mapped below, and nothing else in the program changes.
 *
 *   reinit_weno5 <cells per side> <iterations> <output file>
 * writes the final phi over the ghost box (num_gridpts doubles).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#ifdef LSMGPU_HEADERS
#include "lsmgpu_io.h"
#include "lsmgpu_toolbox3d.h"
typedef LsmgpuGrid Grid;
typedef double LSMLIB_REAL;
#define VERY_HIGH 3
#define LSM3D_HJ_WENO5 lsm3dhjweno5_
#define LSM3D_COMPUTE_REINITIALIZATION_EQN_RHS lsm3dcomputereinitializationeqnrhs_
#define LSM3D_TVD_RK2_STAGE1 lsm3dtvdrk2stage1_
#define LSM3D_TVD_RK2_STAGE2 lsm3dtvdrk2stage2_
#define LSM3D_SIGNED_LINEAR_EXTRAPOLATION lsm3dsignedlinearextrapolation_
#else
#include "lsm_boundary_conditions3d.h"
#include "lsm_grid.h"
#include "lsm_reinitialization3d.h"
#include "lsm_spatial_derivatives3d.h"
#include "lsm_tvd_runge_kutta3d.h"
#endif

#define GB(g) &(g)->ilo_gb, &(g)->ihi_gb, &(g)->jlo_gb, &(g)->jhi_gb, &(g)->klo_gb, &(g)->khi_gb
#define FB(g) &(g)->ilo_fb, &(g)->ihi_fb, &(g)->jlo_fb, &(g)->jhi_fb, &(g)->klo_fb, &(g)->khi_fb

static LSMLIB_REAL *field(const Grid *g) { return (LSMLIB_REAL *)calloc((size_t)g->num_gridpts, sizeof(LSMLIB_REAL)); }

static void boundary(LSMLIB_REAL *a, Grid *g) {
  for (int face = 0; face < 6; face++) LSM3D_SIGNED_LINEAR_EXTRAPOLATION(a, GB(g), FB(g), &face);
}

/* HJ WENO5 plus/minus of `phi`, then the reinitialization right-hand side */
static void rhs(LSMLIB_REAL *out, LSMLIB_REAL *phi, LSMLIB_REAL *phi0, LSMLIB_REAL *gp[3], LSMLIB_REAL *gm[3],
                LSMLIB_REAL *d1, Grid *g) {
  int use_phi0_for_sign = 0;
  LSM3D_HJ_WENO5(gp[0], gp[1], gp[2], GB(g), gm[0], gm[1], gm[2], GB(g), phi, GB(g), d1, GB(g), FB(g), &g->dx[0],
                 &g->dx[1], &g->dx[2]);
  LSM3D_COMPUTE_REINITIALIZATION_EQN_RHS(out, GB(g), phi, GB(g), phi0, GB(g), gp[0], gp[1], gp[2], GB(g), gm[0],
                                         gm[1], gm[2], GB(g), FB(g), &g->dx[0], &g->dx[1], &g->dx[2],
                                         &use_phi0_for_sign);
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s <cells per side> <iterations> <output file>\n", argv[0]);
    return 2;
  }
  const int n = atoi(argv[1]), iters = atoi(argv[2]);
  LSMLIB_REAL x_lo[3] = {-1.0, -1.0, -1.0}, x_hi[3] = {1.0, 1.0, 1.0};
  Grid *g = createGridSetDx(3, 2.0 / n, x_lo, x_hi, VERY_HIGH);
  LSMLIB_REAL *phi = field(g), *phi0 = field(g), *stage1 = field(g), *lse_rhs = field(g), *d1 = field(g);
  LSMLIB_REAL *gp[3] = {field(g), field(g), field(g)}, *gm[3] = {field(g), field(g), field(g)};
  const int nx = g->grid_dims_ghostbox[0], ny = g->grid_dims_ghostbox[1], nz = g->grid_dims_ghostbox[2];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const LSMLIB_REAL x = g->x_lo_ghostbox[0] + (i + 0.5) * g->dx[0];
        const LSMLIB_REAL y = g->x_lo_ghostbox[1] + (j + 0.5) * g->dx[1];
        const LSMLIB_REAL z = g->x_lo_ghostbox[2] + (k + 0.5) * g->dx[2];
        const LSMLIB_REAL r = sqrt(x * x + y * y + z * z);
        phi[i + nx * (j + ny * k)] = (r - 0.5) * (0.1 + (x - 0.3) * (x - 0.3) + (y - 0.3) * (y - 0.3) +
                                                  (z + 0.2) * (z + 0.2));
      }
  for (int q = 0; q < g->num_gridpts; q++) phi0[q] = phi[q];
  LSMLIB_REAL dt = 0.5 * g->dx[0];
  for (int it = 0; it < iters; it++) {
    rhs(lse_rhs, phi, phi0, gp, gm, d1, g);
    LSM3D_TVD_RK2_STAGE1(stage1, GB(g), phi, GB(g), lse_rhs, GB(g), FB(g), &dt);
    boundary(stage1, g);
    rhs(lse_rhs, stage1, phi0, gp, gm, d1, g);
    LSM3D_TVD_RK2_STAGE2(phi, GB(g), stage1, GB(g), phi, GB(g), lse_rhs, GB(g), FB(g), &dt);
    boundary(phi, g);
  }
  FILE *f = fopen(argv[3], "wb");
  if (!f || fwrite(phi, sizeof(LSMLIB_REAL), (size_t)g->num_gridpts, f) != (size_t)g->num_gridpts) {
    fprintf(stderr, "cannot write %s\n", argv[3]);
    return 1;
  }
  fclose(f);
  printf("%d cells, %d iterations: ok\n", g->num_gridpts, iters);
  return 0;
}
