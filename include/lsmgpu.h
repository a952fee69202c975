/*
 * lsmgpu — GB300-native implementation of LSMLIB's data-parallel level-set
 * kernels.
 *
 * This header holds the library's own entry points (runtime control, status,
 * and the fused time-stepping calls).  The drop-in entry points that replace
 * LSMLIB's Fortran toolbox routines, with LSMLIB's symbol names and argument
 * lists, are declared in lsmgpu_toolbox3d.h.
 *
 * Pointer rules for every entry point
 *  - A pointer to device or managed memory is used in place; the call is
 *    asynchronous on the library stream (lsmgpu_set_stream), except that a
 *    scalar result written to host memory (a dt, a norm) waits for the stream.
 *  - A pointer to host memory (pageable or pinned) is staged: copied to the
 *    device, computed, and copied back before the call returns, which is the
 *    synchronous behaviour LSMLIB's serial routines have.
 *  - Scratch arrays of the LSMLIB interface (D1, D2, D3 of the dense
 *    derivative routines) are accepted and not written, unless the exact
 *    side-effect mode is on (lsmgpu_set_exact_side_effects below).
 *
 * Errors: LSMLIB's routines return nothing and do not check their input.  Here
 * each call validates its index boxes (the fill box plus the stencil's reach
 * must lie inside every ghost box it reads) and records a status that
 * lsmgpu_get_last_error() returns; an invalid call computes nothing.
 */
#ifndef LSMGPU_H
#define LSMGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LSMGPU_OK 0
#define LSMGPU_ERR_BOUNDS 1      /* an index box does not cover a stencil  */
#define LSMGPU_ERR_CUDA 2        /* a CUDA runtime call failed             */
#define LSMGPU_ERR_ARGUMENT 3    /* null pointer or unsupported option     */
#define LSMGPU_ERR_CAPACITY 4    /* a size exceeds a documented maximum    */
#define LSMGPU_ERR_TIMEOUT 5     /* a bounded device wait gave up          */

/* Returns the status of the last lsmgpu call made on this host thread and,
 * when msg is not NULL, copies a description into msg (at most len bytes,
 * NUL-terminated). */
int lsmgpu_get_last_error(char *msg, int len);

/* Sets the CUDA stream (a cudaStream_t passed as void*) the library launches
 * on; NULL selects the legacy default stream. */
void lsmgpu_set_stream(void *stream);
void *lsmgpu_get_stream(void);

/* Waits for all work the library queued on its stream. */
int lsmgpu_synchronize(void);

/* Number of kernels the library has launched since the process started (or
 * since lsmgpu_reset_launch_count). */
long long lsmgpu_launch_count(void);
void lsmgpu_reset_launch_count(void);

/* Exact side-effect mode.  LSMLIB's dense HJ ENO1/2/3 and WENO5 routines
 * (plus/minus and upwind) leave their scratch arrays D1, D2, D3 holding the
 * last undivided differences they formed (the z direction's, 1e10 outside
 * their fill range; src/toolbox/lsm_spatial_derivatives3d.f.in:49-176 and
 * the lsm3dComputeDn calls of each routine).  By default these routines do
 * not write the scratch arrays (nothing of LSMLIB reads them back); with the
 * mode on they replay LSMLIB's lsm3dComputeDn calls after the derivative, so
 * a driver that reads D1 / D2 / D3 sees LSMLIB's values.  The mode starts as
 * the environment variable LSMGPU_EXACT_SIDE_EFFECTS says (unset or 0: off).
 * Process-wide. */
void lsmgpu_set_exact_side_effects(int on);
int lsmgpu_get_exact_side_effects(void);

/* Bounds-check build (python -m lsmlib_gb300.build --bounds-check, which
 * writes lsmlib_gb300/liblsmgpu_bc.so): every array access of the drop-in
 * kernels is checked against the array's box; an out-of-range one is
 * counted, the first one's (i, j, k) kept, and the array's first element used
 * instead of memory outside it.  lsmgpu_bounds_check_read waits for the
 * library stream, returns the count and first index of the current device
 * and clears them.  In the regular library it returns LSMGPU_ERR_ARGUMENT. */
int lsmgpu_bounds_check_read(long long *count, int *first);

/* Number of CUDA graphs the fused steppers have captured since the process
 * started.  A stepper call replays a cached graph when its buffers, sizes and
 * parameters were seen before, and captures a new one otherwise. */
long long lsmgpu_graph_capture_count(void);

/* Device memory (bytes, all devices) the library's grow-only staging and
 * temporary arena holds.  It grows with cudaMalloc and is never freed. */
long long lsmgpu_arena_bytes(void);

/* ---------------------------------------------------------------------------
 * Fused WENO5 / TVD-RK3 time steppers.
 *
 * Each call advances phi (column-major over the ghost box gb[6] = {ilo, ihi,
 * jlo, jhi, klo, khi}) by whole TVD-RK3 steps over the fill box fb[6].  Every
 * stage is one kernel that computes the HJ WENO5 derivatives, the right-hand
 * side and the stage update in one pass; after each stage the 3 ghost layers
 * are refreshed with the boundary condition `bc`.  The result equals the
 * LSMLIB call sequence per stage
 *   HJ derivatives -> RHS -> TVDRK3StageN -> ghost fill
 * and, for the _f64 forms, matches it bit for bit.  The fill box needs at
 * least 6 cells per axis and 3 ghost cells on every side; ghost cells beyond
 * the third layer are left untouched.  The _f32 forms store and compute in
 * single precision.  Returns an LSMGPU_* status.
 * ------------------------------------------------------------------------- */
#define LSMGPU_BC_PERIODIC 0      /* periodic wrap of the fill box           */
#define LSMGPU_BC_LINEAR 1        /* lsm3dLinearExtrapolation on the six faces,
                                     x then y then z                         */
#define LSMGPU_BC_SIGNED_LINEAR 2 /* lsm3dSignedLinearExtrapolation, same order */
#define LSMGPU_BC_COPY 3          /* lsm3dCopyExtrapolation (homogeneous
                                     Neumann), same order                    */

/* Reinitialization: n_iter pseudo-time steps of d(phi)/dt = sgn(1 - |grad phi|)
 * (lsm3dComputeReinitializationEqnRHS with HJ WENO5 plus/minus derivatives),
 * step dtau.  use_phi0_for_sgn = 1 takes the smoothed sign from the initial
 * phi, 0 from the current stage's phi. */
int lsmgpu_reinit_weno5_tvdrk3_f64(double *phi, const int *gb, const int *fb, double dx, double dy,
                                   double dz, double dtau, int n_iter, int use_phi0_for_sgn, int bc);
int lsmgpu_reinit_weno5_tvdrk3_f32(float *phi, const int *gb, const int *fb, float dx, float dy,
                                   float dz, float dtau, int n_iter, int use_phi0_for_sgn, int bc);

/* Advection: n_steps steps of d(phi)/dt = -u . grad(phi) with upwind HJ WENO5
 * (lsm3dUpwindHJWENO5 + lsm3dAddAdvectionTermToLSERHS), step dt.  The velocity
 * is either three fields over the ghost box vel_gb (vel_x/y/z non-NULL) or,
 * when vel_x is NULL, the constant vel_const[3]. */
int lsmgpu_advect_weno5_tvdrk3_f64(double *phi, const int *gb, const int *fb, const double *vel_x,
                                   const double *vel_y, const double *vel_z, const int *vel_gb,
                                   const double *vel_const, double dx, double dy, double dz,
                                   double dt, int n_steps, int bc);
int lsmgpu_advect_weno5_tvdrk3_f32(float *phi, const int *gb, const int *fb, const float *vel_x,
                                   const float *vel_y, const float *vel_z, const int *vel_gb,
                                   const float *vel_const, float dx, float dy, float dz, float dt,
                                   int n_steps, int bc);

/* Second-order mean curvature of phi over the fill box fb in one pass: the
 * sequence lsm3dCentralGradOrder2 -> lsm3dGradientMagnitude ->
 * lsm3dComputeMeanCurvatureOrder2.  kappa (and grad_phi_mag when not NULL)
 * are column-major over kappa_gb; phi over phi_gb, which must hold one ghost
 * cell around fb. */
int lsmgpu_mean_curvature_o2_f64(double *kappa, const int *kappa_gb, const double *phi,
                                 const int *phi_gb, double *grad_phi_mag, const int *fb, double dx,
                                 double dy, double dz);
int lsmgpu_mean_curvature_o2_f32(float *kappa, const int *kappa_gb, const float *phi,
                                 const int *phi_gb, float *grad_phi_mag, const int *fb, float dx,
                                 float dy, float dz);

/* Narrow-band curvature flow: n_steps TVD-RK3 steps of
 * phi_t + Vn |grad phi| = 0, Vn = a_n - b_n * kappa, on a narrow band of
 * half-width gamma (inner width beta, 3 neighbour levels) rebuilt from phi
 * every rebuild_every steps (lsm3dDetermineNarrowBand).  Per stage, on
 * level-0 cells: mean curvature (central differences), HJ WENO5 plus/minus on
 * the band, the Godunov normal-velocity RHS, the cubic cut-off between beta
 * and gamma, the TVD-RK3 stage update — the LSMLIB *_LOCAL sequence, one
 * gather kernel per stage.  dt is the CFL-stable normal-velocity dt of stage 1
 * of each step (lsm3dComputeStableNormalVelDtLOCAL, CFL number cfl).  phi is
 * column-major over gb (every band cell must lie 3 cells inside gb); dx is
 * the spacing of all three axes.  dt_log (n_steps doubles) and band_log (one
 * level-0 cell count per rebuild) are optional host outputs.  The _f64 form
 * matches the LSMLIB sequence bit for bit; the _f32 form stores phi in single
 * precision and keeps the band's distance test in double. */
int lsmgpu_band_flow_weno5_tvdrk3_f64(double *phi, const int *gb, const int *fb, double dx, double a_n,
                                      double b_n, double cfl, double gamma, double beta, int n_steps,
                                      int rebuild_every, double *dt_log, long long *band_log);
int lsmgpu_band_flow_weno5_tvdrk3_f32(float *phi, const int *gb, const int *fb, float dx, float a_n,
                                      float b_n, float cfl, float gamma, float beta, int n_steps,
                                      int rebuild_every, double *dt_log, long long *band_log);

/* Batched advection of many independent grids (FP32): n_grids grids packed in
 * one array, grid g occupying (nx+6)(ny+6)(nz+6) values (3 ghost cells per
 * side, column-major) from phi + offsets[g]; dims holds (nx, ny, nz) per grid,
 * vel the constant velocity (u, v, w) per grid, spacing (dx, dy, dz) per grid
 * and dt one step per grid.  Each TVD-RK3 stage of all grids is one
 * persistent kernel launch pulling 32 x 8 x TZ tiles from a work counter; the
 * n_steps x 3 launches are captured in a CUDA graph.  TZ and the CTAs per SM
 * are picked by an autotuner on the first call for a batch shape.  Periodic
 * boundaries only (bc = LSMGPU_BC_PERIODIC).  flags: LSMGPU_BATCH_LOOP runs
 * one single-grid launch per grid per stage instead (for comparison),
 * LSMGPU_BATCH_NO_GRAPH launches without a graph, LSMGPU_BATCH_TZ(n) forces
 * tile depth n (4, 8 or 16) and skips the autotuner.  The result is the same
 * in every mode. */
#define LSMGPU_BATCH_LOOP 1
#define LSMGPU_BATCH_NO_GRAPH 2
#define LSMGPU_BATCH_TZ(n) ((n) << 8)
int lsmgpu_advect_batch_weno5_tvdrk3_f32(float *phi, const long long *offsets, const int *dims,
                                         int n_grids, const float *vel, const float *spacing,
                                         const float *dt, int n_steps, int bc, int flags);

/* Reverse-mode gradient of a periodic advection objective.  No counterpart in
 * LSMLIB (LSMLIB has no adjoint); the forward map is LSMLIB's advection step
 * on a periodic grid (lsm3dUpwindHJWENO5, spatial_derivatives3d.f.in:2628;
 * lsm3dAddAdvectionTermToLSERHS, level_set_evolution3d.f.in:113; TVD RK3,
 * tvd_runge_kutta3d.f:78/403/490), the same arithmetic as
 * lsmgpu_advect_weno5_tvdrk3_* with LSMGPU_BC_PERIODIC:
 *   phi_T = n_steps steps of phi_t + vel . grad phi = 0 from phi (the
 *           periodic extension of its fill-box values; its ghost entries are
 *           ignored), time step dt (held fixed, not differentiated);
 *   J     = sum over fill-box cells of (H(phi_T) - H(phi_target))^2 dx dy dz,
 *           H = LSMLIB's smoothed Heaviside (lsm_calculus_toolbox.h:41) of
 *           width heaviside_eps, accumulated in FP64.
 * Outputs (any may be NULL; velocity gradients all three or none, and only
 * with grad_phi): *J; grad_phi = dJ/dphi over gb; grad_vel_* = dJ/dvel_*
 * over vel_gb.  Ghost entries of the gradients are set to zero.  Forward
 * states are kept every checkpoint_every steps and the steps between are
 * recomputed in the reverse sweep, except the last checkpoint_every steps,
 * whose stage states the forward sweep keeps (device memory: about
 * 3 * checkpoint_every + n_steps / checkpoint_every + 16 padded fields).
 * checkpoint_every >= n_steps keeps the whole trajectory and recomputes
 * nothing; checkpoint_every = 0 picks the largest spacing whose fields fit in
 * half of the free device memory.
 * Arrays may be host or device memory (host arrays are staged).
 * Returns an LSMGPU_* status. */
int lsmgpu_advect_adjoint_weno5_tvdrk3_f64(const double *phi, const int *gb, const int *fb,
                                           const double *vel_x, const double *vel_y, const double *vel_z,
                                           const int *vel_gb, const double *phi_target, double dx, double dy,
                                           double dz, double dt, int n_steps, int checkpoint_every,
                                           double heaviside_eps, double *J, double *grad_phi,
                                           double *grad_vel_x, double *grad_vel_y, double *grad_vel_z);
/* FP32 state and adjoint fields; H and delta of the objective evaluated in FP32, its sum in FP64. */
int lsmgpu_advect_adjoint_weno5_tvdrk3_f32(const float *phi, const int *gb, const int *fb,
                                           const float *vel_x, const float *vel_y, const float *vel_z,
                                           const int *vel_gb, const float *phi_target, float dx, float dy,
                                           float dz, float dt, int n_steps, int checkpoint_every,
                                           double heaviside_eps, double *J, float *grad_phi,
                                           float *grad_vel_x, float *grad_vel_y, float *grad_vel_z);

/* Vector-Jacobian products (reverse mode) of the periodic steppers, for any
 * objective: given grad_out = dJ/dphi_T over gb, return grad_phi =
 * dJ/dphi (and, for advection, grad_vel_* = dJ/dvel_*), with phi_T the
 * state after n_steps steps of lsmgpu_advect_weno5_tvdrk3_* /
 * n_iter iterations of lsmgpu_reinit_weno5_tvdrk3_* (LSMGPU_BC_PERIODIC;
 * reinitialization in the phi0 sign form, use_phi0_for_sgn = 1, whose sign
 * source is phi itself, so its sensitivity is part of grad_phi).  phi_out
 * (optional) receives phi_T over gb.  Checkpointing, derivative conventions
 * (branch taken at the upwind / Godunov maxima, dt fixed) and memory as for
 * lsmgpu_advect_adjoint_weno5_tvdrk3_*.  No counterpart in LSMLIB.  Returns
 * an LSMGPU_* status. */
int lsmgpu_advect_vjp_weno5_tvdrk3_f64(const double *phi, const int *gb, const int *fb, const double *vel_x,
                                       const double *vel_y, const double *vel_z, const int *vel_gb, double dx,
                                       double dy, double dz, double dt, int n_steps, int checkpoint_every,
                                       const double *grad_out, double *phi_out, double *grad_phi,
                                       double *grad_vel_x, double *grad_vel_y, double *grad_vel_z);
int lsmgpu_advect_vjp_weno5_tvdrk3_f32(const float *phi, const int *gb, const int *fb, const float *vel_x,
                                       const float *vel_y, const float *vel_z, const int *vel_gb, float dx,
                                       float dy, float dz, float dt, int n_steps, int checkpoint_every,
                                       const float *grad_out, float *phi_out, float *grad_phi, float *grad_vel_x,
                                       float *grad_vel_y, float *grad_vel_z);
int lsmgpu_reinit_vjp_weno5_tvdrk3_f64(const double *phi, const int *gb, const int *fb, double dx, double dy,
                                       double dz, double dtau, int n_iter, int checkpoint_every,
                                       const double *grad_out, double *phi_out, double *grad_phi);
int lsmgpu_reinit_vjp_weno5_tvdrk3_f32(const float *phi, const int *gb, const int *fb, float dx, float dy,
                                       float dz, float dtau, int n_iter, int checkpoint_every,
                                       const float *grad_out, float *phi_out, float *grad_phi);

/* Allocation-free CFL-stable advection dt.  No counterpart in LSMLIB: it is
 * lsm3dcomputestableadvectiondt_ (same arguments, same result) for callers
 * that cannot let a library allocate device memory — a solver running inside
 * another framework's memory pool that owns all device memory, or a
 * time-step loop that must not stall on the device synchronisation cudaMalloc
 * and cudaFree can cause.  It calls no allocator: its reduction scratch is a
 * fixed 512 KiB __device__ array in the library, so
 *  - the velocity arrays must already be in device (or managed) memory;
 *  - the index box may hold at most 536,870,912 cells (65536 blocks of 8192
 *    cells); larger boxes return LSMGPU_ERR_CAPACITY and compute nothing;
 *  - dt may point to host, managed or device memory (a host or managed dt
 *    waits for the stream; a device dt is written in stream order);
 *  - the first call on each device looks up the scratch address
 *    (cudaGetSymbolAddress); make that first call before any stream capture;
 *  - every call on a device shares the scratch and overwrites it, so calls
 *    that may overlap on the GPU (other streams or host threads) race and
 *    must be serialised by the caller.
 * Returns an LSMGPU_* status. */
int lsmgpu_compute_stable_advection_dt_noalloc(
    double *dt, const double *vel_x, const double *vel_y, const double *vel_z, const int *ilo_vel_gb,
    const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *klo_vel_gb,
    const int *khi_vel_gb, const int *ilo_ib, const int *ihi_ib, const int *jlo_ib, const int *jhi_ib,
    const int *klo_ib, const int *khi_ib, const double *dx, const double *dy, const double *dz,
    const double *cfl_number);

/* Fourth-order mean curvature over an index list, with the argument list of
 * lsm3dComputeMeanCurvatureOrder4Local (src/geometry/lsm_curvature3d_local.f.in:285).
 * That reference routine evaluates the Gaussian-curvature formula (numerator
 * and |grad phi|^4 denominator, lsm_curvature3d_local.f.in:385-410), and its
 * drop-in entry point lsm3dcomputemeancurvatureorder4local_ keeps that; this
 * one evaluates the mean curvature of lsm3dComputeMeanCurvatureOrder4
 * (lsm_curvature3d.f.in:253) on the listed cells.  The 2D drop-in
 * lsm2dcomputemeancurvatureorder4local_ runs on it. */
void lsmgpu_mean_curvature_order4_local(
    double *kappa, const int *ilo_kappa_gb, const int *ihi_kappa_gb, const int *jlo_kappa_gb,
    const int *jhi_kappa_gb, const int *klo_kappa_gb, const int *khi_kappa_gb, const double *phi,
    const int *ilo_phi_gb, const int *ihi_phi_gb, const int *jlo_phi_gb, const int *jhi_phi_gb,
    const int *klo_phi_gb, const int *khi_phi_gb, const double *phi_x, const double *phi_y,
    const double *phi_z, const double *grad_phi_mag, const int *ilo_grad_phi_gb,
    const int *ihi_grad_phi_gb, const int *jlo_grad_phi_gb, const int *jhi_grad_phi_gb,
    const int *klo_grad_phi_gb, const int *khi_grad_phi_gb, const double *dx, const double *dy,
    const double *dz, const int *index_x, const int *index_y, const int *index_z, const int *nlo_index,
    const int *nhi_index, const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb,
    const int *jlo_nb_gb, const int *jhi_nb_gb, const int *klo_nb_gb, const int *khi_nb_gb,
    const unsigned char *mark_fb);

/* The 2D reference routines' formulas on 3D arrays, with the argument lists
 * of the 3D routines named; the 2D drop-in entry points run on them.
 *
 * lsmgpu_orthogonalization_rhs_unit_sgn_smoothing(_local): the
 * orthogonalization RHS of lsm3dComputeOrthogonalizationEqnRHS(LOCAL)
 * (src/reinitialization/lsm_reinitialization3d.f.in:296,
 * lsm_reinitialization3d_local.f.in:326) with sgn(psi) = psi /
 * sqrt(psi^2 + max(dx)^2), as lsm2dComputeOrthogonalizationEqnRHS smooths it
 * (lsm_reinitialization2d.f.in:360); the 3D routines use
 * max(dx)^2 |grad psi|^2.
 *
 * lsmgpu_distance_for_subcell_fix_full_central: the subcell-fix distance of
 * lsm3dComputeDistanceForSubcellFix (lsm_reinitialization3d.f.in:477) in
 * the form of lsm2dComputeDistanceForSubcellFix (lsm_reinitialization2d.f.in:392):
 * sign changes by negative products phi0(neighbour) phi0(cell), the full
 * central difference in delta, and 2 phi0 / delta. */
void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing(
    double *ortho_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb,
    const int *jhi_rhs_gb, const int *klo_rhs_gb, const int *khi_rhs_gb, const double *phi_x_plus,
    const double *phi_y_plus, const double *phi_z_plus, const int *ilo_grad_phi_plus_gb,
    const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb,
    const int *klo_grad_phi_plus_gb, const int *khi_grad_phi_plus_gb, const double *phi_x_minus,
    const double *phi_y_minus, const double *phi_z_minus, const int *ilo_grad_phi_minus_gb,
    const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb,
    const int *klo_grad_phi_minus_gb, const int *khi_grad_phi_minus_gb, const double *psi,
    const int *ilo_psi_gb, const int *ihi_psi_gb, const int *jlo_psi_gb, const int *jhi_psi_gb,
    const int *klo_psi_gb, const int *khi_psi_gb, const double *psi_x_plus, const double *psi_y_plus,
    const double *psi_z_plus, const int *ilo_grad_psi_plus_gb, const int *ihi_grad_psi_plus_gb,
    const int *jlo_grad_psi_plus_gb, const int *jhi_grad_psi_plus_gb, const int *klo_grad_psi_plus_gb,
    const int *khi_grad_psi_plus_gb, const double *psi_x_minus, const double *psi_y_minus,
    const double *psi_z_minus, const int *ilo_grad_psi_minus_gb, const int *ihi_grad_psi_minus_gb,
    const int *jlo_grad_psi_minus_gb, const int *jhi_grad_psi_minus_gb, const int *klo_grad_psi_minus_gb,
    const int *khi_grad_psi_minus_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb,
    const int *jhi_fb, const int *klo_fb, const int *khi_fb, const double *dx, const double *dy,
    const double *dz);
void lsmgpu_orthogonalization_rhs_unit_sgn_smoothing_local(
    double *ortho_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb,
    const int *jhi_rhs_gb, const int *klo_rhs_gb, const int *khi_rhs_gb, const double *phi_x_plus,
    const double *phi_y_plus, const double *phi_z_plus, const int *ilo_grad_phi_plus_gb,
    const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb,
    const int *klo_grad_phi_plus_gb, const int *khi_grad_phi_plus_gb, const double *phi_x_minus,
    const double *phi_y_minus, const double *phi_z_minus, const int *ilo_grad_phi_minus_gb,
    const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb,
    const int *klo_grad_phi_minus_gb, const int *khi_grad_phi_minus_gb, const double *psi,
    const int *ilo_psi_gb, const int *ihi_psi_gb, const int *jlo_psi_gb, const int *jhi_psi_gb,
    const int *klo_psi_gb, const int *khi_psi_gb, const double *psi_x_plus, const double *psi_y_plus,
    const double *psi_z_plus, const int *ilo_grad_psi_plus_gb, const int *ihi_grad_psi_plus_gb,
    const int *jlo_grad_psi_plus_gb, const int *jhi_grad_psi_plus_gb, const int *klo_grad_psi_plus_gb,
    const int *khi_grad_psi_plus_gb, const double *psi_x_minus, const double *psi_y_minus,
    const double *psi_z_minus, const int *ilo_grad_psi_minus_gb, const int *ihi_grad_psi_minus_gb,
    const int *jlo_grad_psi_minus_gb, const int *jhi_grad_psi_minus_gb, const int *klo_grad_psi_minus_gb,
    const int *khi_grad_psi_minus_gb, const double *dx, const double *dy, const double *dz,
    const int *index_x, const int *index_y, const int *index_z, const int *nlo_index, const int *nhi_index,
    const unsigned char *narrow_band, const int *ilo_nb_gb, const int *ihi_nb_gb, const int *jlo_nb_gb,
    const int *jhi_nb_gb, const int *klo_nb_gb, const int *khi_nb_gb, const unsigned char *mark_fb);
void lsmgpu_distance_for_subcell_fix_full_central(
    double *distance0, const double *phi0, const int *ilo_phi0_gb, const int *ihi_phi0_gb,
    const int *jlo_phi0_gb, const int *jhi_phi0_gb, const int *klo_phi0_gb, const int *khi_phi0_gb,
    const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *klo_fb,
    const int *khi_fb, const double *dx, const double *dy, const double *dz);

/* lsmgpu_external_normal_vel_term_fill_box: the combined external and normal
 * velocity term of lsm3dAddExternalAndNormalVelTermToLSERHS
 * (src/toolbox/lsm_level_set_evolution3d.f.in:532), same arguments, in the
 * form of lsm2dAddExternalAndNormalVelTermToLSERHS
 * (lsm_level_set_evolution2d.f.in:399): over the fill box only, and nothing
 * added where |Vn| < zero_tol (the 3D routine loops from the fill box to the
 * ghost box end and adds the advection part there).
 *
 * lsmgpu_signed_linear_extrapolation_inner_sign: lsm3dSignedLinearExtrapolation
 * (src/boundary_conditions/lsm_boundary_conditions3d.f) with the slope's
 * sign taken from the cell next to the edge, as
 * lsm1dSignedLinearExtrapolation does (lsm_boundary_conditions1d.f:103). */
void lsmgpu_external_normal_vel_term_fill_box(
    double *lse_rhs, const int *ilo_rhs_gb, const int *ihi_rhs_gb, const int *jlo_rhs_gb,
    const int *jhi_rhs_gb, const int *klo_rhs_gb, const int *khi_rhs_gb, const double *phi_x_plus,
    const double *phi_y_plus, const double *phi_z_plus, const int *ilo_grad_phi_plus_gb,
    const int *ihi_grad_phi_plus_gb, const int *jlo_grad_phi_plus_gb, const int *jhi_grad_phi_plus_gb,
    const int *klo_grad_phi_plus_gb, const int *khi_grad_phi_plus_gb, const double *phi_x_minus,
    const double *phi_y_minus, const double *phi_z_minus, const int *ilo_grad_phi_minus_gb,
    const int *ihi_grad_phi_minus_gb, const int *jlo_grad_phi_minus_gb, const int *jhi_grad_phi_minus_gb,
    const int *klo_grad_phi_minus_gb, const int *khi_grad_phi_minus_gb, const double *vel_n,
    const double *vel_x, const double *vel_y, const double *vel_z, const int *ilo_vel_gb,
    const int *ihi_vel_gb, const int *jlo_vel_gb, const int *jhi_vel_gb, const int *klo_vel_gb,
    const int *khi_vel_gb, const int *ilo_rhs_fb, const int *ihi_rhs_fb, const int *jlo_rhs_fb,
    const int *jhi_rhs_fb, const int *klo_rhs_fb, const int *khi_rhs_fb);
void lsmgpu_signed_linear_extrapolation_inner_sign(
    double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb,
    const int *klo_gb, const int *khi_gb, const int *ilo_fb, const int *ihi_fb, const int *jlo_fb,
    const int *jhi_fb, const int *klo_fb, const int *khi_fb, const int *bdry_location_idx);

/* lsmgpu_determine_narrow_band_2d_bookkeeping: lsm3dDetermineNarrowBand
 * (src/toolbox/lsm_localization3d.f:174), same arguments, with the list
 * bookkeeping of lsm2dDetermineNarrowBand (lsm_localization2d.f:225-240):
 * n_hi(0) = nlo_index + (level-0 cells) - 1 and the outer-list bounds
 * likewise even for an empty band, neighbour levels only when level 0
 * holds two or more cells. */
void lsmgpu_determine_narrow_band_2d_bookkeeping(
    const double *phi, const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb,
    const int *klo_gb, const int *khi_gb, unsigned char *narrow_band, const int *ilo_nb_gb,
    const int *ihi_nb_gb, const int *jlo_nb_gb, const int *jhi_nb_gb, const int *klo_nb_gb,
    const int *khi_nb_gb, int *index_x, int *index_y, int *index_z, const int *nlo_index,
    const int *nhi_index, int *n_lo, int *n_hi, int *index_outer, const int *nlo_index_outer,
    const int *nhi_index_outer, int *nlo_outer_plus, int *nhi_outer_plus, int *nlo_outer_minus,
    int *nhi_outer_minus, const double *width, const double *width_inner, const int *level);

/* Library version string. */
const char *lsmgpu_version(void);

/* ---------------------------------------------------------------------------
 * Diagnostics.  No counterpart in LSMLIB's library; the first is the GPU
 * form of its EXAMINE_ARRAY macro (lsm_macros.h), which prints the
 * positions of NaN / inf values.
 * ------------------------------------------------------------------------- */

/* Counts the NaN and infinite values of `field` (column-major over gb[6])
 * inside box[6] and, when first is not NULL, stores the first one a serial
 * (k, j, i) sweep of the box meets (box.lo - 1 on each axis when there is
 * none).  Host or device arrays.  Returns an LSMGPU_* status. */
int lsmgpu_count_nonfinite_f64(const double *field, const int *gb, const int *box, long long *count, int *first);
int lsmgpu_count_nonfinite_f32(const float *field, const int *gb, const int *box, long long *count, int *first);

/* Exercises the bounded device wait of the TMA-staged kernels: one block
 * waits on a barrier that is never released, gives up after `polls` polls
 * (at most 1048576), records LSMGPU_ERR_TIMEOUT and returns; the context
 * stays usable.  Returns LSMGPU_ERR_TIMEOUT (the expected outcome). */
int lsmgpu_selftest_bounded_wait(unsigned int polls);

/* Measures the device's sustained arithmetic rates with two fixed-length
 * probe kernels: FP32 lane operations per second through packed FFMA2
 * instructions (one FFMA2 = two lane operations) and FP64 fused
 * multiply-adds per second.  These are the denominators of the FP32-pipe
 * and FP64 rooflines the benchmark reports.  Synchronous; returns an
 * LSMGPU_* status. */
int lsmgpu_measure_fma_rates(double *fp32_lane_ops_per_s, double *fp64_ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* LSMGPU_H */
