/*
 * gpr_gb300.h - C ABI of the GB300-native GPR (Godunov-Peshkov-Romenski)
 * ADER-WENO time step.
 *
 * Every entry point takes plain device pointers for grid data (float64 /
 * int32 / uint8 arrays in the reference's cell-major layouts), HOST pointers
 * for the small control arrays (nX, dX, bcs) and for `gpr_par`, and a CUDA
 * stream (`void*`, NULL = legacy default stream).  Work is enqueued on that stream; functions return 0 on success or
 * a negative GPR_E_* code.  No entry point allocates device memory unless its
 * comment says so; scratch buffers are passed in by the caller.
 *
 * Layouts (identical to the reference, code/cpp/src/etc/grid.cpp:129-130,
 * solvers/weno/weno.cpp:83-124, solvers/fv/fv.cpp:7-9):
 *   u   : [nx][ny][V]                 conserved state, V doubles per cell
 *   ub  : [nx+2N][ny+2N][V]           state with N ghost cells per side
 *   wh  : [nx+2][ny+2][N^d][V]        WENO reconstruction (x-node major)
 *   qh  : [nx+2][ny+2][N][N^d][V]     space-time predictor (time-node major)
 *   mask: [nx+2][ny+2] uint8          predictor/update mask
 * with V = 14 + 3*THERMAL + LSET, N = 2 Gauss-Legendre nodes, d = 1 or 2
 * (ny absent in 1D).  The variable order is
 *   [rho, rho E, rho v(3), A (3x3 row-major), rho J (3, if THERMAL), phi (LSET)].
 */
#ifndef GPR_GB300_H
#define GPR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
#define GPR_OK 0
#define GPR_E_ARG (-1)        /* bad size, dimension, flag or pointer        */
#define GPR_E_CUDA (-2)       /* a CUDA runtime call failed                  */
#define GPR_E_UNSUPPORTED (-3) /* variant (N, V, flux) not compiled in       */
#define GPR_E_TOO_LARGE (-4)  /* size beyond a stated fixed maximum          */

/* Flux codes (code/cpp/src/solvers/fv/fluxes.h:7-9).  Rusanov, Roe and
 * Osher (a V x V eigen-decomposition of the system matrix per face point and
 * path node) in 1D and 2D. */
#define GPR_FLUX_RUSANOV 0
#define GPR_FLUX_ROE 1
#define GPR_FLUX_OSHER 2

/* Boundary codes (code/cpp/src/etc/grid.cpp:5-10). */
#define GPR_BC_TRANSMISSIVE 0
#define GPR_BC_PERIODIC 1
#define GPR_BC_SLIP 2
#define GPR_BC_STICK 3
#define GPR_BC_MOVING 4
#define GPR_BC_SYMMETRIC 5

/* Material flags. */
#define GPR_SOLID 1
#define GPR_POWER_LAW 2
#define GPR_BINGHAM 4

/* Predictor status codes written per cell (see gpr_predictor). */
#define GPR_PRED_PICARD 0   /* Picard fixed point met the reference stopping rule */
#define GPR_PRED_NEWTON 1   /* Picard failed; Newton met the tolerance            */
#define GPR_PRED_FAILED 2   /* neither converged; best iterate written            */

/* Material parameters: the fields of the reference's Par
 * (code/cpp/src/system/objects.h:22-98) that the GPR step reads. */
typedef struct gpr_par {
  int32_t EOS;   /* 0 stiffened gas, 1 shock MG, 2 JWL, 3 Cochran-Chan, 4 GR */
  int32_t flags; /* GPR_SOLID | GPR_POWER_LAW | GPR_BINGHAM                  */
  double rho0, Tref, cv, pINF, Gamma0, c02, s, alpha, beta, gamma;
  double A, B, R1, R2;
  double b02, mu, tau0, sigmaY, n;
  double calpha2, kappa;
  double dp[3]; /* body force */
} gpr_par;

/* ------------------------------------------------------------------------ */
/* Library information.                                                     */

/* Returns the library version as an integer (major*10000+minor*100+patch). */
int gpr_version(void);
/* The scheme's constants on the host (no GPU needed), N = 2 Gauss nodes:
 * out[] = nodes[N], weights[N] (solvers.common.scaled_nodes /
 * scaled_weights, poly/basis.cpp), end values [2][N] (end_values: psi_j(0),
 * psi_j(1)), derivative values [N][N] (derivative_values: psi_j'(x_i)),
 * WENO oscillation indicator [N][N] (solvers.weno.oscillation_indicator,
 * weno_matrices.cpp:31-42).  Returns the count written (16), or GPR_E_ARG
 * when n is smaller. */
int gpr_scheme_constants(double *out, int n);
/* Writes the V values compiled in (up to `cap`) and returns how many. */
int gpr_supported_nvars(int32_t *out, int cap);

/* ------------------------------------------------------------------------ */
/* Grid helpers.                                                            */

/* Replaces GPRpy.boundaries (code/cpp/src/etc/grid.h:6, grid.cpp:147-170):
 * fills ub (with N ghost cells per side) from u under the boundary codes
 * bcs[2*ndim] (left, right per axis). */
int gpr_boundaries(const double *u, double *ub, const int32_t *nX, int ndim,
                   const int32_t *bcs, int nvar, void *stream);

/* Replaces GPRpy.extend_mask (grid.h:10, grid.cpp:176-230). */
int gpr_extend_mask(const uint8_t *mask, uint8_t *maskb, const int32_t *nX,
                    int ndim, void *stream);

/* ------------------------------------------------------------------------ */
/* Stages of the ADER-WENO step.                                            */

/* Replaces GPRpy.solvers.weno.weno_launcher (solvers/weno/weno.h:6,
 * weno.cpp:126-157): WENO reconstruction of ub into wh over the nx+2 (x ny+2)
 * predictor cells.  In 2D both sweeps run in one launch, the x sweep's
 * result kept in shared memory; the scratch argument and its size query
 * gpr_weno_scratch_doubles(nX, 2, nvar) (the x-sweep result of a two-pass
 * form) are kept for callers that pass them, and scratch may be NULL. */
long gpr_weno_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_weno_launcher(double *wh, const double *ub, const int32_t *nX,
                      int ndim, double *scratch, int nvar, void *stream);

/* Replaces solvers.dg.predictor (solvers/dg/dg.h:7, dg1.cpp:58-114,
 * dg2.cpp:102-171): local space-time Galerkin predictor of every masked cell.
 * Picard iteration with the reference's initial guess, update and per-cell
 * stopping rule (|dq| <= 6e-6 (1 + |q|), at most 50 iterations).  Cells where
 * Picard does not converge (the reference leaves their rows unwritten) or
 * produces NaN (the reference switches to Newton-Krylov) are finished by a
 * stiff-source Newton iteration on the same fixed point, implicit in the
 * relaxation sources, to |dq| <= 1e-11 (1 + |q|).  `status` (optional, one
 * int32 per predictor cell) receives GPR_PRED_* in the low byte and the
 * iteration count of the pass that finished the cell << 8.  stiff=1 skips
 * Picard and goes straight to the Newton iteration (the reference's STIFF).
 * The output rows of every masked cell are always written. */
int gpr_predictor(double *qh, const double *wh, double dt, const double *dX,
                  int ndim, const int32_t *nX, int stiff, const gpr_par *par,
                  const uint8_t *mask, int32_t *status, int nvar,
                  void *stream);

/* Replaces solvers.fv.fv_launcher (solvers/fv/fv.h:17, fv.cpp:281-297):
 * u += space-time quadrature of the non-conservative/source terms
 * (SOURCES, TIME) and the path-conservative interface fluxes.  With the
 * Rusanov flux the face terms are applied to u inside the face kernels, as
 * the reference's interfs1/2 update u inside their face loops: in 2D by
 * four passes (x / y faces of even / odd index, which never share a cell),
 * in 1D in one launch with the volume term.  With the Osher and Roe fluxes
 * the face sums go through caller scratch of
 * gpr_fv_scratch_doubles(nX, ndim, nvar) doubles, which a Rusanov call
 * does not touch (it may be NULL there). */
long gpr_fv_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_fv_launcher(double *u, const double *qh, const int32_t *nX, double dt,
                    const double *dX, int ndim, int sources, int time_dg,
                    int flux, const gpr_par *par, const uint8_t *mask,
                    double *scratch, int nvar, void *stream);

/* The two passes of gpr_fv_launcher as separate calls, in place on u:
 * gpr_fv_centers replaces solvers.fv.centers1 / centers2 (fv.h:7-10,
 * fv.cpp:11-109: the space-time volume term of the sources and
 * non-conservative products; no scratch), gpr_fv_interfs replaces
 * solvers.fv.interfs1 / interfs2 (fv.h:12-15, fv.cpp:111-279: the interface
 * fluxes and path integrals, applied in place; scratch as gpr_fv_launcher).
 * The reference's separate nx / ny / dx / dy arguments are nX[ndim] and
 * dX[ndim] here. */
int gpr_fv_centers(double *u, const double *qh, const int32_t *nX, double dt,
                   const double *dX, int ndim, int sources, int time_dg,
                   const gpr_par *par, const uint8_t *mask, int nvar, void *stream);
int gpr_fv_interfs(double *u, const double *qh, const int32_t *nX, double dt,
                   const double *dX, int ndim, int time_dg, int flux,
                   const gpr_par *par, const uint8_t *mask, double *scratch,
                   int nvar, void *stream);

/* The face pass of gpr_fv_launcher alone (interfs1/interfs2, fv.cpp:111-279):
 * writes, per face and direction, the contribution subtracted from the left
 * cell (fb[face][0][V]) and from the right cell (fb[face][1][V]) into fb,
 * which has gpr_fv_scratch_doubles(nX, ndim, nvar) doubles (x faces first,
 * then y faces in 2D, each (nx+1)(ny+1) faces). */
int gpr_fv_face_fluxes(const double *qh, const int32_t *nX, double dt,
                       const double *dX, int ndim, int time_dg, int flux,
                       const gpr_par *par, const uint8_t *mask, double *fb,
                       int nvar, void *stream);

/* Replaces solvers.timestep (solvers/iterator.cpp:54-83) for one material:
 * dt = CFL / max_cells sum_d max_abs_eigs/dx_d, x0.2 while count <= 5,
 * clipped to tf - t.  The result is written to dt_out (device double).
 * `scratch` must hold gpr_timestep_scratch_doubles(ncell) doubles. */
int gpr_timestep_scratch_doubles(int64_t ncell);
int gpr_timestep(const double *u, int64_t ncell, const double *dX, int ndim,
                 double cfl, double t, double tf, int count,
                 const gpr_par *par, double *dt_out, double *scratch,
                 int nvar, void *stream);

/* Replaces solvers.renorm_distortion (solvers/utils.cpp:6-23) for one
 * material: A <- A * cbrt(rho / (rho0 det A)) where rho > 0. */
int gpr_renorm_distortion(double *u, int64_t ncell, const gpr_par *par,
                          int nvar, void *stream);

/* Replaces solvers.split.ode_launcher (solvers/split/ode.cpp:5-11): the
 * analytic stiff-source step (body force, distortion relaxation, thermal
 * impulse relaxation) of every cell over dt. */
int gpr_ode_launcher(double *u, int64_t ncell, double dt, const gpr_par *par,
                     int nvar, void *stream);

/* Replaces solvers.ader_stepper (solvers/steppers.cpp:10-22): one ADER-WENO
 * step u <- u + (WENO -> predictor -> FV) of one material grid, with ub
 * already filled by gpr_boundaries.  Caller scratch of
 * gpr_ader_scratch_doubles(nX, ndim, nvar) doubles holds wh, qh and the
 * stage temporaries; dt is a host value.  status as in gpr_predictor
 * (optional). */
long gpr_ader_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_ader_stepper(double *u, const double *ub, const int32_t *nX, int ndim,
                     double dt, const double *dX, int stiff, int flux,
                     const gpr_par *par, const uint8_t *mask, double *scratch,
                     int32_t *status, int nvar, void *stream);

/* Replaces solvers.iterator (solvers/iterator.cpp:85-170) for one
 * material, device resident: runs `nsteps` steps of
 *   CFL time step -> boundaries -> WENO -> predictor -> FV -> renorm
 * with the clock in device memory, clock[5] = {t, dt, tf, cfl, count}
 * (count stored as a double).  Steps taken once t >= tf change nothing, so
 * a fixed number of steps can be enqueued or captured in a CUDA graph without
 * a host synchronisation.  Caller scratch of
 * gpr_iterate_scratch_doubles(nX, ndim, nvar) doubles; mask may be NULL (all
 * cells); status as in gpr_predictor (optional, last step's). */
long gpr_iterate_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_iterate(double *u, const int32_t *nX, int ndim, const double *dX,
                const int32_t *bcs, int flux, const gpr_par *par,
                const uint8_t *mask, double *clock, int nsteps, double *scratch,
                int32_t *status, double contorted_tol, int nvar, void *stream);

/* After each step of gpr_iterate, gpr_iterate_split and gpr_iterate_multi:
 * contorted + reset_distortion (solvers/utils.cpp:44-85, called by
 * iterator.cpp:150-151 with the driver's contorted_tol, 1.0 in
 * code/python/main.py:21): if any cell's normalised distortion has
 * m0 - 1 > contorted_tol, m0 = |A|_F^2 / (3 |det A|^(2/3)), every cell of a
 * non-vacuum material gets A = (rho / rho0)^(1/3) I and loses its distortion
 * energy.  INFINITY disables it.  gpr_reset_contorted does it once on u
 * (pars[nmat], nmat 1 or 2 with the material from the level set); *flag
 * (device int32) is set to 1 if it reset. */
/* The check alone (GPRpy.solvers.contorted, utils.cpp:65-85): *flag
 * (device int32) = 1 if any cell has m0 - 1 > contorted_tol, else 0. */
int gpr_contorted(const double *u, int64_t ncell, double contorted_tol, int32_t *flag,
                  int nvar, void *stream);
int gpr_reset_contorted(double *u, int64_t ncell, double contorted_tol, const gpr_par *pars,
                        int nmat, int32_t *flag, int nvar, void *stream);

/* One 1D ADER-WENO step that allocates nothing and takes no scratch.  It has
 * no counterpart in the reference.  It is for callers that cannot allocate
 * device memory (an application that owns the device through its own fixed
 * pool, or a loop where an allocation would synchronise the device): the
 * WENO, predictor and face-flux scratch comes from a fixed array compiled
 * into the library, sized for nx <= GPR_NOALLOC_MAX_CELLS cells of at most 17
 * variables (about 4.5 MB, held by every GPU that loads the library until the
 * process exits).  Larger grids are rejected with GPR_E_TOO_LARGE.  The
 * array's device address is looked up on the first call made on each device,
 * so that first call must come before any stream capture; the address is
 * kept for the life of the process, so the entry point must not be used
 * across a cudaDeviceReset.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller.  Otherwise as
 * gpr_ader_stepper with ndim = 1: nvar 17, 15 or 14, any of the three flux
 * codes, mask, status and stiff as there. */
#define GPR_NOALLOC_MAX_CELLS 4096
int gpr_ader_stepper_1d_noalloc(double *u, const double *ub, int32_t nx,
                                double dt, double dx, int stiff, int flux,
                                const gpr_par *par, const uint8_t *mask,
                                int32_t *status, int nvar, void *stream);

/* ------------------------------------------------------------------------ */
/* The step at another number of Gauss nodes.  The reference fixes N (its
 * basis functions / Gauss nodes per dimension) at compile time
 * (code/cpp/src/options.h:15); N = 3 is its third-order scheme: degree-2
 * polynomials in space and time and a WENO reconstruction that adds the
 * central stencil with weight LAMC = 1e5 (solvers/weno/weno.cpp:17-73).
 * These entry points take N as `order`: 3 for V = 17 or 14, and 2 for
 * V = 17 (the same formulation at N = 2, a cross-check of the N = 2 kernels
 * above).  1D and 2D grids (ndim = 1 or 2; every extent at least N); the
 * Rusanov, Roe and Osher fluxes (the eigen dissipation with N path nodes,
 * one thread per face point).  Layouts as
 * above with N = order, n_s = N^ndim space nodes per cell:
 *   ub [nx + 2N] ([ny + 2N]) [V], wh [nx + 2] ([ny + 2]) [n_s][V],
 *   qh [nx + 2] ([ny + 2]) [N][n_s][V], space nodes x-major.
 * Each replaces the entry point of the same name without _n; the predictor
 * runs the reference's Picard iteration (dg/dg1.cpp:58-114, dg2.cpp:
 * 102-171), and the stiff-source Newton pass of gpr_predictor finishes the
 * cells whose iteration does not converge within 50 steps or turns NaN
 * (every cell with stiff != 0), its correction systems (9N) x (9N) for the
 * distortion and (3N) x (3N) for the heat flux; `status` as there.
 * The 2D WENO needs device scratch of gpr_weno_scratch_doubles_n doubles for
 * its x sweep (0 in 1D, where scratch may be NULL).
 * gpr_order_supported returns 1 for the (order, ndim, nvar) compiled in;
 * gpr_scheme_constants_n writes nodes[N], weights[N], end values [2][N],
 * derivative values [N][N] and the oscillation indicator [N][N] (returns
 * the count, 4N + 2N^2). */
int gpr_order_supported(int order, int ndim, int nvar);
int gpr_scheme_constants_n(double *out, int n, int order);
int gpr_boundaries_n(const double *u, double *ub, const int32_t *nX, int ndim,
                     const int32_t *bcs, int nvar, int order, void *stream);
long gpr_weno_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order);
int gpr_weno_launcher_n(double *wh, const double *ub, const int32_t *nX, int ndim,
                        double *scratch, int nvar, int order, void *stream);
int gpr_predictor_n(double *qh, const double *wh, double dt, const double *dX, int ndim,
                    const int32_t *nX, int stiff, const gpr_par *par, const uint8_t *mask,
                    int32_t *status, int nvar, int order, void *stream);
long gpr_fv_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order);
int gpr_fv_launcher_n(double *u, const double *qh, const int32_t *nX, double dt,
                      const double *dX, int ndim, int flux, const gpr_par *par,
                      const uint8_t *mask, double *scratch, int nvar, int order,
                      void *stream);
long gpr_ader_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order);
int gpr_ader_stepper_n(double *u, const double *ub, const int32_t *nX, int ndim, double dt,
                       const double *dX, int stiff, int flux, const gpr_par *par,
                       const uint8_t *mask, double *scratch, int32_t *status, int nvar,
                       int order, void *stream);
long gpr_iterate_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order);
int gpr_iterate_n(double *u, const int32_t *nX, int ndim, const double *dX,
                  const int32_t *bcs, int flux, const gpr_par *par, const uint8_t *mask,
                  double *clock, int nsteps, double *scratch, int32_t *status,
                  double contorted_tol, int nvar, int order, void *stream);

/* ------------------------------------------------------------------------ */
/* Split scheme (the reference driver's default, SPLIT = true):
 * gpr_midstepper      GPRpy.solvers.split.midstepper (split/homogeneous.h:7):
 *                     wh -= dt/2 (dF/dx + B dw/dx)/dx [+ y] at the WENO nodes.
 * gpr_split_stepper   GPRpy.solvers.split_stepper (steppers.h:13-17,
 *                     steppers.cpp:50-66): ODE half step on u and ub (ub is
 *                     modified), WENO, midstepper if half_step, FV update on
 *                     the node values without sources or time integration,
 *                     ODE half step on u.  scratch: gpr_split_scratch_doubles.
 * gpr_iterate_split   gpr_iterate with the split scheme in place of the ADER
 *                     step (iterator.cpp:109-151); scratch: gpr_iterate_scratch_doubles. */
int gpr_midstepper(double *wh, double dt, const double *dX, int ndim, const int32_t *nX,
                   const gpr_par *par, const uint8_t *mask, int nvar, void *stream);
long gpr_split_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_split_stepper(double *u, double *ub, const int32_t *nX, int ndim, double dt,
                      const double *dX, int half_step, int flux, const gpr_par *par,
                      const uint8_t *mask, double *scratch, int nvar, void *stream);
int gpr_iterate_split(double *u, const int32_t *nX, int ndim, const double *dX,
                      const int32_t *bcs, int flux, int half_step, const gpr_par *par,
                      const uint8_t *mask, double *clock, int nsteps, double *scratch,
                      double contorted_tol, int nvar, void *stream);

/* ------------------------------------------------------------------------ */
/* Batched form: many independent 1D grids (instances) of uneven sizes, each
 * with its own material, boundary codes and CFL clock, advanced together by
 * one launch per stage (no counterpart in the reference, which runs one grid
 * per `iterator` call; each instance follows solvers/iterator.cpp:109-151).
 *
 * Instances are packed one after another in u: instance k owns
 * u[off_k .. off_k + nx[k]) cells, off_k = nx[0] + ... + nx[k-1].  The
 * device clock array holds {t, dt, tf, cfl, count} per instance (count as a
 * double); an instance whose t has reached tf gets dt = 0 and its steps
 * change nothing, so a fixed number of steps can be enqueued or captured in
 * a CUDA graph without host synchronisation.
 *
 * gpr_batch_init writes the instance tables (materials, maps, offsets) into
 * the caller's scratch (gpr_batch_scratch_doubles doubles) and sets every
 * clock to t = 0; it synchronises the stream once (the tables are copied from
 * host memory).  gpr_batch_iterate then runs nsteps steps.  `status`
 * (optional) receives the predictor status of each packed predictor cell
 * (nx[k] + 2 per instance); `updates` (optional, device uint64) accumulates
 * the cell-updates performed (sum of nx[k] over instances that advanced). */
long gpr_batch_scratch_doubles(int ninst, const int32_t *nx, int nvar);
int gpr_batch_init(double *clock, int ninst, const int32_t *nx,
                   const double *dx, const int32_t *bcs, const gpr_par *pars,
                   double cfl, double tf, double *scratch, int nvar,
                   void *stream);
int gpr_batch_iterate(double *u, double *clock, int ninst, const int32_t *nx,
                      int nsteps, double *scratch, int32_t *status,
                      unsigned long long *updates, int nvar, void *stream);

/* Autotuner of the batched step's launch shapes (no counterpart in the
 * reference).  The shapes are GPR_BATCH_NSHAPES int32 values:
 *   [0] WENO threads per block (one thread per cell and variable),
 *   [1] first-iterate threads per block (2 lanes per predictor cell),
 *   [2] Picard threads per block (4 lanes per predictor cell),
 *   [3] face-pass lane layout: 0 two lanes per face (one per time node),
 *       1 four lanes per face (per time node and side),
 *   [4] face-pass threads per block,
 *   [5] volume-pass threads per block (4 lanes per cell).
 * gpr_batch_autotune times every candidate of each stage on the batch's
 * current state with CUDA events on `stream` (WENO 64/128/256/512; first
 * iterate x Picard 32/64/128 each; faces both layouts x 32/64/128; volume
 * 32/64/128) and keeps the fastest for this batch (the scratch buffer
 * names the batch): later gpr_batch_iterate calls on it launch with those
 * shapes.  u is unchanged; each clock holds the coming step's dt.  It
 * synchronises the stream (not capturable); `shapes` (optional) receives
 * the choice, `times` (optional, GPR_BATCH_NCAND floats) the mean ms of
 * each candidate in the order above.  gpr_batch_init resets a batch to the
 * default shapes {256, 128, 128, 0, 128, 128}; gpr_batch_get_shapes /
 * gpr_batch_set_shapes read and restore a choice (block sizes 32, 64 or 128,
 * WENO a multiple of 32 up to 1024). */
#define GPR_BATCH_NSHAPES 6
#define GPR_BATCH_NCAND 22
int gpr_batch_autotune(double *u, double *clock, int ninst, const int32_t *nx,
                       double *scratch, int32_t *shapes, float *times, int nvar,
                       void *stream);
int gpr_batch_get_shapes(const double *scratch, int32_t *shapes);
int gpr_batch_set_shapes(const double *scratch, const int32_t *shapes);

/* ------------------------------------------------------------------------ */
/* Adjoint of the batched 1D step (no counterpart in the reference, which
 * has no derivatives): reverse-mode cotangents of a misfit with respect to
 * the initial states and six material fields of every instance.
 *
 * Differentiable model: stiffened-gas EOS, Newtonian viscosity (flags 0),
 * beta = 0, Tref = 0, Rusanov flux, boundary codes other than "moving".
 * The six fields are the DevPar members {gamma, 1/Gamma, b02, rho0 /
 * (2 mu^(1/n)), calpha2, 1/kappa}; the caller maps them to its parameters.
 *
 * gpr_adj_forward_step runs one step of the batched form (gpr_batch_init
 * tables in `scratch`) with the predictor tolerances dg_tol / dg_it (tight,
 * e.g. 1e-13, so the predictor is its fixed point); with a non-NULL `tape`
 * (gpr_adj_tape_doubles doubles) it records what the backward step needs.
 * dt_mode 0 takes the CFL step and writes it to dt_io[ninst] if given;
 * dt_mode 1 takes dt_io as the step (a schedule held fixed).
 *
 * gpr_adj_backward_step maps the cotangent ubar of the state after a
 * recorded step to the cotangent before it (in place), adds the step's
 * material-field cotangents to thbar[ninst][6], and carries tbar[ninst] (the
 * cotangent of the clock t; start it at 0).  frozen_dt = 1 treats each dt as
 * a constant (the adjoint of the fixed-schedule forward); frozen_dt = 0
 * differentiates dt through the CFL rule (at ties of the CFL maximum the
 * smallest cell index is taken).  ascratch: gpr_adj_scratch_doubles
 * doubles.  info[nb] (int32 per packed predictor cell, zero it first) gets
 * bit 0 set where the transposed predictor iteration did not converge (and
 * the dense solve that replaces it failed), and bits 8 and up accumulate
 * the cell's transposed-iteration count over the backward steps. */
int gpr_adj_num_fields(void);
int gpr_adj_supported(int ninst, const gpr_par *pars, const int32_t *bcs, int nvar);
long gpr_adj_tape_doubles(int ninst, const int32_t *nx, int nvar);
long gpr_adj_scratch_doubles(int ninst, const int32_t *nx, int nvar);
int gpr_adj_forward_step(double *u, double *clock, int ninst, const int32_t *nx,
                         double *scratch, double *tape, double *dt_io, int dt_mode,
                         double dg_tol, int dg_it, int32_t *status, int nvar, void *stream);
int gpr_adj_backward_step(double *ubar, double *thbar, double *tbar, int frozen_dt, int ninst,
                          const int32_t *nx, const double *scratch, const double *tape,
                          double *ascratch, int32_t *info, int nvar, void *stream);
/* Jacobians of F_x, S and lambda_x at count states (test hook):
 * JF, JS [count][K][V] (column k = d/d(state k) for k < V, d/d(field k-V)
 * after), dlam [count][K]; K = V + 6. */
int gpr_adj_point_jacobians(const double *Q, int64_t count, const gpr_par *par, double *JF,
                            double *JS, double *dlam, int nvar, void *stream);
/* Reverse-mode products at count states (test hook): qb[count][V] =
 * (dF_x/dq)^T Fb + (dS/dq)^T Sb + lb dlambda_x/dq, thb[count][6] the same
 * with respect to the six material fields; Fb, Sb [count][V], lb [count].
 * The backward step uses these products in place of full Jacobians. */
int gpr_adj_point_vjp(const double *Q, int64_t count, const gpr_par *par, const double *Fb,
                      const double *Sb, const double *lb, double *qb, double *thb, int nvar,
                      void *stream);

/* ------------------------------------------------------------------------ */
/* Level-set ghost fluid (GPRpy.multi.*, code/cpp/src/multi/*.cpp, and
 * system/multi/riemann.cpp) for the V = 15 layout (viscous, one level set,
 * no heat conduction) and exactly two materials: material 0 occupies
 * phi < 0, material 1 phi >= 0 (functions/vectors.cpp:24-31); pars[2].
 * nX[d] >= 3.  Every fill call accumulates error counts in the caller's
 * device status[4] (zero it first): [0] bit 0: the re-distancing did not
 * converge within its budget, bit 2: its grid barrier gave up waiting
 * (~1 s), [1] boundary cells whose fill would read outside the grid in the
 * reference (left unfilled), [2] extrapolation cells whose copy source
 * would lie outside the grid (they copy their layer neighbour), [3]
 * gpr_distance on a 2D grid: the global sweeps its re-distancing took
 * (untouched otherwise).
 *
 * gpr_distance             GPRpy.system.multi.distance (multi/pfmm.cpp:4-26):
 *                          first-order signed distance to the zero level of
 *                          phi[ncell]; zeros if phi has no zero crossing.
 *                          scratch: gpr_distance_scratch_doubles.
 * gpr_finite_difference    GPRpy.multi.finite_difference
 *                          (multi/functions.cpp:16-54): dphi[ncell][ndim].
 * gpr_find_interface_cells GPRpy.multi.find_interface_cells (multi/fill.cpp:20-74):
 *                          intMask[ncell] in {-2, -1, 0, 1}.
 * gpr_left_star_state      GPRpy.system.multi.left_star_state
 *                          (riemann.cpp:203-233), batched: out[k] = left star
 *                          state of QL[k] | QR[k] along n[k][ndim].
 * gpr_fill_boundary_cells  GPRpy.multi.fill_boundary_cells (multi/fill.cpp:200-235):
 *                          grid of material mat, its level set phi, normals
 *                          dphi and intMask; scratch: gpr_fill_scratch_doubles.
 * gpr_fill_neighbor_cells  GPRpy.multi.fill_neighbor_cells (multi/fill.cpp:255-328):
 *                          intMask updated in place; scratch: gpr_fill_scratch_doubles.
 * gpr_fill_ghost_cells     GPRpy.multi.fill_ghost_cells (multi/fill.cpp:330-370):
 *                          re-distances u's level set in place and writes
 *                          grids[2][ncell][V] and masks[2][ncell].
 * gpr_make_u               GPRpy.solvers.make_u (solvers/iterator.cpp:12-42).
 * gpr_renorm_multi         GPRpy.solvers.renorm_distortion (solvers/utils.cpp:6-23)
 *                          with each cell's material from its level set.
 * gpr_timestep_multi       solvers/iterator.cpp:54-83 over the masked cells of
 *                          both grids; dt_out is a device double; scratch: 1 double.
 * gpr_iterate_multi        GPRpy.solvers.iterator (solvers/iterator.cpp:85-170)
 *                          with the ghost fill, ADER scheme, flux
 *                          GPR_FLUX_* (Rusanov, Roe or Osher), device
 *                          resident as gpr_iterate; clock[5] as there (set
 *                          dt = 0 before the first step); scratch:
 *                          gpr_iterate_multi_scratch_doubles.
 * gpr_iterate_multi_scheme the same loop with the reference iterator's
 *                          SPLIT, HALF_STEP and STIFF arguments
 *                          (iterator.cpp:85-88, 123-129): split != 0 steps
 *                          each material with the split scheme (ODE half
 *                          steps around the homogeneous WENO [-> midstepper
 *                          when half_step] -> FV step, as
 *                          gpr_split_stepper); otherwise the ADER step, its
 *                          predictor straight to the Newton iteration when
 *                          stiff != 0 (as gpr_predictor).  The reference's
 *                          Python driver runs this loop with SPLIT = True,
 *                          FLUX = 1 (code/python/main.py:19-22, 43-45). */
long gpr_distance_scratch_doubles(const int32_t *nX, int ndim);
int gpr_distance(const double *phi, double *dist, const int32_t *nX, int ndim,
                 const double *dX, double *scratch, int32_t *status, void *stream);
int gpr_finite_difference(const double *phi, double *dphi, const int32_t *nX, int ndim,
                          const double *dX, void *stream);
int gpr_find_interface_cells(const double *phi, int32_t *intMask, const int32_t *nX, int ndim,
                             void *stream);
int gpr_left_star_state(const double *QL, const double *QR, const double *n, double *out,
                        int64_t count, int ndim, double dt, const gpr_par *parL,
                        const gpr_par *parR, int nvar, void *stream);
long gpr_fill_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_fill_boundary_cells(double *grid, const int32_t *intMask, int mat, const double *phi,
                            const double *dphi, const double *dX, const gpr_par *pars,
                            int nmat, double dt, const int32_t *nX, int ndim, double *scratch,
                            int32_t *status, int nvar, void *stream);
int gpr_fill_neighbor_cells(double *grid, int32_t *intMask, const double *dphi,
                            const double *dX, const int32_t *nX, int ndim, double *scratch,
                            int32_t *status, int nvar, void *stream);
int gpr_fill_ghost_cells(double *grids, uint8_t *masks, double *u, const int32_t *nX, int ndim,
                         const double *dX, double dt, const gpr_par *pars, int nmat,
                         double *scratch, int32_t *status, int nvar, void *stream);
int gpr_make_u(double *u, const double *grids, const uint8_t *masks, int64_t ncell,
               const gpr_par *pars, int nmat, int nvar, void *stream);
int gpr_renorm_multi(double *u, int64_t ncell, const gpr_par *pars, int nmat, int nvar,
                     void *stream);
int gpr_timestep_multi(const double *grids, const uint8_t *masks, int64_t ncell,
                       const double *dX, int ndim, double cfl, double t, double tf, int count,
                       const gpr_par *pars, int nmat, double *dt_out, double *scratch,
                       int nvar, void *stream);
long gpr_iterate_multi_scratch_doubles(const int32_t *nX, int ndim, int nvar);
int gpr_iterate_multi(double *u, const int32_t *nX, int ndim, const double *dX,
                      const int32_t *bcs, int flux, const gpr_par *pars, int nmat,
                      double *clock, int nsteps, double *scratch, int32_t *status,
                      double contorted_tol, int nvar, void *stream);
int gpr_iterate_multi_scheme(double *u, const int32_t *nX, int ndim, const double *dX,
                             const int32_t *bcs, int split, int half_step, int stiff, int flux,
                             const gpr_par *pars, int nmat, double *clock, int nsteps,
                             double *scratch, int32_t *status, double contorted_tol, int nvar,
                             void *stream);

/* ------------------------------------------------------------------------ */
/* Pointwise physics (GPRpy.system.*, code/cpp/src/system/equations.cpp,
 * eig.cpp): batched over `count` states Q[count][V].                        */

/* out[count][V] += F_d(Q) (equations.cpp:11-48). */
int gpr_flux(const double *Q, double *out, int64_t count, int d,
             const gpr_par *par, int nvar, void *stream);
/* out[count][V] = S(Q) (equations.cpp:50-67). */
int gpr_source(const double *Q, double *out, int64_t count,
               const gpr_par *par, int nvar, void *stream);
/* out[count][V] = B_d(Q) x (equations.cpp:89-167). */
int gpr_Bdot(const double *Q, const double *x, double *out, int64_t count,
             int d, const gpr_par *par, int nvar, void *stream);
/* out[count] = max |eigenvalue| of the GPR system in direction d
 * (eig.cpp:66-77). */
int gpr_max_abs_eigs(const double *Q, double *out, int64_t count, int d,
                     const gpr_par *par, int nvar, void *stream);
/* out[count][V][V] (row = equation) = the system matrix dF_d/dQ + B_d of
 * the quasi-linear form along d (system/equations.cpp:169-176). */
int gpr_system_matrix(const double *Q, double *out, int64_t count, int d,
                      const gpr_par *par, int nvar, void *stream);
/* out[count][m][m] = Xi1 Xi2 along d (eig.cpp:55-64), m = 4 with heat
 * conduction (V = 17), else 3. */
int gpr_thermo_acoustic_tensor(const double *Q, double *out, int64_t count, int d,
                               const gpr_par *par, int nvar, void *stream);
/* Interface dissipation / jump terms (solvers/fv/fluxes.cpp:9-75):
 * out[count][V] = D_flux(qL, qR) including F(qL)+F(qR), and
 * bout[count][V] = Bint(qL, qR). */
int gpr_interface_terms(const double *qL, const double *qR, double *out,
                        double *bout, int64_t count, int d, int flux,
                        const gpr_par *par, int nvar, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GPR_GB300_H */
