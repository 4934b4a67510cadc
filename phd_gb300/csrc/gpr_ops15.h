// gpr_ops15.h - the stage launchers for the V = 15 layout (viscous, one level
// set), declared here and instantiated in gpr_multi.cu so that the V = 17 /
// V = 14 translation unit does not compile a third copy of every kernel.
// Same signatures as Ops<L> in gpr_ops.cuh.
#pragma once

#include "gpr_host.cuh"

namespace gpr {
namespace host {

struct Ops15 {
  static int boundaries(const double *u, double *ub, const int32_t *nX, int nd,
                        const int32_t *bcs, cudaStream_t st);
  static long weno_scratch(const int32_t *nX, int nd);
  static int weno(double *wh, const double *ub, const int32_t *nX, int nd, double *scratch,
                  cudaStream_t st);
  static int predictor(double *qh, const double *wh, double dt, const double *dt_dev,
                       const double *dX, int nd, const int32_t *nX, int stiff,
                       const DevPar &P, const uint8_t *mask, int32_t *status,
                       cudaStream_t st);
  static long fv_scratch(const int32_t *nX, int nd);
  static int fv(double *u, const double *qh, const int32_t *nX, double dt,
                const double *dt_dev, const double *dX, int nd, int sources, int time_dg,
                const DevPar &P, const uint8_t *mask, double *scratch, cudaStream_t st,
                int flux = GPR_FLUX_RUSANOV, int parts = 3);
  static int faces(const double *qh, const int32_t *nX, double dt, const double *dX, int nd,
                   int time_dg, const DevPar &P, const uint8_t *mask, double *fb,
                   cudaStream_t st, int flux = GPR_FLUX_RUSANOV);
  static int timestep(const double *u, long ncell, const double *dX, int nd, double cfl,
                      double t, double tf, int count, const DevPar &P, double *dt_out,
                      double *scratch, cudaStream_t st);
  static int renorm(double *u, long ncell, const DevPar &P, cudaStream_t st);
  static void contortion(double *u, long ncell, double tol, const DevPar &P0, const DevPar &P1,
                         int *flag, const double *dt_dev, cudaStream_t st);
  static int pointwise(int what, const double *Q, const double *X, double *out, double *out2,
                       long count, int d, int flux, const DevPar &P, cudaStream_t st);
  static int iterate(double *u, const int32_t *nX, int nd, const double *dX,
                     const int32_t *bcs, const DevPar &P, const uint8_t *mask, double *clk,
                     int nsteps, double *scratch, int32_t *status, cudaStream_t st,
                     int flux = GPR_FLUX_RUSANOV, double contorted_tol = INFINITY);
  static int midstep(double *wh, double dt, const double *dt_dev, const double *dX, int nd,
                     const int32_t *nX, const DevPar &P, const uint8_t *mask, cudaStream_t st);
  static int split_stepper(double *u, double *ub, const int32_t *nX, int nd, double dt,
                           const double *dt_dev, const double *dX, int half_step, int flux,
                           const DevPar &P, const uint8_t *mask, double *scratch,
                           cudaStream_t st);
  static long split_scratch(const int32_t *nX, int nd);
  static int iterate_split(double *u, const int32_t *nX, int nd, const double *dX,
                           const int32_t *bcs, const DevPar &P, const uint8_t *mask,
                           double *clk, int nsteps, double *scratch, int half_step, int flux,
                           cudaStream_t st, double contorted_tol = INFINITY);
  static long iterate_scratch(const int32_t *nX, int nd);
  static BatchLayout batch_layout(int ninst, const int32_t *nx);
  static int batch_iterate(double *u, double *clk, int ninst, const int32_t *nx, int nsteps,
                           double *scr, int32_t *status, unsigned long long *updates,
                           cudaStream_t st, const BatchShapes &sh = BatchShapes{});
  static int batch_autotune(double *u, double *clk, int ninst, const int32_t *nx, double *scr,
                            BatchShapes &sh, float *times, int reps, cudaStream_t st);
  static int ode(double *u, long ncell, double dt, const DevPar &P, cudaStream_t st);
};

}  // namespace host
}  // namespace gpr
