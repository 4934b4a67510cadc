// gpr_order.cu - C ABI of the 1D step at a chosen number of Gauss nodes
// (`order`, the reference's compile-time N): the kernels of gpr_order.cuh for
// N = 3, and the same kernels at N = 2 (a second formulation of the N = 2
// step, which the tests hold against the shuffle-based N = 2 kernels).
// CFL time step, renormalisation and contortion reset do not depend on N and
// are the N = 2 library's (gpr_ops.cuh).
#include <math.h>
#include <stdio.h>

#include "../../include/gpr_gb300.h"
#include "gpr_ops.cuh"
#include "gpr_order.cuh"

using namespace gpr;
using namespace gpr::host;
using namespace gpr::order;

namespace {

template <int NO> const ConstsN<NO> &consts_n() {
  static ConstsN<NO> c = make_consts_n<NO>();
  return c;
}

// The 1D step's stages at NO nodes for the layout L.
template <class L, int NO> struct OpsN {
  static constexpr int V = L::V;
  using NB = NodeBlock<NO>;

  static long ub_doubles(int nx) { return (long)(nx + 2 * NO) * V; }
  static long wh_doubles(int nx) { return (long)(nx + 2) * NO * V; }
  static long qh_doubles(int nx) { return (long)(nx + 2) * NO * NO * V; }
  static long fb_doubles(int nx) { return (long)(nx + 1) * NO * 2 * V; }

  static int boundaries(const double *u, double *ub, int nx, const int32_t *bcs,
                        cudaStream_t st) {
    long n = ub_doubles(nx);
    k_boundaries1d_n<V, NO><<<blocks(n, 256), 256, 0, st>>>(u, ub, nx, bcs[0], bcs[1]);
    return cuda_rc();
  }
  static int weno(double *wh, const double *ub, int nx, cudaStream_t st) {
    const int ncb = nx + 2;
    k_weno1d_n<V, NO><<<blocks((long)ncb * V, 256), 256, 0, st>>>(wh, ub, ncb, consts_n<NO>());
    return cuda_rc();
  }
  static int predictor(double *qh, const double *wh, double dt, const double *dt_dev, double dx,
                       int nx, const DevPar &P, const uint8_t *mask, int32_t *status,
                       cudaStream_t st) {
    const long ncb = nx + 2;
    k_predictor1d_n<L, NO><<<(unsigned)((ncb + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
        qh, wh, ncb, mask, status, dt, dt_dev, 1.0 / dx, P, consts_n<NO>());
    return cuda_rc();
  }
  static int fv(double *u, const double *qh, int nx, double dt, const double *dt_dev, double dx,
                const DevPar &P, const uint8_t *mask, double *fb, cudaStream_t st) {
    const long nf = (long)nx + 1;
    k_faces1d_n<L, NO><<<blocks(nf * NO, 128), 128, 0, st>>>(fb, qh, nf, mask, dt, dt_dev, dx,
                                                             P, consts_n<NO>());
    k_cells1d_n<L, NO><<<(unsigned)((nx + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
        u, qh, fb, nx, mask, dt, dt_dev, dx, P, consts_n<NO>());
    return cuda_rc();
  }
  // scratch: wh, qh, face terms
  static long step_scratch(int nx) { return wh_doubles(nx) + qh_doubles(nx) + fb_doubles(nx); }
  static int step(double *u, const double *ub, int nx, double dt, const double *dt_dev,
                  double dx, const DevPar &P, const uint8_t *mask, double *scr,
                  int32_t *status, cudaStream_t st) {
    double *wh = scr, *qh = wh + wh_doubles(nx), *fb = qh + qh_doubles(nx);
    int rc;
    if ((rc = weno(wh, ub, nx, st)))
      return rc;
    if ((rc = predictor(qh, wh, dt, dt_dev, dx, nx, P, mask, status, st)))
      return rc;
    return fv(u, qh, nx, dt, dt_dev, dx, P, mask, fb, st);
  }
  // scratch: ub, the step's scratch, the CFL maximum and the contortion flag
  static long iterate_scratch(int nx) { return ub_doubles(nx) + step_scratch(nx) + 2; }
  static int iterate(double *u, int nx, double dx, const int32_t *bcs, const DevPar &P,
                     const uint8_t *mask, double *clk, int nsteps, double *scr,
                     int32_t *status, double contorted_tol, cudaStream_t st) {
    double *ub = scr, *sscr = ub + ub_doubles(nx);
    unsigned long long *mx = (unsigned long long *)(sscr + step_scratch(nx));
    const double *dt_dev = clk + 1;
    for (int s = 0; s < nsteps; s++) {
      cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st);
      k_cfl_max<L><<<blocks(nx, 256), 256, 0, st>>>(u, nx, 1, dx, 1.0, mx, P);
      k_clock_finalize<<<1, 1, 0, st>>>(mx, clk);
      int rc = boundaries(u, ub, nx, bcs, st);
      if (!rc)
        rc = step(u, ub, nx, 0.0, dt_dev, dx, P, mask, sscr, status, st);
      if (rc)
        return rc;
      k_renorm<V><<<blocks(nx, 256), 256, 0, st>>>(u, nx, P.rho0, dt_dev);
      Ops<L>::contortion(u, nx, contorted_tol, P, P, (int *)(mx + 1), dt_dev, st);
      k_clock_advance<<<1, 1, 0, st>>>(clk);
    }
    return cuda_rc();
  }
};

// Dispatch on (nvar, order); CALL uses O.
#define DISPATCH_N(nvar, order, CALL)                                                        \
  do {                                                                                       \
    if (nvar == 17 && order == 3) {                                                          \
      using O = OpsN<L17, 3>;                                                                \
      return CALL;                                                                           \
    }                                                                                        \
    if (nvar == 14 && order == 3) {                                                          \
      using O = OpsN<L14, 3>;                                                                \
      return CALL;                                                                           \
    }                                                                                        \
    if (nvar == 17 && order == 2) {                                                          \
      using O = OpsN<L17, 2>;                                                                \
      return CALL;                                                                           \
    }                                                                                        \
    return GPR_E_UNSUPPORTED;                                                                \
  } while (0)

bool bad_grid(const int32_t *nX, int ndim, int order) {
  return !nX || ndim != 1 || nX[0] < order || order < 2;
}

}  // namespace

extern "C" {

int gpr_order_supported(int order, int ndim, int nvar) {
  if (ndim != 1)
    return 0;
  return (order == 3 && (nvar == 17 || nvar == 14)) || (order == 2 && nvar == 17);
}

int gpr_scheme_constants_n(double *out, int n, int order) {
  if (!out)
    return GPR_E_ARG;
  auto put = [&](auto &C, int NO) {
    const int count = 4 * NO + 2 * NO * NO;
    if (n < count)
      return GPR_E_ARG;
    int k = 0;
    for (int i = 0; i < NO; i++)
      out[k++] = C.nodes[i];
    for (int i = 0; i < NO; i++)
      out[k++] = C.w[i];
    for (int e = 0; e < 2; e++)
      for (int i = 0; i < NO; i++)
        out[k++] = C.endv[e][i];
    for (int i = 0; i < NO; i++)
      for (int j = 0; j < NO; j++)
        out[k++] = C.derv[i][j];
    for (int i = 0; i < NO; i++)
      for (int j = 0; j < NO; j++)
        out[k++] = C.sig[i][j];
    return count;
  };
  if (order == 3)
    return put(consts_n<3>(), 3);
  if (order == 2)
    return put(consts_n<2>(), 2);
  return GPR_E_UNSUPPORTED;
}

int gpr_boundaries_n(const double *u, double *ub, const int32_t *nX, int ndim,
                     const int32_t *bcs, int nvar, int order, void *stream) {
  if (!u || !ub || !bcs || bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  for (int s = 0; s < 2; s++)
    if (bcs[s] < 0 || bcs[s] > 5)
      return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::boundaries(u, ub, nX[0], bcs, S(stream)));
}

int gpr_weno_launcher_n(double *wh, const double *ub, const int32_t *nX, int ndim, int nvar,
                        int order, void *stream) {
  if (!wh || !ub || bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::weno(wh, ub, nX[0], S(stream)));
}

int gpr_predictor_n(double *qh, const double *wh, double dt, const double *dX, int ndim,
                    const int32_t *nX, const gpr_par *par, const uint8_t *mask, int32_t *status,
                    int nvar, int order, void *stream) {
  if (!qh || !wh || !dX || !par || bad_grid(nX, ndim, order) || !(dX[0] > 0))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order,
             O::predictor(qh, wh, dt, nullptr, dX[0], nX[0], P, mask, status, S(stream)));
}

long gpr_fv_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::fb_doubles(nX[0]));
}

int gpr_fv_launcher_n(double *u, const double *qh, const int32_t *nX, double dt,
                      const double *dX, int ndim, int flux, const gpr_par *par,
                      const uint8_t *mask, double *scratch, int nvar, int order, void *stream) {
  if (!u || !qh || !dX || !par || !scratch || bad_grid(nX, ndim, order) || !(dX[0] > 0))
    return GPR_E_ARG;
  if (flux != GPR_FLUX_RUSANOV)
    return flux == GPR_FLUX_ROE || flux == GPR_FLUX_OSHER ? GPR_E_UNSUPPORTED : GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order,
             O::fv(u, qh, nX[0], dt, nullptr, dX[0], P, mask, scratch, S(stream)));
}

long gpr_ader_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::step_scratch(nX[0]));
}

int gpr_ader_stepper_n(double *u, const double *ub, const int32_t *nX, int ndim, double dt,
                       const double *dX, int flux, const gpr_par *par, const uint8_t *mask,
                       double *scratch, int32_t *status, int nvar, int order, void *stream) {
  if (!u || !ub || !dX || !par || !scratch || bad_grid(nX, ndim, order) || !(dX[0] > 0))
    return GPR_E_ARG;
  if (flux != GPR_FLUX_RUSANOV)
    return flux == GPR_FLUX_ROE || flux == GPR_FLUX_OSHER ? GPR_E_UNSUPPORTED : GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order,
             O::step(u, ub, nX[0], dt, nullptr, dX[0], P, mask, scratch, status, S(stream)));
}

long gpr_iterate_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::iterate_scratch(nX[0]));
}

int gpr_iterate_n(double *u, const int32_t *nX, int ndim, const double *dX, const int32_t *bcs,
                  int flux, const gpr_par *par, const uint8_t *mask, double *clock, int nsteps,
                  double *scratch, int32_t *status, double contorted_tol, int nvar, int order,
                  void *stream) {
  if (!u || !dX || !bcs || !par || !clock || !scratch || nsteps < 0 ||
      bad_grid(nX, ndim, order) || !(dX[0] > 0))
    return GPR_E_ARG;
  for (int s = 0; s < 2; s++)
    if (bcs[s] < 0 || bcs[s] > 5)
      return GPR_E_ARG;
  if (flux != GPR_FLUX_RUSANOV)
    return flux == GPR_FLUX_ROE || flux == GPR_FLUX_OSHER ? GPR_E_UNSUPPORTED : GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order, O::iterate(u, nX[0], dX[0], bcs, P, mask, clock, nsteps, scratch,
                                     status, contorted_tol, S(stream)));
}

}  // extern "C"
