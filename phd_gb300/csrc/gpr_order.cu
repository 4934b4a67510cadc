// gpr_order.cu - C ABI of the 1D and 2D step at a chosen number of Gauss nodes
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

// The step's stages at NO nodes for the layout L on a 1D or 2D grid
// (nX[0] [x nX[1]] interior cells).
template <class L, int NO> struct OpsN {
  static constexpr int V = L::V;

  struct Grid {
    int nd, nx, ny;
    Grid(const int32_t *nX, int nd_) : nd(nd_), nx(nX[0]), ny(nd_ == 2 ? nX[1] : 1) {}
    long ncell() const { return (long)nx * ny; }
    long ncb() const { return nd == 1 ? nx + 2 : (long)(nx + 2) * (ny + 2); }
    long nub() const { return nd == 1 ? nx + 2 * NO : (long)(nx + 2 * NO) * (ny + 2 * NO); }
    int ns() const { return nd == 1 ? NO : NO * NO; }
    // face grid of one direction: 1D nx + 1 faces; 2D (nx + 1) x (ny + 1)
    long nface() const { return nd == 1 ? nx + 1 : (long)(nx + 1) * (ny + 1); }
  };

  static long ub_doubles(const Grid &g) { return g.nub() * V; }
  static long wh_doubles(const Grid &g) { return g.ncb() * g.ns() * V; }
  static long qh_doubles(const Grid &g) { return g.ncb() * NO * g.ns() * V; }
  // the face terms of every direction (the x sweep's node values of the 2D
  // WENO use the same scratch before them)
  static long fb_doubles(const Grid &g) {
    const long faces = g.nface() * g.ns() * 2 * V * g.nd;
    const long ux = g.nd == 1 ? 0 : (long)(g.nx + 2) * (g.ny + 2 * NO) * NO * V;
    return faces > ux ? faces : ux;
  }

  static int boundaries(const double *u, double *ub, const Grid &g, const int32_t *bcs,
                        cudaStream_t st) {
    k_boundaries_n<V, NO><<<blocks(g.nub(), 128), 128, 0, st>>>(
        u, ub, g.nx, g.ny, g.nd, bcs[0], bcs[1], g.nd == 2 ? bcs[2] : 0,
        g.nd == 2 ? bcs[3] : 0);
    return cuda_rc();
  }
  static int weno(double *wh, const double *ub, const Grid &g, double *tmp, cudaStream_t st) {
    const ConstsN<NO> &C = consts_n<NO>();
    if (g.nd == 1) {
      const int ncb = g.nx + 2;
      k_weno1d_n<V, NO><<<blocks((long)ncb * V, 256), 256, 0, st>>>(wh, ub, ncb, C);
      return cuda_rc();
    }
    const int nxp = g.nx + 2, nyp = g.ny + 2, nyb = g.ny + 2 * NO;
    k_weno2d_x_n<V, NO><<<blocks((long)nxp * nyb * V, 256), 256, 0, st>>>(tmp, ub, nxp, nyb, C);
    k_weno2d_y_n<V, NO><<<blocks((long)nxp * nyp * NO * V, 256), 256, 0, st>>>(wh, tmp, nxp, nyp,
                                                                              C);
    return cuda_rc();
  }
  // Picard pass, then the stiff Newton pass over the cells it marked (all
  // cells with stiff): a persistent grid of one-warp blocks, each taking
  // windows of 32 cells.
  static int predictor(double *qh, const double *wh, double dt, const double *dt_dev,
                       const double *dX, const Grid &g, int stiff, const DevPar &P,
                       const uint8_t *mask, int32_t *status, cudaStream_t st) {
    const long ncb = g.ncb();
    const double idx = 1.0 / dX[0], idy = g.nd == 2 ? 1.0 / dX[1] : 1.0;
    const ConstsN<NO> &C = consts_n<NO>();
    if (g.nd == 1) {
      using NB = NodeBlock<NO, 1>;
      k_predictor_n<L, NO, 1><<<(unsigned)((ncb + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
          qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C);
      k_predictor_stiff_n<L, NO, 1><<<stiff_grid(k_predictor_stiff_n<L, NO, 1>, ncb), 32, 0,
                                      st>>>(qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, P,
                                            C);
    } else {
      using NB = NodeBlock<NO, 2>;
      k_predictor_n<L, NO, 2><<<(unsigned)((ncb + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
          qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, stiff, P, C);
      k_predictor_stiff_n<L, NO, 2><<<stiff_grid(k_predictor_stiff_n<L, NO, 2>, ncb), 32, 0,
                                      st>>>(qh, wh, ncb, mask, status, dt, dt_dev, idx, idy, P,
                                            C);
    }
    return cuda_rc();
  }
  template <class K> static unsigned stiff_grid(K kernel, long ncb) {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32, 0);
    long grid = (long)sm_count() * (per_sm > 0 ? per_sm : 1);
    const long windows = (ncb + 31) / 32;
    return (unsigned)(grid < windows ? grid : windows);
  }
  // Face terms of direction dir: Rusanov, or the Roe / Osher eigen
  // dissipation at one thread per face point in 64-thread blocks (its 17 x 17
  // matrices live in local memory, as in the N = 2 per-point kernel).
  template <int ND>
  static void faces(double *fb, const double *qh, const Grid &g, int dir, double dt,
                    const double *dt_dev, const double *dX, int flux, const DevPar &P,
                    const uint8_t *mask, cudaStream_t st) {
    const ConstsN<NO> &C = consts_n<NO>();
    const long n = g.nface() * (ND == 1 ? NO : NO * NO);
    const double dy = g.nd == 2 ? dX[1] : 1.0;
    if (flux == GPR_FLUX_RUSANOV)
      k_faces_n<L, NO, ND><<<blocks(n, 128), 128, 0, st>>>(fb, qh, g.nx, g.ny, dir, mask, dt,
                                                           dt_dev, dX[0], dy, P, C);
    else
      k_faces_n<L, NO, ND, true><<<blocks(n, 64), 64, 0, st>>>(
          fb, qh, g.nx, g.ny, dir, mask, dt, dt_dev, dX[0], dy, P, C, flux);
  }
  static int fv(double *u, const double *qh, const Grid &g, double dt, const double *dt_dev,
                const double *dX, int flux, const DevPar &P, const uint8_t *mask, double *fb,
                cudaStream_t st) {
    const ConstsN<NO> &C = consts_n<NO>();
    const long nf = g.nface();
    const double dy = g.nd == 2 ? dX[1] : 1.0;
    if (g.nd == 1) {
      using NB = NodeBlock<NO, 1>;
      faces<1>(fb, qh, g, 0, dt, dt_dev, dX, flux, P, mask, st);
      k_cells_n<L, NO, 1><<<(unsigned)((g.nx + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
          u, qh, fb, nullptr, g.nx, 1, mask, dt, dt_dev, dX[0], dy, P, C);
      return cuda_rc();
    }
    using NB = NodeBlock<NO, 2>;
    double *fby = fb + nf * NO * NO * 2 * V;
    for (int d = 0; d < 2; d++)
      faces<2>(d ? fby : fb, qh, g, d, dt, dt_dev, dX, flux, P, mask, st);
    k_cells_n<L, NO, 2><<<(unsigned)((g.ncell() + NB::CPB - 1) / NB::CPB), 128, 0, st>>>(
        u, qh, fb, fby, g.nx, g.ny, mask, dt, dt_dev, dX[0], dy, P, C);
    return cuda_rc();
  }
  // scratch: wh, qh, face terms
  static long step_scratch(const Grid &g) { return wh_doubles(g) + qh_doubles(g) + fb_doubles(g); }
  static int step(double *u, const double *ub, const Grid &g, double dt, const double *dt_dev,
                  const double *dX, int stiff, int flux, const DevPar &P, const uint8_t *mask,
                  double *scr, int32_t *status, cudaStream_t st) {
    double *wh = scr, *qh = wh + wh_doubles(g), *fb = qh + qh_doubles(g);
    int rc;
    if ((rc = weno(wh, ub, g, fb, st)))
      return rc;
    if ((rc = predictor(qh, wh, dt, dt_dev, dX, g, stiff, P, mask, status, st)))
      return rc;
    return fv(u, qh, g, dt, dt_dev, dX, flux, P, mask, fb, st);
  }
  // scratch: ub, the step's scratch, the CFL maximum and the contortion flag
  static long iterate_scratch(const Grid &g) { return ub_doubles(g) + step_scratch(g) + 2; }
  static int iterate(double *u, const Grid &g, const double *dX, const int32_t *bcs, int flux,
                     const DevPar &P, const uint8_t *mask, double *clk, int nsteps, double *scr,
                     int32_t *status, double contorted_tol, cudaStream_t st) {
    double *ub = scr, *sscr = ub + ub_doubles(g);
    unsigned long long *mx = (unsigned long long *)(sscr + step_scratch(g));
    const double *dt_dev = clk + 1;
    const long ncell = g.ncell();
    for (int s = 0; s < nsteps; s++) {
      cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st);
      k_cfl_max<L><<<blocks(ncell, 256), 256, 0, st>>>(u, ncell, g.nd, dX[0],
                                                        g.nd == 2 ? dX[1] : 1.0, mx, P);
      k_clock_finalize<<<1, 1, 0, st>>>(mx, clk);
      int rc = boundaries(u, ub, g, bcs, st);
      if (!rc)
        rc = step(u, ub, g, 0.0, dt_dev, dX, 0, flux, P, mask, sscr, status, st);
      if (rc)
        return rc;
      k_renorm<V><<<blocks(ncell, 256), 256, 0, st>>>(u, ncell, P.rho0, dt_dev);
      Ops<L>::contortion(u, ncell, contorted_tol, P, P, (int *)(mx + 1), dt_dev, st);
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
  return !nX || (ndim != 1 && ndim != 2) || order < 2 || nX[0] < order ||
         (ndim == 2 && nX[1] < order);
}

bool bad_bcs(const int32_t *bcs, int ndim) {
  if (!bcs)
    return true;
  for (int s = 0; s < 2 * ndim; s++)
    if (bcs[s] < 0 || bcs[s] > 5)
      return true;
  return false;
}

bool bad_dX(const double *dX, int ndim) {
  return !dX || !(dX[0] > 0) || (ndim == 2 && !(dX[1] > 0));
}

bool bad_flux(int flux) {
  return flux != GPR_FLUX_RUSANOV && flux != GPR_FLUX_ROE && flux != GPR_FLUX_OSHER;
}

}  // namespace

extern "C" {

int gpr_order_supported(int order, int ndim, int nvar) {
  if (ndim != 1 && ndim != 2)
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
  if (!u || !ub || bad_grid(nX, ndim, order) || bad_bcs(bcs, ndim))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::boundaries(u, ub, typename O::Grid(nX, ndim), bcs, S(stream)));
}

long gpr_weno_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, ndim == 1 ? 0L : O::fb_doubles(typename O::Grid(nX, ndim)));
}

int gpr_weno_launcher_n(double *wh, const double *ub, const int32_t *nX, int ndim,
                        double *scratch, int nvar, int order, void *stream) {
  if (!wh || !ub || bad_grid(nX, ndim, order) || (ndim == 2 && !scratch))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::weno(wh, ub, typename O::Grid(nX, ndim), scratch, S(stream)));
}

int gpr_predictor_n(double *qh, const double *wh, double dt, const double *dX, int ndim,
                    const int32_t *nX, int stiff, const gpr_par *par, const uint8_t *mask,
                    int32_t *status, int nvar, int order, void *stream) {
  if (!qh || !wh || !par || bad_grid(nX, ndim, order) || bad_dX(dX, ndim))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order, O::predictor(qh, wh, dt, nullptr, dX, typename O::Grid(nX, ndim),
                                       stiff, P, mask, status, S(stream)));
}

long gpr_fv_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::fb_doubles(typename O::Grid(nX, ndim)));
}

int gpr_fv_launcher_n(double *u, const double *qh, const int32_t *nX, double dt,
                      const double *dX, int ndim, int flux, const gpr_par *par,
                      const uint8_t *mask, double *scratch, int nvar, int order, void *stream) {
  if (!u || !qh || !par || !scratch || bad_grid(nX, ndim, order) || bad_dX(dX, ndim))
    return GPR_E_ARG;
  if (bad_flux(flux))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order, O::fv(u, qh, typename O::Grid(nX, ndim), dt, nullptr, dX, flux, P,
                                mask, scratch, S(stream)));
}

long gpr_ader_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::step_scratch(typename O::Grid(nX, ndim)));
}

int gpr_ader_stepper_n(double *u, const double *ub, const int32_t *nX, int ndim, double dt,
                       const double *dX, int stiff, int flux, const gpr_par *par,
                       const uint8_t *mask, double *scratch, int32_t *status, int nvar,
                       int order, void *stream) {
  if (!u || !ub || !par || !scratch || bad_grid(nX, ndim, order) || bad_dX(dX, ndim))
    return GPR_E_ARG;
  if (bad_flux(flux))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order, O::step(u, ub, typename O::Grid(nX, ndim), dt, nullptr, dX, stiff,
                                  flux, P, mask, scratch, status, S(stream)));
}

long gpr_iterate_scratch_doubles_n(const int32_t *nX, int ndim, int nvar, int order) {
  if (bad_grid(nX, ndim, order))
    return GPR_E_ARG;
  DISPATCH_N(nvar, order, O::iterate_scratch(typename O::Grid(nX, ndim)));
}

int gpr_iterate_n(double *u, const int32_t *nX, int ndim, const double *dX, const int32_t *bcs,
                  int flux, const gpr_par *par, const uint8_t *mask, double *clock, int nsteps,
                  double *scratch, int32_t *status, double contorted_tol, int nvar, int order,
                  void *stream) {
  if (!u || !par || !clock || !scratch || nsteps < 0 || bad_grid(nX, ndim, order) ||
      bad_dX(dX, ndim) || bad_bcs(bcs, ndim))
    return GPR_E_ARG;
  if (bad_flux(flux))
    return GPR_E_ARG;
  DevPar P = make_devpar(*par);
  DISPATCH_N(nvar, order, O::iterate(u, typename O::Grid(nX, ndim), dX, bcs, flux, P, mask,
                                     clock, nsteps, scratch, status, contorted_tol,
                                     S(stream)));
}

}  // extern "C"
