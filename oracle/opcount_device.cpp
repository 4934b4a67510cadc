// opcount_device.cpp - FP64 operation counts of the device formulation of
// the GPR step (test infrastructure).
//
// The device physics header (phd_gb300/csrc/gpr_device.cuh) is compiled for
// the host with `double` replaced by a counting scalar, and the per-unit
// work of each kernel is assembled from the same device functions the
// kernels call, plus the kernels' own linear algebra counted from their
// source (listed beside each figure).  Convention: add/sub, mul, div, sqrt
// = 1 flop, each transcendental call (cbrt, pow, exp, log, atan, cos) = 1,
// comparisons/fabs/fmax/copysign = 0.  States come from the oracle (a TGV
// tile with the 512^2 cell size, advanced 8 steps).
//
//   python oracle/opcount.py --device
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>  // before the counting macro: CUDA's own headers keep double

#include "../include/gpr_gb300.h"

struct Tally {
  long long add, mul, div, sqrt_, trans;
  long long flops() const { return add + mul + div + sqrt_ + trans; }
};
static Tally T = {0, 0, 0, 0, 0};

struct cdouble {
  double v;
  cdouble() = default;
  constexpr cdouble(double x) : v(x) {}
  cdouble &operator+=(cdouble o) { T.add++; v += o.v; return *this; }
  cdouble &operator-=(cdouble o) { T.add++; v -= o.v; return *this; }
  cdouble &operator*=(cdouble o) { T.mul++; v *= o.v; return *this; }
  cdouble &operator/=(cdouble o) { T.div++; v /= o.v; return *this; }
  cdouble operator-() const { return cdouble(-v); }
  explicit operator float() const { return (float)v; }  // FP32 work is not counted
};
static inline cdouble operator+(cdouble a, cdouble b) { T.add++; return cdouble(a.v + b.v); }
static inline cdouble operator-(cdouble a, cdouble b) { T.add++; return cdouble(a.v - b.v); }
static inline cdouble operator*(cdouble a, cdouble b) { T.mul++; return cdouble(a.v * b.v); }
static inline cdouble operator/(cdouble a, cdouble b) { T.div++; return cdouble(a.v / b.v); }
static inline bool operator<(cdouble a, cdouble b) { return a.v < b.v; }
static inline bool operator>(cdouble a, cdouble b) { return a.v > b.v; }
static inline bool operator<=(cdouble a, cdouble b) { return a.v <= b.v; }
static inline bool operator>=(cdouble a, cdouble b) { return a.v >= b.v; }
static inline bool operator==(cdouble a, cdouble b) { return a.v == b.v; }
static inline bool operator!=(cdouble a, cdouble b) { return a.v != b.v; }
static inline cdouble fabs(cdouble a) { return cdouble(::fabs(a.v)); }
static inline cdouble sqrt(cdouble a) { T.sqrt_++; return cdouble(::sqrt(a.v)); }
static inline cdouble cbrt(cdouble a) { T.trans++; return cdouble(::cbrt(a.v)); }
static inline cdouble exp(cdouble a) { T.trans++; return cdouble(::exp(a.v)); }
static inline cdouble log(cdouble a) { T.trans++; return cdouble(::log(a.v)); }
static inline cdouble atan(cdouble a) { T.trans++; return cdouble(::atan(a.v)); }
static inline cdouble cos(cdouble a) { T.trans++; return cdouble(::cos(a.v)); }
static inline cdouble pow(cdouble a, cdouble b) { T.trans++; return cdouble(::pow(a.v, b.v)); }
static inline cdouble hypot(cdouble a, cdouble b) {
  T.mul += 2; T.add++; T.sqrt_++;
  return cdouble(::hypot(a.v, b.v));
}
static inline cdouble fma(cdouble a, cdouble b, cdouble c) {
  T.mul++; T.add++;
  return cdouble(::fma(a.v, b.v, c.v));
}
static inline cdouble fmax(cdouble a, cdouble b) { return cdouble(::fmax(a.v, b.v)); }
static inline cdouble fmin(cdouble a, cdouble b) { return cdouble(::fmin(a.v, b.v)); }
static inline cdouble copysign(cdouble a, cdouble b) { return cdouble(::copysign(a.v, b.v)); }

// the oracle (plain doubles) provides the states
extern "C" {
int or_configure(int n, int thermal, int lset, double dg_tol, int dg_it);
double or_timestep(const double *u, long ncell, const double *dX, int ndim, double CFL,
                   double t, double tf, int count, const gpr_par *P);
int or_boundaries(const double *u, double *ub, const int *nX, int ndim, const int *bcs);
int or_ader_stepper(double *u, const double *ub, const int *nX, int ndim, double dt,
                    const double *dX, int stiff, int FLUX, const gpr_par *P,
                    const uint8_t *mask, int *status, int newton_fallback);
void or_renorm_distortion(double *u, long ncell, const gpr_par *P);
int or_weno_launcher(double *wh, const double *ub, const int *nX, int ndim);
int or_predictor(double *qh, const double *wh, double dt, const double *dX, int ndim,
                 const int *nX, int stiff, const gpr_par *P, const uint8_t *mask, int *status,
                 int newton_fallback);
}

#define __host__
#define __device__
#define __forceinline__ inline
#define cuda_runtime_h_stub
#define double cdouble
#include "../phd_gb300/csrc/gpr_device.cuh"
#undef double

using namespace gpr;
constexpr int V = 17;
using Pr = Prim<true>;

static Tally run_prim(const cdouble *q, const DevPar &P, Pr &s) {
  T = Tally{};
  prim<true>(q, P, s);
  return T;
}

int main(int argc, char **argv) {
  int n = argc > 1 ? atoi(argv[1]) : 64;
  double cfl = 0.4;
  or_configure(2, 1, 0, 6e-6, 50);
  gpr_par gp;
  memset(&gp, 0, sizeof gp);
  gp.EOS = 0;
  gp.rho0 = 1.0;
  gp.cv = 2.5;
  gp.gamma = 1.4;
  gp.b02 = 100.0;
  gp.mu = 1e-2;
  gp.n = 1.0;
  gp.calpha2 = 1.0;
  gp.kappa = 1e-2 * 1.4 * 2.5 / (2.0 / 3.0);
  DevPar P = make_devpar(gp);
  int kmode = 512 / n;
  double L = 2 * M_PI / kmode, dx = L / n;
  double dX[2] = {dx, dx};
  long ncell = (long)n * n, ncb = (long)(n + 2) * (n + 2);
  double *u = (double *)calloc(ncell * V, sizeof(double));
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double x = kmode * (i + 0.5) * dx, y = kmode * (j + 0.5) * dx;
      double pr = 100 / 1.4 + (::cos(2 * x) + ::cos(2 * y)) / 4;
      double v0 = ::sin(x) * ::cos(y), v1 = -::cos(x) * ::sin(y);
      double *q = u + ((long)i * n + j) * V;
      q[0] = 1.0;
      q[1] = pr / 0.4 + 0.5 * (v0 * v0 + v1 * v1);
      q[2] = v0;
      q[3] = v1;
      q[5] = q[9] = q[13] = 1.0;
    }
  int nX[2] = {n, n}, bcs[4] = {1, 1, 1, 1};
  double *ub = (double *)calloc((long)(n + 4) * (n + 4) * V, sizeof(double));
  uint8_t *mask = (uint8_t *)malloc(ncb);
  memset(mask, 1, ncb);
  int *status = (int *)calloc(ncb, sizeof(int));
  for (int s = 0; s < 8; s++) {
    double dt = or_timestep(u, ncell, dX, 2, cfl, 0, 1e9, s, &gp);
    or_boundaries(u, ub, nX, 2, bcs);
    or_ader_stepper(u, ub, nX, 2, dt, dX, 0, 0, &gp, mask, status, 0);
    or_renorm_distortion(u, ncell, &gp);
  }
  double dt = or_timestep(u, ncell, dX, 2, cfl, 0, 1e9, 8, &gp);
  or_boundaries(u, ub, nX, 2, bcs);
  double *wh = (double *)calloc(ncb * 4 * V, sizeof(double));
  double *qh = (double *)calloc(ncb * 8 * V, sizeof(double));
  or_weno_launcher(wh, ub, nX, 2);
  or_predictor(qh, wh, dt, dX, 2, nX, 0, &gp, mask, status, 0);
  long iters = 0;
  for (long c = 0; c < ncb; c++)
    iters += status[c] > 0 ? status[c] : 0;

  // per-state functions, averaged over the space-time nodes of qh
  Tally tp{}, tf{}, ts{}, tb{}, tm{};
  long nst = 0;
  for (long k = 0; k < ncb * 8; k += 7) {
    cdouble q[V];
    for (int v = 0; v < V; v++)
      q[v] = qh[k * V + v];
    Pr s;
    Tally a = run_prim(q, P, s);
    tp.add += a.add; tp.mul += a.mul; tp.div += a.div; tp.sqrt_ += a.sqrt_; tp.trans += a.trans;
    cdouble F[V];
    for (int v = 0; v < V; v++) F[v] = 0.0;
    T = Tally{};
    flux_add<true, V>(q, s, 0, P, F);
    a = T; tf.add += a.add; tf.mul += a.mul; tf.div += a.div; tf.sqrt_ += a.sqrt_; tf.trans += a.trans;
    T = Tally{};
    source<true, V>(q, s, P, F);
    a = T; ts.add += a.add; ts.mul += a.mul; ts.div += a.div; ts.sqrt_ += a.sqrt_; ts.trans += a.trans;
    T = Tally{};
    bdot<V, 0>(s.v, q, 0, F);
    a = T; tb.add += a.add; tb.mul += a.mul; tb.div += a.div;
    T = Tally{};
    cdouble m = max_abs_eigs<true>(q, s, 0, P);
    (void)m;
    a = T; tm.add += a.add; tm.mul += a.mul; tm.div += a.div; tm.sqrt_ += a.sqrt_; tm.trans += a.trans;
    nst++;
  }
  auto per = [&](Tally t) { return (double)t.flops() / nst; };
  double Fp = per(tp), Ff = per(tf), Fs = per(ts), Fb = per(tb), Fm = per(tm);
  // Bint path node: rho, 1/rho, 3 v (3 fma + 3 mul), bdot, accumulate over
  // the 9 rows where B x can be nonzero (9 fma)
  double Fbint_node = 1 + 1 + 3 * 2 + 3 + Fb + 9 * 2;
  // face quadrature point (k_faces2d): 2 extrapolations (17 x 3 each), 2 prim,
  // 2 max_abs_eigs, dissipation 17 x (sub, mul), 2 fluxes, dq (17 sub),
  // 2 Bint nodes, weighting (kk b, kk f: 34 mul), reduce-scatter over the 4
  // lanes (20 + 10 add per lane) and the 5 kept pairs' sums and differences
  double Fface = 2 * 17 * 3 + 2 * Fp + 2 * Fm + 17 * 2 + 2 * Ff + 17 + 2 * Fbint_node + 34 +
                 30 + 10;
  // predictor node and Picard iteration (dg_rhs_node + dg_solve_node +
  // stopping rule): prim, source (node weight in its factors), 2 x
  // (derivative of the 6 entries bdot reads 6 x 3, bdot, 9 sub), 2 fluxes,
  // 2 x DG_DER term on the 11 entries of the flux's support (2 fma each),
  // r dt + Ww 17 x 2, DG_MAT^-1 17 x 3, |qn - q| > tol (1 + |q|) 17 x 3
  double Fpred_node = Fp + Fs + 2 * (6 * 3 + Fb + 9) + 2 * Ff + 2 * 11 * 4 + 17 * 2 + 17 * 3 +
                      17 * 3;
  // volume node (k_cells): prim, source (weight in its factors), 2 x
  // (derivative 6 x 3, bdot, 9 sub), reduce-scatter over the 8 lanes
  // (12 + 6 + 3 add per lane); cell adds 17 x 5
  double Fcell_node = Fp + Fs + 2 * (6 * 3 + Fb + 9) + 21;
  double Fcell = 8 * Fcell_node + 17 * 5;
  // WENO point (weno_point): 4 coefficients 4 x 3, 2 indicators 2 x 9 + eps,
  // 2 x 3 squarings, tL + tR and its reciprocal, 2 blends (2 mul, add, mul)
  double Fweno = 12 + 2 * 10 + 6 + 2 + 8;
  double Fweno_cell = 2 * Fweno * V * 2;  // x sweep (per ub column cell) + y sweep, ~2 per node
  double Fcfl = Fp + 2 * Fm + 3;
  printf("# FP64 operation counts of the device formulation (gpr_device.cuh compiled\n");
  printf("# for the host with a counting scalar), TGV tile %dx%d with the 512^2 cell size\n", n, n);
  printf("prim                       %8.1f\n", Fp);
  printf("flux_add                   %8.1f\n", Ff);
  printf("source                     %8.1f\n", Fs);
  printf("bdot                       %8.1f\n", Fb);
  printf("max_abs_eigs               %8.1f\n", Fm);
  printf("face_quadrature_point      %8.1f\n", Fface);
  printf("predictor_node_iteration   %8.1f\n", Fpred_node);
  printf("predictor_cell_iteration   %8.1f\n", 8 * Fpred_node);
  printf("cells_per_cell             %8.1f\n", Fcell);
  printf("weno_point                 %8.1f\n", Fweno);
  printf("cfl_per_cell               %8.1f\n", Fcfl);
  printf("mean_picard_iterations     %8.3f\n", (double)iters / ncb);
  // 1D kernels (the batched form and 1D grids), same per-state costs:
  // face point per (face, time node) of k_faces1d: as the 2D point with a
  // 2-lane reduce-scatter of the 17 (b, f) pairs (18 adds) and the 9 kept
  // pairs' sums and differences (18); predictor node: one derivative, one
  // flux and one DG_DER term; volume node: one derivative, a 4-lane
  // reduce-scatter (10 + 5 adds), cell adds 17 x 3; WENO: 17 points per
  // predictor cell; CFL: one wave speed.
  double Fface1 = 2 * 17 * 3 + 2 * Fp + 2 * Fm + 17 * 2 + 2 * Ff + 17 + 2 * Fbint_node + 34 +
                  18 + 18;
  double Fpred_node1 = Fp + Fs + (6 * 3 + Fb + 9) + Ff + 11 * 4 + 17 * 2 + 17 * 3 + 17 * 3;
  double Fcell1 = 4 * (Fp + Fs + (6 * 3 + Fb + 9) + 15) + 17 * 3;
  printf("face_point_1d              %8.1f\n", Fface1);
  printf("predictor_cell_iteration_1d %7.1f\n", 4 * Fpred_node1);
  printf("cells_per_cell_1d          %8.1f\n", Fcell1);
  printf("weno_per_cell_1d           %8.1f\n", Fweno * V);
  printf("cfl_per_cell_1d            %8.1f\n", Fp + Fm + 2);
  return 0;
}
