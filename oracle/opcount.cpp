// opcount.cpp - algorithmic FP64 operation counts of the GPR ADER-WENO step
// (test infrastructure).  Compiles the oracle's C restatement of the
// reference (gpr_oracle.c) with `double` replaced by a counting scalar, runs
// each stage of one step on a Taylor-Green state and prints operations per
// unit of work:
//   add/sub, mul, div, sqrt : 1 flop each
//   transcendental call (pow, cbrt, exp, log, atan, cos) : 1 each, tallied
//   separately; fabs, comparisons, min/max and sign flips : 0
// Operations between two material constants (parameter-only arithmetic) are
// not counted: the gpr_par fields stay plain doubles.
//
// Build and run: python oracle/opcount.py  (writes the table to stdout).
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gpr_gb300.h"

struct Tally {
  long long add, mul, div, sqrt_, trans;
  long long flops() const { return add + mul + div + sqrt_ + trans; }
};
static Tally T = {0, 0, 0, 0, 0};

struct cdouble {
  double v;
  cdouble() = default;
  cdouble(double x) : v(x) {}
  cdouble &operator+=(cdouble o) { T.add++; v += o.v; return *this; }
  cdouble &operator-=(cdouble o) { T.add++; v -= o.v; return *this; }
  cdouble &operator*=(cdouble o) { T.mul++; v *= o.v; return *this; }
  cdouble &operator/=(cdouble o) { T.div++; v /= o.v; return *this; }
  cdouble operator-() const { return cdouble(-v); }
  cdouble operator+() const { return *this; }
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
static inline cdouble pow(cdouble a, double b) { T.trans++; return cdouble(::pow(a.v, b)); }
static inline cdouble pow(double a, cdouble b) { T.trans++; return cdouble(::pow(a, b.v)); }
static inline cdouble hypot(cdouble a, cdouble b) {
  T.mul += 2; T.add++; T.sqrt_++;
  return cdouble(::hypot(a.v, b.v));
}
static inline cdouble fmax(cdouble a, cdouble b) { return cdouble(::fmax(a.v, b.v)); }
static inline cdouble fmax(cdouble a, double b) { return cdouble(::fmax(a.v, b)); }

#define double cdouble
#include "gpr_oracle.c"
#undef double

// ---------------------------------------------------------------------------

static gpr_par tgv_par() {
  gpr_par p;
  memset(&p, 0, sizeof p);
  p.EOS = 0;
  p.rho0 = 1.0;
  p.cv = 2.5;
  p.gamma = 1.4;
  p.b02 = 100.0;
  p.mu = 1e-2;
  p.n = 1.0;
  p.calpha2 = 1.0;
  p.kappa = 1e-2 * 1.4 * 2.5 / (2.0 / 3.0);
  return p;
}

int main(int argc, char **argv) {
  int n = argc > 1 ? atoi(argv[1]) : 64;
  double cfl = argc > 2 ? atof(argv[2]) : 0.4;
  or_configure(2, 1, 0, 6e-6, 50);
  gpr_par P = tgv_par();
  const int V = 17;
  int nX[2] = {n, n};
  long ncell = (long)n * n, ncb = (long)(n + 2) * (n + 2);
  // one period of the k-mode Taylor-Green vortex on an n x n tile whose
  // cells have the size of the 512 x 512 run on [0, 2 pi]^2
  int kmode = 512 / n;
  double L = 2 * M_PI / kmode, dx = L / n;
  cdouble dX[2] = {dx, dx};
  cdouble *u = (cdouble *)calloc(ncell * V, sizeof(cdouble));
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double x = kmode * (i + 0.5) * dx, y = kmode * (j + 0.5) * dx;
      double pr = 100 / 1.4 + (::cos(2 * x) + ::cos(2 * y)) / 4;
      double v0 = ::sin(x) * ::cos(y), v1 = -::cos(x) * ::sin(y);
      cdouble *q = u + ((long)i * n + j) * V;
      q[0] = 1.0;
      q[1] = pr / 0.4 + 0.5 * (v0 * v0 + v1 * v1);
      q[2] = v0;
      q[3] = v1;
      q[5] = 1.0;
      q[9] = 1.0;
      q[13] = 1.0;
    }
  // advance a few steps so the state is generic (untimed, uncounted)
  cdouble *ub = (cdouble *)calloc((long)(n + 4) * (n + 4) * V, sizeof(cdouble));
  int bcs[4] = {1, 1, 1, 1};
  uint8_t *mask = (uint8_t *)malloc(ncb);
  memset(mask, 1, ncb);
  int *status = (int *)calloc(ncb, sizeof(int));
  for (int s = 0; s < 8; s++) {
    cdouble dt = or_timestep(u, ncell, dX, 2, cfl, 0, 1e9, s, &P);
    or_boundaries(u, ub, nX, 2, bcs);
    or_ader_stepper(u, ub, nX, 2, dt, dX, 0, 0, &P, mask, status, 0);
    or_renorm_distortion(u, ncell, &P);
  }
  cdouble *wh = (cdouble *)calloc(ncb * 4 * V, sizeof(cdouble));
  cdouble *qh = (cdouble *)calloc(ncb * 8 * V, sizeof(cdouble));

  T = Tally{};
  cdouble dt = or_timestep(u, ncell, dX, 2, cfl, 0, 1e9, 8, &P);
  Tally cflT = T;

  or_boundaries(u, ub, nX, 2, bcs);
  T = Tally{};
  or_weno_launcher(wh, ub, nX, 2);
  Tally wenoT = T;

  T = Tally{};
  or_predictor(qh, wh, dt, dX, 2, nX, 0, &P, mask, status, 0);
  Tally predT = T;
  long iters = 0, conv = 0;
  for (long c = 0; c < ncb; c++)
    if (status[c] > 0) {
      iters += status[c];
      conv++;
    }

  // face quadrature points: one D_RUS + Bint + the two endpoint
  // extrapolations; count over every x face of the grid
  T = Tally{};
  long nq = 0;
  for (int i = 0; i < n + 1; i++)
    for (int j = 1; j < n + 1; j++) {
      long cb = (long)i * (n + 2) + j;
      for (int t = 0; t < 2; t++) {
        const cdouble *qh0 = qh + (cb * 2 + t) * 4 * V;
        const cdouble *qhx = qh + ((cb + n + 2) * 2 + t) * 4 * V;
        for (int s = 0; s < 2; s++) {
          cdouble q0[MAXV], q1[MAXV], f[MAXV], b[MAXV];
          for (int k = 0; k < V; k++) {
            cdouble s0 = 0, s1 = 0;
            for (int m = 0; m < 2; m++) {
              s0 += ENDVALS[1][m] * qh0[(m * 2 + s) * V + k];
              s1 += ENDVALS[0][m] * qhx[(m * 2 + s) * V + k];
            }
            q0[k] = s0;
            q1[k] = s1;
          }
          interface_D(GPR_FLUX_RUSANOV, q0, q1, 0, &P, f);
          or_Bint(q0, q1, 0, b);
          for (int k = 0; k < V; k++) {
            f[k] = (b[k] + f[k]) * 0.1;  // weight and accumulate (2 ops / var)
            b[k] = (b[k] - f[k]) * 0.1;
          }
          nq++;
        }
      }
    }
  Tally faceT = T;

  T = Tally{};
  for (long c = 0; c < ncell; c++) {
    int i = c / n, j = c % n;
    long cb = (long)(i + 1) * (n + 2) + (j + 1);
    cdouble acc[MAXV];
    for (int t = 0; t < 2; t++)
      centers_cell(acc, qh + (cb * 2 + t) * 4 * V, 2, dX[0], dX[1], dt * WGHTS[t], 1, &P);
  }
  Tally cellT = T;

  T = Tally{};
  cdouble maxe = 0;
  for (long c = 0; c < 64; c++)
    maxe = fmax(maxe, or_max_abs_eigs(u + c * V, 0, &P));
  Tally maeT = T;

  printf("# algorithmic FP64 operation counts, TGV tile %dx%d with the cell size of the\n"
         "# 512x512 run (one k=%d period), V=17, N=2, Rusanov, CFL %.2f, after 8 steps\n",
         n, n, kmode, cfl);
  printf("# unit                          flops   (add mul div sqrt trans)\n");
  auto row = [](const char *name, Tally t, double units) {
    printf("%-28s %10.1f   (%.1f %.1f %.1f %.1f %.1f)\n", name, t.flops() / units,
           t.add / units, t.mul / units, t.div / units, t.sqrt_ / units, t.trans / units);
  };
  row("cfl_per_cell", cflT, (double)ncell);
  row("max_abs_eigs_per_call", maeT, 64.0);
  row("weno_per_predictor_cell", wenoT, (double)ncb);
  row("predictor_per_cell_iter", predT, (double)iters);
  row("face_quadrature_point", faceT, (double)nq);
  row("cells_per_cell", cellT, (double)ncell);
  printf("mean_picard_iterations %.4f  (converged cells %ld of %ld)\n",
         (double)iters / conv, conv, ncb);
  double per_update = cflT.flops() / (double)ncell + wenoT.flops() / (double)ncell +
                      predT.flops() / (double)ncell + 8.0 * faceT.flops() / nq +
                      cellT.flops() / (double)ncell;
  printf("total_per_cell_update %.1f\n", per_update);
  return 0;
}
