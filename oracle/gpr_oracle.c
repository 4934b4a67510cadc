/*
 * gpr_oracle.c - CPU ORACLE (test infrastructure, not product code).
 *
 * A plain-C restatement of the reference GPR ADER-WENO time step
 * (haranjackson/phd, code/cpp/src), used by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * It follows the reference's algorithms and operation order function by
 * function (each function cites the reference file:line it restates); it is
 * never linked into, or called by, the CUDA library.
 *
 * Parity of this oracle against the compiled reference is pinned by the
 * golden fixtures under tests/golden/ (generated from the reference's own
 * C++ by tests/golden/make_golden.py).
 *
 * Runtime configuration: N (Gauss nodes / basis functions), THERMAL and LSET
 * select V = 14 + 3*THERMAL + LSET as the reference's options.h:4-35 does at
 * compile time.  VISCOUS is always on and MULTI always off.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gpr_gb300.h"

#define MAXN 4
#define MAXV 18

/* WENO and DG constants of options.h:24-31. */
static const double LAMS = 1.0;
static const double LAMC = 1e5;
static const double WENO_EPS = 1e-14;
static double DG_TOL = 6e-6;
static int DG_IT = 50;
/* stiff-source Newton iteration: tolerance on the update and iteration cap */
static double STIFF_TOL = 1e-11;
static int STIFF_IT = 60;

static int N = 2, V = 17, THERMAL = 1, LSET = 0;
static int FN2 = 0, CN2 = 1;

static double NODES[MAXN], WGHTS[MAXN];
static double ENDVALS[2][MAXN];
static double DERVALS[MAXN][MAXN];
static double mLinv[MAXN][MAXN], mRinv[MAXN][MAXN], mCLinv[MAXN][MAXN],
    mCRinv[MAXN][MAXN];
static double SIG[MAXN][MAXN];
static double DG_DER[MAXN][MAXN], DG_MAT[MAXN][MAXN], DG_MATinv[MAXN][MAXN];

/* ------------------------------------------------------------------------ */
/* Polynomials in the monomial basis (restates scipy/poly.cpp:6-66).       */

typedef struct {
  int n;
  double c[2 * MAXN + 2];
} poly;

static double poly_eval(const poly *p, double x) {
  double r = 0.0;
  for (int i = p->n - 1; i >= 0; i--)
    r = r * x + p->c[i];
  return r;
}

static poly poly_diff(const poly *p) {
  poly r;
  r.n = p->n > 1 ? p->n - 1 : 1;
  r.c[0] = 0.0;
  for (int i = 0; i < p->n - 1; i++)
    r.c[i] = p->c[i + 1] * (i + 1);
  return r;
}

static poly poly_int(const poly *p) {
  poly r;
  r.n = p->n + 1;
  r.c[0] = 0.0;
  for (int i = 1; i < r.n; i++)
    r.c[i] = p->c[i - 1] / i;
  return r;
}

static poly poly_mul(const poly *a, const poly *b) {
  poly r;
  r.n = a->n + b->n - 1;
  for (int i = 0; i < r.n; i++)
    r.c[i] = 0.0;
  for (int i = 0; i < a->n; i++)
    for (int j = 0; j < b->n; j++)
      r.c[i + j] += a->c[i] * b->c[j];
  return r;
}

static poly basis[MAXN];

/* Gauss-Legendre nodes/weights on [0,1] (restates poly/basis.cpp:7-20 and
 * scipy/legendre.cpp: leggauss): Newton iteration on P_N from the
 * Chebyshev-like initial guesses, weights 2/((1-x^2) P_N'(x)^2). */
static void gauss_legendre(int n, double *x, double *w) {
  for (int i = 0; i < n; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = 0.0;
      for (int k = 1; k <= n; k++) {
        double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      pp = n * (z * p0 - p1) / (z * z - 1.0);
      double dz = p0 / pp;
      z -= dz;
      if (fabs(dz) < 1e-16)
        break;
    }
    /* ascending order on [-1,1] */
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
  /* symmetrise as the reference does (legendre.cpp: w,x symmetrised) */
  for (int i = 0; i < n / 2; i++) {
    double xs = 0.5 * (x[n - 1 - i] - x[i]);
    x[i] = -xs;
    x[n - 1 - i] = xs;
    double ws = 0.5 * (w[i] + w[n - 1 - i]);
    w[i] = ws;
    w[n - 1 - i] = ws;
  }
  if (n % 2)
    x[n / 2] = 0.0;
}

static int invert(int n, double a_[MAXN][MAXN], double out[MAXN][MAXN]) {
  double a[MAXN][2 * MAXN];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < 2 * n; j++)
      a[i][j] = j < n ? a_[i][j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(a[r][c]) > fabs(a[p][c]))
        p = r;
    if (a[p][c] == 0.0)
      return -1;
    for (int j = 0; j < 2 * n; j++) {
      double t = a[c][j];
      a[c][j] = a[p][j];
      a[p][j] = t;
    }
    double inv = 1.0 / a[c][c];
    for (int j = 0; j < 2 * n; j++)
      a[c][j] *= inv;
    for (int r = 0; r < n; r++)
      if (r != c) {
        double f = a[r][c];
        for (int j = 0; j < 2 * n; j++)
          a[r][j] -= f * a[c][j];
      }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      out[i][j] = a[i][j + n];
  return 0;
}

/* Builds every constant of etc/globals.cpp:16-50. */
int or_configure(int n, int thermal, int lset, double dg_tol, int dg_it) {
  if (n < 2 || n > MAXN || lset < 0 || lset > 1)
    return -1;
  N = n;
  THERMAL = thermal ? 1 : 0;
  LSET = lset;
  V = 14 + 3 * THERMAL + LSET;
  FN2 = (int)floor((N - 1) / 2.0);
  CN2 = (int)ceil((N - 1) / 2.0);
  DG_TOL = dg_tol > 0 ? dg_tol : 6e-6;
  DG_IT = dg_it > 0 ? dg_it : 50;

  double x[MAXN], w[MAXN];
  gauss_legendre(N, x, w);
  for (int i = 0; i < N; i++) {
    NODES[i] = (x[i] + 1.0) / 2.0;
    WGHTS[i] = w[i] / 2.0;
  }
  /* Lagrange basis on the scaled nodes (poly/basis.cpp:22-53) */
  for (int i = 0; i < N; i++) {
    poly p;
    p.n = 1;
    p.c[0] = 1.0;
    for (int j = 0; j < N; j++) {
      if (j == i)
        continue;
      poly f;
      f.n = 2;
      f.c[0] = -NODES[j];
      f.c[1] = 1.0;
      p = poly_mul(&p, &f);
      for (int k = 0; k < p.n; k++)
        p.c[k] /= (NODES[i] - NODES[j]);
    }
    basis[i] = p;
  }
  for (int j = 0; j < N; j++) {
    ENDVALS[0][j] = poly_eval(&basis[j], 0.0);
    ENDVALS[1][j] = poly_eval(&basis[j], 1.0);
  }
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      poly d = poly_diff(&basis[j]);
      DERVALS[i][j] = poly_eval(&d, NODES[i]);
    }
  /* WENO stencil matrices (weno/weno_matrices.cpp:9-28) */
  double mL[MAXN][MAXN], mR[MAXN][MAXN], mCL[MAXN][MAXN], mCR[MAXN][MAXN];
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      poly P = poly_int(&basis[j]);
      mL[i][j] = poly_eval(&P, i - N + 2) - poly_eval(&P, i - N + 1);
      mR[i][j] = poly_eval(&P, i + 1) - poly_eval(&P, i);
      mCL[i][j] = poly_eval(&P, i - CN2 + 1) - poly_eval(&P, i - CN2);
      mCR[i][j] = poly_eval(&P, i - FN2 + 1) - poly_eval(&P, i - FN2);
    }
  invert(N, mL, mLinv);
  invert(N, mR, mRinv);
  invert(N, mCL, mCLinv);
  invert(N, mCR, mCRinv);
  /* oscillation indicator (weno_matrices.cpp:30-42) */
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double s = 0.0;
      poly di = basis[i], dj = basis[j];
      for (int a = 1; a < N; a++) {
        di = poly_diff(&di);
        dj = poly_diff(&dj);
        poly p = poly_mul(&di, &dj);
        poly P = poly_int(&p);
        s += poly_eval(&P, 1.0) - poly_eval(&P, 0.0);
      }
      SIG[i][j] = s;
    }
  /* DG matrices (dg/dg_matrices.cpp:29-53, etc/globals.cpp:42-44) */
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double e = poly_eval(&basis[i], 1.0) * poly_eval(&basis[j], 1.0);
      double dd;
      if (i == j) {
        double b1 = poly_eval(&basis[i], 1.0), b0 = poly_eval(&basis[i], 0.0);
        dd = (b1 * b1 - b0 * b0) / 2;
      } else {
        poly d = poly_diff(&basis[j]);
        dd = WGHTS[i] * poly_eval(&d, NODES[i]);
      }
      DG_DER[i][j] = dd;
      (void)e;
    }
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++)
      DG_MAT[i][j] = poly_eval(&basis[i], 1.0) * poly_eval(&basis[j], 1.0) -
                     DG_DER[j][i];
  invert(N, DG_MAT, DG_MATinv);
  return V;
}

int or_nvar(void) { return V; }

void or_set_stiff(double tol, int maxit) {
  STIFF_TOL = tol;
  STIFF_IT = maxit;
}

/* Exposes the constants for the tests: NODES, WGHTS, ENDVALS, DERVALS,
 * DG_DER, DG_MAT, SIG, mLinv, mRinv (each padded to MAXN x MAXN). */
void or_constants(double *out) {
  int k = 0;
  for (int i = 0; i < MAXN; i++)
    out[k++] = i < N ? NODES[i] : 0.0;
  for (int i = 0; i < MAXN; i++)
    out[k++] = i < N ? WGHTS[i] : 0.0;
  for (int e = 0; e < 2; e++)
    for (int i = 0; i < MAXN; i++)
      out[k++] = i < N ? ENDVALS[e][i] : 0.0;
  for (int i = 0; i < MAXN; i++)
    for (int j = 0; j < MAXN; j++)
      out[k++] = DERVALS[i][j];
  for (int i = 0; i < MAXN; i++)
    for (int j = 0; j < MAXN; j++)
      out[k++] = DG_DER[i][j];
  for (int i = 0; i < MAXN; i++)
    for (int j = 0; j < MAXN; j++)
      out[k++] = DG_MAT[i][j];
  for (int i = 0; i < MAXN; i++)
    for (int j = 0; j < MAXN; j++)
      out[k++] = SIG[i][j];
}

/* ------------------------------------------------------------------------ */
/* EOS (restates system/energy/mg.cpp:6-303).                              */

static double Gamma_MG(double r, const gpr_par *P) {
  switch (P->EOS) {
  case 0:
    return P->gamma - 1;
  case 1:
    return P->Gamma0 * P->rho0 / r;
  case 4:
    return P->gamma;
  default:
    return P->Gamma0;
  }
}

static double p_ref(double r, const gpr_par *P) {
  switch (P->EOS) {
  case 0:
    return -P->pINF;
  case 1: {
    if (r > P->rho0) {
      double tmp = 1 / P->rho0 - P->s * (1 / P->rho0 - 1 / r);
      return P->c02 * (1 / P->rho0 - 1 / r) / (tmp * tmp);
    }
    return P->c02 * (r - P->rho0);
  }
  case 4: {
    double tmp = pow(r / P->rho0, P->alpha);
    return P->c02 * r / P->alpha * (tmp - 1) * tmp;
  }
  case 2: {
    double v_ = P->rho0 / r;
    return P->A * exp(-P->R1 * v_) + P->B * exp(-P->R2 * v_);
  }
  default: {
    double v_ = P->rho0 / r;
    return P->A * pow(v_, -P->R1) - P->B * pow(v_, -P->R2);
  }
  }
}

static double e_ref(double r, const gpr_par *P) {
  switch (P->EOS) {
  case 0:
    return P->pINF / r;
  case 1:
    if (r > P->rho0)
      return 0.5 * p_ref(r, P) * (1 / P->rho0 - 1 / r);
    return 0.0;
  case 4: {
    double tmp = pow(r / P->rho0, P->alpha);
    return P->c02 / (2 * P->alpha * P->alpha) * (tmp - 1) * (tmp - 1);
  }
  case 2: {
    double v_ = P->rho0 / r;
    return P->A / (P->rho0 * P->R1) * exp(-P->R1 * v_) +
           P->B / (P->rho0 * P->R2) * exp(-P->R2 * v_);
  }
  default: {
    double v_ = P->rho0 / r;
    return -P->A / (P->rho0 * (1 - P->R1)) * (pow(v_, 1 - P->R1) - 1) +
           P->B / (P->rho0 * (1 - P->R2)) * (pow(v_, 1 - P->R2) - 1);
  }
  }
}

static double pressure_mg(double r, double e, const gpr_par *P) {
  return (e - e_ref(r, P)) * r * Gamma_MG(r, P) + p_ref(r, P);
}

static double phi_mg(double r, const gpr_par *P) {
  switch (P->EOS) {
  case 0:
    return pow(r / P->rho0, P->gamma - 1);
  case 1:
    return exp(P->Gamma0 * (1 - P->rho0 / r));
  case 4:
    return pow(r / P->rho0, P->gamma);
  default:
    return pow(r / P->rho0, P->Gamma0);
  }
}

static double temperature_mg(double r, double p, const gpr_par *P) {
  return phi_mg(r, P) * P->Tref +
         (p - p_ref(r, P)) / (r * Gamma_MG(r, P) * P->cv);
}

static double dGamma_MG(double r, const gpr_par *P) {
  if (P->EOS == 1)
    return -P->Gamma0 * P->rho0 / (r * r);
  return 0.0;
}

static double dp_ref(double r, const gpr_par *P) {
  switch (P->EOS) {
  case 0:
    return 0.0;
  case 1: {
    if (r > P->rho0) {
      double tmp = P->s * (r - P->rho0) - r;
      return P->c02 * P->rho0 * P->rho0 * (P->s * (P->rho0 - r) - r) /
             (tmp * tmp * tmp);
    }
    return P->c02;
  }
  case 4: {
    double tmp = pow(r / P->rho0, P->alpha);
    return P->c02 / P->alpha * tmp * ((1 + P->alpha) * (tmp - 1) + P->alpha * tmp);
  }
  case 2: {
    double v_ = P->rho0 / r;
    return v_ / r * (P->A * P->R1 * exp(-P->R1 * v_) + P->B * P->R2 * exp(-P->R2 * v_));
  }
  default: {
    double v_ = P->rho0 / r;
    return P->A * P->R1 / r * pow(v_, -P->R1) - P->B * P->R2 / r * pow(v_, -P->R2);
  }
  }
}

static double de_ref(double r, const gpr_par *P) {
  if (P->EOS == 1) {
    if (r > P->rho0) {
      double tmp = P->s * (r - P->rho0) - r;
      return -(r - P->rho0) * P->rho0 * P->c02 / (tmp * tmp * tmp);
    }
    return 0.0;
  }
  return p_ref(r, P) / (r * r);
}

static double dedrho(double r, double p, const gpr_par *P) {
  double G = Gamma_MG(r, P), dG = dGamma_MG(r, P), pr = p_ref(r, P),
         dpr = dp_ref(r, P), der = de_ref(r, P);
  return der - (dpr * r * G + (G + r * dG) * (p - pr)) / ((r * G) * (r * G));
}

static double dedp(double r, const gpr_par *P) {
  return 1 / (r * Gamma_MG(r, P));
}

static double dTdrho(double r, double p, const gpr_par *P) {
  double G = Gamma_MG(r, P), dG = dGamma_MG(r, P), pr = p_ref(r, P),
         dpr = dp_ref(r, P);
  return -(dpr * r * G + (G + r * dG) * (p - pr)) / ((r * G) * (r * G)) / P->cv;
}

static double dTdp(double r, const gpr_par *P) { return dedp(r, P) / P->cv; }

/* Shear wave quantities (system/waves/shear.cpp:6-41). */
static double c_s2(double r, const gpr_par *P) {
  return P->b02 * pow(r / P->rho0, P->beta);
}
static double dc_s2drho(double r, const gpr_par *P) {
  return P->beta / r * c_s2(r, P);
}
static double C_0(double r, const gpr_par *P) {
  return (1 - P->beta / Gamma_MG(r, P)) * c_s2(r, P);
}
static double dC_0drho(double r, const gpr_par *P) {
  double cs2 = c_s2(r, P), dcs2 = dc_s2drho(r, P), G = Gamma_MG(r, P),
         dG = dGamma_MG(r, P);
  return (1 - P->beta / G) * dcs2 + P->beta / (G * G) * dG * cs2;
}

/* ------------------------------------------------------------------------ */
/* Matrix functions (system/functions/matrices.cpp:8-27).                  */

/* A is row-major 3x3 at Q+5. */
static void AdevG(const double *A, double *out) {
  double G[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      G[3 * i + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  double x = (G[0] + G[4] + G[8]) / 3;
  G[0] -= x;
  G[4] -= x;
  G[8] -= x;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      out[3 * i + j] = A[3 * i] * G[j] + A[3 * i + 1] * G[3 + j] +
                       A[3 * i + 2] * G[6 + j];
}

static double devGsq(const double *A) {
  double G00 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  double G11 = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  double G22 = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  double G01 = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  double G02 = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  double G12 = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  double t = (G00 + G11 + G22) / 3;
  return ((G00 - t) * (G00 - t) + (G11 - t) * (G11 - t) + (G22 - t) * (G22 - t) +
          2 * (G01 * G01 + G02 * G02 + G12 * G12));
}

static double det3(const double *A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

/* ------------------------------------------------------------------------ */
/* State variables (system/energy/eos.cpp, variables/state.cpp).           */

static double E_2A(double r, const double *A, const gpr_par *P) {
  return C_0(r, P) / 4 * devGsq(A);
}

static double internal_energy(const double *Q, const gpr_par *P) {
  double r = Q[0];
  double E = Q[1] / r;
  double v0 = Q[2] / r, v1 = Q[3] / r, v2 = Q[4] / r;
  double E1 = E - (v0 * v0 + v1 * v1 + v2 * v2) / 2;
  E1 -= E_2A(r, Q + 5, P);
  if (THERMAL) {
    double J0 = Q[14] / r, J1 = Q[15] / r, J2 = Q[16] / r;
    E1 -= P->calpha2 * (J0 * J0 + J1 * J1 + J2 * J2) / 2;
  }
  return E1;
}

double or_pressure(const double *Q, const gpr_par *P) {
  return pressure_mg(Q[0], internal_energy(Q, P), P);
}

double or_temperature(const double *Q, const gpr_par *P) {
  return temperature_mg(Q[0], or_pressure(Q, P), P);
}

/* dEdA_s = cs2 * AdevG(A) (energy/derivatives.cpp:73-79) */
static void dEdA_s(const double *Q, const gpr_par *P, double *out) {
  double cs2 = c_s2(Q[0], P);
  AdevG(Q + 5, out);
  for (int i = 0; i < 9; i++)
    out[i] *= cs2;
}

/* sigma column d: -rho E_A^T A(:,d)   (variables/state.cpp:23-29) */
static void sigma_d(const double *Q, const gpr_par *P, int d, double *out) {
  double EA[9];
  dEdA_s(Q, P, EA);
  const double *A = Q + 5;
  double r = Q[0];
  for (int i = 0; i < 3; i++)
    out[i] = -r * (EA[i] * A[d] + EA[3 + i] * A[3 + d] + EA[6 + i] * A[6 + d]);
}

static void sigma_full(const double *Q, const gpr_par *P, double *out) {
  for (int d = 0; d < 3; d++) {
    double c[3];
    sigma_d(Q, P, d, c);
    for (int i = 0; i < 3; i++)
      out[3 * i + d] = c[i];
  }
}

static void dsigmadrho(const double *Q, const gpr_par *P, int d, double *out) {
  double r = Q[0];
  double cs2 = c_s2(r, P), dcs2 = dc_s2drho(r, P);
  sigma_d(Q, P, d, out);
  double f = 1 / r + dcs2 / cs2;
  for (int i = 0; i < 3; i++)
    out[i] *= f;
}

/* dsigmadA (variables/state.cpp:43-56): -rho cs2 ret^T */
static void dsigmadA(const double *Q, const gpr_par *P, int d, double *out) {
  double r = Q[0];
  double cs2 = c_s2(r, P);
  const double *A = Q + 5;
  double G[9], ret[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      G[3 * i + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  AdevG(A, ret);
  for (int i = 0; i < 3; i++)
    ret[3 * i + d] *= 2.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      ret[3 * i + j] += 1.0 / 3.0 * A[3 * i + d] * G[3 * d + j];
  for (int i = 0; i < 9; i++)
    ret[i] += G[4 * d] * A[i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      out[3 * i + j] = -r * cs2 * ret[3 * j + i];
}

static double sigma_norm(const double *s) {
  double a = s[0] - s[4], b = s[4] - s[8], c = s[8] - s[0];
  double t1 = a * a + b * b + c * c;
  double t2 = s[1] * s[1] + s[5] * s[5] + s[6] * s[6];
  return sqrt(0.5 * t1 + 3 * t2);
}

/* theta1inv (variables/sources.cpp:13-81) */
static double theta1inv(const double *Q, const gpr_par *P) {
  double r = Q[0];
  double A53 = pow(det3(Q + 5), 5.0 / 3.0);
  double cs2 = c_s2(r, P);
  double n = P->n;
  int SOLID = P->flags & GPR_SOLID, PL = P->flags & GPR_POWER_LAW,
      BING = P->flags & GPR_BINGHAM;
  if (SOLID) {
    if (PL) {
      double s[9];
      sigma_full(Q, P, s);
      double sn = sigma_norm(s);
      sn = sn < 1e8 ? sn : 1e8;
      return 3 * A53 / (cs2 * P->tau0) * pow(sn / P->sigmaY, n);
    }
    return 0.0;
  } else if (BING) {
    double s[9];
    sigma_full(Q, P, s);
    double nn = 0;
    for (int i = 0; i < 9; i++)
      nn += s[i] * s[i];
    double sn = sqrt(nn) / sqrt(2.0);
    if (sn > P->sigmaY)
      return A53 * P->rho0 / (2 * P->mu) * (1.0 - P->sigmaY / sn);
    return 0.0;
  } else {
    double c = A53 * P->rho0 / (2 * pow(P->mu, 1 / n));
    if (PL) {
      double s[9];
      sigma_full(Q, P, s);
      double nn = 0;
      for (int i = 0; i < 9; i++)
        nn += s[i] * s[i];
      double sn = sqrt(nn) / sqrt(2.0);
      return c * pow(sn, (1 - n) / n);
    }
    return c;
  }
}

static double theta2inv(const double *Q, const gpr_par *P) {
  return or_temperature(Q, P) / (P->kappa * Q[0]);
}

/* ------------------------------------------------------------------------ */
/* System (system/equations.cpp).                                          */

/* ret += F_d(Q)   (equations.cpp:11-48) */
void or_flux(const double *Q, int d, const gpr_par *P, double *ret) {
  double r = Q[0];
  double rE = Q[1];
  const double *rv = Q + 2;
  double p = or_pressure(Q, P);
  double vd = rv[d] / r;
  ret[0] += rv[d];
  ret[1] += vd * (rE + p);
  for (int i = 0; i < 3; i++)
    ret[2 + i] += vd * rv[i];
  ret[2 + d] += p;
  {
    const double *A = Q + 5;
    double sd[3];
    sigma_d(Q, P, d, sd);
    ret[1] -= (sd[0] * rv[0] + sd[1] * rv[1] + sd[2] * rv[2]) / r;
    for (int i = 0; i < 3; i++)
      ret[2 + i] -= sd[i];
    double Av[3];
    for (int i = 0; i < 3; i++)
      Av[i] = (A[3 * i] * rv[0] + A[3 * i + 1] * rv[1] + A[3 * i + 2] * rv[2]) / r;
    ret[5 + d] += Av[0];
    ret[8 + d] += Av[1];
    ret[11 + d] += Av[2];
  }
  if (THERMAL) {
    const double *rJ = Q + 14;
    double T = temperature_mg(r, p, P);
    ret[1] += P->calpha2 * T * rJ[d] / r;
    for (int i = 0; i < 3; i++)
      ret[14 + i] += vd * rJ[i];
    ret[14 + d] += T;
  }
}

/* ret = S(Q)   (equations.cpp:50-67) */
void or_source(const double *Q, const gpr_par *P, double *ret) {
  for (int i = 0; i < V; i++)
    ret[i] = 0.0;
  ret[2] = P->dp[0];
  ret[3] = P->dp[1];
  ret[4] = P->dp[2];
  {
    double EA[9];
    dEdA_s(Q, P, EA);
    double t1 = theta1inv(Q, P);
    for (int i = 0; i < 9; i++)
      ret[5 + i] = -EA[i] * t1;
  }
  if (THERMAL) {
    double r = Q[0];
    double t2 = theta2inv(Q, P);
    for (int i = 0; i < 3; i++)
      ret[14 + i] = -r * (P->calpha2 * Q[14 + i] / r) * t2;
  }
}

/* ret = B_d(Q) x   (equations.cpp:89-167) */
void or_Bdot(const double *Q, const double *x, int d, double *ret) {
  double r = Q[0];
  double v0 = Q[2] / r, v1 = Q[3] / r, v2 = Q[4] / r;
  for (int i = 0; i < V; i++)
    ret[i] = 0.0;
  if (d == 0) {
    ret[5] = -v1 * x[6] - v2 * x[7];
    ret[6] = v0 * x[6];
    ret[7] = v0 * x[7];
    ret[8] = -v1 * x[9] - v2 * x[10];
    ret[9] = v0 * x[9];
    ret[10] = v0 * x[10];
    ret[11] = -v1 * x[12] - v2 * x[13];
    ret[12] = v0 * x[12];
    ret[13] = v0 * x[13];
  } else if (d == 1) {
    ret[5] = v1 * x[5];
    ret[6] = -v0 * x[5] - v2 * x[7];
    ret[7] = v1 * x[7];
    ret[8] = v1 * x[8];
    ret[9] = -v0 * x[8] - v2 * x[10];
    ret[10] = v1 * x[10];
    ret[11] = v1 * x[11];
    ret[12] = -v0 * x[11] - v2 * x[13];
    ret[13] = v1 * x[13];
  } else {
    ret[5] = v2 * x[5];
    ret[6] = v2 * x[6];
    ret[7] = -v0 * x[5] - v1 * x[6];
    ret[8] = v2 * x[8];
    ret[9] = v2 * x[9];
    ret[10] = -v0 * x[8] - v1 * x[9];
    ret[11] = v2 * x[11];
    ret[12] = v2 * x[12];
    ret[13] = -v0 * x[11] - v1 * x[12];
  }
  double vd = d == 0 ? v0 : (d == 1 ? v1 : v2);
  for (int i = 1; i < LSET + 1; i++)
    ret[V - i] = vd * x[V - i];
}

/* ------------------------------------------------------------------------ */
/* Real nonsymmetric eigenvalues: Householder reduction to upper Hessenberg */
/* form, then the Francis double-shift QR iteration (Golub & Van Loan,      */
/* Matrix Computations, Alg. 7.4.2 / 7.5.1-7.5.2).  Eigen's EigenSolver,    */
/* which the reference calls (system/eig.cpp:73, fv/fluxes.cpp:30-33), is    */
/* the same algorithm family.  With want_vec the Schur vectors are          */
/* accumulated and eigenvectors recovered by back-substitution.             */

#define EMAX 18
/* Eigenvalues closer than MULT_TOL * ||T|| are one (semisimple) multiple
 * eigenvalue: their Schur vectors are kept as independent eigenvectors. */
#define MULT_TOL 1e-12

static void hessenberg(int n, double *H, double *Z) {
  /* H is n x n row-major (stride EMAX); Z accumulates (if not NULL). */
  for (int k = 0; k < n - 2; k++) {
    /* no reflection when the part below the subdiagonal is already zero to
     * the least normal number, as Eigen's makeHouseholder decides
     * (eigen3/src/Householder/Householder.h:76-83): reflecting a column of
     * subnormal entries would divide by an underflowed norm */
    double tail = 0.0;
    for (int i = k + 2; i < n; i++)
      tail += H[i * EMAX + k] * H[i * EMAX + k];
    if (tail <= DBL_MIN)
      continue;
    double alpha = 0.0;
    for (int i = k + 1; i < n; i++)
      alpha += H[i * EMAX + k] * H[i * EMAX + k];
    alpha = sqrt(alpha);
    if (alpha == 0.0)
      continue;
    double x0 = H[(k + 1) * EMAX + k];
    double beta = x0 > 0 ? -alpha : alpha;
    double v[EMAX];
    for (int i = 0; i < n; i++)
      v[i] = 0.0;
    v[k + 1] = x0 - beta;
    for (int i = k + 2; i < n; i++)
      v[i] = H[i * EMAX + k];
    double vv = 0.0;
    for (int i = k + 1; i < n; i++)
      vv += v[i] * v[i];
    if (vv == 0.0)
      continue;
    double tau = 2.0 / vv;
    /* H = (I - tau v v^T) H (I - tau v v^T) */
    for (int j = 0; j < n; j++) {
      double s = 0.0;
      for (int i = k + 1; i < n; i++)
        s += v[i] * H[i * EMAX + j];
      s *= tau;
      for (int i = k + 1; i < n; i++)
        H[i * EMAX + j] -= s * v[i];
    }
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      for (int j = k + 1; j < n; j++)
        s += H[i * EMAX + j] * v[j];
      s *= tau;
      for (int j = k + 1; j < n; j++)
        H[i * EMAX + j] -= s * v[j];
    }
    if (Z) {
      for (int i = 0; i < n; i++) {
        double s = 0.0;
        for (int j = k + 1; j < n; j++)
          s += Z[i * EMAX + j] * v[j];
        s *= tau;
        for (int j = k + 1; j < n; j++)
          Z[i * EMAX + j] -= s * v[j];
      }
    }
    for (int i = k + 2; i < n; i++)
      H[i * EMAX + k] = 0.0;
  }
}

/* Francis double-shift QR on upper Hessenberg H (n x n, stride EMAX).
 * Eigenvalues to (wr, wi).  If Z != NULL the transformations are applied
 * to the whole matrix and accumulated into Z (real Schur form).
 * Returns 0 on success, -1 if it fails to converge. */
static int hqr(int n, double *H, double *wr, double *wi, double *Z) {
  const double eps = 2.220446049250313e-16;
  double norm = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = (i > 0 ? i - 1 : 0); j < n; j++)
      norm += fabs(H[i * EMAX + j]);
  int hi = n - 1;
  int iter = 0, total = 0;
  double exshift = 0.0;
  while (hi >= 0) {
    /* look for a small subdiagonal element */
    int l = hi;
    while (l > 0) {
      double s = fabs(H[(l - 1) * EMAX + l - 1]) + fabs(H[l * EMAX + l]);
      if (s == 0.0)
        s = norm;
      if (fabs(H[l * EMAX + l - 1]) < eps * s)
        break;
      l--;
    }
    if (l == hi) { /* one root */
      H[hi * EMAX + hi] += exshift;
      wr[hi] = H[hi * EMAX + hi];
      wi[hi] = 0.0;
      if (hi > 0)
        H[hi * EMAX + hi - 1] = 0.0;
      hi--;
      iter = 0;
      continue;
    }
    double x = H[hi * EMAX + hi];
    double y = H[(hi - 1) * EMAX + hi - 1];
    double w = H[hi * EMAX + hi - 1] * H[(hi - 1) * EMAX + hi];
    if (l == hi - 1) { /* two roots */
      if (hi >= 2)
        H[(hi - 1) * EMAX + hi - 2] = 0.0;
      double p = 0.5 * (y - x);
      double q = p * p + w;
      /* A complex pair whose imaginary part is at rounding level is a real
       * double root (a semisimple multiple eigenvalue split by rounding). */
      if (q < 0.0 && sqrt(-q) <= MULT_TOL * norm)
        q = 0.0;
      double z = sqrt(fabs(q));
      H[hi * EMAX + hi] = x + exshift;
      H[(hi - 1) * EMAX + hi - 1] = y + exshift;
      x = H[hi * EMAX + hi];
      if (q >= 0.0) { /* real pair */
        z = p >= 0 ? p + z : p - z;
        wr[hi - 1] = x + z;
        wr[hi] = z != 0.0 ? x - w / z : x + z;
        wi[hi - 1] = wi[hi] = 0.0;
        if (Z) {
          /* rotate to upper triangular */
          double xx = H[hi * EMAX + hi - 1];
          double s = fabs(xx) + fabs(z);
          double pp = xx / s, qq = z / s;
          double rr = sqrt(pp * pp + qq * qq);
          pp /= rr;
          qq /= rr;
          for (int j = hi - 1; j < n; j++) {
            double a = H[(hi - 1) * EMAX + j];
            H[(hi - 1) * EMAX + j] = qq * a + pp * H[hi * EMAX + j];
            H[hi * EMAX + j] = qq * H[hi * EMAX + j] - pp * a;
          }
          for (int i = 0; i <= hi; i++) {
            double a = H[i * EMAX + hi - 1];
            H[i * EMAX + hi - 1] = qq * a + pp * H[i * EMAX + hi];
            H[i * EMAX + hi] = qq * H[i * EMAX + hi] - pp * a;
          }
          for (int i = 0; i < n; i++) {
            double a = Z[i * EMAX + hi - 1];
            Z[i * EMAX + hi - 1] = qq * a + pp * Z[i * EMAX + hi];
            Z[i * EMAX + hi] = qq * Z[i * EMAX + hi] - pp * a;
          }
          H[hi * EMAX + hi - 1] = 0.0;
        }
      } else { /* complex pair */
        wr[hi - 1] = wr[hi] = x + p;
        wi[hi - 1] = z;
        wi[hi] = -z;
      }
      hi -= 2;
      iter = 0;
      continue;
    }
    /* form shift */
    if (iter == 10 || iter == 20) { /* exceptional shift */
      exshift += x;
      for (int i = 0; i <= hi; i++)
        H[i * EMAX + i] -= x;
      double s = fabs(H[hi * EMAX + hi - 1]) + fabs(H[(hi - 1) * EMAX + hi - 2]);
      x = y = 0.75 * s;
      w = -0.4375 * s * s;
    }
    iter++;
    total++;
    if (total > 60 * n)
      return -1;
    /* look for two consecutive small subdiagonal elements */
    int m = hi - 2;
    double p = 0, q = 0, r = 0, z;
    while (m >= l) {
      z = H[m * EMAX + m];
      r = x - z;
      double s = y - z;
      p = (r * s - w) / H[(m + 1) * EMAX + m] + H[m * EMAX + m + 1];
      q = H[(m + 1) * EMAX + m + 1] - z - r - s;
      r = H[(m + 2) * EMAX + m + 1];
      s = fabs(p) + fabs(q) + fabs(r);
      p /= s;
      q /= s;
      r /= s;
      if (m == l)
        break;
      double u = fabs(H[m * EMAX + m - 1]) * (fabs(q) + fabs(r));
      double vv = fabs(p) * (fabs(H[(m - 1) * EMAX + m - 1]) + fabs(z) +
                             fabs(H[(m + 1) * EMAX + m + 1]));
      if (u < eps * vv)
        break;
      m--;
    }
    for (int i = m + 2; i <= hi; i++) {
      H[i * EMAX + i - 2] = 0.0;
      if (i > m + 2)
        H[i * EMAX + i - 3] = 0.0;
    }
    /* double QR step on rows l..hi, columns m..hi */
    for (int k = m; k <= hi - 1; k++) {
      int notlast = (k != hi - 1);
      if (k != m) {
        p = H[k * EMAX + k - 1];
        q = H[(k + 1) * EMAX + k - 1];
        r = notlast ? H[(k + 2) * EMAX + k - 1] : 0.0;
        x = fabs(p) + fabs(q) + fabs(r);
        if (x == 0.0)
          continue;
        p /= x;
        q /= x;
        r /= x;
      }
      double s = sqrt(p * p + q * q + r * r);
      if (p < 0)
        s = -s;
      if (k != m)
        H[k * EMAX + k - 1] = -s * x;
      else if (l != m)
        H[k * EMAX + k - 1] = -H[k * EMAX + k - 1];
      p += s;
      x = p / s;
      y = q / s;
      z = r / s;
      q /= p;
      r /= p;
      int jlo = Z ? k : k, jhi = Z ? n - 1 : hi;
      for (int j = jlo; j <= jhi; j++) { /* row modification */
        double pp = H[k * EMAX + j] + q * H[(k + 1) * EMAX + j];
        if (notlast) {
          pp += r * H[(k + 2) * EMAX + j];
          H[(k + 2) * EMAX + j] -= pp * z;
        }
        H[k * EMAX + j] -= pp * x;
        H[(k + 1) * EMAX + j] -= pp * y;
      }
      int ilo = Z ? 0 : l;
      int ihi = hi < k + 3 ? hi : k + 3;
      for (int i = ilo; i <= ihi; i++) { /* column modification */
        double pp = x * H[i * EMAX + k] + y * H[i * EMAX + k + 1];
        if (notlast) {
          pp += z * H[i * EMAX + k + 2];
          H[i * EMAX + k + 2] -= pp * r;
        }
        H[i * EMAX + k] -= pp;
        H[i * EMAX + k + 1] -= pp * q;
      }
      if (Z) {
        for (int i = 0; i < n; i++) {
          double pp = x * Z[i * EMAX + k] + y * Z[i * EMAX + k + 1];
          if (notlast) {
            pp += z * Z[i * EMAX + k + 2];
            Z[i * EMAX + k + 2] -= pp * r;
          }
          Z[i * EMAX + k] -= pp;
          Z[i * EMAX + k + 1] -= pp * q;
        }
      }
    }
  }
  return 0;
}

/* max |lambda| over the eigenvalues of the n x n row-major matrix M. */
static double max_abs_eig(int n, const double *M) {
  double H[EMAX * EMAX], wr[EMAX], wi[EMAX];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      H[i * EMAX + j] = M[i * n + j];
  hessenberg(n, H, NULL);
  if (hqr(n, H, wr, wi, NULL))
    return NAN;
  double m = 0.0;
  for (int i = 0; i < n; i++) {
    double a = hypot(wr[i], wi[i]);
    if (a > m || a != a)
      m = a;
  }
  return m;
}

int or_eigenvalues(int n, const double *M, double *wr, double *wi) {
  double H[EMAX * EMAX];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      H[i * EMAX + j] = M[i * n + j];
  hessenberg(n, H, NULL);
  return hqr(n, H, wr, wi, NULL);
}

/* ------------------------------------------------------------------------ */
/* Thermo-acoustic tensor and max |eig| (system/eig.cpp:8-77).              */

void or_thermo_acoustic_tensor(const double *Q, int d, const gpr_par *P,
                               double *out) {
  int m = THERMAL ? 4 : 3;
  double r = Q[0];
  double p = or_pressure(Q, P);
  double X1[4][5], X2[5][4];
  memset(X1, 0, sizeof X1);
  memset(X2, 0, sizeof X2);
  /* Xi1 (eig.cpp:8-27) */
  X1[0][1] = 1 / r;
  double dsr[3], dsA[9];
  dsigmadrho(Q, P, d, dsr);
  dsigmadA(Q, P, d, dsA);
  for (int i = 0; i < 3; i++) {
    X1[i][0] = -1 / r * dsr[i];
    for (int j = 0; j < 3; j++)
      X1[i][2 + j] = -1 / r * dsA[3 * i + j];
  }
  if (THERMAL) {
    X1[3][0] = dTdrho(r, p, P) / r;
    X1[3][1] = dTdp(r, P) / r;
  }
  /* Xi2 (eig.cpp:29-53) */
  {
    /* c_0 (waves/speeds.cpp:8-18) */
    double dEdr = dedrho(r, p, P) + dC_0drho(r, P) / 4 * devGsq(Q + 5);
    double dEp = dedp(r, P);
    double c0 = sqrt((p / (r * r) - dEdr) / dEp);
    X2[0][0] = r;
    X2[1][d] = r * c0 * c0;
    double sg[3];
    sigma_d(Q, P, d, sg);
    for (int i = 0; i < 3; i++)
      X2[1][i] += sg[i] - r * dsr[i];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        X2[2 + i][j] = Q[5 + 3 * i + j];
    if (THERMAL) {
      double T = temperature_mg(r, p, P);
      double ch = sqrt(P->calpha2 * T / P->cv) / r;
      X2[1][3] = r * ch * ch / dTdp(r, P);
    }
  }
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) {
      double s = 0.0;
      for (int k = 0; k < (THERMAL ? 5 : 5); k++)
        s += X1[i][k] * X2[k][j];
      out[i * m + j] = s;
    }
}

double or_max_abs_eigs(const double *Q, int d, const gpr_par *P) {
  int m = THERMAL ? 4 : 3;
  double Xi[16];
  or_thermo_acoustic_tensor(Q, d, P, Xi);
  double vd = Q[2 + d] / Q[0];
  double lam = sqrt(max_abs_eig(m, Xi));
  if (vd > 0)
    return vd + lam;
  return lam - vd;
}

/* ------------------------------------------------------------------------ */
/* System Jacobian (system/jacobians.cpp:10-152, equations.cpp:69-87, 169-176). */

static double dEdrho_Q(const double *Q, const gpr_par *P) {
  double r = Q[0];
  double p = or_pressure(Q, P);
  return dedrho(r, p, P) + dC_0drho(r, P) / 4 * devGsq(Q + 5);
}

static void dFdP(const double *Q, int d, const gpr_par *P, double *ret) {
  int n = V;
  memset(ret, 0, sizeof(double) * n * n);
#define R_(i, j) ret[(i) * n + (j)]
  double r = Q[0];
  double E = Q[1] / r;
  double p = or_pressure(Q, P);
  double v[3] = {Q[2] / r, Q[3] / r, Q[4] / r};
  const double *A = Q + 5;
  double Er = dEdrho_Q(Q, P);
  double Ep = dedp(r, P);
  double vd = v[d];
  double rvd = r * vd;
  double G[9], AG[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      G[3 * i + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  AdevG(A, AG);
  R_(0, 0) = vd;
  R_(0, 2 + d) = r;
  R_(1, 0) = (E + r * Er) * vd;
  R_(1, 1) = (r * Ep + 1) * vd;
  for (int i = 0; i < 3; i++)
    R_(1, 2 + i) = r * vd * v[i];
  R_(1, 2 + d) += r * E + p;
  for (int i = 0; i < 3; i++)
    R_(2 + i, 0) = vd * v[i];
  for (int i = 2; i < 5; i++)
    R_(i, i) = rvd;
  for (int i = 0; i < 3; i++)
    R_(2 + i, 2 + d) += r * v[i];
  R_(2 + d, 1) = 1.0;
  {
    double sg[3], sr[3], psi[9];
    sigma_d(Q, P, d, sg);
    dsigmadrho(Q, P, d, sr);
    double C0 = C_0(r, P);
    for (int i = 0; i < 9; i++)
      psi[i] = C0 * AG[i];
    double cs2 = c_s2(r, P);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        int ind = i * 3 + j;
        double tmp = 0.0;
        for (int k = 0; k < 3; k++) {
          /* dsigmadA(rho, cs2, A, G, AdevG, d, k, i, j) (state.cpp:58-71) */
          int ii = d, jj = k, mm = i, nn = j;
          double t = A[3 * mm + ii] * G[3 * jj + nn] + A[3 * mm + jj] * G[3 * ii + nn] -
                     2.0 / 3.0 * G[3 * ii + jj] * A[3 * mm + nn];
          if (ii == nn)
            t += AG[3 * mm + jj];
          if (jj == nn)
            t += AG[3 * mm + ii];
          double dsA = -r * cs2 * t;
          R_(2 + k, 5 + ind) = -dsA;
          tmp -= v[k] * dsA;
        }
        R_(1, 5 + ind) = tmp;
      }
    R_(1, 0) -= sr[0] * v[0] + sr[1] * v[1] + sr[2] * v[2];
    for (int i = 0; i < 3; i++)
      R_(1, 2 + i) -= sg[i];
    for (int i = 0; i < 9; i++)
      R_(1, 5 + i) += r * vd * psi[i];
    for (int i = 0; i < 3; i++)
      R_(2 + i, 0) -= sr[i];
    for (int j = 0; j < 3; j++) {
      R_(5 + d, 2 + j) = A[j];
      R_(8 + d, 2 + j) = A[3 + j];
      R_(11 + d, 2 + j) = A[6 + j];
      R_(5 + d, 5 + j) = v[j];
      R_(8 + d, 8 + j) = v[j];
      R_(11 + d, 11 + j) = v[j];
    }
  }
  if (THERMAL) {
    double ca2 = P->calpha2;
    double T = temperature_mg(r, p, P);
    double Tr = dTdrho(r, p, P);
    double Tp = dTdp(r, P);
    double J[3] = {Q[14] / r, Q[15] / r, Q[16] / r};
    double H[3] = {ca2 * Q[14] / r, ca2 * Q[15] / r, ca2 * Q[16] / r};
    R_(1, 0) += Tr * H[d];
    R_(1, 1) += Tp * H[d];
    for (int i = 0; i < 3; i++)
      R_(1, 14 + i) = rvd * H[i];
    R_(1, 14 + d) += ca2 * T;
    for (int i = 0; i < 3; i++)
      R_(14 + i, 0) = v[d] * J[i];
    R_(14 + d, 0) += Tr;
    R_(14 + d, 1) = Tp;
    for (int i = 0; i < 3; i++)
      R_(14 + i, 2 + d) = r * J[i];
    for (int i = 14; i < 17; i++)
      R_(i, i) = rvd;
  }
#undef R_
}

static void dPdQ(const double *Q, const gpr_par *P, double *ret) {
  int n = V;
  memset(ret, 0, sizeof(double) * n * n);
  for (int i = 0; i < n; i++)
    ret[i * n + i] = 1.0;
#define R_(i, j) ret[(i) * n + (j)]
  double r = Q[0];
  double E = Q[1] / r;
  double v[3] = {Q[2] / r, Q[3] / r, Q[4] / r};
  double Er = dEdrho_Q(Q, P);
  double Ep = dedp(r, P);
  double G_ = 1 / (r * Ep);
  double tmp = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) - (E + r * Er);
  double J[3] = {0, 0, 0};
  if (THERMAL) {
    J[0] = Q[14] / r;
    J[1] = Q[15] / r;
    J[2] = Q[16] / r;
    tmp += P->calpha2 * (J[0] * J[0] + J[1] * J[1] + J[2] * J[2]);
  }
  double Ups = G_ * tmp;
  R_(1, 0) = Ups;
  R_(1, 1) = G_;
  for (int i = 0; i < 3; i++) {
    R_(1, 2 + i) = -G_ * v[i];
    R_(2 + i, 0) = -v[i] / r;
  }
  for (int i = 2; i < 5; i++)
    R_(i, i) = 1 / r;
  {
    double AG[9];
    AdevG(Q + 5, AG);
    double C0 = C_0(r, P);
    for (int i = 0; i < 9; i++)
      R_(1, 5 + i) = -G_ * r * (C0 * AG[i]);
  }
  if (THERMAL) {
    for (int i = 0; i < 3; i++) {
      R_(1, 14 + i) = -G_ * (P->calpha2 * Q[14 + i] / r);
      R_(14 + i, 0) = -J[i] / r;
    }
    for (int i = 14; i < 17; i++)
      R_(i, i) = 1 / r;
  }
#undef R_
}

/* system_matrix = dFdP dPdQ + B   (equations.cpp:169-176) */
void or_system_matrix(const double *Q, int d, const gpr_par *P, double *M) {
  int n = V;
  double *F = malloc(sizeof(double) * n * n * 2);
  double *D = F + n * n;
  dFdP(Q, d, P, F);
  dPdQ(Q, P, D);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double s = 0.0;
      for (int k = 0; k < n; k++)
        s += F[i * n + k] * D[k * n + j];
      M[i * n + j] = s;
    }
  free(F);
  /* block (equations.cpp:69-87) */
  double r = Q[0];
  double vd = Q[2 + d] / r;
  for (int i = 5; i < 14; i++)
    M[i * n + i] += vd;
  for (int i = 0; i < 3; i++) {
    double vi = Q[2 + i] / r;
    M[(5 + d) * n + 5 + i] -= vi;
    M[(8 + d) * n + 8 + i] -= vi;
    M[(11 + d) * n + 11 + i] -= vi;
  }
  for (int i = 1; i < LSET + 1; i++)
    M[(V - i) * n + V - i] += vd;
}

/* ------------------------------------------------------------------------ */
/* Interface terms (solvers/fv/fluxes.cpp).                                */

/* Bint (fluxes.cpp:9-20) */
void or_Bint(const double *qL, const double *qR, int d, double *ret) {
  double dq[MAXV], q[MAXV], tmp[MAXV];
  for (int k = 0; k < V; k++) {
    ret[k] = 0.0;
    dq[k] = qR[k] - qL[k];
  }
  for (int i = 0; i < N; i++) {
    for (int k = 0; k < V; k++)
      q[k] = qL[k] + NODES[i] * dq[k];
    or_Bdot(q, dq, d, tmp);
    for (int k = 0; k < V; k++)
      ret[k] += WGHTS[i] * tmp[k];
  }
}

/* D_RUS (fluxes.cpp:66-75) */
void or_D_RUS(const double *qL, const double *qR, int d, const gpr_par *P,
              double *f) {
  double m1 = or_max_abs_eigs(qL, d, P);
  double m2 = or_max_abs_eigs(qR, d, P);
  double m = m1 > m2 ? m1 : m2;
  for (int k = 0; k < V; k++)
    f[k] = m * (qL[k] - qR[k]);
  or_flux(qL, d, P, f);
  or_flux(qR, d, P, f);
}

/* Complex solve of (R) x = b by Gaussian elimination with partial
 * pivoting; R is n x n complex (re, im) row-major, overwritten. */
static int csolve(int n, double *Rr, double *Ri, double *br, double *bi) {
  for (int c = 0; c < n; c++) {
    int p = c;
    double best = hypot(Rr[c * n + c], Ri[c * n + c]);
    for (int r = c + 1; r < n; r++) {
      double a = hypot(Rr[r * n + c], Ri[r * n + c]);
      if (a > best) {
        best = a;
        p = r;
      }
    }
    if (best == 0.0)
      return -1;
    if (p != c) {
      for (int j = 0; j < n; j++) {
        double t = Rr[c * n + j];
        Rr[c * n + j] = Rr[p * n + j];
        Rr[p * n + j] = t;
        t = Ri[c * n + j];
        Ri[c * n + j] = Ri[p * n + j];
        Ri[p * n + j] = t;
      }
      double t = br[c];
      br[c] = br[p];
      br[p] = t;
      t = bi[c];
      bi[c] = bi[p];
      bi[p] = t;
    }
    double pr = Rr[c * n + c], pi = Ri[c * n + c];
    double den = pr * pr + pi * pi;
    for (int r = c + 1; r < n; r++) {
      double ar = Rr[r * n + c], ai = Ri[r * n + c];
      double fr = (ar * pr + ai * pi) / den, fi = (ai * pr - ar * pi) / den;
      for (int j = c; j < n; j++) {
        double xr = Rr[c * n + j], xi = Ri[c * n + j];
        Rr[r * n + j] -= fr * xr - fi * xi;
        Ri[r * n + j] -= fr * xi + fi * xr;
      }
      br[r] -= fr * br[c] - fi * bi[c];
      bi[r] -= fr * bi[c] + fi * br[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    double sr = br[r], si = bi[r];
    for (int j = r + 1; j < n; j++) {
      sr -= Rr[r * n + j] * br[j] - Ri[r * n + j] * bi[j];
      si -= Rr[r * n + j] * bi[j] + Ri[r * n + j] * br[j];
    }
    double pr = Rr[r * n + r], pi = Ri[r * n + r];
    double den = pr * pr + pi * pi;
    br[r] = (sr * pr + si * pi) / den;
    bi[r] = (si * pr - sr * pi) / den;
  }
  return 0;
}

/* Eigenvectors from the real Schur form T (quasi upper triangular) and the
 * Schur vectors Z: back-substitution per eigenvalue, complex pairs handled
 * in complex arithmetic.  Produces the complex eigenvector matrix (columns)
 * in (Rr, Ri), n x n row-major. */
static void schur_eigvecs(int n, const double *T, const double *Z,
                          const double *wr, const double *wi, double *Rr,
                          double *Ri) {
  double norm = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = i > 0 ? i - 1 : 0; j < n; j++)
      norm += fabs(T[i * EMAX + j]);
  for (int k = 0; k < n; k++) {
    double lr = wr[k], li = wi[k];
    double yr[EMAX], yi[EMAX];
    for (int i = 0; i < n; i++)
      yr[i] = yi[i] = 0.0;
    /* find the block containing k */
    int blk2 = (k + 1 < n && T[(k + 1) * EMAX + k] != 0.0) ? 1 : 0;
    int blk1 = (k > 0 && T[k * EMAX + k - 1] != 0.0) ? 1 : 0;
    int top; /* last index of the eigenvector's support */
    if (!blk1 && !blk2) {
      yr[k] = 1.0;
      top = k;
    } else {
      /* 2x2 block at (b, b+1) */
      int b = blk2 ? k : k - 1;
      /* solve (T_bb - lambda I) [y_b; y_b1] = 0 */
      double a11 = T[b * EMAX + b] - lr, a12 = T[b * EMAX + b + 1];
      double a21 = T[(b + 1) * EMAX + b];
      /* choose y_{b+1} = 1, y_b = -a12/(a11 - i li) if possible */
      if (fabs(a12) >= fabs(a21)) {
        /* y_b = 1, y_{b+1} = -(a11 - i li)/a12 */
        yr[b] = 1.0;
        yi[b] = 0.0;
        yr[b + 1] = -a11 / a12;
        yi[b + 1] = li / a12;
      } else {
        /* y_{b+1} = 1, y_b = -a22'/a21 where a22' = T_b1b1 - lambda */
        double a22r = T[(b + 1) * EMAX + b + 1] - lr;
        yr[b + 1] = 1.0;
        yi[b + 1] = 0.0;
        yr[b] = -a22r / a21;
        yi[b] = li / a21;
      }
      top = b + 1;
    }
    /* back-substitute rows above the block */
    int start = (blk1 || blk2) ? (blk2 ? k - 1 : k - 2) : k - 1;
    for (int i = start; i >= 0; i--) {
      int is2 = (i > 0 && T[i * EMAX + i - 1] != 0.0);
      if (!is2) {
        double sr = 0.0, si = 0.0;
        for (int j = i + 1; j <= top; j++) {
          sr += T[i * EMAX + j] * yr[j];
          si += T[i * EMAX + j] * yi[j];
        }
        double dr = T[i * EMAX + i] - lr, di = -li;
        if (hypot(dr, di) <= MULT_TOL * norm) {
          yr[i] = yi[i] = 0.0; /* same eigenvalue: independent Schur vector */
          continue;
        }
        double den = dr * dr + di * di;
        yr[i] = -(sr * dr + si * di) / den;
        yi[i] = -(si * dr - sr * di) / den;
      } else {
        /* 2x2 block rows (i-1, i) */
        int a = i - 1;
        double s1r = 0, s1i = 0, s2r = 0, s2i = 0;
        for (int j = i + 1; j <= top; j++) {
          s1r += T[a * EMAX + j] * yr[j];
          s1i += T[a * EMAX + j] * yi[j];
          s2r += T[i * EMAX + j] * yr[j];
          s2i += T[i * EMAX + j] * yi[j];
        }
        /* [[t11-l, t12],[t21, t22-l]] y = -s */
        double m11r = T[a * EMAX + a] - lr, m11i = -li;
        double m12 = T[a * EMAX + i], m21 = T[i * EMAX + a];
        double m22r = T[i * EMAX + i] - lr, m22i = -li;
        double detr = m11r * m22r - m11i * m22i - m12 * m21;
        double deti = m11r * m22i + m11i * m22r;
        if (hypot(detr, deti) <= MULT_TOL * norm * MULT_TOL * norm) {
          yr[a] = yi[a] = yr[i] = yi[i] = 0.0;
          i--;
          continue;
        }
        double den = detr * detr + deti * deti;
        /* y_a = (-s1*m22 + m12*s2)/det ; y_i = (-m11*s2 + m21*s1)/det */
        double nar = -(s1r * m22r - s1i * m22i) + m12 * s2r;
        double nai = -(s1r * m22i + s1i * m22r) + m12 * s2i;
        double nir = -(m11r * s2r - m11i * s2i) + m21 * s1r;
        double nii = -(m11r * s2i + m11i * s2r) + m21 * s1i;
        yr[a] = (nar * detr + nai * deti) / den;
        yi[a] = (nai * detr - nar * deti) / den;
        yr[i] = (nir * detr + nii * deti) / den;
        yi[i] = (nii * detr - nir * deti) / den;
        i--; /* skip a */
      }
    }
    /* x = Z y */
    for (int i = 0; i < n; i++) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j <= top; j++) {
        sr += Z[i * EMAX + j] * yr[j];
        si += Z[i * EMAX + j] * yi[j];
      }
      Rr[i * n + k] = sr;
      Ri[i * n + k] = si;
    }
  }
}

/* Adds sum_i w_i R_i |Lambda_i| R_i^{-1} dq for J = system_matrix(q) into
 * (acc) -- the eigen-part of D_OSH (fluxes.cpp:22-44) / D_ROE (:46-64). */
static int abs_jac_apply(const double *J, const double *dq, double w,
                         double *acc) {
  int n = V;
  double H[EMAX * EMAX], Z[EMAX * EMAX], wr[EMAX], wi[EMAX];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      H[i * EMAX + j] = J[i * n + j];
      Z[i * EMAX + j] = (i == j) ? 1.0 : 0.0;
    }
  hessenberg(n, H, Z);
  if (hqr(n, H, wr, wi, Z))
    return -1;
  double Rr[EMAX * EMAX], Ri[EMAX * EMAX], Cr[EMAX * EMAX], Ci[EMAX * EMAX];
  schur_eigvecs(n, H, Z, wr, wi, Rr, Ri);
  memcpy(Cr, Rr, sizeof(double) * n * n);
  memcpy(Ci, Ri, sizeof(double) * n * n);
  double br[EMAX], bi[EMAX];
  for (int k = 0; k < n; k++) {
    br[k] = dq[k];
    bi[k] = 0.0;
  }
  if (csolve(n, Cr, Ci, br, bi))
    return -1;
  for (int k = 0; k < n; k++) {
    double a = hypot(wr[k], wi[k]);
    br[k] *= a;
    bi[k] *= a;
  }
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int k = 0; k < n; k++)
      s += Rr[i * n + k] * br[k] - Ri[i * n + k] * bi[k];
    acc[i] += w * s;
  }
  return 0;
}

/* D_OSH (fluxes.cpp:22-44) */
void or_D_OSH(const double *qL, const double *qR, int d, const gpr_par *P,
              double *f) {
  int n = V;
  double dq[MAXV], q[MAXV];
  double *J = malloc(sizeof(double) * n * n);
  for (int k = 0; k < n; k++) {
    dq[k] = qL[k] - qR[k];
    f[k] = 0.0;
  }
  for (int i = 0; i < N; i++) {
    for (int k = 0; k < n; k++)
      q[k] = qR[k] + NODES[i] * dq[k];
    or_system_matrix(q, d, P, J);
    if (abs_jac_apply(J, dq, WGHTS[i], f)) {
      for (int k = 0; k < n; k++)
        f[k] = NAN;
    }
  }
  free(J);
  or_flux(qL, d, P, f);
  or_flux(qR, d, P, f);
}

/* D_ROE (fluxes.cpp:46-64) */
void or_D_ROE(const double *qL, const double *qR, int d, const gpr_par *P,
              double *f) {
  int n = V;
  double dq[MAXV], q[MAXV];
  double *J = calloc(n * n * 2, sizeof(double));
  double *Ji = J + n * n;
  for (int k = 0; k < n; k++) {
    dq[k] = qL[k] - qR[k];
    f[k] = 0.0;
  }
  for (int i = 0; i < N; i++) {
    for (int k = 0; k < n; k++)
      q[k] = qR[k] + NODES[i] * dq[k];
    or_system_matrix(q, d, P, Ji);
    for (int k = 0; k < n * n; k++)
      J[k] += WGHTS[i] * Ji[k];
  }
  if (abs_jac_apply(J, dq, 1.0, f))
    for (int k = 0; k < n; k++)
      f[k] = NAN;
  free(J);
  or_flux(qL, d, P, f);
  or_flux(qR, d, P, f);
}

static void interface_D(int FLUX, const double *qL, const double *qR, int d,
                        const gpr_par *P, double *f) {
  switch (FLUX) {
  case GPR_FLUX_OSHER:
    or_D_OSH(qL, qR, d, P, f);
    break;
  case GPR_FLUX_ROE:
    or_D_ROE(qL, qR, d, P, f);
    break;
  default:
    or_D_RUS(qL, qR, d, P, f);
  }
}

/* ------------------------------------------------------------------------ */
/* Boundaries and masks (etc/grid.cpp:12-230).                              */

static void bc_row(double *dst, const double *src, int code, int d, int side,
                   const double *srcrow0) {
  (void)side;
  memcpy(dst, src, sizeof(double) * V);
  switch (code) {
  case GPR_BC_SLIP:
    dst[2 + d] *= -1.0;
    break;
  case GPR_BC_STICK:
    dst[2] *= -1.0;
    dst[3] *= -1.0;
    dst[4] *= -1.0;
    break;
  case GPR_BC_MOVING:
    dst[2] *= -1.0;
    dst[3] *= -1.0;
    dst[4] *= -1.0;
    dst[2] += 2.0 * dst[0];
    dst[1] += (dst[2] * dst[2] - srcrow0[2] * srcrow0[2]) / (2 * dst[0]);
    break;
  case GPR_BC_SYMMETRIC: {
    dst[2 + d] *= -1.0;
    double *A = dst + 5;
    for (int k = 0; k < 3; k++)
      A[3 * d + k] *= -1.0;
    for (int k = 0; k < 3; k++)
      A[3 * k + d] *= -1.0;
  } break;
  default:
    break;
  }
}

/* boundaries1 (grid.cpp:12-125) over a strided line: u rows at u + i*su,
 * ub rows at ub + i*sb (strides in doubles). */
static void boundaries1(const double *u, long su, double *ub, long sb, int nx,
                        const int *bt, int d) {
  for (int i = 0; i < N; i++) {
    const double *src;
    switch (bt[0]) {
    case GPR_BC_TRANSMISSIVE:
      src = u;
      break;
    case GPR_BC_PERIODIC:
      src = u + (long)(nx - N + i) * su;
      break;
    default:
      src = u + (long)(N - 1 - i) * su;
    }
    bc_row(ub + (long)i * sb, src, bt[0] == GPR_BC_PERIODIC ? 0 : bt[0], d, 0, src);
  }
  for (int i = 0; i < N; i++) {
    const double *src;
    switch (bt[1]) {
    case GPR_BC_TRANSMISSIVE:
      src = u + (long)(nx - 1) * su;
      break;
    case GPR_BC_PERIODIC:
      src = u + (long)i * su;
      break;
    default:
      src = u + (long)(nx - 1 - i) * su;
    }
    bc_row(ub + (long)(i + nx + N) * sb, src, bt[1] == GPR_BC_PERIODIC ? 0 : bt[1],
           d, 1, src);
  }
}

int or_boundaries(const double *u, double *ub, const int *nX, int ndim,
                  const int *bcs) {
  int nx = nX[0];
  if (ndim == 1) {
    memcpy(ub + N * V, u, sizeof(double) * nx * V);
    boundaries1(u, V, ub, V, nx, bcs, 0);
    return 0;
  }
  int ny = nX[1];
  long nyb = ny + 2 * N;
  for (int i = 0; i < nx; i++)
    memcpy(ub + ((long)(i + N) * nyb + N) * V, u + (long)i * ny * V,
           sizeof(double) * ny * V);
  for (int j = 0; j < ny; j++)
    boundaries1(u + (long)j * V, (long)ny * V, ub + (long)(j + N) * V, nyb * V, nx,
                bcs, 0);
  for (int i = 0; i < nx + 2 * N; i++)
    boundaries1(ub + ((long)i * nyb + N) * V, V, ub + (long)i * nyb * V, V, ny,
                bcs + 2, 1);
  return 0;
}

int or_extend_mask(const uint8_t *mask, uint8_t *maskb, const int *nX, int ndim) {
  int nx = nX[0];
  if (ndim == 1) {
    for (int i = 0; i < nx; i++)
      maskb[i + 1] = (mask[i] || (i > 0 && mask[i - 1]) || (i < nx - 1 && mask[i + 1]));
    maskb[0] = maskb[1];
    maskb[nx + 1] = maskb[nx];
    return 0;
  }
  int ny = nX[1];
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      int ind = i * ny + j;
      maskb[(i + 1) * (ny + 2) + (j + 1)] =
          (mask[ind] || (i > 0 && mask[(i - 1) * ny + j]) ||
           (i < nx - 1 && mask[(i + 1) * ny + j]) || (j > 0 && mask[ind - 1]) ||
           (j < ny - 1 && mask[ind + 1]));
    }
  for (int i = 0; i < nx; i++) {
    maskb[(i + 1) * (ny + 2)] = mask[i * ny];
    maskb[(i + 1) * (ny + 2) + (ny + 1)] = mask[i * ny + (ny - 1)];
  }
  for (int j = 0; j < ny; j++) {
    maskb[j + 1] = mask[j];
    maskb[(nx + 1) * (ny + 2) + (j + 1)] = mask[(nx - 1) * ny + j];
  }
  maskb[0] = 0;
  maskb[ny + 1] = 0;
  maskb[(nx + 1) * (ny + 2)] = 0;
  maskb[(nx + 1) * (ny + 2) + (ny + 1)] = 0;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* WENO (solvers/weno/weno.cpp).                                            */

/* weight (weno.cpp:4-15) for one variable */
static double weno_weight(const double *w, double LAM) {
  /* (w^T SIG) w, the reference's evaluation order: on near-constant data
   * w^T SIG is a difference of nearly equal coefficients, and forming it
   * first keeps the indicator accurate where the expanded quadratic form
   * would cancel catastrophically. */
  double t = 0.0;
  for (int b = 0; b < N; b++) {
    double tb = 0.0;
    for (int a = 0; a < N; a++)
      tb += w[a] * SIG[a][b];
    t += tb * w[b];
  }
  t += WENO_EPS;
  double t2 = t * t, t4 = t2 * t2, den = t4 * t4;
  return LAM / den;
}

/* coeffs (weno.cpp:17-73): data rows at data + r*sd (r = 0..2N-2), result
 * rows (N nodes) at ret + a*sr. */
static void weno_coeffs(double *ret, long sr, const double *data, long sd,
                        int nx, int gap, int ind) {
  for (int k = 0; k < V; k++) {
    double wL[MAXN], wR[MAXN], wCL[MAXN], wCR[MAXN];
    for (int a = 0; a < N; a++) {
      double sL = 0, sR = 0, sCL = 0, sCR = 0;
      for (int b = 0; b < N; b++) {
        sL += mLinv[a][b] * data[(long)b * sd + k];
        sR += mRinv[a][b] * data[(long)(N - 1 + b) * sd + k];
        if (N > 2) {
          sCL += mCLinv[a][b] * data[(long)(FN2 + b) * sd + k];
          if (N % 2 == 0)
            sCR += mCRinv[a][b] * data[(long)(CN2 + b) * sd + k];
        }
      }
      wL[a] = sL;
      wR[a] = sR;
      wCL[a] = sCL;
      wCR[a] = sCR;
    }
    double oL = weno_weight(wL, LAMS), oR = weno_weight(wR, LAMS);
    double oCL = 0, oCR = 0;
    if (N > 2) {
      oCL = weno_weight(wCL, LAMC);
      if (N % 2 == 0)
        oCR = weno_weight(wCR, LAMC);
    }
    double num[MAXN] = {0, 0, 0, 0}, den = 0.0;
    if (ind >= gap) {
      for (int a = 0; a < N; a++)
        num[a] += wL[a] * oL;
      den += oL;
    }
    if (ind <= nx - gap - 1) {
      for (int a = 0; a < N; a++)
        num[a] += wR[a] * oR;
      den += oR;
    }
    if (N > 2) {
      if (ind + FN2 >= gap) {
        for (int a = 0; a < N; a++)
          num[a] += wCL[a] * oCL;
        den += oCL;
      }
      if ((N % 2 == 0) && (ind - FN2 <= nx - gap - 1)) {
        for (int a = 0; a < N; a++)
          num[a] += wCR[a] * oCR;
        den += oCR;
      }
    }
    for (int a = 0; a < N; a++)
      ret[(long)a * sr + k] = num[a] / den;
  }
}

int or_weno_launcher(double *wh, const double *ub, const int *nX, int ndim) {
  if (ndim == 1) {
    int nx = nX[0] + 2;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; i++)
      weno_coeffs(wh + (long)i * N * V, V, ub + (long)i * V, V, nx, 0, i);
    return 0;
  }
  int nx = nX[0] + 2, ny = nX[1] + 2;
  int nyb = ny + 2 * (N - 1);
  double *ux = malloc(sizeof(double) * (long)nx * nyb * N * V);
  /* x sweep over every ub column (weno.cpp:93-104) */
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nyb; j++) {
    int gap = (j < N || j >= nyb - N) ? N : 0;
    for (int i = 0; i < nx; i++)
      weno_coeffs(ux + ((long)i * nyb + j) * N * V, V, ub + ((long)i * nyb + j) * V,
                  (long)nyb * V, nx, gap, i);
  }
  /* y sweep per x node (weno.cpp:106-121) */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int ii = 0; ii < N; ii++) {
      int gap = (i == 0 || i == nx - 1) ? 1 : 0;
      for (int j = 0; j < ny; j++)
        weno_coeffs(wh + (((long)i * ny + j) * N * N + ii * N) * V, V,
                    ux + (((long)i * nyb + j) * N + ii) * V, (long)N * V, ny, gap, j);
    }
  free(ux);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Space-time DG predictor (solvers/dg/dg1.cpp, dg2.cpp).                   */

/* rhs1 / rhs2: q, Ww and ret are [N time][N^d space][V]. */
static void dg_rhs(int ndim, const double *q, const double *Ww, double dt,
                   const double *dX, const gpr_par *P, double *ret) {
  int ns = ndim == 1 ? N : N * N;
  int nn = N * ns;
  double *F = malloc(sizeof(double) * nn * V * 4);
  double *G = F + nn * V, *dqx = G + nn * V, *dqy = dqx + nn * V;
  memset(F, 0, sizeof(double) * nn * V * 2);
  double dx = dX[0], dy = ndim == 2 ? dX[1] : 1.0;
  /* spatial derivatives (dg1.cpp:31-32, evaluations.cpp:3-18) */
  for (int t = 0; t < N; t++) {
    if (ndim == 1) {
      for (int i = 0; i < N; i++)
        for (int k = 0; k < V; k++) {
          double s = 0.0;
          for (int m = 0; m < N; m++)
            s += DERVALS[i][m] * q[((t * N) + m) * V + k];
          dqx[(t * N + i) * V + k] = s / dx;
        }
    } else {
      for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
          for (int k = 0; k < V; k++) {
            double sx = 0.0, sy = 0.0;
            for (int m = 0; m < N; m++) {
              sx += DERVALS[i][m] * q[((t * N + m) * N + j) * V + k];
              sy += DERVALS[j][m] * q[((t * N + i) * N + m) * V + k];
            }
            dqx[((t * N + i) * N + j) * V + k] = sx / dx;
            dqy[((t * N + i) * N + j) * V + k] = sy / dy;
          }
    }
  }
  double tmp[MAXV], tmpy[MAXV];
  for (int n = 0; n < nn; n++) {
    const double *qn = q + n * V;
    int t = n / ns, i = (n / (ndim == 1 ? 1 : N)) % N, j = n % N;
    or_source(qn, P, ret + n * V);
    or_Bdot(qn, dqx + n * V, 0, tmp);
    if (ndim == 2)
      or_Bdot(qn, dqy + n * V, 1, tmpy);
    double w = ndim == 1 ? WGHTS[t] * WGHTS[i] : WGHTS[t] * WGHTS[i] * WGHTS[j];
    for (int k = 0; k < V; k++) {
      double r = ret[n * V + k] - (ndim == 2 ? tmp[k] + tmpy[k] : tmp[k]);
      ret[n * V + k] = r * w;
    }
    or_flux(qn, 0, P, F + n * V);
    if (ndim == 2)
      or_flux(qn, 1, P, G + n * V);
  }
  if (ndim == 1) {
    for (int t = 0; t < N; t++)
      for (int i = 0; i < N; i++)
        for (int k = 0; k < V; k++) {
          double s = 0.0;
          for (int m = 0; m < N; m++)
            s += WGHTS[t] * DG_DER[i][m] * F[(t * N + m) * V + k];
          ret[(t * N + i) * V + k] -= s / dx;
        }
  } else {
    /* dg2.cpp:42-66 */
    for (int t = 0; t < N; t++)
      for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
          for (int k = 0; k < V; k++) {
            double sx = 0.0, sy = 0.0;
            for (int m = 0; m < N; m++) {
              sx += WGHTS[t] * DG_DER[i][m] * (WGHTS[j] * F[((t * N + m) * N + j) * V + k]);
              sy += DG_DER[j][m] * G[((t * N + i) * N + m) * V + k];
            }
            ret[((t * N + i) * N + j) * V + k] -= sx / dx;
            ret[((t * N + i) * N + j) * V + k] -= WGHTS[t] * WGHTS[i] * sy / dy;
          }
  }
  for (int n = 0; n < nn * V; n++)
    ret[n] = ret[n] * dt + Ww[n];
  free(F);
}

/* q = DG_U^{-1} r with DG_U = kron(DG_MAT, W [, W]) (etc/globals.cpp:46-50) */
static void dg_solve(int ndim, const double *r, double *q) {
  int ns = ndim == 1 ? N : N * N;
  for (int s = 0; s < ns; s++) {
    double ws = ndim == 1 ? WGHTS[s] : WGHTS[s / N] * WGHTS[s % N];
    for (int t = 0; t < N; t++)
      for (int k = 0; k < V; k++) {
        double acc = 0.0;
        for (int m = 0; m < N; m++)
          acc += DG_MATinv[t][m] * r[(m * ns + s) * V + k];
        q[(t * ns + s) * V + k] = acc / ws;
      }
  }
}

/* obj(q) = rhs(q) - DG_U q   (dg1.cpp:37-49, dg2.cpp:73-90) */
static void dg_obj(int ndim, const double *q, const double *Ww, double dt,
                   const double *dX, const gpr_par *P, double *out) {
  int ns = ndim == 1 ? N : N * N;
  dg_rhs(ndim, q, Ww, dt, dX, P, out);
  for (int t = 0; t < N; t++)
    for (int s = 0; s < ns; s++) {
      double ws = ndim == 1 ? WGHTS[s] : WGHTS[s / N] * WGHTS[s % N];
      for (int m = 0; m < N; m++)
        for (int k = 0; k < V; k++)
          out[(t * ns + s) * V + k] -= DG_MAT[t][m] * ws * q[(m * ns + s) * V + k];
    }
}

/* Dense Newton on obj(q) = 0 with a finite-difference Jacobian: the
 * oracle's check of the device Newton path for cells where the reference's
 * Picard iteration does not converge.  Returns iterations or -1. */
static int dg_newton(int ndim, double *q, const double *Ww, double dt,
                     const double *dX, const gpr_par *P, double tol, int maxit) {
  int ns = ndim == 1 ? N : N * N;
  int n = N * ns * V;
  double *J = malloc(sizeof(double) * ((long)n * n + 4 * n));
  double *f = J + (long)n * n, *f2 = f + n, *qp = f2 + n, *dxv = qp + n;
  int it;
  for (it = 0; it < maxit; it++) {
    dg_obj(ndim, q, Ww, dt, dX, P, f);
    double fn = 0.0;
    for (int i = 0; i < n; i++)
      fn = fmax(fn, fabs(f[i]));
    if (fn != fn)
      break;
    for (int c = 0; c < n; c++) {
      memcpy(qp, q, sizeof(double) * n);
      double h = 1e-7 * (1.0 + fabs(q[c]));
      qp[c] += h;
      dg_obj(ndim, qp, Ww, dt, dX, P, f2);
      for (int r = 0; r < n; r++)
        J[(long)r * n + c] = (f2[r] - f[r]) / h;
    }
    /* solve J dx = -f (partial pivoting) */
    for (int r = 0; r < n; r++)
      dxv[r] = -f[r];
    int ok = 1;
    for (int c = 0; c < n && ok; c++) {
      int p = c;
      for (int r = c + 1; r < n; r++)
        if (fabs(J[(long)r * n + c]) > fabs(J[(long)p * n + c]))
          p = r;
      if (J[(long)p * n + c] == 0.0) {
        ok = 0;
        break;
      }
      if (p != c) {
        for (int j = 0; j < n; j++) {
          double t = J[(long)c * n + j];
          J[(long)c * n + j] = J[(long)p * n + j];
          J[(long)p * n + j] = t;
        }
        double t = dxv[c];
        dxv[c] = dxv[p];
        dxv[p] = t;
      }
      for (int r = c + 1; r < n; r++) {
        double fct = J[(long)r * n + c] / J[(long)c * n + c];
        if (fct == 0.0)
          continue;
        for (int j = c; j < n; j++)
          J[(long)r * n + j] -= fct * J[(long)c * n + j];
        dxv[r] -= fct * dxv[c];
      }
    }
    if (!ok)
      break;
    for (int r = n - 1; r >= 0; r--) {
      double s = dxv[r];
      for (int j = r + 1; j < n; j++)
        s -= J[(long)r * n + j] * dxv[j];
      dxv[r] = s / J[(long)r * n + r];
    }
    int conv = 1;
    for (int i = 0; i < n; i++) {
      q[i] += dxv[i];
      if (fabs(dxv[i]) > tol * (1 + fabs(q[i])))
        conv = 0;
    }
    if (conv) {
      free(J);
      return it + 1;
    }
  }
  free(J);
  return -1;
}

/* Stiff-source Jacobian blocks at one state: the distortion block
 * JA[9][9] = dS_A/dA and the heat-flux block JJ[3][3] = dS_J/d(rho J).
 * S_A = -cs2 theta1(det A) A devG(A) (equations.cpp:156-159), with
 *   d(A devG)/dA : X -> X devG + A X^T A + A A^T X - 2/3 (A:X) A,
 *   d theta1/dA : X -> 5/3 theta1 tr(A^-1 X) (theta1 ~ det(A)^(5/3));
 * S_J = -calpha2 J T / kappa with J = rho J / rho and
 *   dT/d(rho J_k) = -calpha2 J_k / (rho cv Gamma rho) * rho Gamma = -calpha2 J_k / (rho cv).
 * Only the Newtonian relaxation rate is differentiated; other rates use
 * the same expression with their theta1 (a quasi-Newton Jacobian). */
static void stiff_jacobian(const double *Q, const gpr_par *P, double JA[9][9],
                           double JJ[3][3]) {
  double r = Q[0];
  const double *A = Q + 5;
  double cs2 = c_s2(r, P);
  double th = theta1inv(Q, P);
  double G[9], dG[9], H[9], AG[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      G[3 * i + j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
      H[3 * i + j] = A[3 * i] * A[3 * j] + A[3 * i + 1] * A[3 * j + 1] + A[3 * i + 2] * A[3 * j + 2];
    }
  double t3 = (G[0] + G[4] + G[8]) / 3;
  for (int k = 0; k < 9; k++)
    dG[k] = G[k];
  dG[0] -= t3;
  dG[4] -= t3;
  dG[8] -= t3;
  AdevG(A, AG);
  /* A^-1 (for the det term) */
  double d = det3(A);
  double Ai[9];
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) / d;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) / d;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) / d;
  Ai[3] = (A[5] * A[6] - A[3] * A[8]) / d;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) / d;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) / d;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) / d;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) / d;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) / d;
  int newtonian = !(P->flags & (GPR_SOLID | GPR_POWER_LAW | GPR_BINGHAM));
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++) {
      int c = 3 * m + n;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double v = (i == m ? dG[3 * n + j] : 0.0) + A[3 * i + n] * A[3 * m + j] +
                     (n == j ? H[3 * i + m] : 0.0) - 2.0 / 3.0 * A[3 * i + j] * A[3 * m + n];
          double dth = newtonian ? 5.0 / 3.0 * th * Ai[3 * n + m] : 0.0;
          JA[3 * i + j][c] = -cs2 * (th * v + AG[3 * i + j] * dth);
        }
    }
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      JJ[l][k] = 0.0;
  if (THERMAL) {
    double T = or_temperature(Q, P);
    double J[3] = {Q[14] / r, Q[15] / r, Q[16] / r};
    double f = -P->calpha2 / P->kappa;
    for (int l = 0; l < 3; l++)
      for (int k = 0; k < 3; k++) {
        double dT = -P->calpha2 * J[k] / (r * P->cv);
        JJ[l][k] = f * ((l == k ? T / r : 0.0) + J[l] * dT);
      }
  }
}

/* Dense solve with partial pivoting, n <= 24, A row-major n x n. */
static int small_solve(int n, double *A, double *b) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(A[r * n + c]) > fabs(A[p * n + c]))
        p = r;
    if (A[p * n + c] == 0.0)
      return -1;
    if (p != c) {
      for (int j = 0; j < n; j++) {
        double t = A[c * n + j];
        A[c * n + j] = A[p * n + j];
        A[p * n + j] = t;
      }
      double t = b[c];
      b[c] = b[p];
      b[p] = t;
    }
    double inv = 1.0 / A[c * n + c];
    for (int r = c + 1; r < n; r++) {
      double f = A[r * n + c] * inv;
      if (f == 0.0)
        continue;
      for (int j = c; j < n; j++)
        A[r * n + j] -= f * A[c * n + j];
      b[r] -= f * b[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    double s = b[r];
    for (int j = r + 1; j < n; j++)
      s -= A[r * n + j] * b[j];
    b[r] = s / A[r * n + r];
  }
  return 0;
}

/* Stiff-source Newton iteration on the predictor fixed point
 *   Fp(q) = DG_U q - Ww - dt R(q) = 0:
 *   delta = (DG_U - dt W dS/dq)^-1 (Ww + dt R(q) - DG_U q),  q += delta,
 * with dS/dq the local source Jacobian (stiff_jacobian) at each space-time
 * node, so the correction is implicit in the relaxation sources and explicit
 * in the fluxes.  With dS/dq = 0 this is exactly the Picard update of
 * dg1.cpp:110.  Per spatial node the system couples the N time nodes through
 * DG_MAT: an (N*9) system for A, an (N*3) system for rho J and the DG_MAT
 * solve for the other variables.  Returns iterations, or -1. */
static int dg_stiff(int ndim, double *q, const double *Ww, double dt, const double *dX,
                    const gpr_par *P, double tol, int maxit) {
  int ns = ndim == 1 ? N : N * N;
  int nn = N * ns;
  double r[2 * MAXN * MAXN * MAXN * MAXV], g[2 * MAXN * MAXN * MAXN * MAXV];
  double JA[MAXN * MAXN * MAXN][9][9], JJ[MAXN * MAXN * MAXN][3][3];
  for (int it = 0; it < maxit; it++) {
    dg_rhs(ndim, q, Ww, dt, dX, P, r);
    /* g = r - DG_U q */
    for (int t = 0; t < N; t++)
      for (int s = 0; s < ns; s++) {
        double ws = ndim == 1 ? WGHTS[s] : WGHTS[s / N] * WGHTS[s % N];
        for (int k = 0; k < V; k++) {
          double uq = 0.0;
          for (int m = 0; m < N; m++)
            uq += DG_MAT[t][m] * q[(m * ns + s) * V + k];
          g[(t * ns + s) * V + k] = r[(t * ns + s) * V + k] - ws * uq;
        }
      }
    for (int n = 0; n < nn; n++)
      stiff_jacobian(q + n * V, P, JA[n], JJ[n]);
    double dmax = 0.0;
    int bad = 0;
    for (int s = 0; s < ns; s++) {
      double ws = ndim == 1 ? WGHTS[s] : WGHTS[s / N] * WGHTS[s % N];
      /* non-stiff variables: DG_MAT solve (rows of S are zero there) */
      for (int k = 0; k < V; k++) {
        if ((k >= 5 && k < 14) || (THERMAL && k >= 14 && k < 17))
          continue;
        for (int t = 0; t < N; t++) {
          double acc = 0.0;
          for (int m = 0; m < N; m++)
            acc += DG_MATinv[t][m] * g[(m * ns + s) * V + k];
          r[(t * ns + s) * V + k] = acc / ws;
        }
      }
      /* distortion block: (DG_MAT x I9 - dt W_t JA_t) dA = gA / W_s */
      {
        int n9 = 9 * N;
        double K[9 * MAXN * 9 * MAXN], b[9 * MAXN];
        for (int t = 0; t < N; t++)
          for (int i = 0; i < 9; i++) {
            int row = t * 9 + i;
            b[row] = g[(t * ns + s) * V + 5 + i] / ws;
            for (int t2 = 0; t2 < N; t2++)
              for (int j = 0; j < 9; j++)
                K[row * n9 + t2 * 9 + j] =
                    (i == j ? DG_MAT[t][t2] : 0.0) -
                    (t == t2 ? dt * WGHTS[t] * JA[t * ns + s][i][j] : 0.0);
          }
        if (small_solve(n9, K, b))
          bad = 1;
        for (int t = 0; t < N; t++)
          for (int i = 0; i < 9; i++)
            r[(t * ns + s) * V + 5 + i] = b[t * 9 + i];
      }
      if (THERMAL) {
        int n3 = 3 * N;
        double K[3 * MAXN * 3 * MAXN], b[3 * MAXN];
        for (int t = 0; t < N; t++)
          for (int i = 0; i < 3; i++) {
            int row = t * 3 + i;
            b[row] = g[(t * ns + s) * V + 14 + i] / ws;
            for (int t2 = 0; t2 < N; t2++)
              for (int j = 0; j < 3; j++)
                K[row * n3 + t2 * 3 + j] =
                    (i == j ? DG_MAT[t][t2] : 0.0) -
                    (t == t2 ? dt * WGHTS[t] * JJ[t * ns + s][i][j] : 0.0);
          }
        if (small_solve(n3, K, b))
          bad = 1;
        for (int t = 0; t < N; t++)
          for (int i = 0; i < 3; i++)
            r[(t * ns + s) * V + 14 + i] = b[t * 3 + i];
      }
    }
    if (bad)
      return -1;
    int conv = 1;
    for (int k = 0; k < nn * V; k++) {
      q[k] += r[k];
      if (fabs(r[k]) > tol * (1 + fabs(q[k])))
        conv = 0;
      if (r[k] != r[k])
        return -1;
      dmax = fmax(dmax, fabs(r[k]));
    }
    (void)dmax;
    if (conv)
      return it + 1;
  }
  return -1;
}

int or_stiff_iterations_hist[64];

/* predictor1 / predictor2 (dg1.cpp:58-114, dg2.cpp:102-171).  status[cell]
 * receives: Picard iteration count (>0) when the reference's Picard
 * converged; -(Newton iterations) - 1000 when Picard failed and the oracle's
 * Newton solve converged; -1 when neither converged (row left unwritten, as
 * the reference leaves it); 0 for masked-out cells. */
int or_predictor(double *qh, const double *wh, double dt, const double *dX,
                 int ndim, const int *nX, int stiff, const gpr_par *P,
                 const uint8_t *mask, int *status, int newton_fallback) {
  int ncell = ndim == 1 ? nX[0] + 2 : (nX[0] + 2) * (nX[1] + 2);
  int ns = ndim == 1 ? N : N * N;
  int nn = N * ns;
#pragma omp parallel for schedule(dynamic, 16)
  for (int c = 0; c < ncell; c++) {
    if (status)
      status[c] = 0;
    if (!mask[c])
      continue;
    const double *w = wh + (long)c * ns * V;
    double *qi = qh + (long)c * nn * V;
    double Ww[2 * MAXN * MAXN * MAXN * MAXV];
    double q0[2 * MAXN * MAXN * MAXN * MAXV], q1[2 * MAXN * MAXN * MAXN * MAXV],
        r[2 * MAXN * MAXN * MAXN * MAXV];
    /* initial_condition (dg1.cpp:68-73, dg2.cpp:92-100) */
    for (int t = 0; t < N; t++)
      for (int s = 0; s < ns; s++) {
        double ws = ndim == 1 ? WGHTS[s] : WGHTS[s / N] * WGHTS[s % N];
        for (int k = 0; k < V; k++)
          Ww[(t * ns + s) * V + k] = ENDVALS[0][t] * ws * w[s * V + k];
      }
    /* standard_initial_guess (initial_guess.cpp:4-15) */
    for (int t = 0; t < N; t++)
      memcpy(q0 + t * ns * V, w, sizeof(double) * ns * V);
    int done = 0, nan = 0;
    if (!stiff) {
      for (int count = 0; count < DG_IT; count++) {
        dg_rhs(ndim, q0, Ww, dt, dX, P, r);
        dg_solve(ndim, r, q1);
        int big = 0, hasnan = 0;
        for (int k = 0; k < nn * V; k++) {
          if (fabs(q1[k] - q0[k]) > DG_TOL * (1 + fabs(q0[k])))
            big = 1;
          if (q1[k] != q1[k])
            hasnan = 1;
        }
        if (big) {
          memcpy(q0, q1, sizeof(double) * nn * V);
          continue;
        } else if (hasnan) {
          nan = 1;
          break;
        } else {
          memcpy(qi, q1, sizeof(double) * nn * V);
          if (status)
            status[c] = count + 1;
          done = 1;
          break;
        }
      }
    }
    if (!done && newton_fallback) {
      for (int t = 0; t < N; t++)
        memcpy(q0 + t * ns * V, w, sizeof(double) * ns * V);
      int it = newton_fallback == 2 ? dg_newton(ndim, q0, Ww, dt, dX, P, 1e-12, 30)
                                    : dg_stiff(ndim, q0, Ww, dt, dX, P, STIFF_TOL, STIFF_IT);
      if (it > 0) {
        memcpy(qi, q0, sizeof(double) * nn * V);
        if (status)
          status[c] = -1000 - it;
        done = 1;
      }
    }
    if (!done && status)
      status[c] = nan ? -2 : -1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Finite-volume update (solvers/fv/fv.cpp).                               */

static void centers_cell(double *ucell, const double *qh_t, int ndim, double dx,
                         double dy, double wght_t, int SOURCES,
                         const gpr_par *P) {
  int ns = ndim == 1 ? N : N * N;
  double S[MAXV], tmpx[MAXV], tmpy[MAXV], dqx[MAXV], dqy[MAXV];
  for (int s = 0; s < ns; s++) {
    const double *qs = qh_t + s * V;
    int a = ndim == 1 ? s : s / N, b = ndim == 1 ? 0 : s % N;
    for (int k = 0; k < V; k++) {
      double sx = 0.0, sy = 0.0;
      for (int m = 0; m < N; m++) {
        if (ndim == 1)
          sx += DERVALS[a][m] * qh_t[m * V + k];
        else {
          sx += DERVALS[a][m] * qh_t[(m * N + b) * V + k];
          sy += DERVALS[b][m] * qh_t[(a * N + m) * V + k];
        }
      }
      dqx[k] = sx;
      dqy[k] = sy;
    }
    if (SOURCES)
      or_source(qs, P, S);
    else
      for (int k = 0; k < V; k++)
        S[k] = 0.0;
    or_Bdot(qs, dqx, 0, tmpx);
    if (ndim == 2)
      or_Bdot(qs, dqy, 1, tmpy);
    for (int k = 0; k < V; k++) {
      S[k] -= tmpx[k] / dx;
      if (ndim == 2)
        S[k] -= tmpy[k] / dy;
    }
    double w = ndim == 1 ? wght_t * WGHTS[s] : wght_t * WGHTS[a] * WGHTS[b];
    for (int k = 0; k < V; k++)
      ucell[k] += w * S[k];
  }
}

/* fv_launcher's two passes (fv.cpp:11-279): parts bit 0 the volume term
 * (centers1 / centers2), bit 1 the interface terms (interfs1 / interfs2). */
int or_fv_parts(double *u, const double *qh, const int *nX, double dt, const double *dX,
                int ndim, int SOURCES, int TIME, int FLUX, const gpr_par *P,
                const uint8_t *mask, int parts) {
  int nt = TIME ? N : 1;
  int nx = nX[0], ny = ndim == 2 ? nX[1] : 1;
  int ns = ndim == 1 ? N : N * N;
  double dx = dX[0], dy = ndim == 2 ? dX[1] : 1.0;
  long ncellb = ndim == 1 ? nx + 2 : (long)(nx + 2) * (ny + 2);
  (void)ncellb;
  /* centers (fv.cpp:11-109) */
  for (int t = 0; t < nt && (parts & 1); t++) {
    double wt = TIME ? dt * WGHTS[t] : dt;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nx * ny; c++) {
      int i = ndim == 1 ? (int)c : (int)(c / ny), j = ndim == 1 ? 0 : (int)(c % ny);
      long cb = ndim == 1 ? i + 1 : (long)(i + 1) * (ny + 2) + (j + 1);
      if (!mask[cb])
        continue;
      const double *qt = qh + (cb * nt + t) * ns * V;
      centers_cell(u + c * V, qt, ndim, dx, dy, wt, SOURCES, P);
    }
  }
  if (!(parts & 2))
    return 0;
  /* interfaces (fv.cpp:111-279): fluxes per face computed in parallel,
   * then applied in the reference's order. */
  double ENDL[MAXN], ENDR[MAXN];
  for (int m = 0; m < N; m++) {
    ENDL[m] = ENDVALS[1][m];
    ENDR[m] = ENDVALS[0][m];
  }
  if (ndim == 1) {
    double *fb = malloc(sizeof(double) * (nx + 1) * 2 * V);
    for (int t = 0; t < nt; t++) {
      double wt = TIME ? dt * WGHTS[t] : dt;
      double kk = wt / (2.0 * dx);
#pragma omp parallel for schedule(static)
      for (int i = 0; i < nx + 1; i++) {
        double *f = fb + (long)i * 2 * V, *b = f + V;
        if (!(mask[i] && mask[i + 1]))
          continue;
        const double *qhl = qh + ((long)i * nt + t) * N * V;
        const double *qhr = qh + ((long)(i + 1) * nt + t) * N * V;
        double ql[MAXV], qr[MAXV];
        for (int k = 0; k < V; k++) {
          double sl = 0, sr = 0;
          for (int m = 0; m < N; m++) {
            sl += ENDL[m] * qhl[m * V + k];
            sr += ENDR[m] * qhr[m * V + k];
          }
          ql[k] = sl;
          qr[k] = sr;
        }
        interface_D(FLUX, ql, qr, 0, P, f);
        or_Bint(ql, qr, 0, b);
      }
      for (int i = 0; i < nx + 1; i++) {
        if (!(mask[i] && mask[i + 1]))
          continue;
        const double *f = fb + (long)i * 2 * V, *b = f + V;
        if (i > 0)
          for (int k = 0; k < V; k++)
            u[(long)(i - 1) * V + k] -= kk * (b[k] + f[k]);
        if (i < nx)
          for (int k = 0; k < V; k++)
            u[(long)i * V + k] -= kk * (b[k] - f[k]);
      }
    }
    free(fb);
    return 0;
  }
  /* 2D (fv.cpp:162-268): per face (i,j) of the (nx+1)x(ny+1) grid; the x
   * face sits between predictor cells (i,j) and (i+1,j), the y face between
   * (i,j) and (i,j+1). */
  long nfx = (long)(nx + 1) * (ny + 1);
  double *fx = malloc(sizeof(double) * nfx * 4 * V);
  for (int t = 0; t < nt; t++) {
    double wt = TIME ? dt * WGHTS[t] : dt;
    double xW[MAXN], yW[MAXN];
    for (int s = 0; s < N; s++) {
      xW[s] = wt / (2. * dx) * WGHTS[s];
      yW[s] = wt / (2. * dy) * WGHTS[s];
    }
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nfx; c++) {
      int i = (int)(c / (ny + 1)), j = (int)(c % (ny + 1));
      double *ux0 = fx + c * 4 * V, *ux1 = ux0 + V, *uy0 = ux1 + V, *uy1 = uy0 + V;
      for (int k = 0; k < 4 * V; k++)
        ux0[k] = 0.0;
      long cb = (long)i * (ny + 2) + j;
      if (!mask[cb])
        continue;
      const double *qh0 = qh + (cb * nt + t) * N * N * V;
      double q0[MAXV], q1[MAXV], f[MAXV], b[MAXV];
      if (mask[cb + (ny + 2)] && j > 0) {
        const double *qhx = qh + ((cb + (ny + 2)) * nt + t) * N * N * V;
        for (int s = 0; s < N; s++) {
          for (int k = 0; k < V; k++) {
            double s0 = 0, s1 = 0;
            for (int m = 0; m < N; m++) {
              s0 += ENDVALS[1][m] * qh0[(m * N + s) * V + k];
              s1 += ENDVALS[0][m] * qhx[(m * N + s) * V + k];
            }
            q0[k] = s0;
            q1[k] = s1;
          }
          interface_D(FLUX, q0, q1, 0, P, f);
          or_Bint(q0, q1, 0, b);
          for (int k = 0; k < V; k++) {
            ux0[k] += xW[s] * (b[k] + f[k]);
            ux1[k] += xW[s] * (b[k] - f[k]);
          }
        }
      }
      if (mask[cb + 1] && i > 0) {
        const double *qhy = qh + ((cb + 1) * nt + t) * N * N * V;
        for (int s = 0; s < N; s++) {
          for (int k = 0; k < V; k++) {
            double s0 = 0, s1 = 0;
            for (int m = 0; m < N; m++) {
              s0 += ENDVALS[1][m] * qh0[(s * N + m) * V + k];
              s1 += ENDVALS[0][m] * qhy[(s * N + m) * V + k];
            }
            q0[k] = s0;
            q1[k] = s1;
          }
          interface_D(FLUX, q0, q1, 1, P, f);
          or_Bint(q0, q1, 1, b);
          for (int k = 0; k < V; k++) {
            uy0[k] += yW[s] * (b[k] + f[k]);
            uy1[k] += yW[s] * (b[k] - f[k]);
          }
        }
      }
    }
    for (long c = 0; c < nfx; c++) {
      int i = (int)(c / (ny + 1)), j = (int)(c % (ny + 1));
      long cb = (long)i * (ny + 2) + j;
      if (!mask[cb])
        continue;
      const double *ux0 = fx + c * 4 * V, *ux1 = ux0 + V, *uy0 = ux1 + V, *uy1 = uy0 + V;
      long uind0 = ((long)(i - 1) * ny + (j - 1)) * V;
      if (mask[cb + (ny + 2)] && j > 0) {
        long uindx = ((long)i * ny + (j - 1)) * V;
        if (i > 0)
          for (int k = 0; k < V; k++)
            u[uind0 + k] -= ux0[k];
        if (i < nx)
          for (int k = 0; k < V; k++)
            u[uindx + k] -= ux1[k];
      }
      if (mask[cb + 1] && i > 0) {
        long uindy = ((long)(i - 1) * ny + j) * V;
        if (j > 0)
          for (int k = 0; k < V; k++)
            u[uind0 + k] -= uy0[k];
        if (j < ny)
          for (int k = 0; k < V; k++)
            u[uindy + k] -= uy1[k];
      }
    }
  }
  free(fx);
  return 0;
}

int or_fv_launcher(double *u, const double *qh, const int *nX, double dt,
                   const double *dX, int ndim, int SOURCES, int TIME, int FLUX,
                   const gpr_par *P, const uint8_t *mask) {
  return or_fv_parts(u, qh, nX, dt, dX, ndim, SOURCES, TIME, FLUX, P, mask, 3);
}

/* ------------------------------------------------------------------------ */
/* CFL time step, distortion housekeeping (solvers/iterator.cpp:54-83,    */
/* solvers/utils.cpp:6-23).                                                  */

double or_timestep(const double *u, long ncell, const double *dX, int ndim,
                   double CFL, double t, double tf, int count, const gpr_par *P) {
  double MAX = 0.0;
#pragma omp parallel for reduction(max : MAX) schedule(static)
  for (long c = 0; c < ncell; c++) {
    double tmp = 0.0;
    for (int d = 0; d < ndim; d++)
      tmp += or_max_abs_eigs(u + c * V, d, P) / dX[d];
    if (tmp > MAX) /* NaN cells are skipped, as std::max(MAX, NaN) does */
      MAX = tmp;
  }
  double dt = CFL / MAX;
  if (count <= 5)
    dt *= 0.2;
  if (t + dt > tf)
    return tf - t;
  return dt;
}

void or_renorm_distortion(double *u, long ncell, const gpr_par *P) {
#pragma omp parallel for schedule(static)
  for (long c = 0; c < ncell; c++) {
    double *Q = u + c * V;
    double r = Q[0];
    if (r > 0) {
      double cc = cbrt(r / (P->rho0 * det3(Q + 5)));
      for (int k = 5; k < 14; k++)
        Q[k] *= cc;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Split stiff-source ODE step (system/relaxation/analytic.cpp).           */

/* Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations: S = W D W^T
 * (columns of W are eigenvectors). */
static void jacobi3(double S[3][3], double Wm[3][3], double d[3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      Wm[i][j] = i == j;
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = fabs(S[0][1]) + fabs(S[0][2]) + fabs(S[1][2]);
    if (off == 0.0)
      break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (S[p][q] == 0.0)
          continue;
        double theta = (S[q][q] - S[p][p]) / (2 * S[p][q]);
        double t = (theta >= 0 ? 1 : -1) / (fabs(theta) + sqrt(theta * theta + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 3; k++) {
          double a = S[k][p], b = S[k][q];
          S[k][p] = c * a - s * b;
          S[k][q] = s * a + c * b;
        }
        for (int k = 0; k < 3; k++) {
          double a = S[p][k], b = S[q][k];
          S[p][k] = c * a - s * b;
          S[q][k] = s * a + c * b;
        }
        for (int k = 0; k < 3; k++) {
          double a = Wm[k][p], b = Wm[k][q];
          Wm[k][p] = c * a - s * b;
          Wm[k][q] = s * a + c * b;
        }
      }
  }
  for (int i = 0; i < 3; i++)
    d[i] = S[i][i];
}

/* SVD of a 3x3 (row-major) A = U diag(s) V^T, s descending, via the Jacobi
 * eigen-decomposition of A^T A; U = A V / s (re-orthogonalised). */
static void svd3(const double *A, double U[3][3], double s[3], double Vm[3][3]) {
  double S[3][3], W[3][3], d[3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      S[i][j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  jacobi3(S, W, d);
  int idx[3] = {0, 1, 2};
  for (int a = 0; a < 3; a++)
    for (int b = a + 1; b < 3; b++)
      if (d[idx[b]] > d[idx[a]]) {
        int t = idx[a];
        idx[a] = idx[b];
        idx[b] = t;
      }
  for (int c = 0; c < 3; c++) {
    s[c] = sqrt(fmax(d[idx[c]], 0.0));
    for (int r = 0; r < 3; r++)
      Vm[r][c] = W[r][idx[c]];
  }
  /* U columns: A v_c / s_c, Gram-Schmidt for stability */
  for (int c = 0; c < 3; c++) {
    double x[3];
    for (int r = 0; r < 3; r++)
      x[r] = A[3 * r] * Vm[0][c] + A[3 * r + 1] * Vm[1][c] + A[3 * r + 2] * Vm[2][c];
    for (int p = 0; p < c; p++) {
      double dp = x[0] * U[0][p] + x[1] * U[1][p] + x[2] * U[2][p];
      for (int r = 0; r < 3; r++)
        x[r] -= dp * U[r][p];
    }
    double nrm = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (int r = 0; r < 3; r++)
      U[r][c] = x[r] / nrm;
  }
}

static double posd(double x) { return x > 0 ? x : 0.0; }

/* nondimensionalized_time (analytic.cpp:17-69) */
static double nondim_time(double r, double detA3, double m0, double u0,
                          double dt, const gpr_par *P) {
  if (P->flags & GPR_POWER_LAW) {
    double n = P->n;
    double cs2 = c_s2(r, P);
    double a = 9. * m0 - u0 - 9.;
    double b = 6. * m0 - u0 - 6.;
    double c, lam, tmp1, tmp2;
    if (P->flags & GPR_SOLID) {
      c = (108. * a - 324. * b + 108. * a * a - 396. * a * b + 297. * b * b -
           24. * (a * a * b - 2. * a * b * b + b * b * b) - 4. * pow(a - b, 4.));
      if (c <= 0.)
        return 0.;
      lam = c / (18. * a - 36. * b + 9. * a * a - 132. / 5. * a * b +
                 33. / 2. * b * b - 8. / 7. * a * a * b + 2. * a * b * b -
                 8. / 9. * b * b * b - pow(a, 4.) / 6. + 16. / 27. * a * a * a * b -
                 4. / 5. * a * a * b * b + 16. / 33. * a * b * b * b - pow(b, 4.) / 9.);
      tmp1 = n * lam / P->tau0 * pow(detA3, 4. * n + 7.);
      tmp2 = pow(sqrt(c) * r * cs2 / (6. * P->sigmaY), n);
      return 2. / (n * lam) * log(tmp1 * tmp2 * dt + 1.);
    } else {
      double k = (1 - n) / n;
      c = (108. * a - 324. * b + 180. * a * a - 612. * a * b + 459. * b * b -
           24. * (a * a * b - 2. * a * b * b + b * b * b) - 4. * pow(a - b, 4.));
      if (c <= 0.)
        return 0.;
      lam = c / (18. * a - 36. * b + 15. * a * a - 204. / 5. * a * b +
                 51. / 2. * b * b - 8. / 7. * a * a * b + 2. * a * b * b -
                 8. / 9. * b * b * b - pow(a, 4.) / 6. + 16. / 27. * a * a * a * b -
                 4. / 5. * a * a * b * b + 16. / 33. * a * b * b * b - pow(b, 4.) / 9.);
      double tau1 = 6 * pow(P->mu, 1. / n) / (P->rho0 * P->b02);
      tmp1 = k * lam / tau1 * pow(detA3, 4. * k + 7.);
      tmp2 = pow(sqrt(c) * r * cs2 / (6. * sqrt(3.)), k);
      return 2. / (k * lam) * log(tmp1 * tmp2 * dt + 1.);
    }
  }
  return P->rho0 * P->b02 * pow(detA3, 7.) / (3. * P->mu) * dt;
}

/* analyticSolver_distortion (analytic.cpp:71-128) */
static void ode_distortion(double *Q, double dt, const gpr_par *P) {
  double *A = Q + 5;
  double U[3][3], s[3], Vm[3][3];
  svd3(A, U, s, Vm);
  double detA = s[0] * s[1] * s[2];
  double r = detA * P->rho0;
  double detA1_3 = cbrt(detA);
  double detA2_3 = detA1_3 * detA1_3;
  double s0 = s[0] * s[0] / detA2_3;
  double s1 = s[1] * s[1] / detA2_3;
  double s2 = s[2] * s[2] / detA2_3;
  double m0 = (s0 + s1 + s2) / 3.;
  double u0 = ((s0 - s1) * (s0 - s1) + (s1 - s2) * (s1 - s2) + (s2 - s0) * (s2 - s0)) / 3.;
  if (u0 < 1e-12)
    return;
  double tau = nondim_time(r, detA1_3, m0, u0, dt, P);
  double e6 = exp(-6. * tau), e9 = exp(-9. * tau);
  double a = 3. * m0 - u0 / 3. - 3.;
  double b = 2. * m0 - u0 / 3. - 2.;
  double m = 1. + a * e6 - b * e9;
  double u = posd(6. * a * e6 - 9. * b * e9);
  double Dl = -2. * m * m * m + m * u + 2.;
  double arg1 = posd(6. * u * u * u - 81. * Dl * Dl);
  double x1;
  if (fabs(Dl) < 1e-12)
    x1 = sqrt(6. * u) / 3. * cos(M_PI / 6.) + m;
  else if (arg1 == 0.) {
    double tmp = cbrt(54. * Dl);
    x1 = tmp / 6. + u / tmp + m;
  } else {
    double th = atan(sqrt(arg1) / (9. * Dl));
    x1 = sqrt(6. * u) / 3. * cos(th / 3.) + m;
  }
  double tmp2 = 3. * m - x1;
  double arg2 = posd(x1 * tmp2 * tmp2 - 4.);
  double x2 = 0.5 * (sqrt(arg2 / x1) + tmp2);
  double x3 = 1. / (x1 * x2);
  double x[3] = {x1, x2, x3};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (x[j] < x[i]) {
        double t = x[i];
        x[i] = x[j];
        x[j] = t;
      }
  /* A = U diag(detA^1/3 sqrt(x[2-i])) V^T */
  double sc[3];
  for (int i = 0; i < 3; i++)
    sc[i] = detA1_3 * sqrt(x[2 - i]);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double acc = 0.0;
      for (int k = 0; k < 3; k++)
        acc += U[i][k] * sc[k] * Vm[j][k];
      A[3 * i + j] = acc;
    }
}

/* analyticSolver_thermal (analytic.cpp:130-150) */
static void ode_thermal(double *Q, double dt, const gpr_par *P) {
  double r = Q[0];
  double E = Q[1] / r;
  double v0 = Q[2] / r, v1 = Q[3] / r, v2 = Q[4] / r;
  double c1 = E - E_2A(r, Q + 5, P) - (v0 * v0 + v1 * v1 + v2 * v2) / 2;
  double c2 = P->calpha2 / 2.;
  double k = 2 * P->calpha2 / (P->kappa * r * P->cv);
  c1 *= k;
  c2 *= k;
  double ea = exp(-c1 * dt / 2);
  double J2 = Q[14] * Q[14] + Q[15] * Q[15] + Q[16] * Q[16];
  double den = 1 - c2 / c1 * (1 - ea * ea) * J2 / (r * r);
  double f = ea / sqrt(den);
  Q[14] *= f;
  Q[15] *= f;
  Q[16] *= f;
}

void or_ode_cell(double *Q, double dt, const gpr_par *P) {
  Q[2] += P->dp[0] * dt;
  Q[3] += P->dp[1] * dt;
  Q[4] += P->dp[2] * dt;
  ode_distortion(Q, dt, P);
  if (THERMAL)
    ode_thermal(Q, dt, P);
}

void or_ode_launcher(double *u, long ncell, double dt, const gpr_par *P) {
#pragma omp parallel for schedule(static)
  for (long c = 0; c < ncell; c++)
    or_ode_cell(u + c * V, dt, P);
}

/* ------------------------------------------------------------------------ */
/* Steppers (solvers/steppers.cpp:10-66, split/homogeneous.cpp:5-67).       */

int or_ader_stepper(double *u, const double *ub, const int *nX, int ndim,
                    double dt, const double *dX, int stiff, int FLUX,
                    const gpr_par *P, const uint8_t *mask, int *status,
                    int newton_fallback) {
  long ncb = ndim == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
  int ns = ndim == 1 ? N : N * N;
  double *wh = malloc(sizeof(double) * ncb * ns * V);
  double *qh = malloc(sizeof(double) * ncb * N * ns * V);
  for (long k = 0; k < ncb * N * ns * V; k++)
    qh[k] = NAN;
  or_weno_launcher(wh, ub, nX, ndim);
  or_predictor(qh, wh, dt, dX, ndim, nX, stiff, P, mask, status, newton_fallback);
  or_fv_launcher(u, qh, nX, dt, dX, ndim, 1, 1, FLUX, P, mask);
  free(wh);
  free(qh);
  return 0;
}

/* midstepper (split/homogeneous.cpp:5-67) */
int or_midstepper(double *wh, double dt, const double *dX, int ndim,
                  const gpr_par *P, const uint8_t *mask, long ncell) {
  int ns = ndim == 1 ? N : N * N;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < ncell; c++) {
    if (!mask[c])
      continue;
    double *w = wh + c * ns * V;
    double F[MAXN * MAXN * MAXV], G[MAXN * MAXN * MAXV], dwx[MAXN * MAXN * MAXV],
        dwy[MAXN * MAXN * MAXV], dFx[MAXN * MAXN * MAXV], dGy[MAXN * MAXN * MAXV];
    memset(F, 0, sizeof F);
    memset(G, 0, sizeof G);
    for (int s = 0; s < ns; s++) {
      or_flux(w + s * V, 0, P, F + s * V);
      if (ndim == 2)
        or_flux(w + s * V, 1, P, G + s * V);
    }
    for (int s = 0; s < ns; s++) {
      int a = ndim == 1 ? s : s / N, b = ndim == 1 ? 0 : s % N;
      for (int k = 0; k < V; k++) {
        double sx = 0, sf = 0, sy = 0, sg = 0;
        for (int m = 0; m < N; m++) {
          int ix = ndim == 1 ? m : m * N + b;
          sx += DERVALS[a][m] * w[ix * V + k];
          sf += DERVALS[a][m] * F[ix * V + k];
          if (ndim == 2) {
            int iy = a * N + m;
            sy += DERVALS[b][m] * w[iy * V + k];
            sg += DERVALS[b][m] * G[iy * V + k];
          }
        }
        dwx[s * V + k] = sx;
        dFx[s * V + k] = sf;
        dwy[s * V + k] = sy;
        dGy[s * V + k] = sg;
      }
    }
    double Bx[MAXV], By[MAXV];
    for (int s = 0; s < ns; s++) {
      or_Bdot(w + s * V, dwx + s * V, 0, Bx);
      if (ndim == 2)
        or_Bdot(w + s * V, dwy + s * V, 1, By);
      for (int k = 0; k < V; k++) {
        double inc = (dFx[s * V + k] + Bx[k]) / dX[0];
        if (ndim == 2)
          inc += (dGy[s * V + k] + By[k]) / dX[1];
        w[s * V + k] -= dt / 2 * inc;
      }
    }
  }
  return 0;
}

/* split_stepper (steppers.cpp:50-66); ub is modified (ODE half step). */
int or_split_stepper(double *u, double *ub, const int *nX, int ndim, double dt,
                     const double *dX, int HALF_STEP, int FLUX, const gpr_par *P,
                     const uint8_t *mask) {
  long nc = ndim == 1 ? nX[0] : (long)nX[0] * nX[1];
  long ncb = ndim == 1 ? nX[0] + 2 : (long)(nX[0] + 2) * (nX[1] + 2);
  long nub = ndim == 1 ? nX[0] + 2 * N : (long)(nX[0] + 2 * N) * (nX[1] + 2 * N);
  int ns = ndim == 1 ? N : N * N;
  or_ode_launcher(u, nc, dt / 2, P);
  or_ode_launcher(ub, nub, dt / 2, P);
  double *wh = malloc(sizeof(double) * ncb * ns * V);
  or_weno_launcher(wh, ub, nX, ndim);
  if (HALF_STEP)
    or_midstepper(wh, dt, dX, ndim, P, mask, ncb);
  or_fv_launcher(u, wh, nX, dt, dX, ndim, 0, 0, FLUX, P, mask);
  or_ode_launcher(u, nc, dt / 2, P);
  free(wh);
  return 0;
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0)
    omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ======================================================================== */
/* Level-set ghost-fluid fill (LSET = 1, two materials, VISCOUS, no heat     */
/* conduction): multi/pfmm.cpp, multi/functions.cpp, multi/fill.cpp,        */
/* system/multi/{riemann,conditions,eigenvecs,rotations}.cpp and            */
/* solvers/iterator.cpp:12-42 (make_u).                                     */
/* ======================================================================== */

#include <float.h>

/* ---- first-order fast marching (the vendored scikit-fmm's
 * distance_marcher.cpp:5-28,72-151 and base_marcher.cpp:43-198 with
 * ORDER 1, no narrow band, not periodic; called by multi/pfmm.cpp:4-26). */

enum { FMM_FAR = 0, FMM_NARROW = 1, FMM_FROZEN = 2 };

typedef struct {
  int ndim, size, shape[2], shift[2];
  double dx[2], idx2[2];
  const double *phi;
  double *dist;
  unsigned char *flag;
  /* binary min-heap of grid addresses keyed by |distance| */
  int *heap, *pos, n;
  double *key;
} fmm_t;

static int fmm_nb(const fmm_t *m, int i, int dim, int dir) {
  int c = m->ndim == 1 ? i : (dim == 0 ? i / m->shape[1] : i % m->shape[1]);
  int nc = c + dir;
  if (nc < 0 || nc >= m->shape[dim])
    return -1;
  return i + dir * m->shift[dim];
}

static void fmm_swap(fmm_t *m, int a, int b) {
  int t = m->heap[a];
  m->heap[a] = m->heap[b];
  m->heap[b] = t;
  m->pos[m->heap[a]] = a;
  m->pos[m->heap[b]] = b;
}

static void fmm_up(fmm_t *m, int k) {
  while (k > 0) {
    int p = (k - 1) / 2;
    if (m->key[m->heap[p]] <= m->key[m->heap[k]])
      break;
    fmm_swap(m, p, k);
    k = p;
  }
}

static void fmm_down(fmm_t *m, int k) {
  for (;;) {
    int l = 2 * k + 1, r = l + 1, s = k;
    if (l < m->n && m->key[m->heap[l]] < m->key[m->heap[s]])
      s = l;
    if (r < m->n && m->key[m->heap[r]] < m->key[m->heap[s]])
      s = r;
    if (s == k)
      break;
    fmm_swap(m, s, k);
    k = s;
  }
}

static void fmm_push(fmm_t *m, int addr, double key) {
  m->key[addr] = key;
  m->heap[m->n] = addr;
  m->pos[addr] = m->n;
  m->n++;
  fmm_up(m, m->n - 1);
}

static void fmm_set(fmm_t *m, int addr, double key) {
  double old = m->key[addr];
  m->key[addr] = key;
  if (key < old)
    fmm_up(m, m->pos[addr]);
  else
    fmm_down(m, m->pos[addr]);
}

static int fmm_pop(fmm_t *m) {
  int top = m->heap[0];
  m->n--;
  if (m->n > 0) {
    m->heap[0] = m->heap[m->n];
    m->pos[m->heap[0]] = 0;
    fmm_down(m, 0);
  }
  m->pos[top] = -1;
  return top;
}

/* updatePointOrderOne + solveQuadratic (distance_marcher.cpp:5-28,72-88):
 * per axis the frozen neighbour of least |distance|, then the upwind
 * quadratic; the root is chosen by the sign of phi; 0 when it has no real
 * root.  The reference builds with -O3 -march=native (CMakeLists.txt:14),
 * where gcc fuses b -= idx2 2 value, c += idx2 value^2 and b^2 - 4ac into
 * fused multiply-adds; the explicit fma() calls below are that build's
 * roundings (its distances reproduced bit for bit on every test level set),
 * on any host and under any contraction setting.  The quadratic loses ~17
 * bits to cancellation, so these roundings show at ~1e-12. */
static double fmm_point(const fmm_t *m, int i) {
  double a = 0, b = 0, c = 0;
  for (int dim = 0; dim < m->ndim; dim++) {
    double value = DBL_MAX;
    for (int j = -1; j < 2; j += 2) {
      int n = fmm_nb(m, i, dim, j);
      if (n != -1 && m->flag[n] == FMM_FROZEN && fabs(m->dist[n]) < fabs(value))
        value = m->dist[n];
    }
    if (value < DBL_MAX) {
      a += m->idx2[dim];
      b = fma(-(m->idx2[dim] * 2), value, b);
      c = fma(m->idx2[dim], value * value, c);
    }
  }
  c -= 1;
  double det = fma(b, b, -(4 * a * c));
  if (!(det > 0))
    return 0;
  double r0 = (-b + sqrt(det)) / 2.0 / a;
  double r1 = (-b - sqrt(det)) / 2.0 / a;
  return m->phi[i] > DBL_EPSILON ? r0 : r1;
}

/* distance (multi/pfmm.cpp:4-26): signed first-order distance to the zero
 * level of phi on an nx (x ny) grid of spacings dX.  Returns 0, or 2 when
 * phi has no zero crossing (dist is then all zeros, as in the reference). */
int or_distance(const double *phi, const double *dX, const int *nX, int ndim,
                double *dist) {
  fmm_t m;
  memset(&m, 0, sizeof m);
  m.ndim = ndim;
  m.size = 1;
  for (int d = 0; d < ndim; d++) {
    m.shape[d] = nX[d];
    m.size *= nX[d];
    m.dx[d] = dX[d];
    m.idx2[d] = 1 / dX[d] / dX[d];
  }
  m.shift[0] = ndim == 2 ? nX[1] : 1;
  m.shift[1] = 1;
  m.phi = phi;
  m.dist = dist;
  int size = m.size;
  m.flag = calloc(size, 1);
  m.heap = malloc(sizeof(int) * size);
  m.pos = malloc(sizeof(int) * size);
  m.key = malloc(sizeof(double) * size);
  for (int i = 0; i < size; i++)
    dist[i] = 0.0;

  /* initalizeFrozen (distance_marcher.cpp:90-151, with the reference's
   * edit: the least per-axis crossing distance, not their harmonic sum) */
  for (int i = 0; i < size; i++)
    if (phi[i] == 0.0) {
      m.flag[i] = FMM_FROZEN;
      dist[i] = 0.0;
    }
  for (int i = 0; i < size; i++) {
    if (m.flag[i] != FMM_FAR)
      continue;
    double ld[2] = {0, 0};
    int borders = 0;
    for (int dim = 0; dim < ndim; dim++)
      for (int j = -1; j < 2; j += 2) {
        int n = fmm_nb(&m, i, dim, j);
        if (n != -1 && phi[i] * phi[n] < 0) {
          borders = 1;
          double d = m.dx[dim] * phi[i] / (phi[i] - phi[n]);
          if (ld[dim] == 0 || ld[dim] > d)
            ld[dim] = d;
        }
      }
    if (borders) {
      double minDist = DBL_MAX;
      for (int dim = 0; dim < ndim; dim++) {
        double t = fabs(ld[dim]);
        if (t > 0.)
          minDist = t < minDist ? t : minDist;
      }
      dist[i] = phi[i] < 0 ? -minDist : minDist;
      m.flag[i] = FMM_FROZEN;
    }
  }

  /* initalizeNarrow (base_marcher.cpp:62-87) */
  int nfrozen = 0;
  for (int i = 0; i < size; i++)
    nfrozen += m.flag[i] == FMM_FROZEN;
  for (int i = 0; i < size; i++) {
    if (m.flag[i] != FMM_FAR)
      continue;
    int touch = 0;
    for (int dim = 0; dim < ndim && !touch; dim++)
      for (int j = -1; j < 2; j += 2) {
        int n = fmm_nb(&m, i, dim, j);
        if (n != -1 && m.flag[n] == FMM_FROZEN)
          touch = 1;
      }
    if (touch) {
      m.flag[i] = FMM_NARROW;
      double d = fmm_point(&m, i);
      dist[i] = d;
      fmm_push(&m, i, fabs(d));
    }
  }
  int rc = 0;
  if (!nfrozen) {
    rc = 2; /* base_marcher.cpp:103-106: nothing to march from */
  } else {
    /* main loop (base_marcher.cpp:98-188): freeze the least |distance| and
     * every equal key with it, then update their unfrozen neighbours */
    int *batch = malloc(sizeof(int) * size);
    while (m.n > 0) {
      int nb = 0;
      int addr = fmm_pop(&m);
      double value = m.key[addr];
      m.flag[addr] = FMM_FROZEN;
      batch[nb++] = addr;
      while (m.n > 0 && m.key[m.heap[0]] == value) {
        int a2 = fmm_pop(&m);
        m.flag[a2] = FMM_FROZEN;
        batch[nb++] = a2;
      }
      for (int k = 0; k < nb; k++) {
        int a = batch[k];
        for (int dim = 0; dim < ndim; dim++)
          for (int j = -1; j < 2; j += 2) {
            int n = fmm_nb(&m, a, dim, j);
            if (n == -1 || m.flag[n] == FMM_FROZEN)
              continue;
            double d = fmm_point(&m, n);
            if (!d)
              continue;
            dist[n] = d;
            if (m.flag[n] == FMM_NARROW) {
              fmm_set(&m, n, fabs(d));
            } else {
              m.flag[n] = FMM_NARROW;
              fmm_push(&m, n, fabs(d));
            }
          }
      }
    }
    free(batch);
    for (int i = 0; i < size; i++)
      if (m.flag[i] != FMM_FROZEN)
        dist[i] = DBL_MAX;
  }
  free(m.flag);
  free(m.heap);
  free(m.pos);
  free(m.key);
  return rc;
}

/* ---- multi/functions.cpp ---- */

static int ls_sign(double x) { return x <= 0 ? -1 : 1; } /* functions.cpp:7-12 */

/* finite_difference (functions.cpp:16-54): central differences, edge rows
 * copied from their neighbours; dphi is [ncell][ndim]. */
void or_finite_difference(const double *phi, const double *dX, const int *nX,
                          int ndim, double *dphi) {
  if (ndim == 1) {
    int n = nX[0];
    for (int i = 1; i < n - 1; i++)
      dphi[i] = (phi[i + 1] - phi[i - 1]) / (2 * dX[0]);
    dphi[0] = dphi[1];
    dphi[n - 1] = dphi[n - 2];
    return;
  }
  int nx = nX[0], ny = nX[1];
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      int ii = i == 0 ? 1 : (i == nx - 1 ? nx - 2 : i);
      int jj = j == 0 ? 1 : (j == ny - 1 ? ny - 2 : j);
      dphi[2 * (i * ny + j)] =
          (phi[(ii + 1) * ny + j] - phi[(ii - 1) * ny + j]) / (2 * dX[0]);
      dphi[2 * (i * ny + j) + 1] =
          (phi[i * ny + jj + 1] - phi[i * ny + jj - 1]) / (2 * dX[1]);
    }
}

/* find_interface_cells (fill.cpp:11-74): intMask = sign(phi) on both sides
 * of every crossing next to a non-isolated phi <= 0 cell; -2 marks an
 * isolated phi <= 0 cell (2D). */
void or_find_interface_cells(const double *phi, const int *nX, int ndim,
                             int32_t *mask) {
  int nx = nX[0];
  if (ndim == 1) {
    for (int i = 0; i < nx; i++)
      mask[i] = 0;
    for (int i = 0; i < nx - 1; i++)
      if (phi[i] * phi[i + 1] <= 0.) {
        mask[i] = ls_sign(phi[i]);
        mask[i + 1] = ls_sign(phi[i + 1]);
      }
    return;
  }
  int ny = nX[1];
  for (int k = 0; k < nx * ny; k++)
    mask[k] = 0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      int k0 = i * ny + j;
      if (!(phi[k0] <= 0.))
        continue;
      int cl = i > 0 && phi[k0 - ny] <= 0., cr = i < nx - 1 && phi[k0 + ny] <= 0.;
      int cd = j > 0 && phi[k0 - 1] <= 0., cu = j < ny - 1 && phi[k0 + 1] <= 0.;
      if (cl || cr || cd || cu) {
        int nbr[4] = {i > 0 ? k0 - ny : -1, i < nx - 1 ? k0 + ny : -1,
                      j > 0 ? k0 - 1 : -1, j < ny - 1 ? k0 + 1 : -1};
        for (int q = 0; q < 4; q++)
          if (nbr[q] >= 0 && phi[k0] * phi[nbr[q]] <= 0.) {
            mask[k0] = ls_sign(phi[k0]);
            mask[nbr[q]] = ls_sign(phi[nbr[q]]);
          }
      } else {
        mask[k0] = -2;
      }
    }
}

/* ---- system/multi: the interface Riemann problem (non-thermal, slip) ---- */

/* rotation_matrix (rotations.cpp:5-35): rows e1 = n, e2, e3. */
static void ls_rotation(const double *n, int ndim, double R[3][3]) {
  double e1[3] = {0, 0, 0}, e2[3], e3[3], den;
  for (int i = 0; i < ndim; i++)
    e1[i] = n[i];
  double Sq = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  if (fabs(e1[1] + e1[2]) <= fabs(e1[1] - e1[2])) {
    den = sqrt(2 * (1 - e1[0] * e1[1] - e1[1] * e1[2] - e1[2] * e1[0]));
    e2[0] = e1[1] - e1[2];
    e2[1] = e1[2] - e1[0];
    e2[2] = e1[0] - e1[1];
    double Sum = e1[0] + e1[1] + e1[2];
    for (int i = 0; i < 3; i++)
      e3[i] = e1[i] * Sum - Sq;
  } else {
    den = sqrt(2 * (1 + e1[0] * e1[1] + e1[1] * e1[2] - e1[2] * e1[0]));
    e2[0] = e1[1] + e1[2];
    e2[1] = e1[2] - e1[0];
    e2[2] = -e1[0] - e1[1];
    double Sum = e1[0] - e1[1] + e1[2];
    e3[0] = e1[0] * Sum - Sq;
    e3[1] = e1[1] * Sum + Sq;
    e3[2] = e1[2] * Sum - Sq;
  }
  for (int i = 0; i < 3; i++) {
    R[0][i] = e1[i];
    R[1][i] = e2[i] / den;
    R[2][i] = e3[i] / den;
  }
}

/* rotate_tensors (rotations.cpp:37-47): v <- R v, A <- R A R^T. */
static void ls_rotate(double *Q, double R[3][3]) {
  double v[3], A[9], T[9];
  for (int i = 0; i < 3; i++)
    v[i] = R[i][0] * Q[2] + R[i][1] * Q[3] + R[i][2] * Q[4];
  for (int i = 0; i < 3; i++)
    Q[2 + i] = v[i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      T[3 * i + j] = R[i][0] * Q[5 + j] + R[i][1] * Q[8 + j] + R[i][2] * Q[11 + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      A[3 * i + j] = T[3 * i] * R[j][0] + T[3 * i + 1] * R[j][1] + T[3 * i + 2] * R[j][2];
  for (int k = 0; k < 9; k++)
    Q[5 + k] = A[k];
  if (THERMAL) {
    for (int i = 0; i < 3; i++)
      v[i] = R[i][0] * Q[14] + R[i][1] * Q[15] + R[i][2] * Q[16];
    for (int i = 0; i < 3; i++)
      Q[14 + i] = v[i];
  }
}

/* Total stress column 0: Sigma = p e0 - sigma(:,0) (variables/state.cpp:39-46) */
static void ls_Sigma0(const double *Q, const gpr_par *P, double *S) {
  sigma_d(Q, P, 0, S);
  for (int i = 0; i < 3; i++)
    S[i] = -S[i];
  S[0] += or_pressure(Q, P);
}

/* c_0 (waves/speeds.cpp:8-18) */
static double ls_c0(const double *Q, double p, const gpr_par *P) {
  double r = Q[0];
  double dEdr = dedrho(r, p, P) + dC_0drho(r, P) / 4 * devGsq(Q + 5);
  return sqrt((p / (r * r) - dEdr) / dedp(r, P));
}

/* Gaussian elimination with partial pivoting: solves A X = B in place
 * (A n x n, B n x m, both row-major). */
static int ls_solve(int n, int m, double *A, double *B) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(A[r * n + c]) > fabs(A[p * n + c]))
        p = r;
    if (A[p * n + c] == 0.0)
      return -1;
    if (p != c) {
      for (int j = 0; j < n; j++) {
        double t = A[c * n + j];
        A[c * n + j] = A[p * n + j];
        A[p * n + j] = t;
      }
      for (int j = 0; j < m; j++) {
        double t = B[c * m + j];
        B[c * m + j] = B[p * m + j];
        B[p * m + j] = t;
      }
    }
    for (int r = c + 1; r < n; r++) {
      double f = A[r * n + c] / A[c * n + c];
      for (int j = c; j < n; j++)
        A[r * n + j] -= f * A[c * n + j];
      for (int j = 0; j < m; j++)
        B[r * m + j] -= f * B[c * m + j];
    }
  }
  for (int c = n - 1; c >= 0; c--)
    for (int j = 0; j < m; j++) {
      double s = B[c * m + j];
      for (int k = c + 1; k < n; k++)
        s -= A[c * n + k] * B[k * m + j];
      B[c * m + j] = s / A[c * n + c];
    }
  return 0;
}

static int ls_inverse(int n, const double *M, double *out) {
  double A[25];
  memcpy(A, M, sizeof(double) * n * n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      out[i * n + j] = i == j;
  return ls_solve(n, n, A, out);
}

/* Inverse principal square root of a matrix with positive real eigenvalues
 * by the Denman-Beavers iteration (Y -> M^(1/2), Z -> M^(-1/2)).  The
 * reference forms the same matrix function from an eigen-decomposition,
 * Q diag(lambda^(-1/2)) Q^(-1) (riemann.cpp:141-146). */
static int ls_inv_sqrt(int n, const double *M, double *Zout) {
  double Y[16], Z[16], Yi[16], Zi[16];
  memcpy(Y, M, sizeof(double) * n * n);
  for (int i = 0; i < n * n; i++)
    Z[i] = (i % (n + 1)) == 0;
  int extra = 0;
  for (int it = 0; it < 100; it++) {
    if (ls_inverse(n, Y, Yi) || ls_inverse(n, Z, Zi))
      return -1;
    double dmax = 0, ymax = 0;
    for (int k = 0; k < n * n; k++) {
      double y = 0.5 * (Y[k] + Zi[k]);
      double z = 0.5 * (Z[k] + Yi[k]);
      double dy = fabs(y - Y[k]);
      dmax = dy > dmax ? dy : dmax;
      ymax = fabs(y) > ymax ? fabs(y) : ymax;
      Y[k] = y;
      Z[k] = z;
    }
    if (dmax <= 1e-13 * ymax && ++extra == 2)
      break;
  }
  memcpy(Zout, Z, sizeof(double) * n * n);
  return 0;
}

/* The first n1 = 3 columns of riemann_constraints (riemann.cpp:79-154) for
 * the non-thermal system: rows 0-4 are X (the primitive-variable response
 * to a change in the normal traction), rows 11-13 are -sgn Y0 Xi1 X; every
 * other entry of those columns is zero.  The remaining columns of the
 * reference's matrix multiply zero coefficients in star_stepper and are
 * not formed.  R is [V][3]. */
static int ls_constraints(const double *Q, double sgn, const gpr_par *P, double *R) {
  double r = Q[0];
  double p = or_pressure(Q, P);
  const double *A = Q + 5;
  double sr[3], Pi1[9], Pi1i[9], Ai[9], sg[3];
  dsigmadrho(Q, P, 0, sr);
  dsigmadA(Q, P, 0, Pi1);
  sigma_d(Q, P, 0, sg);
  if (ls_inverse(3, A, Ai) || ls_inverse(3, Pi1, Pi1i))
    return -1;
  double tmp[25];
  memset(tmp, 0, sizeof tmp);
  for (int i = 0; i < 3; i++) {
    tmp[5 * i] = -sr[i];
    for (int j = 0; j < 3; j++)
      tmp[5 * i + 2 + j] = -Pi1[3 * i + j];
  }
  tmp[1] = 1.;
  double c0 = ls_c0(Q, p, P);
  double B[6] = {r, 0, 0, 0, 0, 0};
  for (int j = 0; j < 3; j++)
    B[3 + j] = sg[j] - r * sr[j];
  B[3] += r * c0 * c0;
  double C[6]; /* Pi1^-1 [-sr, e0] (3x2) */
  for (int i = 0; i < 3; i++) {
    C[2 * i] = -(Pi1i[3 * i] * sr[0] + Pi1i[3 * i + 1] * sr[1] + Pi1i[3 * i + 2] * sr[2]);
    C[2 * i + 1] = Pi1i[3 * i];
  }
  double BA[6]; /* B A^-1 (2x3) */
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 3; j++)
      BA[3 * i + j] = B[3 * i] * Ai[j] + B[3 * i + 1] * Ai[3 + j] + B[3 * i + 2] * Ai[6 + j];
  double Z[4];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      Z[2 * i + j] = (i == j) - (BA[3 * i] * C[j] + BA[3 * i + 1] * C[2 + j] +
                                 BA[3 * i + 2] * C[4 + j]);
  double dz = Z[0] * Z[3] - Z[1] * Z[2];
  if (dz == 0.0)
    return -1;
  double Zi[4] = {Z[3] / dz, -Z[1] / dz, -Z[2] / dz, Z[0] / dz};
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 5; j++) {
      double w0 = j == 0 ? 1 : (j == 1 ? 0 : -BA[j - 2]);
      double w1 = j == 0 ? 0 : (j == 1 ? 1 : -BA[3 + j - 2]);
      tmp[5 * (3 + i) + j] = Zi[2 * i] * w0 + Zi[2 * i + 1] * w1;
    }
  double X[15]; /* tmp^-1 [:, 0:3] */
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 3; j++)
      X[3 * i + j] = i == j;
  if (ls_solve(5, 3, tmp, X))
    return -1;
  /* Xi1 (3x5), Xi2 (5x3) of eig.cpp:8-53 at d = 0 */
  double X1[15], X2[15], Xi[9], Y0[9];
  memset(X1, 0, sizeof X1);
  memset(X2, 0, sizeof X2);
  X1[1] = 1 / r;
  for (int i = 0; i < 3; i++) {
    X1[5 * i] = -1 / r * sr[i];
    for (int j = 0; j < 3; j++)
      X1[5 * i + 2 + j] = -1 / r * Pi1[3 * i + j];
  }
  X2[0] = r;
  X2[3] = r * c0 * c0;
  for (int j = 0; j < 3; j++)
    X2[3 + j] += sg[j] - r * sr[j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      X2[3 * (2 + i) + j] = A[3 * i + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 5; k++)
        s += X1[5 * i + k] * X2[3 * k + j];
      Xi[3 * i + j] = s;
    }
  /* The reference's Q diag(Re(lambda)^(-1/2)) Q^(-1) with Q = Re(eigenvectors)
   * (riemann.cpp:136-141) is NaN when an eigenvalue has a non-positive real
   * part, and singular for a complex pair (the real parts of conjugate
   * eigenvectors coincide); left_star_state then returns its input.  A pair
   * counts as complex when its imaginary part exceeds 1e-6 of the spectral
   * radius: a double eigenvalue (an isotropic distortion) splits by about
   * sqrt(eps) under rounding, and there the reference's choice is decided
   * by rounding alone. */
  {
    double wr[3], wi[3];
    if (or_eigenvalues(3, Xi, wr, wi))
      return -1;
    double rad = 0;
    for (int i = 0; i < 3; i++)
      rad = fmax(rad, hypot(wr[i], wi[i]));
    for (int i = 0; i < 3; i++)
      if (!(wr[i] > 0) || fabs(wi[i]) > 1e-6 * rad)
        return -1;
  }
  if (ls_inv_sqrt(3, Xi, Y0))
    return -1;
  double X1X[9], YX[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 5; k++)
        s += X1[5 * i + k] * X[3 * k + j];
      X1X[3 * i + j] = s;
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      YX[3 * i + j] = Y0[3 * i] * X1X[j] + Y0[3 * i + 1] * X1X[3 + j] +
                      Y0[3 * i + 2] * X1X[6 + j];
  memset(R, 0, sizeof(double) * V * 3);
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 3; j++)
      R[3 * i + j] = X[3 * i + j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      R[3 * (11 + i) + j] = -sgn * YX[3 * i + j];
  return 0;
}

/* Cvec_to_Pvec / Pvec_to_Cvec (functions/vectors.cpp:85-154), non-thermal:
 * P = [rho, p, A(:,0), A(:,1), A(:,2), v, phi]. */
static void ls_c2p(const double *Q, const gpr_par *P, double *out) {
  double r = Q[0];
  memcpy(out, Q, sizeof(double) * V);
  out[1] = or_pressure(Q, P);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      out[2 + 3 * j + i] = Q[5 + 3 * i + j];
  for (int i = 0; i < 3; i++)
    out[11 + i] = Q[2 + i] / r;
}

static void ls_p2c(const double *Pv, const gpr_par *P, double *Q) {
  double r = Pv[0], p = Pv[1], A[9], v[3];
  memcpy(Q, Pv, sizeof(double) * V);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      A[3 * i + j] = Pv[2 + 3 * j + i];
  for (int i = 0; i < 3; i++)
    v[i] = Pv[11 + i];
  for (int i = 0; i < 3; i++)
    Q[2 + i] = r * v[i];
  for (int k = 0; k < 9; k++)
    Q[5 + k] = A[k];
  /* total_energy (energy/eos.cpp:43-47) with E_1 (eos.cpp:10-19) */
  double G = Gamma_MG(r, P);
  double E = e_ref(r, P) + (p - p_ref(r, P)) / (r * G);
  E += (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 2;
  E += E_2A(r, A, P);
  Q[1] = r * E;
}

static const double STAR_TOL = 1e-8; /* options.h:22 */

/* check_star_convergence (riemann.cpp:26-77), slip conditions. */
static int ls_converged(const double *QL, const double *QR, const gpr_par *PL,
                        const gpr_par *PR) {
  double SL[3];
  ls_Sigma0(QL, PL, SL);
  if (PR->EOS > -1) {
    double r0 = PL->rho0 < PR->rho0 ? PL->rho0 : PR->rho0;
    double b02 = PL->b02 < PR->b02 ? PL->b02 : PR->b02;
    double SR[3];
    ls_Sigma0(QR, PR, SR);
    double vL = QL[2] / QL[0], vR = QR[2] / QR[0];
    return fabs(SL[0] - SR[0]) / (b02 * r0) < STAR_TOL &&
           fabs(vL - vR) / sqrt(b02) < STAR_TOL;
  }
  double mx = fabs(SL[0]);
  for (int i = 1; i < 3; i++)
    mx = fabs(SL[i]) > mx ? fabs(SL[i]) : mx;
  return mx / (PL->b02 * PL->rho0) < STAR_TOL;
}

/* star_stepper (riemann.cpp:156-201) with slip_bcs (conditions.cpp:31-64). */
static int ls_star_step(double *QL, double *QR, const gpr_par *PL, const gpr_par *PR) {
  double RL[MAXV * 3], RR[MAXV * 3], xL[3], xR[3], cL[3], cR[3], Pv[MAXV];
  if (ls_constraints(QL, 1, PL, RL))
    return -1;
  ls_Sigma0(QL, PL, xL);
  if (PR->EOS > -1) {
    if (ls_constraints(QR, -1, PR, RR))
      return -1;
    ls_Sigma0(QR, PR, xR);
    double yL = QL[2] / QL[0], yR = QR[2] / QR[0];
    double dL = RL[33] * xL[0] + RL[34] * xL[1] + RL[35] * xL[2];
    double dR = RR[33] * xR[0] + RR[34] * xR[1] + RR[35] * xR[2];
    double x0 = (yR - yL + dL - dR) / (RL[33] - RR[33]);
    double x_[3] = {x0, 0., 0.};
    for (int i = 0; i < 3; i++) {
      cL[i] = x_[i] - xL[i];
      cR[i] = x_[i] - xR[i];
    }
    ls_c2p(QR, PR, Pv);
    for (int k = 0; k < V; k++)
      Pv[k] += RR[3 * k] * cR[0] + RR[3 * k + 1] * cR[1] + RR[3 * k + 2] * cR[2];
    ls_p2c(Pv, PR, QR);
  } else {
    for (int i = 0; i < 3; i++)
      cL[i] = -xL[i];
    for (int k = 0; k < V; k++)
      QR[k] = 0.0;
  }
  ls_c2p(QL, PL, Pv);
  for (int k = 0; k < V; k++)
    Pv[k] += RL[3 * k] * cL[0] + RL[3 * k + 1] * cL[1] + RL[3 * k + 2] * cL[2];
  ls_p2c(Pv, PL, QL);
  return 0;
}

/* left_star_state (riemann.cpp:203-233): the left star state of the
 * interface Riemann problem between QL (material PL) and QR (material PR)
 * along the normal n, by at most 10 linearised steps with a half-step of
 * the stiff relaxation before each.  Returns QL unchanged when the
 * iteration produced a NaN.  THERMAL must be off. */
int or_left_star_state(const double *QL0, const double *QR0, const gpr_par *PL,
                       const gpr_par *PR, double dt, const double *n, int ndim,
                       double *out) {
  if (THERMAL)
    return -3;
  double QL[MAXV], QR[MAXV], R[3][3];
  memcpy(QL, QL0, sizeof(double) * V);
  memcpy(QR, QR0, sizeof(double) * V);
  ls_rotation(n, ndim, R);
  ls_rotate(QL, R);
  ls_rotate(QR, R);
  int count = 0;
  while (!ls_converged(QL, QR, PL, PR) && count < 10) {
    or_ode_cell(QL, dt / 2, PL);
    if (PR->EOS > -1)
      or_ode_cell(QR, dt / 2, PR);
    if (ls_star_step(QL, QR, PL, PR)) {
      QL[0] = NAN;
      break;
    }
    count++;
  }
  for (int k = 0; k < V; k++)
    if (isnan(QL[k])) {
      memcpy(out, QL0, sizeof(double) * V);
      return count;
    }
  double RT[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      RT[i][j] = R[j][i];
  ls_rotate(QL, RT);
  memcpy(out, QL, sizeof(double) * V);
  return count;
}

/* ---- multi/fill.cpp ---- */

static int ls_mat(const double *Q) { return Q[V - 1] >= 0. ? 1 : 0; } /* vectors.cpp:24-31 */

/* boundary_inds (fill.cpp:96-132): cell indices (not offsets) of the cell
 * itself, of the interface point and of the probes one cell either side. */
static void ls_bound_inds(const int *inds, double phii, const double *n, const double *dX,
                          const int *nX, int ndim, int *ind, int *interf, int *L, int *Rr) {
  int vi[2], vl[2], vr[2];
  for (int d = 0; d < ndim; d++) {
    double xp = (inds[d] + 0.5) * dX[d];
    double xi = xp - phii * n[d];
    double xl = xi - 1. * dX[d] * n[d];
    double xr = xi + 1. * dX[d] * n[d];
    vi[d] = (int)(xi / dX[d]);
    vl[d] = (int)(xl / dX[d]);
    vr[d] = (int)(xr / dX[d]);
  }
  if (ndim == 1) {
    *ind = inds[0];
    *interf = vi[0];
    *L = vl[0];
    *Rr = vr[0];
  } else {
    int ny = nX[1];
    *ind = inds[0] * ny + inds[1];
    *interf = vi[0] * ny + vi[1];
    *L = vl[0] * ny + vl[1];
    *Rr = vr[0] * ny + vr[1];
  }
}

static int ls_neighbor_index(const int32_t *mask, int i, int j, int nx, int ny, int N0) {
  int indn = -1;
  if (i > 0 && mask[(i - 1) * ny + j] == N0)
    indn = (i - 1) * ny + j;
  if (i < nx - 1 && mask[(i + 1) * ny + j] == N0)
    indn = (i + 1) * ny + j;
  if (j > 0 && mask[i * ny + j - 1] == N0)
    indn = i * ny + j - 1;
  if (j < ny - 1 && mask[i * ny + j + 1] == N0)
    indn = i * ny + j + 1;
  return indn;
}

/* fill_boundary_inner (fill.cpp:134-198).  Returns -1 when the reference
 * would read outside the grid. */
static int ls_fill_boundary_inner(double *grid, const int *inds, const double *dX,
                                  const int *nX, int ndim, double phii, int mat,
                                  const gpr_par *MPs, double dt, double *n, int indn) {
  long ncell = ndim == 1 ? nX[0] : (long)nX[0] * nX[1];
  int ind, interf, L, Rr;
  ls_bound_inds(inds, phii, n, dX, nX, ndim, &ind, &interf, &L, &Rr);
  if (interf < 0 || interf >= ncell || L < 0 || L >= ncell || Rr < 0 || Rr >= ncell)
    return -1;
  double QL[MAXV], QR[MAXV], out[MAXV];
  memcpy(QR, grid + (long)Rr * V, sizeof(double) * V);
  int miR = ls_mat(QR);
  if (ls_mat(grid + (long)interf * V) == mat) {
    memcpy(QL, grid + (long)interf * V, sizeof(double) * V);
  } else if (ls_mat(grid + (long)L * V) == mat) {
    memcpy(QL, grid + (long)L * V, sizeof(double) * V);
  } else {
    if (ndim == 1)
      return -1;
    int Li[2] = {inds[0], inds[1]}, Lind;
    int n0 = (n[0] > 0) - (n[0] < 0), n1 = (n[1] > 0) - (n[1] < 0);
    int ny = nX[1];
    if (fabs(n[0]) > fabs(n[1])) {
      Li[0] -= n0;
      Lind = Li[0] * ny + Li[1];
      if (Lind >= 0 && Lind < ncell && ls_mat(grid + (long)Lind * V) == mat) {
        n[0] = n0;
        n[1] = 0.;
      } else {
        Li[0] += n0;
        Li[1] -= n1;
        Lind = Li[0] * ny + Li[1];
        n[0] = 0.;
        n[1] = n1;
      }
    } else {
      Li[1] -= n1;
      Lind = Li[0] * ny + Li[1];
      if (Lind >= 0 && Lind < ncell && ls_mat(grid + (long)Lind * V) == mat) {
        n[0] = 0.;
        n[1] = n1;
      } else {
        Li[0] -= n0;
        Li[1] += n1;
        Lind = Li[0] * ny + Li[1];
        n[0] = n0;
        n[1] = 0.;
      }
    }
    if (Lind < 0 || Lind >= ncell)
      return -1;
    if (ls_mat(grid + (long)Lind * V) == mat)
      memcpy(QL, grid + (long)Lind * V, sizeof(double) * V);
    else if (indn >= 0)
      memcpy(QL, grid + (long)indn * V, sizeof(double) * V);
    else
      return -1;
  }
  or_left_star_state(QL, QR, MPs + mat, MPs + miR, dt, n, ndim, out);
  memcpy(grid + (long)ind * V, out, sizeof(double) * (V - LSET));
  if (ls_mat(grid + (long)interf * V) != mat)
    memcpy(grid + (long)interf * V, out, sizeof(double) * (V - LSET));
  return 0;
}

/* normal (multi/functions.cpp:14); returns 0 when it is not finite (a zero
 * gradient), where the reference would truncate NaN positions to indices. */
static int ls_normal(const double *g, int ndim, double *n) {
  double s = 0;
  for (int d = 0; d < ndim; d++)
    s += g[d] * g[d];
  s = sqrt(s);
  int ok = 1;
  for (int d = 0; d < ndim; d++) {
    n[d] = g[d] / s;
    ok = ok && isfinite(n[d]);
  }
  return ok;
}

/* fill_boundary_cells (fill.cpp:200-235), in the reference's sequential
 * (i, j) order. */
int or_fill_boundary_cells(double *grid, const int32_t *mask, int mat, const double *phi,
                           const double *dphi, const double *dX, const gpr_par *MPs,
                           double dt, const int *nX, int ndim) {
  int nx = nX[0], ny = ndim == 2 ? nX[1] : 1, bad = 0;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      int ind = i * ny + j;
      if (mask[ind] != 1)
        continue;
      int indn = ndim == 2 ? ls_neighbor_index(mask, i, j, nx, ny, -1) : -1;
      double n[2];
      int inds[2] = {i, j};
      if (!ls_normal(dphi + (long)ind * ndim, ndim, n) ||
          ls_fill_boundary_inner(grid, inds, dX, nX, ndim, phi[ind], mat, MPs, dt, n, indn))
        bad++;
    }
  return bad;
}

/* fill_neighbor_inner / fill_neighbor_cells (fill.cpp:237-328): layers
 * N0 = 1 .. 10N-1 grow outwards from the boundary cells; each new cell
 * copies the cell one step towards the interface along the normal if that
 * one is already filled, else the layer neighbour it was reached from. */
static int ls_fill_neighbor_inner(double *grid, const double *g, const int *inds,
                                  const double *dX, const int *nX, int ndim,
                                  const int32_t *mask, int indn) {
  double n[2];
  int finite = ls_normal(g, ndim, n);
  int ni[2] = {0, 0};
  for (int d = 0; d < ndim && finite; d++) {
    double x = (inds[d] + 0.5) * dX[d];
    double xn = x - dX[d] * n[d];
    ni[d] = (int)(xn / dX[d]);
  }
  int ind = ndim == 1 ? inds[0] : inds[0] * nX[1] + inds[1];
  int nind = ndim == 1 ? ni[0] : ni[0] * nX[1] + ni[1];
  long ncell = ndim == 1 ? nX[0] : (long)nX[0] * nX[1];
  /* one cell past the last row: the reference reads outside its mask */
  int off = !finite || nind < 0 || nind >= ncell;
  if (off || mask[nind] < 1)
    nind = indn;
  memcpy(grid + (long)ind * V, grid + (long)nind * V, sizeof(double) * (V - LSET));
  return off ? -1 : 0;
}

int or_fill_neighbor_cells(double *grid, int32_t *mask, const double *dphi,
                           const double *dX, const int *nX, int ndim) {
  int nx = nX[0], bad = 0;
  int *isolates = ndim == 2 ? malloc(sizeof(int) * (long)nx * nX[1]) : NULL;
  for (int N0 = 1; N0 < 10 * N; N0++) {
    if (ndim == 1) {
      for (int i = 0; i < nx; i++) {
        if (mask[i] != 0)
          continue;
        int indn = -1;
        if (i > 0 && mask[i - 1] == N0)
          indn = i - 1;
        if (i < nx - 1 && mask[i + 1] == N0)
          indn = i + 1;
        if (indn > -1) {
          mask[i] = N0 + 1;
          int inds[1] = {i};
          bad += ls_fill_neighbor_inner(grid, dphi + i, inds, dX, nX, 1, mask, indn) != 0;
        }
      }
    } else {
      int ny = nX[1], niso = 0;
      for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
          int ind = i * ny + j;
          if (mask[ind] != 0 && mask[ind] != -2)
            continue;
          int indn = ls_neighbor_index(mask, i, j, nx, ny, N0);
          if (indn > -1) {
            if (mask[ind] == -2)
              isolates[niso++] = ind;
            mask[ind] = N0 + 1;
            int inds[2] = {i, j};
            bad += ls_fill_neighbor_inner(grid, dphi + 2 * (long)ind, inds, dX, nX, 2, mask,
                                          indn) != 0;
          }
        }
      for (int k = 0; k < niso; k++)
        mask[isolates[k]] = -2;
    }
  }
  free(isolates);
  return bad;
}

/* fill_ghost_cells (fill.cpp:330-370) for LSET = 1 and nmat <= 2:
 * re-distances the level set of u in place, then builds each material's
 * grid (nmat x ncell x V) and update mask (nmat x ncell).  Returns the
 * number of boundary cells whose fill would read outside the grid in the
 * reference (they are left unfilled here) or whose layered fill would
 * read past the last cell, or -3 for an unsupported variant. */
int or_fill_ghost_cells(double *grids, uint8_t *masks, double *u, const int *nX,
                        int ndim, const double *dX, double dt, const gpr_par *MPs,
                        int nmat, int32_t *intmask_out) {
  if (LSET != 1 || THERMAL || nmat < 1 || nmat > 2)
    return -3;
  long ncell = ndim == 1 ? nX[0] : (long)nX[0] * nX[1];
  double *col = malloc(sizeof(double) * ncell), *phi = malloc(sizeof(double) * ncell);
  double *dphi = malloc(sizeof(double) * ncell * ndim);
  int32_t *mask = malloc(sizeof(int32_t) * ncell);
  for (long c = 0; c < ncell; c++)
    col[c] = u[c * V + V - 1];
  or_distance(col, dX, nX, ndim, phi);
  for (long c = 0; c < ncell; c++)
    u[c * V + V - 1] = phi[c];
  int bad = 0;
  for (int mat = 0; mat < nmat; mat++) {
    double *grid = grids + (long)mat * ncell * V;
    uint8_t *mk = masks + (long)mat * ncell;
    if (MPs[mat].EOS <= -1) {
      memset(mk, 0, ncell);
      continue;
    }
    memcpy(grid, u, sizeof(double) * ncell * V);
    for (long c = 0; c < ncell; c++)
      phi[c] = mat == 0 ? u[c * V + V - 1] : -u[c * V + V - 1];
    or_finite_difference(phi, dX, nX, ndim, dphi);
    or_find_interface_cells(phi, nX, ndim, mask);
    bad += or_fill_boundary_cells(grid, mask, mat, phi, dphi, dX, MPs, dt, nX, ndim);
    bad += or_fill_neighbor_cells(grid, mask, dphi, dX, nX, ndim);
    for (long c = 0; c < ncell; c++)
      mk[c] = (phi[c] <= 0. && mask[c] != -2) || mask[c] == 1;
    if (intmask_out)
      memcpy(intmask_out + (long)mat * ncell, mask, sizeof(int32_t) * ncell);
  }
  free(col);
  free(phi);
  free(dphi);
  free(mask);
  return bad;
}

/* make_u (solvers/iterator.cpp:12-42) for LSET = 1. */
void or_make_u(double *u, const double *grids, const uint8_t *masks, long ncell,
               const gpr_par *MPs, int nmat) {
  for (long c = 0; c < ncell; c++) {
    double s = 0, cnt = 0;
    for (int mat = 0; mat < nmat; mat++)
      if (masks[(long)mat * ncell + c]) {
        s += grids[((long)mat * ncell + c) * V + V - 1];
        cnt += 1.;
      }
    if (cnt > 0.)
      u[c * V + V - 1] = s / cnt;
    int mi = ls_mat(u + c * V);
    if (MPs[mi].EOS > -1)
      memcpy(u + c * V, grids + ((long)mi * ncell + c) * V, sizeof(double) * (V - 1));
    else
      memset(u + c * V, 0, sizeof(double) * (V - 1));
  }
}

/* timestep (iterator.cpp:54-83) over the masked cells of every material. */
double or_timestep_multi(const double *grids, const uint8_t *masks, long ncell,
                         const double *dX, int ndim, double cfl, double t, double tf,
                         int count, const gpr_par *MPs, int nmat) {
  double MAX = 0.;
  for (int mat = 0; mat < nmat; mat++) {
    if (MPs[mat].EOS <= -1)
      continue;
    for (long c = 0; c < ncell; c++) {
      if (!masks[(long)mat * ncell + c])
        continue;
      double tmp = 0.;
      for (int d = 0; d < ndim; d++)
        tmp += or_max_abs_eigs(grids + ((long)mat * ncell + c) * V, d, MPs + mat) / dX[d];
      MAX = tmp > MAX ? tmp : MAX;
    }
  }
  double dt = cfl / MAX;
  if (count <= 5)
    dt *= 0.2;
  return t + dt > tf ? tf - t : dt;
}

/* renorm_distortion (solvers/utils.cpp:6-24) with the material of each cell
 * taken from its level set. */
void or_renorm_multi(double *u, long ncell, const gpr_par *MPs) {
  for (long c = 0; c < ncell; c++) {
    double *Q = u + c * V;
    const gpr_par *P = MPs + ls_mat(Q);
    if (P->EOS > -1 && Q[0] > 0) {
      double k = cbrt(Q[0] / (P->rho0 * det3(Q + 5)));
      for (int i = 0; i < 9; i++)
        Q[5 + i] *= k;
    }
  }
}

/* contorted (solvers/utils.cpp:66-85): a cell is contorted when its
 * normalised distortion has m0 - 1 > tol, m0 the mean of s_i^2 / det^(2/3)
 * over the singular values s_i of A, i.e. |A|_F^2 / (3 |det A|^(2/3));
 * then reset_distortion (:44-64) gives every cell of a non-vacuum material
 * A = (rho / rho0)^(1/3) I and removes its distortion energy rho E_2A.
 * Returns 1 if it reset. */
int or_reset_contorted(double *u, long ncell, double tol, const gpr_par *MPs, int nmat) {
  int hit = 0;
  for (long c = 0; c < ncell && !hit; c++) {
    const double *A = u + c * V + 5;
    double f2 = 0;
    for (int k = 0; k < 9; k++)
      f2 += A[k] * A[k];
    double d13 = cbrt(fabs(det3(A)));
    if (f2 / (3 * d13 * d13) - 1 > tol)
      hit = 1;
  }
  if (!hit)
    return 0;
  for (long c = 0; c < ncell; c++) {
    double *Q = u + c * V;
    int mi = LSET ? ls_mat(Q) : 0;
    const gpr_par *P = MPs + (mi < nmat ? mi : 0);
    if (P->EOS <= -1)
      continue;
    double r = Q[0];
    double cc = cbrt(r / P->rho0);
    Q[1] -= r * E_2A(r, Q + 5, P);
    for (int k = 0; k < 9; k++)
      Q[5 + k] = 0.0;
    Q[5] = Q[9] = Q[13] = cc;
  }
  return 1;
}
