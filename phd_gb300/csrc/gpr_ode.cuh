// gpr_ode.cuh - analytic split stiff-source step (body force, distortion
// relaxation, thermal impulse relaxation), restating
// system/relaxation/analytic.cpp:11-162 and solvers/split/ode.cpp:5-11.
#pragma once

#include "gpr_device.cuh"

namespace gpr {

// Symmetric 3x3 eigen-decomposition S = W diag(d) W^T by cyclic Jacobi
// rotations (register resident).  The ODE step is one lane's serial FP64
// chain per cell, so each rotation takes its tangent in one division,
// t = sgn(d) e / (|d| + sqrt(d^2 + e^2)) with d = S_qq - S_pp, e = 2 S_pq
// (the same t as sgn(theta) / (|theta| + sqrt(theta^2 + 1)), theta = d / e),
// and c = rsqrt(t^2 + 1); the sweeps stop once the off-diagonal sum is
// below 2^-60 of the trace (S = A^T A is positive semidefinite), where a
// further rotation moves the eigenvalues by less than a rounding and the
// eigenvectors only within a subspace of equal eigenvalues, which the
// distortion update A' = U diag(s') V^T does not see.
GPR_D void jacobi3(double S[3][3], double W[3][3], double d[3]) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      W[i][j] = i == j ? 1.0 : 0.0;
  const double stop = 0x1p-60 * (S[0][0] + S[1][1] + S[2][2]);
  for (int sweep = 0; sweep < 12; sweep++) {
    double off = fabs(S[0][1]) + fabs(S[0][2]) + fabs(S[1][2]);
    if (off <= stop)
      break;
#pragma unroll
    for (int pq = 0; pq < 3; pq++) {
      const int p = pq == 2 ? 1 : 0;
      const int q = pq == 0 ? 1 : 2;
      if (S[p][q] != 0.0) {
        const double dd = S[q][q] - S[p][p], e = 2.0 * S[p][q];
        const double rr = sqrt(dd * dd + e * e);
        double t = (dd >= 0 ? e : -e) / (fabs(dd) + rr);
        double c = rsqrt(t * t + 1.0), s = t * c;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          double a = S[k][p], b = S[k][q];
          S[k][p] = c * a - s * b;
          S[k][q] = s * a + c * b;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
          double a = S[p][k], b = S[q][k];
          S[p][k] = c * a - s * b;
          S[q][k] = s * a + c * b;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
          double a = W[k][p], b = W[k][q];
          W[k][p] = c * a - s * b;
          W[k][q] = s * a + c * b;
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
    d[i] = S[i][i];
}

// SVD of a 3x3 (row-major) A = U diag(s) V^T with s descending: V from the
// eigenvectors of A^T A, U = A V / s re-orthonormalised.  The distortion
// update A' = U diag(s') V^T does not depend on the sign/order conventions
// of the factors.
GPR_D void svd3(const double *A, double U[3][3], double s[3], double Vm[3][3]) {
  double S[3][3], W[3][3], d[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      S[i][j] = A[i] * A[j] + A[3 + i] * A[3 + j] + A[6 + i] * A[6 + j];
  jacobi3(S, W, d);
  // sort descending (3-element network, no dynamic indexing)
  int i0 = 0, i1 = 1, i2 = 2;
  if (d[i1] > d[i0]) { int t = i0; i0 = i1; i1 = t; }
  if (d[i2] > d[i1]) { int t = i1; i1 = i2; i2 = t; }
  if (d[i1] > d[i0]) { int t = i0; i0 = i1; i1 = t; }
  int idx[3] = {i0, i1, i2};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    int ic = idx[c];
    double dv = ic == 0 ? d[0] : (ic == 1 ? d[1] : d[2]);
    s[c] = sqrt(fmax(dv, 0.0));
#pragma unroll
    for (int r = 0; r < 3; r++)
      Vm[r][c] = ic == 0 ? W[r][0] : (ic == 1 ? W[r][1] : W[r][2]);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double x[3];
#pragma unroll
    for (int r = 0; r < 3; r++)
      x[r] = A[3 * r] * Vm[0][c] + A[3 * r + 1] * Vm[1][c] + A[3 * r + 2] * Vm[2][c];
#pragma unroll
    for (int p = 0; p < 3; p++) {
      if (p < c) {
        double dp = x[0] * U[0][p] + x[1] * U[1][p] + x[2] * U[2][p];
#pragma unroll
        for (int r = 0; r < 3; r++)
          x[r] -= dp * U[r][p];
      }
    }
    double inv = 1.0 / sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
#pragma unroll
    for (int r = 0; r < 3; r++)
      U[r][c] = x[r] * inv;
  }
}

GPR_D double posd(double x) { return x > 0.0 ? x : 0.0; }

// nondimensionalized_time (analytic.cpp:17-69)
GPR_D double nondim_time(double r, double detA3, double m0, double u0, double dt,
                         const DevPar &P) {
  if (P.flags & GPR_POWER_LAW) {
    double n = P.n;
    double cs2 = P.beta == 0.0 ? P.b02 : P.b02 * pow(r * P.ir0, P.beta);
    double a = 9. * m0 - u0 - 9.;
    double b = 6. * m0 - u0 - 6.;
    double amb = a - b, amb2 = amb * amb;
    double a2 = a * a, b2 = b * b;
    if (P.flags & GPR_SOLID) {
      double c = 108. * a - 324. * b + 108. * a2 - 396. * a * b + 297. * b2 -
                 24. * (a2 * b - 2. * a * b2 + b2 * b) - 4. * amb2 * amb2;
      if (c <= 0.)
        return 0.;
      double lam = c / (18. * a - 36. * b + 9. * a2 - 132. / 5. * a * b + 33. / 2. * b2 -
                        8. / 7. * a2 * b + 2. * a * b2 - 8. / 9. * b2 * b - a2 * a2 / 6. +
                        16. / 27. * a2 * a * b - 4. / 5. * a2 * b2 + 16. / 33. * a * b2 * b -
                        b2 * b2 / 9.);
      double tmp1 = n * lam / P.tau0 * pow(detA3, 4. * n + 7.);
      double tmp2 = pow(sqrt(c) * r * cs2 / (6. * P.sigmaY), n);
      return 2. / (n * lam) * log(tmp1 * tmp2 * dt + 1.);
    }
    double k = (1 - n) / n;
    double c = 108. * a - 324. * b + 180. * a2 - 612. * a * b + 459. * b2 -
               24. * (a2 * b - 2. * a * b2 + b2 * b) - 4. * amb2 * amb2;
    if (c <= 0.)
      return 0.;
    double lam = c / (18. * a - 36. * b + 15. * a2 - 204. / 5. * a * b + 51. / 2. * b2 -
                      8. / 7. * a2 * b + 2. * a * b2 - 8. / 9. * b2 * b - a2 * a2 / 6. +
                      16. / 27. * a2 * a * b - 4. / 5. * a2 * b2 + 16. / 33. * a * b2 * b -
                      b2 * b2 / 9.);
    double tmp1 = k * lam / P.tau1 * pow(detA3, 4. * k + 7.);
    double tmp2 = pow(sqrt(c) * r * cs2 / (6. * sqrt(3.)), k);
    return 2. / (k * lam) * log(tmp1 * tmp2 * dt + 1.);
  }
  double d2 = detA3 * detA3, d4 = d2 * d2;
  return P.rho0 * P.b02 * (d4 * d2 * detA3) / (3. * P.mu) * dt;
}

// analyticSolver_distortion (analytic.cpp:71-128)
GPR_D void ode_distortion(double *q, double dt, const DevPar &P) {
  double *A = q + 5;
  double U[3][3], s[3], Vm[3][3];
  svd3(A, U, s, Vm);
  double detA = s[0] * s[1] * s[2];
  double r = detA * P.rho0;
  double d13 = cbrt(detA);
  double id23 = 1.0 / (d13 * d13);
  double s0 = s[0] * s[0] * id23, s1 = s[1] * s[1] * id23, s2 = s[2] * s[2] * id23;
  // divisions by constants as products with the rounded reciprocal (one
  // rounding apart; each IEEE division is a long FP64 sequence on this
  // one-lane chain)
  const double third = 1.0 / 3.0;
  double m0 = (s0 + s1 + s2) * third;
  double u0 = ((s0 - s1) * (s0 - s1) + (s1 - s2) * (s1 - s2) + (s2 - s0) * (s2 - s0)) * third;
  if (u0 < 1e-12)
    return;
  double tau = nondim_time(r, d13, m0, u0, dt, P);
  double e6 = exp(-6. * tau), e9 = exp(-9. * tau);
  double a = 3. * m0 - u0 * third - 3.;
  double b = 2. * m0 - u0 * third - 2.;
  double m = 1. + a * e6 - b * e9;
  double u = posd(6. * a * e6 - 9. * b * e9);
  double Dl = -2. * m * m * m + m * u + 2.;
  double arg1 = posd(6. * u * u * u - 81. * Dl * Dl);
  double x1;
  if (fabs(Dl) < 1e-12)
    x1 = sqrt(6. * u) * third * 0.86602540378443864676 + m;  // cos(pi/6)
  else if (arg1 == 0.) {
    double tmp = cbrt(54. * Dl);
    x1 = tmp * (1.0 / 6.0) + u / tmp + m;
  } else {
    double th = atan(sqrt(arg1) / (9. * Dl));
    x1 = sqrt(6. * u) * third * cos(th * third) + m;
  }
  double tmp2 = 3. * m - x1;
  double arg2 = posd(x1 * tmp2 * tmp2 - 4.);
  double x2 = 0.5 * (sqrt(arg2 / x1) + tmp2);
  double x3 = 1. / (x1 * x2);
  // ascending sort, then the largest goes with the largest singular value
  double lo = fmin(fmin(x1, x2), x3), hi = fmax(fmax(x1, x2), x3);
  double mid = x1 + x2 + x3 - lo - hi;
  double sc[3] = {d13 * sqrt(hi), d13 * sqrt(mid), d13 * sqrt(lo)};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      A[3 * i + j] = U[i][0] * sc[0] * Vm[j][0] + U[i][1] * sc[1] * Vm[j][1] +
                     U[i][2] * sc[2] * Vm[j][2];
}

// analyticSolver_thermal (analytic.cpp:130-150)
template <bool TH>
GPR_D void ode_thermal(double *q, double dt, const DevPar &P) {
  if (!TH)
    return;
  double r = q[0], ir = 1.0 / r;
  double E = q[1] * ir;
  double v0 = q[2] * ir, v1 = q[3] * ir, v2 = q[4] * ir;
  const double *A = q + 5;
  double G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  double G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  double G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  double G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  double G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  double G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  double t = (G00 + G11 + G22) / 3.0;
  double dg = (G00 - t) * (G00 - t) + (G11 - t) * (G11 - t) + (G22 - t) * (G22 - t) +
              2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
  double Gm = eos_rho(r, ir, P).G;
  double cs2 = P.beta == 0.0 ? P.b02 : P.b02 * pow(r * P.ir0, P.beta);
  double C0 = (1.0 - P.beta / Gm) * cs2;
  double c1 = E - 0.25 * C0 * dg - 0.5 * (v0 * v0 + v1 * v1 + v2 * v2);
  double c2 = P.calpha2 / 2.;
  double k = 2 * P.calpha2 / (P.kappa * r * P.cv);
  c1 *= k;
  c2 *= k;
  double ea = exp(-c1 * dt / 2);
  double J2 = q[14] * q[14] + q[15] * q[15] + q[16] * q[16];
  double den = 1 - c2 / c1 * (1 - ea * ea) * J2 * ir * ir;
  double f = ea / sqrt(den);
  q[14] *= f;
  q[15] *= f;
  q[16] *= f;
}

// ode_stepper_analytic (analytic.cpp:152-161) on the state at uc
template <class L> GPR_D void ode_cell(double *uc, double dt, const DevPar &P) {
  constexpr int V = L::V;
  double q[V];
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = uc[k];
  q[2] += P.dp0 * dt;
  q[3] += P.dp1 * dt;
  q[4] += P.dp2 * dt;
  ode_distortion(q, dt, P);
  ode_thermal<L::THERMAL>(q, dt, P);
#pragma unroll
  for (int k = 2; k < 17 && k < V; k++)
    uc[k] = q[k];
}

// The ODE step of every cell of u (ncell cells) and, in the same launch, of
// u2 (ncell2 cells, optional): the split stepper's two independent half
// steps on u and ub (steppers.cpp:50-66) take one launch, so on small grids
// one serial per-cell chain instead of two.
template <class L>
__global__ void k_ode(double *__restrict__ u, long ncell, double dt,
                      const double *__restrict__ dt_dev, double dt_scale, DevPar P,
                      double *__restrict__ u2 = nullptr, long ncell2 = 0) {
  constexpr int V = L::V;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell + ncell2)
    return;
  if (dt_dev)
    dt = *dt_dev * dt_scale;
  ode_cell<L>(c < ncell ? u + c * V : u2 + (c - ncell) * V, dt, P);
}

}  // namespace gpr
