// gpr_device.cuh - device-side GPR (Godunov-Peshkov-Romenski) physics in FP64.
//
// Pointwise functions of one conserved state Q[V] (registers), restating the
// reference's system library (code/cpp/src/system/*.cpp) with the derived
// quantities of a state computed once (`Prim`) and shared by flux, source,
// the non-conservative product and the wave-speed bound, instead of being
// recomputed per call as the reference does (pressure() alone is evaluated
// 4-6 times per node there).  Every function cites the reference it restates.
//
// Layout of Q: [rho, rho E, rho v(3), A(3x3 row-major), rho J(3) if THERMAL,
// phi(LSET)].
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/gpr_gb300.h"

#define GPR_HD __host__ __device__ __forceinline__
#define GPR_D __device__ __forceinline__

namespace gpr {

// the least positive normal double (DBL_MIN)
constexpr double DBL_MIN_NORMAL = 2.2250738585072014e-308;

// Material parameters with the per-material constants the kernels need
// hoisted out of the per-node code (e.g. rho0 / (2 mu^(1/n)), 1/kappa).
struct DevPar {
  int EOS, flags;
  double rho0, ir0, Tref, cv, icv, pINF, Gamma0, c02, s, alpha, beta, gamma;
  double A, B, R1, R2;
  double b02, mu, tau0, sigmaY, n, calpha2, kappa, ikappa;
  double dp0, dp1, dp2;
  double th1c;   // rho0 / (2 mu^(1/n))          (sources.cpp:71)
  double tau1;   // 6 mu^(1/n) / (rho0 b02)      (analytic.cpp:62)
  double iG;     // 1/Gamma for the constant-Gamma EOS; 1/(Gamma0 rho0) for shock MG
  double C0f;    // 1 - beta/Gamma for the constant-Gamma EOS
};

inline DevPar make_devpar(const gpr_par &p) {
  DevPar d;
  d.EOS = p.EOS;
  d.flags = p.flags;
  d.rho0 = p.rho0;
  d.ir0 = 1.0 / p.rho0;
  d.Tref = p.Tref;
  d.cv = p.cv;
  d.icv = 1.0 / p.cv;
  d.pINF = p.pINF;
  d.Gamma0 = p.Gamma0;
  d.c02 = p.c02;
  d.s = p.s;
  d.alpha = p.alpha;
  d.beta = p.beta;
  d.gamma = p.gamma;
  d.A = p.A;
  d.B = p.B;
  d.R1 = p.R1;
  d.R2 = p.R2;
  d.b02 = p.b02;
  d.mu = p.mu;
  d.tau0 = p.tau0;
  d.sigmaY = p.sigmaY;
  d.n = p.n;
  d.calpha2 = p.calpha2;
  d.kappa = p.kappa;
  d.ikappa = 1.0 / p.kappa;
  d.dp0 = p.dp[0];
  d.dp1 = p.dp[1];
  d.dp2 = p.dp[2];
  d.th1c = p.rho0 / (2.0 * pow(p.mu, 1.0 / p.n));
  d.tau1 = 6.0 * pow(p.mu, 1.0 / p.n) / (p.rho0 * p.b02);
  double G = p.EOS == 0 ? p.gamma - 1.0 : (p.EOS == 4 ? p.gamma : p.Gamma0);
  d.iG = p.EOS == 1 ? 1.0 / (p.Gamma0 * p.rho0) : 1.0 / G;
  d.C0f = 1.0 - p.beta / G;
  return d;
}

// ---------------------------------------------------------------------------
// Mie-Gruneisen EOS family (system/energy/mg.cpp:6-303).  EOS codes:
// 0 stiffened gas, 1 shock MG, 2 JWL, 3 Cochran-Chan, 4 Godunov-Romenski.

struct EosRho {  // density-only EOS quantities
  double G;      // Gamma_MG
  double dG;     // dGamma/drho
  double pr;     // p_ref
  double dpr;    // dp_ref/drho
  double er;     // e_ref
  double der;    // de_ref/drho
  double phi;    // integrating factor (only multiplied by Tref)
};

GPR_D EosRho eos_rho(double r, double ir, const DevPar &P) {
  EosRho e;
  switch (P.EOS) {
  case 0: {  // stiffened gas
    e.G = P.gamma - 1.0;
    e.dG = 0.0;
    e.pr = -P.pINF;
    e.dpr = 0.0;
    e.er = P.pINF * ir;
    e.der = e.pr * ir * ir;
    e.phi = P.Tref != 0.0 ? pow(r * P.ir0, P.gamma - 1.0) : 0.0;
  } break;
  case 1: {  // shock Mie-Gruneisen
    e.G = P.Gamma0 * P.rho0 * ir;
    e.dG = -P.Gamma0 * P.rho0 * ir * ir;
    if (r > P.rho0) {
      double tmp = P.ir0 - P.s * (P.ir0 - ir);
      e.pr = P.c02 * (P.ir0 - ir) / (tmp * tmp);
      double t2 = P.s * (r - P.rho0) - r;
      e.dpr = P.c02 * P.rho0 * P.rho0 * (P.s * (P.rho0 - r) - r) / (t2 * t2 * t2);
      e.er = 0.5 * e.pr * (P.ir0 - ir);
      e.der = -(r - P.rho0) * P.rho0 * P.c02 / (t2 * t2 * t2);
    } else {
      e.pr = P.c02 * (r - P.rho0);
      e.dpr = P.c02;
      e.er = 0.0;
      e.der = 0.0;
    }
    e.phi = P.Tref != 0.0 ? exp(P.Gamma0 * (1.0 - P.rho0 * ir)) : 0.0;
  } break;
  case 4: {  // Godunov-Romenski
    e.G = P.gamma;
    e.dG = 0.0;
    double tmp = pow(r * P.ir0, P.alpha);
    e.pr = P.c02 * r / P.alpha * (tmp - 1.0) * tmp;
    e.dpr = P.c02 / P.alpha * tmp * ((1.0 + P.alpha) * (tmp - 1.0) + P.alpha * tmp);
    e.er = P.c02 / (2.0 * P.alpha * P.alpha) * (tmp - 1.0) * (tmp - 1.0);
    e.der = e.pr * ir * ir;
    e.phi = P.Tref != 0.0 ? pow(r * P.ir0, P.gamma) : 0.0;
  } break;
  case 2: {  // JWL
    e.G = P.Gamma0;
    e.dG = 0.0;
    double v_ = P.rho0 * ir;
    double e1 = exp(-P.R1 * v_), e2 = exp(-P.R2 * v_);
    e.pr = P.A * e1 + P.B * e2;
    e.dpr = v_ * ir * (P.A * P.R1 * e1 + P.B * P.R2 * e2);
    e.er = P.A / (P.rho0 * P.R1) * e1 + P.B / (P.rho0 * P.R2) * e2;
    e.der = e.pr * ir * ir;
    e.phi = P.Tref != 0.0 ? pow(r * P.ir0, P.Gamma0) : 0.0;
  } break;
  default: {  // Cochran-Chan
    e.G = P.Gamma0;
    e.dG = 0.0;
    double v_ = P.rho0 * ir;
    double a1 = pow(v_, -P.R1), a2 = pow(v_, -P.R2);
    e.pr = P.A * a1 - P.B * a2;
    e.dpr = P.A * P.R1 * ir * a1 - P.B * P.R2 * ir * a2;
    e.er = -P.A / (P.rho0 * (1.0 - P.R1)) * (pow(v_, 1.0 - P.R1) - 1.0) +
           P.B / (P.rho0 * (1.0 - P.R2)) * (pow(v_, 1.0 - P.R2) - 1.0);
    e.der = e.pr * ir * ir;
    e.phi = P.Tref != 0.0 ? pow(r * P.ir0, P.Gamma0) : 0.0;
  } break;
  }
  return e;
}

// ---------------------------------------------------------------------------
// Derived quantities of one state (variables/state.cpp, energy/eos.cpp,
// functions/matrices.cpp).  G = A^T A, devG = G - tr(G)/3 I.  |dev G|^2 is
// evaluated from A^T A; the reference's devGsq (matrices.cpp:16-26) uses the
// rows of A (A A^T), which has the same trace and Frobenius norm.
template <bool TH> struct Prim {
  double r, ir;          // rho, 1/rho
  double v[3];           // velocity
  double J[3];           // thermal impulse (TH)
  double AdG[9];         // A devG (row-major)
  double cs2;            // b02 (rho/rho0)^beta
  double devGsq;         // |dev G|^2
  double p, T;           // pressure, temperature
  double irG;            // 1 / (rho Gamma)
  EosRho e;
};

template <bool TH>
GPR_D void prim(const double *q, const DevPar &P, Prim<TH> &s) {
  s.r = q[0];
  s.ir = 1.0 / s.r;
  s.v[0] = q[2] * s.ir;
  s.v[1] = q[3] * s.ir;
  s.v[2] = q[4] * s.ir;
  const double *A = q + 5;
  double G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  double G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  double G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  double G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  double G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  double G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  double t = (G00 + G11 + G22) * (1.0 / 3.0);
  double D00 = G00 - t, D11 = G11 - t, D22 = G22 - t;
  s.devGsq = D00 * D00 + D11 * D11 + D22 * D22 + 2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double a0 = A[3 * i], a1 = A[3 * i + 1], a2 = A[3 * i + 2];
    s.AdG[3 * i + 0] = a0 * D00 + a1 * G01 + a2 * G02;
    s.AdG[3 * i + 1] = a0 * G01 + a1 * D11 + a2 * G12;
    s.AdG[3 * i + 2] = a0 * G02 + a1 * G12 + a2 * D22;
  }
  s.e = eos_rho(s.r, s.ir, P);
  s.cs2 = P.beta == 0.0 ? P.b02 : P.b02 * pow(s.r * P.ir0, P.beta);
  // C_0 = (1 - beta/Gamma) cs2 (shear.cpp:23-29); rho Gamma = Gamma0 rho0 for shock MG
  double C0 = P.beta == 0.0 ? s.cs2
                            : (P.EOS == 1 ? (1.0 - P.beta / s.e.G) : P.C0f) * s.cs2;
  s.irG = P.EOS == 1 ? P.iG : s.ir * P.iG;
  double E1 = q[1] * s.ir - 0.5 * (s.v[0] * s.v[0] + s.v[1] * s.v[1] + s.v[2] * s.v[2]) -
              0.25 * C0 * s.devGsq;
  if (TH) {
    s.J[0] = q[14] * s.ir;
    s.J[1] = q[15] * s.ir;
    s.J[2] = q[16] * s.ir;
    E1 -= 0.5 * P.calpha2 * (s.J[0] * s.J[0] + s.J[1] * s.J[1] + s.J[2] * s.J[2]);
  }
  // pressure_mg (mg.cpp:126-131), temperature_mg (mg.cpp:133-139)
  double rG = s.r * s.e.G;
  s.p = (E1 - s.e.er) * rG + s.e.pr;
  s.T = s.e.phi * P.Tref + (s.p - s.e.pr) * s.irG * P.icv;
}

// sigma column d: -rho cs2 (A devG)^T A(:,d)   (state.cpp:23-29)
template <bool TH>
GPR_D void sigma_col(const double *q, const Prim<TH> &s, int d, double *sg) {
  const double *A = q + 5;
  double f = -s.r * s.cs2;
#pragma unroll
  for (int i = 0; i < 3; i++)
    sg[i] = f * (s.AdG[i] * A[d] + s.AdG[3 + i] * A[3 + d] + s.AdG[6 + i] * A[6 + d]);
}

// ret += F_d(Q)   (equations.cpp:11-48)
template <bool TH, int V>
GPR_D void flux_add(const double *q, const Prim<TH> &s, int d, const DevPar &P, double *F) {
  double vd = s.v[d];
  double sg[3];
  sigma_col(q, s, d, sg);
  F[0] += q[2 + d];
  F[1] += vd * (q[1] + s.p) - (sg[0] * s.v[0] + sg[1] * s.v[1] + sg[2] * s.v[2]);
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[2 + i] += vd * q[2 + i] - sg[i];
  F[2 + d] += s.p;
  const double *A = q + 5;
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[5 + 3 * i + d] += A[3 * i] * s.v[0] + A[3 * i + 1] * s.v[1] + A[3 * i + 2] * s.v[2];
  if (TH) {
    F[1] += P.calpha2 * s.T * s.J[d];
#pragma unroll
    for (int i = 0; i < 3; i++)
      F[14 + i] += vd * q[14 + i];
    F[14 + d] += s.T;
  }
}

// Entries of F_d(Q) that can be nonzero (flux_add / flux_set write only
// these; the rest are exact zeros).
template <bool TH> __host__ __device__ constexpr bool flux_support(int k, int d) {
  return k < 5 || (k >= 5 && k < 14 && (k - 5) % 3 == d) || (TH && k >= 14 && k < 17);
}

// F = F_d(Q): flux_add into a zeroed array without the additions to zero
// (which the compiler must keep: 0.0 + x is not x for x = -0.0).
template <bool TH, int V>
GPR_D void flux_set(const double *q, const Prim<TH> &s, int d, const DevPar &P, double *F) {
#pragma unroll
  for (int k = 0; k < V; k++)
    F[k] = 0.0;
  double vd = s.v[d];
  double sg[3];
  sigma_col(q, s, d, sg);
  F[0] = q[2 + d];
  F[1] = vd * (q[1] + s.p) - (sg[0] * s.v[0] + sg[1] * s.v[1] + sg[2] * s.v[2]);
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[2 + i] = vd * q[2 + i] - sg[i];
  F[2 + d] += s.p;
  const double *A = q + 5;
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[5 + 3 * i + d] = A[3 * i] * s.v[0] + A[3 * i + 1] * s.v[1] + A[3 * i + 2] * s.v[2];
  if (TH) {
    F[1] += P.calpha2 * s.T * s.J[d];
#pragma unroll
    for (int i = 0; i < 3; i++)
      F[14 + i] = vd * q[14 + i];
    F[14 + d] += s.T;
  }
}

GPR_D double det3(const double *A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

// Sigma Frobenius-type norms used by the non-Newtonian relaxation rates.
template <bool TH>
GPR_D void sigma_full(const double *q, const Prim<TH> &s, double *sf) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double c[3];
    sigma_col(q, s, d, c);
    sf[d] = c[0];
    sf[3 + d] = c[1];
    sf[6 + d] = c[2];
  }
}

// theta1inv (sources.cpp:13-81)
template <bool TH>
GPR_D double theta1inv(const double *q, const Prim<TH> &s, const DevPar &P) {
  double dA = det3(q + 5);
  double cb = cbrt(dA);
  double A53 = dA * cb * cb;  // det(A)^(5/3)
  int SOLID = P.flags & GPR_SOLID, PL = P.flags & GPR_POWER_LAW, BING = P.flags & GPR_BINGHAM;
  if (!SOLID && !BING && !PL)
    return A53 * P.th1c;
  double sf[9];
  sigma_full(q, s, sf);
  if (SOLID) {
    if (!PL)
      return 0.0;
    double a = sf[0] - sf[4], b = sf[4] - sf[8], c = sf[8] - sf[0];
    double sn = sqrt(0.5 * (a * a + b * b + c * c) + 3.0 * (sf[1] * sf[1] + sf[5] * sf[5] + sf[6] * sf[6]));
    sn = fmin(sn, 1e8);
    return 3.0 * A53 / (s.cs2 * P.tau0) * pow(sn / P.sigmaY, P.n);
  }
  double nn = 0.0;
#pragma unroll
  for (int i = 0; i < 9; i++)
    nn += sf[i] * sf[i];
  double sn = sqrt(nn) * 0.70710678118654752440;
  if (BING)
    return sn > P.sigmaY ? A53 * P.rho0 / (2.0 * P.mu) * (1.0 - P.sigmaY / sn) : 0.0;
  return A53 * P.th1c * pow(sn, (1.0 - P.n) / P.n);
}

// S(Q)   (equations.cpp:50-67)
template <bool TH, int V>
GPR_D void source(const double *q, const Prim<TH> &s, const DevPar &P, double *S,
                  double scale = 1.0) {
  // scale multiplies the result (through its scalar factors)
#pragma unroll
  for (int k = 0; k < V; k++)
    S[k] = 0.0;
  S[2] = P.dp0 * scale;
  S[3] = P.dp1 * scale;
  S[4] = P.dp2 * scale;
  double f = -s.cs2 * theta1inv(q, s, P) * scale;
#pragma unroll
  for (int i = 0; i < 9; i++)
    S[5 + i] = s.AdG[i] * f;
  if (TH) {
    // -rho (calpha2 J) T / (kappa rho)
    double g = -P.calpha2 * s.T * P.ikappa * scale;
#pragma unroll
    for (int i = 0; i < 3; i++)
      S[14 + i] = g * s.J[i];
  }
}

// B_d(Q) x   (equations.cpp:89-167); v = rho v / rho.
template <int V, int LSET>
GPR_D void bdot(const double *v, const double *x, int d, double *out) {
#pragma unroll
  for (int k = 0; k < 5; k++)
    out[k] = 0.0;
#pragma unroll
  for (int k = 14; k < V; k++)
    out[k] = 0.0;
  double v0 = v[0], v1 = v[1], v2 = v[2];
  if (d == 0) {
#pragma unroll
    for (int r = 0; r < 3; r++) {
      out[5 + 3 * r] = -v1 * x[6 + 3 * r] - v2 * x[7 + 3 * r];
      out[6 + 3 * r] = v0 * x[6 + 3 * r];
      out[7 + 3 * r] = v0 * x[7 + 3 * r];
    }
  } else if (d == 1) {
#pragma unroll
    for (int r = 0; r < 3; r++) {
      out[5 + 3 * r] = v1 * x[5 + 3 * r];
      out[6 + 3 * r] = -v0 * x[5 + 3 * r] - v2 * x[7 + 3 * r];
      out[7 + 3 * r] = v1 * x[7 + 3 * r];
    }
  } else {
#pragma unroll
    for (int r = 0; r < 3; r++) {
      out[5 + 3 * r] = v2 * x[5 + 3 * r];
      out[6 + 3 * r] = v2 * x[6 + 3 * r];
      out[7 + 3 * r] = -v0 * x[5 + 3 * r] - v1 * x[6 + 3 * r];
    }
  }
  if (LSET > 0) {
    double vd = d == 0 ? v0 : (d == 1 ? v1 : v2);
#pragma unroll
    for (int i = 1; i <= LSET; i++)
      out[V - i] = vd * x[V - i];
  }
}

// ---------------------------------------------------------------------------
// Eigenvalues of a small real nonsymmetric matrix: Householder reduction to
// Hessenberg form, then Francis double-shift QR with deflation (Golub & Van
// Loan, Matrix Computations, Alg. 7.4.2, 7.5.1-7.5.2).  Returns the largest
// eigenvalue modulus (the reference calls Eigen's EigenSolver and takes
// max |lambda|, system/eig.cpp:73).  Returns NaN if it does not converge.
template <int n> GPR_D double max_abs_eig(double (&H)[n][n]) {
  const double eps = 2.220446049250313e-16;
  // Hessenberg reduction
#pragma unroll
  for (int k = 0; k < n - 2; k++) {
    double v[n];
    double alpha = 0.0, tail = 0.0;
#pragma unroll
    for (int i = 0; i < n; i++) {
      if (i > k)
        alpha += H[i][k] * H[i][k];
      if (i > k + 1)
        tail += H[i][k] * H[i][k];
    }
    alpha = sqrt(alpha);
    // no reflection when the column below the subdiagonal is zero to the
    // least normal number (Eigen's makeHouseholder rule): a reflector of
    // subnormal entries would divide by an underflowed norm
    if (alpha != 0.0 && tail > DBL_MIN_NORMAL) {
      double x0 = H[k + 1][k];
      double beta = x0 > 0 ? -alpha : alpha;
#pragma unroll
      for (int i = 0; i < n; i++)
        v[i] = i > k + 1 ? H[i][k] : 0.0;
      v[k + 1] = x0 - beta;
      double vv = 0.0;
#pragma unroll
      for (int i = 0; i < n; i++)
        vv += v[i] * v[i];
      if (vv != 0.0) {
        double tau = 2.0 / vv;
#pragma unroll
        for (int j = 0; j < n; j++) {
          double sacc = 0.0;
#pragma unroll
          for (int i = 0; i < n; i++)
            sacc += v[i] * H[i][j];
          sacc *= tau;
#pragma unroll
          for (int i = 0; i < n; i++)
            H[i][j] -= sacc * v[i];
        }
#pragma unroll
        for (int i = 0; i < n; i++) {
          double sacc = 0.0;
#pragma unroll
          for (int j = 0; j < n; j++)
            sacc += H[i][j] * v[j];
          sacc *= tau;
#pragma unroll
          for (int j = 0; j < n; j++)
            H[i][j] -= sacc * v[j];
        }
      }
    }
  }
  double norm = 0.0;
#pragma unroll
  for (int i = 0; i < n; i++)
#pragma unroll
    for (int j = 0; j < n; j++)
      if (j >= i - 1)
        norm += fabs(H[i][j]);
  double best = 0.0;
  int hi = n - 1, iter = 0, total = 0;
  double exshift = 0.0;
  while (hi >= 0) {
    int l = hi;
    while (l > 0) {
      double s = fabs(H[l - 1][l - 1]) + fabs(H[l][l]);
      if (s == 0.0)
        s = norm;
      if (fabs(H[l][l - 1]) < eps * s)
        break;
      l--;
    }
    if (l == hi) {
      best = fmax(best, fabs(H[hi][hi] + exshift));
      hi--;
      iter = 0;
      continue;
    }
    double x = H[hi][hi], y = H[hi - 1][hi - 1], w = H[hi][hi - 1] * H[hi - 1][hi];
    if (l == hi - 1) {
      double p = 0.5 * (y - x), q = p * p + w, z = sqrt(fabs(q));
      x += exshift;
      if (q >= 0.0) {
        z = p >= 0 ? p + z : p - z;
        best = fmax(best, fabs(x + z));
        best = fmax(best, fabs(z != 0.0 ? x - w / z : x + z));
      } else {
        best = fmax(best, hypot(x + p, z));
      }
      hi -= 2;
      iter = 0;
      continue;
    }
    if (iter == 10 || iter == 20) {
      exshift += x;
      for (int i = 0; i <= hi; i++)
        H[i][i] -= x;
      double s = fabs(H[hi][hi - 1]) + fabs(H[hi - 1][hi - 2]);
      x = y = 0.75 * s;
      w = -0.4375 * s * s;
    }
    iter++;
    if (++total > 30 * n)
      return nan("");
    int m = hi - 2;
    double p = 0, q = 0, r = 0, z;
    while (m >= l) {
      z = H[m][m];
      r = x - z;
      double s = y - z;
      p = (r * s - w) / H[m + 1][m] + H[m][m + 1];
      q = H[m + 1][m + 1] - z - r - s;
      r = H[m + 2][m + 1];
      s = fabs(p) + fabs(q) + fabs(r);
      p /= s;
      q /= s;
      r /= s;
      if (m == l)
        break;
      double u = fabs(H[m][m - 1]) * (fabs(q) + fabs(r));
      double vv = fabs(p) * (fabs(H[m - 1][m - 1]) + fabs(z) + fabs(H[m + 1][m + 1]));
      if (u < eps * vv)
        break;
      m--;
    }
    for (int i = m + 2; i <= hi; i++) {
      H[i][i - 2] = 0.0;
      if (i > m + 2)
        H[i][i - 3] = 0.0;
    }
    for (int k = m; k <= hi - 1; k++) {
      bool notlast = (k != hi - 1);
      if (k != m) {
        p = H[k][k - 1];
        q = H[k + 1][k - 1];
        r = notlast ? H[k + 2][k - 1] : 0.0;
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
        H[k][k - 1] = -s * x;
      else if (l != m)
        H[k][k - 1] = -H[k][k - 1];
      p += s;
      x = p / s;
      y = q / s;
      z = r / s;
      q /= p;
      r /= p;
      for (int j = k; j <= hi; j++) {
        double pp = H[k][j] + q * H[k + 1][j];
        if (notlast) {
          pp += r * H[k + 2][j];
          H[k + 2][j] -= pp * z;
        }
        H[k][j] -= pp * x;
        H[k + 1][j] -= pp * y;
      }
      int ihi = hi < k + 3 ? hi : k + 3;
      for (int i = l; i <= ihi; i++) {
        double pp = x * H[i][k] + y * H[i][k + 1];
        if (notlast) {
          pp += z * H[i][k + 2];
          H[i][k + 2] -= pp * r;
        }
        H[i][k] -= pp;
        H[i][k + 1] -= pp * q;
      }
    }
  }
  return best;
}

// Largest eigenvalue of a small real matrix whose spectrum is dominated by a
// simple, real, positive eigenvalue (the squared fastest wave speed of the
// thermo-acoustic tensor): characteristic polynomial by principal minors,
// Laguerre's iteration (cubically convergent, monotone from an upper bound
// for real-rooted polynomials) started at the infinity-norm bound, then a
// certificate: the polynomial deflated by (x - lambda) must have every root
// strictly inside |z| < (1 - 1e-9) lambda (Jury's criterion on the scaled
// quotient).  Returns false when the certificate fails (complex roots of
// larger modulus, a multiple largest root, no convergence); the caller then
// runs the QR iteration, so the result is max |eig| either way.
// Z: X[1][m-1] and X[2][m-1] are known zeros (the heat-conduction column of
// the acoustic tensor), left out of the characteristic polynomial.
template <int m, bool Z = false>
GPR_D bool max_eig_laguerre(const double (&X)[m][m], double &lam) {
  static_assert(m == 3 || m == 4, "3x3 or 4x4");
  double c1 = 0.0, c2 = 0.0, c3 = 0.0, c4 = 0.0;
#pragma unroll
  for (int i = 0; i < m; i++)
    c1 += X[i][i];
  if (m == 3) {
#pragma unroll
    for (int i = 0; i < m; i++)
#pragma unroll
      for (int j = i + 1; j < m; j++)
        c2 += X[i][i] * X[j][j] - X[i][j] * X[j][i];
    c3 = X[0][0] * (X[1][1] * X[2][2] - X[1][2] * X[2][1]) -
         X[0][1] * (X[1][0] * X[2][2] - X[1][2] * X[2][0]) +
         X[0][2] * (X[1][0] * X[2][1] - X[1][1] * X[2][0]);
  } else {
    // the 2x2 minors of rows (0, 1) and of rows (2, 3) give c2 (the two
    // principal ones), the four principal 3x3 minors (expanded along the
    // third row) and det X (Laplace along rows (0, 1))
    // (explicit fused multiply-adds: the same rounding in every kernel that
    // inlines this, whatever contraction the compiler would choose there)
    const int r2 = m == 4 ? 2 : 0, r3 = m == 4 ? 3 : 0;
    auto mn = [](double a, double b, double c, double d) { return fma(a, b, -(c * d)); };
    auto s = [&](int a, int b) { return mn(X[0][a], X[1][b], X[0][b], X[1][a]); };
    auto t = [&](int a, int b) { return mn(X[r2][a], X[r3][b], X[r2][b], X[r3][a]); };
    // with Z, X[1][3] = X[2][3] = 0 drop out of the minors that contain them
    const double s01 = s(0, 1), s02 = s(0, 2), s12 = s(1, 2);
    const double s03 = Z ? -(X[0][r3] * X[1][0]) : s(0, 3);
    const double s13 = Z ? -(X[0][r3] * X[1][1]) : s(1, 3);
    const double s23 = Z ? -(X[0][r3] * X[1][r2]) : s(2, 3);
    const double t01 = t(0, 1), t02 = t(0, 2), t12 = t(1, 2);
    const double t03 = Z ? X[r2][0] * X[r3][r3] : t(0, 3);
    const double t13 = Z ? X[r2][1] * X[r3][r3] : t(1, 3);
    const double t23 = Z ? X[r2][r2] * X[r3][r3] : t(2, 3);
    c2 = ((s01 + t23) + (mn(X[0][0], X[r2][r2], X[0][r2], X[r2][0]) +
                         mn(X[0][0], X[r3][r3], X[0][r3], X[r3][0]))) +
         (mn(X[1][1], X[r2][r2], X[1][r2], X[r2][1]) +
          (Z ? X[1][1] * X[r3][r3] : mn(X[1][1], X[r3][r3], X[1][r3], X[r3][1])));
    auto e3 = [](double a, double sa, double b, double sb, double c, double sc) {
      return fma(c, sc, fma(a, sa, -(b * sb)));
    };
    c3 = (e3(X[r2][r2], s01, X[r2][1], s02, X[r2][0], s12) +
          e3(X[r3][r3], s01, X[r3][1], s03, X[r3][0], s13)) +
         (e3(X[0][0], t23, X[0][r2], t03, X[0][r3], t02) +
          (Z ? fma(X[1][1], t23, -(X[1][r2] * t13))
             : e3(X[1][1], t23, X[1][r2], t13, X[1][r3], t12)));
    c4 = (mn(s01, t23, s02, t13) + fma(s03, t12, s12 * t03)) - fma(s13, t02, -(s23 * t01));
  }
  // p(x) = x^m - c1 x^(m-1) + c2 x^(m-2) - c3 x^(m-3) [+ c4]
  double R = 0.0;
#pragma unroll
  for (int i = 0; i < m; i++) {
    double rs = 0.0;
#pragma unroll
    for (int j = 0; j < m; j++)
      rs += fabs(X[i][j]);
    R = fmax(R, rs);
  }
  const double Rs = R * (1.0 + 1e-12) + 1e-300;
  // Starting point in FP32: Laguerre on the scaled polynomial p(Rs y) / Rs^m
  // (O(1) coefficients, every root |y| <= 1) from y = 1 down to ~1e-4.  On
  // this GPU FP32 runs at full rate beside the FP64 pipe, so the FP64
  // iteration below, started just above that estimate, needs one or two
  // steps instead of ~5 from the bound.  A failed FP32 run (non-finite or out
  // of (0, 1]) leaves the start at the bound.
  double x = Rs;
  {
    // scaled coefficients in FP32 (a coefficient beyond the FP32 range makes
    // the start fail, and the FP64 iteration then starts at the bound)
    const float iR = 1.0f / (float)Rs;
    float cs[4];
    cs[0] = -(float)c1 * iR;
    cs[1] = ((float)c2 * iR) * iR;
    cs[2] = -(((float)c3 * iR) * iR) * iR;
    cs[3] = ((((float)c4 * iR) * iR) * iR) * iR;
    float y = 1.0f;
    for (int it = 0; it < 24; it++) {
      float p = 1.0f, dp = 0.0f, d2p = 0.0f;
#pragma unroll
      for (int k = 0; k < m; k++) {
        d2p = fmaf(d2p, y, 2.0f * dp);
        dp = fmaf(dp, y, p);
        p = fmaf(p, y, cs[k]);
      }
      if (p == 0.0f)
        break;
      float ip = 1.0f / p;
      float G = dp * ip;
      float H = fmaf(G, G, -(d2p * ip));
      float disc = fmaxf((m - 1) * fmaf((float)m, H, -(G * G)), 0.0f);
      float a = m / (G + copysignf(sqrtf(disc), G));
      y -= a;
      if (!(fabsf(a) > 1e-4f * fabsf(y)))
        break;
    }
    if (y > 0.0f && y <= 1.0f)
      x = fmin((double)y * (1.0 + 4e-6), 1.0) * Rs;
  }
  for (int it = 0; it < 16; it++) {
    double p = 1.0, dp = 0.0, d2p = 0.0;
    const double cf[4] = {-c1, c2, -c3, c4};
#pragma unroll
    for (int k = 0; k < m; k++) {
      d2p = fma(d2p, x, 2.0 * dp);
      dp = fma(dp, x, p);
      p = fma(p, x, cf[k]);
    }
    if (p == 0.0)
      break;
    double ip = 1.0 / p;
    double G = dp * ip;
    double H = fma(G, G, -(d2p * ip));
    double disc = fmax((m - 1) * fma((double)m, H, -(G * G)), 0.0);
    double a = m / (G + copysign(sqrt(disc), G));
    x -= a;
    if (!(fabs(a) > 1e-5 * fabs(x)))  // cubic convergence: the error is now ~|a|^3
      break;
  }
  lam = x;
  if (!(x > 0.0) || !(x <= R * (1.0 + 1e-9)))
    return false;
  // deflate and certify: all other roots strictly inside |z| < (1-1e-9) lam
  double l = x * (1.0 - 1e-9);
  double q2 = -c1 + x, q1 = fma(x, q2, c2);
  if (m == 3) {
    const double il = 1.0 / l;
    double a1 = q2 * il, a0 = q1 * il * il;
    return fabs(a0) < 1.0 && fabs(a1) < 1.0 + a0;
  }
  double q0 = fma(x, q1, -c3);
  const double il = 1.0 / l;
  double a2 = q2 * il, a1 = q1 * il * il, a0 = q0 * il * il * il;
  return (1.0 + a2 + a1 + a0 > 0.0) && (1.0 - a2 + a1 - a0 > 0.0) && fabs(a0) < 1.0 &&
         fabs(a0 * a0 - 1.0) > fabs(a0 * a2 - a1);
}

// max |eigenvalue| of the GPR system in direction d (system/eig.cpp:8-77):
// |v_d| + sqrt(max |eig(Xi1 Xi2)|).  Xi1 (4x5) and Xi2 (5x4) are assembled
// implicitly: Xi = Xi1 Xi2 is formed directly from its nonzero blocks.
// Xo (m x m, row-major) and l2o, when given, receive Xi and its dominant
// eigenvalue (for the adjoint's wave-speed derivative).
template <bool TH>
GPR_D double max_abs_eigs(const double *q, const Prim<TH> &s, int d, const DevPar &P,
                          double *Xo = nullptr, double *l2o = nullptr) {
  const double *A = q + 5;
  const double r = s.r, ir = s.ir;
  // G = A^T A (row d only needed) and dsigma/dA (state.cpp:43-56):
  // ret = A devG with column d doubled + 1/3 A(:,d) G(d,:) + G(d,d) A
  double Gd[3];
#pragma unroll
  for (int j = 0; j < 3; j++)
    Gd[j] = A[d] * A[j] + A[3 + d] * A[3 + j] + A[6 + d] * A[6 + j];
  double ret[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      ret[3 * i + j] = (j == d ? 2.0 : 1.0) * s.AdG[3 * i + j] +
                       (1.0 / 3.0) * A[3 * i + d] * Gd[j] + Gd[d] * A[3 * i + j];
  // Xi1 top-right block: -dsigmadA/rho = cs2 ret^T  ->  Mt[i][j] = cs2 ret[j][i]
  double sg[3];
  sigma_col(q, s, d, sg);
  // dsigma/drho = (1/rho + dcs2/drho / cs2) sigma = (1 + beta)/rho sigma
  double fr = (1.0 + P.beta) * ir;
  double dsr[3] = {fr * sg[0], fr * sg[1], fr * sg[2]};
  // c0^2 = (p/rho^2 - dE/drho) / dE/dp   (waves/speeds.cpp:8-18)
  const EosRho &e = s.e;
  double rG = r * e.G, irG2 = s.irG * s.irG;
  double dnum = e.dpr * rG + (e.G + r * e.dG) * (s.p - e.pr);
  double dedr = e.der - dnum * irG2;
  double cs2 = s.cs2;
  double dC0 = 0.0;
  if (P.beta != 0.0) {
    double dcs2 = P.beta * ir * cs2;
    dC0 = (1.0 - P.beta / e.G) * dcs2 + P.beta / (e.G * e.G) * e.dG * cs2;
  }
  double dEdr = dedr + 0.25 * dC0 * s.devGsq;
  double c02 = (s.p * ir * ir - dEdr) * rG;  // dE/dp = 1/(rho Gamma)
  // Xi2 row 1: b = sigma - rho dsigma/drho + rho c0^2 e_d ; h = calpha2 T Gamma
  double b[3] = {sg[0] - r * dsr[0], sg[1] - r * dsr[1], sg[2] - r * dsr[2]};
  b[d] += r * c02;
  constexpr int m = TH ? 4 : 3;
  double X[m][m];
  // rows 0..2, cols 0..2: rho a_i delta_c0 + delta_i0 b_c/rho + (Mt A)_ic
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double acc = cs2 * (ret[i] * A[c] + ret[3 + i] * A[3 + c] + ret[6 + i] * A[6 + c]);
      if (c == 0)
        acc += -dsr[i];  // rho * (-dsigma_i/drho / rho)
      if (i == 0)
        acc += b[c] * ir;
      X[i][c] = acc;
    }
  if (TH) {
    double h = P.calpha2 * s.T * e.G;
    double tp = ir * s.irG * P.icv;  // dT/dp / rho
    double dTr = -dnum * irG2 * P.icv;
    X[0][m - 1] = h * ir;
    X[1][m - 1] = 0.0;
    X[2][m - 1] = 0.0;
    X[m - 1][0] = dTr + tp * b[0];
    X[m - 1][1] = tp * b[1];
    X[m - 1][2] = tp * b[2];
    X[m - 1][m - 1] = tp * h;
  }
  if (Xo) {
#pragma unroll
    for (int i = 0; i < m; i++)
#pragma unroll
      for (int c = 0; c < m; c++)
        Xo[i * m + c] = X[i][c];
  }
  double l2;
  if (!max_eig_laguerre<m, TH>(X, l2))
    l2 = max_abs_eig<m>(X);  // QR fallback: complex or multiple dominant roots
  if (l2o)
    *l2o = l2;
  double lam = sqrt(l2);
  double vd = s.v[d];
  return vd > 0 ? vd + lam : lam - vd;
}

}  // namespace gpr
