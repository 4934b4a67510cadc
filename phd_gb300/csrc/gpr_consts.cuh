// gpr_consts.cuh - quadrature, WENO and space-time DG constants for N = 2
// Gauss-Legendre nodes, built once on the host in FP64 and passed to every
// kernel by value (kernel parameters live in the constant bank, so no
// per-device upload and nothing to do before stream capture).
//
// Restates etc/globals.cpp:16-50, poly/basis.cpp:7-72,
// weno/weno_matrices.cpp:9-42 and dg/dg_matrices.cpp:29-53 of the reference.
#pragma once

#include <math.h>

namespace gpr {

constexpr int NN = 2;  // Gauss nodes / basis functions (the reference's N)

struct Consts {
  double nodes[NN], w[NN];       // Gauss-Legendre on [0, 1]
  double endv[2][NN];            // psi_j(0), psi_j(1)
  double derv[NN][NN];           // psi_j'(x_i)
  double mLinv[NN][NN], mRinv[NN][NN];  // WENO stencil inverses
  double sig[NN][NN];            // oscillation indicator
  double dgder[NN][NN];          // <psi_i, psi_j'>
  double dgmat[NN][NN];          // DG_END - DG_DER^T
  double dgmatinv[NN][NN];       // (DG_END - DG_DER^T)^-1
  double wprod2[NN][NN];         // w_i w_j
  // predictor stopping rules: Picard |dq| <= dg_tol (1 + |q|) within dg_it
  // iterations (options.h:29-30), stiff-source Newton |delta| <= stiff_tol
  // (1 + |q|) within stiff_it; the differentiable step tightens them so the
  // predictor result is its fixed point to rounding
  double dg_tol, stiff_tol;
  int dg_it, stiff_it;
};

// Lagrange basis on the two nodes: psi_0(x) = (x - x1)/(x0 - x1), ...
inline Consts make_consts() {
  Consts c;
  const double s = 1.0 / sqrt(3.0);
  c.nodes[0] = (1.0 - s) / 2.0;
  c.nodes[1] = (1.0 + s) / 2.0;
  c.w[0] = c.w[1] = 0.5;
  const double x0 = c.nodes[0], x1 = c.nodes[1];
  const double h = x1 - x0;
  // psi_0 = (x1 - x)/h, psi_1 = (x - x0)/h
  auto psi = [&](int j, double x) { return j == 0 ? (x1 - x) / h : (x - x0) / h; };
  auto dpsi = [&](int j) { return j == 0 ? -1.0 / h : 1.0 / h; };
  // antiderivative with zero constant term
  auto Psi = [&](int j, double x) {
    return j == 0 ? (x1 * x - 0.5 * x * x) / h : (0.5 * x * x - x0 * x) / h;
  };
  for (int j = 0; j < NN; j++) {
    c.endv[0][j] = psi(j, 0.0);
    c.endv[1][j] = psi(j, 1.0);
  }
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      c.derv[i][j] = dpsi(j);
  // WENO stencil matrices (weno_matrices.cpp:9-28): mL(i,j) = int over cell
  // i-N+1 of psi_j, mR(i,j) = int over cell i.
  double mL[NN][NN], mR[NN][NN];
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++) {
      mL[i][j] = Psi(j, i - NN + 2) - Psi(j, i - NN + 1);
      mR[i][j] = Psi(j, i + 1) - Psi(j, i);
    }
  auto inv2 = [](double m[NN][NN], double out[NN][NN]) {
    double det = m[0][0] * m[1][1] - m[0][1] * m[1][0];
    out[0][0] = m[1][1] / det;
    out[0][1] = -m[0][1] / det;
    out[1][0] = -m[1][0] / det;
    out[1][1] = m[0][0] / det;
  };
  inv2(mL, c.mLinv);
  inv2(mR, c.mRinv);
  // oscillation indicator (weno_matrices.cpp:30-42): int_0^1 psi_i' psi_j'
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      c.sig[i][j] = dpsi(i) * dpsi(j);
  // DG matrices (dg_matrices.cpp:29-53, globals.cpp:42-44)
  double dgmat[NN][NN];
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++) {
      if (i == j)
        c.dgder[i][j] = (psi(i, 1.0) * psi(i, 1.0) - psi(i, 0.0) * psi(i, 0.0)) / 2.0;
      else
        c.dgder[i][j] = c.w[i] * dpsi(j);
    }
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      dgmat[i][j] = psi(i, 1.0) * psi(j, 1.0) - c.dgder[j][i];
  inv2(dgmat, c.dgmatinv);
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      c.dgmat[i][j] = dgmat[i][j];
  for (int i = 0; i < NN; i++)
    for (int j = 0; j < NN; j++)
      c.wprod2[i][j] = c.w[i] * c.w[j];
  c.dg_tol = 6e-6;
  c.dg_it = 50;
  c.stiff_tol = 1e-11;
  c.stiff_it = 60;
  return c;
}

}  // namespace gpr
