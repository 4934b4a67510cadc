// gpr_adjoint.cuh - hand-written adjoint (reverse mode) of the 1D ADER-WENO
// step of gpr_kernels.cuh, for the batched packing of many instances.
//
// Forward step n (per instance, solvers/iterator.cpp:109-151 with
// solvers/steppers.cpp:10-48):
//   dt   = CFL dx / max_c lambda(u_c)        (x 0.2 for the first steps,
//                                             clipped to tf - t)
//   ub   = boundaries(u)                     (etc/grid.cpp:12-125)
//   wh   = WENO(ub)                          (weno/weno.cpp:4-157)
//   qh   = fixed point of q = DG_U^-1 (W w + dt R(q))   (dg/dg1.cpp:8-114)
//   u'   = u + FV(qh, dt)                    (fv/fv.cpp:11-160)
//   u+   = renorm(u')                        (solvers/utils.cpp:6-23)
// Backward step n: given the cotangent of u+, produce the cotangent of u, add
// the material-parameter cotangents, and carry the cotangent of the clock t
// (the last step's dt = tf - t depends on every earlier dt).
//
// The predictor is differentiated at its converged fixed point by one
// transposed linear solve per cell, (DG_U - dt dR/dq)^T mu = qbar, iterated
// as the transposed Picard map mu <- DG_U^-T (qbar + dt dR/dq^T mu), which
// contracts exactly when the forward Picard iteration does.  The WENO
// weights, the Rusanov flux with its max-wave-speed switch, the path integral
// of B, the renormalisation and the CFL time step are differentiated exactly.
//
// The point functions (F, S and lambda along x, for the differentiable
// model: stiffened-gas EOS, Newtonian viscosity, beta = 0, Tref = 0) enter
// only through products with one cotangent, so the backward step applies
// hand-written reverse sweeps of them (point_vjp; pcache_vjp over a cached
// primal inside the transposed predictor iteration).  Forward-mode dual
// numbers over the same restatement give full Jacobians where they are
// needed: the dense fallback solve, the CFL argmax cell, and as the test
// reference of the reverse sweeps.  The eigenvalue derivative of the
// acoustic tensor uses d lambda = tr(adj(lambda I - X) dX) /
// tr(adj(lambda I - X)) for the simple dominant eigenvalue.
#pragma once

#include "gpr_kernels.cuh"

namespace gpr {

// Differentiable material fields (DevPar members).  The host maps user
// parameters (mu, cs, calpha, gamma, ...) onto them by the chain rule.
constexpr int NPD = 6;
enum { PD_GAMMA = 0, PD_IG = 1, PD_B02 = 2, PD_TH1C = 3, PD_CALPHA2 = 4, PD_IKAPPA = 5 };

// ---------------------------------------------------------------------------
// Dual numbers with one tangent.
struct Dual {
  double v, d;
};
GPR_D Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
GPR_D Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
GPR_D Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
GPR_D Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
GPR_D Dual operator+(Dual a, double b) { return Dual{a.v + b, a.d}; }
GPR_D Dual operator+(double b, Dual a) { return Dual{a.v + b, a.d}; }
GPR_D Dual operator-(Dual a, double b) { return Dual{a.v - b, a.d}; }
GPR_D Dual operator-(double b, Dual a) { return Dual{b - a.v, -a.d}; }
GPR_D Dual operator*(Dual a, double b) { return Dual{a.v * b, a.d * b}; }
GPR_D Dual operator*(double b, Dual a) { return Dual{a.v * b, a.d * b}; }
GPR_D Dual operator/(Dual a, Dual b) {
  double iv = 1.0 / b.v, r = a.v * iv;
  return Dual{r, (a.d - r * b.d) * iv};
}
GPR_D Dual operator/(double a, Dual b) {
  double iv = 1.0 / b.v, r = a * iv;
  return Dual{r, -r * b.d * iv};
}
GPR_D Dual dsqrt(Dual a) {
  double s = sqrt(a.v);
  return Dual{s, 0.5 * a.d / s};
}
GPR_D Dual dcbrt(Dual a) {
  double c = cbrt(a.v);
  return Dual{c, a.d / (3.0 * c * c)};
}

struct DPar {
  Dual gamma, iG, b02, th1c, calpha2, ikappa;
  double pINF, icv, dp0, dp1, dp2;
};

// p: index of the seeded material field, or < 0 for none
GPR_D DPar dpar_seed(const DevPar &P, int p) {
  DPar D;
  D.gamma = Dual{P.gamma, p == PD_GAMMA ? 1.0 : 0.0};
  D.iG = Dual{P.iG, p == PD_IG ? 1.0 : 0.0};
  D.b02 = Dual{P.b02, p == PD_B02 ? 1.0 : 0.0};
  D.th1c = Dual{P.th1c, p == PD_TH1C ? 1.0 : 0.0};
  D.calpha2 = Dual{P.calpha2, p == PD_CALPHA2 ? 1.0 : 0.0};
  D.ikappa = Dual{P.ikappa, p == PD_IKAPPA ? 1.0 : 0.0};
  D.pINF = P.pINF;
  D.icv = P.icv;
  D.dp0 = P.dp0;
  D.dp1 = P.dp1;
  D.dp2 = P.dp2;
  return D;
}

template <bool TH> struct DPrim {
  Dual r, ir, v[3], J[3], AdG[9], devGsq, G, irG, p, T;
};

// prim() of gpr_device.cuh for EOS 0 with beta = 0 and Tref = 0
// (state.cpp, eos.cpp, mg.cpp:126-139)
template <bool TH>
GPR_D void dprim(const Dual *q, const DPar &P, DPrim<TH> &s) {
  s.r = q[0];
  s.ir = 1.0 / s.r;
#pragma unroll
  for (int i = 0; i < 3; i++)
    s.v[i] = q[2 + i] * s.ir;
  const Dual *A = q + 5;
  Dual G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  Dual G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  Dual G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  Dual G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  Dual G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  Dual G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  Dual t = (G00 + G11 + G22) * (1.0 / 3.0);
  Dual D00 = G00 - t, D11 = G11 - t, D22 = G22 - t;
  s.devGsq = D00 * D00 + D11 * D11 + D22 * D22 + 2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    Dual a0 = A[3 * i], a1 = A[3 * i + 1], a2 = A[3 * i + 2];
    s.AdG[3 * i + 0] = a0 * D00 + a1 * G01 + a2 * G02;
    s.AdG[3 * i + 1] = a0 * G01 + a1 * D11 + a2 * G12;
    s.AdG[3 * i + 2] = a0 * G02 + a1 * G12 + a2 * D22;
  }
  s.G = P.gamma - 1.0;
  s.irG = s.ir * P.iG;
  Dual E1 = q[1] * s.ir - 0.5 * (s.v[0] * s.v[0] + s.v[1] * s.v[1] + s.v[2] * s.v[2]) -
            0.25 * (P.b02 * s.devGsq);
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      s.J[i] = q[14 + i] * s.ir;
    E1 = E1 - 0.5 * (P.calpha2 * (s.J[0] * s.J[0] + s.J[1] * s.J[1] + s.J[2] * s.J[2]));
  }
  Dual er = P.pINF * s.ir;
  s.p = (E1 - er) * (s.r * s.G) - P.pINF;
  s.T = (s.p + P.pINF) * s.irG * P.icv;
}

// sigma column 0: -rho cs2 (A devG)^T A(:,0)   (state.cpp:23-29)
template <bool TH>
GPR_D void dsigma0(const Dual *q, const DPrim<TH> &s, const DPar &P, Dual *sg) {
  const Dual *A = q + 5;
  Dual f = -(s.r * P.b02);
#pragma unroll
  for (int i = 0; i < 3; i++)
    sg[i] = f * (s.AdG[i] * A[0] + s.AdG[3 + i] * A[3] + s.AdG[6 + i] * A[6]);
}

// F_x(Q)   (equations.cpp:11-48)
template <bool TH, int V>
GPR_D void dflux0(const Dual *q, const DPrim<TH> &s, const DPar &P, Dual *F) {
  const Dual *A = q + 5;
  Dual sg[3];
  dsigma0<TH>(q, s, P, sg);
  Dual v0 = s.v[0];
#pragma unroll
  for (int k = 0; k < V; k++)
    F[k] = Dual{0.0, 0.0};
  F[0] = q[2];
  F[1] = v0 * (q[1] + s.p) - (sg[0] * s.v[0] + sg[1] * s.v[1] + sg[2] * s.v[2]);
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[2 + i] = v0 * q[2 + i] - sg[i];
  F[2] = F[2] + s.p;
#pragma unroll
  for (int i = 0; i < 3; i++)
    F[5 + 3 * i] = A[3 * i] * s.v[0] + A[3 * i + 1] * s.v[1] + A[3 * i + 2] * s.v[2];
  if (TH) {
    F[1] = F[1] + P.calpha2 * s.T * s.J[0];
#pragma unroll
    for (int i = 0; i < 3; i++)
      F[14 + i] = v0 * q[14 + i];
    F[14] = F[14] + s.T;
  }
}

GPR_D Dual ddet3(const Dual *A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

// S(Q) for Newtonian viscosity (equations.cpp:50-67, sources.cpp:13-93)
template <bool TH, int V>
GPR_D void dsource(const Dual *q, const DPrim<TH> &s, const DPar &P, Dual *S) {
#pragma unroll
  for (int k = 0; k < V; k++)
    S[k] = Dual{0.0, 0.0};
  S[2] = Dual{P.dp0, 0.0};
  S[3] = Dual{P.dp1, 0.0};
  S[4] = Dual{P.dp2, 0.0};
  Dual dA = ddet3(q + 5);
  Dual cb = dcbrt(dA);
  Dual th = dA * cb * cb * P.th1c;  // det(A)^(5/3) rho0 / (2 mu)
  Dual f = -(P.b02 * th);
#pragma unroll
  for (int i = 0; i < 9; i++)
    S[5 + i] = s.AdG[i] * f;
  if (TH) {
    Dual g = -(P.calpha2 * s.T * P.ikappa);
#pragma unroll
    for (int i = 0; i < 3; i++)
      S[14 + i] = g * s.J[i];
  }
}

// adjugate of a small matrix (adj[j][i] = cofactor (i, j))
GPR_D double det3m(double a, double b, double c, double d, double e, double f, double g,
                   double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

template <int m> GPR_D void adjugate(const double (&M)[m][m], double (&adj)[m][m]);

template <> GPR_D void adjugate<3>(const double (&M)[3][3], double (&adj)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      int r0 = i == 0 ? 1 : 0, r1 = i == 2 ? 1 : 2;
      int c0 = j == 0 ? 1 : 0, c1 = j == 2 ? 1 : 2;
      double minor = M[r0][c0] * M[r1][c1] - M[r0][c1] * M[r1][c0];
      adj[j][i] = ((i + j) & 1) ? -minor : minor;
    }
}

template <> GPR_D void adjugate<4>(const double (&M)[4][4], double (&adj)[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int r[3], c[3];
      int nr = 0, nc = 0;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        if (k != i)
          r[nr++] = k;
        if (k != j)
          c[nc++] = k;
      }
      double minor = det3m(M[r[0]][c[0]], M[r[0]][c[1]], M[r[0]][c[2]], M[r[1]][c[0]],
                           M[r[1]][c[1]], M[r[1]][c[2]], M[r[2]][c[0]], M[r[2]][c[1]],
                           M[r[2]][c[2]]);
      adj[j][i] = ((i + j) & 1) ? -minor : minor;
    }
}

// lambda_x(Q) = |v_x| + sqrt(max eig(Xi1 Xi2)) (system/eig.cpp:8-77), the
// restatement of max_abs_eigs for EOS 0 and beta = 0.  The value of the
// dominant eigenvalue comes from the same solver as the forward step.
template <bool TH> struct Xi {
  static constexpr int m = TH ? 4 : 3;
  static constexpr int ND = m * m + 1;  // eigen data: l2, then Y (m x m)
};

template <bool TH>
GPR_D void dxi0(const Dual *q, const DPrim<TH> &s, const DPar &P, Dual (&X)[Xi<TH>::m][Xi<TH>::m]) {
  constexpr int m = Xi<TH>::m;
  const Dual *A = q + 5;
  Dual Gd[3];
#pragma unroll
  for (int j = 0; j < 3; j++)
    Gd[j] = A[0] * A[j] + A[3] * A[3 + j] + A[6] * A[6 + j];
  Dual ret[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      ret[3 * i + j] = (j == 0 ? 2.0 : 1.0) * s.AdG[3 * i + j] +
                       (1.0 / 3.0) * (A[3 * i] * Gd[j]) + Gd[0] * A[3 * i + j];
  Dual sg[3];
  dsigma0<TH>(q, s, P, sg);
  Dual dsr[3] = {s.ir * sg[0], s.ir * sg[1], s.ir * sg[2]};
  // EOS 0: dp_ref/drho = 0, dGamma/drho = 0, de_ref/drho = -pINF / rho^2
  Dual irG2 = s.irG * s.irG;
  Dual dnum = s.G * (s.p + P.pINF);
  Dual dedr = -(P.pINF * (s.ir * s.ir)) - dnum * irG2;
  Dual rG = s.r * s.G;
  Dual c02 = (s.p * (s.ir * s.ir) - dedr) * rG;
  Dual b[3] = {sg[0] - s.r * dsr[0], sg[1] - s.r * dsr[1], sg[2] - s.r * dsr[2]};
  b[0] = b[0] + s.r * c02;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      Dual acc = P.b02 * (ret[i] * A[c] + ret[3 + i] * A[3 + c] + ret[6 + i] * A[6 + c]);
      if (c == 0)
        acc = acc - dsr[i];
      if (i == 0)
        acc = acc + b[c] * s.ir;
      X[i][c] = acc;
    }
  if constexpr (TH) {
    Dual h = P.calpha2 * s.T * s.G;
    Dual tp = s.ir * s.irG * P.icv;
    Dual dTr = -(dnum * irG2 * P.icv);
    X[0][m - 1] = h * s.ir;
    X[1][m - 1] = Dual{0.0, 0.0};
    X[2][m - 1] = Dual{0.0, 0.0};
    X[m - 1][0] = dTr + tp * b[0];
    X[m - 1][1] = tp * b[1];
    X[m - 1][2] = tp * b[2];
    X[m - 1][m - 1] = tp * h;
  }
}

// Eigen data of the dominant eigenvalue l2 of X: eig[0] = l2,
// eig[1 + i m + j] = Y[i][j] with d l2 = sum_ij Y[i][j] dX[i][j],
// Y = adj(l2 I - X)^T / tr(adj(l2 I - X)).
template <int m> GPR_D void xi_eigdata_l2(const double (&Xv)[m][m], double l2, double *eig) {
  double M[m][m], adj[m][m];
#pragma unroll
  for (int i = 0; i < m; i++)
#pragma unroll
    for (int j = 0; j < m; j++)
      M[i][j] = (i == j ? l2 : 0.0) - Xv[i][j];
  adjugate<m>(M, adj);
  double den = 0.0;
#pragma unroll
  for (int i = 0; i < m; i++)
    den += adj[i][i];
  double iden = 1.0 / den;
  eig[0] = l2;
#pragma unroll
  for (int i = 0; i < m; i++)
#pragma unroll
    for (int j = 0; j < m; j++)
      eig[1 + i * m + j] = adj[j][i] * iden;
}

template <int m> GPR_D void xi_eigdata(const double (&Xv)[m][m], double *eig) {
  double Xc[m][m];
#pragma unroll
  for (int i = 0; i < m; i++)
#pragma unroll
    for (int j = 0; j < m; j++)
      Xc[i][j] = Xv[i][j];
  double l2;
  if (!max_eig_laguerre<m>(Xc, l2))
    l2 = max_abs_eig<m>(Xc);
  xi_eigdata_l2<m>(Xv, l2, eig);
}

// lambda with its tangent; eig: eigen data of X (computed here when null)
template <bool TH>
GPR_D Dual dlambda0(const Dual *q, const DPrim<TH> &s, const DPar &P,
                    const double *eig = nullptr) {
  constexpr int m = Xi<TH>::m;
  Dual X[m][m];
  dxi0<TH>(q, s, P, X);
  double loc[Xi<TH>::ND];
  if (!eig) {
    double Xv[m][m];
#pragma unroll
    for (int i = 0; i < m; i++)
#pragma unroll
      for (int j = 0; j < m; j++)
        Xv[i][j] = X[i][j].v;
    xi_eigdata<m>(Xv, loc);
    eig = loc;
  }
  double dl2 = 0.0;
#pragma unroll
  for (int i = 0; i < m; i++)
#pragma unroll
    for (int j = 0; j < m; j++)
      dl2 += eig[1 + i * m + j] * X[i][j].d;
  Dual lam = dsqrt(Dual{eig[0], dl2});
  Dual v0 = s.v[0];
  return v0.v > 0 ? v0 + lam : lam - v0;
}

// One tangent of the point functions at state qp: k < V seeds state
// variable k, k >= V seeds material field k - V.
template <class L>
GPR_D void point_tangent(const double *qp, int k, const DevPar &P, Dual *F, Dual *S,
                         Dual *lam, const double *eig = nullptr) {
  constexpr int V = L::V;
  Dual q[V];
#pragma unroll
  for (int j = 0; j < V; j++)
    q[j] = Dual{qp[j], j == k ? 1.0 : 0.0};
  DPar D = dpar_seed(P, k - V);
  DPrim<L::THERMAL> s;
  dprim<L::THERMAL>(q, D, s);
  if (F)
    dflux0<L::THERMAL, V>(q, s, D, F);
  if (S)
    dsource<L::THERMAL, V>(q, s, D, S);
  if (lam)
    *lam = dlambda0<L::THERMAL>(q, s, D, eig);
}

// ---------------------------------------------------------------------------
// Reverse mode of the point functions: for cotangents Fb (of F_x), Sb (of S)
// and lb (of lambda_x) at state q,
//   qb  += (dF/dq)^T Fb + (dS/dq)^T Sb + lb dlambda/dq,
//   thb += the same with respect to the six material fields,
// the exact derivative of dprim / dflux0 / dsource / dlambda0 above (same
// operations, traversed backwards), at ~3 evaluations of the point functions
// instead of one dual evaluation per column.  HF / HS / HL select the terms;
// eig: eigen data of the acoustic tensor (xi_eigdata; computed here when
// null); thb may be null.
template <class L, bool HF, bool HS, bool HL>
GPR_D void point_vjp(const double *q, const DevPar &P, const double *Fb, const double *Sb,
                     double lb, const double *eig, double *qb, double *thb) {
  constexpr bool TH = L::THERMAL;
  constexpr int m = Xi<TH>::m;
  const double *A = q + 5;
  // ---- primal (dprim)
  const double r = q[0], ir = 1.0 / r;
  double v[3], J[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 3; i++)
    v[i] = q[2 + i] * ir;
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      J[i] = q[14 + i] * ir;
  }
  const double G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  const double G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  const double G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  const double G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  const double G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  const double G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  const double tG = (G00 + G11 + G22) * (1.0 / 3.0);
  const double Dm[3][3] = {{G00 - tG, G01, G02}, {G01, G11 - tG, G12}, {G02, G12, G22 - tG}};
  const double devGsq = Dm[0][0] * Dm[0][0] + Dm[1][1] * Dm[1][1] + Dm[2][2] * Dm[2][2] +
                        2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
  double AdG[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      AdG[3 * i + j] = A[3 * i] * Dm[0][j] + A[3 * i + 1] * Dm[1][j] + A[3 * i + 2] * Dm[2][j];
  const double Gm1 = P.gamma - 1.0, irG = ir * P.iG;
  const double vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const double Jsq = J[0] * J[0] + J[1] * J[1] + J[2] * J[2];
  double E1 = q[1] * ir - 0.5 * vsq - 0.25 * (P.b02 * devGsq);
  if (TH)
    E1 = E1 - 0.5 * (P.calpha2 * Jsq);
  const double er = P.pINF * ir;
  const double p = (E1 - er) * (r * Gm1) - P.pINF;
  const double T = (p + P.pINF) * irG * P.icv;
  // sigma column 0 (dsigma0)
  const double sgf = -(r * P.b02);
  double sgm[3], sg[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    sgm[i] = AdG[i] * A[0] + AdG[3 + i] * A[3] + AdG[6 + i] * A[6];
    sg[i] = sgf * sgm[i];
  }
  // ---- adjoints
  double rb = 0.0, irb = 0.0, vb[3] = {0.0, 0.0, 0.0}, Jb[3] = {0.0, 0.0, 0.0};
  double Ab[9], AdGb[9], sgb[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 9; k++) {
    Ab[k] = 0.0;
    AdGb[k] = 0.0;
  }
  double pb = 0.0, Tb = 0.0, Gm1b = 0.0, irGb = 0.0;
  double b02b = 0.0, ca2b = 0.0, th1cb = 0.0, ikb = 0.0, q1b = 0.0;
  double q2b[3] = {0.0, 0.0, 0.0}, qJb[3] = {0.0, 0.0, 0.0};
  if (HL) {
    // lambda = sqrt(l2) +- v0 (dlambda0), d l2 = sum Y dX
    double le[1 + m * m];
    const double *ed = eig;
    double X0[m][m];
    if (!ed) {
      Dual qd[L::V];
#pragma unroll
      for (int j = 0; j < L::V; j++)
        qd[j] = Dual{q[j], 0.0};
      DPar D = dpar_seed(P, -1);
      DPrim<TH> s;
      dprim<TH>(qd, D, s);
      Dual X[m][m];
      dxi0<TH>(qd, s, D, X);
#pragma unroll
      for (int i = 0; i < m; i++)
#pragma unroll
        for (int j = 0; j < m; j++)
          X0[i][j] = X[i][j].v;
      xi_eigdata<m>(X0, le);
      ed = le;
    }
    vb[0] += v[0] > 0 ? lb : -lb;
    const double l2b = 0.5 * lb / sqrt(ed[0]);
    double Xb[m][m];
#pragma unroll
    for (int i = 0; i < m; i++)
#pragma unroll
      for (int j = 0; j < m; j++)
        Xb[i][j] = l2b * ed[1 + i * m + j];
    // reverse of dxi0
    double Gd[3];
#pragma unroll
    for (int j = 0; j < 3; j++)
      Gd[j] = A[0] * A[j] + A[3] * A[3 + j] + A[6] * A[6 + j];
    double ret[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        ret[3 * i + j] = (j == 0 ? 2.0 : 1.0) * AdG[3 * i + j] +
                         (1.0 / 3.0) * (A[3 * i] * Gd[j]) + Gd[0] * A[3 * i + j];
    const double dsr[3] = {ir * sg[0], ir * sg[1], ir * sg[2]};
    const double irG2 = irG * irG;
    const double dnum = Gm1 * (p + P.pINF);
    const double dedr = -(P.pINF * (ir * ir)) - dnum * irG2;
    const double rG = r * Gm1;
    const double c02 = (p * (ir * ir) - dedr) * rG;
    double bv[3] = {sg[0] - r * dsr[0], sg[1] - r * dsr[1], sg[2] - r * dsr[2]};
    bv[0] = bv[0] + r * c02;
    double bb[3] = {0.0, 0.0, 0.0}, dsrb[3] = {0.0, 0.0, 0.0}, retb[9];
#pragma unroll
    for (int k = 0; k < 9; k++)
      retb[k] = 0.0;
    double dnumb = 0.0, irG2b = 0.0;
    if constexpr (TH) {
      const double h = P.calpha2 * T * Gm1;
      const double tp = ir * irG * P.icv;
      const double hb = Xb[0][m - 1] * ir + Xb[m - 1][m - 1] * tp;
      irb += Xb[0][m - 1] * h;
      const double tpb = Xb[m - 1][0] * bv[0] + Xb[m - 1][1] * bv[1] + Xb[m - 1][2] * bv[2] +
                         Xb[m - 1][m - 1] * h;
      const double dTrb = Xb[m - 1][0];
#pragma unroll
      for (int c = 0; c < 3; c++)
        bb[c] += Xb[m - 1][c] * tp;
      dnumb -= dTrb * irG2 * P.icv;
      irG2b -= dTrb * dnum * P.icv;
      irb += tpb * irG * P.icv;
      irGb += tpb * ir * P.icv;
      ca2b += hb * T * Gm1;
      Tb += hb * P.calpha2 * Gm1;
      Gm1b += hb * P.calpha2 * T;
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double xb = Xb[i][c];
        const double Mv = ret[i] * A[c] + ret[3 + i] * A[3 + c] + ret[6 + i] * A[6 + c];
        b02b += xb * Mv;
        const double f = xb * P.b02;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          retb[3 * k + i] += f * A[3 * k + c];
          Ab[3 * k + c] += f * ret[3 * k + i];
        }
        if (c == 0)
          dsrb[i] -= xb;
        if (i == 0) {
          bb[c] += xb * ir;
          irb += xb * bv[c];
        }
      }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      sgb[c] += bb[c];
      rb -= bb[c] * dsr[c];
      dsrb[c] -= bb[c] * r;
    }
    rb += bb[0] * c02;
    const double c02b = bb[0] * r;
    pb += c02b * (ir * ir) * rG;
    irb += c02b * p * 2.0 * ir * rG;
    const double dedrb = -c02b * rG;
    const double rGb = c02b * (p * (ir * ir) - dedr);
    rb += rGb * Gm1;
    Gm1b += rGb * r;
    irb -= dedrb * 2.0 * P.pINF * ir;
    dnumb -= dedrb * irG2;
    irG2b -= dedrb * dnum;
    Gm1b += dnumb * (p + P.pINF);
    pb += dnumb * Gm1;
    irGb += irG2b * 2.0 * irG;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      irb += dsrb[i] * sg[i];
      sgb[i] += dsrb[i] * ir;
    }
    double Gdb[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const double g = retb[3 * i + j];
        AdGb[3 * i + j] += (j == 0 ? 2.0 : 1.0) * g;
        Ab[3 * i] += g * (1.0 / 3.0) * Gd[j];
        Gdb[j] += g * (1.0 / 3.0) * A[3 * i];
        Gdb[0] += g * A[3 * i + j];
        Ab[3 * i + j] += g * Gd[0];
      }
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        Ab[3 * k] += Gdb[j] * A[3 * k + j];
        Ab[3 * k + j] += Gdb[j] * A[3 * k];
      }
  }
  if (HF) {
    // reverse of dflux0
    q2b[0] += Fb[0];
    const double f1 = Fb[1];
    vb[0] += f1 * (q[1] + p);
    q1b += f1 * v[0];
    pb += f1 * v[0];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      sgb[i] -= f1 * v[i];
      vb[i] -= f1 * sg[i];
    }
    if (TH) {
      ca2b += f1 * T * J[0];
      Tb += f1 * P.calpha2 * J[0];
      Jb[0] += f1 * P.calpha2 * T;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double f = Fb[2 + i];
      vb[0] += f * q[2 + i];
      q2b[i] += f * v[0];
      sgb[i] -= f;
    }
    pb += Fb[2];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double f = Fb[5 + 3 * i];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        Ab[3 * i + j] += f * v[j];
        vb[j] += f * A[3 * i + j];
      }
    }
    if (TH) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const double f = Fb[14 + i];
        vb[0] += f * q[14 + i];
        qJb[i] += f * v[0];
      }
      Tb += Fb[14];
    }
  }
  if (HS) {
    // reverse of dsource
    const double dA = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                      A[2] * (A[3] * A[7] - A[4] * A[6]);
    const double cb = cbrt(dA);
    const double th = dA * cb * cb * P.th1c;
    const double f = -(P.b02 * th);
    double fb = 0.0;
#pragma unroll
    for (int i = 0; i < 9; i++) {
      AdGb[i] += Sb[5 + i] * f;
      fb += Sb[5 + i] * AdG[i];
    }
    b02b -= fb * th;
    const double thb_ = -fb * P.b02;
    th1cb += thb_ * dA * cb * cb;
    const double dAb = thb_ * P.th1c * (5.0 / 3.0) * cb * cb;
    Ab[0] += dAb * (A[4] * A[8] - A[5] * A[7]);
    Ab[1] += dAb * (A[5] * A[6] - A[3] * A[8]);
    Ab[2] += dAb * (A[3] * A[7] - A[4] * A[6]);
    Ab[3] += dAb * (A[2] * A[7] - A[1] * A[8]);
    Ab[4] += dAb * (A[0] * A[8] - A[2] * A[6]);
    Ab[5] += dAb * (A[1] * A[6] - A[0] * A[7]);
    Ab[6] += dAb * (A[1] * A[5] - A[2] * A[4]);
    Ab[7] += dAb * (A[2] * A[3] - A[0] * A[5]);
    Ab[8] += dAb * (A[0] * A[4] - A[1] * A[3]);
    if (TH) {
      const double g = -(P.calpha2 * T * P.ikappa);
      double gb = 0.0;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        gb += Sb[14 + i] * J[i];
        Jb[i] += Sb[14 + i] * g;
      }
      ca2b -= gb * T * P.ikappa;
      Tb -= gb * P.calpha2 * P.ikappa;
      ikb -= gb * P.calpha2 * T;
    }
  }
  // reverse of dsigma0
  {
    const double sgfb = sgb[0] * sgm[0] + sgb[1] * sgm[1] + sgb[2] * sgm[2];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double f = sgb[i] * sgf;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        AdGb[3 * k + i] += f * A[3 * k];
        Ab[3 * k] += f * AdG[3 * k + i];
      }
    }
    rb -= sgfb * P.b02;
    b02b -= sgfb * r;
  }
  // reverse of dprim
  pb += Tb * irG * P.icv;
  irGb += Tb * (p + P.pINF) * P.icv;
  const double E1b = pb * (r * Gm1);
  const double erb = -E1b;
  rb += pb * (E1 - er) * Gm1;
  Gm1b += pb * (E1 - er) * r;
  irb += erb * P.pINF;
  q1b += E1b * ir;
  irb += E1b * q[1];
#pragma unroll
  for (int i = 0; i < 3; i++)
    vb[i] -= E1b * v[i];
  b02b -= 0.25 * E1b * devGsq;
  const double devGsqb = -0.25 * E1b * P.b02;
  if (TH) {
    ca2b -= 0.5 * E1b * Jsq;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Jb[i] -= E1b * P.calpha2 * J[i];
      qJb[i] += Jb[i] * ir;
      irb += Jb[i] * q[14 + i];
    }
  }
  irb += irGb * P.iG;
  const double iGb = irGb * ir;
  // AdG = A Dm
  double Dmb[3][3];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < 3; i++)
        s += AdGb[3 * i + j] * A[3 * i + k];
      Dmb[k][j] = s;
    }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++)
      Ab[3 * i + k] += AdGb[3 * i] * Dm[k][0] + AdGb[3 * i + 1] * Dm[k][1] +
                       AdGb[3 * i + 2] * Dm[k][2];
  double D00b = Dmb[0][0] + devGsqb * 2.0 * Dm[0][0];
  double D11b = Dmb[1][1] + devGsqb * 2.0 * Dm[1][1];
  double D22b = Dmb[2][2] + devGsqb * 2.0 * Dm[2][2];
  const double G01b = Dmb[0][1] + Dmb[1][0] + devGsqb * 4.0 * G01;
  const double G02b = Dmb[0][2] + Dmb[2][0] + devGsqb * 4.0 * G02;
  const double G12b = Dmb[1][2] + Dmb[2][1] + devGsqb * 4.0 * G12;
  const double tb = -(D00b + D11b + D22b) * (1.0 / 3.0);
  const double G00b = D00b + tb, G11b = D11b + tb, G22b = D22b + tb;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double a0 = A[3 * k], a1 = A[3 * k + 1], a2 = A[3 * k + 2];
    Ab[3 * k] += 2.0 * G00b * a0 + G01b * a1 + G02b * a2;
    Ab[3 * k + 1] += 2.0 * G11b * a1 + G01b * a0 + G12b * a2;
    Ab[3 * k + 2] += 2.0 * G22b * a2 + G02b * a0 + G12b * a1;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    q2b[i] += vb[i] * ir;
    irb += vb[i] * q[2 + i];
  }
  rb -= irb * ir * ir;
  qb[0] += rb;
  qb[1] += q1b;
#pragma unroll
  for (int i = 0; i < 3; i++)
    qb[2 + i] += q2b[i];
#pragma unroll
  for (int k = 0; k < 9; k++)
    qb[5 + k] += Ab[k];
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      qb[14 + i] += qJb[i];
  }
  if (thb) {
    thb[PD_GAMMA] += Gm1b;
    thb[PD_IG] += iGb;
    thb[PD_B02] += b02b;
    thb[PD_TH1C] += th1cb;
    thb[PD_CALPHA2] += ca2b;
    thb[PD_IKAPPA] += ikb;
  }
}

// ---------------------------------------------------------------------------
// B_x(v) x (bdot, d = 0, no level sets): transposes.
template <int V>
GPR_D void bdot0_xT(const double *v, const double *yb, double *xb) {  // xb += B^T yb
#pragma unroll
  for (int r = 0; r < 3; r++) {
    xb[6 + 3 * r] += -v[1] * yb[5 + 3 * r] + v[0] * yb[6 + 3 * r];
    xb[7 + 3 * r] += -v[2] * yb[5 + 3 * r] + v[0] * yb[7 + 3 * r];
  }
}

GPR_D void bdot0_vT(const double *x, const double *yb, double *vb) {  // vb = d(B(v)x)/dv^T yb
  double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
  for (int r = 0; r < 3; r++) {
    a += x[6 + 3 * r] * yb[6 + 3 * r] + x[7 + 3 * r] * yb[7 + 3 * r];
    b -= x[6 + 3 * r] * yb[5 + 3 * r];
    c -= x[7 + 3 * r] * yb[5 + 3 * r];
  }
  vb[0] = a;
  vb[1] = b;
  vb[2] = c;
}

// qb += (dv/dq)^T vb for v = q[2..4] / q[0]
GPR_D void vel_T(const double *q, const double *vb, double *qb, double scale) {
  double ir = 1.0 / q[0];
  double v0 = q[2] * ir, v1 = q[3] * ir, v2 = q[4] * ir;
  qb[0] -= scale * (vb[0] * v0 + vb[1] * v1 + vb[2] * v2) * ir;
  qb[2] += scale * vb[0] * ir;
  qb[3] += scale * vb[1] * ir;
  qb[4] += scale * vb[2] * ir;
}

// Sign of a ghost value relative to its source for the linear boundary codes
// (bc_value: slip / symmetric flip the normal momentum and, for symmetric,
// the A entries of row or column 0; stick flips the momentum).
GPR_D double bc_sign(int code, int k) {
  switch (code) {
  case GPR_BC_SLIP:
    return k == 2 ? -1.0 : 1.0;
  case GPR_BC_SYMMETRIC: {
    double s = k == 2 ? -1.0 : 1.0;
    if (k >= 5 && k < 14) {
      int r = (k - 5) / 3, c = (k - 5) % 3;
      if (r == 0)
        s = -s;
      if (c == 0)
        s = -s;
    }
    return s;
  }
  case GPR_BC_STICK:
    return (k >= 2 && k < 5) ? -1.0 : 1.0;
  default:
    return 1.0;
  }
}

// ---------------------------------------------------------------------------
// Forward-step recording.

// argmax cell of the CFL maximum (smallest packed index among the cells that
// attain it), from the per-cell values k_b_cfl_max stored
static __global__ void __launch_bounds__(256) k_adj_argmax(const double *__restrict__ mcell, long ncell,
                                                    const unsigned long long *__restrict__ mx,
                                                    unsigned int *__restrict__ amax, Batch B) {
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  int inst = B.inst_u[c];
  double m = mcell[c];
  if (m > 0.0 && (unsigned long long)__double_as_longlong(m) == mx[inst])
    atomicMin(amax + inst, (unsigned int)c);
}

// k_b_clock_finalize with recording: dt_mode 0 takes the CFL step (and
// writes it to dt_io if given), dt_mode 1 takes dt from dt_io (a step
// schedule held fixed).  tclk receives {t, dt, tf, cfl, count} of the step,
// aux {clipped, argmax cell}.
static __global__ void k_adj_clock_finalize(unsigned long long *__restrict__ mx, Batch B,
                                     double *__restrict__ dt_io, int dt_mode,
                                     double *__restrict__ tclk, double *__restrict__ aux,
                                     const unsigned int *__restrict__ amax) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B.ninst)
    return;
  double *c = B.clk + 5 * k;
  double t = c[0], tf = c[2], cfl = c[3];
  long count = (long)c[4];
  double dt = 0.0;
  bool clipped = false;
  if (t < tf) {
    if (dt_mode == 1) {
      dt = dt_io[k];
    } else {
      double MAX = __longlong_as_double((long long)mx[k]);
      dt = cfl / MAX;
      if (count <= 5)
        dt *= 0.2;
      if (t + dt > tf) {
        dt = tf - t;
        clipped = true;
      }
    }
  }
  c[1] = dt;
  mx[k] = 0ull;
  if (dt_mode == 0 && dt_io)
    dt_io[k] = dt;
  if (tclk) {
#pragma unroll
    for (int j = 0; j < 5; j++)
      tclk[5 * k + j] = c[j];
    aux[2 * k] = clipped ? 1.0 : 0.0;
    aux[2 * k + 1] = (amax && amax[k] != 0xffffffffu) ? (double)amax[k] : -1.0;
  }
}

// ---------------------------------------------------------------------------
// Backward-step kernels.  B.clk points at the recorded clock of the step.

// renormalisation: A+ = c A', c = cbrt(rho / (rho0 det A'))  (utils.cpp:6-23)
template <int V>
__global__ void k_adj_renorm(double *__restrict__ ub, const double *__restrict__ up, long ncell,
                             Batch B) {
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= ncell)
    return;
  int inst = B.inst_u[c];
  if (B.clk[5 * inst + 1] == 0.0)
    return;
  const double *q = up + c * V;
  double r = q[0];
  if (!(r > 0))
    return;
  double A[9];
#pragma unroll
  for (int k = 0; k < 9; k++)
    A[k] = q[5 + k];
  double dA = det3(A);
  double f = cbrt(r / (B.P[inst].rho0 * dA));
  double *g = ub + c * V;
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++)
    s += g[5 + k] * A[k];
  // df/dA = -f/3 A^-T, df/drho = f / (3 rho)
  double cof[9];
  cof[0] = A[4] * A[8] - A[5] * A[7];
  cof[1] = A[5] * A[6] - A[3] * A[8];
  cof[2] = A[3] * A[7] - A[4] * A[6];
  cof[3] = A[2] * A[7] - A[1] * A[8];
  cof[4] = A[0] * A[8] - A[2] * A[6];
  cof[5] = A[1] * A[6] - A[0] * A[7];
  cof[6] = A[1] * A[5] - A[2] * A[4];
  cof[7] = A[2] * A[3] - A[0] * A[5];
  cof[8] = A[0] * A[4] - A[1] * A[3];
  double h = s * f / (3.0 * dA);
#pragma unroll
  for (int k = 0; k < 9; k++)
    g[5 + k] = f * g[5 + k] - h * cof[k];
  g[0] += s * f / (3.0 * r);
}

// Cell-end states qL / qR of predictor cell c at time node t (side 0:
// x = 0, side 1: x = 1), the same expressions as k_faces1d.
template <int V>
GPR_D void end_state(const double *qh, long c, int t, int side, const Consts &C, double *qp) {
  const double *q0 = qh + (c * 4 + 2 * t) * V;
#pragma unroll
  for (int j = 0; j < V; j++)
    qp[j] = C.endv[side][0] * q0[j] + C.endv[side][1] * q0[V + j];
}

// Per cell end (4 per predictor cell, e = 2t + side): lambda (EV, the value
// the forward's Rusanov switch compared) and the eigen data of the acoustic
// tensor (EIG) for the wave speed's reverse-mode product, from the tensor
// and dominant eigenvalue of the same max_abs_eigs evaluation.
// Points nb*4 .. nb*4 + ninst - 1: the state entering the step at each
// instance's CFL argmax cell (for the derivative of dt).
template <class L>
__global__ void __launch_bounds__(128) k_adj_eig(const double *__restrict__ qh, long nb,
                                                 const double *__restrict__ un,
                                                 const double *__restrict__ aux,
                                                 double *__restrict__ EV,
                                                 double *__restrict__ EIG, Consts C, Batch B) {
  constexpr int V = L::V, m = Xi<L::THERMAL>::m, ND = Xi<L::THERMAL>::ND;
  long gid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (gid >= nb * 4 + B.ninst)
    return;
  double qp[V];
  int inst;
  if (gid < nb * 4) {
    long c = gid / 4;
    int e = gid % 4;
    inst = B.inst_b[c];
    if (B.clk[5 * inst + 1] == 0.0)
      return;
    end_state<V>(qh, c, e / 2, e % 2, C, qp);
  } else {
    inst = (int)(gid - nb * 4);
    long cs = (long)aux[2 * inst + 1];
    if (B.clk[5 * inst + 1] == 0.0 || cs < 0)
      return;
#pragma unroll
    for (int j = 0; j < V; j++)
      qp[j] = un[cs * V + j];
  }
  const DevPar &P = B.P[inst];
  Prim<L::THERMAL> sp;
  prim<L::THERMAL>(qp, P, sp);
  double Xv[m][m], l2;
  EV[gid] = max_abs_eigs<L::THERMAL>(qp, sp, 0, P, &Xv[0][0], &l2);
  xi_eigdata_l2<m>(Xv, l2, EIG + gid * ND);
}

// One face's contribution to the cotangent of the state on one side.
// Face flux f = max(lamL, lamR)(qL - qR) + F(qL) + F(qR) (fluxes.cpp:66-75),
// path integral b = sum_n w_n B(qL + x_n dq) dq (fluxes.cpp:9-20); the left
// cell receives -kk (b + f), the right -kk (b - f) (fv.cpp:143-146).
// Face cotangents (fb, bb) of the flux and path-integral terms from the
// cotangents of the two cells the face updates.
template <int V>
GPR_D void face_cot(const double *ubL, const double *ubR, double kk, double *Fb, double *Bb) {
#pragma unroll
  for (int k = 0; k < V; k++) {
    double a = ubL ? ubL[k] : 0.0, b = ubR ? ubR[k] : 0.0;
    Fb[k] = -kk * (a - b);
    Bb[k] = -kk * (a + b);
  }
}

// One face's adjoint on the side of this cell (mineL: the cell is the face's
// left neighbour): the flux VJP at this cell's end state (with the Rusanov
// speed's cotangent where this end attains the maximum), the dissipation
// and the path integral of B.  eig: eigen data at this cell's end.
template <class L>
GPR_D void face_adj(const double *ql, const double *qr, double lamL, double lamR,
                    const double *ubL, const double *ubR, double kk, bool mineL,
                    const double *eig, const DevPar &P, const Consts &C, double *qb,
                    double *thb) {
  constexpr int V = L::V;
  double Fb[V], Bb[V];
  face_cot<V>(ubL, ubR, kk, Fb, Bb);
  bool Lmax = lamL > lamR;  // std::max(m1, m2) picks m2 on ties
  double sm = Lmax ? lamL : lamR;
  double sbar = 0.0;
#pragma unroll
  for (int k = 0; k < V; k++)
    sbar += Fb[k] * (ql[k] - qr[k]);
  const bool mine_max = mineL ? Lmax : !Lmax;
  point_vjp<L, true, false, true>(mineL ? ql : qr, P, Fb, nullptr, mine_max ? sbar : 0.0, eig,
                                  qb, thb);
  double sgn = mineL ? sm : -sm;
#pragma unroll
  for (int k = 0; k < V; k++)
    qb[k] += sgn * Fb[k];
  double dq[V], dqb[V];
#pragma unroll
  for (int k = 0; k < V; k++) {
    dq[k] = qr[k] - ql[k];
    dqb[k] = 0.0;
  }
#pragma unroll
  for (int n = 0; n < NN; n++) {
    double xn = C.nodes[n];
    double rho = ql[0] + xn * dq[0];
    double ir = 1.0 / rho;
    double v[3] = {(ql[2] + xn * dq[2]) * ir, (ql[3] + xn * dq[3]) * ir,
                   (ql[4] + xn * dq[4]) * ir};
    double yb[V];
#pragma unroll
    for (int k = 0; k < V; k++)
      yb[k] = C.w[n] * Bb[k];
    bdot0_xT<V>(v, yb, dqb);
    double vb[3];
    bdot0_vT(dq, yb, vb);
    double f = mineL ? 1.0 - xn : xn;
    qb[0] -= f * (vb[0] * v[0] + vb[1] * v[1] + vb[2] * v[2]) * ir;
    qb[2] += f * vb[0] * ir;
    qb[3] += f * vb[1] * ir;
    qb[4] += f * vb[2] * ir;
  }
#pragma unroll
  for (int k = 0; k < V; k++)
    qb[k] += mineL ? -dqb[k] : dqb[k];
}

// FV adjoint: cotangent of qh from the cotangent ubar of u' (faces and the
// volume term), one thread per (predictor cell, time node), with the
// reverse-mode products of F, lambda (cell ends) and S (volume nodes).  Also
// the material-field cotangents (thf) and <ubar, u' - u> / dt (dtf) since
// the FV increment is linear in dt.
// Block = 4 warps over the same 32 (predictor cell, time node) pairs; warp
// w takes one term (0: the face on the cell's right, 1: the face on its
// left, 2 / 3: the volume term at spatial node 0 / 1), so that the lanes of
// a warp run the same reverse sweep; the four partial cotangents are summed
// in shared memory.
constexpr int ADJ_FV_PAIRS = 32;

template <class L>
__global__ void __launch_bounds__(4 * ADJ_FV_PAIRS) k_adj_fv(
    const double *__restrict__ ubar, const double *__restrict__ qh, const double *__restrict__ EV,
    const double *__restrict__ EIG, const double *__restrict__ un,
    const double *__restrict__ up, long nb, double *__restrict__ qbar, double *__restrict__ thf,
    double *__restrict__ dtf, Consts C, Batch B) {
  constexpr int V = L::V, ND = Xi<L::THERMAL>::ND, NO = 2 * V + NPD;
  __shared__ double red[4][NO][ADJ_FV_PAIRS];
  const int role = threadIdx.x / ADJ_FV_PAIRS, lane = threadIdx.x % ADJ_FV_PAIRS;
  const long ct = (long)blockIdx.x * ADJ_FV_PAIRS + lane;
  const bool valid = ct < nb * 2;
  const long c = valid ? ct / 2 : 0;
  const int t = (int)(ct % 2);
  const int inst = B.inst_b[c];
  const double dt = B.clk[5 * inst + 1];
  const DevPar &P = B.P[inst];
  double acc[2][V], th[NPD];
#pragma unroll
  for (int k = 0; k < V; k++) {
    acc[0][k] = 0.0;
    acc[1][k] = 0.0;
  }
#pragma unroll
  for (int p = 0; p < NPD; p++)
    th[p] = 0.0;
  const int li = (int)(c - B.off_b[inst]), nx = B.nx[inst];
  if (valid && dt != 0.0) {
    const double idx = B.idx[inst];
    const double kk = (dt * C.w[t]) / (2.0 * (1.0 / idx));
    const double *ubi = ubar + (long)B.off_u[inst] * V;
    const double *qc = qh + (c * 4 + 2 * t) * V;
    if (role < 2 && (role == 0 ? li <= nx : li >= 1)) {
      // role 0: face li (this cell on the left); role 1: face li - 1
      const int f = role == 0 ? li : li - 1;
      const double *qa = role == 0 ? qc : qh + ((c - 1) * 4 + 2 * t) * V;
      const double *qn = role == 0 ? qh + ((c + 1) * 4 + 2 * t) * V : qc;
      const long cl = role == 0 ? c : c - 1;
      double ql[V], qr[V], eb[V];
#pragma unroll
      for (int k = 0; k < V; k++) {
        ql[k] = C.endv[1][0] * qa[k] + C.endv[1][1] * qa[V + k];
        qr[k] = C.endv[0][0] * qn[k] + C.endv[0][1] * qn[V + k];
        eb[k] = 0.0;
      }
      face_adj<L>(ql, qr, EV[cl * 4 + 2 * t + 1], EV[(cl + 1) * 4 + 2 * t],
                  f > 0 ? ubi + (long)(f - 1) * V : nullptr,
                  f < nx ? ubi + (long)f * V : nullptr, kk, role == 0,
                  EIG + (c * 4 + 2 * t + (role == 0 ? 1 : 0)) * ND, P, C, eb, th);
      // this cell's end state: ENDVALS[side] . (node 0, node 1)
      const int side = role == 0 ? 1 : 0;
#pragma unroll
      for (int m = 0; m < 2; m++)
#pragma unroll
        for (int k = 0; k < V; k++)
          acc[m][k] = C.endv[side][m] * eb[k];
    } else if (role >= 2 && li >= 1 && li <= nx) {
      // volume term: u += (dt w_t) w_s (S - idx B(v) dq)   (fv.cpp:11-109)
      const int s = role - 2;
      const double *ubc = ubi + (long)(li - 1) * V;
      const double a = (dt * C.w[t]) * C.w[s];
      const double *qs = qc + s * V, *qo = qc + (1 - s) * V;
      double Sb[V];
#pragma unroll
      for (int k = 0; k < V; k++)
        Sb[k] = a * ubc[k];
      point_vjp<L, false, true, false>(qs, P, nullptr, Sb, 0.0, nullptr, acc[s], th);
      double yb[V], dq[V], xb[V];
      double ir = 1.0 / qs[0];
      double v[3] = {qs[2] * ir, qs[3] * ir, qs[4] * ir};
#pragma unroll
      for (int k = 0; k < V; k++) {
        yb[k] = -a * idx * ubc[k];
        dq[k] = C.derv[s][s] * qs[k] + C.derv[s][1 - s] * qo[k];
        xb[k] = 0.0;
      }
      double vb[3];
      bdot0_vT(dq, yb, vb);
      vel_T(qs, vb, acc[s], 1.0);
      bdot0_xT<V>(v, yb, xb);
#pragma unroll
      for (int k = 0; k < V; k++) {
        acc[s][k] += C.derv[s][s] * xb[k];
        acc[1 - s][k] += C.derv[s][1 - s] * xb[k];
      }
      if (s == 1 && t == 0) {
        long j = (long)B.off_u[inst] + li - 1;
        double x = 0.0;
#pragma unroll
        for (int k = 0; k < V; k++)
          x += ubc[k] * (up[j * V + k] - un[j * V + k]);
        dtf[c] = x / dt;
      }
    }
  }
  if (valid && role == 3 && t == 0 && !(dt != 0.0 && li >= 1 && li <= nx))
    dtf[c] = 0.0;
#pragma unroll
  for (int k = 0; k < V; k++) {
    red[role][k][lane] = acc[0][k];
    red[role][V + k][lane] = acc[1][k];
  }
#pragma unroll
  for (int p = 0; p < NPD; p++)
    red[role][2 * V + p][lane] = th[p];
  __syncthreads();
  if (!valid)
    return;
  double *qb = qbar + (c * 4 + 2 * t) * V;
  for (int k = role; k < NO; k += 4) {
    const double x = (red[0][k][lane] + red[1][k][lane]) + (red[2][k][lane] + red[3][k][lane]);
    if (k < 2 * V)
      qb[k] = x;
    else
      thf[(c * 2 + t) * NPD + (k - 2 * V)] = x;
  }
}

// Predictor adjoint at the converged fixed point.  With
//   R(q)_{t,i} = w_t w_i (S(q_ti) - B(q_ti) x_ti) - w_t idx sum_m DG_DER[i][m] F(q_tm),
//   x_ti = idx sum_m DERVALS[i][m] q_tm                      (dg1.cpp:8-66)
// the fixed point q = DG_U^-1 (W w + dt R(q)) gives, for the cotangent qbar
// of q, mu = (DG_U - dt dR/dq)^-T qbar, and then
//   wbar = (d(W w)/dw)^T mu,  dtbar = mu . R(q),  thbar = dt mu . dR/dth.
// Stage 1 (k_adj_pred_iter, 4 lanes per cell as in k_predictor_picard)
// iterates mu <- DG_U^-T (qbar + dt (dR/dq)^T mu), which contracts exactly
// where the forward Picard iteration does, each lane applying (dR/dq)^T at
// its node by one reverse-mode product of F and S; cells it leaves
// unconverged (those the forward hands to its Newton pass) get the exact
// dense solve of stage 2 (k_adj_pred_dense, one block per cell, building
// that cell's node Jacobians itself); stage 3
// (k_adj_pred_post) forms the cotangents from mu.
// Primal values that the reverse sweep of F and S reads at one node, cached
// once per node for the transposed iteration (structure of arrays with
// stride ST: entry k of a node at c[k * ST]).  wn (the node's quadrature
// weight w_t w_i) is folded into the source terms so that the S cotangent
// is mu itself.
template <class L> struct PCache {
  static constexpr int V = L::V;
  enum {
    IR, IR2, VV, JJ = VV + 3, CJ = JJ + 3, CA2T = CJ + 3, Q1PP, Q1M, DM, ADG = DM + 6,
    SG = ADG + 9, SGM = SG + 3, SGF = SGM + 3, FSW, COFK, GSW = COFK + 9, GTW, IRGICV, PPICV,
    RGM1, E1GM1, Q, N = Q + V
  };
};

template <class L>
GPR_D void pcache_init(const double *q, const DevPar &P, double wn, double *c, int ST) {
  using PC = PCache<L>;
  constexpr bool TH = L::THERMAL;
  const double *A = q + 5;
  const double r = q[0], ir = 1.0 / r;
  double v[3], J[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 3; i++)
    v[i] = q[2 + i] * ir;
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      J[i] = q[14 + i] * ir;
  }
  const double G00 = A[0] * A[0] + A[3] * A[3] + A[6] * A[6];
  const double G11 = A[1] * A[1] + A[4] * A[4] + A[7] * A[7];
  const double G22 = A[2] * A[2] + A[5] * A[5] + A[8] * A[8];
  const double G01 = A[0] * A[1] + A[3] * A[4] + A[6] * A[7];
  const double G02 = A[0] * A[2] + A[3] * A[5] + A[6] * A[8];
  const double G12 = A[1] * A[2] + A[4] * A[5] + A[7] * A[8];
  const double tG = (G00 + G11 + G22) * (1.0 / 3.0);
  const double Dm[3][3] = {{G00 - tG, G01, G02}, {G01, G11 - tG, G12}, {G02, G12, G22 - tG}};
  const double devGsq = Dm[0][0] * Dm[0][0] + Dm[1][1] * Dm[1][1] + Dm[2][2] * Dm[2][2] +
                        2.0 * (G01 * G01 + G02 * G02 + G12 * G12);
  double AdG[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      AdG[3 * i + j] = A[3 * i] * Dm[0][j] + A[3 * i + 1] * Dm[1][j] + A[3 * i + 2] * Dm[2][j];
  const double Gm1 = P.gamma - 1.0, irG = ir * P.iG;
  double E1 = q[1] * ir - 0.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) -
              0.25 * (P.b02 * devGsq);
  if (TH)
    E1 = E1 - 0.5 * (P.calpha2 * (J[0] * J[0] + J[1] * J[1] + J[2] * J[2]));
  const double er = P.pINF * ir;
  const double p = (E1 - er) * (r * Gm1) - P.pINF;
  const double T = (p + P.pINF) * irG * P.icv;
  const double sgf = -(r * P.b02);
  const double dA = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                    A[2] * (A[3] * A[7] - A[4] * A[6]);
  const double cb = cbrt(dA);
  const double th = dA * cb * cb * P.th1c;
  const double kc = wn * (-P.b02) * P.th1c * (5.0 / 3.0) * cb * cb;
  const double cof[9] = {A[4] * A[8] - A[5] * A[7], A[5] * A[6] - A[3] * A[8],
                         A[3] * A[7] - A[4] * A[6], A[2] * A[7] - A[1] * A[8],
                         A[0] * A[8] - A[2] * A[6], A[1] * A[6] - A[0] * A[7],
                         A[1] * A[5] - A[2] * A[4], A[2] * A[3] - A[0] * A[5],
                         A[0] * A[4] - A[1] * A[3]};
  c[PC::IR * ST] = ir;
  c[PC::IR2 * ST] = ir * ir;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    c[(PC::VV + i) * ST] = v[i];
    c[(PC::JJ + i) * ST] = J[i];
    c[(PC::CJ + i) * ST] = P.calpha2 * J[i];
    double sm = AdG[i] * A[0] + AdG[3 + i] * A[3] + AdG[6 + i] * A[6];
    c[(PC::SGM + i) * ST] = sm;
    c[(PC::SG + i) * ST] = sgf * sm;
  }
  c[PC::CA2T * ST] = P.calpha2 * T;
  c[PC::Q1PP * ST] = q[1] + p;
  c[PC::Q1M * ST] = q[1] - P.pINF;
  c[(PC::DM + 0) * ST] = Dm[0][0];
  c[(PC::DM + 1) * ST] = Dm[1][1];
  c[(PC::DM + 2) * ST] = Dm[2][2];
  c[(PC::DM + 3) * ST] = G01;
  c[(PC::DM + 4) * ST] = G02;
  c[(PC::DM + 5) * ST] = G12;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    c[(PC::ADG + k) * ST] = AdG[k];
    c[(PC::COFK + k) * ST] = kc * cof[k];
  }
  c[PC::SGF * ST] = sgf;
  c[PC::FSW * ST] = wn * (-(P.b02 * th));
  c[PC::GSW * ST] = wn * (-(P.calpha2 * T * P.ikappa));
  c[PC::GTW * ST] = wn * (P.calpha2 * P.ikappa);
  c[PC::IRGICV * ST] = irG * P.icv;
  c[PC::PPICV * ST] = (p + P.pINF) * P.icv;
  c[PC::RGM1 * ST] = r * Gm1;
  c[PC::E1GM1 * ST] = (E1 - er) * Gm1;
#pragma unroll
  for (int k = 0; k < L::V; k++)
    c[(PC::Q + k) * ST] = q[k];
}

// r += (dF/dq)^T Fb + wn (dS/dq)^T mu from the cached primal values: the
// reverse sweep of point_vjp (HF, HS, no material fields), term by term, in
// the arithmetic type S of the cache (FP64, or FP32 for the correction
// solves of k_adj_pred_iter).
template <class L, class S>
GPR_D void pcache_vjp(const S *c, int ST, S b02, S iG, const S *Fb, const S *mu, S *r) {
  using PC = PCache<L>;
  constexpr bool TH = L::THERMAL;
#define PCV(k) c[(k) * ST]
  const S *qc = c + PC::Q * ST;
#define PQ(k) qc[(k) * ST]
  S A[9];
#pragma unroll
  for (int k = 0; k < 9; k++)
    A[k] = PQ(5 + k);
  const S v[3] = {PCV(PC::VV), PCV(PC::VV + 1), PCV(PC::VV + 2)};
  S vb[3], sgb[3], Ab[9], AdGb[9], Jb[3] = {S(0), S(0), S(0)}, qJb[3] = {S(0), S(0), S(0)};
  S q2b[3];
  // flux
  const S f1 = Fb[1];
  vb[0] = f1 * PCV(PC::Q1PP);
  vb[1] = S(0);
  vb[2] = S(0);
  S q1b = f1 * v[0];
  S pb = f1 * v[0] + Fb[2];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    sgb[i] = -(f1 * v[i]) - Fb[2 + i];
    vb[i] -= f1 * PCV(PC::SG + i);
    vb[0] += Fb[2 + i] * PQ(2 + i);
    q2b[i] = Fb[2 + i] * v[0];
  }
  q2b[0] += Fb[0];
  S Tb = S(0);
  if (TH) {
    Tb = f1 * PCV(PC::CJ) + Fb[14];
    Jb[0] = f1 * PCV(PC::CA2T);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      vb[0] += Fb[14 + i] * PQ(14 + i);
      qJb[i] = Fb[14 + i] * v[0];
    }
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const S f = Fb[5 + 3 * i];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Ab[3 * i + j] = f * v[j];
      vb[j] += f * A[3 * i + j];
    }
  }
  // source (wn folded into FSW, COFK, GSW)
  S fb = S(0);
  const S fsw = PCV(PC::FSW);
#pragma unroll
  for (int i = 0; i < 9; i++) {
    fb += mu[5 + i] * PCV(PC::ADG + i);
    AdGb[i] = mu[5 + i] * fsw;
  }
#pragma unroll
  for (int k = 0; k < 9; k++)
    Ab[k] += fb * PCV(PC::COFK + k);
  if (TH) {
    const S gsw = PCV(PC::GSW);
    S gb = S(0);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      gb += mu[14 + i] * PCV(PC::JJ + i);
      Jb[i] += mu[14 + i] * gsw;
    }
    Tb -= gb * PCV(PC::GTW);
  }
  // sigma column 0
  const S sgf = PCV(PC::SGF);
  S sgfb = S(0);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    sgfb += sgb[i] * PCV(PC::SGM + i);
    const S f = sgb[i] * sgf;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      AdGb[3 * k + i] += f * A[3 * k];
      Ab[3 * k] += f * PCV(PC::ADG + 3 * k + i);
    }
  }
  S rb = -(sgfb * b02);
  // prim
  pb += Tb * PCV(PC::IRGICV);
  const S irGb = Tb * PCV(PC::PPICV);
  const S E1b = pb * PCV(PC::RGM1);
  rb += pb * PCV(PC::E1GM1);
  const S ir = PCV(PC::IR);
  S irb = E1b * PCV(PC::Q1M) + irGb * iG;
  q1b += E1b * ir;
#pragma unroll
  for (int i = 0; i < 3; i++)
    vb[i] -= E1b * v[i];
  const S devGsqb = S(-0.25) * b02 * E1b;
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Jb[i] -= E1b * PCV(PC::CJ + i);
      qJb[i] += Jb[i] * ir;
      irb += Jb[i] * PQ(14 + i);
    }
  }
  // AdG = A Dm
  const S D00 = PCV(PC::DM), D11 = PCV(PC::DM + 1), D22 = PCV(PC::DM + 2);
  const S G01 = PCV(PC::DM + 3), G02 = PCV(PC::DM + 4), G12 = PCV(PC::DM + 5);
  const S Dm[3][3] = {{D00, G01, G02}, {G01, D11, G12}, {G02, G12, D22}};
  S Dmb[3][3];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      Dmb[k][j] = AdGb[j] * A[k] + AdGb[3 + j] * A[3 + k] + AdGb[6 + j] * A[6 + k];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++)
      Ab[3 * i + k] += AdGb[3 * i] * Dm[k][0] + AdGb[3 * i + 1] * Dm[k][1] +
                       AdGb[3 * i + 2] * Dm[k][2];
  const S D00b = Dmb[0][0] + devGsqb * S(2) * D00;
  const S D11b = Dmb[1][1] + devGsqb * S(2) * D11;
  const S D22b = Dmb[2][2] + devGsqb * S(2) * D22;
  const S G01b = Dmb[0][1] + Dmb[1][0] + devGsqb * S(4) * G01;
  const S G02b = Dmb[0][2] + Dmb[2][0] + devGsqb * S(4) * G02;
  const S G12b = Dmb[1][2] + Dmb[2][1] + devGsqb * S(4) * G12;
  const S tb = -(D00b + D11b + D22b) * S(1.0 / 3.0);
  const S G00b = D00b + tb, G11b = D11b + tb, G22b = D22b + tb;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const S a0 = A[3 * k], a1 = A[3 * k + 1], a2 = A[3 * k + 2];
    Ab[3 * k] += S(2) * G00b * a0 + G01b * a1 + G02b * a2;
    Ab[3 * k + 1] += S(2) * G11b * a1 + G01b * a0 + G12b * a2;
    Ab[3 * k + 2] += S(2) * G22b * a2 + G02b * a0 + G12b * a1;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    q2b[i] += vb[i] * ir;
    irb += vb[i] * PQ(2 + i);
  }
  rb -= irb * PCV(PC::IR2);
  r[0] += rb;
  r[1] += q1b;
#pragma unroll
  for (int i = 0; i < 3; i++)
    r[2 + i] += q2b[i];
#pragma unroll
  for (int k = 0; k < 9; k++)
    r[5 + k] += Ab[k];
  if (TH) {
#pragma unroll
    for (int i = 0; i < 3; i++)
      r[14 + i] += qJb[i];
  }
#undef PCV
#undef PQ
}

constexpr int ADJ_PRED_IT = 100;
constexpr double ADJ_PRED_TOL = 1e-11;
constexpr int ADJ_INNER = 6;  // FP32 iterations per correction solve
constexpr int ADJ_IT_T = 32;  // threads (8 cells) per block of k_adj_pred_iter

// max(a, |d|) on the IEEE bit patterns of non-negative doubles (integer
// order equals numeric order there; NaN patterns sort above every number)
GPR_D unsigned long long absmax_bits(unsigned long long a, double d) {
  unsigned long long b = (unsigned long long)__double_as_longlong(d) & 0x7fffffffffffffffULL;
  return b > a ? b : a;
}

template <class S, int V> GPR_D void shfl_vec_t(const S *src, S *dst, int lanemask) {
#pragma unroll
  for (int k = 0; k < V; k++)
    dst[k] = __shfl_xor_sync(0xffffffffu, src[k], lanemask);
}

// Per-lane coefficients of the transposed Picard map at node (t, i).
template <class S> struct TCoef {
  S fa, fo, xa, xo, ga, go, dt, wn, iq0, v0, v1, v2, b02, iG;
};

// y = DG_U^-T (z0 + dt R^T x) at this lane's node, where R^T x = (dR/dq)^T
// x: the F part with cotangent -wti sum_i DG_DER[i][m] x_i, the S part with
// cotangent wn x, and -wn B(v)^T x through the node derivative x_ti and
// through v(q).  z0 = nullptr for the homogeneous map (z0 = 0).  All lanes
// of the warp take part (shuffles with the node partners g ^ 1, g ^ 2).
template <class L, class S>
GPR_D void tmap(const S *x, const double *z0, const S *pc, const S *xs, int ST, bool active,
                const TCoef<S> &k, S *y) {
  constexpr int V = L::V;
  S Fb[V], r[V], tmp[V];
  shfl_vec_t<S, V>(x, tmp, 1);
#pragma unroll
  for (int j = 0; j < V; j++) {
    Fb[j] = k.fa * x[j] + k.fo * tmp[j];
    r[j] = S(0);
  }
  if (active)
    pcache_vjp<L, S>(pc, ST, k.b02, k.iG, Fb, x, r);
  S xb[6], xq[6];
#pragma unroll
  for (int rr = 0; rr < 3; rr++) {
    xb[2 * rr] = -k.v1 * x[5 + 3 * rr] + k.v0 * x[6 + 3 * rr];
    xb[2 * rr + 1] = -k.v2 * x[5 + 3 * rr] + k.v0 * x[7 + 3 * rr];
  }
  S vb0 = S(0), vb1 = S(0), vb2 = S(0);
#pragma unroll
  for (int rr = 0; rr < 3; rr++) {
    const S x6 = xs[(2 * rr) * ST], x7 = xs[(2 * rr + 1) * ST];
    vb0 += x6 * x[6 + 3 * rr] + x7 * x[7 + 3 * rr];
    vb1 -= x6 * x[5 + 3 * rr];
    vb2 -= x7 * x[5 + 3 * rr];
  }
  const S wq = k.wn * k.iq0;
  r[0] += wq * (vb0 * k.v0 + vb1 * k.v1 + vb2 * k.v2);
  r[2] -= wq * vb0;
  r[3] -= wq * vb1;
  r[4] -= wq * vb2;
#pragma unroll
  for (int m = 0; m < 6; m++)
    xq[m] = __shfl_xor_sync(0xffffffffu, xb[m], 1);
#pragma unroll
  for (int rr = 0; rr < 3; rr++)
#pragma unroll
    for (int m = 0; m < 2; m++)
      r[6 + 3 * rr + m] += k.xa * xb[2 * rr + m] + k.xo * xq[2 * rr + m];
#pragma unroll
  for (int j = 0; j < V; j++)
    r[j] = z0 ? S(z0[j]) + k.dt * r[j] : k.dt * r[j];
  shfl_vec_t<S, V>(r, tmp, 2);
#pragma unroll
  for (int j = 0; j < V; j++)
    y[j] = k.ga * r[j] + k.go * tmp[j];
}

// Mixed-precision iterative refinement of the fixed point mu = T(mu),
// T(mu) = DG_U^-T (qbar + dt R^T mu) (a published technique: the defect in
// the working precision, the correction equation in a cheaper one).  Each
// outer step forms the defect d = T(mu) - mu in FP64 (one FP64 evaluation,
// the convergence test |d| <= tol |T(mu)| as in the plain iteration), then
// solves the correction equation e = d + T_0(e) (T_0: T without qbar) by
// ADJ_INNER FP32 iterations over an FP32 copy of the primal cache, and sets
// mu += e.  The FP32 solve costs little beside the FP64 evaluation on this
// GPU's FP64 pipe and brings ~6 digits per outer step; a non-finite FP32
// correction falls back to the plain step mu = T(mu).
template <class L>
__global__ void __launch_bounds__(ADJ_IT_T) k_adj_pred_iter(
    const double *__restrict__ qh, const double *__restrict__ qbar, long nb,
    double *__restrict__ mu_buf, int32_t *__restrict__ need, int32_t *__restrict__ info,
    Consts C, Batch B) {
  constexpr int V = L::V, NC = PCache<L>::N, ST = ADJ_IT_T;
  __shared__ double cache[(NC + 6) * ST];
  __shared__ float cachef[(NC + 6) * ST];
  double *pc = cache + threadIdx.x;
  double *xs = cache + NC * ST + threadIdx.x;  // x at 6, 7, 9, 10, 12, 13
  float *pcf = cachef + threadIdx.x;
  float *xsf = cachef + NC * ST + threadIdx.x;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int g = threadIdx.x % 4;
  const long c = gt / 4;
  const bool valid = c < nb;
  const long cc = valid ? c : 0;
  const int t = g / 2, i = g % 2;
  const int inst = B.inst_b[cc];
  const double dt = B.clk[5 * inst + 1];
  const double idx = B.idx[inst];
  const DevPar &P = B.P[inst];
  const bool active = valid && dt != 0.0;
  const double wn = C.w[t] * C.w[i], wno = C.w[t] * C.w[1 - i], wti = C.w[t] * idx;
  // node data: the primal cache, x_ti = idx sum_m DERVALS[i][m] q_tm
  double mu[V], qb[V], y[V];
  {
    double q[V];
#pragma unroll
    for (int k = 0; k < V; k++)
      q[k] = qh[(cc * 4 + g) * V + k];
    shfl_vec<V>(q, y, 1);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int m = 0; m < 2; m++) {
        int k = 6 + 3 * r + m;
        xs[(2 * r + m) * ST] = idx * (C.derv[i][i] * q[k] + C.derv[i][1 - i] * y[k]);
      }
    pcache_init<L>(q, P, wn, pc, ST);
  }
  for (int k = 0; k < NC + 6; k++)
    pcf[k * ST] = (float)pc[k * ST];
#pragma unroll
  for (int k = 0; k < V; k++) {
    qb[k] = active ? qbar[(cc * 4 + g) * V + k] : 0.0;
    mu[k] = 0.0;
  }
  TCoef<double> kd;
  kd.fa = -wti * C.dgder[i][i];
  kd.fo = -wti * C.dgder[1 - i][i];
  kd.xa = -wn * idx * C.derv[i][i];
  kd.xo = -wno * idx * C.derv[1 - i][i];
  kd.ga = C.dgmatinv[t][t] / C.w[i];
  kd.go = C.dgmatinv[1 - t][t] / C.w[i];
  kd.dt = dt;
  kd.wn = wn;
  kd.iq0 = pc[PCache<L>::IR * ST];
  kd.v0 = pc[PCache<L>::VV * ST];
  kd.v1 = pc[(PCache<L>::VV + 1) * ST];
  kd.v2 = pc[(PCache<L>::VV + 2) * ST];
  kd.b02 = P.b02;
  kd.iG = P.iG;
  TCoef<float> kf;
  kf.fa = (float)kd.fa;
  kf.fo = (float)kd.fo;
  kf.xa = (float)kd.xa;
  kf.xo = (float)kd.xo;
  kf.ga = (float)kd.ga;
  kf.go = (float)kd.go;
  kf.dt = (float)kd.dt;
  kf.wn = (float)kd.wn;
  kf.iq0 = (float)kd.iq0;
  kf.v0 = (float)kd.v0;
  kf.v1 = (float)kd.v1;
  kf.v2 = (float)kd.v2;
  kf.b02 = (float)kd.b02;
  kf.iG = (float)kd.iG;
  bool conv = !active, done = !active;
  int nit = 0;
  for (int it = 0; it < ADJ_PRED_IT; it++) {
    if (__all_sync(0xffffffffu, done))
      break;
    nit += done ? 0 : 1;
    tmap<L, double>(mu, qb, pc, xs, ST, active, kd, y);
    unsigned long long ddb = 0, scb = 0;
#pragma unroll
    for (int k = 0; k < V; k++) {
      ddb = absmax_bits(ddb, y[k] - mu[k]);
      scb = absmax_bits(scb, y[k]);
    }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) {
      unsigned long long a = __shfl_xor_sync(0xffffffffu, ddb, o);
      unsigned long long b = __shfl_xor_sync(0xffffffffu, scb, o);
      ddb = a > ddb ? a : ddb;
      scb = b > scb ? b : scb;
    }
    bool upd = false;
    if (!done) {
      if (scb > 0x7ff0000000000000ULL) {  // NaN
#pragma unroll
        for (int k = 0; k < V; k++)
          mu[k] = y[k];
        done = true;
      } else if (__longlong_as_double((long long)ddb) <=
                 ADJ_PRED_TOL * __longlong_as_double((long long)scb)) {
#pragma unroll
        for (int k = 0; k < V; k++)
          mu[k] = y[k];
        conv = true;
        done = true;
      } else {
        upd = true;
      }
    }
    if (__any_sync(0xffffffffu, upd)) {
      float df[V], e[V], te[V];
#pragma unroll
      for (int k = 0; k < V; k++) {
        df[k] = (float)(y[k] - mu[k]);
        e[k] = df[k];
      }
      for (int j = 1; j < ADJ_INNER; j++) {
        tmap<L, float>(e, nullptr, pcf, xsf, ST, active, kf, te);
#pragma unroll
        for (int k = 0; k < V; k++)
          e[k] = df[k] + te[k];
      }
      if (upd) {
        bool fin = true;
#pragma unroll
        for (int k = 0; k < V; k++)
          fin = fin && isfinite(e[k]);
#pragma unroll
        for (int k = 0; k < V; k++)
          mu[k] = fin ? mu[k] + (double)e[k] : y[k];
      }
    }
  }
  if (!valid)
    return;
#pragma unroll
  for (int k = 0; k < V; k++)
    mu_buf[(c * 4 + g) * V + k] = mu[k];
  if (g == 0) {
    need[c] = conv ? 0 : 1;
    info[c] += nit << 8;
  }
}

// d(B_x(v(q)) x)_r / dq_c and B_x(v)[r][c] (bdot, d = 0)
GPR_D double dBx_dq(int r, int c, const double *x, const double *v, double iq0) {
  double dv[3] = {0.0, 0.0, 0.0};
  if (r >= 5 && r < 14) {
    int rr = (r - 5) / 3, cc = (r - 5) % 3;
    if (cc == 0) {
      dv[1] = -x[6 + 3 * rr];
      dv[2] = -x[7 + 3 * rr];
    } else {
      dv[0] = x[5 + 3 * rr + cc];
    }
  }
  if (c == 0)
    return -(dv[0] * v[0] + dv[1] * v[1] + dv[2] * v[2]) * iq0;
  if (c >= 2 && c < 5)
    return dv[c - 2] * iq0;
  return 0.0;
}

GPR_D double Bx_mat(int r, int c, const double *v) {
  if (r < 5 || r >= 14)
    return 0.0;
  int rr = (r - 5) / 3, cc = (r - 5) % 3;
  if (cc == 0) {
    if (c == 6 + 3 * rr)
      return -v[1];
    if (c == 7 + 3 * rr)
      return -v[2];
    return 0.0;
  }
  return c == r ? v[0] : 0.0;
}

// Exact transposed solve (DG_U - dt dR/dq)^T mu = qbar for the cells the
// iteration left unconverged: the cell's node Jacobians (state columns, by
// dual numbers, one thread per node and column) and the 4V x 4V system in
// dynamic shared memory (dense_smem_bytes), Gaussian elimination with
// partial pivoting.
template <int V> constexpr size_t dense_smem_bytes() {
  return sizeof(double) * ((size_t)4 * V * (4 * V + 1) + (size_t)4 * V * 2 * V);
}

template <class L>
__global__ void __launch_bounds__(128) k_adj_pred_dense(
    const double *__restrict__ qh, const double *__restrict__ qbar, long nb,
    const int32_t *__restrict__ need, double *__restrict__ mu_buf, int32_t *__restrict__ info,
    Consts C, Batch B) {
  constexpr int V = L::V, NQ = 4 * V, LD = NQ + 1;
  extern __shared__ double dsm[];
  double *A = dsm;              // [NQ][LD], transposed system
  double *JS = dsm + NQ * LD;   // [node][j][F_o, S_o] = d(F_o, S_o)/dq_j
  __shared__ double b[NQ], lcol[NQ];
  __shared__ double xs[4][V], vs[4][3], iq0[4];
  __shared__ int piv;
  __shared__ int bad;
  const long c = blockIdx.x;
  if (c >= nb || !need[c])
    return;
  const int inst = B.inst_b[c];
  const double dt = B.clk[5 * inst + 1];
  const double idx = B.idx[inst];
  const double *qc = qh + c * 4 * V;
  if (threadIdx.x < 4) {
    int g = threadIdx.x, i = g % 2;
    const double *q = qc + g * V, *qo = qc + (g ^ 1) * V;
    for (int k = 0; k < V; k++)
      xs[g][k] = idx * (C.derv[i][i] * q[k] + C.derv[i][1 - i] * qo[k]);
    double ir = 1.0 / q[0];
    iq0[g] = ir;
    vs[g][0] = q[2] * ir;
    vs[g][1] = q[3] * ir;
    vs[g][2] = q[4] * ir;
  }
  if (threadIdx.x == 0)
    bad = 0;
  for (int e = threadIdx.x; e < 4 * V; e += blockDim.x) {
    const int g = e / V, j = e % V;
    Dual F[V], S[V];
    point_tangent<L>(qc + g * V, j, B.P[inst], F, S, nullptr);
    double *o = JS + (g * V + j) * 2 * V;
#pragma unroll
    for (int k = 0; k < V; k++) {
      o[k] = F[k].d;
      o[V + k] = S[k].d;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NQ * NQ; e += blockDim.x) {
    int row = e / NQ, col = e % NQ;  // entry M[row][col]
    int gr = row / V, vr = row % V, gc = col / V, vc = col % V;
    int t = gr / 2, i = gr % 2, tc = gc / 2, m = gc % 2;
    double val = (i == m && vr == vc) ? C.dgmat[t][tc] * C.w[i] : 0.0;
    if (t == tc) {
      const double *Jn = JS + gc * V * 2 * V;
      double wn = C.w[t] * C.w[i];
      double r = -C.w[t] * idx * C.dgder[i][m] * Jn[vc * 2 * V + vr];
      if (i == m)
        r += wn * (Jn[vc * 2 * V + V + vr] - dBx_dq(vr, vc, xs[gr], vs[gr], iq0[gr]));
      r -= wn * Bx_mat(vr, vc, vs[gr]) * idx * C.derv[i][m];
      val -= dt * r;
    }
    A[col * LD + row] = val;  // transposed
  }
  for (int r = threadIdx.x; r < NQ; r += blockDim.x)
    b[r] = qbar[c * 4 * V + r];
  __syncthreads();
  for (int k = 0; k < NQ; k++) {
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = k;
      for (int r = k + threadIdx.x; r < NQ; r += 32) {
        double a = fabs(A[r * LD + k]);
        if (a > best) {
          best = a;
          bi = r;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_down_sync(0xffffffffu, best, o);
        int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        piv = bi;
        if (!(best > 0.0))
          bad = 1;
      }
    }
    __syncthreads();
    if (bad)
      break;
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < NQ; j += blockDim.x) {
        double tmp = A[k * LD + j];
        A[k * LD + j] = A[p * LD + j];
        A[p * LD + j] = tmp;
      }
      if (threadIdx.x == 0) {
        double tmp = b[k];
        b[k] = b[p];
        b[p] = tmp;
      }
    }
    __syncthreads();
    const double ia = 1.0 / A[k * LD + k];
    for (int r = k + 1 + threadIdx.x; r < NQ; r += blockDim.x)
      lcol[r] = A[r * LD + k] * ia;
    __syncthreads();
    const int w = NQ - k - 1;
    for (int e = threadIdx.x; e < w * (w + 1); e += blockDim.x) {
      int r = k + 1 + e / (w + 1), j = k + 1 + e % (w + 1);
      if (j < NQ)
        A[r * LD + j] -= lcol[r] * A[k * LD + j];
      else
        b[r] -= lcol[r] * b[k];
    }
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0)
      info[c] |= 1;
    return;
  }
  // back substitution by warp 0
  if (threadIdx.x < 32) {
    for (int k = NQ - 1; k >= 0; k--) {
      double s = 0.0;
      for (int j = k + 1 + threadIdx.x; j < NQ; j += 32)
        s += A[k * LD + j] * b[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0)
        b[k] = (b[k] - s) / A[k * LD + k];
      __syncwarp();
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < NQ; r += blockDim.x)
    mu_buf[c * 4 * V + r] = b[r];
}

template <class L>
__global__ void __launch_bounds__(128) k_adj_pred_post(
    const double *__restrict__ qh, const double *__restrict__ mu_buf, long nb,
    double *__restrict__ wbar, double *__restrict__ thp, double *__restrict__ dtp, Consts C,
    Batch B) {
  constexpr int V = L::V;
  long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int g = threadIdx.x % 4;
  const long c = gt / 4;
  const bool valid = c < nb;
  const long cc = valid ? c : 0;
  const int t = g / 2, i = g % 2;
  const int inst = B.inst_b[cc];
  const double dt = B.clk[5 * inst + 1];
  const DevPar &P = B.P[inst];
  const double idx = B.idx[inst];
  const bool active = valid && dt != 0.0;
  double q[V], mu[V], other[V], y[V];
#pragma unroll
  for (int k = 0; k < V; k++) {
    q[k] = qh[(cc * 4 + g) * V + k];
    mu[k] = active ? mu_buf[(cc * 4 + g) * V + k] : 0.0;
  }
  const double wn = C.w[t] * C.w[i], wti = C.w[t] * idx;
  shfl_vec<V>(mu, other, 1);
#pragma unroll
  for (int k = 0; k < V; k++)
    y[k] = C.dgder[i][i] * mu[k] + C.dgder[1 - i][i] * other[k];
  // R(q) at this node: dg_rhs_node with dt = 1 and W w = 0
  double R[V], zero[V];
#pragma unroll
  for (int k = 0; k < V; k++)
    zero[k] = 0.0;
  dg_rhs_node<L, 1>(q, zero, R, t, i, 0, 1.0, idx, 1.0, P, C);
  double dtb = 0.0;
#pragma unroll
  for (int k = 0; k < V; k++)
    dtb += mu[k] * R[k];
  // thbar = dt (wn dS/dth^T mu - wti dF/dth^T y)
  double th[NPD];
#pragma unroll
  for (int p = 0; p < NPD; p++)
    th[p] = 0.0;
  if (active) {
    double Fb[V], Sb[V], qd[V];
#pragma unroll
    for (int k = 0; k < V; k++) {
      Fb[k] = -(dt * wti) * y[k];
      Sb[k] = (dt * wn) * mu[k];
      qd[k] = 0.0;
    }
    point_vjp<L, true, true, false>(q, P, Fb, Sb, 0.0, nullptr, qd, th);
  }
  // W w: Ww(t, s) = ENDVALS[0][t] w_s wh(s)  (dg1.cpp:68-73)
  double wb[V];
  const double f = C.endv[0][t] * C.w[i];
#pragma unroll
  for (int k = 0; k < V; k++)
    wb[k] = f * mu[k];
  shfl_vec<V>(wb, other, 2);
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
    dtb += __shfl_xor_sync(0xffffffffu, dtb, o);
#pragma unroll
    for (int p = 0; p < NPD; p++)
      th[p] += __shfl_xor_sync(0xffffffffu, th[p], o);
  }
  if (!valid)
    return;
  if (t == 0) {
#pragma unroll
    for (int k = 0; k < V; k++)
      wbar[(c * 2 + i) * V + k] = active ? wb[k] + other[k] : 0.0;
  }
  if (g == 0) {
    dtp[c] = active ? dtb : 0.0;
#pragma unroll
    for (int p = 0; p < NPD; p++)
      thp[c * NPD + p] = active ? th[p] : 0.0;
  }
}

// WENO adjoint: per (predictor cell, variable), the cotangents of the three
// stencil values (weno.cpp:4-73 with the gap-free 1D stencils).
template <int V>
__global__ void k_adj_weno(const double *__restrict__ wbar, const double *__restrict__ un,
                           long nb, double *__restrict__ gst, Consts C, Batch B) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= nb * V)
    return;
  int k = idx % V;
  long c = idx / V;
  int inst = B.inst_b[c];
  double *out = gst + (c * V + k) * 3;
  if (B.clk[5 * inst + 1] == 0.0) {
    out[0] = out[1] = out[2] = 0.0;
    return;
  }
  int li = (int)(c - B.off_b[inst]), nx = B.nx[inst];
  const double *ui = un + (long)B.off_u[inst] * V;
  double d[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    int b = li + m;
    if (b >= NN && b < nx + NN) {
      d[m] = ui[(long)(b - NN) * V + k];
    } else {
      int side = b >= nx + NN;
      int gi = side ? b - nx - NN : b;
      int code = B.bc[2 * inst + side];
      int si = bc_src_index(code, side, gi, nx);
      if (code == GPR_BC_PERIODIC)
        code = GPR_BC_TRANSMISSIVE;
      d[m] = bc_value<V>(code, 0, k, ui + (long)si * V);
    }
  }
  double a = d[0], b = d[1], cc = d[2];
  double wL0 = C.mLinv[0][0] * a + C.mLinv[0][1] * b;
  double wL1 = C.mLinv[1][0] * a + C.mLinv[1][1] * b;
  double wR0 = C.mRinv[0][0] * b + C.mRinv[0][1] * cc;
  double wR1 = C.mRinv[1][0] * b + C.mRinv[1][1] * cc;
  double tL = (wL0 * C.sig[0][0] + wL1 * C.sig[1][0]) * wL0 +
              (wL0 * C.sig[0][1] + wL1 * C.sig[1][1]) * wL1 + WENO_EPS;
  double tR = (wR0 * C.sig[0][0] + wR1 * C.sig[1][0]) * wR0 +
              (wR0 * C.sig[0][1] + wR1 * C.sig[1][1]) * wR1 + WENO_EPS;
  double pL = tL * tL, pR = tR * tR;
  pL *= pL;
  pL *= pL;
  pR *= pR;
  pR *= pR;
  double oL = LAMS / pL, oR = LAMS / pR;
  double iden = 1.0 / (oL + oR);
  double o0 = (wL0 * oL + wR0 * oR) * iden, o1 = (wL1 * oL + wR1 * oR) * iden;
  double g0 = wbar[(c * 2 + 0) * V + k], g1 = wbar[(c * 2 + 1) * V + k];
  double oLb = (g0 * (wL0 - o0) + g1 * (wL1 - o1)) * iden;
  double oRb = (g0 * (wR0 - o0) + g1 * (wR1 - o1)) * iden;
  double tLb = -8.0 * oL / tL * oLb, tRb = -8.0 * oR / tR * oRb;
  double sx = C.sig[0][1] + C.sig[1][0];
  double wL0b = g0 * oL * iden + tLb * (2.0 * C.sig[0][0] * wL0 + sx * wL1);
  double wL1b = g1 * oL * iden + tLb * (sx * wL0 + 2.0 * C.sig[1][1] * wL1);
  double wR0b = g0 * oR * iden + tRb * (2.0 * C.sig[0][0] * wR0 + sx * wR1);
  double wR1b = g1 * oR * iden + tRb * (sx * wR0 + 2.0 * C.sig[1][1] * wR1);
  out[0] = C.mLinv[0][0] * wL0b + C.mLinv[1][0] * wL1b;
  out[1] = C.mLinv[0][1] * wL0b + C.mLinv[1][1] * wL1b + C.mRinv[0][0] * wR0b +
           C.mRinv[1][0] * wR1b;
  out[2] = C.mRinv[0][1] * wR0b + C.mRinv[1][1] * wR1b;
}

// ubar(u) += sum of the stencil cotangents of every ub cell that copies u
// (interior cell j+N, and the ghost cells whose source is j).
template <int V>
__global__ void k_adj_gather(double *__restrict__ ubar, const double *__restrict__ gst,
                             long nu, Batch B) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= nu * V)
    return;
  int k = idx % V;
  long j = idx / V;
  int inst = B.inst_u[j];
  if (B.clk[5 * inst + 1] == 0.0)
    return;
  int lj = (int)(j - B.off_u[inst]), nx = B.nx[inst];
  const double *gi = gst + (long)B.off_b[inst] * V * 3;
  auto G = [&](int b) {
    double s = 0.0;
    for (int c = b - 2; c <= b; c++)
      if (c >= 0 && c <= nx + 1)
        s += gi[((long)c * V + k) * 3 + (b - c)];
    return s;
  };
  double add = G(lj + NN);
#pragma unroll
  for (int side = 0; side < 2; side++) {
    int code = B.bc[2 * inst + side];
#pragma unroll
    for (int g = 0; g < NN; g++) {
      if (bc_src_index(code, side, g, nx) == lj) {
        int b = side ? nx + NN + g : g;
        add += bc_sign(code == GPR_BC_PERIODIC ? GPR_BC_TRANSMISSIVE : code, k) * G(b);
      }
    }
  }
  ubar[j * V + k] += add;
}

// Per instance (one block each): sum the material-field and dt cotangents
// of the step, and propagate dt through the CFL rule.  tbar carries the
// cotangent of the clock: the clipped last step dt = tf - t passes -dtbar
// to every earlier step's dt.
template <class L>
__global__ void __launch_bounds__(128) k_adj_reduce(
    double *__restrict__ ubar, double *__restrict__ thbar, double *__restrict__ tbar,
    const double *__restrict__ thf, const double *__restrict__ thp, const double *__restrict__ dtf,
    const double *__restrict__ dtp, const double *__restrict__ un, const double *__restrict__ aux,
    const double *__restrict__ EVs, const double *__restrict__ EIGs, int frozen, Batch B) {
  constexpr int V = L::V, K = V + NPD, ND = Xi<L::THERMAL>::ND;
  const int inst = blockIdx.x;
  const double dt = B.clk[5 * inst + 1];
  if (dt == 0.0)
    return;
  __shared__ double red[128][NPD + 1];
  __shared__ double cf;
  const long ob = B.off_b[inst];
  const int nbi = B.nx[inst] + 2;
  double acc[NPD + 1];
#pragma unroll
  for (int p = 0; p <= NPD; p++)
    acc[p] = 0.0;
  for (int c = threadIdx.x; c < nbi; c += blockDim.x) {
    long cb = ob + c;
#pragma unroll
    for (int p = 0; p < NPD; p++)
      acc[p] += thf[(cb * 2) * NPD + p] + thf[(cb * 2 + 1) * NPD + p] + thp[cb * NPD + p];
    acc[NPD] += dtf[cb] + dtp[cb];
  }
#pragma unroll
  for (int p = 0; p <= NPD; p++)
    red[threadIdx.x][p] = acc[p];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int p = 0; p <= NPD; p++)
        red[threadIdx.x][p] += red[threadIdx.x + s][p];
    __syncthreads();
  }
  const bool clipped = aux[2 * inst] != 0.0;
  const long cstar = (long)aux[2 * inst + 1];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int p = 0; p < NPD; p++)
      thbar[inst * NPD + p] += red[0][p];
    double dtb = red[0][NPD];
    cf = 0.0;
    if (!frozen) {
      if (clipped) {
        tbar[inst] = -dtb;
      } else if (cstar >= 0) {
        double dtot = dtb + tbar[inst];
        double lam = EVs[inst];
        cf = -dtot * dt / lam;  // dt = cfl dx / lam  =>  d dt / d lam = -dt / lam
      }
    }
  }
  __syncthreads();
  if (cf != 0.0 && threadIdx.x < K) {
    const int k = threadIdx.x;
    double q[V];
#pragma unroll
    for (int j = 0; j < V; j++)
      q[j] = un[cstar * V + j];
    Dual lam;
    point_tangent<L>(q, k, B.P[inst], nullptr, nullptr, &lam, EIGs + (long)inst * ND);
    if (k < V)
      ubar[cstar * V + k] += cf * lam.d;
    else
      thbar[inst * NPD + (k - V)] += cf * lam.d;
  }
}

// Pointwise Jacobians (test hook): JF, JS [count][K][V], dlam [count][K].
template <class L>
__global__ void k_adj_point(const double *__restrict__ Q, long count, double *__restrict__ JF,
                            double *__restrict__ JS, double *__restrict__ dlam, DevPar P) {
  constexpr int V = L::V, K = V + NPD;
  long gid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (gid >= count * K)
    return;
  int k = gid % K;
  long c = gid / K;
  double q[V];
#pragma unroll
  for (int j = 0; j < V; j++)
    q[j] = Q[c * V + j];
  Dual F[V], S[V], lam;
  point_tangent<L>(q, k, P, F, S, &lam);
#pragma unroll
  for (int j = 0; j < V; j++) {
    JF[(c * K + k) * V + j] = F[j].d;
    JS[(c * K + k) * V + j] = S[j].d;
  }
  dlam[c * K + k] = lam.d;
}

// Pointwise VJPs (test hook): per point c, qb[c] = (dF/dq)^T Fb[c] +
// (dS/dq)^T Sb[c] + lb[c] dlambda/dq and thb[c] the same for the fields.
template <class L>
__global__ void k_adj_point_vjp(const double *__restrict__ Q, long count,
                                const double *__restrict__ Fb, const double *__restrict__ Sb,
                                const double *__restrict__ lb, double *__restrict__ qb,
                                double *__restrict__ thb, DevPar P) {
  constexpr int V = L::V;
  long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (c >= count)
    return;
  double q[V], f[V], s[V], o[V], th[NPD];
#pragma unroll
  for (int j = 0; j < V; j++) {
    q[j] = Q[c * V + j];
    f[j] = Fb[c * V + j];
    s[j] = Sb[c * V + j];
    o[j] = 0.0;
  }
#pragma unroll
  for (int p = 0; p < NPD; p++)
    th[p] = 0.0;
  point_vjp<L, true, true, true>(q, P, f, s, lb[c], nullptr, o, th);
#pragma unroll
  for (int j = 0; j < V; j++)
    qb[c * V + j] = o[j];
#pragma unroll
  for (int p = 0; p < NPD; p++)
    thb[c * NPD + p] = th[p];
}

}  // namespace gpr
