// gpr_order.cuh - the 1D ADER-WENO step for a general number of Gauss nodes
// NO (the reference's compile-time N, options.h:15), used for NO = 3 (third
// order: degree-2 polynomials in space and time).  The N = 2 kernels in
// gpr_kernels.cuh map a cell's N^(d+1) = 4 / 8 space-time nodes onto aligned
// lane groups and exchange values with warp shuffles; 9 nodes per cell do not
// align with a warp, so these kernels keep one thread per space-time node and
// exchange a cell's node values through shared memory.
//
// Restates for general N: etc/grid.cpp:12-146 (ghost cells), weno/weno.cpp:
// 4-81 (WENO with the central stencil of odd N, LAMC = 1e5), dg/dg1.cpp:
// 8-114 (Picard predictor), fv/fv.cpp:11-160 and fv/fluxes.cpp:9-75 (volume
// term and Rusanov interface terms of the 1D FV update).
#pragma once

#include <math.h>

#include "gpr_kernels.cuh"

namespace gpr {
namespace order {

constexpr double LAMC = 1e5;  // WENO central-stencil weight (options.h:25)

// The scheme's constants for NO Gauss-Legendre nodes on [0, 1], built on the
// host in FP64 and passed to the kernels by value.
template <int NO> struct ConstsN {
  double nodes[NO], w[NO];
  double endv[2][NO];                  // psi_j(0), psi_j(1)
  double derv[NO][NO];                 // psi_j'(x_i)
  double mLinv[NO][NO], mRinv[NO][NO];  // side stencils (cells i-N+1.., i..)
  double mCinv[NO][NO];                // central stencil of odd N
  double sig[NO][NO];                  // oscillation indicator
  double dgder[NO][NO];                // DG_DER
  double dgmatinv[NO][NO];             // (DG_END - DG_DER^T)^-1
  double dg_tol;
  int dg_it;
};

// ---- host construction (polynomials in the monomial basis) ----------------

template <int M> struct Poly {
  int n = 0;  // number of coefficients
  double c[M] = {};
  double eval(double x) const {
    double r = 0.0;
    for (int k = n - 1; k >= 0; k--)
      r = r * x + c[k];
    return r;
  }
  Poly diff() const {
    Poly d;
    d.n = n > 1 ? n - 1 : 1;
    for (int k = 1; k < n; k++)
      d.c[k - 1] = k * c[k];
    return d;
  }
  Poly integ() const {  // antiderivative with zero constant term
    Poly p;
    p.n = n + 1;
    for (int k = 0; k < n; k++)
      p.c[k + 1] = c[k] / (k + 1);
    return p;
  }
  Poly mul(const Poly &o) const {
    Poly p;
    p.n = n + o.n - 1;
    for (int a = 0; a < n; a++)
      for (int b = 0; b < o.n; b++)
        p.c[a + b] += c[a] * o.c[b];
    return p;
  }
};

// Gauss-Jordan inverse with partial pivoting (small matrices).
template <int NO> inline bool invert_small(const double (&a_)[NO][NO], double (&out)[NO][NO]) {
  double a[NO][2 * NO];
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < 2 * NO; j++)
      a[i][j] = j < NO ? a_[i][j] : (j - NO == i ? 1.0 : 0.0);
  for (int c = 0; c < NO; c++) {
    int p = c;
    for (int r = c + 1; r < NO; r++)
      if (fabs(a[r][c]) > fabs(a[p][c]))
        p = r;
    if (a[p][c] == 0.0)
      return false;
    for (int j = 0; j < 2 * NO; j++) {
      double t = a[c][j];
      a[c][j] = a[p][j];
      a[p][j] = t;
    }
    const double inv = 1.0 / a[c][c];
    for (int j = 0; j < 2 * NO; j++)
      a[c][j] *= inv;
    for (int r = 0; r < NO; r++)
      if (r != c) {
        const double f = a[r][c];
        for (int j = 0; j < 2 * NO; j++)
          a[r][j] -= f * a[c][j];
      }
  }
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++)
      out[i][j] = a[i][j + NO];
  return true;
}

template <int NO> inline ConstsN<NO> make_consts_n() {
  ConstsN<NO> C;
  // Gauss-Legendre nodes on [-1, 1]: Newton on P_NO from cos(pi (i + 3/4) /
  // (NO + 1/2)), weights 2 / ((1 - x^2) P'(x)^2), then symmetrised
  double x[NO], w[NO];
  for (int i = 0; i < NO; i++) {
    double z = cos(M_PI * (i + 0.75) / (NO + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = 0.0;
      for (int k = 1; k <= NO; k++) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      dp = NO * (z * p0 - p1) / (z * z - 1.0);
      const double dz = p0 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16)
        break;
    }
    x[NO - 1 - i] = z;
    w[NO - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  for (int i = 0; i < NO / 2; i++) {
    const double xs = 0.5 * (x[NO - 1 - i] - x[i]), ws = 0.5 * (w[i] + w[NO - 1 - i]);
    x[i] = -xs;
    x[NO - 1 - i] = xs;
    w[i] = w[NO - 1 - i] = ws;
  }
  if (NO % 2)
    x[NO / 2] = 0.0;
  for (int i = 0; i < NO; i++) {
    C.nodes[i] = (x[i] + 1.0) / 2.0;
    C.w[i] = w[i] / 2.0;
  }
  // Lagrange basis on the scaled nodes (poly/basis.cpp:22-53)
  Poly<2 * NO + 2> psi[NO];
  for (int i = 0; i < NO; i++) {
    Poly<2 * NO + 2> p;
    p.n = 1;
    p.c[0] = 1.0;
    for (int j = 0; j < NO; j++) {
      if (j == i)
        continue;
      Poly<2 * NO + 2> f;
      f.n = 2;
      f.c[0] = -C.nodes[j];
      f.c[1] = 1.0;
      p = p.mul(f);
      for (int k = 0; k < p.n; k++)
        p.c[k] /= (C.nodes[i] - C.nodes[j]);
    }
    psi[i] = p;
  }
  for (int j = 0; j < NO; j++) {
    C.endv[0][j] = psi[j].eval(0.0);
    C.endv[1][j] = psi[j].eval(1.0);
  }
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++)
      C.derv[i][j] = psi[j].diff().eval(C.nodes[i]);
  // WENO stencil matrices (weno/weno_matrices.cpp:9-28): the cell averages
  // of psi_j over the stencil's cells, cell 0 being [0, 1]
  const int cn2 = (NO - 1 + 1) / 2;  // ceil((N - 1) / 2)
  double mL[NO][NO], mR[NO][NO], mC[NO][NO];
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++) {
      const Poly<2 * NO + 2> P = psi[j].integ();
      mL[i][j] = P.eval(i - NO + 2) - P.eval(i - NO + 1);
      mR[i][j] = P.eval(i + 1) - P.eval(i);
      mC[i][j] = P.eval(i - cn2 + 1) - P.eval(i - cn2);
    }
  invert_small<NO>(mL, C.mLinv);
  invert_small<NO>(mR, C.mRinv);
  invert_small<NO>(mC, C.mCinv);
  // oscillation indicator (weno_matrices.cpp:30-42): sum over the
  // derivative orders 1..N-1 of int_0^1 psi_i^(a) psi_j^(a)
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++) {
      double s = 0.0;
      Poly<2 * NO + 2> di = psi[i], dj = psi[j];
      for (int a = 1; a < NO; a++) {
        di = di.diff();
        dj = dj.diff();
        const Poly<2 * NO + 2> P = di.mul(dj).integ();
        s += P.eval(1.0) - P.eval(0.0);
      }
      C.sig[i][j] = s;
    }
  // DG matrices (dg/dg_matrices.cpp:29-53)
  double dgmat[NO][NO];
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++) {
      if (i == j) {
        const double b1 = psi[i].eval(1.0), b0 = psi[i].eval(0.0);
        C.dgder[i][j] = (b1 * b1 - b0 * b0) / 2;
      } else {
        C.dgder[i][j] = C.w[i] * psi[j].diff().eval(C.nodes[i]);
      }
    }
  for (int i = 0; i < NO; i++)
    for (int j = 0; j < NO; j++)
      dgmat[i][j] = psi[i].eval(1.0) * psi[j].eval(1.0) - C.dgder[j][i];
  invert_small<NO>(dgmat, C.dgmatinv);
  C.dg_tol = 6e-6;
  C.dg_it = 50;
  return C;
}

// ---- kernels ---------------------------------------------------------------

// ub from u with NO ghost cells per side (grid.cpp:12-146 for 1D): one
// thread per (ub cell, variable).
template <int V, int NO>
__global__ void k_boundaries1d_n(const double *__restrict__ u, double *__restrict__ ub, int nx,
                                 int bcl, int bcr) {
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)(nx + 2 * NO) * V)
    return;
  const int k = idx % V;
  const int c = idx / V;
  if (c >= NO && c < nx + NO) {
    ub[idx] = u[(long)(c - NO) * V + k];
    return;
  }
  const int side = c >= nx + NO;
  const int i = side ? c - nx - NO : c;  // ghost 0..NO-1 of that side
  int code = side ? bcr : bcl;
  int si;
  if (code == GPR_BC_TRANSMISSIVE)
    si = side == 0 ? 0 : nx - 1;
  else if (code == GPR_BC_PERIODIC)
    si = side == 0 ? nx - NO + i : i;
  else
    si = side == 0 ? NO - 1 - i : nx - 1 - i;  // reflecting types
  if (code == GPR_BC_PERIODIC)
    code = GPR_BC_TRANSMISSIVE;  // plain copy
  ub[idx] = bc_value<V>(code, 0, k, u + (long)si * V);
}

// 1D WENO (weno.cpp:17-81): one thread per (predictor cell, variable);
// predictor cell i reads ub rows i .. i + 2N - 2.
template <int NO> GPR_D double weno_weight_n(const double *wv, const ConstsN<NO> &C, double lam) {
  double t = 0.0;
#pragma unroll
  for (int b = 0; b < NO; b++) {
    double tb = 0.0;
#pragma unroll
    for (int a = 0; a < NO; a++)
      tb += wv[a] * C.sig[a][b];
    t += tb * wv[b];
  }
  t += WENO_EPS;
  t *= t;
  t *= t;
  t *= t;
  return lam / t;
}

template <int V, int NO>
__global__ void k_weno1d_n(double *__restrict__ wh, const double *__restrict__ ub, int ncb,
                           ConstsN<NO> C) {
  static_assert(NO % 2 == 1 || NO == 2, "odd N (central stencil) or N = 2");
  long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)ncb * V)
    return;
  const int k = idx % V;
  const int i = idx / V;
  const double *d = ub + (long)i * V + k;
  double row[2 * NO - 1];
#pragma unroll
  for (int r = 0; r < 2 * NO - 1; r++)
    row[r] = d[(long)r * V];
  constexpr int FN2 = (NO - 1) / 2;  // floor((N - 1) / 2)
  double wL[NO], wR[NO], wC[NO];
#pragma unroll
  for (int a = 0; a < NO; a++) {
    double sL = 0.0, sR = 0.0, sC = 0.0;
#pragma unroll
    for (int b = 0; b < NO; b++) {
      sL += C.mLinv[a][b] * row[b];
      sR += C.mRinv[a][b] * row[NO - 1 + b];
      sC += C.mCinv[a][b] * row[FN2 + b];
    }
    wL[a] = sL;
    wR[a] = sR;
    wC[a] = sC;
  }
  const double oL = weno_weight_n<NO>(wL, C, LAMS), oR = weno_weight_n<NO>(wR, C, LAMS);
  const double oC = NO > 2 ? weno_weight_n<NO>(wC, C, LAMC) : 0.0;
  const double den = NO > 2 ? oL + oR + oC : oL + oR;
  double *out = wh + (long)i * NO * V + k;
#pragma unroll
  for (int a = 0; a < NO; a++) {
    double num = wL[a] * oL + wR[a] * oR;
    if (NO > 2)
      num += wC[a] * oC;
    out[(long)a * V] = num / den;
  }
}

// Cells per block of the node kernels: NP = N^2 threads per cell.
template <int NO> struct NodeBlock {
  static constexpr int NP = NO * NO;
  static constexpr int CPB = 128 / NP;
  static constexpr int THREADS = CPB * NP;
};

// Picard predictor (dg1.cpp:58-114): q <- DG_U^-1 (W w + dt R(q)) with the
// reference's initial guess q(t, s) = w(s), per-cell stopping rule |q1 - q0|
// <= dg_tol (1 + |q0|) and iteration cap.  One thread per space-time node
// g = t N + i of a cell; the cell's node values pass through shared memory.
// status[c]: GPR_PRED_PICARD | iterations << 8 when converged; cells that do
// not converge within the cap, or whose iterate turns NaN, get their last
// iterate and GPR_PRED_FAILED | iterations << 8 (there is no Newton pass for
// N != 2; the reference leaves such rows unwritten or calls its
// Newton-Krylov solver).
template <class L, int NO>
__global__ void __launch_bounds__(128) k_predictor1d_n(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, int32_t *__restrict__ status, double dt,
    const double *__restrict__ dt_dev, double idx, DevPar P, ConstsN<NO> C) {
  constexpr int V = L::V;
  using NB = NodeBlock<NO>;
  constexpr int NP = NB::NP, CPB = NB::CPB;
  __shared__ double sq[CPB][NP][V];
  __shared__ int cflag[CPB];
  if (dt_dev)
    dt = *dt_dev;
  const int lc = threadIdx.x / NP;  // cell within the block
  const int g = threadIdx.x % NP;
  const bool in_block = threadIdx.x < NB::THREADS;
  const long c = (long)blockIdx.x * CPB + lc;
  const bool valid = in_block && c < ncb;
  const bool active = valid && (mask == nullptr || mask[c]);
  const int t = g / NO, i = g % NO;
  const long cc = valid ? c : 0;  // lanes without a cell read cell 0's data
  double w[V], Ww[V], q[V], r[V], qn[V];
  const double *wc = wh + (cc * NO + i) * V;
  const double f = C.endv[0][t] * C.w[i];
#pragma unroll
  for (int k = 0; k < V; k++) {
    w[k] = wc[k];
    Ww[k] = f * w[k];
    q[k] = w[k];
  }
  bool done = !active, nan_seen = false;
  int iters = 0;
  const double wn = C.w[t] * C.w[i];
  for (int it = 0; it < C.dg_it; it++) {
    if (!__syncthreads_or(!done))
      break;
    Prim<L::THERMAL> s;
    prim<L::THERMAL>(q, P, s);
    // W (S - B dq/dx) with the node weight in the source's factors
    source<L::THERMAL, V>(q, s, P, r, wn);
    if (in_block) {
#pragma unroll
      for (int k = 0; k < V; k++)
        sq[lc][g][k] = q[k];
    }
    __syncthreads();
    {
      double dq[V];
#pragma unroll
      for (int k = 0; k < V; k++) {
        double a = 0.0;
#pragma unroll
        for (int m = 0; m < NO; m++)
          a += C.derv[i][m] * (in_block ? sq[lc][t * NO + m][k] : 0.0);
        dq[k] = a * idx * wn;
      }
      double bd[V];
      bdot<V, L::LSET>(s.v, dq, 0, bd);
#pragma unroll
      for (int k = 0; k < V; k++)
        r[k] -= bd[k];
    }
    __syncthreads();
    // - W_t DG_DER(i, m) F(t, m) / dx
    double F[V];
    flux_set<L::THERMAL, V>(q, s, 0, P, F);
    if (in_block) {
#pragma unroll
      for (int k = 0; k < V; k++)
        sq[lc][g][k] = F[k];
    }
    __syncthreads();
    const double wx = C.w[t] * idx;
#pragma unroll
    for (int k = 0; k < V; k++) {
      if (!flux_support<L::THERMAL>(k, 0))
        continue;
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.dgder[i][m] * (in_block ? sq[lc][t * NO + m][k] : 0.0);
      r[k] -= wx * a;
    }
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] = r[k] * dt + Ww[k];
    __syncthreads();
    if (in_block) {
#pragma unroll
      for (int k = 0; k < V; k++)
        sq[lc][g][k] = r[k];
    }
    if (in_block && g == 0)
      cflag[lc] = 0;
    __syncthreads();
    // q_new(t, i) = sum_m DG_MATinv[t][m] r(m, i) / W_i
    const double iw = 1.0 / C.w[i];
#pragma unroll
    for (int k = 0; k < V; k++) {
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.dgmatinv[t][m] * (in_block ? sq[lc][m * NO + i][k] : 0.0);
      qn[k] = a * iw;
    }
    bool big = false, hasnan = false;
#pragma unroll
    for (int k = 0; k < V; k++) {
      if (fabs(qn[k] - q[k]) > C.dg_tol * (1.0 + fabs(q[k])))
        big = true;
      if (qn[k] != qn[k])
        hasnan = true;
    }
    if (in_block && !done && (big || hasnan))
      atomicOr(&cflag[lc], (big ? 1 : 0) | (hasnan ? 2 : 0));
    __syncthreads();
    if (!done) {
      const int fl = cflag[lc];
      iters = it + 1;
#pragma unroll
      for (int k = 0; k < V; k++)
        q[k] = qn[k];
      if (fl & 1) {
        // not converged: iterate on
      } else if (fl & 2) {
        nan_seen = true;
        done = true;
      } else {
        done = true;
        double *out = qh + (c * NP + g) * V;
#pragma unroll
        for (int k = 0; k < V; k++)
          out[k] = q[k];
        if (status && g == 0)
          status[c] = GPR_PRED_PICARD | (iters << 8);
      }
    }
  }
  if (active && (!done || nan_seen)) {
    double *out = qh + (c * NP + g) * V;
#pragma unroll
    for (int k = 0; k < V; k++)
      out[k] = q[k];
    if (status && g == 0)
      status[c] = GPR_PRED_FAILED | (iters << 8);
  }
  if (valid && !active && status && g == 0)
    status[c] = GPR_PRED_PICARD;
}

// 1D face terms (interfs1, fv.cpp:111-160; D_RUS and Bint, fluxes.cpp:9-75):
// one thread per (face, time node t); face f lies between predictor cells f
// and f + 1.  fb[f][t][0][V] = k (b + f) is subtracted from the left cell,
// fb[f][t][1][V] = k (b - f) from the right one, k = W_t dt / (2 dx).
template <class L, int NO>
__global__ void __launch_bounds__(128) k_faces1d_n(
    double *__restrict__ fb, const double *__restrict__ qh, long nface,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    DevPar P, ConstsN<NO> C) {
  constexpr int V = L::V;
  if (dt_dev)
    dt = *dt_dev;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long face = gt / NO;
  const int t = gt % NO;
  if (face >= nface)
    return;
  double *o = fb + ((face * NO + t) * 2) * V;
  const bool active = mask == nullptr || (mask[face] && mask[face + 1]);
  if (!active) {
#pragma unroll
    for (int k = 0; k < V; k++)
      o[k] = o[V + k] = 0.0;
    return;
  }
  const double *ql_ = qh + (face * NO + t) * NO * V;
  const double *qr_ = qh + ((face + 1) * NO + t) * NO * V;
  double ql[V], qr[V], f[V], b[V], dq[V];
#pragma unroll
  for (int k = 0; k < V; k++) {
    double a = 0.0, e = 0.0;
#pragma unroll
    for (int j = 0; j < NO; j++) {
      a += C.endv[1][j] * ql_[j * V + k];
      e += C.endv[0][j] * qr_[j * V + k];
    }
    ql[k] = a;
    qr[k] = e;
  }
  Prim<L::THERMAL> sl, sr;
  prim<L::THERMAL>(ql, P, sl);
  prim<L::THERMAL>(qr, P, sr);
  const double m1 = max_abs_eigs<L::THERMAL>(ql, sl, 0, P);
  const double m2 = max_abs_eigs<L::THERMAL>(qr, sr, 0, P);
  const double m = m1 > m2 ? m1 : m2;
#pragma unroll
  for (int k = 0; k < V; k++) {
    f[k] = m * (ql[k] - qr[k]);
    dq[k] = qr[k] - ql[k];
    b[k] = 0.0;
  }
  flux_add<L::THERMAL, V>(ql, sl, 0, P, f);
  flux_add<L::THERMAL, V>(qr, sr, 0, P, f);
  // Bint: sum_n W_n B(qL + x_n dq) dq over the NO path nodes
#pragma unroll
  for (int n = 0; n < NO; n++) {
    const double ir = 1.0 / (ql[0] + C.nodes[n] * dq[0]);
    double v[3] = {(ql[2] + C.nodes[n] * dq[2]) * ir, (ql[3] + C.nodes[n] * dq[3]) * ir,
                   (ql[4] + C.nodes[n] * dq[4]) * ir};
    double bd[V];
    bdot<V, L::LSET>(v, dq, 0, bd);
#pragma unroll
    for (int k = 5; k < V; k++)
      if (k < 14 || k >= V - L::LSET)
        b[k] += C.w[n] * bd[k];
  }
  const double kk = dt * C.w[t] / (2.0 * dx);
#pragma unroll
  for (int k = 0; k < V; k++) {
    o[k] = kk * (b[k] + f[k]);
    o[V + k] = kk * (b[k] - f[k]);
  }
}

// The 1D FV update of interior cell c (predictor cell c + 1): the volume
// term (centers1, fv.cpp:11-58) over its NO x NO space-time nodes, one
// thread per node, summed through shared memory, then the face terms of its
// left face c (right part) and right face c + 1 (left part).
template <class L, int NO>
__global__ void __launch_bounds__(128) k_cells1d_n(
    double *__restrict__ u, const double *__restrict__ qh, const double *__restrict__ fb, int nx,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    DevPar P, ConstsN<NO> C) {
  constexpr int V = L::V;
  using NB = NodeBlock<NO>;
  constexpr int NP = NB::NP, CPB = NB::CPB;
  __shared__ double sq[CPB][NP][V];
  if (dt_dev)
    dt = *dt_dev;
  const int lc = threadIdx.x / NP;
  const int g = threadIdx.x % NP;
  const bool in_block = threadIdx.x < NB::THREADS;
  const long c = (long)blockIdx.x * CPB + lc;
  const bool valid = in_block && c < nx;
  const long cb = (valid ? c : 0) + 1;  // lanes without a cell read cell 0's nodes
  const bool active = valid && (mask == nullptr || mask[cb]);
  const int t = g / NO, i = g % NO;
  const double idx = 1.0 / dx;
  double q[V], acc[V];
  const double *qc = qh + (cb * NP + (in_block ? g : 0)) * V;
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = qc[k];
  if (in_block) {
#pragma unroll
    for (int k = 0; k < V; k++)
      sq[lc][g][k] = q[k];
  }
  __syncthreads();
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(q, P, s);
  const double wn = dt * C.w[t] * C.w[i];
  source<L::THERMAL, V>(q, s, P, acc, wn);
  {
    double dq[V];
#pragma unroll
    for (int k = 0; k < V; k++) {
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.derv[i][m] * (in_block ? sq[lc][t * NO + m][k] : 0.0);
      dq[k] = a * idx * wn;
    }
    double bd[V];
    bdot<V, L::LSET>(s.v, dq, 0, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      acc[k] -= bd[k];
  }
  __syncthreads();
  if (in_block) {
#pragma unroll
    for (int k = 0; k < V; k++)
      sq[lc][g][k] = acc[k];
  }
  __syncthreads();
  if (!active)
    return;
  // lane g sums variables g, g + NP, ... over the cell's nodes in node order
  const double *fl = fb + (long)c * NO * 2 * V;        // left face c: right part
  const double *fr = fb + (long)(c + 1) * NO * 2 * V;  // right face c + 1: left part
  const bool okl = mask == nullptr || (mask[cb - 1] && mask[cb]);
  const bool okr = mask == nullptr || (mask[cb] && mask[cb + 1]);
  double *uc = u + c * V;
  for (int k = g; k < V; k += NP) {
    double x = 0.0;
#pragma unroll
    for (int n = 0; n < NP; n++)
      x += sq[lc][n][k];
    x += uc[k];
#pragma unroll
    for (int tt = 0; tt < NO; tt++) {
      if (okr)
        x -= fr[tt * 2 * V + k];
      if (okl)
        x -= fl[tt * 2 * V + V + k];
    }
    uc[k] = x;
  }
}

}  // namespace order
}  // namespace gpr
