// gpr_order.cuh - the 1D and 2D ADER-WENO step for a general number of
// Gauss nodes NO (the reference's compile-time N, options.h:15), used for
// NO = 3 (third order: degree-2 polynomials in space and time).  The N = 2
// kernels in gpr_kernels.cuh map a cell's N^(d+1) = 4 / 8 space-time nodes
// onto aligned lane groups and exchange values with warp shuffles; 9 or 27
// nodes per cell do not align with a warp, so these kernels keep one thread
// per space-time node and exchange a cell's node values through shared
// memory.
//
// Restates for general N: etc/grid.cpp:12-170 (ghost cells), weno/weno.cpp:
// 4-124 (WENO with the central stencil of odd N, LAMC = 1e5), dg/dg1.cpp:
// 8-114 and dg/dg2.cpp:8-171 (Picard predictor), fv/fv.cpp:11-279 and
// fv/fluxes.cpp:9-75 (volume term and Rusanov interface terms of the FV
// update).
#pragma once

#include <math.h>

#include "gpr_kernels.cuh"
#include "gpr_osher.cuh"

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
  double dgmat[NO][NO];                // DG_END - DG_DER^T
  double dgmatinv[NO][NO];             // its inverse
  double dg_tol, stiff_tol;
  int dg_it, stiff_it;
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
      C.dgmat[i][j] = psi[i].eval(1.0) * psi[j].eval(1.0) - C.dgder[j][i];
  invert_small<NO>(C.dgmat, C.dgmatinv);
  C.dg_tol = 6e-6;
  C.dg_it = 50;
  C.stiff_tol = 1e-11;  // the stiff Newton pass: as the N = 2 library's
  C.stiff_it = 60;
  return C;
}

// ---- kernels ---------------------------------------------------------------

// Ghost-cell index along one axis (etc/grid.cpp:12-146): ghost i (0..NO-1)
// of side `side` reads interior line index bc_src; periodic reads wrap.
template <int NO> GPR_D int bc_src_n(int code, int side, int i, int n) {
  if (code == GPR_BC_TRANSMISSIVE)
    return side == 0 ? 0 : n - 1;
  if (code == GPR_BC_PERIODIC)
    return side == 0 ? n - NO + i : i;
  return side == 0 ? NO - 1 - i : n - 1 - i;  // reflecting types
}

// ub from u with NO ghost cells per side (grid.cpp:12-170): one thread per
// ub cell.  In 2D the x ghosts of the interior rows come first and the y
// ghosts of every row (corners included) are taken from them, as the
// reference's two passes do: a corner is the y boundary transform of the x
// boundary transform of its interior source.
template <int V, int NO>
__global__ void k_boundaries_n(const double *__restrict__ u, double *__restrict__ ub, int nx,
                               int ny, int nd, int bx0, int bx1, int by0, int by1) {
  const long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int nyb = nd == 1 ? 1 : ny + 2 * NO;
  if (c >= (long)(nx + 2 * NO) * nyb)
    return;
  const int a = nd == 1 ? (int)c : (int)(c / nyb), b = nd == 1 ? 0 : (int)(c % nyb);
  int ai = a - NO, bj = nd == 1 ? 0 : b - NO;
  int cx = -1, cy = -1;  // boundary codes applied (-1: interior along that axis)
  if (ai < 0 || ai >= nx) {
    const int side = ai >= nx;
    cx = side ? bx1 : bx0;
    ai = bc_src_n<NO>(cx, side, side ? ai - nx : a, nx);
  }
  if (nd == 2 && (bj < 0 || bj >= ny)) {
    const int side = bj >= ny;
    cy = side ? by1 : by0;
    bj = bc_src_n<NO>(cy, side, side ? bj - ny : b, ny);
  }
  double q[V], w[V];
  const double *src = u + ((long)ai * (nd == 1 ? 1 : ny) + bj) * V;
#pragma unroll
  for (int k = 0; k < V; k++)
    q[k] = src[k];
  if (cx >= 0 && cx != GPR_BC_PERIODIC) {
#pragma unroll
    for (int k = 0; k < V; k++)
      w[k] = bc_value<V>(cx, 0, k, q);
#pragma unroll
    for (int k = 0; k < V; k++)
      q[k] = w[k];
  }
  if (cy >= 0 && cy != GPR_BC_PERIODIC) {
#pragma unroll
    for (int k = 0; k < V; k++)
      w[k] = bc_value<V>(cy, 1, k, q);
#pragma unroll
    for (int k = 0; k < V; k++)
      q[k] = w[k];
  }
  double *dst = ub + c * V;
#pragma unroll
  for (int k = 0; k < V; k++)
    dst[k] = q[k];
}

// WENO (weno.cpp:4-124) at general N.
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

// coeffs (weno.cpp:17-73) for one variable: data rows d[r * sd] (r = 0 ..
// 2N-2), node values out[a * so]; the side stencils are left out near the
// ends (`gap`, the reference's NO_CORNERS handling) as the reference does.
template <int NO>
GPR_D void weno_point_n(const double *__restrict__ d, long sd, double *__restrict__ out, long so,
                        int ind, int n, int gap, const ConstsN<NO> &C) {
  static_assert(NO % 2 == 1 || NO == 2, "odd N (central stencil) or N = 2");
  double row[2 * NO - 1];
#pragma unroll
  for (int r = 0; r < 2 * NO - 1; r++)
    row[r] = d[(long)r * sd];
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
  const bool useL = ind >= gap, useR = ind <= n - gap - 1, useC = NO > 2 && ind + FN2 >= gap;
  const double oL = weno_weight_n<NO>(wL, C, LAMS), oR = weno_weight_n<NO>(wR, C, LAMS);
  const double oC = NO > 2 ? weno_weight_n<NO>(wC, C, LAMC) : 0.0;
  double den = 0.0;
  if (useL)
    den += oL;
  if (useR)
    den += oR;
  if (useC)
    den += oC;
#pragma unroll
  for (int a = 0; a < NO; a++) {
    double num = 0.0;
    if (useL)
      num += wL[a] * oL;
    if (useR)
      num += wR[a] * oR;
    if (useC)
      num += wC[a] * oC;
    out[(long)a * so] = num / den;
  }
}

// 1D: wh[i][a][k] for predictor cell i from ub rows i .. i + 2N - 2.
template <int V, int NO>
__global__ void k_weno1d_n(double *__restrict__ wh, const double *__restrict__ ub, int ncb,
                           ConstsN<NO> C) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)ncb * V)
    return;
  const int k = idx % V;
  const int i = idx / V;
  weno_point_n<NO>(ub + (long)i * V + k, V, wh + (long)i * NO * V + k, V, i, ncb, 0, C);
}

// 2D x sweep (weno.cpp:93-104): ux[i][j][a][k] for i < nx + 2 over every
// ub column j < ny + 2N; the columns within N of the edges leave out their
// side stencils beyond the first N rows.
template <int V, int NO>
__global__ void k_weno2d_x_n(double *__restrict__ ux, const double *__restrict__ ub, int nxp,
                             int nyb, ConstsN<NO> C) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)nxp * nyb * V)
    return;
  const int k = idx % V;
  const long rest = idx / V;
  const int j = rest % nyb, i = rest / nyb;
  const int gap = (j < NO || j >= nyb - NO) ? NO : 0;
  weno_point_n<NO>(ub + ((long)i * nyb + j) * V + k, (long)nyb * V,
                   ux + ((long)i * nyb + j) * NO * V + k, V, i, nxp, gap, C);
}

// 2D y sweep (weno.cpp:106-121): wh[i][j][ii][jj][k] from ux rows j .. j + 2N - 2.
template <int V, int NO>
__global__ void k_weno2d_y_n(double *__restrict__ wh, const double *__restrict__ ux, int nxp,
                             int nyp, ConstsN<NO> C) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)nxp * nyp * NO * V)
    return;
  const int k = idx % V;
  long rest = idx / V;
  const int ii = rest % NO;
  rest /= NO;
  const int j = rest % nyp, i = rest / nyp;
  const int nyb = nyp + 2 * (NO - 1);
  const int gap = (i == 0 || i == nxp - 1) ? 1 : 0;
  weno_point_n<NO>(ux + (((long)i * nyb + j) * NO + ii) * V + k, (long)NO * V,
                   wh + (((long)i * nyp + j) * NO * NO + ii * NO) * V + k, V, j, nyp, gap, C);
}

// Node kernels: one thread per space-time node, NP = N^(d+1) per cell,
// g = t NS + s with s = i (1D) or i N + j (2D, x-node major), NS = N^d.
template <int NO, int ND> struct NodeBlock {
  static constexpr int NS = ND == 1 ? NO : NO * NO;
  static constexpr int NP = NO * NS;
  static constexpr int CPB = 128 / NP;
  static constexpr int THREADS = CPB * NP;
};

// r = W w + dt R(q) at one space-time node (the Picard right-hand side,
// dg1.cpp:75-89, dg2.cpp:115-150): R = W (S - B dq/dx [- B dq/dy]) - W_t
// [W_j] DG_DER F_x / dx [- W_t W_i DG_DER F_y / dy].  The cell's node values
// pass through sq (NP x V doubles); every thread of the block calls it (it
// synchronises the block) and threads without a node (in_block false) read
// zeros.
template <class L, int NO, int ND>
GPR_D void picard_rhs_n(const double *q, const double *Ww, double *r, double (*sq)[L::V],
                        bool in_block, int g, int t, int i, int j, double wn, double dt,
                        double idx, double idy, const DevPar &P, const ConstsN<NO> &C) {
  constexpr int V = L::V;
  constexpr int NS = NodeBlock<NO, ND>::NS;
  // the partner node of this one with the x (y) index replaced by m
  auto nx_of = [&](int m) { return ND == 1 ? t * NS + m : t * NS + m * NO + j; };
  auto ny_of = [&](int m) { return t * NS + i * NO + m; };
  Prim<L::THERMAL> s;
  prim<L::THERMAL>(q, P, s);
  // W (S - B dq/dx [- B dq/dy]) with the node weight in the source's factors
  source<L::THERMAL, V>(q, s, P, r, wn);
  if (in_block) {
#pragma unroll
    for (int k = 0; k < V; k++)
      sq[g][k] = q[k];
  }
  __syncthreads();
#pragma unroll
  for (int dir = 0; dir < ND; dir++) {
    const int e = dir == 0 ? i : j;
    const double h = dir == 0 ? idx : idy;
    double dq[V];
#pragma unroll
    for (int k = 0; k < V; k++) {
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.derv[e][m] * (in_block ? sq[dir == 0 ? nx_of(m) : ny_of(m)][k] : 0.0);
      dq[k] = a * h * wn;
    }
    double bd[V];
    bdot<V, L::LSET>(s.v, dq, dir, bd);
#pragma unroll
    for (int k = 0; k < V; k++)
      r[k] -= bd[k];
  }
  // - W_t [W_j] DG_DER(i, m) F_x(t, m, j) / dx [- W_t W_i DG_DER(j, m) F_y(t, i, m) / dy]
#pragma unroll
  for (int dir = 0; dir < ND; dir++) {
    double F[V];
    flux_set<L::THERMAL, V>(q, s, dir, P, F);
    __syncthreads();
    if (in_block) {
#pragma unroll
      for (int k = 0; k < V; k++)
        sq[g][k] = F[k];
    }
    __syncthreads();
    const int e = dir == 0 ? i : j;
    const double wx = dir == 0 ? C.w[t] * (ND == 1 ? 1.0 : C.w[j]) * idx
                               : C.w[t] * C.w[i] * idy;
#pragma unroll
    for (int k = 0; k < V; k++) {
      if (!flux_support<L::THERMAL>(k, dir))
        continue;
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.dgder[e][m] * (in_block ? sq[dir == 0 ? nx_of(m) : ny_of(m)][k] : 0.0);
      r[k] -= wx * a;
    }
  }
#pragma unroll
  for (int k = 0; k < V; k++)
    r[k] = r[k] * dt + Ww[k];
}

// Picard predictor (dg1.cpp:58-114, dg2.cpp:102-171): q <- DG_U^-1 (W w +
// dt R(q)) with the reference's initial guess q(t, s) = w(s), per-cell
// stopping rule |q1 - q0| <= dg_tol (1 + |q0|) and iteration cap (none with
// STIFF: every cell goes to the Newton pass).  The cell's node values pass
// through shared memory.  status[c]: GPR_PRED_PICARD | iterations << 8 when
// converged; a cell that does not converge within the cap, or whose
// iterate turns NaN, gets the initial guess with a NaN marker in its first
// entry (0x7ff8000000000bad) and GPR_PRED_FAILED | iterations << 8, and
// k_predictor_stiff_n finishes it (the reference leaves such rows unwritten
// or calls its Newton-Krylov solver).
template <class L, int NO, int ND>
__global__ void __launch_bounds__(128) k_predictor_n(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, int32_t *__restrict__ status, double dt,
    const double *__restrict__ dt_dev, double idx, double idy, int stiff, DevPar P,
    ConstsN<NO> C) {
  constexpr int V = L::V;
  using NB = NodeBlock<NO, ND>;
  constexpr int NS = NB::NS, NP = NB::NP, CPB = NB::CPB;
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
  const int t = g / NS, sidx = g % NS;
  const int i = ND == 1 ? sidx : sidx / NO, j = ND == 1 ? 0 : sidx % NO;
  const long cc = valid ? c : 0;  // lanes without a cell read cell 0's data
  double w[V], Ww[V], q[V], r[V], qn[V];
  const double *wc = wh + (cc * NS + (in_block ? sidx : 0)) * V;
  const double ws = ND == 1 ? C.w[i] : C.w[i] * C.w[j];
  const double f = C.endv[0][t] * ws;
#pragma unroll
  for (int k = 0; k < V; k++) {
    w[k] = wc[k];
    Ww[k] = f * w[k];
    q[k] = w[k];
  }
  bool done = !active, nan_seen = false;
  int iters = 0;
  const double wn = C.w[t] * ws;
  double(*sqc)[V] = sq[in_block ? lc : 0];
  const int maxit = stiff ? 0 : C.dg_it;
  for (int it = 0; it < maxit; it++) {
    if (!__syncthreads_or(!done))
      break;
    picard_rhs_n<L, NO, ND>(q, Ww, r, sqc, in_block, g, t, i, j, wn, dt, idx, idy, P, C);
    __syncthreads();
    if (in_block) {
#pragma unroll
      for (int k = 0; k < V; k++)
        sq[lc][g][k] = r[k];
    }
    if (in_block && g == 0)
      cflag[lc] = 0;
    __syncthreads();
    // q_new(t, s) = sum_m DG_MATinv[t][m] r(m, s) / W_s
    const double iw = 1.0 / ws;
#pragma unroll
    for (int k = 0; k < V; k++) {
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++)
        a += C.dgmatinv[t][m] * (in_block ? sq[lc][m * NS + sidx][k] : 0.0);
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
      out[k] = w[k];
    if (g == 0)
      out[0] = __longlong_as_double(0x7ff8000000000badll);
    if (status && g == 0)
      status[c] = GPR_PRED_FAILED | (iters << 8);
  }
  if (valid && !active && status && g == 0)
    status[c] = GPR_PRED_PICARD;
}

// Stiff-source Newton pass at NO nodes for the cells the Picard pass marked
// (first entry 0x7ff8000000000bad): the N = 2 pass's iteration (the exact
// local Jacobian of the relaxation sources, stiff_jacobian_rows, with the
// correction systems in FP32 and the residual in FP64, so the converged
// point is the FP64 fixed point), from the initial guess, with the NO time
// nodes of a spatial node coupled through DG_MAT in one (9 NO) x (9 NO)
// system for A and one (3 NO) x (3 NO) system for rho J, as the oracle's
// dg_stiff:
//   (DG_MAT (x) I - dt W_t dS/dq) delta = (W w + dt R(q) - W_s DG_MAT q) / W_s,
// the other variables by DG_MAT^-1.  One cell at a time per one-warp block
// (NP <= 27 node lanes); the lanes first test 32 cells' markers at once and
// the block then takes the marked ones in turn.
template <class L, int NO, int ND> struct StiffN {
  static constexpr int NS = NodeBlock<NO, ND>::NS;
  static constexpr int NP = NodeBlock<NO, ND>::NP;
  static constexpr int NA = 9 * NO, NJ = 3 * NO;
  // odd: the solver lanes of neighbouring spatial nodes start on different banks
  static constexpr int per_node = (NA * NA + NA + (L::THERMAL ? NJ * NJ + NJ : 0)) | 1;
};

template <class L, int NO, int ND>
__global__ void __launch_bounds__(32) k_predictor_stiff_n(
    double *__restrict__ qh, const double *__restrict__ wh, long ncb,
    const uint8_t *__restrict__ mask, int32_t *__restrict__ status, double dt,
    const double *__restrict__ dt_dev, double idx, double idy, DevPar P, ConstsN<NO> C) {
  constexpr int V = L::V;
  using SN = StiffN<L, NO, ND>;
  constexpr int NS = SN::NS, NP = SN::NP, NA = SN::NA, NJ = SN::NJ;
  static_assert(NP <= 32, "one cell per warp");
  __shared__ double sq[NP][V];
  __shared__ float sm[NS * SN::per_node];
  if (dt_dev)
    dt = *dt_dev;
  const int lane = threadIdx.x;
  const bool in_block = lane < NP;
  const int g = in_block ? lane : 0;
  const int t = g / NS, sidx = g % NS;
  const int i = ND == 1 ? sidx : sidx / NO, j = ND == 1 ? 0 : sidx % NO;
  const double ws = ND == 1 ? C.w[i] : C.w[i] * C.w[j];
  const double f = C.endv[0][t] * ws;
  const double wn = C.w[t] * ws;
  const double a_t = dt * C.w[t];
  float *Am = sm + sidx * SN::per_node;  // (9 NO) x (9 NO)
  float *Ab = Am + NA * NA;              // 9 NO
  float *Jm = Ab + NA;                   // (3 NO) x (3 NO)
  float *Jb = Jm + NJ * NJ;              // 3 NO
  for (long base = (long)blockIdx.x * 32; base < ncb; base += (long)gridDim.x * 32) {
    const long cl = base + lane;
    bool marked = false;
    if (cl < ncb && (mask == nullptr || mask[cl])) {
      const double flag = qh[cl * NP * V];
      marked = flag != flag;
    }
    unsigned todo = __ballot_sync(0xffffffffu, marked);
    while (todo) {  // uniform over the block (one warp)
      const long c = base + __ffs(todo) - 1;
      todo &= todo - 1;
      double Ww[V], q[V], r[V], delta[V];
      const double *wc = wh + (c * NS + sidx) * V;
#pragma unroll
      for (int k = 0; k < V; k++) {
        const double w = wc[k];
        Ww[k] = f * w;
        q[k] = w;
      }
      bool ok = false;
      int iters = 0;
      for (int it = 0; it < C.stiff_it; it++) {
        __syncthreads();  // the previous iteration's reads of sq and sm are done
        picard_rhs_n<L, NO, ND>(q, Ww, r, sq, in_block, g, t, i, j, wn, dt, idx, idy, P, C);
        // residual r - W_s sum_m DG_MAT[t][m] q(m, s)
        __syncthreads();
        if (in_block) {
#pragma unroll
          for (int k = 0; k < V; k++)
            sq[g][k] = q[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < V; k++) {
          double uq = 0.0;
#pragma unroll
          for (int m = 0; m < NO; m++)
            uq += C.dgmat[t][m] * sq[m * NS + sidx][k];
          r[k] -= ws * uq;
        }
        if (in_block) {
          // this time node's rows of the two systems: the diagonal block
          // DG_MAT[t][t] I - dt W_t dS/dq, the others DG_MAT[t][t2] I
          Prim<L::THERMAL> st;
          prim<L::THERMAL>(q, P, st);
          stiff_jacobian_rows<L::THERMAL>(q, st, P, a_t, C.dgmat[t][t], Am + t * 9 * NA + t * 9,
                                          NA, Jm + t * 3 * NJ + t * 3, NJ);
#pragma unroll
          for (int t2 = 0; t2 < NO; t2++) {
            if (t2 == t)
              continue;
            const float m = (float)C.dgmat[t][t2];
#pragma unroll
            for (int a = 0; a < 9; a++)
#pragma unroll
              for (int b = 0; b < 9; b++)
                Am[(t * 9 + a) * NA + t2 * 9 + b] = a == b ? m : 0.0f;
            if (L::THERMAL) {
#pragma unroll
              for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++)
                  Jm[(t * 3 + a) * NJ + t2 * 3 + b] = a == b ? m : 0.0f;
            }
          }
#pragma unroll
          for (int a = 0; a < 9; a++)
            Ab[t * 9 + a] = (float)(r[5 + a] / ws);
          if (L::THERMAL) {
#pragma unroll
            for (int a = 0; a < 3; a++)
              Jb[t * 3 + a] = (float)(r[14 + a] / ws);
          }
        }
        __syncthreads();
        bool solved = true;
        if (in_block && t == 0)
          solved = smem_solve<NA>(Am, NA, Ab);
        else if (L::THERMAL && in_block && t == 1)
          solved = smem_solve<NJ>(Jm, NJ, Jb);
        // the other variables: DG_MAT^-1 of the residual, / W_s
        if (in_block) {
#pragma unroll
          for (int k = 0; k < V; k++)
            sq[g][k] = r[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < V; k++) {
          double acc = 0.0;
#pragma unroll
          for (int m = 0; m < NO; m++)
            acc += C.dgmatinv[t][m] * sq[m * NS + sidx][k];
          delta[k] = acc / ws;
        }
#pragma unroll
        for (int a = 0; a < 9; a++)
          delta[5 + a] = (double)Ab[t * 9 + a];
        if (L::THERMAL) {
#pragma unroll
          for (int a = 0; a < 3; a++)
            delta[14 + a] = (double)Jb[t * 3 + a];
        }
        bool big = false, bad = !solved;
#pragma unroll
        for (int k = 0; k < V; k++) {
          const double qn = q[k] + delta[k];
          if (fabs(delta[k]) > C.stiff_tol * (1.0 + fabs(qn)))
            big = true;
          if (qn != qn)
            bad = true;
          q[k] = qn;
        }
        const int anybad = __syncthreads_or(in_block && bad);
        const int anybig = __syncthreads_or(in_block && big);
        iters = it + 1;
        if (anybad)
          break;
        if (!anybig) {
          ok = true;
          break;
        }
      }
      if (in_block) {
        double *out = qh + (c * NP + g) * V;
#pragma unroll
        for (int k = 0; k < V; k++)
          out[k] = q[k];
        if (status && g == 0)
          status[c] = (ok ? GPR_PRED_NEWTON : GPR_PRED_FAILED) | (iters << 8);
      }
    }
  }
}

// Interface terms of one face point (D_RUS / D_ROE / D_OSH and Bint,
// fluxes.cpp:9-75, with NO path nodes): f = D + F(qL) + F(qR), D =
// max(lambda_L, lambda_R) (qL - qR) for Rusanov (EIG false) or the eigen
// part of D_ROE / D_OSH (EIG true, flux GPR_FLUX_ROE or GPR_FLUX_OSHER, one
// 17 x 17 eigen-decomposition per path node for Osher, one of the
// path-averaged matrix for Roe); b = sum_n W_n B(qL + x_n dq) dq.
template <class L, int NO, bool EIG = false>
GPR_D void interface_point_n(const double *ql, const double *qr, int d, const DevPar &P,
                             const ConstsN<NO> &C, double *f, double *b, int flux = 0) {
  constexpr int V = L::V;
  Prim<L::THERMAL> sl, sr;
  prim<L::THERMAL>(ql, P, sl);
  prim<L::THERMAL>(qr, P, sr);
  double dq[V];
  if (EIG) {
    eig_dissipation_qd<L, NO>(ql, qr, d, flux, P, C.nodes, C.w, f);
#pragma unroll
    for (int k = 0; k < V; k++) {
      dq[k] = qr[k] - ql[k];
      b[k] = 0.0;
    }
  } else {
    const double m1 = max_abs_eigs<L::THERMAL>(ql, sl, d, P);
    const double m2 = max_abs_eigs<L::THERMAL>(qr, sr, d, P);
    const double m = m1 > m2 ? m1 : m2;
#pragma unroll
    for (int k = 0; k < V; k++) {
      f[k] = m * (ql[k] - qr[k]);
      dq[k] = qr[k] - ql[k];
      b[k] = 0.0;
    }
  }
  flux_add<L::THERMAL, V>(ql, sl, d, P, f);
  flux_add<L::THERMAL, V>(qr, sr, d, P, f);
#pragma unroll
  for (int n = 0; n < NO; n++) {
    const double ir = 1.0 / (ql[0] + C.nodes[n] * dq[0]);
    double v[3] = {(ql[2] + C.nodes[n] * dq[2]) * ir, (ql[3] + C.nodes[n] * dq[3]) * ir,
                   (ql[4] + C.nodes[n] * dq[4]) * ir};
    double bd[V];
    bdot<V, L::LSET>(v, dq, d, bd);
#pragma unroll
    for (int k = 5; k < V; k++)
      if (k < 14 || k >= V - L::LSET)
        b[k] += C.w[n] * bd[k];
  }
}

// Face terms (interfs1 / interfs2, fv.cpp:111-279): one thread per (face,
// face point p) of direction dir; 1D: face f between predictor cells f and
// f + 1, p = t; 2D: faces (i, j) of the (nx + 1) x (ny + 1) face grid between
// predictor cells (i, j) and (i + 1, j) (dir 0) or (i, j + 1) (dir 1), p = t
// N + s over time node t and transverse node s.  fb[face][p][0][V] = k (b +
// f) is subtracted from the left cell, fb[face][p][1][V] = k (b - f) from the
// right one, k = W_t [W_s] dt / (2 dx_dir).  EIG: the Roe or Osher
// dissipation (flux), one thread per face point as for Rusanov.
template <class L, int NO, int ND, bool EIG = false>
__global__ void __launch_bounds__(128) k_faces_n(
    double *__restrict__ fb, const double *__restrict__ qh, int nx, int ny, int dir,
    const uint8_t *__restrict__ mask, double dt, const double *__restrict__ dt_dev, double dx,
    double dy, DevPar P, ConstsN<NO> C, int flux = 0) {
  constexpr int V = L::V;
  constexpr int NQ = ND == 1 ? NO : NO * NO;  // points per face
  constexpr int NS = ND == 1 ? NO : NO * NO;
  if (dt_dev)
    dt = *dt_dev;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long face = gt / NQ;
  const int p = gt % NQ;
  const long nf = ND == 1 ? (long)nx + 1 : (long)(nx + 1) * (ny + 1);
  if (face >= nf)
    return;
  const int t = ND == 1 ? p : p / NO, sq = ND == 1 ? 0 : p % NO;
  long cb, cn;
  bool geo = true;
  if (ND == 1) {
    cb = face;
    cn = face + 1;
  } else {
    const int i = face / (ny + 1), j = face % (ny + 1);
    cb = (long)i * (ny + 2) + j;
    cn = dir == 0 ? cb + (ny + 2) : cb + 1;
    geo = dir == 0 ? (j > 0) : (i > 0);
  }
  double *o = fb + ((face * NQ + p) * 2) * V;
  const bool active = geo && (mask == nullptr || (mask[cb] && mask[cn]));
  if (!active) {
#pragma unroll
    for (int k = 0; k < V; k++)
      o[k] = o[V + k] = 0.0;
    return;
  }
  // endpoint extrapolation (evaluations.cpp:20-35): 1D nodes m; 2D dir 0
  // nodes (m, s), dir 1 nodes (s, m)
  const double *ql_ = qh + (cb * NO + t) * NS * V;
  const double *qr_ = qh + (cn * NO + t) * NS * V;
  double ql[V], qr[V], f[V], b[V];
#pragma unroll
  for (int k = 0; k < V; k++) {
    double a = 0.0, e = 0.0;
#pragma unroll
    for (int m = 0; m < NO; m++) {
      const int node = ND == 1 ? m : (dir == 0 ? m * NO + sq : sq * NO + m);
      a += C.endv[1][m] * ql_[node * V + k];
      e += C.endv[0][m] * qr_[node * V + k];
    }
    ql[k] = a;
    qr[k] = e;
  }
  interface_point_n<L, NO, EIG>(ql, qr, dir, P, C, f, b, flux);
  const double kk = dt * C.w[t] * (ND == 1 ? 1.0 : C.w[sq]) / (2.0 * (dir == 0 ? dx : dy));
#pragma unroll
  for (int k = 0; k < V; k++) {
    o[k] = kk * (b[k] + f[k]);
    o[V + k] = kk * (b[k] - f[k]);
  }
}

// The FV update of each interior cell (centers1/2 and the interface sums,
// fv.cpp:11-109, 143-146, 253-276): the volume term over its space-time
// nodes, one thread per node, summed through shared memory in node order,
// then the face terms of its faces (1D: left face c (right part), right
// face c + 1 (left part); 2D: the x faces (ci + 1, cj + 1) and (ci, cj + 1),
// the y faces (ci + 1, cj + 1) and (ci + 1, cj)), each summed over its points.
template <class L, int NO, int ND>
__global__ void __launch_bounds__(128) k_cells_n(
    double *__restrict__ u, const double *__restrict__ qh, const double *__restrict__ fbx,
    const double *__restrict__ fby, int nx, int ny, const uint8_t *__restrict__ mask, double dt,
    const double *__restrict__ dt_dev, double dx, double dy, DevPar P, ConstsN<NO> C) {
  constexpr int V = L::V;
  using NB = NodeBlock<NO, ND>;
  constexpr int NS = NB::NS, NP = NB::NP, CPB = NB::CPB;
  constexpr int NQ = NS;  // points per face
  __shared__ double sq[CPB][NP][V];
  if (dt_dev)
    dt = *dt_dev;
  const int lc = threadIdx.x / NP;
  const int g = threadIdx.x % NP;
  const bool in_block = threadIdx.x < NB::THREADS;
  const long ncell = ND == 1 ? nx : (long)nx * ny;
  const long c = (long)blockIdx.x * CPB + lc;
  const bool valid = in_block && c < ncell;
  const long cc = valid ? c : 0;  // lanes without a cell read cell 0's nodes
  const long ci = ND == 1 ? cc : cc / ny;
  const int cj = ND == 1 ? 0 : (int)(cc % ny);
  const long cb = ND == 1 ? ci + 1 : (ci + 1) * (ny + 2) + (cj + 1);
  const bool active = valid && (mask == nullptr || mask[cb]);
  const int t = g / NS, sidx = g % NS;
  const int i = ND == 1 ? sidx : sidx / NO, j = ND == 1 ? 0 : sidx % NO;
  const double idx = 1.0 / dx, idy = 1.0 / dy;
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
  const double wn = dt * C.w[t] * C.w[i] * (ND == 1 ? 1.0 : C.w[j]);
  source<L::THERMAL, V>(q, s, P, acc, wn);
#pragma unroll
  for (int dir = 0; dir < ND; dir++) {
    const int e = dir == 0 ? i : j;
    const double h = dir == 0 ? idx : idy;
    double dq[V];
#pragma unroll
    for (int k = 0; k < V; k++) {
      double a = 0.0;
#pragma unroll
      for (int m = 0; m < NO; m++) {
        const int node = ND == 1 ? t * NS + m
                                 : (dir == 0 ? t * NS + m * NO + j : t * NS + i * NO + m);
        a += C.derv[e][m] * (in_block ? sq[lc][node][k] : 0.0);
      }
      dq[k] = a * h * wn;
    }
    double bd[V];
    bdot<V, L::LSET>(s.v, dq, dir, bd);
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
  double *uc = u + c * V;
  if (ND == 1) {
    const double *fl = fbx + (long)c * NQ * 2 * V;        // left face c: right part
    const double *fr = fbx + (long)(c + 1) * NQ * 2 * V;  // right face c + 1: left part
    const bool okl = mask == nullptr || (mask[cb - 1] && mask[cb]);
    const bool okr = mask == nullptr || (mask[cb] && mask[cb + 1]);
    for (int k = g; k < V; k += NP) {
      double x = 0.0;
#pragma unroll
      for (int n = 0; n < NP; n++)
        x += sq[lc][n][k];
      x += uc[k];
#pragma unroll
      for (int p = 0; p < NQ; p++) {
        if (okr)
          x -= fr[p * 2 * V + k];
        if (okl)
          x -= fl[p * 2 * V + V + k];
      }
      uc[k] = x;
    }
  } else {
    const long fxl = (ci + 1) * (ny + 1) + (cj + 1), fxr = ci * (ny + 1) + (cj + 1);
    const long fyl = (ci + 1) * (ny + 1) + (cj + 1), fyr = (ci + 1) * (ny + 1) + cj;
    for (int k = g; k < V; k += NP) {
      double x = 0.0;
#pragma unroll
      for (int n = 0; n < NP; n++)
        x += sq[lc][n][k];
      x += uc[k];
#pragma unroll
      for (int p = 0; p < NQ; p++) {
        x -= fbx[(fxl * NQ + p) * 2 * V + k];
        x -= fbx[(fxr * NQ + p) * 2 * V + V + k];
        x -= fby[(fyl * NQ + p) * 2 * V + k];
        x -= fby[(fyr * NQ + p) * 2 * V + V + k];
      }
      uc[k] = x;
    }
  }
}

}  // namespace order
}  // namespace gpr
